/*
 * Oracle (test infrastructure only): a plain-C restatement of the reference's
 * neighbour-list builder, used to check the CUDA cell-list build and timed as
 * the CPU baseline of the neighbour stage. It is never linked into the product.
 *
 * Follows MolEmb.Make_NListNaive (C_API/MolEmb.cpp:1180-1251):
 *   - argsort atoms by x;
 *   - for each atom I in that order, sweep J over the atoms after it until
 *     |x_I - x_J| > rng;
 *   - skip the pair unless I < nreal or J < nreal;
 *   - accept when sqrt(dx*dx + dy*dy + dz*dz) + 1e-13 < rng, evaluated in
 *     IEEE double in exactly this order, with no fused multiply-add;
 *   - store J under min(I, J); with doperms, also store the reverse entry under
 *     max(I, J) when that index is < nreal.
 * Output is the set of ordered (centre, neighbour) entries; the reference's
 * order inside a centre's list depends on its unstable sort and is not
 * reproduced (callers sort).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

static const double *g_x;

static int cmp_x(const void *a, const void *b) {
  double xa = g_x[3 * (*(const int *)a)], xb = g_x[3 * (*(const int *)b)];
  if (xa < xb) return -1;
  if (xa > xb) return 1;
  return (*(const int *)a) - (*(const int *)b);
}

/* Distance test of MolEmb.cpp:1214-1218. volatile keeps each product and sum
 * rounded separately, so no compiler contraction changes the decision. */
static int within(const double *xi, const double *xj, double rng) {
  volatile double dx = xi[0] - xj[0];
  volatile double dy = xi[1] - xj[1];
  volatile double dz = xi[2] - xj[2];
  volatile double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
  volatile double s = dx2 + dy2;
  s = s + dz2;
  double dij = sqrt(s) + 0.0000000000001;
  return dij < rng;
}

/*
 * Writes entries (centre[e], nbr[e]) for e < return value. If more than cap
 * entries exist the function returns -(needed) and writes nothing useful.
 */
int64_t tmo_nlist_naive(const double *x, int nat, double rng, int nreal,
                        int doperms, int32_t *centre, int32_t *nbr,
                        int64_t cap) {
  int *y = (int *)malloc(sizeof(int) * (size_t)(nat > 0 ? nat : 1));
  if (!y) return -1;
  for (int i = 0; i < nat; ++i) y[i] = i;
  g_x = x;
  qsort(y, (size_t)nat, sizeof(int), cmp_x);
  int64_t n = 0;
  for (int i = 0; i < nat; ++i) {
    int I = y[i];
    for (int j = i + 1; j < nat; ++j) {
      int J = y[j];
      if (!(I < nreal || J < nreal)) continue;
      if (fabs(x[3 * I] - x[3 * J]) > rng) break;
      if (!within(x + 3 * I, x + 3 * J, rng)) continue;
      int lo = I < J ? I : J, hi = I < J ? J : I;
      if (n < cap) { centre[n] = lo; nbr[n] = hi; }
      n++;
      if (hi < nreal && doperms == 1) {
        if (n < cap) { centre[n] = hi; nbr[n] = lo; }
        n++;
      }
    }
  }
  free(y);
  return n <= cap ? n : -n;
}

/*
 * Same membership rule over an explicit candidate set: the periodic images of
 * atom j are x_j + i*a0 + j*a1 + k*a2, formed left to right exactly as
 * Lattice.TessLattice builds them (ForceModifiers/Periodic.py:170-173).
 * Used by the oracle's tessellated periodic lists.
 */
void tmo_image_coords(const double *x, int nat, const double *lat, int ntess,
                      double *out) {
  int ind = 1;
  for (int a = 0; a < 3 * nat; ++a) out[a] = x[a];
  for (int i = -ntess; i <= ntess; ++i)
    for (int j = -ntess; j <= ntess; ++j)
      for (int k = -ntess; k <= ntess; ++k) {
        if (i == 0 && j == 0 && k == 0) continue;
        for (int a = 0; a < nat; ++a)
          for (int c = 0; c < 3; ++c) {
            volatile double v = x[3 * a + c] + (double)i * lat[c];
            v = v + (double)j * lat[3 + c];
            v = v + (double)k * lat[6 + c];
            out[3 * (ind * nat + a) + c] = v;
          }
        ind++;
      }
}
