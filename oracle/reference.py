"""CPU restatement (FP64) of TensorMol's BP+EE energy/force path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg, never by the product.

Each function cites the reference code it restates. Integer work (neighbour
lists, triples, element tags, lexsorts, slot indices) is numpy over the C
restatement in ``nlist.c``; the floating-point graph is PyTorch-CPU float64
with autograd forces, like the reference's ``tf.gradients``
(TFBehlerParinelloSymEE.py:1490).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np
import torch

from tensormol_gb300.params import (BOHRPERA, JOULEPERHARTREE, PARAMS, ani1_grids,
                                    coulomb_constants, element_pairs, vdw_tables)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build_oracle_lib():
    """Compile ``nlist.c`` (plain C, IEEE double, no contraction)."""
    src = os.path.join(_HERE, "nlist.c")
    out = os.path.join(_HERE, "libtmoracle.so")
    if (not os.path.exists(out)) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-o", out, src, "-lm"])
    return out


def _lib():
    global _LIB
    if _LIB is None:
        lib = ctypes.CDLL(build_oracle_lib())
        lib.tmo_nlist_naive.restype = ctypes.c_int64
        lib.tmo_nlist_naive.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int64]
        lib.tmo_image_coords.restype = None
        lib.tmo_image_coords.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_void_p]
        _LIB = lib
    return _LIB


# ---------------------------------------------------------------------------
# Neighbour lists
# ---------------------------------------------------------------------------
def nlist_entries(x, rc, nreal=None, doperms=True):
    """(centre, nbr) entries of ``Make_NListNaive`` (MolEmb.cpp:1180-1251),
    sorted by (centre, nbr)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    nat = x.shape[0]
    nreal = nat if nreal is None else int(nreal)
    cap = max(1024, nat * 64)
    while True:
        c = np.empty(cap, dtype=np.int32)
        n = np.empty(cap, dtype=np.int32)
        got = _lib().tmo_nlist_naive(x.ctypes.data, nat, float(rc), nreal, int(doperms),
                                     c.ctypes.data, n.ctypes.data, cap)
        if got >= 0:
            break
        cap = int(-got) + 16
    c, n = c[:got].astype(np.int64), n[:got].astype(np.int64)
    o = np.lexsort((n, c))
    return c[o], n[o]


def _triples_from_entries(c, n):
    """All unordered {j, k} (j < k) from each centre's list, as the double loop
    of NeighborList.buildPairsAndTriples (Neighbors.py:173-197) enumerates
    them. Input sorted by (centre, nbr)."""
    if len(c) == 0:
        e = np.zeros(0, dtype=np.int64)
        return e, e, e
    starts = np.r_[0, np.flatnonzero(np.diff(c)) + 1]
    cnt = np.diff(np.r_[starts, len(c)])
    grp = np.repeat(np.arange(len(starts)), cnt)
    local = np.arange(len(c)) - starts[grp]
    rep = cnt[grp] - 1 - local
    p = np.repeat(np.arange(len(c)), rep)
    blk = np.cumsum(rep) - rep
    q = p + 1 + (np.arange(rep.sum()) - np.repeat(blk, rep))
    return c[p], n[p], n[q]


def _slot_index(keys):
    """Running index inside runs of equal key rows (Neighbors.py:395-413)."""
    if len(keys) == 0:
        return np.zeros(0, dtype=np.int64)
    change = np.r_[True, np.any(keys[1:] != keys[:-1], axis=1)]
    starts = np.flatnonzero(change)
    grp = np.cumsum(change) - 1
    return np.arange(len(keys)) - starts[grp]


def pairs_and_triples(mols, eles, rr_cut=4.6, ra_cut=3.1, nreal=None):
    """``NeighborListSet(...).buildPairsAndTriplesWithEleIndexLinear``.

    mols: list of (x [n,3], Z [n]) per molecule (tessellated coordinates for a
    periodic cell, with ``nreal`` real atoms first).
    Returns (RadpEle [P,4]=(mol,i,j,l), AngtEle [T,5]=(mol,i,j,k,l),
    mil_j [P,4], mil_jk [T,4]) as int64, in the reference's sorted order
    (Neighbors.py:344-467).
    """
    eles = list(eles)
    elep = element_pairs(eles)
    e_index = {e: i for i, e in enumerate(eles)}
    ep_index = {}
    for i, (a, b) in enumerate(elep):
        ep_index[(a, b)] = i
        ep_index[(b, a)] = i
    P, T = [], []
    for m, (x, Z) in enumerate(mols):
        Z = np.asarray(Z)
        nr = None if nreal is None else nreal[m]
        pc, pn = nlist_entries(x, rr_cut, nr, True)
        tc, tn = nlist_entries(x, ra_cut, nr, True)
        # pairs (mol, i, j, l)
        l = np.array([e_index[int(z)] for z in Z[pn]], dtype=np.int64)
        P.append(np.stack([np.full_like(pc, m), pc, pn, l], 1))
        # triples, lower element first; equal elements keep j < k
        ti, tj, tk = _triples_from_entries(tc, tn)
        swap = Z[tj] > Z[tk]
        j2 = np.where(swap, tk, tj)
        k2 = np.where(swap, tj, tk)
        lt = np.array([ep_index[(int(a), int(b))] for a, b in zip(Z[j2], Z[k2])], dtype=np.int64)
        T.append(np.stack([np.full_like(ti, m), ti, j2, k2, lt], 1))
    P = np.concatenate(P) if P else np.zeros((0, 4), np.int64)
    T = np.concatenate(T) if T else np.zeros((0, 5), np.int64)
    P = P[np.lexsort((P[:, 2], P[:, 3], P[:, 1], P[:, 0]))]           # Neighbors.py:380
    T = T[np.lexsort((T[:, 2], T[:, 3], T[:, 4], T[:, 1], T[:, 0]))]  # Neighbors.py:382
    mil_j = np.concatenate([P[:, [0, 1, 3]], _slot_index(P[:, [0, 1, 3]])[:, None]], 1)
    mil_jk = np.concatenate([T[:, [0, 1, 4]], _slot_index(T[:, [0, 1, 4]])[:, None]], 1)
    return P, T, mil_j, mil_jk


def ee_pairs(mols, rc=15.0, nreal=None, doperms=False):
    """``NeighborListSet(x, n, False, False, None).buildPairs(rc)``
    (TFMolManage.py:1430-1431, Neighbors.py:262-282): (mol, i, j) with i < j
    (doperms=False), sorted by (mol, i, j)."""
    out = []
    for m, (x, _) in enumerate(mols):
        nr = None if nreal is None else nreal[m]
        c, n = nlist_entries(x, rc, nr, doperms)
        out.append(np.stack([np.full_like(c, m), c, n], 1))
    return np.concatenate(out) if out else np.zeros((0, 3), np.int64)


def tessellate(x, lattice, ntess=1):
    """Real atoms first, then the 26 images in (i, j, k) raster order
    (Lattice.TessLattice, Periodic.py:131-181)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    lat = np.ascontiguousarray(lattice, dtype=np.float64)
    nimg = (2 * ntess + 1) ** 3
    out = np.empty((nimg * x.shape[0], 3))
    _lib().tmo_image_coords(x.ctypes.data, x.shape[0], lat.ctypes.data, ntess, out.ctypes.data)
    return out


def image_shift_table(lattice, ntess=1):
    """Shift vectors of the tessellated images in the same raster order."""
    s = [np.zeros(3)]
    for i in range(-ntess, ntess + 1):
        for j in range(-ntess, ntess + 1):
            for k in range(-ntess, ntess + 1):
                if i == 0 and j == 0 and k == 0:
                    continue
                s.append(i * lattice[0] + j * lattice[1] + k * lattice[2])
    return np.array(s)


def modulo_lattice(x, lattice):
    """Fractional-coordinate wrap into [0, 1) (Lattice.ModuloLattice,
    Periodic.py:87-100), written with a plain inverse."""
    inv = np.linalg.inv(lattice)
    f = np.fmod(x @ inv, 1.0)
    f = np.where(f < 0.0, f + 1.0, f)
    return f @ lattice


# ---------------------------------------------------------------------------
# FP64 graph
# ---------------------------------------------------------------------------
_PI_TF = 3.14159265359   # literal of RawSymFunc.py:935-936, 1799


def _act(name, alpha):
    if name == "relu":
        return torch.relu
    if name == "sigmoid_with_param":   # Util.py:200-201, stable form
        return lambda z: torch.logaddexp(alpha * z, torch.zeros_like(z)) / alpha
    if name == "softplus":
        return torch.nn.functional.softplus
    if name == "tanh":
        return torch.tanh
    if name == "elu":
        return torch.nn.functional.elu
    raise ValueError(name)


class Model:
    """FP64 BP+EE model: descriptors, per-element energy/charge MLPs,
    charge neutralisation, DSF/elu Coulomb and C6 vdW."""

    def __init__(self, eles, weights, params=None, has_vdw=True):
        self.p = dict(PARAMS if params is None else params)
        self.eles = list(eles)
        self.elep = element_pairs(self.eles)
        self.weights = weights
        self.has_vdw = has_vdw
        rs_r, rs_a, th = ani1_grids(self.p)
        self.rs_r = torch.tensor(rs_r, dtype=torch.float64)
        self.rs_a = torch.tensor(rs_a, dtype=torch.float64)
        self.th = torch.tensor(th, dtype=torch.float64)
        self.cc = coulomb_constants(self.p)
        c6, r0 = vdw_tables(self.eles, self.p)
        self.c6 = torch.tensor(c6, dtype=torch.float64)
        self.r0 = torch.tensor(r0, dtype=torch.float64)
        self.act = _act(self.p["NeuronType"], self.p["sigmoid_alpha"])
        self.tW = {net: {e: [(torch.tensor(W, dtype=torch.float64), torch.tensor(b, dtype=torch.float64))
                             for (W, b) in self.weights[net][e]] for e in self.eles}
                   for net in ("E", "Q")}

    # RawSymFunc.py:1757-1810
    def radial(self, X, pi, pj, pl, nrow):
        nele, nr = len(self.eles), len(self.rs_r)
        R = X[pi] - X[pj]
        r = torch.sqrt((R * R).sum(1) + 1e-27)
        t = r[:, None] - self.rs_r[None, :]
        fac1 = torch.exp(-self.p["AN1_eta"] * t * t)
        fac2 = 0.5 * (torch.cos(_PI_TF * r / self.p["AN1_r_Rc"]) + 1.0)
        g = fac1 * fac2[:, None]
        out = torch.zeros(nrow * nele, nr, dtype=X.dtype)
        out = out.index_add(0, pi * nele + pl, g)
        return out.reshape(nrow, nele * nr)

    # RawSymFunc.py:868-963
    def angular(self, X, ti, tj, tk, tl, nrow):
        nelep, na, nt = len(self.elep), len(self.rs_a), len(self.th)
        zeta, eta, rc = self.p["AN1_zeta"], self.p["AN1_eta"], self.p["AN1_a_Rc"]
        Rij = X[ti] - X[tj]
        Rik = X[ti] - X[tk]
        rij = torch.sqrt((Rij * Rij).sum(1) + 1e-27)
        rik = torch.sqrt((Rik * Rik).sum(1) + 1e-27)
        c = (Rij * Rik).sum(1) / (rij * rik)
        one = 1.0 - 0.0000000000000001
        c = torch.where(c >= 1.0, torch.full_like(c, one), c)
        c = torch.where(c <= -1.0, torch.full_like(c, -one), c)
        theta = torch.acos(c)
        T = torch.cos(theta[:, None] - self.th[None, :])              # [T, nt]
        fac1 = (2.0 ** (1.0 - zeta)) * torch.pow(1.0 + T, zeta)
        ravg = (rij + rik) / 2.0
        u = ravg[:, None] - self.rs_a[None, :]
        fac2 = torch.exp(-eta * u * u)                                # [T, na]
        fac3 = 0.5 * (torch.cos(_PI_TF * rij / rc) + 1.0)
        fac4 = 0.5 * (torch.cos(_PI_TF * rik / rc) + 1.0)
        g = fac1[:, :, None] * fac2[:, None, :] * (fac3 * fac4)[:, None, None]
        out = torch.zeros(nrow * nelep, nt * na, dtype=X.dtype)
        out = out.index_add(0, ti * nelep + tl, g.reshape(-1, nt * na))
        return out.reshape(nrow, nelep * nt * na)

    def mlp(self, net, G, Zc):
        out = torch.zeros(G.shape[0], dtype=G.dtype)
        for e in self.eles:
            idx = torch.nonzero(Zc == e).flatten()
            if idx.numel() == 0:
                continue
            h = G[idx]
            layers = self.tW[net][e]
            for (W, b) in layers[:-1]:
                h = self.act(h @ W + b)
            W, b = layers[-1]
            out = out.index_put((idx,), (h @ W + b).flatten())
        return out

    # RawSymFunc.py:1307-1359
    def coulomb(self, Xb, q, ei, ej):
        cc = self.cc
        R = Xb[ei] - Xb[ej]
        r = torch.sqrt((R * R).sum(1) + 1e-27)
        sr_sub = torch.where(r > cc["r_sr"], cc["elu_a"] * (r - cc["r_sr"]) + cc["elu_shift"],
                             cc["elu_a"] * (torch.exp(r - cc["r_sr"]) - 1.0) + cc["elu_shift"])
        qq = q[ei] * q[ej]
        xx = cc["alpha"] * cc["r_lr"]
        zz = math.erfc(xx) / cc["r_lr"]
        yy = 1.1283791671 * cc["alpha"] * math.exp(-xx * xx) / cc["r_lr"]
        lr = qq * (torch.special.erfc(cc["alpha"] * r) / r - zz + (r - cc["r_lr"]) * (zz / cc["r_lr"] + yy))
        lr = torch.where(torch.isnan(lr), torch.zeros_like(lr), lr)
        lr = torch.where(r > cc["r_lr"], torch.zeros_like(lr), lr)
        return torch.where(r > cc["r_sr"], lr, qq * sr_sub)

    # RawSymFunc.py:1361-1414 (coordinates arrive in bohr and are scaled again)
    def vdw(self, Xb, eidx, ei, ej):
        R2 = Xb * BOHRPERA
        width = self.p["Poly_Width"] * BOHRPERA
        begin = self.p["EECutoffOn"] * BOHRPERA
        D = R2[ei] - R2[ej]
        r = torch.sqrt((D * D).sum(1) + 1e-27)
        t = (r - begin) / width
        cut1 = torch.where(t > 0.0, -t * t * (2.0 * t - 3.0), torch.zeros_like(t))
        cut = torch.where(t > 1.0, torch.ones_like(t), cut1)
        a, b = eidx[ei], eidx[ej]
        return -cut * torch.sqrt(self.c6[a] * self.c6[b]) / torch.pow(r, 6.0) * 1.0 / (
            1.0 + 6.0 * torch.pow(r / (self.r0[a] + self.r0[b]), -12.0))

    def energy_terms(self, Xall, Z, mol_of_row, nmol, natom_of_mol, nl, nreal_rows=None,
                     periodic=False):
        """Energies of the graph for coordinates ``Xall`` (rows = atoms,
        including images when periodic). ``nl`` holds global row indices:
        pairs (pi, pj, pl), triples (ti, tj, tk, tl), ee pairs (ei, ej).
        Centres are rows < nreal_rows."""
        nrow = Xall.shape[0] if nreal_rows is None else nreal_rows
        Zc = Z[:nrow]
        G = torch.cat([self.radial(Xall, *nl["pairs"], nrow),
                       self.angular(Xall, *nl["triples"], nrow)], 1)
        Ea = self.mlp("E", G, Zc)
        qa = self.mlp("Q", G, Zc)
        mol = mol_of_row[:nrow]
        dt = Xall.dtype
        net = torch.zeros(nmol, dtype=dt).index_add(0, mol, qa)
        qs = qa - (net / natom_of_mol)[mol]       # TFBehlerParinelloSymEE.py:1006-1009
        Ebp = torch.zeros(nmol, dtype=dt).index_add(0, mol, Ea)
        Xb = Xall * BOHRPERA
        dip = torch.zeros(nmol, 3, dtype=dt).index_add(0, mol, Xb[:nrow] * qs[:, None])
        ei, ej = nl["ee"]
        qall = qs if not periodic else qs.repeat(Xall.shape[0] // nrow)
        emol = mol_of_row[ei]
        Ecc = torch.zeros(nmol, dtype=dt)
        if self.p["AddEcc"]:
            Ecc = Ecc.index_add(0, emol, self.coulomb(Xb, qall, ei, ej))
        Evdw = torch.zeros(nmol, dtype=dt)
        if self.has_vdw:
            eidx = torch.tensor([self.eles.index(int(z)) for z in Z.tolist()], dtype=torch.int64)
            Evdw = Evdw.index_add(0, emol, self.vdw(Xb, eidx, ei, ej))
        if periodic:                              # TFBehlerParinelloSymEE.py:1550,1620
            Ecc = Ecc / 2.0
            Evdw = Evdw / 2.0
        Etot = Ebp + Ecc + Evdw
        return dict(Etotal=Etot, Ebp=Ebp, Ecc=Ecc, Evdw=Evdw, Ebp_atom=Ea, charge=qs,
                    dipole=dip, G=G)


def _to_global(system_offsets, P, T, EE):
    off = np.asarray(system_offsets)
    gp = (off[P[:, 0]] + P[:, 1], off[P[:, 0]] + P[:, 2], P[:, 3])
    gt = (off[T[:, 0]] + T[:, 1], off[T[:, 0]] + T[:, 2], off[T[:, 0]] + T[:, 3], T[:, 4])
    ge = (off[EE[:, 0]] + EE[:, 1], off[EE[:, 0]] + EE[:, 2])
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.int64)
    return dict(pairs=tuple(map(t, gp)), triples=tuple(map(t, gt)), ee=tuple(map(t, ge)))


class OpenSystemOracle:
    """Reference E+F of an open-boundary batch (``EvalBPDirectEELinearSingle`` /
    ``EvalBPDirectEEUpdateSet``, TFMolManage.py:1260-1288, 1410-1439)."""

    def __init__(self, model, x, Z, offsets, rr_cut=4.6, ra_cut=3.1, ree_cut=15.0):
        self.model = model
        self.Z = np.asarray(Z)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        nmol = len(self.offsets) - 1
        mols = [(x[self.offsets[m]:self.offsets[m + 1]], self.Z[self.offsets[m]:self.offsets[m + 1]])
                for m in range(nmol)]
        self.P, self.T, self.mil_j, self.mil_jk = pairs_and_triples(mols, model.eles, rr_cut, ra_cut)
        self.EE = ee_pairs(mols, ree_cut)
        self.nl = _to_global(self.offsets, self.P, self.T, self.EE)
        self.nmol = nmol
        counts = np.diff(self.offsets)
        self.mol_of_row = torch.as_tensor(np.repeat(np.arange(nmol), counts), dtype=torch.int64)
        self.natom = torch.as_tensor(counts, dtype=torch.float64)
        self.tZ = torch.as_tensor(self.Z, dtype=torch.int64)

    def terms(self, x, grad=True):
        X = torch.tensor(np.asarray(x), dtype=torch.float64, requires_grad=grad)
        out = self.model.energy_terms(X, self.tZ, self.mol_of_row, self.nmol, self.natom, self.nl)
        if grad:
            g, = torch.autograd.grad(out["Etotal"].sum(), X)
            out["gradient"] = g
            out["force"] = -JOULEPERHARTREE * g      # TFMolManage.py:1439
        return {k: v.detach().numpy() for k, v in out.items()}

    def energy(self, x):
        with torch.no_grad():
            X = torch.tensor(np.asarray(x), dtype=torch.float64)
            return self.model.energy_terms(X, self.tZ, self.mol_of_row, self.nmol, self.natom,
                                           self.nl)["Etotal"].numpy()

    def fd_gradient(self, x, atoms, h=1e-4):
        """Central finite differences of the total energy (fixed lists), h in A."""
        x = np.array(x, dtype=np.float64)
        g = np.zeros((len(atoms), 3))
        for a_i, a in enumerate(atoms):
            for c in range(3):
                xp = x.copy(); xp[a, c] += h
                xm = x.copy(); xm[a, c] -= h
                g[a_i, c] = (self.energy(xp).sum() - self.energy(xm).sum()) / (2 * h)
        return g


class PeriodicOracle:
    """Reference E+F of a periodic cell via 27-image tessellation
    (PeriodicForce.__call__ Periodic.py:376-400 ->
    EvalBPDirectEEUpdateSinglePeriodic TFMolManage.py:1324-1358 ->
    evaluate_periodic TFBehlerParinelloSymEE.py:1641-1669).

    ``force_ref`` is the reference's returned force: the gradient with respect to
    the first nreal rows of the tessellated coordinates, images held fixed.
    ``force`` is the gradient of the same energy with images moving with their
    atoms (the conservative force of the periodic energy)."""

    def __init__(self, model, x, Z, lattice, rr_cut=4.6, ra_cut=3.1, ree_cut=15.0, ntess=1):
        self.model = model
        self.lattice = np.asarray(lattice, dtype=np.float64)
        self.nreal = x.shape[0]
        self.ntess = ntess
        self.Z = np.asarray(Z)
        xt = tessellate(x, self.lattice, ntess)
        nimg = xt.shape[0] // self.nreal
        Zt = np.tile(self.Z, nimg)
        mols = [(xt, Zt)]
        self.P, self.T, self.mil_j, self.mil_jk = pairs_and_triples(mols, model.eles, rr_cut, ra_cut,
                                                                    nreal=[self.nreal])
        self.EE = ee_pairs(mols, ree_cut, nreal=[self.nreal], doperms=True)
        self.nl = _to_global(np.array([0]), self.P, self.T, self.EE)
        self.shifts = torch.tensor(image_shift_table(self.lattice, ntess), dtype=torch.float64)
        self.tZ = torch.as_tensor(Zt, dtype=torch.int64)
        self.mol_of_row = torch.zeros(xt.shape[0], dtype=torch.int64)
        self.natom = torch.tensor([float(self.nreal)], dtype=torch.float64)

    def terms(self, x, grad=True):
        X = torch.tensor(np.asarray(x), dtype=torch.float64, requires_grad=grad)
        # images as functions of the real coordinates (same values as tessellate)
        Xall = (X[None, :, :] + self.shifts[:, None, :]).reshape(-1, 3)
        Xall_leaf = Xall.detach().clone().requires_grad_(grad)
        out = self.model.energy_terms(Xall_leaf if grad else Xall, self.tZ, self.mol_of_row, 1,
                                      self.natom, self.nl, nreal_rows=self.nreal, periodic=True)
        if grad:
            g_all, = torch.autograd.grad(out["Etotal"].sum(), Xall_leaf)
            g_cons = g_all.reshape(-1, self.nreal, 3).sum(0)
            out["gradient"] = g_cons
            out["force"] = -JOULEPERHARTREE * g_cons
            out["force_ref"] = -JOULEPERHARTREE * g_all[:self.nreal]
        return {k: v.detach().numpy() for k, v in out.items()}


# ---------------------------------------------------------------------------
# Integrators (FP64), Simulations/SimpleMD.py
# ---------------------------------------------------------------------------
def anharmonic_wells(x0, k=4.0e5, c=1.0e5):
    """A force field for pinning the integrators, not a reference function:
    every atom sits in its own well E = k/2 |d|^2 + c/4 |d|^4 about x0
    (d = x - x0; k in J/mol/A^2, c in J/mol/A^4, about an O-H stretch).
    Returns ef(x) -> (E [J/mol], F [N,3] J/mol/A), the (energy, force)
    routine the integrators take."""
    x0 = np.array(x0, dtype=np.float64)

    def ef(x):
        d = x - x0
        r2 = np.einsum("ia,ia->i", d, d)
        e = float(np.sum(0.5 * k * r2 + 0.25 * c * r2 * r2))
        f = -(k + c * r2)[:, None] * d
        return e, f

    return ef


def kinetic_energy(v, m):
    """Per-atom KE in J/mol (SimpleMD.py:40-51)."""
    return 0.5 * np.dot(np.einsum("ia,ia->i", v, v) * 1e10, m) / len(m)


def vv_step(ef, a, x, v, m, dt):
    """VelocityVerletStep (SimpleMD.py:14-38)."""
    x = x + v * dt + 0.5 * a * dt * dt
    e, f = ef(x)
    a_new = 1e-10 * np.einsum("ax,a->ax", f, 1.0 / m)
    v = v + 0.5 * (a + a_new) * dt
    return x, v, a_new, e


class Nose:
    """NoseThermostat.step (SimpleMD.py:104-129)."""

    def __init__(self, m, T, dt):
        from tensormol_gb300.params import IDEALGASR
        self.m, self.N, self.T, self.dt = m, len(m), T, dt
        self.eta = 0.0
        self.kT = IDEALGASR * 1e-10 * T
        tau = 20.0 * dt * self.N
        self.Q = self.kT * tau * tau

    def step(self, ef, a, x, v):
        dt, m, N, kT = self.dt, self.m, self.N, self.kT
        x = x + v * dt + 0.5 * (a - self.eta * v) * dt * dt
        vdto2 = v + 0.5 * (a - self.eta * v) * dt
        e, f = ef(x)
        a_new = 1e-10 * np.einsum("ax,a->ax", f, 1.0 / m)
        ke = 0.5 * np.dot(np.einsum("ia,ia->i", v, v), m)
        etadto2 = self.eta + (dt / (2.0 * self.Q)) * (ke - ((3.0 * N + 1) / 2.0) * kT)
        kedto2 = 0.5 * np.dot(np.einsum("ia,ia->i", vdto2, vdto2), m)
        self.eta = etadto2 + (dt / (2.0 * self.Q)) * (kedto2 - ((3.0 * N + 1) / 2.0) * kT)
        v = (vdto2 + (dt / 2.0) * a_new) / (1 + (dt / 2.0) * self.eta)
        return x, v, a_new, e


class NoseHooverChain:
    """Nose-Hoover chain VV step after Martyna, Tuckerman, Tobias & Klein,
    Mol. Phys. 87, 1117 (1996), Appendix A, with the reference's choices
    (SimpleMD.py:206-320): nc = 2, ny = 3 Suzuki-Yoshida weights,
    Q0 = 3 N kT tau^2, Qi = kT tau^2, tau = 80 dt, Nf = 3N. The particle
    velocities are scaled by the first chain element (the paper), not by the
    second one as SimpleMD.py:304 does.

    as_simplemd=True reproduces SimpleMD.py's two departures from the paper,
    for pinning this restatement against the reference's own code: the
    velocity scale uses the second chain element (SimpleMD.py:304), and the
    chain forces G[1:] start at zero (SimpleMD.py:245) and carry over between
    half steps instead of being formed from the chain velocities at the start
    of each half step (SimpleMD.py:291). After the first half step the carried
    values equal the formed ones, so only the first half step and the scale
    differ."""

    def __init__(self, m, T, dt, M=3, as_simplemd=False):
        from tensormol_gb300.params import IDEALGASR
        if as_simplemd and M < 2:
            raise ValueError("SimpleMD.py's velocity scale reads the second chain element")
        self.as_simplemd = as_simplemd
        self.m, self.N, self.M, self.dt = m, len(m), M, dt
        self.kT = IDEALGASR * 1e-10 * T
        self.GNKT = 3 * self.N * self.kT
        self.nc = 2
        w = 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
        self.wj = np.array([w, 1.0 - 2.0 * w, w])
        tau = 80.0 * dt
        self.Q = np.ones(M) * self.kT * tau * tau
        self.Q[0] = 3.0 * self.N * self.kT * tau * tau
        self.eta = np.zeros(M)
        self.veta = np.zeros(M)
        self.G = np.zeros(M)

    def _ke2(self, v):
        return np.dot(np.einsum("ia,ia->i", v, v), self.m)   # 2 * KE

    def half_chain(self, v):
        M, Q, kT = self.M, self.Q, self.kT
        ake2 = self._ke2(v)
        self.G[0] = (ake2 - self.GNKT) / Q[0]
        if not self.as_simplemd:
            for i in range(M - 1):
                self.G[i + 1] = (Q[i] * self.veta[i] ** 2 - kT) / Q[i + 1]
        iscale = 1 if self.as_simplemd else 0
        scale = 1.0
        for _ in range(self.nc):
            for wj in self.wj:
                d2 = (wj * self.dt / self.nc) / 2.0
                d4, d8 = d2 / 2.0, d2 / 4.0
                self.veta[M - 1] += self.G[M - 1] * d4
                for i in range(M - 2, -1, -1):
                    aa = math.exp(-d8 * self.veta[i + 1])
                    self.veta[i] = self.veta[i] * aa * aa + d4 * self.G[i] * aa
                aa = math.exp(-d2 * self.veta[iscale])
                scale *= aa
                self.G[0] = (scale * scale * ake2 - self.GNKT) / Q[0]
                self.eta += self.veta * d2
                for i in range(M - 1):
                    aa = math.exp(-d8 * self.veta[i + 1])
                    self.veta[i] = self.veta[i] * aa * aa + d4 * self.G[i] * aa
                    self.G[i + 1] = (Q[i] * self.veta[i] ** 2 - kT) / Q[i + 1]
                self.veta[M - 1] += self.G[M - 1] * d4
        return v * scale

    def step(self, ef, a, x, v):
        dt = self.dt
        v = self.half_chain(v)
        v = v + 0.5 * dt * a
        x = x + dt * v
        e, f = ef(x)
        a_new = 1e-10 * np.einsum("ax,a->ax", f, 1.0 / self.m)
        v = v + 0.5 * dt * a_new
        v = self.half_chain(v)
        return x, v, a_new, e

    def conserved(self, v, epot_jmol):
        """KE + PE + chain energy, all in J/mol."""
        ke = 0.5 * self._ke2(v) * 1e10
        chain = (0.5 * np.sum(self.Q * self.veta ** 2) + self.GNKT * self.eta[0]
                 + self.kT * np.sum(self.eta[1:])) * 1e10
        return ke + epot_jmol + chain
