"""Edge cases of the CUDA path (through the C ABI): ragged batches with
one- and two-atom molecules, neighbour rows that outgrow their initial
capacity, atoms exactly at the cutoff, non-finite and malformed input.
Tolerances as in test_gpu_parity.py; neighbour sets bit-exact.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu

E_TOL = 1e-5   # eV / atom
F_TOL = 1e-4   # eV / A


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import model
    return model


def _model(gpu, eles, **kw):
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    p.update(kw)
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    return gpu.BPEEModel(eles, W, params=p, precision="fp32"), orc.Model(eles, W, params=p)


def _check(out, ref, offsets):
    n_per = np.diff(offsets)
    dE = np.max(np.abs(out["Etotal"] - ref["Etotal"]) * EV_PER_HARTREE / n_per)
    dF = np.abs(out["force"] - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    assert dE < E_TOL and dF < F_TOL, (dE, dF)


def test_ragged_batch_with_tiny_molecules(gpu):
    """Molecules of 1, 2, 3 and 60 atoms (isolated atoms have no neighbours,
    pairs no triples) in one batch."""
    w = systems.water_cluster_60(seed=0)
    xs = [np.zeros((1, 3)), np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.97]]),
          np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]]), w.x]
    Zs = [np.array([8]), np.array([8, 1]), np.array([8, 1, 1]), w.Z]
    x = np.concatenate(xs)
    Z = np.concatenate(Zs).astype(np.int32)
    off = np.concatenate([[0], np.cumsum([len(z) for z in Zs])]).astype(np.int64)
    m, om = _model(gpu, [1, 8])
    s = m.system(x, Z, off)
    out = s.energy_force(x, True)
    ref = orc.OpenSystemOracle(om, x, Z, off).terms(x)
    _check(out, ref, off)
    assert np.all(out["force"][0] == 0.0)   # a lone atom feels nothing


def test_neighbour_rows_grow_beyond_initial_capacity(gpu):
    """Water compressed to 60 % of its spacing: more than 64 radial neighbours
    per centre, so the rows are grown and the evaluation repeated; lists stay
    bit-exact and forces match."""
    w = systems.water(125, seed=21, spacing=3.1 * 0.6)
    m, om = _model(gpu, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    out = s.energy_force(w.x, True)
    assert s.nlist_counts()["max_radial"] > 64
    radp, angt, milj, miljk = s.export_nlist()
    P, T, mj, mjk = orc.pairs_and_triples([(w.x, w.Z)], [1, 8])
    assert np.array_equal(radp, P) and np.array_equal(angt, T)
    assert np.array_equal(milj, mj) and np.array_equal(miljk, mjk)
    ref = orc.OpenSystemOracle(om, w.x, w.Z, w.offsets).terms(w.x)
    _check(out, ref, w.offsets)


def test_pairs_at_the_cutoff(gpu):
    """Atoms placed at 4.6 A and 3.1 A (the radial and angular cutoffs) and at
    15 A (Coulomb) from a centre, and 1e-9 A inside/outside: membership follows
    the reference's FP64 rule sqrt(d2) + 1e-13 < rc."""
    d = [4.6, 4.6 - 1e-9, 4.6 + 1e-9, 3.1, 3.1 - 1e-9, 3.1 + 1e-9, 15.0, 15.0 - 1e-9]
    x = [[0.0, 0.0, 0.0]]
    for q, r in enumerate(d):
        ang = 2 * np.pi * q / len(d)
        x.append([r * np.cos(ang), r * np.sin(ang), 0.1 * q])
    x = np.array(x)
    x[1:] = x[1:] * (np.array(d) / np.linalg.norm(x[1:], axis=1))[:, None]
    Z = np.array([8] + [1] * len(d), dtype=np.int32)
    off = np.array([0, len(Z)], dtype=np.int64)
    m, _ = _model(gpu, [1, 8])
    s = m.system(x, Z, off)
    s.build_nlist()
    radp, angt, milj, miljk = s.export_nlist()
    P, T, mj, mjk = orc.pairs_and_triples([(x, Z)], [1, 8])
    assert np.array_equal(radp, P) and np.array_equal(angt, T)
    ee = s.export_ee()
    ref = orc.ee_pairs([(x, Z)], 15.0)
    key = lambda a: a[np.lexsort((a[:, 2], a[:, 1], a[:, 0]))]
    assert np.array_equal(key(ee), key(ref))


def test_non_finite_positions_are_rejected(gpu):
    from tensormol_gb300._lib import TmError
    w = systems.water_cluster_60(seed=0)
    m, _ = _model(gpu, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    x = w.x.copy()
    x[7, 1] = np.nan
    with pytest.raises(TmError):
        s.energy_force(x, True)
    out = s.energy_force(w.x, True)          # the system stays usable
    assert np.all(np.isfinite(out["force"]))


def test_malformed_systems_are_rejected(gpu):
    from tensormol_gb300._lib import TmError
    m, _ = _model(gpu, [1, 8])
    x = np.zeros((3, 3))
    with pytest.raises(TmError):
        m.system(x, np.array([8, 1, 1]), np.array([0, 2, 2, 3]))      # empty molecule
    with pytest.raises(TmError):
        m.system(x, np.array([8, 1, 6]), None)                         # element not in the model
    with pytest.raises(TmError):
        m.system(x, np.array([8, 1, 1]), np.array([0, 4]))             # offsets beyond natoms


def test_pair_sums_are_bit_reproducible(gpu):
    """The pair-term sums are 64-bit fixed point added by integer atomics from
    many warps, and the pair terms run on a second stream beside the network
    backward pass: repeated evaluations, on the same system and on a new one,
    give bit-identical energies and forces."""
    w = systems.water(1000, seed=3, spacing=3.1)
    m, _ = _model(gpu, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    a = s.energy_force(w.x, True)
    b = s.energy_force(w.x, True)
    s.close()
    s2 = m.system(w.x, w.Z, w.offsets)
    c = s2.energy_force(w.x, True)
    s2.close()
    for key in ("Etotal", "force"):
        assert np.array_equal(a[key], b[key]) and np.array_equal(a[key], c[key]), key


def test_pair_sums_out_of_range_are_reported(gpu):
    """Charge networks whose outputs are absurd (|q| ~ 1e19) drive the pair
    sums past the fixed-point range: the evaluation fails with a status
    naming the pair terms, and the context stays usable."""
    from tensormol_gb300._lib import TmError
    w = systems.water_cluster_60(seed=0)
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    for e, shift in ((1, 1e19), (8, -2e19)):
        Wl, bl = W["Q"][e][-1]
        W["Q"][e][-1] = (Wl, bl + shift)
    bad = gpu.BPEEModel([1, 8], W, params=p, precision="fp32")
    s = bad.system(w.x, w.Z, w.offsets)
    with pytest.raises(TmError, match="pair terms"):
        s.energy_force(w.x, True)
    s.close()
    m, om = _model(gpu, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    out = s.energy_force(w.x, True)
    ref = orc.OpenSystemOracle(om, w.x, w.Z, w.offsets).terms(w.x)
    _check(out, ref, w.offsets)
    s.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_bounded_wait_runs_out_and_the_context_recovers(gpu, prec):
    """The tensor-core layer kernel's mbarrier waits are bounded. A selftest
    product with one pipeline stage's operand loads withheld (never issued, so
    nothing faults) and waits limited to 2^20 SM cycles must report
    TM_E_TIMEOUT; the kernel frees its tensor memory on that path, so the next
    launches on the same context (which allocate tensor memory again) and on a
    fresh context compute the product correctly."""
    import ctypes

    from tensormol_gb300 import _lib
    rng = np.random.default_rng(1)
    M, N, K = 256, 512, 256
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = (rng.normal(size=(N, K)) * 0.05).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    tol = 2e-5 if prec == 0 else 2e-2

    def product(ctx):
        C = np.zeros((M, N), np.float32)
        ctx.check(ctx.lib.tm_selftest_gemm(ctx.h, prec, M, N, K, A.ctypes.data, B.ctypes.data,
                                           C.ctypes.data))
        return np.abs(C - ref).max() / np.abs(ref).max()

    ctx = gpu.default_context()
    rc = ctx.lib.tm_selftest_gemm_timeout(ctx.h, prec, ctypes.c_int64(1 << 20))
    assert rc == _lib.ERROR_CODES["TM_E_TIMEOUT"], rc
    buf = ctypes.create_string_buffer(256)
    ctx.lib.tm_ctx_last_error(ctx.h, buf, 256)
    assert b"device status 6" in buf.value, buf.value
    for _ in range(2):
        assert product(ctx) < tol
    fresh = gpu.Context(0)
    try:
        assert product(fresh) < tol
    finally:
        fresh.close()
