"""Periodic cells of any shape (Periodic.py:12-181 takes any three lattice
vectors): a triclinic water box of 512 H2O whose plane spacings are all above
twice the 9 A Coulomb cutoff. Lists bit-exact against the oracle's 27-image
tessellation; FP32 energies within 1e-5 eV/atom and forces within 1e-4 eV/A of
the FP64 oracle (conservative force and the reference's own, images held
fixed); skin lists in a device MD run follow a full rebuild every step (the
positions are wrapped through fractional coordinates). Lattice vectors without
volume are rejected with TM_E_ARG (cells below twice the cutoff are covered in
test_gpu_periodic_small.py).
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu

L = 49.7 / 2.0


def _lattice():
    return np.array([[L, 0.0, 0.0], [0.25 * L, L, 0.0], [0.1 * L, -0.2 * L, L]])


def _plane_spacings(B):
    vol = abs(np.linalg.det(B))
    return [vol / np.linalg.norm(np.cross(B[(d + 1) % 3], B[(d + 2) % 3])) for d in range(3)]


@pytest.fixture(scope="module")
def tric():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import md, model
    b = systems.water(512, seed=5, spacing=L / 8.0, box=L, n_side=8)
    B = _lattice()
    assert min(_plane_spacings(B)) >= 18.0
    x = orc.modulo_lattice((b.x / L) @ B, B)       # the orthorhombic box's fractional sites
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    p["EECutoffOff"] = 9.0
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    return model, md, b, B, x, p, W


def test_triclinic_lists_bit_exact(tric):
    model, md, b, B, x, p, W = tric
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    s = m.system(x, b.Z, None, B)
    s.build_nlist()
    radp, angt, milj, miljk = s.export_nlist()
    xt = orc.tessellate(x, B)
    Zt = np.tile(b.Z, 27)
    P, T, mj, mjk = orc.pairs_and_triples([(xt, Zt)], [1, 8], nreal=[len(b.Z)])
    assert np.array_equal(radp, P) and np.array_equal(angt, T)
    assert np.array_equal(milj, mj) and np.array_equal(miljk, mjk)
    ee = s.export_ee()
    ref = orc.ee_pairs([(xt, Zt)], 9.0, nreal=[len(b.Z)], doperms=True)
    key = lambda a: a[np.lexsort((a[:, 2], a[:, 1], a[:, 0]))]
    assert np.array_equal(key(ee), key(ref))


def test_triclinic_energy_force(tric):
    model, md, b, B, x, p, W = tric
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    s = m.system(x, b.Z, None, B)
    out = s.energy_force(x, True)
    ref = orc.PeriodicOracle(orc.Model([1, 8], W, p), x, b.Z, B, ree_cut=9.0).terms(x)
    dE = abs(out["Etotal"][0] - ref["Etotal"][0]) * EV_PER_HARTREE / len(b.Z)
    dF = np.abs(out["force"] - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    out_r = s.energy_force(x, True, reference_periodic_force=True)
    dFr = np.abs(out_r["force"] - ref["force_ref"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    print(f"triclinic: dE/atom={dE:.2e} eV  max|dF|={dF:.2e}  reference force {dFr:.2e} eV/A")
    assert dE < 1e-5 and dF < 1e-4 and dFr < 1e-4, (dE, dF, dFr)


def test_triclinic_skin_lists_follow_the_full_rebuild(tric):
    model, md, b, B, x, p, W = tric
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    v0 = systems.maxwell_boltzmann(b.Z, 600.0, seed=15)
    out = []
    for skin in (0.0, 1.0):
        s = m.system(x, b.Z, None, B)
        dyn = md.DeviceMD(s, "nhc", dt=0.5, T=300.0)
        dyn.set_velocities(v0)
        log = dyn.run(40, skin=skin)
        out.append((s.positions(), dyn.velocities(), log))
        dyn.close()
        s.close()
    (x_a, v_a, l_a), (x_b, v_b, l_b) = out
    binv = np.linalg.inv(B)
    df = (x_a - x_b) @ binv
    d = (df - np.round(df)) @ B
    f_b = x_b @ binv
    assert np.all(f_b >= -1e-12) and np.all(f_b < 1.0 + 1e-12)   # handed back inside the cell
    assert np.abs(d).max() < 2e-5 and np.abs(v_a - v_b).max() < 2e-5
    np.testing.assert_allclose(l_a[:, 0], l_b[:, 0], rtol=0, atol=1e-8 * len(b.Z))


def test_degenerate_lattices_are_rejected(tric):
    from tensormol_gb300 import _lib
    model, md, b, B, x, p, W = tric
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    flat = B.copy()
    flat[2] = B[0] + B[1]                                # no volume
    with pytest.raises(_lib.TmError) as err:
        m.system(x, b.Z, None, flat)
    assert err.value.code == _lib.ERROR_CODES["TM_E_ARG"]
