"""The oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from Neighbors.py + MolEmb built from source)."""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import PARAMS, descriptor_width


def _mols(g):
    x, Z, off = g["x"], g["Z"], g["offsets"]
    return [(x[off[m]:off[m + 1]], Z[off[m]:off[m + 1]]) for m in range(len(off) - 1)]


@pytest.mark.parametrize("name,eles", [("water60", [1, 8]), ("chno6", [1, 6, 7, 8])])
def test_open_lists_bit_exact(golden_loader, name, eles):
    g = golden_loader(name)
    P, T, mj, mjk = orc.pairs_and_triples(_mols(g), eles)
    assert np.array_equal(P, g["RadpEle"].astype(np.int64))
    assert np.array_equal(T, g["AngtEle"].astype(np.int64))
    assert np.array_equal(mj, g["mil_j"].astype(np.int64))
    assert np.array_equal(mjk, g["mil_jk"].astype(np.int64))
    EE = orc.ee_pairs(_mols(g), 15.0)
    ref = g["rad_eep"].astype(np.int64)
    ref = ref[np.lexsort((ref[:, 2], ref[:, 1], ref[:, 0]))]
    assert np.array_equal(EE, ref)


def test_periodic_lists_bit_exact(golden_loader):
    g = golden_loader("waterbox192")
    n = len(g["Z"])
    xt = orc.tessellate(g["x"], g["lattice"])
    Zt = np.tile(g["Z"], 27)
    P, T, mj, mjk = orc.pairs_and_triples([(xt, Zt)], [1, 8], nreal=[n])
    assert np.array_equal(P, g["RadpEle"].astype(np.int64))
    assert np.array_equal(T, g["AngtEle"].astype(np.int64))
    assert np.array_equal(mj, g["mil_j"].astype(np.int64))
    assert np.array_equal(mjk, g["mil_jk"].astype(np.int64))
    EE = orc.ee_pairs([(xt, Zt)], float(g["ree_cut"]), nreal=[n], doperms=True)
    ref = g["rad_eep_e1e2"].astype(np.int64)
    assert np.array_equal(ref[:, 3], (Zt[ref[:, 1]] == 8).astype(np.int64))
    ref = ref[:, :3][np.lexsort((ref[:, 2], ref[:, 1], ref[:, 0]))]
    assert np.array_equal(EE, ref)


def _water_oracle(g, act="relu"):
    p = dict(PARAMS)
    p["NeuronType"] = act
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    model = orc.Model([1, 8], W, params=p)
    return orc.OpenSystemOracle(model, g["x"], g["Z"], g["offsets"])


def test_descriptor_matches_molemb(golden_loader):
    g = golden_loader("water60")
    out = _water_oracle(g).terms(g["x"], grad=False)
    # MolEmb writes pi as 3.14159265358979, the TF graph as 3.14159265359
    np.testing.assert_allclose(out["G"], g["ani1_G"], rtol=0, atol=1e-11)


def test_descriptor_chno_matches_molemb(golden_loader):
    g = golden_loader("chno6")
    W = systems.random_weights([1, 6, 7, 8], descriptor_width(4), seed=7)
    model = orc.Model([1, 6, 7, 8], W)
    x0 = g["x"][g["offsets"][0]:g["offsets"][1]]
    Z0 = g["Z"][g["offsets"][0]:g["offsets"][1]]
    o = orc.OpenSystemOracle(model, x0, Z0, np.array([0, len(Z0)]))
    out = o.terms(x0, grad=False)
    np.testing.assert_allclose(out["G"], g["ani1_G_mol0"], rtol=0, atol=1e-11)


def test_descriptor_jacobian_matches_molemb(golden_loader):
    import torch
    g = golden_loader("water60")
    o = _water_oracle(g)
    X = torch.tensor(g["x"], requires_grad=True)
    m = o.model

    def rows(X):
        n = X.shape[0]
        return torch.cat([m.radial(X, *o.nl["pairs"], n), m.angular(X, *o.nl["triples"], n)], 1)

    J = torch.autograd.functional.jacobian(rows, X).numpy()
    for ia, a in enumerate(g["ani1_deri_atoms"]):
        np.testing.assert_allclose(J[a].reshape(J.shape[1], -1), g["ani1_deri"][ia], rtol=0, atol=1e-11)


@pytest.mark.parametrize("act", ["sigmoid_with_param", "tanh"])
def test_forces_central_fd(golden_loader, act):
    g = golden_loader("water60")
    o = _water_oracle(g, act)
    out = o.terms(g["x"])
    atoms = [0, 1, 2, 17, 44]
    fd = o.fd_gradient(g["x"], atoms, h=1e-4)
    np.testing.assert_allclose(out["gradient"][atoms], fd, rtol=0, atol=1e-7)


def test_periodic_oracle_conservative_force_fd(golden_loader):
    g = golden_loader("waterbox192")
    p = dict(PARAMS)
    p["NeuronType"] = "tanh"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    model = orc.Model([1, 8], W, params=p)
    o = orc.PeriodicOracle(model, g["x"], g["Z"], g["lattice"], ree_cut=6.0)
    out = o.terms(g["x"])
    x = g["x"].copy()
    h = 1e-4
    for a in (0, 5):
        for c in range(3):
            xp = x.copy(); xp[a, c] += h
            xm = x.copy(); xm[a, c] -= h
            ep = o.terms(xp, grad=False)["Etotal"].sum()
            em = o.terms(xm, grad=False)["Etotal"].sum()
            assert abs((ep - em) / (2 * h) - out["gradient"][a, c]) < 1e-7
