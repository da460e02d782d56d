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


def test_ragged_batch_equals_molecules_alone():
    """Molecules of 1, 2, 3 and 60 atoms in one batch, all overlapping in
    space, give the same energies and forces as each molecule evaluated
    alone: no pair, triple or Coulomb term crosses a molecule boundary. A
    lone atom has no neighbours and feels no force; a two-atom molecule has
    pairs but no triples. The GPU ragged-batch test compares against this
    batched oracle, so the batching itself is checked here."""
    w = systems.water_cluster_60(seed=0)
    xs = [np.zeros((1, 3)), np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.97]]),
          np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]]), w.x]
    Zs = [np.array([8]), np.array([8, 1]), np.array([8, 1, 1]), w.Z]
    x = np.concatenate(xs)
    Z = np.concatenate(Zs).astype(np.int32)
    off = np.concatenate([[0], np.cumsum([len(z) for z in Zs])]).astype(np.int64)
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    model = orc.Model([1, 8], W, params=p)
    batch = orc.OpenSystemOracle(model, x, Z, off)
    out = batch.terms(x)
    assert not np.any(batch.P[:, 0] == 0) and not np.any(batch.T[:, 0] == 0)   # lone atom
    assert np.any(batch.P[:, 0] == 1) and not np.any(batch.T[:, 0] == 1)       # pair only
    assert np.all(out["force"][0] == 0.0)
    for m, (xm, Zm) in enumerate(zip(xs, Zs)):
        alone = orc.OpenSystemOracle(model, xm, Zm, np.array([0, len(Zm)])).terms(xm)
        for key in ("Etotal", "Ebp", "Ecc", "Evdw"):
            np.testing.assert_allclose(out[key][m], alone[key][0], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(out["force"][off[m]:off[m + 1]], alone["force"], rtol=0, atol=1e-8)


def test_periodic_descriptor_matches_molemb(golden_loader):
    """Descriptor rows of the 192 real atoms of the periodic box against
    MolEmb's Make_ANI1_Sym over the tessellated cell (real atoms first)."""
    g = golden_loader("waterbox192")
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    model = orc.Model([1, 8], W)
    o = orc.PeriodicOracle(model, g["x"], g["Z"], g["lattice"], ree_cut=float(g["ree_cut"]))
    out = o.terms(g["x"], grad=False)
    # MolEmb writes pi as 3.14159265358979, the TF graph as 3.14159265359
    np.testing.assert_allclose(out["G"], g["ani1_G"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("case", ["a", "b"])
def test_tessellation_matches_lattice(golden_loader, case):
    """Image coordinates and order against the reference's Lattice.TessLattice
    (one shell for the water box, three for a small orthorhombic cell):
    real atoms first, then the images in (i, j, k) raster order, each
    coordinate x + i a0 + j a1 + k a2 in FP64, bit for bit."""
    g = golden_loader("lattice")
    x, lat = g["tess_%s_x" % case], g["tess_%s_lattice" % case]
    ntess = int(g["tess_%s_ntess" % case])
    xt = orc.tessellate(x, lat, ntess)
    assert np.array_equal(xt, g["tess_%s_coords" % case])
    shifts = orc.image_shift_table(lat, ntess)
    assert shifts.shape[0] * x.shape[0] == g["tess_%s_atoms" % case].shape[0]


@pytest.mark.parametrize("name", ["orth", "tric"])
def test_modulo_lattice_matches_reference(golden_loader, name):
    """Wrap into the cell against Lattice.ModuloLattice. The oracle uses a
    plain inverse, the reference an SVD matrix power, so the two agree to
    rounding, not bit for bit."""
    g = golden_loader("lattice")
    lat = g["mod_%s_lattice" % name]
    out = orc.modulo_lattice(g["mod_%s_in" % name], lat)
    np.testing.assert_allclose(out, g["mod_%s_out" % name], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case,eles", [("water60", [1, 8]), ("chno6", [1, 6, 7, 8])])
def test_pair_energies_match_reference_functions(golden_loader, case, eles):
    """Molecular Coulomb (DSF/elu) and vdW energies of the oracle against the
    reference's own TFCoulombEluSRDSFLR and TFVdwPolyLR, run on a numpy
    implementation of the TF ops. Both use the same seeded charges and the
    reference's own Coulomb pair list (tests/golden/make_golden_pairs.py)."""
    import torch
    from tensormol_gb300.params import BOHRPERA
    g = golden_loader(case)
    gp = golden_loader("pairs")
    x, Z, off = g["x"], g["Z"], g["offsets"]
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    model = orc.Model(eles, W)
    pairs = g["rad_eep"].astype(np.int64)
    ei = torch.as_tensor(off[pairs[:, 0]] + pairs[:, 1])
    ej = torch.as_tensor(off[pairs[:, 0]] + pairs[:, 2])
    mol = torch.as_tensor(pairs[:, 0])
    nmol = len(off) - 1
    Xb = torch.as_tensor(x * BOHRPERA)
    q = torch.as_tensor(gp[case + "_q"])
    eidx = torch.as_tensor([eles.index(int(z)) for z in Z])
    ecc = torch.zeros(nmol, dtype=torch.float64).index_add(0, mol, model.coulomb(Xb, q, ei, ej))
    evdw = torch.zeros(nmol, dtype=torch.float64).index_add(0, mol, model.vdw(Xb, eidx, ei, ej))
    np.testing.assert_allclose(ecc.numpy(), gp[case + "_Ecc"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(evdw.numpy(), gp[case + "_Evdw"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("case,eles", [("water60", [1, 8]), ("chno6", [1, 6, 7, 8])])
def test_descriptors_match_reference_tf_functions(golden_loader, case, eles):
    """Descriptor rows and element partition against the reference's own
    TFSymSet_Scattered_Linear_WithEle_Release (radial + angular TF functions,
    run on a numpy implementation of the TF ops, fed the reference's own
    neighbour lists; tests/golden/make_golden_desc.py). Each element's rows
    come in (molecule, atom) order. The library's element-sorted network rows
    use the same order. The values agree to rounding: same formulas, same
    pi literal and clamps."""
    g = golden_loader(case)
    gd = golden_loader("desc")
    x, Z, off = g["x"], g["Z"], g["offsets"]
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    G = orc.OpenSystemOracle(orc.Model(eles, W), x, Z, off).terms(x, grad=False)["G"]
    maxn = int(gd[case + "_maxn"])
    for e, z in enumerate(eles):
        idx = gd["%s_idx%d" % (case, e)]
        atoms = off[idx[:, 0]] + (idx[:, 1] - idx[:, 0] * maxn)
        assert np.array_equal(atoms, np.flatnonzero(Z == z))
        ref = gd["%s_G%d" % (case, e)]
        np.testing.assert_allclose(G[atoms[:len(ref)]], ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("tag", ["c0", "c1", "c2"])
def test_energy_terms_match_reference_graph(golden_loader, tag):
    """Total, network, Coulomb and vdW energies, neutralised charges, dipoles
    and per-atom network energies. They are compared with the reference's
    own graph (SetANI1Param, the descriptor set, dipole_inference and
    energy_inference), run on a numpy implementation of the TF ops and fed
    its own neighbour and Coulomb lists (tests/golden/make_golden_nets.py).
    Cases: 60-atom water with relu and with sigmoid_with_param, six CHNO
    molecules with sigmoid_with_param. The weights are seeded with random
    biases, and the reference's graph reads them by its own variable names."""
    gn = golden_loader("nets")
    case, act = str(gn[tag + "_case"]), str(gn[tag + "_act"])
    eles = [1, 8] if case == "water60" else [1, 6, 7, 8]
    g = golden_loader(case)
    x, Z, off = g["x"], g["Z"], g["offsets"]
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    flat, k = gn[tag + "_biases"], 0
    for net in ("E", "Q"):
        for e in eles:
            for li, (w, b) in enumerate(W[net][e]):
                W[net][e][li] = (w, flat[k:k + b.size].reshape(b.shape))
                k += b.size
    assert k == flat.size
    p = dict(PARAMS)
    p["NeuronType"] = act
    out = orc.OpenSystemOracle(orc.Model(eles, W, params=p), x, Z, off).terms(x, grad=False)
    for key in ("Etotal", "Ebp", "Ecc", "Evdw"):
        np.testing.assert_allclose(out[key], gn[tag + "_" + key], rtol=1e-12, atol=1e-14, err_msg=key)
    np.testing.assert_allclose(out["dipole"], gn[tag + "_dipole"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(out["charge"], gn[tag + "_charge"], rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(out["Ebp_atom"], gn[tag + "_Ebp_atom"], rtol=1e-11, atol=1e-14)


def test_periodic_energy_terms_match_reference_graph(golden_loader):
    """The periodic box: the oracle's per-cell Etotal, Ebp, Ecc, Evdw,
    charges and dipole against the reference's own periodic graph
    (TFSymSet_Scattered_Linear_WithEle_Periodic, dipole_inference_periodic,
    energy_inference_periodic, TFVdwPolyLRWithEle; halved pair sums) on the
    tessellated cell and its own periodic lists."""
    gn = golden_loader("nets")
    g = golden_loader("waterbox192")
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    flat, k = gn["p_biases"], 0
    for net in ("E", "Q"):
        for e in eles:
            for li, (w, b) in enumerate(W[net][e]):
                W[net][e][li] = (w, flat[k:k + b.size].reshape(b.shape))
                k += b.size
    p = dict(PARAMS)
    p["NeuronType"] = str(gn["p_act"])
    o = orc.PeriodicOracle(orc.Model(eles, W, params=p), g["x"], g["Z"], g["lattice"],
                           ree_cut=float(g["ree_cut"]))
    out = o.terms(g["x"], grad=False)
    for key in ("Etotal", "Ebp", "Ecc", "Evdw"):
        np.testing.assert_allclose(out[key], gn["p_" + key], rtol=1e-12, atol=1e-14, err_msg=key)
    np.testing.assert_allclose(out["dipole"], gn["p_dipole"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(out["charge"], gn["p_charge"], rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(out["Ebp_atom"], gn["p_Ebp_atom"], rtol=1e-11, atol=1e-14)


@pytest.mark.parametrize("tag", ["c1", "c2"])
def test_forces_match_reference_energy_differences(golden_loader, tag):
    """The oracle's autograd gradient (the force before the -JOULEPERHARTREE
    scale) against central differences of the reference's own total energy
    graph (tests/golden/make_golden_nets.py; lists held fixed, h = 1e-4 A)
    for water and CHNO molecules with the smooth activation."""
    gn = golden_loader("nets")
    case, act = str(gn[tag + "_case"]), str(gn[tag + "_act"])
    eles = [1, 8] if case == "water60" else [1, 6, 7, 8]
    g = golden_loader(case)
    x, Z, off = g["x"], g["Z"], g["offsets"]
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    flat, k = gn[tag + "_biases"], 0
    for net in ("E", "Q"):
        for e in eles:
            for li, (w, b) in enumerate(W[net][e]):
                W[net][e][li] = (w, flat[k:k + b.size].reshape(b.shape))
                k += b.size
    p = dict(PARAMS)
    p["NeuronType"] = act
    out = orc.OpenSystemOracle(orc.Model(eles, W, params=p), x, Z, off).terms(x)
    atoms = gn[tag + "_fd_atoms"]
    np.testing.assert_allclose(out["gradient"][atoms], gn[tag + "_fd_grad"], rtol=0, atol=1e-7)


def test_periodic_reference_force_matches_reference_energy_differences(golden_loader):
    """The reference's returned periodic force is the gradient with respect
    to the real rows of the tessellated input, images held fixed
    (TFMolManage.py:1353). The oracle's force_ref, which
    TM_F_REFERENCE_PERIODIC_FORCE reproduces on the GPU, must match central
    differences of the reference's own periodic energy graph that move only
    those rows. The conservative force, images moving with their atoms, is a
    different quantity."""
    from tensormol_gb300.params import JOULEPERHARTREE
    gn = golden_loader("nets")
    g = golden_loader("waterbox192")
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    flat, k = gn["p_biases"], 0
    for net in ("E", "Q"):
        for e in eles:
            for li, (w, b) in enumerate(W[net][e]):
                W[net][e][li] = (w, flat[k:k + b.size].reshape(b.shape))
                k += b.size
    p = dict(PARAMS)
    p["NeuronType"] = str(gn["p_act"])
    o = orc.PeriodicOracle(orc.Model(eles, W, params=p), g["x"], g["Z"], g["lattice"],
                           ree_cut=float(g["ree_cut"]))
    out = o.terms(g["x"])
    atoms = gn["p_fd_atoms"]
    grad_ref = -out["force_ref"][atoms] / JOULEPERHARTREE
    fd = gn["p_fd_grad_real_rows"]
    np.testing.assert_allclose(grad_ref, fd, rtol=0, atol=1e-7)
    assert np.abs(out["gradient"][atoms] - fd).max() > 1e-4
