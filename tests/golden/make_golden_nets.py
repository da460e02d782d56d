"""Golden energies, charges and dipoles from the reference's own network
graph, run on a numpy implementation of the TF ops.

``MolInstance_DirectBP_EE_SymFunction.energy_inference`` and
``dipole_inference`` (TFNetworks/TFBehlerParinelloSymEE.py:884-1015) and
``SetANI1Param`` (:738-777) are taken from the file's syntax tree and run
unchanged on a stand-in instance. So are the functions they call from
TFDescriptors/RawSymFunc.py (the descriptor set, TFCoulombEluSRDSFLR,
TFVdwPolyLR and helpers) and ``sigmoid_with_param``, ``DSF`` and
``DSF_Gradient`` from Util.py. ``tf`` is the numpy stand-in of
``numpy_tf.py``. The graph is wired as ``EvalPrepare`` wires it
(:826-841): descriptors, then the charge network with neutralisation, dipole
and Coulomb, then the energy network with vdW. It is fed the reference's own
neighbour and Coulomb lists from the water60 and chno6 fixtures, with
keep = 1 and natom = 1/N per molecule. The 192-atom periodic water box goes
through the periodic variants (EvalPrepare_Periodic, :1503-1621, 1671-1703,
and the periodic descriptor and vdW functions of RawSymFunc.py).

For the smooth activation it also stores central differences of the
reference's own total energy at a few atoms (lists held fixed, as
tf.gradients differentiates the graph), which pin the oracle's forces.

The weights are the seeded ``random_weights`` of this package with seeded
random biases (stored here). The reference's graph code looks them up by
its own variable names, and every name that ``weights.tensormol_names``
writes must be looked up, so the naming is checked too.

Writes ``tests/golden/nets.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_nets.py
"""
from __future__ import annotations

import ast
import importlib.util
import math
import os
import sys
import warnings
from math import pi as Pi

import numpy as np
import scipy.special

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "TensorMol")
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import numpy_tf  # noqa: E402
from numpy_tf import constant_tensor, tf  # noqa: E402
from tensormol_gb300 import systems  # noqa: E402
from tensormol_gb300.params import descriptor_width  # noqa: E402
from tensormol_gb300.weights import tensormol_names  # noqa: E402

HIDDEN = [512, 512, 512]
CASES = (("water60", [1, 8], "relu"), ("water60", [1, 8], "sigmoid_with_param"),
         ("chno6", [1, 6, 7, 8], "sigmoid_with_param"))


def take(path, names, ns, cls=None):
    with warnings.catch_warnings():   # escape sequences in the file's docstrings
        warnings.simplefilter("ignore", SyntaxWarning)
        tree = ast.parse(open(path).read())
    body = tree.body
    if cls is not None:
        body = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == cls).body
    defs = [n for n in body if isinstance(n, ast.FunctionDef) and n.name in names]
    assert len(defs) == len(names), names
    exec(compile(ast.Module(body=defs, type_ignores=[]), path, "exec"), ns)


class _Lookups(dict):
    """The weight table, recording which names the graph code reads."""

    def __init__(self, *a):
        super().__init__(*a)
        self.read = set()

    def __contains__(self, k):
        return dict.__contains__(self, k)

    def __getitem__(self, k):
        self.read.add(k)
        return dict.__getitem__(self, k)


class _Instance:
    """What SetANI1Param and the two inference methods read from the model."""

    def __init__(self, eles, act, nmol, maxn, dsf):
        self.eles = list(eles)
        self.eles_pairs = [[a, b] for i, a in enumerate(eles) for b in eles[i:]]   # :679-682
        self.HasANI1PARAMS = False
        self.HiddenLayers = HIDDEN
        self.batch_size, self.MaxNAtoms = nmol, maxn
        self.tf_prec = np.float64
        self.activation_function = act
        self.DSFAlpha, self.elu_alpha, self.elu_shift = dsf

    def _variable_with_weight_decay(self, var_name, var_shape, var_stddev, var_wd):
        w = numpy_tf.VARIABLES[numpy_tf.scoped(var_name)]
        assert w.shape == tuple(var_shape), (numpy_tf.scoped(var_name), w.shape, var_shape)
        return w


def padded(x, Z, off):
    nmol = len(off) - 1
    n = int(np.max(np.diff(off)))
    R = np.zeros((nmol, n, 3))
    Zs = np.zeros((nmol, n), dtype=np.int64)
    for m in range(nmol):
        a, b = off[m], off[m + 1]
        R[m, :b - a] = x[a:b]
        Zs[m, :b - a] = Z[a:b]
    return R, Zs


def periodic_case(ns, pd, dsf, rng, act_name="sigmoid_with_param"):
    """The 192-atom water box as EvalPrepare_Periodic wires it
    (TFBehlerParinelloSymEE.py:1671-1703) and EvalBPDirectEEUpdateSinglePeriodic
    feeds it (TFMolManage.py:1324-1358): the tessellated cell, real atoms first
    (the oracle's tessellate, equal to Lattice.TessLattice bit for bit), the
    periodic lists of the waterbox192 fixture, natom = 1/nreal."""
    from oracle import reference as orc
    b = pd.BOHRPERA
    eles = [1, 8]
    g = np.load(os.path.join(HERE, "waterbox192.npz"))
    nreal = len(g["Z"])
    xt = orc.tessellate(g["x"], g["lattice"], 1)
    R = xt[None]
    Zs = np.tile(g["Z"], xt.shape[0] // nreal)[None].astype(np.int64)
    W = systems.random_weights(eles, descriptor_width(len(eles)), hidden=tuple(HIDDEN), seed=7)
    biases = []
    for net in ("E", "Q"):
        for e in eles:
            for li, (w, bb) in enumerate(W[net][e]):
                nb = rng.normal(0.0, 0.05, size=bb.shape)
                W[net][e][li] = (w, nb)
                biases.append(nb)
    table = _Lookups(tensormol_names(W))
    numpy_tf.VARIABLES = table
    inst = _Instance(eles, ns[act_name], 1, R.shape[1], dsf)
    inst.nreal = nreal
    ns["SetANI1Param"](inst)
    Ele = constant_tensor(np.asarray(eles).reshape(len(eles), 1), np.int64)
    Elep = constant_tensor(np.asarray(inst.eles_pairs), np.int64)
    lists = [g[key].astype(np.int64) for key in ("RadpEle", "AngtEle", "mil_j", "mil_jk")]
    c6 = np.array([pd.C6_coff[e] * (b * 10.0) ** 6.0 / pd.JOULEPERHARTREE for e in eles])
    rvdw = np.array([pd.atomic_vdw_radius[e] * b for e in eles])
    reep5 = g["rad_eep_e1e2"].astype(np.int64)
    keep = np.ones(len(HIDDEN) + 1)
    natom = np.array([1.0 / nreal])

    def graph(RR):
        sym, idx = ns["TFSymSet_Scattered_Linear_WithEle_Periodic"](
            RR, Zs, Ele, inst.SFPr2, inst.Rr_cut, Elep, inst.SFPa2, inst.zeta, inst.eta, inst.Ra_cut, *lists,
            nreal)
        ecc, dipole, charge_all, _ = ns["dipole_inference_periodic"](inst, sym, idx, RR, natom, 4.6, 15.0,
                                                                     reep5[:, :3], True, keep)
        etot, ebp, evdw, _, ebp_atom = ns["energy_inference_periodic"](inst, sym, idx, ecc, RR, Zs, Ele, c6,
                                                                       rvdw, reep5, 0.0, 15.0, keep)
        return etot, ebp, ecc, evdw, dipole, charge_all, ebp_atom

    etot, ebp, ecc, evdw, dipole, charge_all, ebp_atom = graph(R)
    assert table.read == set(table), sorted(set(table) - table.read)
    # the reference's returned periodic force is tf.gradients with respect to
    # the real rows of the tessellated input, images held fixed
    # (TFMolManage.py:1353): central differences moving those rows alone
    fd_atoms = np.array([0, 1, 2, 100])
    fd = np.zeros((len(fd_atoms), 3))
    for ai, a in enumerate(fd_atoms):
        for c in range(3):
            Rp = R.copy(); Rp[0, a, c] += 1e-4
            Rm = R.copy(); Rm[0, a, c] -= 1e-4
            fd[ai, c] = (np.sum(graph(Rp)[0]) - np.sum(graph(Rm)[0])) / 2e-4
    print("waterbox192", act_name, "Etotal", np.asarray(etot))
    return {"p_act": np.array(act_name), "p_biases": np.concatenate([v.ravel() for v in biases]),
            "p_Etotal": etot, "p_Ebp": ebp, "p_Ecc": ecc, "p_Evdw": evdw, "p_dipole": dipole,
            "p_charge": np.asarray(charge_all)[0, :nreal], "p_Ebp_atom": np.asarray(ebp_atom)[0],
            "p_fd_atoms": fd_atoms, "p_fd_grad_real_rows": fd}


def main():
    spec = importlib.util.spec_from_file_location("tm_ref_physicaldata", os.path.join(REF, "PhysicalData.py"))
    pd = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pd)
    b = pd.BOHRPERA
    params = {"AN1_r_Rc": 4.6, "AN1_a_Rc": 3.1, "AN1_eta": 4.0, "AN1_zeta": 8.0, "AN1_num_r_Rs": 32,
              "AN1_num_a_Rs": 8, "AN1_num_a_As": 8, "EECutoffOff": 15.0, "Poly_Width": 4.6,
              "sigmoid_alpha": 100.0}
    ns = {"tf": tf, "np": np, "math": math, "scipy": scipy, "Pi": Pi, "PARAMS": params, "BOHRPERA": b,
          "print": lambda *a, **k: None}
    take(os.path.join(REF, "TFDescriptors", "RawSymFunc.py"),
         ("DifferenceVectorsLinear", "AllSinglesSet", "AllDoublesSet", "TFSymRSet_Linear_WithEle_Release",
          "TFSymASet_Linear_WithEle", "TFSymSet_Scattered_Linear_WithEle_Release",
          "TFCoulombEluSRDSFLR", "TFVdwPolyLR", "TFSymRSet_Linear_WithElePeriodic",
          "TFSymASet_Linear_WithElePeriodic", "TFSymSet_Scattered_Linear_WithEle_Periodic",
          "TFVdwPolyLRWithEle"), ns)
    take(os.path.join(REF, "Util.py"), ("DSF", "DSF_Gradient", "sigmoid_with_param"), ns)
    take(os.path.join(REF, "TFNetworks", "TFBehlerParinelloSymEE.py"),
         ("SetANI1Param", "energy_inference", "dipole_inference", "energy_inference_periodic",
          "dipole_inference_periodic"), ns,
         cls="MolInstance_DirectBP_EE_SymFunction")
    elu_w, dsf_alpha = 4.6, 0.18
    dsf = (dsf_alpha, ns["DSF_Gradient"](elu_w * b, 15.0 * b, dsf_alpha / b),
           ns["DSF"](elu_w * b, 15.0 * b, dsf_alpha / b))
    rng = np.random.default_rng(41)
    out = {}
    for k, (case, eles, act) in enumerate(CASES):
        g = np.load(os.path.join(HERE, case + ".npz"))
        x, Z, off = g["x"], g["Z"], g["offsets"]
        R0, Zs = padded(x, Z, off)
        nmol, maxn = R0.shape[0], R0.shape[1]
        W = systems.random_weights(eles, descriptor_width(len(eles)), hidden=tuple(HIDDEN), seed=7)
        biases = []
        for net in ("E", "Q"):
            for e in eles:
                for li, (w, bb) in enumerate(W[net][e]):
                    nb = rng.normal(0.0, 0.05, size=bb.shape)
                    W[net][e][li] = (w, nb)
                    biases.append(nb)
        table = _Lookups(tensormol_names(W))
        numpy_tf.VARIABLES = table
        inst = _Instance(eles, tf.nn.relu if act == "relu" else ns["sigmoid_with_param"], nmol, maxn, dsf)
        ns["SetANI1Param"](inst)
        Ele = constant_tensor(np.asarray(eles).reshape(len(eles), 1), np.int64)
        Elep = constant_tensor(np.asarray(inst.eles_pairs), np.int64)
        lists = [g[key].astype(np.int64) for key in ("RadpEle", "AngtEle", "mil_j", "mil_jk")]
        c6 = np.array([pd.C6_coff[e] * (b * 10.0) ** 6.0 / pd.JOULEPERHARTREE for e in eles])   # :719-723
        rvdw = np.array([pd.atomic_vdw_radius[e] * b for e in eles])
        reep = g["rad_eep"].astype(np.int64)
        keep = np.ones(len(HIDDEN) + 1)
        natom = 1.0 / np.diff(off).astype(np.float64)

        def graph(xx):
            R, _ = padded(xx, Z, off)
            sym, idx = ns["TFSymSet_Scattered_Linear_WithEle_Release"](
                R, Zs, Ele, inst.SFPr2, inst.Rr_cut, Elep, inst.SFPa2, inst.zeta, inst.eta, inst.Ra_cut, *lists)
            ecc, dipole, charge, _ = ns["dipole_inference"](inst, sym, idx, R, natom, elu_w, 15.0, reep, True,
                                                            keep)
            etot, ebp, evdw, _, ebp_atom = ns["energy_inference"](inst, sym, idx, ecc, R, Zs, Ele, c6, rvdw,
                                                                  reep, 0.0, 15.0, keep)
            return etot, ebp, ecc, evdw, dipole, charge, ebp_atom

        etot, ebp, ecc, evdw, dipole, charge, ebp_atom = graph(x)
        assert table.read == set(table), sorted(set(table) - table.read)
        real = np.concatenate([np.arange(off[m + 1] - off[m]) + m * maxn for m in range(nmol)])
        tag = "c%d" % k
        out.update({tag + "_case": np.array(case), tag + "_act": np.array(act),
                    tag + "_biases": np.concatenate([v.ravel() for v in biases]),
                    tag + "_Etotal": etot, tag + "_Ebp": ebp, tag + "_Ecc": ecc, tag + "_Evdw": evdw,
                    tag + "_dipole": dipole, tag + "_charge": np.asarray(charge).ravel()[real],
                    tag + "_Ebp_atom": np.asarray(ebp_atom).ravel()[real]})
        if act != "relu":
            # central differences of the reference's own total energy, lists
            # held fixed (what tf.gradients differentiates), h = 1e-4 A
            fd_atoms = np.array([0, 1, 2, 17, 44]) if case == "water60" else np.array([0, 5, 40, 120])
            fd = np.zeros((len(fd_atoms), 3))
            for ai, a in enumerate(fd_atoms):
                for c in range(3):
                    xp = x.copy(); xp[a, c] += 1e-4
                    xm = x.copy(); xm[a, c] -= 1e-4
                    fd[ai, c] = (np.sum(graph(xp)[0]) - np.sum(graph(xm)[0])) / 2e-4
            out.update({tag + "_fd_atoms": fd_atoms, tag + "_fd_grad": fd})
        print(case, act, "Etotal", np.asarray(etot)[:3])
    out.update(periodic_case(ns, pd, dsf, rng))
    path = os.path.join(HERE, "nets.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
