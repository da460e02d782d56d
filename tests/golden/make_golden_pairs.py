"""Golden molecular Coulomb and vdW energies from the reference's own
TensorFlow-graph functions, run on a numpy implementation of the TF ops.

``TFCoulombEluSRDSFLR`` and ``TFVdwPolyLR`` (TFDescriptors/RawSymFunc.py:1307-1414)
and the helpers they call, ``DifferenceVectorsLinear`` (:123-133) and
``AllDoublesSet`` (:63-78), are taken from the file's syntax tree and run
unchanged. TensorFlow is absent, so ``tf`` in their namespace is the numpy
stand-in of ``numpy_tf.py`` beside this file. Arguments follow the reference's calls
(TFBehlerParinelloSymEE.py:941, 1012):
* positions in bohr, as a padded [nmol, maxnatom, 3] tensor;
* charges as [nmol, maxnatom];
* the Coulomb pair list (mol, i, j) the reference's ``buildPairs`` made,
  stored in the water60 and chno6 fixtures;
* C6 and vdW radii converted as the model constructor does
  (TFBehlerParinelloSymEE.py:719-723), from the reference's own
  PhysicalData.py;
* the elu shift and slope from its own ``DSF`` / ``DSF_Gradient`` (Util.py).
Charges are seeded values, not network outputs: the functions do not care
where the charges come from.

Writes ``tests/golden/pairs.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_pairs.py
"""
from __future__ import annotations

import ast
import importlib.util
import math
import os
import sys
import warnings

import numpy as np
import scipy.special

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "TensorMol")
sys.path.insert(0, HERE)

from numpy_tf import tf as _NumpyTF  # noqa: E402


def load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def reference_functions(params, pd):
    def take(path, names, ns):
        with warnings.catch_warnings():   # escape sequences in the file's docstrings
            warnings.simplefilter("ignore", SyntaxWarning)
            tree = ast.parse(open(path).read())
        defs = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
        assert len(defs) == len(names), names
        exec(compile(ast.Module(body=defs, type_ignores=[]), path, "exec"), ns)

    ns = {"tf": _NumpyTF, "np": np, "PARAMS": params, "BOHRPERA": pd.BOHRPERA}
    take(os.path.join(REF, "TFDescriptors", "RawSymFunc.py"),
         ("DifferenceVectorsLinear", "AllDoublesSet", "TFCoulombEluSRDSFLR", "TFVdwPolyLR"), ns)
    util = {"math": math, "scipy": scipy}
    take(os.path.join(REF, "Util.py"), ("DSF", "DSF_Gradient"), util)
    return ns, util


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


def main():
    pd = load("tm_ref_physicaldata", os.path.join(REF, "PhysicalData.py"))
    params = {"EECutoffOff": 15.0, "Poly_Width": 4.6}
    ns, util = reference_functions(params, pd)
    b = pd.BOHRPERA
    elu_width, dsf_alpha, ee_on = 4.6, 0.18, 0.0
    elu_shift = util["DSF"](elu_width * b, params["EECutoffOff"] * b, dsf_alpha / b)
    elu_alpha = util["DSF_Gradient"](elu_width * b, params["EECutoffOff"] * b, dsf_alpha / b)
    out = {}
    rng = np.random.default_rng(31)
    for case, eles in (("water60", [1, 8]), ("chno6", [1, 6, 7, 8])):
        g = np.load(os.path.join(HERE, case + ".npz"))
        x, Z, off = g["x"], g["Z"], g["offsets"]
        R, Zs = padded(x, Z, off)
        q = rng.normal(0.0, 0.4, size=len(Z))
        Qs, _ = padded(np.repeat(q[:, None], 3, 1), Z, off)
        Qs = Qs[:, :, 0]
        pairs = g["rad_eep"].astype(np.int64)
        c6 = np.array([pd.C6_coff[e] * (b * 10.0) ** 6.0 / pd.JOULEPERHARTREE for e in eles])
        rvdw = np.array([pd.atomic_vdw_radius[e] * b for e in eles])
        Rb = R * b
        ecc = ns["TFCoulombEluSRDSFLR"](Rb, Qs, elu_width * b, pairs, dsf_alpha, elu_alpha, elu_shift)
        evdw = ns["TFVdwPolyLR"](Rb, Zs, np.array(eles, dtype=np.int64), c6, rvdw, ee_on * b, pairs)
        out[case + "_q"] = q
        out[case + "_Ecc"] = np.asarray(ecc)
        out[case + "_Evdw"] = np.asarray(evdw)
        print(case, "Ecc", out[case + "_Ecc"][:3], "Evdw", out[case + "_Evdw"][:3])
    path = os.path.join(HERE, "pairs.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
