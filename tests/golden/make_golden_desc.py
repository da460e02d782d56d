"""Golden descriptor rows from the reference's own TensorFlow-graph
descriptor functions, run on a numpy implementation of the TF ops.

``TFSymSet_Scattered_Linear_WithEle_Release`` (TFDescriptors/RawSymFunc.py:2267-2309)
and what it calls, ``TFSymRSet_Linear_WithEle_Release`` (:1757-1810),
``TFSymASet_Linear_WithEle`` (:868-963), ``DifferenceVectorsLinear``
(:123-133) and ``AllSinglesSet`` (:80-93), are taken from the file's syntax
tree and run unchanged, with ``tf`` the numpy stand-in of ``numpy_tf.py``.
Their parameter tensors come from the reference's own ``SetANI1Param``
(TFNetworks/TFBehlerParinelloSymEE.py:738-777), run on a stand-in object.
The arguments follow ``EvalPrepare`` (TFBehlerParinelloSymEE.py:826-839):
* padded positions in Angstrom;
* atomic numbers, the element and element-pair tables;
* the cutoffs, zeta and eta;
* the reference's own RadpEle / AngtEle / mil_j / mil_jk lists, stored in
  the water60 and chno6 fixtures.
The outputs are each element's descriptor rows and their (molecule, flat
atom index) pairs, i.e. the element partition the networks consume (for the
CHNO batch, every index pair but only the first 8 rows of each element).

Writes ``tests/golden/desc.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_desc.py
"""
from __future__ import annotations

import ast
import os
import sys
import warnings
from math import pi as Pi

import numpy as np

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "TensorMol")
sys.path.insert(0, HERE)

from numpy_tf import constant_tensor, tf  # noqa: E402

PARAMS = {"AN1_r_Rc": 4.6, "AN1_a_Rc": 3.1, "AN1_eta": 4.0, "AN1_zeta": 8.0,
          "AN1_num_r_Rs": 32, "AN1_num_a_Rs": 8, "AN1_num_a_As": 8}   # TMParams.py:26-35


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


class _Instance:
    """What SetANI1Param reads from and writes to the model instance."""

    def __init__(self, eles):
        self.eles = list(eles)
        self.eles_pairs = [[a, b] for i, a in enumerate(eles) for b in eles[i:]]   # :679-682
        self.HasANI1PARAMS = False


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
    raw = os.path.join(REF, "TFDescriptors", "RawSymFunc.py")
    ns = {"tf": tf, "np": np}
    take(raw, ("DifferenceVectorsLinear", "AllSinglesSet", "TFSymRSet_Linear_WithEle_Release",
               "TFSymASet_Linear_WithEle", "TFSymSet_Scattered_Linear_WithEle_Release"), ns)
    model_ns = {"np": np, "PARAMS": PARAMS, "Pi": Pi, "print": lambda *a, **k: None}
    take(os.path.join(REF, "TFNetworks", "TFBehlerParinelloSymEE.py"), ("SetANI1Param",), model_ns,
         cls="MolInstance_DirectBP_EE_SymFunction")
    out = {}
    for case, eles in (("water60", [1, 8]), ("chno6", [1, 6, 7, 8])):
        g = np.load(os.path.join(HERE, case + ".npz"))
        inst = _Instance(eles)
        model_ns["SetANI1Param"](inst)
        R, Zs = padded(g["x"], g["Z"], g["offsets"])
        Ele = constant_tensor(np.asarray(eles).reshape(len(eles), 1), np.int64)
        Elep = constant_tensor(np.asarray(inst.eles_pairs), np.int64)
        lists = [g[k].astype(np.int64) for k in ("RadpEle", "AngtEle", "mil_j", "mil_jk")]
        sym, idx = ns["TFSymSet_Scattered_Linear_WithEle_Release"](
            R, Zs, Ele, inst.SFPr2, inst.Rr_cut, Elep, inst.SFPa2, inst.zeta, inst.eta, inst.Ra_cut,
            *lists)
        keep = None if case == "water60" else 8    # CHNO: first 8 rows of each element
        for e, (s, i) in enumerate(zip(sym, idx)):
            out["%s_G%d" % (case, e)] = np.asarray(s)[:keep]
            out["%s_idx%d" % (case, e)] = np.asarray(i)
        out[case + "_maxn"] = np.array(R.shape[1])
        print(case, [np.asarray(s).shape for s in sym])
    path = os.path.join(HERE, "desc.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
