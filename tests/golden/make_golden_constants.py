"""Golden constants of the reference: units, element tables, PARAMS defaults
and the DSF shift/slope of the electrostatic embedding.

* ``PhysicalData.py`` (numpy only) is imported unchanged: BOHRPERA,
  KJPERHARTREE, JOULEPERHARTREE, IDEALGASR, ATOMICMASSES, C6_coff,
  atomic_vdw_radius.
* ``TMParams.py`` imports TensorFlow at module level, so its defaults are read
  from the source: every ``self["key"] = <literal>`` of ``TMParams.__init__``.
* ``Util.py`` creates directories and probes optional packages when imported,
  so its ``DSF`` and ``DSF_Gradient`` definitions (Util.py:172-192) are taken
  from the file's syntax tree and run unchanged in a namespace with ``math``
  and ``scipy``. They are evaluated on a grid of radii and at the elu radius,
  as ``MolInstance_DirectBP_EE_SymFunction.__init__`` calls them
  (TFBehlerParinelloSymEE.py:727-729).

Writes ``tests/golden/constants.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_constants.py
"""
from __future__ import annotations

import ast
import importlib.util
import json
import math
import os
import sys

import numpy as np
import scipy.special

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "TensorMol")


def load_physical_data():
    spec = importlib.util.spec_from_file_location("tm_ref_physicaldata",
                                                  os.path.join(REF, "PhysicalData.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def tmparams_defaults():
    tree = ast.parse(open(os.path.join(REF, "TMParams.py")).read())
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "TMParams")
    init = next(n for n in cls.body if isinstance(n, ast.FunctionDef) and n.name == "__init__")
    out = {}
    for st in ast.walk(init):
        if not (isinstance(st, ast.Assign) and len(st.targets) == 1):
            continue
        t = st.targets[0]
        if not (isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and t.value.id == "self"):
            continue
        try:
            key = ast.literal_eval(t.slice)
            val = ast.literal_eval(st.value)
        except ValueError:
            continue   # computed defaults (arrays, expressions) are left out
        if isinstance(key, str) and isinstance(val, (bool, int, float, str, list, tuple, type(None))):
            out[key] = val
    return out


def util_dsf():
    tree = ast.parse(open(os.path.join(REF, "Util.py")).read())
    defs = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in ("DSF", "DSF_Gradient")]
    ns = {"math": math, "scipy": scipy}
    exec(compile(ast.Module(body=defs, type_ignores=[]), os.path.join(REF, "Util.py"), "exec"), ns)
    return ns["DSF"], ns["DSF_Gradient"]


def main():
    pd = load_physical_data()
    defaults = tmparams_defaults()
    dsf, dsf_grad = util_dsf()
    b = pd.BOHRPERA
    rc = defaults["EECutoffOff"] * b
    alpha = defaults["DSFAlpha"] / b
    r = np.linspace(0.5, 16.0, 64) * b          # bohr, both sides of the cutoff
    out = dict(
        BOHRPERA=pd.BOHRPERA, KJPERHARTREE=pd.KJPERHARTREE, JOULEPERHARTREE=pd.JOULEPERHARTREE,
        IDEALGASR=pd.IDEALGASR, ATOMICMASSES=np.asarray(pd.ATOMICMASSES)[:10],
        C6_coff=np.array([pd.C6_coff[z] for z in range(1, 11)]),
        atomic_vdw_radius=np.array([pd.atomic_vdw_radius[z] for z in range(1, 11)]),
        tmparams=np.array(json.dumps(defaults)),
        dsf_r=r, dsf_rc=rc, dsf_alpha=alpha,
        dsf=np.array([dsf(x, rc, alpha) for x in r]),
        dsf_grad=np.array([dsf_grad(x, rc, alpha) for x in r]),
        elu_shift=dsf(defaults["Elu_Width"] * b, rc, alpha),
        elu_alpha=dsf_grad(defaults["Elu_Width"] * b, rc, alpha),
    )
    path = os.path.join(HERE, "constants.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes;", len(defaults), "PARAMS defaults")


if __name__ == "__main__":
    main()
