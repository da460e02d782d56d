"""Golden XYZ text from the reference's own ``Mol`` formatting.

``Containers/Mol.py`` cannot be imported under numpy 2 (a default argument
uses ``np.float``), so ``Mol.__str__`` and ``Mol.PropertyString``
(Mol.py:286-345), the text ``WriteXYZfile`` writes, are taken from the file's
syntax tree and run unchanged. They are applied to a stand-in object holding
atoms, coordinates and properties, with the element table ``atoi`` of the
reference's own ``PhysicalData.py``. Cases: the 60-atom water cluster
without and with properties, and a CHNO molecule.

Writes ``tests/golden/xyz.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_xyz.py
"""
from __future__ import annotations

import ast
import importlib.util
import os
import sys

import numpy as np

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "TensorMol")
sys.path.insert(0, REPO)

from tensormol_gb300 import systems  # noqa: E402


def load_mol_text():
    spec = importlib.util.spec_from_file_location("tm_ref_physicaldata",
                                                  os.path.join(REF, "PhysicalData.py"))
    pd = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pd)
    path = os.path.join(REF, "Containers", "Mol.py")
    tree = ast.parse(open(path).read())
    mol = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "Mol")
    defs = [n for n in mol.body if isinstance(n, ast.FunctionDef) and n.name in ("__str__", "PropertyString")]
    ns = {"np": np, "atoi": pd.atoi}
    exec(compile(ast.Module(body=defs, type_ignores=[]), path, "exec"), ns)
    return ns["__str__"], ns["PropertyString"]


class _Stand:
    """Holds what the two methods read."""

    def __init__(self, atoms, coords, properties, prop_fn):
        self.atoms = np.asarray(atoms, dtype=np.uint8)
        self.coords = np.asarray(coords, dtype=np.float64)
        self.properties = dict(properties)
        self._prop_fn = prop_fn

    def PropertyString(self):
        return self._prop_fn(self)


def main():
    to_str, prop = load_mol_text()
    w = systems.water_cluster_60(seed=0)
    b = systems.chno_batch(nmol=2, seed=3)
    xb, zb = b.molecule(0)
    cases = {
        "water60": (w.Z, w.x, {}, False),
        "water60_props": (w.Z, w.x, {"energy": -76.123456789, "name": "w60"}, True),
        "chno0": (zb, xb, {}, False),
    }
    out = {}
    for name, (z, x, props, wprop) in cases.items():
        s = _Stand(z, x, props, prop)
        out[name + "_Z"] = np.asarray(z)
        out[name + "_x"] = np.asarray(x)
        out[name + "_props"] = np.array(repr(props))
        out[name + "_wprop"] = np.array(wprop)
        out[name + "_text"] = np.array(to_str(s, wprop))
    path = os.path.join(HERE, "xyz.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
