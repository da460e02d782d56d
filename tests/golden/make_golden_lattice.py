"""Golden periodic images and wraps from the reference's own ``Lattice``.

``ForceModifiers/Periodic.py`` imports the whole package (neighbour lists,
electrostatics, MD) at module level, so its ``Lattice`` class
(Periodic.py:12-181) is taken from the file's syntax tree and run unchanged,
with numpy, ``MatrixPower`` from the reference's own
``Math/LinearOperations.py`` (numpy only, imported unchanged) and ``MolEmb``
built from the reference's source by ``oracle/build_ref.sh``.

Cases:
* ``TessLattice`` of the first 24 atoms of the 192-atom water box (cubic
  cell, range below the cell's diameter: one shell, 27 images) and of 6
  atoms in a small orthorhombic cell whose range needs three shells
  (343 images);
* ``ModuloLattice`` of points up to two cells outside the cell, for an
  orthorhombic and a triclinic lattice.

Writes ``tests/golden/lattice.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_lattice.py
"""
from __future__ import annotations

import ast
import importlib.util
import os
import subprocess
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


def load_lattice_class():
    spec = importlib.util.spec_from_file_location(
        "tm_ref_linearoperations", os.path.join(REF, "Math", "LinearOperations.py"))
    linops = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(linops)
    path = os.path.join(REF, "ForceModifiers", "Periodic.py")
    tree = ast.parse(open(path).read())
    cls = [n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "Lattice"]
    subprocess.check_call([os.path.join(REPO, "oracle", "build_ref.sh")])
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    import MolEmb
    ns = {"np": np, "MatrixPower": linops.MatrixPower, "MolEmb": MolEmb}
    exec(compile(ast.Module(body=cls, type_ignores=[]), path, "exec"), ns)
    return ns["Lattice"]


def main():
    Lattice = load_lattice_class()
    box = np.load(os.path.join(HERE, "waterbox192.npz"))
    out = {}

    # cubic water box: one shell
    lat_a = np.array(box["lattice"], dtype=np.float64)
    x_a = np.array(box["x"][:24], dtype=np.float64)
    z_a = np.array(box["Z"][:24], dtype=np.uint8)
    L = Lattice(lat_a)
    rng_a = 0.9 * L.latticeMinDiameter
    at, xt = L.TessLattice(z_a, x_a, rng_a)
    out.update(tess_a_lattice=lat_a, tess_a_x=x_a, tess_a_rng=rng_a, tess_a_ntess=L.ntess,
               tess_a_coords=xt, tess_a_atoms=at)

    # small orthorhombic cell, 15 A range: three shells
    rng = np.random.default_rng(21)
    lat_b = np.diag([7.1, 8.3, 9.7])
    x_b = rng.uniform(0.0, 1.0, size=(6, 3)) @ lat_b
    z_b = np.array([8, 1, 1, 6, 7, 1], dtype=np.uint8)
    L = Lattice(lat_b)
    at, xt = L.TessLattice(z_b, x_b, 15.0)
    out.update(tess_b_lattice=lat_b, tess_b_x=x_b, tess_b_rng=15.0, tess_b_ntess=L.ntess,
               tess_b_coords=xt, tess_b_atoms=at)

    # wraps into the cell
    lat_t = np.array([[9.0, 0.0, 0.0], [2.5, 8.0, 0.0], [1.0, 1.5, 10.0]])
    for name, lat in (("orth", lat_b), ("tric", lat_t)):
        pts = rng.uniform(-2.0, 3.0, size=(64, 3)) @ lat
        out["mod_%s_lattice" % name] = lat
        out["mod_%s_in" % name] = pts
        out["mod_%s_out" % name] = Lattice(lat).ModuloLattice(pts)

    path = os.path.join(HERE, "lattice.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes; ntess", out["tess_a_ntess"], out["tess_b_ntess"])


if __name__ == "__main__":
    main()
