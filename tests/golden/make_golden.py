"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference tree is present (``TM_REFERENCE``, or a ``reference``
directory beside the repository checkout; see ``refpath.py``); the resulting .npz files are committed and travel with the
tests, so nothing at test time reads the reference tree.

What is produced, per case (seeded inputs from ``tensormol_gb300.systems``):

* neighbour data from the reference's ``ForceModifiers/Neighbors.py``, imported
  unchanged (``TensorMol.Util`` stubbed with numpy and a no-op timer), driving
  ``MolEmb`` built from ``C_API/MolEmb.cpp`` by ``oracle/build_ref.sh``:
  ``buildPairsAndTriplesWithEleIndexLinear(4.6, 3.1, eles, elep)`` and the
  Coulomb list ``buildPairs(15.0)`` exactly as
  ``TFMolManage.EvalBPDirectEELinearSingle`` calls them (TFMolManage.py:1428-1431),
  plus the periodic ``NeighborListSetWithImages`` calls of
  ``EvalBPDirectEEUpdateSinglePeriodic`` (TFMolManage.py:1342-1345) on a
  tessellated box;
* ``MolEmb.Make_ANI1_Sym`` descriptor rows and ``Make_ANI1_Sym_deri`` Jacobian
  slices (C_API/MolEmb.cpp:1844-1988); for the periodic box, the rows of its
  real atoms computed over the tessellated cell (no Jacobian there).

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import os
import subprocess
import sys
import types

import numpy as np

# the reference's modules are imported from its own (read-only) tree: no
# bytecode caches may be written there
sys.dont_write_bytecode = True

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from refpath import reference_root  # noqa: E402

REF = reference_root()
sys.path.insert(0, REPO)

from tensormol_gb300 import systems  # noqa: E402
from tensormol_gb300.params import PARAMS, element_pairs  # noqa: E402
from oracle import reference as orc  # noqa: E402


def load_reference_neighbors():
    subprocess.check_call([os.path.join(REPO, "oracle", "build_ref.sh")])
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    pkg = types.ModuleType("TensorMol")
    pkg.__path__ = []
    util = types.ModuleType("TensorMol.Util")
    util.np = np

    def TMTiming(name):
        def deco(f):
            return f
        return deco

    util.TMTiming = TMTiming
    util.__all__ = ["np", "TMTiming"]
    fm = types.ModuleType("TensorMol.ForceModifiers")
    fm.__path__ = []
    sys.modules.update({"TensorMol": pkg, "TensorMol.Util": util,
                        "TensorMol.ForceModifiers": fm})
    path = os.path.join(REF, "TensorMol", "ForceModifiers", "Neighbors.py")
    spec = importlib.util.spec_from_file_location("TensorMol.ForceModifiers.Neighbors", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    import MolEmb
    return mod, MolEmb


def padded(sysm):
    nmol = sysm.nmol
    counts = np.diff(sysm.offsets)
    maxn = int(counts.max())
    xyzs = np.zeros((nmol, maxn, 3))
    Zs = np.zeros((nmol, maxn), dtype=np.int32)
    for m in range(nmol):
        x, Z = sysm.molecule(m)
        xyzs[m, :len(Z)] = x
        Zs[m, :len(Z)] = Z
    return xyzs, Zs, counts.astype(np.int32)


def open_case(nb, sysm, eles):
    """TFMolManage.py:1418-1431 call sequence."""
    xyzs, Zs, natom = padded(sysm)
    eles_np = np.asarray(eles).reshape((len(eles), 1))
    elep_np = np.asarray(element_pairs(eles))
    NL = nb.NeighborListSet(xyzs, natom, True, True, Zs, sort_=True)
    rad_p_ele, ang_t_elep, mil_j, mil_jk = NL.buildPairsAndTriplesWithEleIndexLinear(
        4.6, 3.1, eles_np, elep_np)
    NLEE = nb.NeighborListSet(xyzs, natom, False, False, None)
    rad_eep = NLEE.buildPairs(15.0)
    return dict(RadpEle=np.asarray(rad_p_ele, dtype=np.float64),
                AngtEle=np.asarray(ang_t_elep, dtype=np.float64),
                mil_j=np.asarray(mil_j, dtype=np.float64),
                mil_jk=np.asarray(mil_jk, dtype=np.float64),
                rad_eep=np.asarray(rad_eep, dtype=np.float64))


def periodic_case(nb, x, Z, lattice, eles, ree_cut):
    """TFMolManage.py:1339-1345 on the tessellated cell (Periodic.py:131-181).
    ``ree_cut`` is kept below half the cell edge so that the 27-image list is
    the minimum-image list."""
    xt = orc.tessellate(x, lattice, 1)
    Zt = np.tile(Z, xt.shape[0] // len(Z))
    nreal = len(Z)
    xyzs = xt[None]
    Zs = Zt[None].astype(np.int32)
    eles_np = np.asarray(eles).reshape((len(eles), 1))
    elep_np = np.asarray(element_pairs(eles))
    NL = nb.NeighborListSetWithImages(xyzs, np.array([xt.shape[0]]), np.array([nreal]), True, True,
                                      Zs, sort_=True)
    rad_p_ele, ang_t_elep, mil_j, mil_jk = NL.buildPairsAndTriplesWithEleIndexPeriodic(
        4.6, 3.1, eles_np, elep_np)
    NLEE = nb.NeighborListSetWithImages(xyzs, np.array([xt.shape[0]]), np.array([nreal]), False,
                                        True, Zs)
    rad_eep_e1e2 = NLEE.buildPairsWithBothEleIndex(ree_cut, eles_np)
    return dict(RadpEle=np.asarray(rad_p_ele, dtype=np.float64),
                AngtEle=np.asarray(ang_t_elep, dtype=np.float64),
                mil_j=np.asarray(mil_j, dtype=np.float64),
                mil_jk=np.asarray(mil_jk, dtype=np.float64),
                rad_eep_e1e2=np.asarray(rad_eep_e1e2, dtype=np.float64))


def ani1(molemb, x, Z, eles, atoms_deri):
    prm = {k: PARAMS[k] for k in ("AN1_num_r_Rs", "AN1_num_a_Rs", "AN1_num_a_As",
                                  "AN1_r_Rc", "AN1_a_Rc", "AN1_eta", "AN1_zeta")}
    from tensormol_gb300.params import ani1_grids
    rs_r, rs_a, th = ani1_grids()
    prm.update(AN1_r_Rs=rs_r, AN1_a_Rs=rs_a, AN1_a_As=th)
    xyz = np.ascontiguousarray(x, dtype=np.float64)
    at = np.ascontiguousarray(Z, dtype=np.uint8)
    el = np.ascontiguousarray(eles, dtype=np.uint8)
    # -1: every atom, each in its own iteration of the outer parallel loop
    G = molemb.Make_ANI1_Sym(prm, xyz, at, el, -1)
    if not len(atoms_deri):
        return G, None
    J = np.stack([molemb.Make_ANI1_Sym_deri(prm, xyz, at, el, int(a))[0] for a in atoms_deri])
    return G, J


def main():
    nb, molemb = load_reference_neighbors()
    out = {}
    # 20-H2O open cluster (60 atoms), seed 0
    w = systems.water_cluster_60(seed=0)
    c = open_case(nb, w, [1, 8])
    G, J = ani1(molemb, w.x, w.Z, [1, 8], [0, 1, 2, 30])
    np.savez_compressed(os.path.join(HERE, "water60.npz"), x=w.x, Z=w.Z, offsets=w.offsets,
                        ani1_G=G, ani1_deri=J, ani1_deri_atoms=np.array([0, 1, 2, 30]), **c)
    out["water60"] = {k: v.shape for k, v in c.items()}
    # ragged CHNO batch (6 molecules of 8-64 atoms), seed 3
    b = systems.chno_batch(nmol=6, seed=3)
    c = open_case(nb, b, [1, 6, 7, 8])
    x0, Z0 = b.molecule(0)
    G, J = ani1(molemb, x0, Z0, [1, 6, 7, 8], [0, 3])
    np.savez_compressed(os.path.join(HERE, "chno6.npz"), x=b.x, Z=b.Z, offsets=b.offsets,
                        ani1_G_mol0=G, ani1_deri_mol0=J, ani1_deri_atoms=np.array([0, 3]), **c)
    out["chno6"] = {k: v.shape for k, v in c.items()}
    # periodic water box: 64 H2O at 1 g/cm^3, cubic cell 12.42 A, wrapped
    L = 49.7 / 4.0
    pb = systems.water(64, seed=5, spacing=L / 4.0, box=L, n_side=4)
    lat = np.eye(3) * L
    xw = orc.modulo_lattice(pb.x, lat)
    c = periodic_case(nb, xw, pb.Z, lat, [1, 8], 6.0)
    # descriptor rows of the real atoms among their 26 image shells
    # (tessellated cell, real atoms first; Periodic.py:131-181)
    xt = orc.tessellate(xw, lat, 1)
    Gt, _ = ani1(molemb, xt, np.tile(pb.Z, xt.shape[0] // len(pb.Z)), [1, 8], [])
    np.savez_compressed(os.path.join(HERE, "waterbox192.npz"), x=xw, Z=pb.Z, lattice=lat,
                        ree_cut=np.array(6.0), ani1_G=Gt[:len(pb.Z)], **c)
    out["waterbox192"] = {k: v.shape for k, v in c.items()}
    for k, v in out.items():
        print(k, v)


if __name__ == "__main__":
    main()
