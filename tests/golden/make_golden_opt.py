"""Golden trajectories of the reference's own optimisation drivers.

Runs the reference's ``GeomOptimizer`` (Simulations/Opt.py), ``ConjGradient``
and ``RemoveInvariantForce`` (Math/QuasiNewtonTools.py) and
``NudgedElasticBand`` with its default ``VerletOptimizer`` (Simulations/Neb.py,
Math/BFGS.py), imported unchanged from the reference tree with the package's
TensorFlow-dependent modules replaced by stubs (containers, logger, PARAMS),
driven by the FP64 oracle's energy/force routine. Writes
``tests/golden/opt_water.npz`` and ``tests/golden/neb_water.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_opt.py
"""
from __future__ import annotations

import importlib.util
import os
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

REF = os.path.join(reference_root(), "TensorMol")
sys.path.insert(0, REPO)

from oracle import reference as orc  # noqa: E402
from tensormol_gb300 import systems  # noqa: E402
from tensormol_gb300.params import PARAMS, descriptor_width  # noqa: E402


class _Logger:
    def info(self, *a, **k):
        pass


class _Mol:
    """Stand-in for Containers/Mol.py: the drivers only read atoms/coords and
    write trajectories (skipped here)."""

    def __init__(self, atoms=None, coords=None):
        self.atoms = np.array(atoms)
        self.coords = np.array(coords, dtype=np.float64)
        self.properties = {}

    def WriteXYZfile(self, *a, **k):
        pass


def load_reference_drivers(params):
    mods = {}
    pkg = types.ModuleType("TensorMol")
    pkg.__path__ = []
    mods["TensorMol"] = pkg
    for sub in ("Math", "Simulations", "Containers", "TFNetworks"):
        m = types.ModuleType("TensorMol." + sub)
        m.__path__ = []
        mods["TensorMol." + sub] = m
    common = {"np": np, "PARAMS": params, "LOGGER": _Logger(), "Mol": _Mol}
    for name in ("TensorMol.Util", "TensorMol.Containers.Sets", "TensorMol.TFNetworks.TFManage",
                 "TensorMol.ForceModels"):
        m = types.ModuleType(name)
        m.__dict__.update(common)
        m.__all__ = list(common)
        mods[name] = m
    sys.modules.update(mods)

    def load(name, path):
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        mod.PARAMS = params
        return mod

    load("TensorMol.PhysicalData", os.path.join(REF, "PhysicalData.py"))
    load("TensorMol.Math.LinearOperations", os.path.join(REF, "Math", "LinearOperations.py"))
    qnt = load("TensorMol.Math.QuasiNewtonTools", os.path.join(REF, "Math", "QuasiNewtonTools.py"))
    load("TensorMol.Math.DIIS", os.path.join(REF, "Math", "DIIS.py"))
    load("TensorMol.Math.BFGS", os.path.join(REF, "Math", "BFGS.py"))
    opt = load("TensorMol.Simulations.Opt", os.path.join(REF, "Simulations", "Opt.py"))
    neb = load("TensorMol.Simulations.Neb", os.path.join(REF, "Simulations", "Neb.py"))
    return qnt, opt, neb


def oracle_ef(om, Z):
    off = np.array([0, len(Z)])

    def ef(x, DoForce=True):
        o = orc.OpenSystemOracle(om, np.asarray(x), Z, off)
        if DoForce:
            t = o.terms(np.asarray(x))
            return float(t["Etotal"].sum()), t["force"]
        return float(o.energy(np.asarray(x)).sum())
    return ef


def main():
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    om = orc.Model([1, 8], W, params=p)
    w = systems.water(12, seed=31, spacing=3.1)
    params = dict(PARAMS)
    params.update(OptMaxCycles=10, NebNumBeads=6, NebSolver="Verlet")
    qnt, opt, neb = load_reference_drivers(params)
    ef = oracle_ef(om, w.Z)

    # geometry optimisation: the reference's Opt loop, recording each CG step
    g = opt.GeomOptimizer(ef)
    m = _Mol(w.Z, w.x)
    g.m = m
    CG = qnt.ConjGradient(g.WrappedEForce, m.coords)
    xs, es = [], []
    for _ in range(params["OptMaxCycles"]):
        m.coords, energy, frc = CG(m.coords)
        xs.append(m.coords.copy())
        es.append(energy)
    final = opt.GeomOptimizer(ef).Opt(_Mol(w.Z, w.x))
    np.savez_compressed(os.path.join(HERE, "opt_water.npz"), Z=w.Z, x0=w.x, x_steps=np.array(xs),
                        e_steps=np.array(es), x_final_prev=final.coords,
                        max_cycles=params["OptMaxCycles"])

    # nudged elastic band: one water molecule moved by 1 A between the ends
    x1 = w.x.copy()
    x1[:3, 0] += 1.0
    band = neb.NudgedElasticBand(ef, _Mol(w.Z, w.x), _Mol(w.Z, x1))
    beads, Es = [], []
    band.Fs = np.ones(band.beads.shape)
    for step in range(4):
        band.step = step
        band.beads, energy, band.Fs = band.Solver(band.beads)
        band.TSI = int(np.argmax(band.Es))
        beads.append(band.beads.copy())
        Es.append(band.Es.copy())
    np.savez_compressed(os.path.join(HERE, "neb_water.npz"), Z=w.Z, x0=w.x, x1=x1,
                        beads=np.array(beads), Es=np.array(Es), nbeads=params["NebNumBeads"])
    print("wrote opt_water.npz, neb_water.npz")


if __name__ == "__main__":
    main()
