"""Golden trajectories of the reference's own MD integrators.

Runs ``VelocityVerletStep``, ``NoseThermostat.step`` and
``NoseChainThermostat.step`` (Simulations/SimpleMD.py:14-38, 90-129, 206-320),
imported unchanged from the reference tree with the package modules it
star-imports replaced by stubs (numpy, PARAMS, the gas constant of the
reference's own PhysicalData.py), on a 60-atom water cluster in the
``anharmonic_wells`` force field of the oracle. The thermostats' constructors
rescale the starting velocities in place (SimpleMD.py:82-88); the rescaled
velocities are stored as each run's start. It also runs the driver
``VelocityVerlet.Prop`` (SimpleMD.py:322-424), NVE from the same start, and
stores its ``md_log``. Writes ``tests/golden/md_simplemd.npz``.

Usage (where the reference tree is present): python tests/golden/make_golden_md.py
"""
from __future__ import annotations

import contextlib
import importlib.util
import io
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
from tensormol_gb300.params import PARAMS  # noqa: E402

DT = 0.2        # fs, PARAMS["MDdt"]
TEMP = 300.0    # K, PARAMS["MDTemp"]
NCHAIN = 3      # PARAMS["MNHChain"]
NSTEPS = 30
KEEP = [0, 1, 9, 29]   # stored steps (0-based): 1, 2, 10 and 30


def load_simplemd(params):
    def load(name, path):
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    pkg = types.ModuleType("TensorMol")
    pkg.__path__ = []
    sys.modules["TensorMol"] = pkg
    for sub in ("Containers", "TFNetworks", "ForceModels", "Math", "Simulations"):
        m = types.ModuleType("TensorMol." + sub)
        m.__path__ = []
        sys.modules["TensorMol." + sub] = m
    phys = load("TensorMol.PhysicalData", os.path.join(REF, "PhysicalData.py"))

    class _Logger:
        def info(self, *a, **k):
            pass

    common = {"np": np, "PARAMS": params, "IDEALGASR": phys.IDEALGASR,
              "ATOMICMASSES": phys.ATOMICMASSES, "JOULEPERHARTREE": phys.JOULEPERHARTREE,
              "KJPERHARTREE": phys.KJPERHARTREE, "time": __import__("time"), "LOGGER": _Logger(),
              # running energy statistics of Prop, never logged (Math/Statistics.py)
              "OnlineEstimator": lambda e0: (lambda e: (0.0, 0.0))}
    for name in ("TensorMol.Containers.Sets", "TensorMol.TFNetworks.TFManage",
                 "TensorMol.ForceModels.Electrostatics", "TensorMol.Math.QuasiNewtonTools",
                 "TensorMol.Math.Statistics"):
        m = types.ModuleType(name)
        m.__dict__.update(common)
        m.__all__ = list(common)
        sys.modules[name] = m
    return load("TensorMol.Simulations.SimpleMD", os.path.join(REF, "Simulations", "SimpleMD.py"))


def start_state():
    """Positions displaced from the wells' minima, velocities at 300 K."""
    w = systems.water_cluster_60(seed=0)
    rng = np.random.default_rng(11)
    x = w.x + 0.05 * rng.normal(size=w.x.shape)
    v = systems.maxwell_boltzmann(w.Z, TEMP, seed=12)
    return w.x.copy(), x, v, systems.masses(w.Z)


def main():
    params = dict(PARAMS)
    params.update(MDdt=DT, MDTemp=TEMP, MNHChain=NCHAIN)
    smd = load_simplemd(params)
    x0, xs, vs, m = start_state()
    ef = orc.anharmonic_wells(x0)
    out = {"x0": x0, "x_start": xs, "v_start": vs, "m": m,
           "dt": DT, "T": TEMP, "nsteps": NSTEPS}

    # velocity Verlet (SimpleMD.py:14-38); a = 0 at the first step (SimpleMD.py:359)
    x, v, a = xs.copy(), vs.copy(), np.zeros_like(xs)
    X, V, A, E = [], [], [], []
    for _ in range(NSTEPS):
        x, v, a, e = smd.VelocityVerletStep(None, a, x, v, m, DT, ef)
        X.append(x); V.append(v); A.append(a); E.append(e)
    out.update(vv_x=np.array(X), vv_v=np.array(V), vv_a=np.array(A), vv_e=np.array(E))

    # Nose thermostat (SimpleMD.py:90-129)
    x, v, a = xs.copy(), vs.copy(), np.zeros_like(xs)
    with contextlib.redirect_stdout(io.StringIO()):
        th = smd.NoseThermostat(m, v)   # rescales v in place
    out["nose_v0"] = v.copy()
    X, V, ETA = [], [], []
    for _ in range(NSTEPS):
        x, v, a, e, _f = th.step(None, a, x, v, m, DT, ef)
        X.append(x); V.append(v); ETA.append(th.eta)
    out.update(nose_x=np.array(X), nose_v=np.array(V), nose_eta=np.array(ETA))

    # Nose-Hoover chain (SimpleMD.py:206-320)
    # Its constructor's Rescale reads self.m (SimpleMD.py:85), which no line of
    # that constructor sets: the instance is given the masses before it runs.
    x, v, a = xs.copy(), vs.copy(), np.zeros_like(xs)
    th = smd.NoseChainThermostat.__new__(smd.NoseChainThermostat)
    th.m = m.copy()
    with contextlib.redirect_stdout(io.StringIO()):
        th.__init__(m, v)   # rescales v in place
    out["nhc_v0"] = v.copy()
    X, V, ETA, VETA = [], [], [], []
    for _ in range(NSTEPS):
        with contextlib.redirect_stdout(io.StringIO()):
            x, v, a, e = th.step(None, a, x, v, m, DT, ef)
        X.append(x); V.append(v); ETA.append(th.eta.copy()); VETA.append(th.Veta.copy())
    out.update(nhc_x=np.array(X), nhc_v=np.array(V), nhc_eta=np.array(ETA), nhc_veta=np.array(VETA))

    # the driver's log: VelocityVerlet.Prop (SimpleMD.py:391-424), NVE, zero
    # starting velocities, energies in Hartree (the wells' J/mol scaled), run in
    # a scratch directory because Prop saves ./results/MDLog<name>.txt
    import tempfile

    class _G0:
        atoms = np.asarray(systems.water_cluster_60(seed=0).Z)
        coords = xs.copy()

    jph = smd.JOULEPERHARTREE   # the reference's own constant

    def ef_h(x):
        e, f = ef(x)
        return e / jph, f

    params.update(MDMaxStep=20, MDV0=None, MDThermostat=None, MDLogTrajectory=False)
    here = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        os.makedirs("results")
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                vv = smd.VelocityVerlet(None, _G0(), "w60", ef_h)
                vv.Prop()
        finally:
            os.chdir(here)
    out.update(prop_md_log=vv.md_log, prop_x=vv.x, prop_v=vv.v, prop_nsteps=20)

    for key in list(out):
        if key.startswith(("vv_", "nose_", "nhc_")) and not key.endswith("_v0"):
            out[key] = out[key][KEEP]
    out["keep"] = np.array(KEEP)
    path = os.path.join(HERE, "md_simplemd.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
