"""The optimisation drivers' restatement (tensormol_gb300.opt) against golden
trajectories of the reference's own GeomOptimizer / ConjGradient /
RemoveInvariantForce and NudgedElasticBand / VerletOptimizer
(tests/golden/make_golden_opt.py), both driven by the FP64 oracle: on the CPU
the trajectories agree to round-off (1e-8 A)."""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import opt, systems
from tensormol_gb300.model import Mol
from tensormol_gb300.params import PARAMS, descriptor_width


def _ef(Z):
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    om = orc.Model([1, 8], W, params=p)
    off = np.array([0, len(Z)])

    def ef(x, DoForce=True):
        o = orc.OpenSystemOracle(om, np.asarray(x), Z, off)
        if DoForce:
            t = o.terms(np.asarray(x))
            return float(t["Etotal"].sum()), t["force"]
        return float(o.energy(np.asarray(x)).sum())
    return ef


@pytest.fixture
def params():
    saved = dict(PARAMS)
    yield PARAMS
    PARAMS.clear()
    PARAMS.update(saved)


def test_geometry_optimiser_matches_reference(golden_loader, params):
    g = golden_loader("opt_water")
    params.update(OptMaxCycles=int(g["max_cycles"]))
    go = opt.GeomOptimizer(_ef(g["Z"]))
    prev = go.Opt(Mol(g["Z"], g["x0"]))
    xs = np.array([h[1] for h in go.history])
    n = min(len(xs), len(g["x_steps"]))
    assert n == len(g["x_steps"])
    np.testing.assert_allclose(xs[:n], g["x_steps"][:n], rtol=0, atol=1e-8)
    np.testing.assert_allclose(prev.coords, g["x_final_prev"], rtol=0, atol=1e-8)


def test_neb_matches_reference(golden_loader, params):
    g = golden_loader("neb_water")
    params.update(NebSolver="Verlet")
    band = opt.NudgedElasticBand(_ef(g["Z"]), Mol(g["Z"], g["x0"]), Mol(g["Z"], g["x1"]),
                                 nbeads_=int(g["nbeads"]))
    band.Fs = band.Fs + 1.0
    for step in range(len(g["beads"])):
        band.step = step
        band.beads, energy, band.Fs = band.Solver(band.beads)
        band.TSI = int(np.argmax(band.Es))
        np.testing.assert_allclose(band.beads.numpy(), g["beads"][step], rtol=0, atol=1e-8)
        np.testing.assert_allclose(band.Es, g["Es"][step], rtol=0, atol=1e-10)
