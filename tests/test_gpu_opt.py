"""Device-resident optimisation drivers (tensormol_gb300.opt over the fused
path) against the golden trajectories of the reference's own GeomOptimizer
(conjugate gradient + golden-section line search) and NudgedElasticBand
(Verlet solver), which were driven by the FP64 oracle. The two differ only by
the FP32-level force/energy error, so the band (no discrete decisions) agrees
to 1e-5 A and the conjugate-gradient path to 1e-4 A over ten steps
(measured: 2e-6 A after ten), energies to 1e-5 eV/atom."""
import numpy as np
import pytest

from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import model, opt
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    return model, opt, m


@pytest.fixture
def params():
    saved = dict(PARAMS)
    yield PARAMS
    PARAMS.clear()
    PARAMS.update(saved)


def test_device_cg_optimiser_follows_reference(env, golden_loader, params):
    model, opt, m = env
    g = golden_loader("opt_water")
    params.update(OptMaxCycles=int(g["max_cycles"]))
    EF = model.EnergyAndForce(model.TFMolManage(m), g["Z"])
    go = opt.GeomOptimizer(EF)
    go.Opt(model.Mol(g["Z"], g["x0"]))
    xs = np.array([h[1] for h in go.history])
    es = np.array([h[0] for h in go.history])
    n = len(g["Z"])
    dx = [float(np.abs(xs[k] - g["x_steps"][k]).max()) for k in range(min(len(xs), len(g["x_steps"])))]
    de = np.abs(es[:len(g["e_steps"])] - g["e_steps"][:len(es)]) * EV_PER_HARTREE / n
    print("CG max|dx| per step", ["%.1e" % v for v in dx], "max dE/atom %.1e eV" % de.max())
    assert max(dx) < 1e-4 and de.max() < 1e-5


def test_device_neb_follows_reference(env, golden_loader, params):
    model, opt, m = env
    g = golden_loader("neb_water")
    params.update(NebSolver="Verlet")
    EF = model.EnergyAndForce(model.TFMolManage(m), g["Z"])
    band = opt.NudgedElasticBand(EF, model.Mol(g["Z"], g["x0"]), model.Mol(g["Z"], g["x1"]),
                                 nbeads_=int(g["nbeads"]))
    assert band._ev.system is not None          # all beads in one batch on the device
    band.Fs = band.Fs + 1.0
    n = len(g["Z"])
    for step in range(len(g["beads"])):
        band.step = step
        band.beads, energy, band.Fs = band.Solver(band.beads)
        band.TSI = int(np.argmax(band.Es))
        dx = np.abs(band.beads.cpu().numpy() - g["beads"][step]).max()
        de = np.abs(band.Es - g["Es"][step]).max() * EV_PER_HARTREE / n
        assert dx < 1e-5 and de < 1e-5, (step, dx, de)
    band.close()
