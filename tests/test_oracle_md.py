"""The oracle's FP64 integrators against the reference's own.

The golden trajectories come from tests/golden/make_golden_md.py, which runs
the reference's VelocityVerletStep, NoseThermostat.step and
NoseChainThermostat.step (Simulations/SimpleMD.py) unchanged. Its 60-atom
water cluster sits in the oracle's anharmonic wells. Velocity Verlet and
the Nose thermostat must match step for step. The Nose-Hoover chain must
match with as_simplemd=True, the reference's velocity scale and starting
chain forces. In its default form (Martyna et al. 1996, which the CUDA
integrator follows) it must differ from the reference only through those
two choices. The CUDA integrators are compared with these oracle steps in
tests/test_gpu_md.py.
"""
import numpy as np
import pytest

from oracle import reference as orc

RTOL = 1e-12   # same formulas in FP64; numpy's and libm's exp may differ in the last bit


@pytest.fixture(scope="module")
def g(golden_loader):
    return golden_loader("md_simplemd")


def _run(step, x, v, n):
    a = np.zeros_like(v)
    X, V = [], []
    for _ in range(n):
        x, v, a, _e = step(x, v, a)
        X.append(x)
        V.append(v)
    return np.array(X), np.array(V)


def _check(X, V, g, prefix):
    keep = g["keep"]
    np.testing.assert_allclose(X[keep], g[prefix + "_x"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(V[keep], g[prefix + "_v"], rtol=RTOL, atol=1e-18)


def test_velocity_verlet_matches_simplemd(g):
    ef = orc.anharmonic_wells(g["x0"])
    m, dt = g["m"], float(g["dt"])
    X, V = _run(lambda x, v, a: orc.vv_step(ef, a, x, v, m, dt),
                g["x_start"].copy(), g["v_start"].copy(), int(g["nsteps"]))
    _check(X, V, g, "vv")


def test_nose_matches_simplemd(g):
    ef = orc.anharmonic_wells(g["x0"])
    th = orc.Nose(g["m"], float(g["T"]), float(g["dt"]))
    etas = []

    def step(x, v, a):
        out = th.step(ef, a, x, v)
        etas.append(th.eta)
        return out

    X, V = _run(step, g["x_start"].copy(), g["nose_v0"].copy(), int(g["nsteps"]))
    _check(X, V, g, "nose")
    np.testing.assert_allclose(np.array(etas)[g["keep"]], g["nose_eta"], rtol=RTOL, atol=0)


def _nhc(g, as_simplemd):
    ef = orc.anharmonic_wells(g["x0"])
    th = orc.NoseHooverChain(g["m"], float(g["T"]), float(g["dt"]), M=3, as_simplemd=as_simplemd)
    etas, vetas = [], []

    def step(x, v, a):
        out = th.step(ef, a, x, v)
        etas.append(th.eta.copy())
        vetas.append(th.veta.copy())
        return out

    X, V = _run(step, g["x_start"].copy(), g["nhc_v0"].copy(), int(g["nsteps"]))
    return X, V, np.array(etas), np.array(vetas)


def test_nose_hoover_chain_matches_simplemd_in_its_mode(g):
    X, V, eta, veta = _nhc(g, as_simplemd=True)
    _check(X, V, g, "nhc")
    keep = g["keep"]
    np.testing.assert_allclose(eta[keep], g["nhc_eta"], rtol=RTOL, atol=1e-30)
    np.testing.assert_allclose(veta[keep], g["nhc_veta"], rtol=RTOL, atol=1e-30)


def test_nose_hoover_chain_default_is_the_papers_form(g):
    """The default (the paper's form, which the CUDA integrator follows)
    differs from the reference's chain from the first step on. The first
    chain element scales the velocities, and the chain forces are formed
    from the chain velocities, so the switch is not a no-op. The matching
    test above shows that these two choices are the whole difference."""
    X, V, eta, veta = _nhc(g, as_simplemd=False)
    keep = g["keep"]
    assert not np.allclose(veta[keep][0], g["nhc_veta"][0], rtol=1e-6, atol=0)
    assert not np.allclose(V[keep][0], g["nhc_v"][0], rtol=1e-9, atol=0)
