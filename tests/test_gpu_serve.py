"""Serving loop on the GPU (tm_serve through the C ABI).

* Each request's results are the same alone and in a mix of requests that
  join and leave while it is in flight: positions, velocities, forces and
  per-step energies are compared bit for bit (molecules never interact in any
  kernel, so the batch composition cannot change a request's arithmetic).
* An MD request served in a batch follows the oracle's velocity-Verlet
  trajectory (FP64 forces) within the integrator tolerances of
  test_gpu_md.py.
* The batch never exceeds its atom capacity; oversize requests are refused.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import model, serve
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    return m, serve, orc.Model([1, 8], W, params=p)


def _req(serve, nmol, seed, kind="md", nsteps=10):
    w = systems.water(nmol, seed, 3.1)
    v = systems.maxwell_boltzmann(w.Z, 300.0, seed=seed + 100)
    return serve.Request(w.Z, w.x, kind=kind, nsteps=nsteps, v=v)


def _clone(serve, r):
    return serve.Request(r.Z, r.x0, kind=r.kind, nsteps=r.nsteps, v=r.v0)


def test_results_same_alone_and_in_the_mix(env):
    m, serve, _ = env
    A = _req(serve, 10, 1, "md", 12)
    B = _req(serve, 50, 2, "md", 6)
    C = _req(serve, 20, 3, "ef")
    D = _req(serve, 5, 4, "md", 9)
    srv = serve.Server(m, max_atoms=4096, max_mols=8)
    schedule = {0: [A], 2: [B, C], 5: [D]}
    for k in range(40):
        for r in schedule.get(k, []):
            srv.submit(r)
        srv.step()
        if not srv.pending and all(r.done for r in (A, B, C, D)):
            break
    srv.close()
    assert all(r.done for r in (A, B, C, D))
    for r in (A, B, C, D):
        alone = _clone(serve, r)
        s1 = serve.Server(m, max_atoms=1024, max_mols=2)
        s1.submit(alone)
        s1.drain()
        s1.close()
        assert np.array_equal(r.x, alone.x) and np.array_equal(r.v, alone.v), r.rid
        assert np.array_equal(r.F, alone.F), r.rid
        assert np.array_equal(np.array(r.energies), np.array(alone.energies)), r.rid


def test_served_md_follows_oracle(env):
    m, serve, om = env
    r = _req(serve, 20, 5, "md", 10)
    other = _req(serve, 30, 6, "md", 4)
    srv = serve.Server(m, max_atoms=4096, max_mols=4)
    srv.submit(other)
    srv.submit(r)
    srv.drain()
    srv.close()
    off = np.array([0, r.natoms])

    def ef(x):
        o = orc.OpenSystemOracle(om, x, r.Z, off).terms(x)
        return float(o["Etotal"].sum()), o["force"]

    x, v, a = r.x0.copy(), r.v0.copy(), np.zeros_like(r.x0)
    mass = systems.masses(r.Z)
    for _ in range(r.nsteps):
        x, v, a, e = orc.vv_step(ef, a, x, v, mass, 0.5)
    assert np.abs(r.x - x).max() < 1e-5
    assert np.abs(r.v - v).max() < 5e-6
    assert abs(r.energies[-1][0] - e) * EV_PER_HARTREE / r.natoms < 1e-5


def test_capacity_is_respected(env):
    m, serve, _ = env
    srv = serve.Server(m, max_atoms=400, max_mols=3)
    reqs = [_req(serve, n, 10 + n, "md", 3) for n in (40, 60, 80, 30, 20)]
    for r in reqs:
        srv.submit(r)
    srv.drain()
    assert all(r.done for r in reqs)
    assert max(srv.step_atoms) <= 400
    with pytest.raises(ValueError):
        srv.submit(_req(serve, 200, 99, "ef"))
        srv.step()
    srv.close()


def test_capacity_for_budget(env):
    m, serve, _ = env
    n = serve.Server.capacity_for_budget(m, 2 << 30, max_mols=64)
    assert n > 10000
    srv = serve.Server(m, max_atoms=n, max_mols=64)
    assert srv.bytes <= (2 << 30) * 1.01
    srv.close()


def test_optimisation_requests_relax_and_match_alone(env):
    """FIRE optimisation requests next to MD and E+F requests: each reaches
    fmax <= 0.05 eV/A (or its step limit) with a non-increasing trend of the
    energy, and gives the same positions alone and in the mix."""
    m, serve, _ = env
    from tensormol_gb300 import systems as sy
    rng = np.random.default_rng(5)
    xo, Zo = sy.chno_molecule(rng, 12)
    Zo = np.where(np.isin(Zo, [1, 8]), Zo, 8).astype(np.int32)   # the water model's H and O
    O = serve.Request(Zo, xo, kind="opt", nsteps=400, fmax=0.05)
    A = _req(serve, 10, 1, "md", 30)
    C = _req(serve, 20, 3, "ef")
    srv = serve.Server(m, max_atoms=2048, max_mols=8)
    for r in (A, O, C):
        srv.submit(r)
    srv.drain()
    srv.close()
    assert O.done and (O.converged or O.steps_done == O.nsteps)
    e = np.array([x[0] for x in O.energies])
    assert e[-1] < e[0]
    alone = serve.Request(Zo, xo, kind="opt", nsteps=400, fmax=0.05)
    s1 = serve.Server(m, max_atoms=1024, max_mols=2)
    s1.submit(alone)
    s1.drain()
    s1.close()
    assert alone.steps_done == O.steps_done
    assert np.array_equal(alone.x, O.x)
