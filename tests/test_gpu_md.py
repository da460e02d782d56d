"""GPU parity of the device integrators (tm_md_*, through the C ABI) against
the oracle's FP64 restatement of Simulations/SimpleMD.py driven by the oracle's
own FP64 forces.

The two trajectories differ only through the FP32 force error (~1e-5 eV/A
here), so after 20 steps of 0.5 fs they agree to well below the stated bounds:
positions 1e-5 A, velocities 5e-6 A/fs, potential 1e-5 eV/atom, kinetic and
conserved energies 0.5 J/mol per atom (about 1e-4 of the kinetic energy per
atom at 300 K, 3.7 kJ/mol), T_eff 1e-4 relative. The smooth activation
(sigmoid_with_param) is used: relu forces jump at kinks, which makes any two
trajectories separate at the first kink crossing.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, IDEALGASR, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu

X_TOL = 1e-5       # A
V_TOL = 5e-6       # A/fs
E_TOL = 1e-5       # eV / atom (potential)
J_TOL = 0.5        # J/mol per atom (kinetic, conserved)


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import md, model
    return model, md


def _models(model, eles, **kw):
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    p.update(kw)
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    return model.BPEEModel(eles, W, params=p, precision="fp32"), orc.Model(eles, W, params=p)


def _open_ef(om, Z, off):
    def ef(x):
        o = orc.OpenSystemOracle(om, x, Z, off).terms(x)
        return float(o["Etotal"].sum()), o["force"]
    return ef


def _compare(log, X, V, ref_x, ref_v, ref_log, n):
    dx = np.abs(X - ref_x).max()
    dv = np.abs(V - ref_v).max()
    dpe = np.abs(log[:, 0] - ref_log[:, 0]).max() * EV_PER_HARTREE / n
    dke = np.abs(log[:, 1] - ref_log[:, 1]).max()
    dcons = np.abs(log[:, 2] - ref_log[:, 2]).max() / n
    assert dx < X_TOL and dv < V_TOL, (dx, dv)
    assert dpe < E_TOL and dke < J_TOL and dcons < J_TOL, (dpe, dke, dcons)
    np.testing.assert_allclose(log[:, 3], ref_log[:, 3], rtol=1e-4, atol=1e-3)


def _teff(ke_per_atom):
    return (2.0 / 3.0) * ke_per_atom / IDEALGASR


def test_nve_velocity_verlet_water60(gpu):
    model, md = gpu
    w = systems.water_cluster_60(seed=0)
    m, om = _models(model, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    v0 = systems.maxwell_boltzmann(w.Z, 300.0, seed=11)
    dyn = md.DeviceMD(s, "nve", dt=0.5, T=300.0)
    dyn.set_velocities(v0)
    nst = 20
    log = dyn.run(nst)
    X, V = s.positions(), dyn.velocities()
    # oracle: VelocityVerletStep with a0 = 0 (SimpleMD.py:14-38, :359)
    ef = _open_ef(om, w.Z, w.offsets)
    mass = systems.masses(w.Z)
    x, v, a = w.x.copy(), v0.copy(), np.zeros_like(w.x)
    ref = np.zeros((nst, 4))
    for k in range(nst):
        x, v, a, e = orc.vv_step(ef, a, x, v, mass, 0.5)
        ke = orc.kinetic_energy(v, mass)
        ref[k] = (e, ke, ke * w.natoms + e * JOULEPERHARTREE, _teff(ke))
    _compare(log, X, V, x, v, ref, w.natoms)
    dyn.close()
    s.close()


def test_nose_thermostat_water60(gpu):
    model, md = gpu
    w = systems.water_cluster_60(seed=0)
    m, om = _models(model, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    v0 = systems.maxwell_boltzmann(w.Z, 300.0, seed=12) * 1.5   # start hot: eta moves
    dt, T, nst = 0.5, 300.0, 20
    dyn = md.DeviceMD(s, "nose", dt=dt, T=T)
    dyn.set_velocities(v0)
    log = dyn.run(nst)
    X, V = s.positions(), dyn.velocities()
    ef = _open_ef(om, w.Z, w.offsets)
    mass = systems.masses(w.Z)
    th = orc.Nose(mass, T, dt)
    x, v, a = w.x.copy(), v0.copy(), np.zeros_like(w.x)
    ref = np.zeros((nst, 4))
    xi = 0.0
    for k in range(nst):
        e0 = th.eta
        x, v, a, e = th.step(ef, a, x, v)
        xi += 0.5 * (e0 + th.eta) * dt
        ke = orc.kinetic_energy(v, mass)
        ext = (0.5 * th.Q * th.eta ** 2 + (3.0 * w.natoms + 1.0) * th.kT * xi) * 1e10
        ref[k] = (e, ke, ke * w.natoms + e * JOULEPERHARTREE + ext, _teff(ke))
    assert abs(th.eta) > 0.0
    _compare(log, X, V, x, v, ref, w.natoms)
    dyn.close()
    s.close()


def _nhc_reference(ef, x, v, mass, T, dt, nst, M=3, wrap=None):
    th = orc.NoseHooverChain(mass, T, dt, M=M)
    a = np.zeros_like(x)
    ref = np.zeros((nst, 4))
    n = len(mass)
    for k in range(nst):
        x, v, a, e = th.step(ef, a, x, v)
        if wrap is not None:
            x = wrap(x)
        ke = orc.kinetic_energy(v, mass)
        ref[k] = (e, ke, th.conserved(v, e * JOULEPERHARTREE), _teff(ke))
    return x, v, ref


def test_nose_hoover_chain_water60(gpu):
    model, md = gpu
    w = systems.water_cluster_60(seed=0)
    m, om = _models(model, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    v0 = systems.maxwell_boltzmann(w.Z, 300.0, seed=13) * 1.5
    dt, T, nst = 0.5, 300.0, 20
    dyn = md.DeviceMD(s, "nhc", dt=dt, T=T, chain=3)
    dyn.set_velocities(v0)
    log = dyn.run(nst)
    X, V = s.positions(), dyn.velocities()
    x, v, ref = _nhc_reference(_open_ef(om, w.Z, w.offsets), w.x.copy(), v0.copy(),
                               systems.masses(w.Z), T, dt, nst)
    _compare(log, X, V, x, v, ref, w.natoms)
    dyn.close()
    s.close()


def test_nose_hoover_chain_periodic_box(gpu):
    """NHC-3 in a periodic water box (216 H2O, 18.6 A cell, 9 A Coulomb
    cutoff): positions wrapped into the cell each step, as Prop does with a
    cellsize (SimpleMD.py:398-399)."""
    model, md = gpu
    L = 18.6
    b = systems.water(216, seed=6, spacing=L / 6.0, box=L, n_side=6)
    lat = np.eye(3) * L
    x0 = orc.modulo_lattice(b.x, lat)
    m, om = _models(model, [1, 8], EECutoffOff=9.0)
    s = m.system(x0, b.Z, None, lat)
    v0 = systems.maxwell_boltzmann(b.Z, 300.0, seed=14)
    dt, T, nst = 0.5, 300.0, 10
    dyn = md.DeviceMD(s, "nhc", dt=dt, T=T, chain=3)
    dyn.set_velocities(v0)
    log = dyn.run(nst)
    X, V = s.positions(), dyn.velocities()

    def ef(x):
        o = orc.PeriodicOracle(om, x, b.Z, lat, ree_cut=9.0).terms(x)
        return float(o["Etotal"].sum()), o["force"]

    x, v, ref = _nhc_reference(ef, x0.copy(), v0.copy(), systems.masses(b.Z), T, dt, nst,
                               wrap=lambda y: orc.modulo_lattice(y, lat))
    d = X - x
    d -= L * np.round(d / L)   # same point of the cell
    X = x + d
    _compare(log, X, V, x, v, ref, len(b.Z))
    dyn.close()
    s.close()


def test_nve_100_steps_conserves_energy_water60(gpu):
    """C0: E+F then 100 NVE steps of 0.5 fs; the conserved energy drifts by
    less than 1% of the kinetic energy."""
    model, md = gpu
    w = systems.water_cluster_60(seed=0)
    m, _ = _models(model, [1, 8])
    s = m.system(w.x, w.Z, w.offsets)
    dyn = md.DeviceMD(s, "nve", dt=0.5, T=300.0)
    dyn.set_velocities(systems.maxwell_boltzmann(w.Z, 300.0, seed=11))
    log = dyn.run(100)
    ke_tot = log[:, 1].mean() * w.natoms
    drift = abs(log[-1, 2] - log[0, 2])
    print(f"NVE water60 100 steps: drift {drift:.3e} J/mol, <KE> {ke_tot:.3e} J/mol")
    assert np.all(np.isfinite(log)) and drift < 0.01 * ke_tot
    dyn.close()
    s.close()


def test_velocity_verlet_driver_mirror(gpu):
    """tensormol_gb300.md.VelocityVerlet: the reference driver's interface
    (SimpleMD.py:322-424) over the device integrator."""
    model, md = gpu
    from tensormol_gb300.model import EnergyAndForce, Mol, TFMolManage
    w = systems.water_cluster_60(seed=0)
    m, om = _models(model, [1, 8])
    EF = EnergyAndForce(TFMolManage(m), w.Z)
    saved = {k: PARAMS.get(k) for k in ("MDMaxStep", "MDdt", "MDThermostat", "MDV0")}
    try:
        PARAMS.update(MDMaxStep=10, MDdt=0.5, MDThermostat=None, MDV0=None)
        vv = md.VelocityVerlet(None, Mol(w.Z, w.x), "w60", EF)
        mdlog = vv.Prop()
    finally:
        PARAMS.update(saved)
    ef = _open_ef(om, w.Z, w.offsets)
    e0, _ = ef(w.x)
    assert abs(vv.EPot0 - e0) * EV_PER_HARTREE / w.natoms < E_TOL
    # zero initial velocities: the first step does not move the atoms (a0 = 0)
    x, v, a = w.x.copy(), np.zeros_like(w.x), np.zeros_like(w.x)
    mass = systems.masses(w.Z)
    for _ in range(10):
        x, v, a, e = orc.vv_step(ef, a, x, v, mass, 0.5)
    assert np.abs(vv.x - x).max() < X_TOL
    assert mdlog.shape == (10, 7) and mdlog[0, 4] == 0.0
    assert abs(mdlog[-1, 5] - e) * EV_PER_HARTREE / w.natoms < E_TOL


def test_velocity_verlet_trajectory_files(gpu, tmp_path, monkeypatch):
    """MDLogTrajectory: frames at steps 0, 3, 6, ... in ./results, positions equal
    to an uninterrupted device run of the same steps; md_log saved."""
    model, md = gpu
    from tensormol_gb300.model import EnergyAndForce, Mol, TFMolManage
    w = systems.water_cluster_60(seed=0)
    m, _ = _models(model, [1, 8])
    monkeypatch.chdir(tmp_path)
    saved = {k: PARAMS.get(k) for k in ("MDMaxStep", "MDdt", "MDThermostat", "MDV0", "MDLogTrajectory")}
    try:
        PARAMS.update(MDMaxStep=8, MDdt=0.5, MDThermostat=None, MDV0="Thermal", MDLogTrajectory=True)
        vv = md.VelocityVerlet(None, Mol(w.Z, w.x), "w60", EnergyAndForce(TFMolManage(m), w.Z),
                               seed=5)
        v0 = vv.v.copy()
        vv.Prop()
    finally:
        PARAMS.update(saved)
    text = (tmp_path / "results" / "MDTrajectoryw60.xyz").read_text()
    frames = [f for f in text.split("60\nComment:") if f.strip()]
    assert len(frames) == 3                                   # steps 0, 3, 6
    assert (tmp_path / "results" / "MDLogw60.txt").exists()
    s = m.system(w.x, w.Z, w.offsets)
    dyn = md.DeviceMD(s, "nve", dt=0.5)
    dyn.set_velocities(v0)
    dyn.run(7)
    last = Mol()
    last.FromXYZString("60\nComment:" + frames[-1])
    np.testing.assert_allclose(last.coords, s.positions(), rtol=0, atol=1e-12)


@pytest.mark.parametrize("periodic", [False, True])
def test_skin_lists_follow_the_full_rebuild(gpu, periodic):
    """Skin lists (1.0 A; candidates rebuilt on displacement, exact rows every
    step) against a full build every step. The neighbour rows are the same;
    the pair-term sums run over the cells of an older build, so the FP32
    summation order differs (1e-9 A after 5 steps). At 600 K the difference
    grows about tenfold per 10 fs, faster whenever a pair crosses the Coulomb
    cutoff, where the truncated vdW term jumps; after 40 steps (measured
    2e-6 A, 3e-6 A/fs) positions and velocities agree to 2e-5."""
    model, md = gpu
    if periodic:
        L = 18.6
        b = systems.water(216, seed=6, spacing=L / 6.0, box=L, n_side=6)
        lat = np.eye(3) * L
        x0, Z, off, kw = orc.modulo_lattice(b.x, lat), b.Z, None, {"EECutoffOff": 9.0}
    else:
        b = systems.water(300, seed=9, spacing=3.1)
        x0, Z, off, lat, kw = b.x, b.Z, b.offsets, None, {}
    m, _ = _models(model, [1, 8], **kw)
    v0 = systems.maxwell_boltzmann(Z, 600.0, seed=15)
    out = []
    for skin in (0.0, 1.0):
        s = m.system(x0, Z, off, lat)
        dyn = md.DeviceMD(s, "nhc" if periodic else "nve", dt=0.5, T=300.0)
        dyn.set_velocities(v0)
        log = dyn.run(40, skin=skin)
        out.append((s.positions(), dyn.velocities(), log))
        dyn.close()
        s.close()
    (x_a, v_a, l_a), (x_b, v_b, l_b) = out
    d = x_a - x_b
    if periodic:
        d -= 18.6 * np.round(d / 18.6)
    print("skin vs full rebuild: max|dx| %.1e A, max|dv| %.1e A/fs"
          % (np.abs(d).max(), np.abs(v_a - v_b).max()))
    assert np.abs(d).max() < 2e-5 and np.abs(v_a - v_b).max() < 2e-5
    np.testing.assert_allclose(l_a[:, 0], l_b[:, 0], rtol=0, atol=1e-8 * len(Z))   # Hartree


def test_skin_replays_are_limited_per_chunk(gpu):
    """A skin far below one step's displacement (0.002 A at 600 K) makes
    nearly every chunk replay shorter until it is one step long: about 20
    replays over 20 steps, every chunk completing on its retry. The replay
    limit (16) applies to one chunk, so the run finishes, and its rows are
    still exact: it follows the full-build run."""
    model, md = gpu
    w = systems.water_cluster_60(seed=0)
    m, _ = _models(model, [1, 8])
    v0 = systems.maxwell_boltzmann(w.Z, 600.0, seed=15)
    out = []
    for skin in (0.0, 0.002):
        s = m.system(w.x, w.Z, w.offsets)
        dyn = md.DeviceMD(s, "nve", dt=0.5, T=300.0)
        dyn.set_velocities(v0)
        log = dyn.run(20, skin=skin)
        out.append((s.positions(), dyn.velocities(), log))
        dyn.close()
        s.close()
    (x_a, v_a, l_a), (x_b, v_b, l_b) = out
    assert np.abs(x_a - x_b).max() < 2e-5 and np.abs(v_a - v_b).max() < 2e-5
    np.testing.assert_allclose(l_a[:, 0], l_b[:, 0], rtol=0, atol=1e-8 * len(w.Z))
