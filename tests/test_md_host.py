"""The MD driver mirror (tensormol_gb300.md.VelocityVerlet) against the
reference's own VelocityVerlet.Prop, on CPU.

The device integrator is replaced by a stand-in that steps the oracle's
velocity Verlet, which is bit-exact with the reference's VelocityVerletStep
(tests/test_oracle_md.py). The stand-in returns (EPot, KE) rows the way
tm_md_run logs them. The driver's md_log is then compared with the
md_log that the reference's Prop wrote for the same start
(tests/golden/make_golden_md.py): time, the kinetic energy of the step
before, the potential, and the conserved energy. So are the final positions
and velocities.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import md, systems
from tensormol_gb300.params import JOULEPERHARTREE, PARAMS


class _System:
    def __init__(self, x):
        self.x = np.array(x, dtype=np.float64)

    def positions(self):
        return self.x.copy()


class _EnergyAndForce:
    """Energy (Hartree) and force (J/mol/A) of the oracle's anharmonic wells,
    with the system hook the driver asks an EnergyAndForce closure for."""

    def __init__(self, x0, m):
        self.ef = orc.anharmonic_wells(x0)
        self.m = m
        self.system = None

    def __call__(self, x):
        e, f = self.ef(x)
        return e / JOULEPERHARTREE, f

    def system_for(self, x):
        self.system = _System(x)
        return self.system


class _DeviceMD:
    """tm_md_run's contract on the CPU: NVE steps from the resident state,
    rows (EPot Hartree, KE J/mol per atom, conserved, T_eff)."""

    EF = None

    def __init__(self, system, kind="nve", dt=0.5, T=300.0, chain=3):
        assert kind == "nve"
        self.s, self.dt = system, dt
        self.v = np.zeros_like(system.x)
        self.a = np.zeros_like(system.x)

    def set_velocities(self, v):
        self.v = np.array(v, dtype=np.float64)

    def velocities(self):
        return self.v.copy()

    def run(self, n, skin=0.0):
        rows = np.zeros((n, 4))
        for k in range(n):
            x, self.v, self.a, e = orc.vv_step(self.EF, self.a, self.s.x, self.v, self.EF.m, self.dt)
            self.s.x = x
            rows[k, 0], rows[k, 1] = e, orc.kinetic_energy(self.v, self.EF.m)
        return rows


def test_driver_md_log_matches_reference_prop(golden_loader, monkeypatch, tmp_path):
    g = golden_loader("md_simplemd")
    w = systems.water_cluster_60(seed=0)
    n = int(g["prop_nsteps"])
    for key, val in dict(MDMaxStep=n, MDdt=float(g["dt"]), MDTemp=float(g["T"]), MDV0=None,
                         MDThermostat=None, MDLogTrajectory=False).items():
        monkeypatch.setitem(PARAMS, key, val)
    monkeypatch.chdir(tmp_path)
    ef = _EnergyAndForce(g["x0"], g["m"])
    monkeypatch.setattr(_DeviceMD, "EF", ef)
    monkeypatch.setattr(md, "DeviceMD", _DeviceMD)

    class _G0:
        atoms = w.Z
        coords = g["x_start"]

    vv = md.VelocityVerlet(None, _G0(), "w60", ef)
    log = vv.Prop()
    ref = g["prop_md_log"]
    assert log.shape == ref.shape == (n, 7)
    np.testing.assert_array_equal(log[:, 0], ref[:, 0])                      # time
    np.testing.assert_allclose(log[:, 4], ref[:, 4], rtol=1e-13, atol=0)     # KE of the step before
    np.testing.assert_allclose(log[:, 5], ref[:, 5], rtol=1e-13, atol=0)     # EPot
    np.testing.assert_allclose(log[:, 6], ref[:, 6], rtol=1e-11, atol=1e-9)  # conserved
    np.testing.assert_allclose(vv.x, g["prop_x"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(vv.v, g["prop_v"], rtol=1e-13, atol=1e-20)
    assert (tmp_path / "results" / "MDLogw60.txt").exists() is False   # no results dir, no file


def test_driver_rejects_host_force_routines():
    """Without an EnergyAndForce closure of this package there is no
    integrator to run: the driver raises instead of falling back to the host."""
    w = systems.water_cluster_60(seed=0)

    class _G0:
        atoms = w.Z
        coords = w.x

    with pytest.raises(RuntimeError):
        md.VelocityVerlet(None, _G0(), "x", lambda x: (0.0, np.zeros_like(x)))
