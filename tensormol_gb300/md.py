"""Device-resident molecular dynamics over the BP+EE energy/force path.

``DeviceMD`` wraps ``tm_md_*``: positions, velocities, accelerations and the
thermostat state stay in HBM; one ``run(n)`` call integrates n steps with one
energy+force evaluation each and no host round trip.

``VelocityVerlet`` mirrors the reference driver
(Simulations/SimpleMD.py:322-424): the same constructor arguments, PARAMS keys
(MDMaxStep, MDTemp, MDdt, MDV0, MDThermostat) and ``Prop()`` filling
``md_log[maxstep, 7]`` with time (column 0), the kinetic energy carried from
the previous step (column 4, J/mol per atom), the potential (column 5,
Hartree) and KE + (EPot - EPot0) * JOULEPERHARTREE (column 6). It runs on the
device when the energy/force routine is an ``EnergyAndForce`` closure of this
package; any other routine raises (there is no host integrator here).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from .params import IDEALGASR, JOULEPERHARTREE, PARAMS
from .systems import masses

_KINDS = {None: "nve", "Nose": "nose", "NoseHooverChain": "nhc"}


class DeviceMD:
    """tm_md: kind "nve" (VelocityVerletStep, SimpleMD.py:14-38), "nose"
    (NoseThermostat.step, :104-129) or "nhc" (Martyna chain, :206-320)."""

    def __init__(self, system, kind="nve", dt=0.5, T=300.0, chain=3):
        self.system = system
        self.ctx = system.ctx
        self.lib = system.lib
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.tm_md_create(system.h, _lib.TM_MD[kind], float(dt), float(T),
                                             int(chain), ctypes.byref(h)))
        self.h = h
        self.kind, self.dt, self.T = kind, dt, T

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        assert v.shape == (self.system.N, 3)
        self.ctx.check(self.lib.tm_md_set_velocities(self.h, ctypes.c_void_p(v.ctypes.data), 0))

    def velocities(self):
        v = np.empty((self.system.N, 3))
        self.ctx.check(self.lib.tm_md_get_velocities(self.h, ctypes.c_void_p(v.ctypes.data), 0))
        return v

    def run(self, nsteps, skin=0.0):
        """Integrate nsteps; returns the log [nsteps, 4] = (potential Hartree,
        KE J/mol per atom, conserved J/mol, T_eff K). skin > 0 (A): neighbour
        candidates within the cutoffs + skin are rebuilt only when atoms may
        have moved skin/2; the rows used by every step are still exact."""
        log = np.zeros((max(nsteps, 1), 4))
        self.ctx.check(self.lib.tm_md_run(self.h, int(nsteps), float(skin),
                                          ctypes.c_void_p(log.ctypes.data)))
        return log[:nsteps]

    def close(self):
        if self.h:
            self.lib.tm_md_destroy(self.h)
            self.h = None


def kinetic_energy(v, m):
    """Per-atom KE in J/mol (SimpleMD.py:40-51)."""
    return 0.5 * float(np.dot(np.einsum("ia,ia->i", v, v) * 1e10, m)) / len(m)


class VelocityVerlet:
    """SimpleMD.VelocityVerlet over the device integrator."""

    def __init__(self, f_, g0_, name_="", EandF_=None, cellsize_=None, seed=None):
        if EandF_ is None or not hasattr(EandF_, "system_for"):
            raise RuntimeError("VelocityVerlet here needs an EnergyAndForce closure of "
                               "tensormol_gb300 (the integrator runs on the device)")
        thermo = PARAMS.get("MDThermostat")
        if thermo not in _KINDS:
            raise ValueError(f"MDThermostat {thermo!r}: supported None, 'Nose', 'NoseHooverChain'")
        self.name = name_
        self.cellsize = cellsize_
        self.maxstep = int(PARAMS["MDMaxStep"])
        self.T = float(PARAMS["MDTemp"])
        self.dt = float(PARAMS["MDdt"])
        self.EnergyAndForce = EandF_
        self.atoms = np.array(g0_.atoms).copy()
        self.x = np.array(g0_.coords, dtype=np.float64).copy()
        self.EPot0, self.f0 = EandF_(self.x)
        self.EPot = self.EPot0
        self.m = masses(self.atoms)
        self.natoms = len(self.atoms)
        self.t = 0.0
        self.KE = 0.0
        rng = np.random.default_rng(seed)
        self.v = np.zeros(self.x.shape)
        if PARAMS.get("MDV0") == "Random":
            # Thermostat(m, v) rescales to MDTemp (SimpleMD.py:362-365)
            self.v = rng.normal(size=self.x.shape)
            ke = kinetic_energy(self.v, self.m)
            self.v *= np.sqrt(self.T / ((2.0 / 3.0) * ke / IDEALGASR))
        elif PARAMS.get("MDV0") == "Thermal":
            self.v = rng.normal(size=self.x.shape) * np.sqrt(1.38064852e-23 * self.T / self.m)[:, None]
        self.system = EandF_.system_for(self.x)
        self.md = DeviceMD(self.system, _KINDS[thermo], self.dt, self.T,
                           int(PARAMS.get("MNHChain", 3)))
        self.md.set_velocities(self.v)
        self.md_log = None

    def WriteTrajectory(self):
        """Append the current frame to ./results/MDTrajectory<name>.xyz with
        Time, KineticEnergy and PotEnergy (SimpleMD.py:383-389)."""
        from .model import Mol
        m = Mol(self.atoms, self.x)
        m.properties["Time"] = self.t
        m.properties["KineticEnergy"] = self.KE
        m.properties["PotEnergy"] = self.EPot
        m.WriteXYZfile("./results/", "MDTrajectory" + self.name)

    def Prop(self):
        """Propagate maxstep steps on the device (SimpleMD.py:391-424). With
        PARAMS["MDLogTrajectory"] the run pauses every third step to append a
        frame (positions come back only then); md_log is saved to
        ./results/MDLog<name>.txt every 500 steps and at the end."""
        if PARAMS.get("MDLogTrajectory"):
            logs = []
            done = 0
            while done < self.maxstep:
                n = min(3 if done else 1, self.maxstep - done)
                part = self.md.run(n)
                logs.append(part)
                done += n
                self.x = self.system.positions()
                self.t = (done - 1) * self.dt
                self.EPot = float(part[-1, 0])
                self.KE = float(part[-1, 1])
                if (done - 1) % 3 == 0:
                    self.WriteTrajectory()
            log = np.concatenate(logs)
        else:
            log = self.md.run(self.maxstep)
        self.md_log = np.zeros((self.maxstep, 7))
        self.md_log[:, 0] = np.arange(self.maxstep) * self.dt
        ke_prev = np.concatenate([[0.0], log[:-1, 1]])
        self.md_log[:, 4] = ke_prev
        self.md_log[:, 5] = log[:, 0]
        self.md_log[:, 6] = ke_prev + (log[:, 0] - self.EPot0) * JOULEPERHARTREE
        self.x = self.system.positions()
        self.v = self.md.velocities()
        self.t = (self.maxstep - 1) * self.dt
        self.EPot = float(log[-1, 0]) if self.maxstep else self.EPot0
        self.KE = float(log[-1, 1]) if self.maxstep else 0.0
        if PARAMS.get("MDLogTrajectory") or os.path.isdir("./results"):
            os.makedirs("./results", exist_ok=True)
            np.savetxt("./results/" + "MDLog" + self.name + ".txt", self.md_log)
        return self.md_log
