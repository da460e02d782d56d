"""Geometry optimisation and nudged elastic band drivers, device-resident.

The algorithms are the reference's own, restated on torch tensors so that the
positions, search directions and bead arrays stay in HBM and every energy or
energy+force evaluation is one fused call of the library (only scalars come
back for the line-search decisions):

* ``remove_invariant_force``   RemoveInvariantForce (Math/QuasiNewtonTools.py:551-577)
* ``ConjGradient``             Polak-Ribiere CG with the golden-section line
                               search (QuasiNewtonTools.py:350-450)
* ``VerletOptimizer``          momentum optimiser (Math/BFGS.py:39-76)
* ``SteepestDescent``          (BFGS.py:9-37)
* ``GeomOptimizer``            Opt.py:18-75 (``Opt`` returns the geometry
                               before the last step, as the reference does)
* ``NudgedElasticBand``        Simulations/Neb.py:17-230; all beads are
                               evaluated together as the molecules of one batch
                               (one fused launch sequence per evaluation).

Reference behaviour kept on purpose: the invariant-force projection is called
with the atomic numbers in the place of masses (Opt.py:39, Neb.py:139), the
inertia tensor is taken about the origin, and the "pseudo-inverse" is
U diag(1/s) V of the SVD (LinearOperations.py:16-23). One change: the line
search stops after ``max_iter`` rounds (the reference can loop forever once
its step has shrunk below 1e-5 while the first point stays lowest).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .params import JOULEPERHARTREE, PARAMS

GOLDENRATIO = (math.sqrt(5.0) + 1.0) / 2.0   # PhysicalData.py:28
_F64 = torch.float64


# ---------------------------------------------------------------------------
def remove_invariant_force(x, f, m):
    """Remove the net force and the rigid-rotation part of f (one structure
    [N, 3] or a batch [B, N, 3]); m are the per-atom weights [N]."""
    if not PARAMS.get("RemoveInvariant", True):
        return f
    squeeze = x.dim() == 2
    if squeeze:
        x, f = x[None], f[None]
    m = m.to(x)
    fnet = f.sum(1)                                                  # [B, 3]
    fnew = f - m[None, :, None] * fnet[:, None, :] / m.sum()
    torque = torch.cross(x, fnew, dim=2).sum(1)                      # [B, 3]
    # inertia tensor about the origin (QuasiNewtonTools.py:14-26)
    xx = x * x
    I = torch.zeros(x.shape[0], 3, 3, dtype=x.dtype, device=x.device)
    I[:, 0, 0] = (m * (xx[:, :, 1] + xx[:, :, 2])).sum(1)
    I[:, 1, 1] = (m * (xx[:, :, 0] + xx[:, :, 2])).sum(1)
    I[:, 2, 2] = (m * (xx[:, :, 1] + xx[:, :, 0])).sum(1)
    I[:, 0, 1] = -(m * x[:, :, 0] * x[:, :, 1]).sum(1)
    I[:, 0, 2] = -(m * x[:, :, 0] * x[:, :, 2]).sum(1)
    I[:, 1, 2] = -(m * x[:, :, 1] * x[:, :, 2]).sum(1)
    I[:, 1, 0] = I[:, 0, 1]
    I[:, 2, 0] = I[:, 0, 2]
    I[:, 2, 1] = I[:, 1, 2]
    U, s, V = torch.linalg.svd(I)
    sinv = torch.where(s.abs() > 1e-7, 1.0 / torch.where(s == 0, torch.ones_like(s), s),
                       torch.zeros_like(s))
    Iinv = U @ torch.diag_embed(sinv) @ V
    dwdt = (Iinv @ torque[:, :, None])[:, :, 0]                      # [B, 3]
    fcorr = m[None, :, None] * torch.cross(dwdt[:, None, :].expand_as(x), x, dim=2)
    out = fnew - fcorr
    return out[0] if squeeze else out


def _rms_rows(a):
    """sum over rows of the norm along axis 1, over shape[0] (the reference's
    rmsdist / rmsgrad, whatever the array rank)."""
    return float(torch.linalg.norm(a, dim=1).sum() / a.shape[0])


class ConjGradient:
    def __init__(self, f_, x0_, thresh_=0.0001, max_iter=200):
        self.EForce = f_
        self.Energy = lambda x: self.EForce(x, False)
        self.x0 = x0_.clone()
        self.xold = x0_.clone()
        self.e, self.gold = self.EForce(x0_)
        self.s = self.gold.clone()
        self.thresh = thresh_
        self.alpha = PARAMS["GSSearchAlpha"]
        self.max_iter = max_iter

    def BetaPR(self, g):
        betapr = float((g * (g - self.gold)).sum() / (self.gold * self.gold).sum())
        self.gold = g.clone()
        return max(0.0, betapr)

    def __call__(self, x0):
        e, g = self.EForce(x0)
        beta_n = self.BetaPR(g)
        self.s = g + beta_n * self.s
        self.xold = self.LineSearch(x0, self.s, self.thresh)
        return self.xold, e, g

    def LineSearch(self, x0_, p_, thresh=0.0001):
        a = x0_
        b = x0_ + self.alpha * p_
        c = b - (b - a) / GOLDENRATIO
        d = a + (b - a) / GOLDENRATIO
        fa, fb, fc, fd = self.Energy(a), self.Energy(b), self.Energy(c), self.Energy(d)
        rmsdist = 10.0
        k = 0
        while rmsdist > thresh and k < self.max_iter:
            if fa < fc and fa < fd and fa < fb:        # overstep
                if self.alpha > 0.00001:
                    self.alpha /= 1.8001
                elif self.alpha >= 0.0001:
                    return a
                a = x0_
                b = x0_ + self.alpha * p_
                c = b - (b - a) / GOLDENRATIO
                d = a + (b - a) / GOLDENRATIO
                fa, fb, fc, fd = self.Energy(a), self.Energy(b), self.Energy(c), self.Energy(d)
            elif fb < fc and fb < fd and fb < fa:      # understep: take the midpoint
                if self.alpha < 100.0:
                    self.alpha *= 1.8
                a = x0_
                b = x0_ + self.alpha * p_
                return (b + a) / 2
            elif fc < fd:
                b = d
                c = b - (b - a) / GOLDENRATIO
                d = a + (b - a) / GOLDENRATIO
                fb = fd
                fc, fd = self.Energy(c), self.Energy(d)
            else:
                a = c
                c = b - (b - a) / GOLDENRATIO
                d = a + (b - a) / GOLDENRATIO
                fa = fc
                fc, fd = self.Energy(c), self.Energy(d)
            rmsdist = _rms_rows(a - b)
            k += 1
        return (b + a) / 2


class SteepestDescent:
    def __init__(self, f_, x0_):
        self.step = 0
        self.x0 = x0_.clone()
        self.EForce = f_

    def __call__(self, new_vec_):
        e, g = self.EForce(new_vec_)
        self.step += 1
        return new_vec_ + PARAMS["SDStep"] * g, e, g


class VerletOptimizer:
    def __init__(self, f_, x0_):
        self.step = 0
        self.x0 = x0_.clone()
        self.v = torch.zeros_like(x0_)
        self.a = torch.zeros_like(x0_)   # never updated, as in BFGS.py:51,68
        self.dt = 0.1
        self.EForce = f_

    def __call__(self, x_):
        x = x_ + self.v * self.dt + 0.5 * self.a * self.dt * self.dt
        e, f_x_ = self.EForce(x)
        self.v = self.v + 0.5 * (self.a + f_x_) * self.dt
        if float((self.v * f_x_).sum()) < 0:
            self.v = self.v * 0.0
            self.a = self.a * 0.0
        self.step += 1
        return x, e, f_x_


# ---------------------------------------------------------------------------
class _Evaluator:
    """Energies (Hartree) and forces (J/mol/A) of B copies of one molecule
    (B = 1 for an optimisation, the beads for a band) as one fused batch,
    with device-resident torch positions [B, N, 3]. Falls back to calling a
    foreign EnergyAndForce routine per structure."""

    def __init__(self, f_, atoms, nbatch, device):
        self.f = f_
        self.atoms = np.asarray(atoms, dtype=np.int32)
        self.N = len(self.atoms)
        self.B = nbatch
        self.system = None
        self.device = device
        model = getattr(f_, "model", None)
        if model is not None and device.type == "cuda":
            Z = np.tile(self.atoms, nbatch)
            off = np.arange(nbatch + 1, dtype=np.int64) * self.N
            self.system = model.system(None, Z, off)
            self.E = torch.zeros((nbatch, 4), dtype=_F64, device=device)
            self.F = torch.zeros((nbatch * self.N, 3), dtype=_F64, device=device)
        self.calls = 0

    def __call__(self, x, do_force=True):
        """x [B, N, 3] -> (E [B] host float64 array, F [B, N, 3] torch or None)."""
        self.calls += 1
        if self.system is not None:
            from . import _lib
            xc = x.reshape(-1, 3).contiguous()
            lib_stream = torch.cuda.ExternalStream(int(self.system.ctx.stream or 0), device=x.device)
            lib_stream.wait_stream(torch.cuda.current_stream(x.device))
            flags = 0 if do_force else _lib.TM_F_ENERGY_ONLY
            self.system.energy_force_device(xc.data_ptr(), self.E.data_ptr(), self.F.data_ptr(), flags)
            torch.cuda.current_stream(x.device).wait_stream(lib_stream)
            E = self.E[:, 0].cpu().numpy().copy()
            return E, (self.F.view(self.B, self.N, 3).clone() if do_force else None)
        E = np.zeros(self.B)
        F = torch.zeros_like(x) if do_force else None
        for b in range(self.B):
            xb = x[b].detach().cpu().numpy()
            if do_force:
                e, fb = self.f(xb, True)
                F[b] = torch.as_tensor(np.asarray(fb), dtype=x.dtype, device=x.device)
            else:
                e = self.f(xb, False)
            E[b] = float(np.asarray(e).reshape(-1)[0])
        return E, F

    def close(self):
        if self.system is not None:
            self.system.close()
            self.system = None


def _device_for(f_):
    return torch.device("cuda") if getattr(f_, "model", None) is not None and torch.cuda.is_available() \
        else torch.device("cpu")


class GeomOptimizer:
    """Opt.py:18-75 over the device evaluator."""

    def __init__(self, f_):
        self.thresh = PARAMS["OptThresh"]
        self.maxstep = PARAMS["OptMaxStep"]
        self.fscale = PARAMS["OptStepSize"]
        self.momentum = PARAMS["OptMomentum"]
        self.momentum_decay = PARAMS["OptMomentumDecay"]
        self.max_opt_step = PARAMS["OptMaxCycles"]
        self.step = self.maxstep
        self.EnergyAndForce = f_
        self.m = None
        self.history = []      # (energy at the start of the step, coords after it)

    def WrappedEForce(self, x_, DoForce=True):
        E, F = self._ev(x_[None], DoForce)
        if DoForce:
            frc = remove_invariant_force(x_, F[0], self._w)
            return float(E[0]), frc / JOULEPERHARTREE
        return float(E[0])

    def Opt(self, m_, filename="OptLog", Debug=False):
        from .model import Mol
        device = _device_for(self.EnergyAndForce)
        self._ev = _Evaluator(self.EnergyAndForce, m_.atoms, 1, device)
        self._w = torch.as_tensor(np.asarray(m_.atoms, dtype=np.float64), device=device)
        x = torch.as_tensor(np.asarray(m_.coords, dtype=np.float64), device=device).clone()
        self.m = Mol(m_.atoms, m_.coords)
        rmsdisp = 10.0
        rmsgrad = 10.0
        step = 0
        prev = x.clone()
        CG = ConjGradient(self.WrappedEForce, x)
        while step < self.max_opt_step and rmsgrad > self.thresh and (rmsdisp > 0.000001 or step < 5):
            prev = x.clone()
            x, energy, frc = CG(x)
            rmsgrad = _rms_rows(frc)
            rmsdisp = _rms_rows(x - prev)
            self.history.append((energy, x.cpu().numpy()))
            step += 1
        self.m.coords = x.cpu().numpy()
        self.evaluations = self._ev.calls
        self._ev.close()
        return Mol(m_.atoms, prev.cpu().numpy())


class NudgedElasticBand:
    """Neb.py:17-230 with all beads evaluated as one batch."""

    def __init__(self, f_, g0_, g1_, name_="Neb", thresh_=None, nbeads_=None):
        self.name = name_
        self.thresh = PARAMS["OptThresh"] if thresh_ is None else thresh_
        self.max_opt_step = PARAMS["OptMaxCycles"]
        self.nbeads = PARAMS["NebNumBeads"] if nbeads_ is None else nbeads_
        self.k = PARAMS["NebK"]
        self.f = f_
        self.atoms = np.asarray(g0_.atoms).copy()
        self.natoms = len(self.atoms)
        device = _device_for(f_)
        self.device = device
        c0 = torch.as_tensor(np.asarray(g0_.coords, dtype=np.float64), device=device)
        c1 = torch.as_tensor(np.asarray(g1_.coords, dtype=np.float64), device=device)
        ls = torch.linspace(0.0, 1.0, self.nbeads, dtype=_F64, device=device)
        self.beads = (1.0 - ls)[:, None, None] * c0[None] + ls[:, None, None] * c1[None]
        self.Fs = torch.zeros_like(self.beads)
        self.Ss = torch.zeros_like(self.beads)
        self.Ts = torch.zeros_like(self.beads)
        self.Es = np.zeros(self.nbeads)
        self.Esi = np.zeros(self.nbeads)
        self.step = 0
        self.TSI = 0
        self._w = torch.as_tensor(self.atoms.astype(np.float64), device=device)
        self._ev = _Evaluator(f_, self.atoms, self.nbeads, device)
        solver = PARAMS["NebSolver"]
        if solver == "SD":
            self.Solver = SteepestDescent(self.WrappedEForce, self.beads)
        elif solver == "Verlet":
            self.Solver = VerletOptimizer(self.WrappedEForce, self.beads)
        elif solver == "CG":
            self.Solver = ConjGradient(self.WrappedEForce, self.beads)
        else:
            raise Exception("Missing Neb Solver")

    # -- band geometry, vectorised over beads --------------------------------
    def Tangents(self, beads_):
        t = torch.zeros_like(beads_)
        if self.nbeads > 2:
            tt = beads_[2:] - beads_[:-2]           # (b_i - b_{i-1}) + (b_{i+1} - b_i)
            t[1:-1] = tt / torch.sqrt((tt * tt).sum((1, 2)))[:, None, None]
        return t

    def SpringEnergy(self, beads_):
        d = beads_[1:] - beads_[:-1]
        return float(0.5 * self.k * self.nbeads * (d * d).sum())

    def SpringDerivs(self, beads_):
        s = torch.zeros_like(beads_)
        s[1:-1] = self.k * self.nbeads * (2.0 * beads_[1:-1] - beads_[2:] - beads_[:-2])
        return s

    @staticmethod
    def _dot(v, t):
        return (v * t).sum((1, 2))[:, None, None]

    def WrappedEForce(self, beads_, DoForce=True):
        E, F = self._ev(beads_, DoForce)
        self.Es = E.copy()
        if not DoForce:
            return float(self.Es.sum()) + self.SpringEnergy(beads_)
        F[0] = 0.0
        F[-1] = 0.0
        self.Fs = F
        t = self.Tangents(beads_)
        self.Ts = t
        S = -1.0 * self.SpringDerivs(beads_)
        Spara = t * self._dot(S, t)
        self.Ss = Spara
        Fperp = F - t * self._dot(F, t)
        Fneb = Spara + Fperp
        if PARAMS["NebClimbingImage"] and self.step > 10 and 0 < self.TSI < self.nbeads - 1:
            i = self.TSI
            Fneb[i] = F[i] - 2.0 * (F[i] * t[i]).sum() * t[i]
        Fneb = remove_invariant_force(beads_, Fneb, self._w) / JOULEPERHARTREE
        TE = float(self.Es.sum()) + self.SpringEnergy(beads_)
        return TE, Fneb

    def IntegrateEnergy(self):
        self.Esi[0] = self.Es[0]
        dR = self.beads[1:] - self.beads[:-1]
        dV = -1.0 * (self.Fs[1:] + self.Fs[:-1]) / 2.0
        inc = (dR * dV).sum((1, 2)).cpu().numpy()
        for i in range(1, self.nbeads):
            self.Esi[i] = self.Esi[i - 1] + inc[i - 1]

    def Opt(self, filename="Neb", Debug=False):
        self.step = 0
        self.Fs = torch.ones_like(self.beads)
        self.PES = np.zeros((self.max_opt_step, self.nbeads))
        while self.step < self.max_opt_step and float(torch.sqrt((self.Fs * self.Fs).mean())) > self.thresh:
            self.beads, energy, self.Fs = self.Solver(self.beads)
            self.PES[self.step] = self.Es.copy()
            self.IntegrateEnergy()
            self.TSI = int(np.argmax(self.Es))
            self.step += 1
        return self.beads.cpu().numpy()

    def close(self):
        self._ev.close()
