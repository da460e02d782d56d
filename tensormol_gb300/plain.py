"""The plain-autograd form of the energy+force evaluation, for comparison.

This is the reference's own structure (TFDescriptors/RawSymFunc.py:868-963,
1307-1414, 1757-1810; TFNetworks/TFBehlerParinelloSymEE.py:884-1015, forces by
tf.gradients at :1490) written as framework ops on the GPU: gathers over
materialised pair / triple / Coulomb-pair lists, scatter-adds into descriptor
rows, per-element FP32 matmuls, and torch.autograd.grad for the forces. It uses
the same neighbour lists (built by libtmgpu and exported to device tensors), so
the only difference from the fused path is how the arithmetic and its
derivative are executed. Pair vectors are formed in FP64 and cast to FP32.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .params import BOHRPERA, JOULEPERHARTREE, ani1_grids, coulomb_constants, element_pairs, vdw_tables


class PlainAutograd:
    def __init__(self, model, weights):
        self.m = model
        p = model.p
        self.p = p
        self.eles = model.eles
        self.nele = len(self.eles)
        self.nelep = len(element_pairs(self.eles))
        dev = torch.device("cuda")
        self.dev = dev
        rs_r, rs_a, th = ani1_grids(p)
        self.rs_r = torch.tensor(rs_r, dtype=torch.float32, device=dev)
        self.rs_a = torch.tensor(rs_a, dtype=torch.float32, device=dev)
        self.th = torch.tensor(th, dtype=torch.float32, device=dev)
        self.cc = coulomb_constants(p)
        c6, r0 = vdw_tables(self.eles, p)
        self.c6 = torch.tensor(c6, dtype=torch.float32, device=dev)
        self.r0 = torch.tensor(r0, dtype=torch.float32, device=dev)
        self.W = {net: {e: [(torch.tensor(np.asarray(Wm), dtype=torch.float32, device=dev),
                             torch.tensor(np.asarray(b), dtype=torch.float32, device=dev))
                            for (Wm, b) in weights[net][e]] for e in self.eles} for net in ("E", "Q")}
        act = p["NeuronType"]
        a = float(p["sigmoid_alpha"])
        if act == "relu":
            self.act = torch.relu
        elif act == "sigmoid_with_param":
            # log(1 + exp(a z)) / a; above a z = 20 it equals z to 2e-9 / a, and
            # exp(a z) would overflow FP32 beyond a z = 88
            self.act = lambda z: torch.nn.functional.softplus(z, beta=a, threshold=20.0)
        elif act == "tanh":
            self.act = torch.tanh
        elif act == "softplus":
            self.act = torch.nn.functional.softplus
        else:
            self.act = torch.nn.functional.elu

    def prepare(self, system):
        """Exports the lists of ``system`` (a tensormol_gb300.model.System whose
        lists are current) to device index tensors in global atom numbering."""
        dev = self.dev
        off = torch.tensor(system.offsets, dtype=torch.int64, device=dev)
        c = system.nlist_counts()
        P, T, Pee = c["pairs"], c["triples"], c["ee_pairs"]
        radp = torch.zeros((P, 4), dtype=torch.int64, device=dev)
        angt = torch.zeros((T, 5), dtype=torch.int64, device=dev)
        eep = torch.zeros((max(Pee, 1), 3), dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        ctx = system.ctx
        ctx.check(system.lib.tm_system_export_nlist(system.h, ctypes.c_void_p(radp.data_ptr()),
                                                    ctypes.c_void_p(angt.data_ptr()), None, None, 1))
        ctx.check(system.lib.tm_system_export_ee(system.h, ctypes.c_void_p(eep.data_ptr()), Pee, 1))
        torch.cuda.synchronize()
        eep = eep[:Pee]
        self.pi = off[radp[:, 0]] + radp[:, 1]
        self.pj = off[radp[:, 0]] + radp[:, 2]
        self.pl = radp[:, 3]
        self.ti = off[angt[:, 0]] + angt[:, 1]
        self.tj = off[angt[:, 0]] + angt[:, 2]
        self.tk = off[angt[:, 0]] + angt[:, 3]
        self.tl = angt[:, 4]
        self.ei = off[eep[:, 0]] + eep[:, 1]
        self.ej = off[eep[:, 0]] + eep[:, 2]
        self.emol = eep[:, 0]
        self.N = system.N
        self.nmol = system.nmol
        Z = torch.tensor(system.Z, dtype=torch.int64, device=dev)
        self.Z = Z
        self.eidx = torch.zeros_like(Z)
        for i, e in enumerate(self.eles):
            self.eidx[Z == e] = i
        counts = np.diff(system.offsets)
        self.mol = torch.tensor(np.repeat(np.arange(self.nmol), counts), dtype=torch.int64, device=dev)
        self.natom = torch.tensor(counts, dtype=torch.float32, device=dev)
        self.rows = {e: torch.nonzero(Z == e).flatten() for e in self.eles}
        return dict(pairs=P, triples=T, ee_pairs=Pee)

    def energy_force(self, x):
        """x: [N,3] float64 CUDA tensor. Returns (Etotal[nmol] float64, F[N,3]
        float64 in J/mol/A)."""
        X = x.detach().requires_grad_(True)
        p = self.p
        nrow = self.N
        # radial (RawSymFunc.py:1757-1810)
        R = (X[self.pi] - X[self.pj]).float()
        r = torch.sqrt((R * R).sum(1) + 1e-27)
        t = r[:, None] - self.rs_r[None, :]
        g = torch.exp(-p["AN1_eta"] * t * t) * (0.5 * (torch.cos(3.14159265359 * r / p["AN1_r_Rc"]) + 1.0))[:, None]
        Gr = torch.zeros(nrow * self.nele, g.shape[1], device=self.dev).index_add(0, self.pi * self.nele + self.pl, g)
        # angular (RawSymFunc.py:868-963)
        Rij = (X[self.ti] - X[self.tj]).float()
        Rik = (X[self.ti] - X[self.tk]).float()
        rij = torch.sqrt((Rij * Rij).sum(1) + 1e-27)
        rik = torch.sqrt((Rik * Rik).sum(1) + 1e-27)
        c = ((Rij * Rik).sum(1) / (rij * rik)).clamp(-1.0 + 1e-7, 1.0 - 1e-7)
        theta = torch.acos(c)
        T = torch.cos(theta[:, None] - self.th[None, :])
        zeta = p["AN1_zeta"]
        fac1 = (2.0 ** (1.0 - zeta)) * torch.pow(1.0 + T, zeta)
        u = ((rij + rik) / 2.0)[:, None] - self.rs_a[None, :]
        fac2 = torch.exp(-p["AN1_eta"] * u * u)
        fc = 0.5 * (torch.cos(3.14159265359 * rij / p["AN1_a_Rc"]) + 1.0) * \
            0.5 * (torch.cos(3.14159265359 * rik / p["AN1_a_Rc"]) + 1.0)
        ga = (fac1[:, :, None] * fac2[:, None, :] * fc[:, None, None]).reshape(-1, 64)
        Ga = torch.zeros(nrow * self.nelep, 64, device=self.dev).index_add(0, self.ti * self.nelep + self.tl, ga)
        G = torch.cat([Gr.reshape(nrow, -1), Ga.reshape(nrow, -1)], 1)
        # per-element networks (TFBehlerParinelloSymEE.py:884-1015)
        Ea = torch.zeros(nrow, device=self.dev)
        qa = torch.zeros(nrow, device=self.dev)
        for e in self.eles:
            idx = self.rows[e]
            if idx.numel() == 0:
                continue
            for net, out in (("E", Ea), ("Q", qa)):
                h = G[idx]
                layers = self.W[net][e]
                for (Wm, b) in layers[:-1]:
                    h = self.act(h @ Wm + b)
                Wm, b = layers[-1]
                val = (h @ Wm + b).flatten()
                if net == "E":
                    Ea = Ea.index_put((idx,), val)
                else:
                    qa = qa.index_put((idx,), val)
        net_q = torch.zeros(self.nmol, device=self.dev).index_add(0, self.mol, qa)
        qs = qa - (net_q / self.natom)[self.mol]
        Ebp = torch.zeros(self.nmol, device=self.dev).index_add(0, self.mol, Ea)
        # DSF/elu Coulomb + C6 vdW over the materialised pair list
        cc = self.cc
        D = (X[self.ei] - X[self.ej]).float()
        rA = torch.sqrt((D * D).sum(1) + 1e-27)
        rb = rA * BOHRPERA
        qq = qs[self.ei] * qs[self.ej]
        xx = cc["alpha"] * cc["r_lr"]
        zz = float(np.float64(__import__("math").erfc(xx)) / cc["r_lr"])
        yy = 1.1283791671 * cc["alpha"] * float(np.exp(-xx * xx)) / cc["r_lr"]
        lr = qq * (torch.special.erfc(cc["alpha"] * rb) / rb - zz + (rb - cc["r_lr"]) * (zz / cc["r_lr"] + yy))
        lr = torch.where(rb > cc["r_lr"], torch.zeros_like(lr), lr)
        sr = qq * (cc["elu_a"] * (torch.exp(rb - cc["r_sr"]) - 1.0) + cc["elu_shift"])
        K = torch.where(rb > cc["r_sr"], lr, sr)
        Ecc = torch.zeros(self.nmol, device=self.dev).index_add(0, self.emol, K)
        r2 = rA * (BOHRPERA * BOHRPERA)
        tt = r2 / (p["Poly_Width"] * BOHRPERA)
        cut = torch.where(tt > 1.0, torch.ones_like(tt), torch.where(tt > 0.0, -tt * tt * (2.0 * tt - 3.0), torch.zeros_like(tt)))
        a, b2 = self.eidx[self.ei], self.eidx[self.ej]
        kv = -cut * torch.sqrt(self.c6[a] * self.c6[b2]) / torch.pow(r2, 6.0) / (
            1.0 + 6.0 * torch.pow(r2 / (self.r0[a] + self.r0[b2]), -12.0))
        Ev = torch.zeros(self.nmol, device=self.dev).index_add(0, self.emol, kv)
        E = Ebp.double() + Ecc.double() + Ev.double()
        g, = torch.autograd.grad(E.sum(), X)
        return E.detach(), -JOULEPERHARTREE * g
