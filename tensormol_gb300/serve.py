"""Continuous-batching serving loop over ``tm_serve`` (libtmgpu).

Requests are energy+force evaluations ("ef", one step), NVE molecular
dynamics runs ("md", ``nsteps`` velocity-Verlet steps of SimpleMD.py:14-38) or
geometry optimisations ("opt": FIRE steps until the largest atomic force is
below ``fmax`` eV/A, at most ``nsteps``).
Every request in flight is one molecule of a single device-resident batch, and
one ``Server.step()`` advances all of them with one fused energy+force
evaluation. Between steps, finished requests leave and waiting requests are
admitted first-come-first-served while the batch stays within the capacity
allocated once against an HBM budget (atoms and molecule slots); the
positions, velocities and accelerations of requests that stay are re-ordered on
the device, never copied through the host. Step latencies are recorded for
p50/p99 reporting.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from .params import EV_PER_HARTREE, JOULEPERHARTREE

_F64 = np.float64


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Request:
    """One serving request: a molecule (Z, x[N,3] in Angstrom), its kind, the
    number of steps, and optionally initial velocities (A/fs)."""

    _next = 0

    def __init__(self, Z, x, kind="md", nsteps=50, v=None, arrival=0.0, fmax=0.05):
        if kind not in _lib.TM_SERVE:
            raise ValueError("kind must be 'ef', 'md' or 'opt'")
        self.Z = np.ascontiguousarray(Z, dtype=np.int32)
        self.x0 = np.ascontiguousarray(x, dtype=_F64).reshape(-1, 3)
        self.v0 = (np.zeros_like(self.x0) if v is None
                   else np.ascontiguousarray(v, dtype=_F64).reshape(-1, 3))
        self.kind = kind
        self.nsteps = 1 if kind == "ef" else int(nsteps)
        self.fmax = float(fmax)          # eV/A, optimisation requests
        self.fmax_last = None
        self.converged = False
        self.error = None                # set when the request had to be dropped
        self.arrival = float(arrival)
        self.rid = Request._next
        Request._next += 1
        self.steps_done = 0
        self.overtaken = 0        # times a later request was admitted first
        self.energies = []        # per step: (Etotal, Ebp, Ecc, Evdw) Hartree
        self.x = self.v = self.F = None
        self.t_submit = self.t_admit = self.t_done = None

    @property
    def natoms(self):
        return int(self.Z.shape[0])

    @property
    def done(self):
        return self.steps_done >= self.nsteps or self.converged or self.error is not None


class Server:
    """Continuous batching over one tm_serve. ``max_atoms``/``max_mols`` bound
    the batch; ``capacity_for_budget`` derives ``max_atoms`` from an HBM byte
    budget.

    admission: "fifo" admits strictly in arrival order (a request that does not
    fit blocks the ones behind it); "first_fit" looks at up to ``lookahead``
    waiting requests in arrival order and admits every one that fits, so a
    large request at the head does not leave the batch half empty, but a
    request that has been overtaken ``max_overtakes`` times stops later ones
    from passing it until it is admitted (no request waits forever)."""

    def __init__(self, model, max_atoms=65536, max_mols=512, dt=0.5, admission="fifo",
                 lookahead=64, max_overtakes=8):
        if admission not in ("fifo", "first_fit"):
            raise ValueError("admission must be 'fifo' or 'first_fit'")
        self.admission = admission
        self.lookahead = int(lookahead)
        self.max_overtakes = int(max_overtakes)
        self.model = model
        self.ctx = model.ctx
        self.lib = model.lib
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.tm_serve_create(model.h, int(max_atoms), int(max_mols), float(dt),
                                                ctypes.byref(h)))
        self.h = h
        self.max_atoms, self.max_mols, self.dt = int(max_atoms), int(max_mols), float(dt)
        b = ctypes.c_size_t()
        self.ctx.check(self.lib.tm_serve_info(h, None, None, None, None, ctypes.byref(b)))
        self.bytes = int(b.value)
        self.pending = []         # FIFO of submitted requests
        self.active = []          # requests in the current layout, in layout order
        self.finished = []
        self.step_ms = []         # wall time of each step (admission + layout + step)
        self.step_atoms = []
        self.step_info = []       # (relayout?, layout ms, step ms, atoms) per step
        self.atom_steps = 0

    @staticmethod
    def capacity_for_budget(model, budget_bytes, max_mols=512, dt=0.5):
        """Largest max_atoms whose buffers fit in budget_bytes, from two probe
        allocations (the footprint is affine in the atom capacity)."""
        sizes = []
        for n in (4096, 8192):
            s = Server(model, n, max_mols, dt)
            sizes.append(s.bytes)
            s.close()
        per_atom = (sizes[1] - sizes[0]) / 4096.0
        fixed = sizes[0] - 4096 * per_atom
        return int(max(0, (budget_bytes - fixed) / per_atom))

    def submit(self, req, now=None):
        req.t_submit = time.perf_counter() if now is None else now
        self.pending.append(req)

    # -- batch composition ----------------------------------------------------
    def _relayout(self, keep, admit):
        old_off = {}
        o = 0
        for r in self.active:
            old_off[r.rid] = o
            o += r.natoms
        reqs = keep + admit
        nmol = len(reqs)
        if nmol == 0:
            self.ctx.check(self.lib.tm_serve_layout(self.h, 0, None, None, None, None, None, None))
            self.active = []
            return
        Z = np.concatenate([r.Z for r in reqs]).astype(np.int32)
        counts = np.fromiter((r.natoms for r in reqs), dtype=np.int64, count=nmol)
        offs = np.zeros(nmol + 1, dtype=np.int64)
        np.cumsum(counts, out=offs[1:])
        mode = np.fromiter((_lib.TM_SERVE[r.kind] for r in reqs), dtype=np.int32, count=nmol)
        # gather map, vectorised: kept rows point at their old index, the k-th
        # new row is -(k+1) (new rows numbered in layout order)
        is_new = np.fromiter((r.rid not in old_off for r in reqs), dtype=bool, count=nmol)
        new_counts = np.where(is_new, counts, 0)
        new_start = np.cumsum(new_counts) - new_counts
        base = np.where(is_new, -1 - new_start,
                        np.fromiter((old_off.get(r.rid, 0) for r in reqs), dtype=np.int64, count=nmol))
        local = np.arange(int(offs[-1]), dtype=np.int64) - np.repeat(offs[:-1], counts)
        src = (np.repeat(base, counts) + np.where(np.repeat(is_new, counts), -local, local)).astype(np.int32)
        xn = [r.x0 for r in admit]
        vn = [r.v0 for r in admit]
        xn = np.ascontiguousarray(np.concatenate(xn)) if xn else None
        vn = np.ascontiguousarray(np.concatenate(vn)) if vn else None
        self.ctx.check(self.lib.tm_serve_layout(self.h, nmol, _p(Z), _p(offs), _p(mode), _p(src),
                                                _p(xn), _p(vn)))
        self.active = reqs

    def _admit(self, keep):
        atoms = sum(r.natoms for r in keep)
        slots = len(keep)
        admit = []
        if self.admission == "fifo":
            while self.pending:
                r = self.pending[0]
                if r.natoms > self.max_atoms:
                    raise ValueError(f"request of {r.natoms} atoms exceeds the capacity {self.max_atoms}")
                if atoms + r.natoms > self.max_atoms or slots + 1 > self.max_mols:
                    break
                self.pending.pop(0)
                atoms += r.natoms
                slots += 1
                admit.append(r)
            return admit
        rest, skipped = [], []
        last_admitted = -1
        blocked = False       # a request overtaken too often holds back later ones
        for i, r in enumerate(self.pending):
            if r.natoms > self.max_atoms:
                raise ValueError(f"request of {r.natoms} atoms exceeds the capacity {self.max_atoms}")
            fits = atoms + r.natoms <= self.max_atoms and slots + 1 <= self.max_mols
            if fits and not blocked and i < self.lookahead:
                atoms += r.natoms
                slots += 1
                admit.append(r)
                last_admitted = i
                continue
            if not fits and not blocked and i < self.lookahead:
                if r.overtaken >= self.max_overtakes:
                    blocked = True
                else:
                    skipped.append((i, r))
            rest.append(r)
        # a request counts as overtaken when one behind it got in
        for i, r in skipped:
            if i < last_admitted:
                r.overtaken += 1
        self.pending = rest
        return admit

    # -- one step -------------------------------------------------------------
    def step(self):
        """Admit, re-lay out if the membership changed, advance every request
        by one step, retire finished ones. Returns the number of requests that
        were stepped."""
        t0 = time.perf_counter()
        keep = [r for r in self.active if not r.done]
        admit = self._admit(keep)
        relayout = bool(admit or len(keep) != len(self.active))
        if relayout:
            self._relayout(keep, admit)
            for r in admit:
                r.t_admit = t0
        t1 = time.perf_counter()
        if not self.active:
            return 0
        E = np.zeros((len(self.active), 4))
        fmax = np.zeros(len(self.active))
        try:
            self.ctx.check(self.lib.tm_serve_step(self.h, _p(E), _p(fmax)))
        except _lib.TmError as exc:
            # non-finite positions belong to one request (molecules never
            # interact): drop those requests, the others' step is valid
            if exc.code != _lib.ERROR_CODES["TM_E_NONFINITE"]:
                raise
            for q, r in enumerate(self.active):
                x = np.empty((r.natoms, 3))
                self.ctx.check(self.lib.tm_serve_read(self.h, q, _p(x), None, None))
                if not np.all(np.isfinite(x)):
                    r.error = "non-finite positions"
        natoms = 0
        for r, e, fm in zip(self.active, E, fmax):   # rows of fresh arrays: no copies
            r.steps_done += 1
            r.energies.append(e)
            natoms += r.natoms
            if r.kind == "opt":
                # the force of the positions just evaluated (the step's x)
                r.fmax_last = fm / JOULEPERHARTREE * EV_PER_HARTREE
                r.converged = r.fmax_last <= r.fmax
        for q, r in enumerate(self.active):
            if r.done:
                r.x = np.empty((r.natoms, 3))
                r.v = np.empty((r.natoms, 3))
                r.F = np.empty((r.natoms, 3))
                self.ctx.check(self.lib.tm_serve_read(self.h, q, _p(r.x), _p(r.v), _p(r.F)))
                r.t_done = time.perf_counter()
                self.finished.append(r)
        t2 = time.perf_counter()
        self.step_ms.append((t2 - t0) * 1e3)
        self.step_info.append((relayout, (t1 - t0) * 1e3, (t2 - t1) * 1e3, natoms))
        self.step_atoms.append(natoms)
        self.atom_steps += natoms
        return len(self.active)

    def drain(self):
        """Step until nothing is pending or in flight."""
        while self.pending or any(not r.done for r in self.active):
            self.step()
        # retire the last finished requests from the layout
        if self.active:
            self._relayout([], [])

    def run_arrivals(self, requests, t_start=None):
        """Serve requests whose ``arrival`` times (s, relative to t_start) are
        honoured on the wall clock; returns the wall time taken."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t_start = time.perf_counter() if t_start is None else t_start
        i = 0
        while i < len(reqs) or self.pending or any(not r.done for r in self.active):
            now = time.perf_counter() - t_start
            while i < len(reqs) and reqs[i].arrival <= now:
                self.submit(reqs[i], now=t_start + reqs[i].arrival)
                i += 1
            if not self.pending and all(r.done for r in self.active) and i < len(reqs):
                if self.active:
                    self._relayout([], [])
                time.sleep(max(0.0, reqs[i].arrival - (time.perf_counter() - t_start)))
                continue
            self.step()
        if self.active:
            self._relayout([], [])
        return time.perf_counter() - t_start

    def stats(self, wall_s):
        ms = np.asarray(self.step_ms)
        return {"steps": int(ms.size),
                "p50_ms": float(np.percentile(ms, 50)) if ms.size else None,
                "p99_ms": float(np.percentile(ms, 99)) if ms.size else None,
                "atom_steps": int(self.atom_steps),
                "atom_steps_per_s": self.atom_steps / wall_s if wall_s > 0 else None,
                "mean_batch_atoms": float(np.mean(self.step_atoms)) if self.step_atoms else 0.0}

    def close(self):
        if self.h:
            self.lib.tm_serve_destroy(self.h)
            self.h = None
