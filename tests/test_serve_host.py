"""Host logic of the serving loop on CPU, against a stand-in for the C ABI.

The stand-in keeps per-atom positions in numpy and applies tm_serve_layout's
gather rule (src >= 0: previous index; -(k+1): k-th new row), and a step
moves every atom of an "md" molecule by +1 along x. The tests check that the
loop's layouts keep each request's rows, admit first-come-first-served within
the atom and slot capacity, and retire requests after their step count.
"""
import ctypes

import numpy as np

from tensormol_gb300 import _lib, serve


class _Ctx:
    def check(self, rc):
        assert rc == 0


def _arr(p, dtype, n):
    if p is None:
        return None
    return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(dtype)), shape=(n,))


class _FakeLib:
    def __init__(self):
        self.x = np.zeros((0, 3))
        self.mode = np.zeros(0, np.int32)
        self.offs = np.zeros(1, np.int64)
        self.layouts = 0

    def tm_serve_create(self, model_h, max_atoms, max_mols, dt, out):
        return 0

    def tm_serve_info(self, h, a, b, c, d, nbytes):
        nbytes._obj.value = 1234
        return 0

    def tm_serve_layout(self, h, nmol, Z, offs, mode, src, xn, vn):
        self.layouts += 1
        if nmol == 0:
            self.x = np.zeros((0, 3))
            return 0
        offs = _arr(offs, ctypes.c_int64, nmol + 1).copy()
        n = int(offs[-1])
        src = _arr(src, ctypes.c_int32, n).copy()
        nnew = int((src < 0).sum())
        xn = _arr(xn, ctypes.c_double, 3 * nnew).reshape(-1, 3) if nnew else None
        x = np.empty((n, 3))
        for i, s in enumerate(src):
            x[i] = self.x[s] if s >= 0 else xn[-s - 1]
        self.x, self.offs = x, offs
        self.mode = _arr(mode, ctypes.c_int32, nmol).copy()
        return 0

    def tm_serve_step(self, h, E, fmax=None):
        E = _arr(E, ctypes.c_double, 4 * len(self.mode)).reshape(-1, 4)
        for q, md in enumerate(self.mode):
            a, b = self.offs[q], self.offs[q + 1]
            if md == _lib.TM_SERVE["md"]:
                self.x[a:b, 0] += 1.0
            E[q] = (b - a, 0, 0, 0)
        if fmax is not None:     # optimisation requests: converged at once
            _arr(fmax, ctypes.c_double, len(self.mode))[:] = 0.0
        return 0

    def tm_serve_read(self, h, q, x, v, F):
        a, b = self.offs[q], self.offs[q + 1]
        _arr(x, ctypes.c_double, 3 * (b - a))[:] = self.x[a:b].ravel()
        return 0

    def tm_serve_destroy(self, h):
        return 0


class _Model:
    def __init__(self):
        self.ctx = _Ctx()
        self.lib = _FakeLib()
        self.h = None


def _req(n, kind="md", nsteps=3, x0=0.0):
    x = np.zeros((n, 3))
    x[:, 1] = np.arange(n) + 1000 * x0   # row identity
    return serve.Request(np.full(n, 1), x, kind=kind, nsteps=nsteps)


def test_rows_follow_their_requests_through_relayouts():
    m = _Model()
    srv = serve.Server(m, max_atoms=100, max_mols=4)
    reqs = [_req(10, "md", 4, 1), _req(20, "md", 2, 2), _req(5, "ef", 1, 3), _req(7, "md", 3, 4)]
    srv.submit(reqs[0])
    srv.step()
    srv.submit(reqs[1])
    srv.submit(reqs[2])
    srv.step()
    srv.submit(reqs[3])
    srv.drain()
    for r in reqs:
        assert r.done and r.steps_done == r.nsteps
        np.testing.assert_array_equal(r.x[:, 1], r.x0[:, 1])           # same rows
        expect = r.nsteps if r.kind == "md" else 0
        np.testing.assert_array_equal(r.x[:, 0], np.full(r.natoms, float(expect)))
        assert [e[0] for e in r.energies] == [r.natoms] * r.nsteps


def test_admission_is_fifo_within_capacity():
    m = _Model()
    srv = serve.Server(m, max_atoms=30, max_mols=2)
    a, b, c = _req(20, "md", 2), _req(15, "md", 2), _req(5, "md", 2)
    for r in (a, b, c):
        srv.submit(r)
    srv.step()
    # b (15) does not fit beside a (20); c must wait behind b (first come, first served)
    assert [r.rid for r in srv.active] == [a.rid]
    srv.drain()
    assert all(r.done for r in (a, b, c))
    assert max(srv.step_atoms) <= 30
    assert a.t_admit <= b.t_admit <= c.t_admit


def test_first_fit_admission_fills_the_batch_and_bounds_overtaking():
    m = _Model()
    srv = serve.Server(m, max_atoms=30, max_mols=4, admission="first_fit", max_overtakes=2)
    a, b, c = _req(20, "md", 2), _req(15, "md", 2), _req(5, "md", 2)
    for r in (a, b, c):
        srv.submit(r)
    srv.step()
    # b (15) does not fit beside a (20); c (5) does and goes ahead of it
    assert [r.rid for r in srv.active] == [a.rid, c.rid]
    assert b.overtaken == 1
    srv.drain()
    assert all(r.done for r in (a, b, c)) and max(srv.step_atoms) <= 30


def test_first_fit_stops_overtaking_a_request_that_waited_long_enough():
    m = _Model()
    srv = serve.Server(m, max_atoms=30, max_mols=8, admission="first_fit", max_overtakes=1)
    big = _req(20, "md", 50)
    srv.submit(big)
    srv.step()                                 # big runs for 50 steps
    head = _req(15, "md", 1)                   # cannot fit beside big
    srv.submit(head)
    small = [_req(6, "md", 1) for _ in range(3)]
    for r in small:
        srv.submit(r)
    srv.step()                                 # small[0] overtakes head
    assert head.overtaken == 1
    admitted = {r.rid for r in srv.active}
    assert small[0].rid in admitted and small[1].rid not in admitted
    srv.step()                                 # head may not be overtaken again
    admitted = {r.rid for r in srv.active}
    assert small[1].rid not in admitted and small[2].rid not in admitted
    srv.drain()
    assert head.t_admit <= small[1].t_admit and head.t_admit <= small[2].t_admit


def test_vectorised_gather_map_matches_the_rule():
    m = _Model()
    srv = serve.Server(m, max_atoms=200, max_mols=8)
    reqs = [_req(n, "md", s, k) for k, (n, s) in enumerate([(7, 1), (3, 5), (11, 2), (4, 4)])]
    for r in reqs[:3]:
        srv.submit(r)
    srv.step()
    srv.submit(reqs[3])
    srv.drain()
    for r in reqs:
        np.testing.assert_array_equal(r.x[:, 1], r.x0[:, 1])


def test_optimisation_requests_retire_on_convergence():
    m = _Model()
    srv = serve.Server(m, max_atoms=100, max_mols=4, admission="first_fit")
    a, b = _req(6, "opt", 200), _req(8, "md", 3)
    srv.submit(a)
    srv.submit(b)
    srv.drain()
    assert a.converged and a.steps_done == 1 and a.fmax_last == 0.0
    assert b.steps_done == 3
