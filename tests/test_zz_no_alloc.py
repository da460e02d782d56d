"""The allocation-free neighbour-list entry point (tm_nlist_build_static).

Some callers of this library cannot let it allocate device memory: an MD
engine or plugin that owns a fixed device arena, or a server that budgets
memory up front. For them tm_nlist_build_static builds the radial and angular
lists of one open-boundary molecule into buffers the caller owns, with its own
scratch in a fixed-size device array compiled into the library. This test
calls it through the C ABI twice in a row (two different molecules, the larger
first so stale scratch would show) and checks each result against the regular
entry point (tm_system_build_nlist + tm_system_export_nlist): the neighbour
sets must be identical, which is the bar for integer list work.
"""
import ctypes

import numpy as np
import pytest

from tensormol_gb300 import systems
from tensormol_gb300.params import PARAMS, descriptor_width

pytestmark = pytest.mark.gpu


def _regular_pairs(model, sysm):
    s = model.system(sysm.x, sysm.Z, sysm.offsets)
    s.build_nlist()
    radp, angt, _, _ = s.export_nlist()
    s.close()
    # molecule-local (i, j) of the radial list; angular neighbours from triples
    return radp[:, 1:3]


def _static_lists(lib, x, elem, KR=64, KA=48, expect=0):
    import torch
    n = x.shape[0]
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    ed = torch.tensor(elem, dtype=torch.int32, device="cuda")
    cr = torch.zeros(n, dtype=torch.int32, device="cuda")
    ca = torch.zeros(n, dtype=torch.int32, device="cuda")
    nr = torch.zeros(n * KR, dtype=torch.int32, device="cuda")
    na = torch.zeros(n * KA, dtype=torch.int32, device="cuda")
    need = (ctypes.c_int32 * 2)()
    torch.cuda.synchronize()
    rc = lib.tm_nlist_build_static(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(ed.data_ptr()), n,
                                   PARAMS["AN1_r_Rc"], PARAMS["AN1_a_Rc"],
                                   ctypes.c_void_p(cr.data_ptr()), ctypes.c_void_p(nr.data_ptr()), KR,
                                   ctypes.c_void_p(ca.data_ptr()), ctypes.c_void_p(na.data_ptr()), KA,
                                   need, None)
    assert rc == expect, rc
    if rc:
        return None, None, (need[0], need[1])
    cr, ca = cr.cpu().numpy(), ca.cpu().numpy()
    mask = (1 << 27) - 1                       # low 27 bits: neighbour index
    nr = nr.cpu().numpy().reshape(n, KR) & mask
    na = na.cpu().numpy().reshape(n, KA) & mask
    pairs = np.concatenate([np.stack([np.full(c, i), nr[i, :c]], 1) for i, c in enumerate(cr)])
    ang = np.concatenate([np.stack([np.full(c, i), na[i, :c]], 1) for i, c in enumerate(ca)])
    return pairs.astype(np.int64), ang.astype(np.int64), (need[0], need[1])


def test_static_nlist_matches_regular_twice_in_a_row():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import reference as orc
    from tensormol_gb300.model import BPEEModel
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    model = BPEEModel(eles, W, precision="fp32")
    big = systems.water(1000, seed=11)          # 3,000 atoms
    small = systems.water_cluster_60(seed=0)    # 60 atoms
    lib = model.lib
    for sysm in (big, small):
        elem = (sysm.Z == 8).astype(np.int32)   # element index in sorted [H, O]
        pairs, ang, need = _static_lists(lib, sysm.x, elem)
        ref_pairs = _regular_pairs(model, sysm)
        # the regular export is (element, index)-sorted per centre, like the rows
        assert np.array_equal(pairs, ref_pairs)
        tc, tn = orc.nlist_entries(sysm.x, PARAMS["AN1_a_Rc"])
        key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
        assert np.array_equal(key(ang), key(np.stack([tc, tn], 1)))
        assert need == (0, 0)
    # rows too short: a clean TM_E_CAPACITY with the counts the rows needed
    elem = (big.Z == 8).astype(np.int32)
    _, _, need = _static_lists(lib, big.x, elem, KR=16, KA=8, expect=3)
    ref = _regular_pairs(model, big)
    tc, _ = orc.nlist_entries(big.x, PARAMS["AN1_a_Rc"])
    assert need == (np.bincount(ref[:, 0]).max(), np.bincount(tc).max())
    model.close()


def test_static_nlist_refuses_a_capturing_stream():
    """The entry point copies counts to the host and synchronises its stream,
    which a stream capture forbids: on a capturing stream it returns TM_E_ARG
    before it enqueues anything, and the capture stays valid."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import _lib
    from tensormol_gb300.model import BPEEModel
    eles = [1, 8]
    W = systems.random_weights(eles, descriptor_width(2), seed=7)
    model = BPEEModel(eles, W, precision="fp32")
    small = systems.water_cluster_60(seed=0)
    elem = (small.Z == 8).astype(np.int32)
    _static_lists(model.lib, small.x, elem)     # first call outside any capture
    n, KR, KA = small.x.shape[0], 64, 48
    xd = torch.tensor(small.x, dtype=torch.float64, device="cuda")
    ed = torch.tensor(elem, dtype=torch.int32, device="cuda")
    out = [torch.zeros(k, dtype=torch.int32, device="cuda") for k in (n, n * KR, n, n * KA)]
    y = torch.zeros(4, device="cuda")
    need = (ctypes.c_int32 * 2)()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rc = model.lib.tm_nlist_build_static(
            ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(ed.data_ptr()), n, PARAMS["AN1_r_Rc"],
            PARAMS["AN1_a_Rc"], ctypes.c_void_p(out[0].data_ptr()), ctypes.c_void_p(out[1].data_ptr()),
            KR, ctypes.c_void_p(out[2].data_ptr()), ctypes.c_void_p(out[3].data_ptr()), KA, need,
            ctypes.c_void_p(s.cuda_stream))
        y += 1.0
    assert rc == _lib.ERROR_CODES["TM_E_ARG"], rc
    g.replay()
    torch.cuda.synchronize()
    assert float(y.sum()) == 4.0
    model.close()
