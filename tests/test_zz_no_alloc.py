"""p2m_map_sums_noalloc -- map sums from a statically sized device scratch, no allocation --
against the context path's map sums (p2m_get_stats, whose scratch the context allocates),
through the C ABI.  Kept in its own file, collected after the other GPU tests."""
import ctypes
import warnings

import numpy as np
import pytest

import catalogs
import matt_young_mapmaking_gb300 as p2m

pytestmark = pytest.mark.gpu

SUM_REL = 1e-12  # same per-thread partial sums; only the FP64 atomic order differs


def sums_noalloc(lib, ptrs, npix, stream=0):
    arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
    out = np.full(len(ptrs), np.nan, dtype=np.float64)
    st = lib.p2m_map_sums_noalloc(arr, len(ptrs), npix, out.ctypes.data, ctypes.c_void_p(stream))
    return st, out


def painted_maps(nside):
    import torch
    rec = catalogs.shell(31, 40_000, r=(100.0, 8000.0), m=(1e12, 3e15))
    tab = catalogs.table(nu=0.0)
    npix = 12 * nside * nside
    outs = [torch.empty(npix, dtype=torch.float32, device="cuda") for _ in range(2)]
    with p2m.Painter(nside=nside, precision="mixed", maps=((0, 1), (0, 2)), zmax=6.0,
                     max_records=len(rec)) as pt:
        pt.load_table(0, tab)
        for m in range(2):
            pt.bind_healpix_device(m, outs[m].data_ptr())
        pt.paint_records(rec)
        for m in range(2):
            pt.healpix_device(m, outs[m].data_ptr())
        pt.synchronize()
        ref = pt.stats()["hp_sum"]
    torch.cuda.synchronize()
    return outs, ref, npix


def test_noalloc_sums_match_context_sums_twice():
    import torch
    lib = p2m.load_library()
    outs, ref, npix = painted_maps(512)
    assert abs(ref[0]) > 0 and abs(ref[1]) > 0
    ptrs = [o.data_ptr() for o in outs]
    free_before = None
    for call in range(3):  # each call clears the shared scratch itself
        st, sums = sums_noalloc(lib, ptrs, npix)
        assert st == 0, "call %d: status %d" % (call, st)
        for m in range(2):
            assert abs(sums[m] - ref[m]) <= SUM_REL * abs(ref[m]), (call, m, sums[m], ref[m])
        # the first call may load the module (code and the static scratch); after it,
        # a call takes no device memory: the device's free bytes and the torch caching
        # allocator's reserved bytes stay the same from call to call
        free_now = (torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved())
        if free_before is not None:
            assert free_now == free_before, "call %d: (free, reserved) %s -> %s" % (
                call, free_before, free_now)
        free_before = free_now
    host = [o.cpu().numpy().astype(np.float64) for o in outs]
    for m in range(2):
        assert abs(sums[m] - host[m].sum()) <= 1e-9 * np.abs(host[m]).sum()
    # one map alone gives the same total as in the pair
    st, one = sums_noalloc(lib, ptrs[1:], npix)
    assert st == 0 and abs(one[0] - ref[1]) <= SUM_REL * abs(ref[1])


def test_noalloc_rejects_bad_sizes():
    import torch
    lib = p2m.load_library()
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    too_many = [buf.data_ptr()] * (p2m.capi.NOALLOC_MAXMAPS + 1)
    st, _ = sums_noalloc(lib, too_many, 1024)
    assert st == p2m.capi.P2M_ERR_CAPACITY
    st, _ = sums_noalloc(lib, [], 1024)
    assert st == p2m.capi.P2M_ERR_BADARG
    st, empty = sums_noalloc(lib, [buf.data_ptr()], 0)
    assert st == 0 and empty[0] == 0.0


def test_noalloc_refuses_a_capturing_stream():
    """The call ends in a copy to host memory and a stream synchronisation, neither of
    which a stream under capture allows: it returns P2M_ERR_STATE and queues nothing, so
    the capture ends cleanly (an empty graph)."""
    import torch
    lib = p2m.load_library()
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    st, _ = sums_noalloc(lib, [buf.data_ptr()], 1024)  # the one-time set-up, uncaptured
    assert st == 0
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    results = []
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)  # torch notes that the graph is empty
        with torch.cuda.graph(graph, stream=side):
            results.append(sums_noalloc(lib, [buf.data_ptr()], 1024,
                                        stream=side.cuda_stream)[0])
    assert results == [p2m.capi.P2M_ERR_STATE]
    st, out = sums_noalloc(lib, [buf.data_ptr()], 1024)  # usable after the capture
    assert st == 0 and out[0] == 0.0
