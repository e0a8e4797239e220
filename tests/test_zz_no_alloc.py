"""The allocation-free entry point cytom_tile_batch_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory (applications that own the device
heap through their own pool, streams that must not see an allocation). Its output must
equal the allocating path's -- insert the batch into an empty store, compact, read the
tiles -- and the CPU oracle's compaction, bit for bit, on two calls in a row (the second
call reuses the shared static scratch array the first one left behind). Edge cases: an
unweighted call (w = NULL), an empty batch, a tile whose only edge is the local corner
edge (65535, 65535) at 65,536 vertices per tile, and an out-of-range id. Collected last
on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_tiles(cg, n, vpt, s, t, w):
    with cg.Engine(n, vpt, weight_type=cg.WEIGHT_U32) as eng:
        eng.insert_edges(s, t, w)
        eng.do_global_compaction()
        return eng.dump_tiles(weights=True)


def oracle_tiles(orc, n, vpt, s, t, w):
    st = orc.Store(n, vpt, w is not None)
    st.insert(s, t, w)
    st.compact()
    return st.dump()


def call_noalloc(cg, torch, n, vpt, s, t, w):
    """Returns (status, tile_ptr, edges, weights); weights is None for an unweighted call."""
    lib = cg.load()
    T = n // vpt
    m = len(s)
    ds = torch.from_numpy(s.view(np.int32)).cuda()
    dt = torch.from_numpy(t.view(np.int32)).cuda()
    dw = torch.from_numpy(w.view(np.int32)).cuda() if w is not None else None
    tp = torch.full((T * T + 1,), -1, dtype=torch.int64, device="cuda")
    ed = torch.full((max(m, 1),), -1, dtype=torch.int32, device="cuda")
    wt = torch.full((max(m, 1),), -1, dtype=torch.int32, device="cuda") if w is not None else None
    cnt = C.c_uint64(12345)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.cytom_tile_batch_noalloc(ds.data_ptr() if m else None, dt.data_ptr() if m else None,
                                      dw.data_ptr() if dw is not None else None, m, n, vpt, tp.data_ptr(),
                                      ed.data_ptr(), wt.data_ptr() if wt is not None else None, C.byref(cnt),
                                      stream)
    if rc != 0:
        return rc, None, None, None
    e = cnt.value
    return (0, tp.cpu().numpy().view(np.uint64), ed[:e].cpu().numpy().view(np.uint32),
            wt[:e].cpu().numpy().view(np.uint32) if wt is not None else None)


def noalloc_tiles(cg, torch, n, vpt, s, t, w):
    rc, tp, ed, wt = call_noalloc(cg, torch, n, vpt, s, t, w)
    assert rc == 0, rc
    return tp, ed, wt


def test_noalloc_matches_store_on_two_calls(cg, orc):
    torch = pytest.importorskip("torch")
    cases = [(1 << 16, 4096, 1 << 18, 3), (1 << 12, 256, 50000, 4)]  # second call smaller
    for n, vpt, m, seed in cases:
        scale = n.bit_length() - 1
        s, t = orc.rmat(scale, 0, m, seed)
        w = orc.edge_weights(s, t, seed)
        gtp, ged, gw = noalloc_tiles(cg, torch, n, vpt, s, t, w)
        rtp, red, rw, _ = reference_tiles(cg, n, vpt, s, t, w)
        assert np.array_equal(gtp, rtp)
        assert np.array_equal(ged, red)
        assert np.array_equal(gw, rw)
        otp, oed, ow, _ = oracle_tiles(orc, n, vpt, s, t, w)
        assert np.array_equal(gtp, otp) and np.array_equal(ged, oed) and np.array_equal(gw, ow)


def test_noalloc_unweighted_and_empty(cg, orc):
    torch = pytest.importorskip("torch")
    n, vpt = 1 << 14, 1024
    s, t = orc.rmat(14, 0, 40000, 9)
    for _ in range(2):  # twice in a row on the shared scratch
        gtp, ged, gw = noalloc_tiles(cg, torch, n, vpt, s, t, None)
        assert gw is None
        otp, oed, _, _ = oracle_tiles(orc, n, vpt, s, t, None)
        assert np.array_equal(gtp, otp) and np.array_equal(ged, oed)
    e = np.zeros(0, np.uint32)
    gtp, ged, _ = noalloc_tiles(cg, torch, n, vpt, e, e, None)
    assert len(ged) == 0 and not gtp.any() and len(gtp) == (n // vpt) ** 2 + 1


def test_noalloc_corner_edge_and_keep_min(cg, orc):
    torch = pytest.importorskip("torch")
    n, vpt = 1 << 17, 1 << 16
    # tile (0,1): only the local corner edge (65535, 65535) -> dropped, as the reference's
    # fillCSR filter drops it; tile (1,0): the corner edge next to another edge -> kept;
    # tile (0,0): (7,9) three times with different weights -> one copy, least weight
    s = np.array([65535, 65535, 65536 + 65535, 65536 + 5, 7, 7, 7], np.uint32)
    t = np.array([65536 + 65535, 65536 + 65535, 65535, 65535, 9, 9, 9], np.uint32)
    w = np.array([5, 5, 3, 4, 30, 10, 20], np.uint32)
    for _ in range(2):
        gtp, ged, gw = noalloc_tiles(cg, torch, n, vpt, s, t, w)
        otp, oed, ow, _ = oracle_tiles(orc, n, vpt, s, t, w)
        assert np.array_equal(gtp, otp) and np.array_equal(ged, oed) and np.array_equal(gw, ow)
        assert gtp[1] - gtp[0] == 1 and gw[0] == 10
        assert gtp[2] - gtp[1] == 0
        assert gtp[3] - gtp[2] == 2


def test_noalloc_rejects_out_of_range_id(cg, orc):
    torch = pytest.importorskip("torch")
    n, vpt = 1 << 12, 256
    s = np.array([1, 2, 4096], np.uint32)  # 4096 = the vertex count
    t = np.array([3, 4, 5], np.uint32)
    rc, _, _, _ = call_noalloc(cg, torch, n, vpt, s, t, None)
    assert rc == -3  # CYTOM_ERR_RANGE
    # the next call on the same scratch is unaffected
    s2, t2 = orc.rmat(12, 0, 20000, 5)
    gtp, ged, _ = noalloc_tiles(cg, torch, n, vpt, s2, t2, None)
    otp, oed, _, _ = oracle_tiles(orc, n, vpt, s2, t2, None)
    assert np.array_equal(gtp, otp) and np.array_equal(ged, oed)


def test_noalloc_rejects_oversized_batch(cg):
    lib = cg.load()
    cnt = C.c_uint64(0)
    limit = 1 << 18  # CYTOM_NOALLOC_MAX_EDGES
    rc = lib.cytom_tile_batch_noalloc(None, None, None, limit + 1, 1 << 16, 4096, None, None, None,
                                      C.byref(cnt), None)
    assert rc == -1  # CYTOM_ERR_INVAL, before any device work
