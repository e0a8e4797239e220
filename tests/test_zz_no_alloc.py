"""The allocation-free entry point cytom_tile_batch_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory (applications that own the device
heap through their own pool, streams that must not see an allocation). Its output must
equal the allocating path's -- insert the batch into an empty store, compact, read the
tiles -- bit for bit, on two calls in a row (the second call reuses the shared static
scratch array the first one left behind). Collected last on purpose.
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


def noalloc_tiles(cg, torch, n, vpt, s, t, w):
    lib = cg.load()
    T = n // vpt
    ds = torch.from_numpy(s.view(np.int32)).cuda()
    dt = torch.from_numpy(t.view(np.int32)).cuda()
    dw = torch.from_numpy(w.view(np.int32)).cuda()
    tp = torch.full((T * T + 1,), -1, dtype=torch.int64, device="cuda")
    ed = torch.full((len(s),), -1, dtype=torch.int32, device="cuda")
    wt = torch.full((len(s),), -1, dtype=torch.int32, device="cuda")
    cnt = C.c_uint64(0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.cytom_tile_batch_noalloc(ds.data_ptr(), dt.data_ptr(), dw.data_ptr(), len(s), n, vpt,
                                      tp.data_ptr(), ed.data_ptr(), wt.data_ptr(), C.byref(cnt), stream)
    assert rc == 0, rc
    e = cnt.value
    return (tp.cpu().numpy().view(np.uint64), ed[:e].cpu().numpy().view(np.uint32),
            wt[:e].cpu().numpy().view(np.uint32))


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


def test_noalloc_rejects_oversized_batch(cg):
    lib = cg.load()
    cnt = C.c_uint64(0)
    limit = 1 << 18  # CYTOM_NOALLOC_MAX_EDGES
    rc = lib.cytom_tile_batch_noalloc(None, None, None, limit + 1, 1 << 16, 4096, None, None, None,
                                      C.byref(cnt), None)
    assert rc == -1  # CYTOM_ERR_INVAL, before any device work
