"""The no-allocation task compaction (tp_compact_tile_ops_noalloc) against the
handle path (tp_set_tile_ops + tp_get_task_tiles / tp_get_num_tasks) on the
GPU: two calls in a row with different tile-op patterns, bit-exact task lists.
The test allocates its own device buffers (torch); the entry point allocates
nothing and keeps its per-block counts in a fixed device array."""
import ctypes as C

import numpy as np
import pytest

from tileproc import GPUTileProcessor, synth
from tileproc import _lib as L

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, ops, disp, tiles_x, stream):
    n = ops.numel()
    txy = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    top = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    tdisp = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
    num = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    st = lib.tp_compact_tile_ops_noalloc(C.c_void_p(ops.data_ptr()), C.c_void_p(disp.data_ptr()), tiles_x, n,
                                         C.c_void_p(txy.data_ptr()), C.c_void_p(top.data_ptr()),
                                         C.c_void_p(tdisp.data_ptr()), C.c_void_p(num.data_ptr()),
                                         C.c_void_p(stream.cuda_stream))
    assert st == L.TP_OK
    stream.synchronize()
    k = int(num.item())
    return k, txy[:k].cpu().numpy(), top[:k].cpu().numpy(), tdisp[:k].cpu().numpy()


@pytest.mark.parametrize("size", [(512, 384), (2592, 1936)])
def test_noalloc_compaction_matches_handle_path(size):
    torch = pytest.importorskip("torch")
    W, H = size
    tx, ty = W // 8, H // 8
    T = tx * ty
    lib = L.load()
    stream = torch.cuda.Stream()
    tp = GPUTileProcessor(4, W, H)
    try:
        tp.setGeometry(synth.quad_geometry(W, H))
        rng = np.random.default_rng(T)
        for call in range(2):  # two calls in a row, different patterns, same scratch array
            ops = np.where(rng.random(T) < (0.5 if call == 0 else 0.9), rng.integers(1, 0x200, T), 0)
            ops = ops.astype(np.int32)
            disp = rng.uniform(0, 8, T).astype(np.float32)
            tp.setFullFrameImages(disp, tile_op=ops)
            want_txy = tp.getTaskTiles()
            want_n = tp.numTasks()
            k, txy, top, tdisp = _noalloc(lib, torch, torch.from_numpy(ops).cuda(), torch.from_numpy(disp).cuda(),
                                          tx, stream)
            assert k == want_n
            assert np.array_equal(txy, want_txy)
            idx = np.nonzero(ops)[0]
            assert np.array_equal(top, ops[idx])
            assert np.array_equal(tdisp, disp[idx])
    finally:
        tp.close()


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    lib = L.load()
    one = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = C.c_void_p(one.data_ptr())
    st = lib.tp_compact_tile_ops_noalloc(p, None, 1024, L.TP_COMPACT_MAX_TILES + 1024, p, p, p, p, None)
    assert st == L.TP_ERR_SCRATCH_LIMIT
