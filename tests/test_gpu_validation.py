"""Task-input validation and device-memory limits of the C ABI (tp_create needs a device).

Bad ports (tp_set_tasks) and bad target disparities (tp_set_tile_ops) are rejected
on the host with TP_ERR_ARG before anything is uploaded or launched, and leave
the handle as it was: no kernel ever runs on them.  Ports that the device
computes from the geometry far outside the image are accepted; their window
corners are moved to the margin with their parity kept, which leaves the
edge-mirrored window content unchanged, so CLT and correlation still match the
oracle, which keeps the unmoved corners.  The allocation cap turns device
allocations into TP_ERR_NOMEM without exhausting the GPU."""
import ctypes as C

import numpy as np
import pytest

from helpers import make_gpu, rel_l2, run_oracle
from tileproc import _lib as L
from tileproc import GPUTileProcessor, synth

pytestmark = pytest.mark.gpu

M = 1024            # TP_PORT_MARGIN
MAX_DISP = 4096.0   # TP_MAX_DISPARITY


def _scene():
    return synth.make_scene("quad_mono", seed=7, width=128, height=96)


def _status(fn, *a):
    with pytest.raises(L.TpError) as ei:
        fn(*a)
    return ei.value.status


def test_set_tasks_rejects_bad_ports(oracle):
    sc = _scene()
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 2.0, np.float32))
        tp.process()
        ports = tp.getPorts().astype(np.float32)
        txy = tp.getTaskTiles()
        packed = GPUTileProcessor.packTasks(np.full(T, 0xF), txy & 0xffff, txy >> 16, ports)
        tp.setTasks(packed)
        tp.process()
        d0 = tp.getDisparity()
        bad = [(5, 0, 0, np.nan), (5, 1, 1, np.inf), (6, 2, 0, -np.inf), (7, 3, 0, 1e30), (8, 0, 1, -1e30),
               (9, 1, 0, W + M + 1.0), (10, 2, 0, -M - 1.0), (11, 3, 1, H + M + 1.0), (12, 0, 1, -M - 0.5)]
        for task, s, k, v in bad:
            p = packed.copy()
            p[task, 2 + 2 * s + k] = v
            assert _status(tp.setTasks, p) == L.TP_ERR_ARG, (task, s, k, v)
            assert tp.numTasks() == T
        # the handle still holds the good task list: the same forward as before
        tp.process()
        assert np.array_equal(tp.getDisparity(), d0, equal_nan=True)
        # ports exactly at the margin are accepted; their windows read mirrored edge pixels as in the oracle
        edge = packed.copy()
        edge[3, 2:4] = (-M, -M)
        edge[4, 4:6] = (W + M, H + M)
        edge[20, 6:8] = (W + 3.25, -2.75)
        tp.setTasks(edge)
        tp.process()
        xy = edge[:, 2:].reshape(T, 4, 2).astype(np.float64)
        ref = run_oracle(oracle, sc, 2.0, ports_in=xy)
        e = rel_l2(tp.getClt().astype(np.float64), ref["clt"], axis=(-2, -1))
        assert e.max() <= 2e-6, e.max()
        # tasks 3 and 4 have windows entirely outside the image: a repeated 2x2 edge pattern whose
        # fat-zero normalised correlation is ill-conditioned (FP32 vs FP64 ~1e-3); their CLT is checked above
        real = np.ones(T, bool)
        real[[3, 4]] = False
        e = rel_l2(tp.getCorr().astype(np.float64), ref["corr"], axis=-1)[real]
        assert e.max() <= 1e-5, e.max()


def test_set_tile_ops_rejects_bad_disparity():
    sc = _scene()
    T = (sc["width"] // 8) * (sc["height"] // 8)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        op = np.ones(T, np.int32)
        disp = np.full(T, 3.0, np.float32)
        tp.setFullFrameImages(disp, tile_op=op)
        tp.process()
        d0 = tp.getDisparity()
        for v in (np.nan, np.inf, -np.inf, MAX_DISP * 1.001, -1e30):
            dd = disp.copy()
            dd[17] = v
            assert _status(tp.setFullFrameImages, dd, op) == L.TP_ERR_ARG, v
        tp.process()
        assert np.array_equal(tp.getDisparity(), d0, equal_nan=True)
        # a NaN on a tile that is not processed is allowed; +-TP_MAX_DISPARITY is allowed
        dd = disp.copy()
        dd[17] = np.nan
        dd[18] = MAX_DISP
        dd[19] = -MAX_DISP
        op2 = op.copy()
        op2[17] = 0
        tp.setFullFrameImages(dd, tile_op=op2)
        assert tp.numTasks() == T - 1


def test_far_geometry_ports_keep_window_content(oracle):
    """Disparities of +-4000 px move these ports ~2000 px outside a 128x96 image: beyond the
    margin, so the plan moves their corners; CLT and correlation still equal the oracle's."""
    sc = _scene()
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    disp = np.full(T, 2.0)
    disp[:12] = 4000.0
    disp[40:52] = -4000.0
    disp[60] = 1500.0
    ref = run_oracle(oracle, sc, disp)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp.astype(np.float32))
        tp.process()
        ports = tp.getPorts()
        assert np.array_equal(ports, ref["ports"])
        far = (np.abs(ports[..., 0] - W / 2) > W / 2 + M) | (np.abs(ports[..., 1] - H / 2) > H / 2 + M)
        assert far.sum() >= 40
        tl, res = tp.getSubtiles()
        rtl = ref["int_tl"]
        lim = np.array([W, H])
        inside = (rtl >= -(M + 16)) & (rtl <= lim + M)
        assert np.array_equal(tl[inside], rtl[inside])
        assert np.array_equal(tl[~inside] & 1, rtl[~inside] & 1)
        assert (~inside).sum() > 0
        assert np.array_equal(res, ref["residual"].astype(np.float32))
        e = rel_l2(tp.getClt().astype(np.float64), ref["clt"], axis=(-2, -1))
        assert e.max() <= 2e-6, e.max()
        # correlation where every window has image content (an all-outside window is a repeated 2x2 edge
        # pattern whose normalised correlation is ill-conditioned in FP32)
        off = (ports[..., 0] < -16) | (ports[..., 0] > W + 16) | (ports[..., 1] < -16) | (ports[..., 1] > H + 16)
        real = ~off.any(axis=1)
        assert real.sum() >= T - 30
        e = rel_l2(tp.getCorr().astype(np.float64), ref["corr"], axis=-1)[real]
        assert e.max() <= 1e-5, e.max()


def test_memory_limit_gives_nomem():
    lib = L.load()
    sc = _scene()
    T = (sc["width"] // 8) * (sc["height"] // 8)
    try:
        lib.tp_set_memory_limit(1 << 20)  # below what a 4-sensor 128x96 handle needs
        with pytest.raises(L.TpError) as ei:
            GPUTileProcessor(4, sc["width"], sc["height"])
        assert ei.value.status == L.TP_ERR_NOMEM
        lib.tp_set_memory_limit(0)
        with make_gpu(sc) as tp:
            tp.setCorrelation()
            tp.setFullFrameImages(np.full(T, 2.0, np.float32))
            tp.process()
            used = C.c_size_t()
            assert lib.tp_get_memory_usage(tp.h, C.byref(used)) == L.TP_OK
            # the frame buffer of tp_imclt is allocated on first use: refused under a cap at the current use
            lib.tp_set_memory_limit(used.value)
            assert _status(tp.execImcltRbg) == L.TP_ERR_NOMEM
            lib.tp_set_memory_limit(0)
            tp.execImcltRbg()
            rbg = tp.getRBG(0)
            assert np.isfinite(rbg).all() and np.abs(rbg).max() > 0
            used2 = C.c_size_t()
            lib.tp_get_memory_usage(tp.h, C.byref(used2))
            assert used2.value == used.value + 4 * 4 * (sc["width"] + 8) * (sc["height"] + 8)  # 4 sensors, f32
    finally:
        lib.tp_set_memory_limit(0)
