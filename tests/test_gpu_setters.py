"""Setters that overwrite device buffers while the handle's work is still in flight on another
stream (needs a GB300): tp_process is enqueued on a caller's stream and returns at once, then
tp_set_kernels / tp_set_geometry / tp_set_corr replace what that forward reads.  Each setter waits
for the work already enqueued, so the forward in flight sees the old inputs: its CLT, correlation
surfaces and disparities equal those of the same forward run alone, bit for bit.  The scene is
large enough (19,602 tiles, a forward of about 0.3 ms) that the setter's call lands while the
forward runs."""
import copy
import ctypes as C

import numpy as np
import pytest

from helpers import make_gpu
from tileproc import synth

pytestmark = pytest.mark.gpu

W, H = 1296, 968
T = (W // 8) * (H // 8)


def _scene():
    sc = synth.make_scene("quad_bayer", seed=17, width=W, height=H)
    rng = np.random.default_rng(18)
    k1, e1 = synth.random_clt_kernels(rng, 4, H // 16 + 2, W // 16 + 2, 3)
    k2, e2 = synth.random_clt_kernels(rng, 4, H // 16 + 2, W // 16 + 2, 3)
    return sc, (k1, e1), (k2, e2)


def _outputs(tp):
    return tp.getClt(), tp.getCorr(), tp.getDisparity()


@pytest.mark.parametrize("what", ["kernels", "geometry", "corr"])
def test_setter_waits_for_the_forward_in_flight(what):
    import torch
    from tileproc import _lib
    sc, (k1, e1), (k2, e2) = _scene()
    g2 = copy.deepcopy(sc["geometry"])
    g2["azimuth"] = (np.asarray(g2["azimuth"]) + 2e-3).tolist()
    with make_gpu(sc, k1, e1) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32), tile_op=np.full(T, 0xF, np.int32))
        tp.process()
        ref = _outputs(tp)
        stream = torch.cuda.Stream()
        sp = C.c_void_p(stream.cuda_stream)
        for _ in range(3):
            tp._ck(tp._lib.tp_process(tp.h, sp), "tp_process")  # enqueued; returns at once
            if what == "kernels":
                tp.setConvolutionKernels(k2, e2, layout=_lib.TP_KERNELS_CPU)
            elif what == "geometry":
                tp.setGeometry(g2)
            else:
                tp.setCorrelation(fat_zero=0.3)
            got = _outputs(tp)
            for a, b in zip(ref, got):
                assert np.array_equal(a, b, equal_nan=True)
            # back to the first inputs for the next round
            tp.setConvolutionKernels(k1, e1, layout=_lib.TP_KERNELS_CPU)
            tp.setGeometry(sc["geometry"])
            tp.setCorrelation()
            tp.setFullFrameImages(np.full(T, 4.0, np.float32), tile_op=np.full(T, 0xF, np.int32))
        torch.cuda.synchronize()
