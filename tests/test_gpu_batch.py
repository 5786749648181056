"""Batched persistent forward (tp_batch_*) vs the per-scene forward on the GPU:
four scenes of different kinds (4 Bayer sensors with kernel tables, 4 mono
sensors, 16 mono sensors with 120 pairs, and a large 4-sensor Bayer scene that
keeps its own launch) in one batch step and through a captured CUDA graph.  The batch runs the same per-tile code as the per-scene kernels,
so CLT, correlation surfaces and disparities agree to FP32 rounding."""
import numpy as np
import pytest

from helpers import make_gpu, rel_l2
from tileproc import synth
from tileproc.batch import Batch

pytestmark = pytest.mark.gpu


def _scenes():
    rng = np.random.default_rng(11)
    out = []
    sc = synth.make_scene("quad_bayer", seed=51, width=192, height=128)
    k, e = synth.random_clt_kernels(rng, 4, 128 // 16 + 2, 192 // 16 + 2, 3)
    out.append((sc, k, e, None, 4.0))
    out.append((synth.make_scene("quad_mono", seed=52, width=128, height=96), None, None, None, 3.0))
    sc = synth.make_scene("circle_lwir", seed=53, width=160, height=128)
    out.append((sc, None, None, synth.circle_pairs(sc["geometry"]), 2.0))
    # 162 x 121 = 19602 tiles: enough waves to keep its own launch inside the batch
    out.append((synth.make_scene("quad_bayer", seed=54, width=1296, height=968), None, None, None, 3.0))
    return out


def _twelve_pairs():
    """The quad pairs and the same six the other way round (general kind, reversed strip axis)."""
    quad = [(0, 1, 0, 1, 1.0, 0.0), (2, 3, 0, 1, 1.0, 0.0), (0, 2, 1, 1, 0.0, 1.0), (1, 3, 1, 1, 0.0, 1.0),
            (0, 3, 2, 1, 1.0, 1.0), (2, 1, 3, 1, 1.0, -1.0)]
    return quad + [(b, a, 4, 1, -bx, -by) for a, b, _, _, bx, by in quad]


def _make(sc, k, e, pairs, disp):
    tp = make_gpu(sc, k, e)
    tp.setCorrelation(pairs=pairs)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    tp.setFullFrameImages(np.full(T, disp, np.float32))
    return tp


def _results(tp):
    return tp.getClt().astype(np.float64), tp.getCorr().astype(np.float64), tp.getDisparity().astype(np.float64)


def _same(a, b):
    clt_a, corr_a, d_a = a
    clt_b, corr_b, d_b = b
    assert rel_l2(clt_a, clt_b, axis=(-2, -1)).max() <= 1e-6
    assert rel_l2(corr_a, corr_b, axis=-1).max() <= 1e-5
    ok = np.isfinite(d_b[:, 1]) & (d_a[:, 8] == d_b[:, 8])
    assert ok.mean() > 0.99
    assert np.abs(d_a[ok, 1] - d_b[ok, 1]).max() <= 1e-4


def test_batch_matches_per_scene():
    tps = [_make(*s) for s in _scenes()]
    try:
        ref = []
        for tp in tps:
            tp.process()
            ref.append(_results(tp))
        with Batch(tps) as b:
            b.process(replan=True)
            b.synchronize()
            for tp, r in zip(tps, ref):
                _same(_results(tp), r)
            b.run_graph()
            b.synchronize()
            b.run_graph()
            b.synchronize()
            for tp, r in zip(tps, ref):
                _same(_results(tp), r)
            # new images, same tasks: the graph replay picks them up
            sc = _scenes()[1][0]
            imgs = np.roll(sc["images"], 3, axis=2)
            tps[1].setBayerImages(imgs)
            tps[1].process()
            want = _results(tps[1])
            b.run_graph()
            b.synchronize()
            _same(_results(tps[1]), want)
            # more pairs: the correlation buffer is reallocated and the scene changes schedule class;
            # the next replay must not reuse the captured step
            tps[1].setCorrelation(pairs=_twelve_pairs())
            tps[1].process()
            want = _results(tps[1])
            assert want[1].shape[1] == 12
            b.run_graph()
            b.synchronize()
            _same(_results(tps[1]), want)
            # a correlation parameter of the scene with its own launch (captured by value)
            tps[3].setCorrelation(fat_zero=0.1)
            tps[3].process()
            want = _results(tps[3])
            b.run_graph()
            b.synchronize()
            _same(_results(tps[3]), want)
            b.process(replan=False)
            b.synchronize()
            _same(_results(tps[3]), want)
    finally:
        for tp in tps:
            tp.close()
