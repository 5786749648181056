"""LMA disparity (Correlation2d.corrLMA, the reference's default "POLY" disparity) on the GPU
against the FP64 oracle restatement (needs a GB300).

The oracle is fed the GPU's own correlation surfaces and CM disparity, so the check isolates the
LMA stage: group combination, convex-cell selection, samples and the Levenberg-Marquardt fit.
The device fit runs in FP32 and the oracle in FP64: success flags agree on >= 98% of the tiles and
disparity / strength agree to 0.005 px / 1e-3 relative on >= 98% of the tiles both fitted.
"""
import numpy as np
import pytest

from helpers import make_gpu
from tileproc import synth

pytestmark = pytest.mark.gpu

KINDS = [0, 0, 1, 1, 2, 3]  # the quad PAIRS[0..5]


def _compare(oracle, corr, disp, lma, min_frac=0.98):
    p = oracle.default_lma_params()
    n = agree = both = close = 0
    errs = []
    for t in range(disp.shape[0]):
        cm, st = disp[t, oracle.DISP_CM], disp[t, oracle.DISP_STRENGTH]
        if not np.isfinite(cm) or not st > p.min_poly_strength:
            assert np.all(np.isnan(lma[t])), "tile %d: LMA ran where the reference does not" % t
            continue
        ok, out, ns = oracle.corr_lma(corr[t].astype(np.float64), KINDS, -float(cm), p)
        n += 1
        gok = bool(np.isfinite(lma[t, 0]))
        agree += (gok == ok)
        if ok and gok:
            both += 1
            e = abs(lma[t, 0] - out[0])
            errs.append(e)
            close += (e <= 0.005) and abs(lma[t, 1] - out[1]) <= 1e-3 * abs(out[1]) + 1e-6
    assert n > 20
    assert agree >= min_frac * n, "success flags agree on %d of %d" % (agree, n)
    assert close >= min_frac * both, "disparity/strength agree on %d of %d (max err %.3g)" % (close, both, max(errs))
    return np.array(errs)


@pytest.mark.parametrize("kind,size", [("quad_mono", (128, 96)), ("quad_bayer", (128, 96))])
def test_lma_matches_oracle(oracle, kind, size):
    sc = synth.make_scene(kind, seed=41, width=size[0], height=size[1])
    T = (size[0] // 8) * (size[1] // 8)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        corr, disp = tp.getCorr(), tp.getDisparity()
        lma = tp.lmaRefine(mix_corr_poly=0, fo_correct=0)
        assert np.array_equal(tp.getDisparity(), disp, equal_nan=True), "mix_corr_poly=0 changed the record"
        errs = _compare(oracle, corr, disp, lma)
        print("%s: LMA |gpu - oracle| median %.2g max %.2g px over %d tiles" % (kind, np.median(errs), errs.max(),
                                                                              len(errs)))


def test_lma_mix_replaces_cm_and_needs_a_new_forward(oracle):
    from tileproc import _lib
    sc = synth.make_scene("quad_mono", seed=42, width=128, height=96)
    T = 16 * 12
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        d0 = tp.getDisparity()
        lma = tp.lmaRefine(fo_correct=0)
        d1 = tp.getDisparity()
        fit = np.isfinite(lma[:, 0])
        assert fit.sum() > 20
        assert np.array_equal(d1[fit, oracle.DISP_CM], lma[fit, 0])
        assert np.array_equal(d1[fit, oracle.DISP_STRENGTH], lma[fit, 1])
        assert np.array_equal(d1[~fit], d0[~fit], equal_nan=True)
        with pytest.raises(_lib.TpError, match="run tp_process"):
            tp.lmaRefine(fo_correct=0)
        tp.process()
        assert np.array_equal(tp.getDisparity(), d0, equal_nan=True)
        tp.lmaRefine()


@pytest.mark.parametrize("kind,size", [("quad_mono", (128, 96)), ("quad_bayer", (128, 96))])
def test_lma_record_update_matches_oracle(oracle, kind, size):
    """Default settings: the LMA mixed into CM / strength and the far/foreground correction
    (four orientation fits + foregroundCorrect) applied to CM, as ImageDtt.java:2254-2335 does.
    Oracle on the GPU's surfaces and record; CM within 0.005 px and strength within 1e-3 relative
    on >= 97% of the refined tiles (the correction's threshold tests may fall either side in FP32)."""
    sc = synth.make_scene(kind, seed=44, width=size[0], height=size[1])
    T = (size[0] // 8) * (size[1] // 8)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        corr, d0 = tp.getCorr(), tp.getDisparity()
        lma = tp.lmaRefine()
        d1 = tp.getDisparity()
    n = ok = moved = 0
    for t in range(T):
        ran, rec, lm = oracle.lma_tile(corr[t].astype(np.float64), KINDS, float(d0[t, oracle.DISP_CM]),
                                       float(d0[t, oracle.DISP_STRENGTH]))
        if not ran:
            continue
        n += 1
        moved += rec[0] != lm[0]
        ok += (abs(d1[t, oracle.DISP_CM] - rec[0]) <= 0.005 and
               abs(d1[t, oracle.DISP_STRENGTH] - rec[1]) <= 1e-3 * abs(rec[1]) + 1e-6)
    assert n > 20 and moved > 0
    assert ok >= 0.97 * n, "record agrees on %d of %d tiles (%d moved by the foreground correction)" % (ok, n, moved)
    print("%s: record agrees on %d of %d tiles, %d moved by the foreground correction" % (kind, ok, n, moved))


def test_lma_mismatch_matches_oracle(oracle):
    """Lazy-eye mismatch (ImageDtt.java:2340-2418, Correlation2d.mismatchPairsCM): per pair the peak's
    centre of mass around the LMA disparity, where the four orientation fits agree to 1 px; the
    record's CM keeps the LMA value (no foreground correction while measuring).  Oracle on the GPU's
    surfaces and record; {dx, dy, strength} within 1e-3 on >= 97% of the refined tiles."""
    sc = synth.make_scene("quad_mono", seed=45, width=128, height=96)
    T = 16 * 12
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        corr, d0 = tp.getCorr(), tp.getDisparity()
        tp.lmaRefine(mismatch=1)
        d1, mm = tp.getDisparity(), tp.getLmaMismatch()
    n = ok = measured = 0
    for t in range(T):
        ran, rec, lm, om = oracle.lma_tile_mismatch(corr[t].astype(np.float64), KINDS, float(d0[t, oracle.DISP_CM]),
                                                    float(d0[t, oracle.DISP_STRENGTH]))
        if not ran:
            assert np.all(np.isnan(mm[t, :, :2])) and np.all(mm[t, :, 2] == 0)
            continue
        n += 1
        measured += bool(np.isfinite(om[:, 0]).all())
        same = np.allclose(mm[t], om, atol=1e-3, equal_nan=True) and abs(d1[t, oracle.DISP_CM] - rec[0]) <= 0.005
        ok += same
    assert n > 20 and measured > 0.5 * n
    assert ok >= 0.97 * n, "mismatch agrees on %d of %d tiles" % (ok, n)
    print("mismatch: agrees on %d of %d tiles, measured on %d" % (ok, n, measured))


@pytest.mark.parametrize("backup", [True, False])
def test_lma_poly_mismatch_matches_oracle(oracle, backup):
    """The polynomial mismatch (ly_poly; ImageDtt.java:2349-2383, Correlation2d.mismatchPairs): each pair
    alone, the maximum of its weighted quadric; implausible pairs (offset > ly_crazy_poly) get zero
    strength and, with ly_poly_backup, send the tile to the centre of mass.  Oracle on the GPU's
    surfaces and record; {dx, dy, strength} within 1e-3 on >= 97% of the refined tiles, and the quadric
    (not the centre of mass) decides a share of them."""
    sc = synth.make_scene("quad_mono", seed=45, width=128, height=96)
    T = 16 * 12
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        corr, d0 = tp.getCorr(), tp.getDisparity()
        tp.lmaRefine(mismatch=1, ly_poly=1, ly_poly_backup=int(backup))
        mm = tp.getLmaMismatch()
    n = ok = by_poly = 0
    for t in range(T):
        args = (corr[t].astype(np.float64), KINDS, float(d0[t, oracle.DISP_CM]), float(d0[t, oracle.DISP_STRENGTH]))
        ran, _, _, om = oracle.lma_tile_mismatch(*args, ly_poly=True, ly_poly_backup=backup)
        if not ran:
            assert np.all(np.isnan(mm[t, :, :2])) and np.all(mm[t, :, 2] == 0)
            continue
        n += 1
        _, _, _, ocm = oracle.lma_tile_mismatch(*args)
        by_poly += not np.allclose(om, ocm, atol=1e-9, equal_nan=True)
        ok += np.allclose(mm[t], om, atol=1e-3, equal_nan=True)
    assert n > 20 and by_poly > 0.2 * n
    assert ok >= 0.97 * n, "poly mismatch agrees on %d of %d tiles" % (ok, n)
    print("poly mismatch (backup %s): agrees on %d of %d tiles, %d by the quadric" % (backup, ok, n, by_poly))


def test_lma_rejects_general_pairs(oracle):
    from tileproc import _lib
    sc = synth.make_scene("circle_lwir", seed=43, width=64, height=64)
    with make_gpu(sc) as tp:
        tp.setCorrelation(pairs=synth.circle_pairs(sc["geometry"]))
        tp.setFullFrameImages(np.full(64, 2.0, np.float32))
        tp.process()
        with pytest.raises(_lib.TpError, match="quad kinds"):
            tp.lmaRefine()
