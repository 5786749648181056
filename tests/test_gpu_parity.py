"""GPU path vs the FP64 oracle on seeded synthetic scenes (needs a GB300).

Tolerances (stated by the port specification):
  * tile list, task order, integer window corners, kernel tiles: bit-exact;
  * ports (FP64 on the device): bit-exact;
  * CLT coefficients: relative L2 per (tile, sensor, colour) <= 2e-6;
  * correlation surfaces: relative L2 per (tile, pair) <= 1e-5;
  * disparity (centroid and ortho): |gpu - oracle| <= 0.005 px on every tile the
    oracle processed, no quantile.  Where the GPU's integer maximum differs from
    the oracle's, the oracle's own values at the two maxima must be a near tie
    (relative gap <= 1e-4, helpers.NEAR_TIE) and the GPU's disparity must equal
    the oracle's evaluated at the GPU's maximum (helpers.check_disparity_strict).
"""
import numpy as np
import pytest

from helpers import check_disparity_strict, make_gpu, rel_l2, run_oracle
from tileproc import synth

pytestmark = pytest.mark.gpu

CLT_TOL = 2e-6
CORR_TOL = 1e-5
DISP_TOL = 0.005


def _check_tiles(O, tp, ref, num_colors):
    ports = tp.getPorts()
    assert np.array_equal(ports, ref["ports"]), "ports differ: max %g" % np.abs(ports - ref["ports"]).max()
    tl, res = tp.getSubtiles()
    assert np.array_equal(tl, ref["int_tl"]), "integer window corners differ at %d sub-tiles" % (tl != ref["int_tl"]).sum()
    assert np.array_equal(res, ref["residual"].astype(np.float32)), "residual shifts differ"


def _check_clt(tp, ref, tile_mask=None):
    clt = tp.getClt().astype(np.float64)
    e = rel_l2(clt, ref["clt"], axis=(-2, -1))
    if tile_mask is not None:
        e = e[tile_mask]
    assert e.max() <= CLT_TOL, "CLT rel L2 max %.3g (median %.3g)" % (e.max(), np.median(e))
    return e


def _check_corr(tp, ref, tile_mask=None):
    corr = tp.getCorr().astype(np.float64)
    e = rel_l2(corr, ref["corr"], axis=-1)
    if tile_mask is not None:
        e = e[tile_mask]
    assert e.max() <= CORR_TOL, "corr rel L2 max %.3g (median %.3g)" % (e.max(), np.median(e))
    return e


def _check_disp(O, tp, ref, check_ortho=True):
    return check_disparity_strict(O, tp.getDisparity().astype(np.float64), ref, check_ortho=check_ortho)


def test_quad_mono_identity(oracle):
    """4 mono sensors 512x384, identity kernels, 6 pairs, fat zero 0.05 (the CPU-runnable config)."""
    sc = synth.make_scene("quad_mono", seed=1)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    ref = run_oracle(oracle, sc, 4.0)
    with make_gpu(sc) as tp:
        tp.setCorrelation(fat_zero=0.05)
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        assert tp.numTasks() == T
        txy = tp.getTaskTiles()
        assert np.array_equal(txy, (np.arange(T) % (sc["width"] // 8)) | ((np.arange(T) // (sc["width"] // 8)) << 16))
        _check_tiles(oracle, tp, ref, 1)
        _check_clt(tp, ref)
        _check_corr(tp, ref)
        _check_disp(oracle, tp, ref)


def test_quad_bayer_kernels(oracle):
    """4 Bayer sensors (uint16, GR/BG), per-sensor/colour CLT kernels on a 16-px grid with margins."""
    sc = synth.make_scene("quad_bayer", seed=3, width=256, height=192)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    rng = np.random.default_rng(7)
    kv, kh = H // 16 + 2, W // 16 + 2
    k, e = synth.random_clt_kernels(rng, 4, kv, kh, 3)
    disp = rng.uniform(2.0, 6.0, T).astype(np.float32)
    ref = run_oracle(oracle, sc, disp.astype(np.float64), kernels=k, kext=e)
    with make_gpu(sc, k, e) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp)
        tp.process()
        _check_tiles(oracle, tp, ref, 3)
        _check_clt(tp, ref)
        _check_corr(tp, ref)
        _check_disp(oracle, tp, ref)


def test_quad_bayer_rggb(oracle):
    """Same path with the RGGB phase (red at row 0, column 0)."""
    sc = synth.make_scene("quad_bayer", seed=4, width=128, height=96, bayer_red_row=0, bayer_red_col=0)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    ref = run_oracle(oracle, sc, 4.0)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        _check_tiles(oracle, tp, ref, 3)
        _check_clt(tp, ref)
        _check_corr(tp, ref)


@pytest.mark.parametrize("sched", [(0, 0), (1, 1), (4, 4), (1, 2)])
def test_circle16_extrinsics(oracle, sched):
    """16 LWIR sensors on a circle with extrinsic perturbations, all 120 pairs (generalised strips),
    under the default (pair per warp, 4 warps), warp-per-tile and 2-warp schedules."""
    sc = synth.make_scene("circle_lwir", seed=5, width=160, height=128)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    pairs = synth.circle_pairs(sc["geometry"])
    opairs = [(a, b, bx, by, kind) for (a, b, kind, _, bx, by) in pairs]
    ref = run_oracle(oracle, sc, 2.0, pairs=opairs)
    with make_gpu(sc) as tp:
        tp.setCorrelation(pairs=pairs)
        tp.setFullFrameImages(np.full(T, 2.0, np.float32))
        tp.setSchedule(*sched)
        tp.process()
        _check_tiles(oracle, tp, ref, 1)
        _check_clt(tp, ref)
        _check_corr(tp, ref)
        _check_disp(oracle, tp, ref, check_ortho=False)


def test_float_tasks_ragged(oracle):
    """setTasks with reference-layout float ports on a ragged subset of tiles incl. borders."""
    sc = synth.make_scene("quad_mono", seed=6, width=128, height=96)
    W, H = sc["width"], sc["height"]
    tX, tY = W // 8, H // 8
    T = tX * tY
    rng = np.random.default_rng(11)
    sel = np.sort(rng.choice(T, size=T // 3, replace=False))
    sel = np.union1d(sel, [0, tX - 1, T - tX, T - 1])
    tx, ty = sel % tX, sel // tX
    cx, cy = tx * 8 + 4.0, ty * 8 + 4.0
    # ports pushed out of the image on some tiles to exercise the mirrored border
    xy = np.stack([np.stack([cx - d * 5 * r[0], cy - d * 5 * r[1]], -1) for d, r in zip([1, 1, 1, 1], synth.QUAD_RXY)],
                  1).astype(np.float32) + rng.uniform(-3, 3, size=(len(sel), 4, 2)).astype(np.float32)
    ports_in = np.zeros((T, 4, 2))
    ports_in[sel] = xy.astype(np.float64)
    op = np.zeros(T, np.int32)
    op[sel] = 1
    ref = run_oracle(oracle, sc, 0.0, tile_op=op, ports_in=ports_in)
    from tileproc import GPUTileProcessor
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setTasks(GPUTileProcessor.packTasks(np.ones(len(sel)), tx, ty, xy))
        tp.process()
        assert np.array_equal(tp.getPorts(), ports_in[sel])
        tl, res = tp.getSubtiles()
        assert np.array_equal(tl, ref["int_tl"][sel])
        _check_clt(tp, ref, tile_mask=sel)
        _check_corr(tp, ref, tile_mask=sel)
        d = tp.getDisparity()
        untasked = np.setdiff1d(np.arange(T), sel)
        assert np.all(np.isnan(d[untasked, oracle.DISP_CM])) and np.all(d[untasked, oracle.DISP_STRENGTH] == 0)


def test_empty_task_list(oracle):
    sc = synth.make_scene("quad_mono", seed=8, width=64, height=64)
    T = 64
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.zeros(T, np.float32), tile_op=np.zeros(T, np.int32))
        tp.process()
        assert tp.numTasks() == 0
        d = tp.getDisparity()
        assert np.all(np.isnan(d[:, oracle.DISP_CM]))


def _oracle_rbg(O, clt, tilesX, tilesY, S, C, W, H, lpf=None):
    frames = np.zeros((S, C, H + 8, W + 8))
    for s in range(S):
        for c in range(C):
            f = frames[s, c]
            for t in range(tilesX * tilesY):
                q = clt[t, s, c]
                if lpf is not None:
                    q = q * lpf[c][None, :]
                O.iclt_tile_add(q, 0.25, t % tilesX, t // tilesX, f)
    return frames


def test_imclt(oracle):
    """IMCLT overlap-add into (W+8)x(H+8) frames vs ImageDtt.iclt_2d (x0.25) on the GPU's own CLT."""
    sc = synth.make_scene("quad_bayer", seed=9, width=192, height=128)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.process()
        tp.execImcltRbg()
        clt = tp.getClt().astype(np.float64)
        want = _oracle_rbg(oracle, clt, W // 8, H // 8, 4, 3, W, H)
        for s in range(4):
            got = tp.getRBG(s).astype(np.float64)
            err = np.abs(got - want[s]).max() / np.abs(want[s]).max()
            assert err < 2e-6, "sensor %d IMCLT max rel err %.3g" % (s, err)
        lpf = np.stack([oracle.clt_lpf(sg) for sg in (1.1, 1.1, 0.7)])
        tp.setLpfRbg(lpf)
        tp.execImcltRbg()
        want = _oracle_rbg(oracle, clt, W // 8, H // 8, 4, 3, W, H, lpf=lpf)
        got = tp.getRBG(2).astype(np.float64)
        assert np.abs(got - want[2]).max() / np.abs(want[2]).max() < 2e-6


@pytest.mark.parametrize("sched", [(0, 0), (1, 1), (2, 2), (4, 4), (1, 2), (1, 3), (1, 4)])
def test_stage_kernels_and_schedules_agree(oracle, sched):
    """Per-stage kernels (execConverCorrectTiles/execCorrelate/execExtract) and the fused
    kernel under several CTA schedules give the same results."""
    sc = synth.make_scene("quad_bayer", seed=12, width=192, height=128)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    rng = np.random.default_rng(3)
    k, e = synth.random_clt_kernels(rng, 4, 128 // 16 + 2, 192 // 16 + 2, 3)
    ref = run_oracle(oracle, sc, 4.0, kernels=k, kext=e)
    with make_gpu(sc, k, e) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 4.0, np.float32))
        tp.execPorts()
        tp.execConverCorrectTiles()
        tp.execCorrelate()
        tp.execExtract()
        clt_s, corr_s, d_s = tp.getClt(), tp.getCorr(), tp.getDisparity()
        tp.setSchedule(*sched)
        tp.process()
        clt_f, corr_f, d_f = tp.getClt(), tp.getCorr(), tp.getDisparity()
    for clt in (clt_s, clt_f):
        e1 = rel_l2(clt.astype(np.float64), ref["clt"], axis=(-2, -1))
        assert e1.max() <= CLT_TOL
    for corr in (corr_s, corr_f):
        e2 = rel_l2(corr.astype(np.float64), ref["corr"], axis=-1)
        assert e2.max() <= CORR_TOL
    for d in (d_s, d_f):
        check_disparity_strict(oracle, d.astype(np.float64), ref)


def test_bayer_planes_input_matches_mosaic(oracle):
    """setBayerPlanes (colour planes summed into a float mosaic, as GPUTileProcessor.setBayerImages
    does) with unit colour scales gives the CLT of the uint16 mosaic with scales (1, 1, 0.5)."""
    from helpers import oracle_planes
    sc = synth.make_scene("quad_bayer", seed=31, width=128, height=96)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    planes = oracle_planes(sc)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 3.0, np.float32))
        tp.process()
        ref = tp.getClt()
        tp.setBayerPlanes(planes)
        tp.setColorScales([1.0, 1.0, 1.0])
        tp.process()
        got = tp.getClt()
    assert np.array_equal(got, ref)


def test_zero_contrast_tiles(oracle):
    """Flat regions (all zero, all one) with a step edge: tiles without contrast have 0/0 in the
    fat-zero normalisation, so their surfaces are NaN and they get no disparity, as in the oracle;
    the tiles on the edge are compared as usual."""
    sc = synth.make_scene("quad_mono", seed=8, width=64, height=64)
    sc["images"][:] = 0.0
    sc["images"][:, 32:, :] = 1.0
    T = 64
    ref = run_oracle(oracle, sc, 2.0)
    with make_gpu(sc) as tp:
        tp.setCorrelation(fat_zero=0.05)
        tp.setFullFrameImages(np.full(T, 2.0, np.float32))
        tp.process()
        corr = tp.getCorr().astype(np.float64)
        d = tp.getDisparity()
    nan_ref, nan_gpu = np.isnan(ref["corr"]), np.isnan(corr)
    assert nan_ref.any() and np.array_equal(nan_ref, nan_gpu)
    fin = ~np.isnan(ref["corr"]).any(axis=-1)
    e = rel_l2(np.where(fin[..., None], corr, 0), np.where(fin[..., None], ref["corr"], 0), axis=-1)[fin]
    assert e.max() <= CORR_TOL, e.max()
    cm_ref, cm_gpu = ref["disp"][:, oracle.DISP_CM], d[:, oracle.DISP_CM]
    assert np.array_equal(np.isnan(cm_ref), np.isnan(cm_gpu))
    ok = ~np.isnan(cm_ref)
    assert np.abs(cm_gpu[ok] - cm_ref[ok]).max() <= DISP_TOL


def test_full_size_bayer_sampled_tiles(oracle):
    """The full-size workload (4 Bayer sensors 2592x1936 uint16, per-sensor/colour kernel tables on a
    16-px grid, 78,408 tiles, per-tile disparity in [0, 8] px) forward on the GPU; the oracle checks
    every 97th tile plus the four corners (about 800 tiles) at the stated tolerances, and the task
    list covers the frame in row-major order (bit-exact)."""
    sc = synth.make_scene("quad_bayer", seed=21, width=2592, height=1936)
    W, H = sc["width"], sc["height"]
    tX, tY = W // 8, H // 8
    T = tX * tY
    rng = np.random.default_rng(23)
    k, e = synth.random_clt_kernels(rng, 4, H // 16 + 2, W // 16 + 2, 3)
    disp = rng.uniform(0.0, 8.0, T).astype(np.float32)
    sel = np.union1d(np.arange(0, T, 97), [0, tX - 1, T - tX, T - 1])
    op = np.zeros(T, np.int32)
    op[sel] = 1
    ref = run_oracle(oracle, sc, disp.astype(np.float64), kernels=k, kext=e, tile_op=op)
    with make_gpu(sc, k, e) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp)
        tp.process()
        assert tp.numTasks() == T
        assert np.array_equal(tp.getTaskTiles(), (np.arange(T) % tX) | ((np.arange(T) // tX) << 16))
        assert np.array_equal(tp.getPorts()[sel], ref["ports"][sel])
        tl, res = tp.getSubtiles()
        assert np.array_equal(tl[sel], ref["int_tl"][sel])
        assert np.array_equal(res[sel], ref["residual"][sel].astype(np.float32))
        clt = tp.getClt()[sel].astype(np.float64)
        ec = rel_l2(clt, ref["clt"][sel], axis=(-2, -1))
        assert ec.max() <= CLT_TOL, "CLT rel L2 max %.3g" % ec.max()
        del clt
        corr = tp.getCorr()[sel].astype(np.float64)
        er = rel_l2(corr, ref["corr"][sel], axis=-1)
        assert er.max() <= CORR_TOL, "corr rel L2 max %.3g" % er.max()
        d = tp.getDisparity().astype(np.float64)
    assert np.isfinite(ref["disp"][sel, oracle.DISP_CM]).sum() > 0.9 * len(sel)
    summ = check_disparity_strict(oracle, d, ref, tiles=sel)
    print("full size: %d tiles checked, CLT max %.3g, corr max %.3g, disparity %s" % (len(sel), ec.max(), er.max(),
                                                                                       summ))


def test_full_size_circle16_sampled_tiles(oracle):
    """The full-size 16-sensor LWIR workload (640x512, 5120 tiles, all 120 pairs, extrinsic
    perturbations, per-tile disparity in [0, 4] px) under the default schedule; the oracle checks
    every 7th tile plus the corners (about 730 tiles)."""
    sc = synth.make_scene("circle_lwir", seed=25, dmax=4.0)
    W, H = sc["width"], sc["height"]
    tX, T = W // 8, (W // 8) * (H // 8)
    pairs = synth.circle_pairs(sc["geometry"])
    opairs = [(a, b, bx, by, kind) for (a, b, kind, _, bx, by) in pairs]
    disp = np.random.default_rng(27).uniform(0.0, 4.0, T).astype(np.float32)
    sel = np.union1d(np.arange(0, T, 7), [0, tX - 1, T - tX, T - 1])
    op = np.zeros(T, np.int32)
    op[sel] = 1
    ref = run_oracle(oracle, sc, disp.astype(np.float64), pairs=opairs, tile_op=op)
    with make_gpu(sc) as tp:
        tp.setCorrelation(pairs=pairs)
        tp.setFullFrameImages(disp)
        tp.process()
        assert tp.numTasks() == T
        assert np.array_equal(tp.getPorts()[sel], ref["ports"][sel])
        tl, _ = tp.getSubtiles()
        assert np.array_equal(tl[sel], ref["int_tl"][sel])
        ec = rel_l2(tp.getClt()[sel].astype(np.float64), ref["clt"][sel], axis=(-2, -1))
        assert ec.max() <= CLT_TOL, "CLT rel L2 max %.3g" % ec.max()
        er = rel_l2(tp.getCorr()[sel].astype(np.float64), ref["corr"][sel], axis=-1)
        assert er.max() <= CORR_TOL, "corr rel L2 max %.3g" % er.max()
        d = tp.getDisparity().astype(np.float64)
    assert np.isfinite(ref["disp"][sel, oracle.DISP_CM]).sum() > 0.9 * len(sel)
    summ = check_disparity_strict(oracle, d, ref, tiles=sel, check_ortho=False)
    print("full size LWIR: %d tiles checked, CLT max %.3g, corr max %.3g, disparity %s" % (
        len(sel), ec.max(), er.max(), summ))

