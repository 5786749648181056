"""Rig (main + auxiliary quad camera) inter-camera correlation against the oracle (needs a GB300).

The oracle is fed the GPU's own CLTs of both cameras, so the check isolates the
rig stage: sensor averaging, the pair correlation with the main camera's
settings, the horizontal strip, argmax and the centroid with its second moment.
Tolerances: correlation relative L2 per tile <= 1e-5; disparity <= 0.005 px
and strength relative <= 1e-3 on tiles whose integer argmax agrees.
"""
import numpy as np
import pytest

from helpers import make_gpu, rel_l2
from tileproc import synth

pytestmark = pytest.mark.gpu


def _rig_check(oracle, main_tp, aux_tp, aux_op, no_int_x0=False):
    corr, rec = main_tp.rigCorrelate(aux_tp, no_int_x0=no_int_x0)
    cm = main_tp.getClt().astype(np.float64)
    ca = aux_tp.getClt().astype(np.float64)
    T = cm.shape[0]
    n_ok = 0
    errs = []
    for t in range(T):
        if not aux_op[t]:
            assert np.isnan(rec[t, 0]) and rec[t, 1] == 0.0, "tile %d without an aux task" % t
            continue
        oc, orec = oracle.rig_tile(cm[t], ca[t], no_int_x0=no_int_x0)
        e = rel_l2(corr[t].astype(np.float64), oc, axis=-1)
        assert e <= 1e-5, "tile %d: rig corr rel L2 %.3g" % (t, e)
        assert np.isnan(rec[t, 2]) and np.isnan(rec[t, 3])
        if np.isnan(orec[0]):
            assert np.isnan(rec[t, 0]) and rec[t, 1] == 0.0
            continue
        if np.isnan(rec[t, 0]) or abs(rec[t, 0] - orec[0]) > 0.5:
            continue  # near-tie of the integer argmax (counted below)
        n_ok += 1
        errs.append(abs(rec[t, 0] - orec[0]))
        assert abs(rec[t, 1] - orec[1]) <= 1e-3 * abs(orec[1]) + 1e-6, "tile %d strength %g vs %g" % (
            t, rec[t, 1], orec[1])
    assert n_ok >= 0.9 * aux_op.sum()
    assert max(errs) <= 0.005, "rig disparity max err %.4g px" % max(errs)
    return rec


@pytest.mark.parametrize("kind", ["quad_bayer", "quad_mono"])
def test_rig_inter_camera(oracle, kind):
    """Auxiliary camera = the main scene shifted by 2 px, with a ragged task subset; the rig
    disparity of textured tiles recovers the shift."""
    sc = synth.make_scene(kind, seed=21, width=128, height=96)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    aux = dict(sc)
    aux["images"] = np.ascontiguousarray(np.roll(sc["images"], 2, axis=-1))
    rng = np.random.default_rng(5)
    aux_op = (rng.uniform(size=T) > 0.25).astype(np.int32)
    with make_gpu(sc) as tm, make_gpu(aux) as ta:
        for tp, op in ((tm, np.ones(T, np.int32)), (ta, aux_op)):
            tp.setCorrelation()
            tp.setFullFrameImages(np.full(T, 2.0, np.float32), tile_op=op)
            tp.process()
        rec = _rig_check(oracle, tm, ta, aux_op)
        # the 2-pixel roll shows up as the inter-camera disparity on most textured interior tiles
        tx, ty = np.arange(T) % (W // 8), np.arange(T) // (W // 8)
        inner = (aux_op > 0) & (tx > 1) & (tx < W // 8 - 2) & (ty > 1) & (ty < H // 8 - 2) & (rec[:, 1] > 0)
        d = rec[inner, 0]
        assert np.median(np.abs(np.abs(d) - 2.0)) < 0.5, "median rig disparity %g" % np.median(d)
        _rig_check(oracle, tm, ta, aux_op, no_int_x0=True)


def _rig_lma_compare(oracle, corr, rec0, rec, use_poly, use_xy_poly):
    """GPU rig record after rigLma against oracle.rig_lma fed the GPU's surfaces and CM record:
    disparity 0.005 px, strength 1e-3 relative, dx / dy 1e-3 px (or NaN on both) on >= 97% of the
    tiles the branch runs on; the rest keep the CM record unchanged."""
    p = oracle.default_lma_params()
    n = ok = fitted = 0
    bad = []
    for t in range(rec0.shape[0]):
        if not (np.isfinite(rec0[t, 0]) and rec0[t, 1] > p.min_poly_strength):
            assert np.array_equal(rec[t], rec0[t], equal_nan=True), "tile %d changed without the LMA" % t
            continue
        conv, want = oracle.rig_lma(corr[t], rec0[t], use_poly=use_poly, use_xy_poly=use_xy_poly)
        n += 1
        fitted += conv
        g = rec[t].astype(np.float64)
        same = (abs(g[0] - want[0]) <= 0.005 and abs(g[1] - want[1]) <= 1e-3 * abs(want[1]) + 1e-6 and
                np.allclose(g[2:], want[2:], rtol=0, atol=1e-3, equal_nan=True))
        ok += same
        if not same:
            bad.append((t, g.tolist(), want.tolist()))
    assert n > 20 and fitted > 0.5 * n, "rig LMA ran on %d tiles, converged on %d" % (n, fitted)
    assert ok >= 0.97 * n, "rig LMA record agrees on %d of %d tiles: %s" % (ok, n, bad[:3])


@pytest.mark.parametrize("kind", ["quad_bayer", "quad_mono"])
def test_rig_lma(oracle, kind):
    """The LMA branch of tileInterCamCorrs (ImageDtt.java:7497-7560) with rig.use_poly and
    rig.use_xy_poly on and off: the rig surface fitted like corrLMA, then single2dPoly or single2dCM."""
    from tileproc import _lib
    sc = synth.make_scene(kind, seed=23, width=128, height=96)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    aux = dict(sc)
    aux["images"] = np.ascontiguousarray(np.roll(sc["images"], 2, axis=-1))
    with make_gpu(sc) as tm, make_gpu(aux) as ta:
        for tp in (tm, ta):
            tp.setCorrelation()
            tp.setFullFrameImages(np.full(T, 2.0, np.float32))
            tp.process()
        for use_poly, use_xy_poly in ((True, True), (True, False), (False, True)):
            corr, rec0 = tm.rigCorrelate(ta)
            rec = tm.rigLma(use_poly=use_poly, use_xy_poly=use_xy_poly)
            _rig_lma_compare(oracle, corr, rec0, rec, use_poly, use_xy_poly)
            if not use_poly:
                assert np.array_equal(rec[:, :2], rec0[:, :2], equal_nan=True)
        with pytest.raises(_lib.TpError, match="already holds"):
            tm.rigLma()


def test_rig_rejects_mismatched_cameras():
    from tileproc import _lib
    sc = synth.make_scene("quad_mono", seed=22, width=64, height=64)
    sc2 = synth.make_scene("quad_mono", seed=22, width=128, height=64)
    with make_gpu(sc) as tm, make_gpu(sc2) as ta:
        tm.setCorrelation()
        with pytest.raises(_lib.TpError, match="differ in tile grid"):
            tm.rigCorrelate(ta)


def _aux_geometry(g, rng):
    """Another quad camera: its own lens (focal length, distortion, sensor centres) and extrinsics."""
    a = {k: (np.array(v, dtype=np.float64).copy() if isinstance(v, (list, tuple, np.ndarray)) else v)
         for k, v in g.items()}
    a["focal_length"] = g["focal_length"] * 1.05
    a["distortion"] = np.asarray(g["distortion"], np.float64) * 0.9
    a["pXY0"] = np.asarray(g["pXY0"], np.float64) + rng.uniform(-1.5, 1.5, (g["num_sensors"], 2))
    for k in ("azimuth", "tilt", "roll"):
        a[k] = np.asarray(g[k], np.float64) + rng.normal(0, 2e-3, g["num_sensors"])
    a["zoom"] = np.asarray(g["zoom"], np.float64) + rng.normal(0, 1e-3, g["num_sensors"])
    return a


RIG = dict(main_disparity_radius=21.0, aux_disparity_radius=18.5, baseline=6.0, aux_angle=0.35,
           aux_azimuth=1.5e-3, aux_tilt=-2e-3, aux_roll=4e-3, aux_zoom=1e-3)


def test_rig_aux_geometry(oracle):
    """The auxiliary camera's ports with GeometryCorrection.RigOffset (ImageDtt.clt_bi_quad,
    ImageDtt.java:8972-8996): main-camera disparities scaled by the radii, the centre undistorted with
    the main camera's lens, rXY_aux and the rig rotation.  Ports bit-exact against the oracle on every
    tile, the auxiliary CLT / correlation at the forward's tolerances, then the rig correlation."""
    from helpers import run_oracle
    sc = synth.make_scene("quad_mono", seed=31, width=128, height=96)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    rng = np.random.default_rng(32)
    g_main = sc["geometry"]
    g_aux = _aux_geometry(g_main, rng)
    disp = rng.uniform(0.5, 4.0, T).astype(np.float32)  # main-camera disparities
    tx, ty = np.arange(T) % (W // 8), np.arange(T) // (W // 8)
    want = np.array([oracle.rig_aux_ports(g_aux, g_main, RIG, x * 8 + 4, y * 8 + 4, d)
                     for x, y, d in zip(tx, ty, disp.astype(np.float64))])
    ref = run_oracle(oracle, sc, 0.0, ports_in=want)
    with make_gpu(sc) as tm, make_gpu(sc) as ta:
        ta.setRigGeometry(g_aux, g_main, RIG)
        for tp in (tm, ta):
            tp.setCorrelation()
            tp.setFullFrameImages(disp)
            tp.process()
        got = ta.getPorts()
        assert np.array_equal(got, want), "aux ports differ: max %g" % np.abs(got - want).max()
        e = rel_l2(ta.getClt().astype(np.float64), ref["clt"], axis=(-2, -1))
        assert e.max() <= 2e-6, "aux CLT rel L2 max %.3g" % e.max()
        e = rel_l2(ta.getCorr().astype(np.float64), ref["corr"], axis=-1)
        assert e.max() <= 1e-5, "aux corr rel L2 max %.3g" % e.max()
        _rig_check(oracle, tm, ta, np.ones(T, np.int32))
        # without the rig the same handle computes the camera's own ports
        ta.setGeometry(g_aux)
        ta.process()
        own = np.array([oracle.ports(g_aux, x * 8 + 4, y * 8 + 4, d) for x, y, d in zip(tx, ty, disp.astype(np.float64))])
        assert np.array_equal(ta.getPorts(), own)


def test_rig_geometry_rejects_bad_radii():
    from tileproc import _lib
    sc = synth.make_scene("quad_mono", seed=33, width=64, height=64)
    bad = dict(RIG, aux_disparity_radius=0.0)
    with make_gpu(sc) as ta:
        with pytest.raises(_lib.TpError, match="disparity radii"):
            ta.setRigGeometry(sc["geometry"], sc["geometry"], bad)
