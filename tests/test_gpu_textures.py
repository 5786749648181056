"""GPU texture tiles (ImageDtt.java:2662-2812) vs the FP64 oracle (needs a GB300).

The oracle is fed the GPU's own CLT (so only the texture stage is compared) and,
in the end-to-end case, its own CLT.  Tolerances per tile: relative L2 <= 2e-5
for RGB and alpha, <= 1e-4 for the port weights (exp of a weighted squared
difference divided by window^2), absolute <= 1e-3 x the tile's RGB scale for the
rms rows (the oracle's s0*s2 - s1^2 loses digits the GPU's centred sum keeps),
<= 1e-4 of the tile's scale for max_diff and 1e-5 for ports_rgb, and the same
NaN pattern (the FP64 reference's weights underflow to 0/0 -> NaN where every
weight exponent exceeds 745.13; the GPU reproduces it).

The texture stage makes discrete per-pixel choices (the second port of the best
pair against the next port, dust_remove's weakest port) on weights that FP32
computes to about 1e-6 relative (an exponent argument of tens carries ~6e-8 relative error each), so a choice whose FP64 margin is below
TIE_RES = 1e-5 may go either way.  The oracle evaluates each tile both ways
(oracle.texture_tile(..., diag=True): every such near tie taken the other way).
Every tile must meet the bounds against the reference in which each output
element is the closer of the two resolutions -- for a tile without such ties
that is the oracle's own output.  max_diff is checked on the tiles without
such ties, and tiles in which a pixel's weight exponents come within UF_MARGIN
of the double underflow of exp (745.13: FP32 may land on the other side of it)
compare the elements that are finite in both.  The tiles with ties are counted
and printed.
"""
import numpy as np
import pytest

from helpers import make_gpu, rel_l2, run_oracle
from tileproc import synth

pytestmark = pytest.mark.gpu

RGB_TOL = 2e-5
W_TOL = 1e-4


def _col_weights(corr_red=0.5, corr_blue=0.2):
    g = 1.0 / (1.0 + corr_red + corr_blue)
    return np.array([corr_red * g, corr_blue * g, g])


UF_MARGIN = 0.05
TIE_RES = 1e-5


def _oracle_textures(O, clt, disp, tile_op, tiles, extra_slot=None, params=None, **kw):
    lpf = O.corr_lpf(0.8)
    cw = _col_weights()
    outs, auxs, diags, alts = [], [], [], []
    for t in tiles:
        op = int(tile_op[t])
        extra = 0.0
        if extra_slot is not None and not (op & 0x100):
            extra = float(disp[t, extra_slot])
            if not np.isfinite(extra):
                extra = 0.0
        o, a, dg, alt = O.texture_tile(clt[t], lpf, op & 0xF, cw, extra, params or O.texture_params(**kw),
                                       diag=True, near_tie=TIE_RES)
        outs.append(o)
        auxs.append(a)
        diags.append(dg)
        alts.append(alt)
    return np.array(outs), np.array(auxs), np.array(diags), np.array(alts)


def _compare(got, aux, want, want_aux, diag, alt, rows=12):
    n = len(got)
    tied = ~np.all(np.isclose(np.nan_to_num(alt[:, :8]), np.nan_to_num(want[:, :8]), rtol=0, atol=0), axis=(1, 2))
    uflow = diag[:, 2] < UF_MARGIN
    # the reference: each element the closer of the two tie resolutions (the oracle's own where none)
    k = min(rows, 8)
    want = want.copy()
    closer = np.abs(np.nan_to_num(got[:, :k] - alt[:, :k])) < np.abs(np.nan_to_num(got[:, :k] - want[:, :k]))
    want[:, :k] = np.where(closer, alt[:, :k], want[:, :k])
    nan_g, nan_w = np.isnan(got[:, :min(rows, 8)]), np.isnan(want[:, :min(rows, 8)])
    nan_bad = (nan_g != nan_w).reshape(n, -1).any(axis=-1) & ~uflow
    both = nan_g | nan_w
    g8 = np.where(both, 0.0, got[:, :min(rows, 8)])
    w8 = np.where(both, 0.0, want[:, :min(rows, 8)])
    e_rgb = rel_l2(g8[:, 0:3].reshape(n, -1), w8[:, 0:3].reshape(n, -1), axis=-1)
    e_a = rel_l2(g8[:, 3], w8[:, 3], axis=-1)
    bad = nan_bad | (e_rgb > RGB_TOL) | (e_a > RGB_TOL)
    e_w = e_r = np.zeros(n)
    if rows > 4:
        e_w = rel_l2(g8[:, 4:8].reshape(n, -1), w8[:, 4:8].reshape(n, -1), axis=-1)
        scale = np.abs(w8[:, 0:3]).reshape(n, -1).max(axis=-1)
        rms_d = np.where(np.isnan(want[:, 8:12]), 0.0, np.abs(got[:, 8:12] - want[:, 8:12]))
        e_r = rms_d.reshape(n, -1).max(axis=-1) / np.maximum(scale, 1e-30)
        bad |= (e_w > W_TOL) | (e_r > 1e-3)
    if aux is not None:
        e_md = (np.abs(aux[:, :4] - want_aux[:, :4]) / np.maximum(np.abs(want_aux[:, :4]).max(), 1e-30)).max(axis=-1)
        e_pr = (np.abs(aux[:, 4:] - want_aux[:, 4:]) / np.maximum(np.abs(want_aux[:, 4:]).max(), 1e-30)).max(axis=-1)
        bad |= ((e_md > 1e-4) & ~tied) | (e_pr > 1e-5)
    msg = "%d tiles: rgb %.3g alpha %.3g weights %.3g rms %.3g (max); %d with near ties, %d at the underflow" % (
        n, np.nanmax(e_rgb), np.nanmax(e_a), np.nanmax(e_w), np.nanmax(e_r), tied.sum(), uflow.sum())
    fails = np.nonzero(bad)[0]
    assert len(fails) == 0, "%d tiles out of tolerance %s (rgb %s, alpha %s, weights %s, near ties %s); %s" % (
        len(fails), fails[:6].tolist(), e_rgb[fails[:6]].tolist(), e_a[fails[:6]].tolist(), e_w[fails[:6]].tolist(),
        tied[fails[:6]].tolist(), msg)
    return msg


def _scene_ops(T, rng):
    ops = np.full(T, 0xF, np.int32)
    k = rng.integers(0, 10, T)
    ops[k == 0] = 0x7
    ops[k == 1] = 0x9
    ops[k == 2] = 0x4
    ops[k == 3] |= 0x100  # forced disparity: no extra shift
    ops[rng.integers(0, 25, T) == 0] = 0  # no task
    return ops


def test_textures_on_gpu_clt(oracle):
    """Texture stage alone: the oracle gets the GPU's CLT and centroid disparity (corr_mode 1)."""
    sc = synth.make_scene("quad_bayer", seed=21, width=192, height=128)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    rng = np.random.default_rng(22)
    ops = _scene_ops(T, rng)
    disp = sc["disparity_gt"].reshape(-1).astype(np.float32) + rng.normal(0, 0.3, T).astype(np.float32)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp, tile_op=ops)
        tp.process()
        tp.setTextureParams(corr_mode=1)
        tp.execTextures()
        got = tp.getTextures().astype(np.float64)
        aux = tp.getTextureAux().astype(np.float64)
        clt = tp.getClt().astype(np.float64)
        d = tp.getDisparity().astype(np.float64)
    tiles = np.nonzero(ops)[0]
    want, want_aux, diag, alt = _oracle_textures(oracle, clt, d, ops, tiles, extra_slot=oracle.DISP_CM)
    print(_compare(got[tiles], aux[tiles], want, want_aux, diag, alt))


def test_textures_poly_shift_after_lma(oracle):
    """corr_mode 2 (the default): the extra shift is the LMA ("POLY") disparity of tp_lma_refine on the
    current forward (ImageDtt.java:2424), zero where the LMA did not fit; the oracle gets the GPU's CLT
    and LMA record.  Without an LMA pass after the forward there is no extra shift."""
    sc = synth.make_scene("quad_bayer", seed=29, width=192, height=128)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    rng = np.random.default_rng(30)
    ops = _scene_ops(T, rng)
    disp = sc["disparity_gt"].reshape(-1).astype(np.float32) + rng.normal(0, 0.3, T).astype(np.float32)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp, tile_op=ops)
        tp.process()
        lma = tp.lmaRefine().astype(np.float64)
        tp.setTextureParams(corr_mode=2)
        tp.execTextures()
        got = tp.getTextures().astype(np.float64)
        aux = tp.getTextureAux().astype(np.float64)
        clt = tp.getClt().astype(np.float64)
        tp.process()  # a new forward drops the LMA: no extra shift
        tp.execTextures()
        got0 = tp.getTextures().astype(np.float64)
    tiles = np.nonzero(ops)[0]
    shifted = tiles[np.isfinite(lma[tiles, 0]) & (lma[tiles, 0] != 0) & ((ops[tiles] & 0x100) == 0)]
    assert len(shifted) > 0.5 * len(tiles)
    want, want_aux, diag, alt = _oracle_textures(oracle, clt, lma, ops, tiles, extra_slot=0)
    print(_compare(got[tiles], aux[tiles], want, want_aux, diag, alt))
    want0, _, _, _ = _oracle_textures(oracle, clt, lma, ops, tiles)
    g0 = np.nan_to_num(got0[tiles, :4])
    assert np.allclose(g0, np.nan_to_num(want0[:, :4]), rtol=1e-3, atol=1e-3 * np.abs(g0).max())


def test_textures_end_to_end(oracle):
    """Image -> CLT -> textures on the GPU vs the oracle's own chain (default corr_mode: no extra shift)."""
    sc = synth.make_scene("quad_bayer", seed=23, width=128, height=96)
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    ops = _scene_ops(T, np.random.default_rng(24))
    disp = sc["disparity_gt"].reshape(-1).astype(np.float64)
    ref = run_oracle(oracle, sc, disp, tile_op=ops)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(disp.astype(np.float32), tile_op=ops)
        tp.process()
        tp.setTextureParams()
        tp.execTextures()
        got = tp.getTextures().astype(np.float64)
        aux = tp.getTextureAux().astype(np.float64)
    tiles = np.nonzero(ops)[0]
    want, want_aux, diag, alt = _oracle_textures(oracle, ref["clt"], ref["disp"], ops, tiles)
    print(_compare(got[tiles], aux[tiles], want, want_aux, diag, alt))


def test_textures_rgba_only_and_no_shot(oracle):
    """keep_weights off (4 rows), shot-noise correction and dust removal off."""
    sc = synth.make_scene("quad_bayer", seed=25, width=128, height=96)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    ops = np.full(T, 0xF, np.int32)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full(T, 3.0, np.float32), tile_op=ops)
        tp.process()
        tp.setTextureParams(keep_weights=0, scale_shot=0.0, dust_remove=0, aux=0)
        tp.execTextures()
        got = tp.getTextures().astype(np.float64)
        clt = tp.getClt().astype(np.float64)
        d = tp.getDisparity().astype(np.float64)
    assert got.shape[1] == 4
    tiles = np.arange(T)
    want, _, diag, alt = _oracle_textures(oracle, clt, d, ops, tiles, scale_shot=0.0, dust_remove=0)
    print(_compare(got, None, want, None, diag, alt, rows=4))


def test_textures_reject_mono(oracle):
    sc = synth.make_scene("quad_mono", seed=2, width=128, height=96)
    with make_gpu(sc) as tp:
        tp.setCorrelation()
        tp.setFullFrameImages(np.full((sc["width"] // 8) * (sc["height"] // 8), 2.0, np.float32))
        tp.process()
        with pytest.raises(RuntimeError, match="4 sensors x 3 colours"):
            tp.execTextures()
