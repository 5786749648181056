"""Adjoint of the forward chain (tp_backward) on the GPU, checked by central
finite differences of the FP64 oracle and against the oracle's FP64 port
derivatives (GeometryCorrection.getPortsCoordinatesAndDerivatives).

Scene: 16 mono LWIR sensors on a circle (radius 100 mm, f 4.9 mm, 12 um
pixels), 160x128 (320 tiles), all 120 pairs, extrinsics perturbed by
N(0, 1e-3) rad and target disparities off the truth by N(0, 0.2) px so the
measured residual disparities d are not zero.

Tolerances: port derivatives (FP64 on the device) to 1e-10 relative; the
per-tile port sensitivities dd/dport to 2e-3 + 3% of the finite difference;
the loss gradient at 200 seeded coordinates to 3% of the finite difference.
Every sample is held to its tolerance except the ones whose central difference
straddles a discontinuity of the forward, which the oracle lists: an integer
window corner (-round(-px)), a tile's integer argmax, or a combined-strip
sample clipped to zero (a pair's strip value + offset <= 0 zeroes the geometric
mean, and a small change un-clips it: x^(1/n) has an infinite slope at 0) that
differs between the + and the - evaluation.  The adjoint holds those fixed, so
there the finite difference measures a jump, not the derivative.  Steps: 1e-4 for the tile
disparities (as specified); 1e-6 rad for the extrinsics, because 1e-4 rad
moves every port of a sensor by ~0.04 px and switches the corners of ~8% of
its sub-tiles: on this scene the central difference for sensor 0's azimuth is
9029 at 1e-4, 3821 at 1e-5 and 4242 at 3e-6 ... 3e-7, so only the small step
measures the derivative.
"""
import copy

import numpy as np
import pytest

from tileproc import GPUTileProcessor, synth

pytestmark = pytest.mark.gpu

W, H = 160, 128
T = (W // 8) * (H // 8)


def _setup(seed=31):
    sc = synth.make_scene("circle_lwir", seed=seed, width=W, height=H)
    rng = np.random.default_rng(seed + 1)
    g = copy.deepcopy(sc["geometry"])
    for k in ("azimuth", "tilt", "roll", "zoom"):
        g[k] = (np.asarray(g[k]) + rng.normal(0, 1e-3, 16)).tolist()
    pairs = synth.circle_pairs(g)
    D = (sc["disparity_gt"].reshape(-1) + rng.normal(0, 0.2, T)).astype(np.float32)
    return sc, g, pairs, D


def _gpu(sc, g, pairs, D):
    tp = GPUTileProcessor(16, W, H)
    tp.setGeometry(g)
    tp.setBayerImages(sc["images"])
    tp.setCorrelation(pairs=pairs)
    tp.setFullFrameImages(D, tile_op=np.ones(T, np.int32))
    tp.process()
    return tp


def _oracle_run(O, sc, g, pairs, D, tile_op=None, ports_in=None):
    """(centroid disparity [T], integer window corners [T][S][1][2], integer argmax [T], clipped
    combined-strip samples [T][rows * 15] (exactly 0 or NaN))"""
    op = np.ones(T, np.int32) if tile_op is None else tile_op
    P = O.make_pairs([(a, b, bx, by, kind) for (a, b, kind, _, bx, by) in pairs])
    r = O.run(W, H, sc["images"][:, None].astype(np.float64), op, np.asarray(D, np.float64),
              geometry=None if ports_in is not None else g, ports_in=ports_in, pairs=P,
              want=("disp", "int_tl", "diag"))
    rows = O.default_corr_params().corr_wndy_size  # the rows the centroid reads
    combo = r["diag"][:, :15 * rows]
    return r["disp"][:, O.DISP_CM], r["int_tl"], r["disp"][:, O.DISP_IXY], (combo == 0.0) | np.isnan(combo)


def _oracle_d(O, sc, g, pairs, D, tile_op=None, ports_in=None):
    return _oracle_run(O, sc, g, pairs, D, tile_op, ports_in)[0]


def _switched(a, b, tiles=slice(None)):
    """a discontinuity of the forward between two oracle evaluations: a window corner, an integer
    argmax or a clipped combined-strip sample of one of the tiles differs"""
    _, tl_a, ix_a, z_a = a
    _, tl_b, ix_b, z_b = b
    return (not np.array_equal(tl_a[tiles], tl_b[tiles])) or (
        not np.array_equal(ix_a[tiles], ix_b[tiles], equal_nan=True)) or (not np.array_equal(z_a[tiles], z_b[tiles]))


def test_port_derivatives_match_oracle(oracle):
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        ports0 = tp.getPorts()
        tp.backward()
        assert np.array_equal(tp.getPorts(), ports0), "the backward plan moved the ports"
        dv = tp.getPortDerivatives()
        txy = tp.getTaskTiles()
    rng = np.random.default_rng(5)
    for t in rng.choice(len(txy), 24, replace=False):
        tx, ty = txy[t] & 0xFFFF, txy[t] >> 16
        cx, cy, dd = tx * 8 + 4.0, ty * 8 + 4.0, float(D[t])
        pref, dref = oracle.ports(g, cx, cy, dd, deriv=True)
        assert np.allclose(dv[t, :, :, :4], dref, rtol=1e-10, atol=1e-12)
        h = 1e-4
        fd = (oracle.ports(g, cx, cy, dd + h) - oracle.ports(g, cx, cy, dd - h)) / (2 * h)
        assert np.allclose(dv[t, :, :, 4], fd, rtol=1e-6, atol=1e-8)


def test_port_sensitivities_match_finite_differences(oracle):
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        tp.backward()
        sens = tp.getPortSensitivities()
        ports = tp.getPorts()
        txy = tp.getTaskTiles()
    d0 = _oracle_d(oracle, sc, g, pairs, D)
    rng = np.random.default_rng(6)
    valid = np.nonzero(np.isfinite(d0))[0]
    h = 1e-3
    errs = []
    for t in rng.choice(valid, 10, replace=False):
        tile = (txy[t] >> 16) * (W // 8) + (txy[t] & 0xFFFF)
        op = np.zeros(T, np.int32)
        op[tile] = 1
        for s in rng.choice(16, 3, replace=False):
            for ax in range(2):
                pp = ports.copy()
                pp[t, s, ax] += h
                rp = _oracle_run(oracle, sc, g, pairs, D, op, pp)
                pp[t, s, ax] -= 2 * h
                rm = _oracle_run(oracle, sc, g, pairs, D, op, pp)
                fd = (rp[0][tile] - rm[0][tile]) / (2 * h)
                errs.append((sens[tile, s, ax], fd, _switched(rp, rm, tile)))
    e = np.array([(a, b) for a, b, _ in errs])
    sw = np.array([c for _, _, c in errs])
    bad = (np.abs(e[:, 0] - e[:, 1]) > 2e-3 + 0.03 * np.abs(e[:, 1])) & ~sw
    print("dd/dport: max |fd| %.3g, max err %.3g, %d of %d samples straddle a switch" % (
        np.abs(e[:, 1]).max(), np.abs(e[~sw, 0] - e[~sw, 1]).max(), sw.sum(), len(sw)))
    assert not bad.any(), e[bad]
    assert sw.mean() <= 0.2


def test_loss_gradient_matches_finite_differences(oracle):
    """200 seeded coordinates, central differences of L = sum d^2 (FP64 oracle; steps in the module
    docstring); the adjoint is driven with dL/dd = 2 d of the oracle so only its Jacobian is compared."""
    sc, g, pairs, D = _setup()
    d0 = _oracle_d(oracle, sc, g, pairs, D)
    dl = np.where(np.isfinite(d0), 2 * d0, 0.0).astype(np.float32)
    with _gpu(sc, g, pairs, D) as tp:
        ge, gd = tp.backward(dl_ddisp=dl)
        ports = tp.getPorts()
        txy = tp.getTaskTiles()
    rng = np.random.default_rng(7)
    keys = ("azimuth", "tilt", "roll", "zoom")
    h, he = 1e-4, 1e-6

    def loss(r):
        d = r[0]
        return float(np.nansum(np.where(np.isfinite(d), d * d, 0.0)))

    rows = []
    for flat in rng.choice(64, 40, replace=False):
        s, k = flat // 4, flat % 4
        gp, gm = copy.deepcopy(g), copy.deepcopy(g)
        gp[keys[k]][s] += he
        gm[keys[k]][s] -= he
        rp, rm = _oracle_run(oracle, sc, gp, pairs, D), _oracle_run(oracle, sc, gm, pairs, D)
        rows.append(("e", ge[s, k], (loss(rp) - loss(rm)) / (2 * he), _switched(rp, rm)))
    valid = np.nonzero(np.isfinite(d0))[0]
    for t in rng.choice(valid, 160, replace=False):
        op = np.zeros(T, np.int32)
        op[t] = 1
        Dp, Dm = D.astype(np.float64), D.astype(np.float64)
        Dp[t] += h
        Dm[t] -= h
        rp = _oracle_run(oracle, sc, g, pairs, Dp, op)
        rm = _oracle_run(oracle, sc, g, pairs, Dm, op)
        dp, dm = rp[0][t], rm[0][t]
        rows.append(("d", gd[t], (dp * dp - dm * dm) / (2 * h), _switched(rp, rm, t)))
    got = np.array([r[1] for r in rows], np.float64)
    fd = np.array([r[2] for r in rows], np.float64)
    sw = np.array([r[3] for r in rows])
    held = ~sw
    scale = np.array([np.abs(fd[:40][held[:40]]).max()] * 40 + [np.abs(fd[40:][held[40:]]).max()] * 160)
    rel = np.abs(got - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
    print("loss gradient: extrinsic rel err median %.3g max %.3g (%d of 40 straddle a switch); disparity median "
          "%.3g max %.3g (%d of 160)" % (np.median(rel[:40][held[:40]]), rel[:40][held[:40]].max(), sw[:40].sum(),
                                       np.median(rel[40:][held[40:]]), rel[40:][held[40:]].max(), sw[40:].sum()))
    bad = (rel > 0.03) & held
    assert not bad.any(), [(i, rows[i][0], got[i], fd[i]) for i in np.nonzero(bad)[0]]
    assert sw[:40].sum() <= 16 and sw[40:].sum() <= 16


def test_recompute_mode_matches_stored_clt(oracle):
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        ge0, gd0 = tp.backward()
        tp.setAdjointMode(recompute_clt=True)
        ge1, gd1 = tp.backward()
    assert np.allclose(ge1, ge0, rtol=1e-4, atol=1e-4 * np.abs(ge0).max())
    assert np.allclose(gd1, gd0, rtol=1e-4, atol=1e-4 * np.abs(gd0).max())


def test_recorded_strip_samples_match_reinterpolation(oracle):
    """The first backward re-interpolates the strips from the correlation surfaces; forwards after
    it record the samples, which the next backward reads.  The samples are the same numbers up to
    the rounding of the two interpolation routes, so the gradients agree to that rounding."""
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        ge0, gd0 = tp.backward()
        tp.process()
        ge1, gd1 = tp.backward()
        jd1 = tp.getDisparityJacobian()
        tp.process()
        ge2, gd2 = tp.backward()
    for a, b in ((ge1, ge0), (gd1, gd0), (ge2, ge1), (gd2, gd1)):
        assert np.allclose(a, b, rtol=1e-5, atol=1e-5 * np.abs(b).max())
    assert np.isfinite(ge0).all() and np.abs(ge0).max() > 0 and jd1 is not None


def test_lma_reduces_cost(oracle):
    """Levenberg-Marquardt on the analytic Jacobian alone (no coarse stage) from extrinsics perturbed
    by N(0, 3e-3) rad on the 160x128 crop, target disparities at the scene truth
    (free_disparity=False): the cost (d^2 capped at 1 px^2, 1 px^2 for a tile without a peak) falls
    at every step and to below half.  The crop's 320 tiles do not pin the 64 extrinsics (the fit
    lowers the cost without approaching the truth); the full scene does,
    test_lma_recovers_extrinsics_full_scene."""
    from tileproc import lma
    sc = synth.make_scene("circle_lwir", seed=41, width=W, height=H)
    rng = np.random.default_rng(42)
    g0 = copy.deepcopy(sc["geometry"])
    for k in lma.KEYS:
        g0[k] = (np.asarray(g0[k]) + rng.normal(0, 3e-3, 16)).tolist()
    D = sc["disparity_gt"].reshape(-1).astype(np.float32)
    with _gpu(sc, g0, synth.circle_pairs(g0), D) as tp:
        g, Dn, hist = lma.refine(tp, g0, D, iterations=20, free_disparity=False, coarse=0)
    print("LMA cost:", ["%.4g" % c for c in hist])
    assert all(b <= a for a, b in zip(hist, hist[1:]))
    assert hist[-1] < 0.5 * hist[0]


def test_lma_recovers_extrinsics_full_scene(oracle):
    """The same on the full 16x640x512 scene (5120 tiles), with the coarse stage first (Gauss-Newton
    on every pair's 2D correlation maximum) and 80 iterations: the error of the extrinsics against
    the seeded truth, less each parameter's mean over the 16 sensors (a rotation or zoom of the whole
    camera, which pair disparities do not see), falls to below a fifth (measured: from 2.6e-3 to
    about 1e-4 rad; the adjoint is deterministic, so the run repeats exactly)."""
    from tileproc import lma
    w, h = 640, 512
    t = (w // 8) * (h // 8)
    sc = synth.make_scene("circle_lwir", seed=1, width=w, height=h)
    rng = np.random.default_rng(12)
    gt = sc["geometry"]
    g0 = copy.deepcopy(gt)
    for k in lma.KEYS:
        g0[k] = (np.asarray(g0[k]) + rng.normal(0, 3e-3, 16)).tolist()
    D = sc["disparity_gt"].reshape(-1).astype(np.float32)
    with GPUTileProcessor(16, w, h) as tp:
        tp.setGeometry(g0)
        tp.setBayerImages(sc["images"])
        tp.setCorrelation(pairs=synth.circle_pairs(gt))
        tp.setFullFrameImages(D, tile_op=np.ones(t, np.int32))
        g, Dn, hist = lma.refine(tp, g0, D, iterations=80, free_disparity=False)

    def err(gg):
        e = np.array([np.asarray(gg[k]) - np.asarray(gt[k]) for k in lma.KEYS])
        e -= e.mean(axis=1, keepdims=True)
        return float(np.sqrt(np.mean(e * e)))

    print("LMA cost %.4g -> %.4g, error %.3g -> %.3g" % (hist[0], hist[-1], err(g0), err(g)))
    assert all(b <= a for a, b in zip(hist, hist[1:]))
    assert err(g) < err(g0) / 5


def test_backward_is_deterministic():
    """The adjoint's sums over pairs and tiles are taken in a fixed order (the pairs of a tile in
    rounds on distinct sensors, the tiles' gradient terms in block order; only a pair's own strip
    taps use one warp's shared-memory atomics), and repeated backward passes over the same forward
    agree bit for bit; the extrinsic refinement then repeats exactly."""
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        runs = []
        for _ in range(3):
            ge, gd = tp.backward()
            runs.append((ge, gd, tp.getPortSensitivities()) + tuple(tp.getDisparityJacobian()))
    assert np.isfinite(runs[0][2]).any()
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("seed,free", [(13, False), (14, False), (13, True)])
def test_coarse_stage_recovers_extrinsics(seed, free):
    """The coarse stage alone (lma._coarse_stage) on the full 16x640x512 scene from extrinsics off
    by N(0, 3e-3) rad, the starts where the adjoint-driven iteration alone stops in a dead end: the
    error less each parameter's mean over the sensors falls below a twentieth (measured: 2.6e-3 ..
    3.3e-3 to 3e-5 rad for azimuth and tilt, 1e-5 for roll and zoom, in 3 to 5 steps), and the sums
    over the sensors, which the offsets barely see, are held.  With free disparities (target
    disparities also off by N(0, 0.3) px and fitted per tile) the extrinsics reach 1e-5 rad and the
    disparities' median error falls from 0.20 to 0.14 px (measured)."""
    from tileproc import lma
    w, h = 640, 512
    t = (w // 8) * (h // 8)
    sc = synth.make_scene("circle_lwir", seed=1, width=w, height=h)
    rng = np.random.default_rng(seed)
    gt = sc["geometry"]
    g0 = copy.deepcopy(gt)
    for k in lma.KEYS:
        g0[k] = (np.asarray(g0[k]) + rng.normal(0, 3e-3, 16)).tolist()
    Dt = sc["disparity_gt"].reshape(-1).astype(np.float64)
    D = Dt + rng.normal(0, 0.3, t) if free else Dt
    with GPUTileProcessor(16, w, h) as tp:
        tp.setGeometry(g0)
        tp.setBayerImages(sc["images"])
        tp.setCorrelation(pairs=synth.circle_pairs(gt))
        g, Dn, costs = lma._coarse_stage(tp, g0, D, np.ones(t, np.int32), lma.COARSE, free, None)

    def err(gg):
        e = np.array([np.asarray(gg[k]) - np.asarray(gt[k]) for k in lma.KEYS])
        e -= e.mean(axis=1, keepdims=True)
        return float(np.sqrt(np.mean(e * e)))

    print("coarse stage: costs %s, error %.3g -> %.3g" % ([round(c) for c in costs], err(g0), err(g)))
    assert all(b < a for a, b in zip(costs, costs[1:]))
    assert err(g) < err(g0) / 20
    for k in lma.KEYS:
        assert abs(sum(g[k]) - sum(g0[k])) < 1e-6
    if free:
        before, after = np.median(np.abs(D - Dt)), np.median(np.abs(Dn - Dt))
        print("disparity median error %.3f -> %.3f px" % (before, after))
        assert after < 0.8 * before


def test_pair_maxima_match_host_statement():
    """tp_get_pair_maxima (a warp per pair surface on the device) against lma.pair_peaks on the
    surfaces read back: the same cells (border and non-finite maxima in the same places), the same
    strengths, offsets within 1e-4 px (the device evaluates the parabola in FP32, the host in FP64)."""
    from tileproc import lma
    sc, g, pairs, D = _setup()
    with _gpu(sc, g, pairs, D) as tp:
        pm = tp.getPairMaxima()
        corr = tp.getCorr()
    P = len(pairs)
    off, st = lma.pair_peaks(corr.reshape(-1, 225))
    off, st = off.reshape(T, P, 2), st.reshape(T, P)
    ok = np.isfinite(off).all(axis=-1)
    assert ok.mean() > 0.9
    assert np.array_equal(ok, np.isfinite(pm[..., :2]).all(axis=-1))
    assert np.abs(pm[..., :2][ok] - off[ok]).max() < 1e-4
    assert np.array_equal(pm[..., 2][ok], st[ok].astype(np.float32))
    assert (pm[..., 2][~ok] == 0).all()
