"""CPU checks of the oracle's LMA restatement (Correlation2d.corrLMA / Correlations2dLMA) on surfaces
built from its own model, where the fitted centre is known."""
import numpy as np

from oracle import oracle as O

KINDS = [0, 0, 1, 1, 2, 3]


def _model_surfaces(x0, amp=(0.6, 0.5), w=2.0):
    """The six quad pair surfaces of Ag (1 - ((x - x0) s / W)^2 - (y s / W)^2), s = 1 (ortho) or
    sqrt 2 (diagonal), in each pair's own orientation (vertical pairs transposed, other diagonal
    flipped).  With W equal to the default half-width and no x/y asymmetry the model is exact, so
    the regularised fit has zero residual at the true centre."""
    yy, xx = np.mgrid[-7:8, -7:8].astype(np.float64)
    ortho = amp[0] * (1 - ((xx - x0) / w) ** 2 - (yy / w) ** 2)
    # diagonal group: disparity along the main diagonal; rotate into (along, across) coordinates
    a = (xx + yy) / 2.0
    b = (yy - xx) / 2.0
    s = np.sqrt(2.0)
    diag = amp[1] * (1 - ((a - x0) * s / w) ** 2 - (b * s / w) ** 2)
    return np.stack([ortho, ortho, ortho.T, ortho.T, diag, diag[::-1]]).reshape(6, 225)


def test_filter_convex_takes_the_window_of_a_paraboloid():
    yy, xx = np.mgrid[-7:8, -7:8].astype(np.float64)
    w = O.filter_convex((1 - (xx / 3) ** 2 - (yy / 3) ** 2).ravel(), 4, 0, 0, True, 0.5).reshape(15, 15)
    assert np.all(w[4:11, 4:11] == 1.0)       # interior of the 9x9 window: convex, reached
    assert np.all(w[:3] == 0) and np.all(w[:, :3] == 0)
    assert np.count_nonzero(w) <= 81


def test_filter_convex_stops_at_a_ridge():
    yy, xx = np.mgrid[-7:8, -7:8].astype(np.float64)
    d = -(xx ** 2) + 0.0 * yy  # convex only across x: no cell is bi-convex
    w = O.filter_convex(d.ravel(), 4, 0, 0, True, 0.5).reshape(15, 15)
    assert np.count_nonzero(w) == 9 and np.all(w[6:9, 6:9] == 0.5)  # the 3x3 added around the centre


def test_lma_recovers_model_centre():
    for x0 in (-2.3, 0.0, 0.37, 1.8):
        ok, out, ns = O.corr_lma(_model_surfaces(x0), KINDS, x0 + 0.2, O.default_lma_params())
        assert ok and ns > 20
        assert abs(out[0] - (-x0)) < 2e-3, (x0, out)
        assert abs(out[2] - 2.0) < 2e-2          # half-width WM
        assert 0.5 < out[1] < 0.6                # strength: weighted mean of the group amplitudes


def test_lma_without_diagonal_pairs_uses_one_group():
    p = O.default_lma_params(pair_mask=0x0f)
    ok, out, ns = O.corr_lma(_model_surfaces(0.8), KINDS, 1.0, p)
    assert ok and abs(out[0] + 0.8) < 2e-3 and abs(out[1] - 0.6) < 1e-2


def test_foreground_correct_picks_the_nearest_strong_orientation():
    f = O.default_fo_params()
    # horizontal and vertical strong and narrow, 0.6 px apart: the larger disparity wins (fo_far = 0)
    dirs = np.array([[1.0, 0.8, 1.0, 0.1], [1.6, 0.7, 1.0, 0.1], [1.2, 0.5, 1.0, 0.1], [1.3, 0.5, 1.0, 0.1]])
    out = np.zeros(4)
    L = O._lma_lib()
    O.default_fo_params()
    L.or_foreground_correct.argtypes = [O.C.c_int, O.C.c_int, O._dp, O.C.POINTER(O.C.c_int), O.C.c_double,
                                        O.C.POINTER(O.FoParams), O._dp]
    L.or_foreground_correct.restype = None
    valid = (O.C.c_int * 4)(1, 1, 1, 1)
    d = np.ascontiguousarray(dirs)
    L.or_foreground_correct(0, 1, O._d(d), valid, 1.3, O.C.byref(f), O._d(out))
    assert out[0] == 1.6 and out[3] == 1.0
    # the extreme orientation too wide in disparity: no correction
    d[1, 2] = 3.5
    L.or_foreground_correct(0, 1, O._d(d), valid, 1.3, O.C.byref(f), O._d(out))
    assert out[0] == 1.3


def test_quadratic_max_recovers_an_exact_quadric():
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-4, 4, 60), rng.uniform(-4, 4, 60)
    A, B, Cc, D, E, F = -0.3, -0.2, 0.05, 0.4, -0.1, 0.7
    v = A * x * x + B * y * y + Cc * x * y + D * x + E * y + F
    ok, out = O.quadratic_max(x, y, v, rng.uniform(0.1, 1.0, 60))
    xy = np.linalg.solve([[2 * A, Cc], [Cc, 2 * B]], [-D, -E])
    assert ok and np.allclose(out[:2], xy, atol=1e-10)
    assert abs(out[2] - (A * xy[0] ** 2 + B * xy[1] ** 2 + Cc * xy[0] * xy[1] + D * xy[0] + E * xy[1] + F)) < 1e-10
    # a minimum, a collinear sample set and no positive weight have no maximum
    assert not O.quadratic_max(x, y, -v, np.ones(60))[0]
    assert not O.quadratic_max(x, 0.5 * x, v, np.ones(60))[0]
    assert not O.quadratic_max(x, y, v, np.zeros(60))[0]


def _offset_surfaces(x0, offs, amp=(0.6, 0.5), w=2.0):
    """Quad pair surfaces with each pair's peak moved by its own (along, across) offset."""
    yy, xx = np.mgrid[-7:8, -7:8].astype(np.float64)
    out = []
    for k, (px, py) in zip(KINDS, offs):
        if k < 2:
            c = amp[0] * (1 - ((xx - x0 - px) / w) ** 2 - ((yy - py) / w) ** 2)
        else:
            a, b, s = (xx + yy) / 2.0, (yy - xx) / 2.0, np.sqrt(2.0)
            c = amp[1] * (1 - ((a - x0 - px) * s / w) ** 2 - ((b - py) * s / w) ** 2)
        out.append((c.T if k == 1 else (c[::-1] if k == 3 else c)).ravel())
    return np.stack(out)


def _expected_mismatch(xc, x0, offs):
    """mismatchPairs' per-kind offsets (Correlation2d.java:1474-1490) of peaks at x0 + px, py."""
    rows = []
    for k, (px, py) in zip(KINDS, offs):
        X, Y = x0 + px, py
        rows.append({0: (xc - X, -Y), 1: (-Y, xc - X), 2: (xc - X + Y, xc - X - Y), 3: (xc - X + Y, -xc + X + Y)}[k])
    return np.array(rows)


def test_poly_mismatch_recovers_pair_offsets():
    offs = [(0.1, 0.05), (-0.1, 0.0), (0.15, -0.1), (0.0, 0.1), (0.05, 0.05), (-0.05, 0.1)]
    x0 = 1.3
    s = _offset_surfaces(x0, offs)
    ran, rec, _, m = O.lma_tile_mismatch(s, KINDS, -x0, 0.6, ly_poly=True)
    assert ran
    assert np.allclose(m[:, :2], _expected_mismatch(-rec[0], x0, offs), atol=1e-9)
    assert np.allclose(m[:, 2], [0.6] * 4 + [0.5] * 2, atol=1e-9)  # the quadric's value at its peak
    # the centre of mass sees the same offsets only roughly
    _, _, _, mc = O.lma_tile_mismatch(s, KINDS, -x0, 0.6, ly_poly=False)
    assert not np.allclose(mc, m, atol=1e-3)


def test_poly_mismatch_crazy_pair_falls_back_to_centre_of_mass():
    offs = [(0.1, 0.05), (-0.1, 0.0), (0.15, -0.1), (0.0, 0.1), (0.05, 0.05), (-0.05, 0.1)]
    s = _offset_surfaces(1.3, offs)
    _, _, _, mc = O.lma_tile_mismatch(s, KINDS, -1.3, 0.6, ly_poly=False)
    # a limit below the largest offset: one implausible pair sends every pair to the CM measure
    _, _, _, mb = O.lma_tile_mismatch(s, KINDS, -1.3, 0.6, ly_poly=True, ly_crazy_poly=0.1)
    assert np.array_equal(mb, mc)
    # without the backup the implausible pairs keep their offsets with zero strength
    _, rec, _, mn = O.lma_tile_mismatch(s, KINDS, -1.3, 0.6, ly_poly=True, ly_crazy_poly=0.1, ly_poly_backup=False)
    big = np.max(np.abs(mn[:, :2]), axis=1) > 0.1
    assert big.any() and not big.all()
    assert np.all(mn[big, 2] == 0.0) and np.all(mn[~big, 2] > 0.4)


def test_rig_lma_branch():
    """tileInterCamCorrs' LMA branch (ImageDtt.java:7497-7560) on the model surface of one horizontal
    pair: the fit recovers the disparity, the quadric (single2dPoly) an exact peak offset, the centre
    of mass (single2dCM) one close to it; use_poly off keeps the CM record, a weak tile is left alone."""
    x0 = -1.3
    corr = _model_surfaces(x0)[0]
    rec = [-x0 + 0.2, 0.9, np.nan, np.nan]
    ok, r = O.rig_lma(corr, rec, use_poly=True, use_xy_poly=True)
    assert ok and abs(r[0] - (-x0)) < 1e-6 and abs(r[2] - (-x0)) < 1e-9 and abs(r[3]) < 1e-9
    ok, r = O.rig_lma(corr, rec, use_poly=False, use_xy_poly=False)
    assert ok and r[0] == rec[0] and r[1] == rec[1] and abs(r[2] - (-x0)) < 0.3 and abs(r[3]) < 1e-12
    ok, r = O.rig_lma(corr, [1.0, 0.1, np.nan, np.nan])
    assert not ok and r[0] == 1.0 and np.isnan(r[2])
