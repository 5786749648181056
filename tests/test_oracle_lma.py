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
