"""CPU checks of the oracle's per-tile diagnostics and of the strict disparity checker the GPU
parity tests use: the diagnostics reproduce the oracle's own disparity record, the checker
accepts the oracle's record, and it rejects a planted centroid error, a planted argmax switch
that is not a near tie, and a planted ortho error."""
import numpy as np
import pytest

from helpers import NEAR_TIE, _first_max, check_disparity_strict, run_oracle
from tileproc import synth


@pytest.fixture(scope="module")
def scene_ref(oracle):
    sc = synth.make_scene("quad_mono", seed=1, width=128, height=96)
    T = (sc["width"] // 8) * (sc["height"] // 8)
    disp = np.random.default_rng(3).uniform(0.0, 6.0, T)
    return sc, run_oracle(oracle, sc, disp)


def test_diag_reproduces_disparity_record(oracle, scene_ref):
    O = oracle
    _, ref = scene_ref
    r, dg, cp = ref["disp"], ref["diag"], ref["cp"]
    n = 0
    for t in range(len(r)):
        row0 = dg[t, :15]
        if np.isnan(r[t, O.DISP_IXY]):
            assert not row0[_first_max(row0)] >= cp.min_corr
            continue
        ix = _first_max(row0) - 7
        assert ix == r[t, O.DISP_IXY]
        cm = O.cm_at(cp, dg[t, :15 * O.DIAG_ROWS], cp.corr_strip_hight, ix)
        if cm is not None:
            assert -cm[0] == r[t, O.DISP_CM]
            n += 1
        for k, off in ((O.DISP_HOR, O.DIAG_HOR), (O.DISP_VERT, O.DIAG_VERT)):
            prof = dg[t, off:off + 15]
            hv = O.ortho_at(prof, int(np.argmax(prof)))
            assert -hv[0] == r[t, k]
    assert n > 0.9 * len(r)


def test_checker_accepts_oracle_and_rejects_planted_errors(oracle, scene_ref):
    O = oracle
    _, ref = scene_ref
    r, dg = ref["disp"], ref["diag"]
    summ = check_disparity_strict(O, r.copy(), ref)
    assert summ["cm_ties"] == 0 and summ["cm_err"] == 0.0
    good = np.nonzero(np.isfinite(r[:, O.DISP_CM]))[0]
    t = good[5]
    d = r.copy()
    d[t, O.DISP_CM] += 0.006
    with pytest.raises(AssertionError, match="centroid"):
        check_disparity_strict(O, d, ref)
    # an integer maximum moved to a clearly lower entry is not a near tie
    d = r.copy()
    row0 = dg[t, :15]
    i0 = int(r[t, O.DISP_IXY]) + 7
    lower = [i for i in range(15) if np.isfinite(row0[i]) and row0[i0] - row0[i] > 10 * NEAR_TIE * abs(row0[i0])]
    d[t, O.DISP_IXY] = lower[0] - 7
    with pytest.raises(AssertionError, match="integer maximum"):
        check_disparity_strict(O, d, ref)
    d = r.copy()
    d[t, O.DISP_HOR] -= 0.01
    with pytest.raises(AssertionError, match="ortho"):
        check_disparity_strict(O, d, ref)


def test_checker_accepts_a_near_tie_at_the_other_maximum(oracle, scene_ref):
    """A tile whose top two row-0 values are made equal: the checker takes the other maximum only
    with the oracle's centroid evaluated there."""
    O = oracle
    _, ref = scene_ref
    ref = dict(ref)
    ref["diag"] = ref["diag"].copy()
    r, dg, cp = ref["disp"], ref["diag"], ref["cp"]
    good = np.nonzero(np.isfinite(r[:, O.DISP_CM]))[0]
    t = good[7]
    i0 = int(r[t, O.DISP_IXY]) + 7
    j = i0 + 1 if i0 < 14 else i0 - 1
    dg[t, j] = dg[t, i0] * (1 - 0.5 * NEAR_TIE)
    alt = O.cm_at(cp, dg[t, :15 * O.DIAG_ROWS], cp.corr_strip_hight, j - 7)
    d = r.copy()
    d[t, O.DISP_IXY] = j - 7
    d[t, O.DISP_STRENGTH] = dg[t, j]
    d[t, O.DISP_CM] = -alt[0]
    summ = check_disparity_strict(O, d, ref)
    assert summ["cm_ties"] == 1
    d[t, O.DISP_CM] = r[t, O.DISP_CM] if abs(r[t, O.DISP_CM] + alt[0]) > 0.01 else -alt[0] + 0.01
    with pytest.raises(AssertionError, match="centroid"):
        check_disparity_strict(O, d, ref)
