"""Host side of the extrinsic / disparity refinement (tileproc.lma) on fake
processors: one whose residual disparity is linear in the parameters (the damped
step with the disparity block eliminated must equal the full normal-equation
solve, and the iterations must drive the cost down), and one whose pair
correlation surfaces peak at the difference of the two sensors' port errors
(the coarse stage must find the extrinsics and disparities from them)."""
import copy

import numpy as np

from tileproc import lma

S, TX, TY = 4, 6, 5
T = TX * TY


class LinearProcessor:
    """d = r0 + A e + b * (D - D0): the interface lma.refine uses."""

    def __init__(self, rng):
        self.tilesX, self.tilesY, self.num_sensors = TX, TY, S
        self.A = rng.normal(size=(T, S * 4))
        self.b = rng.uniform(0.5, 1.5, T)
        self.r0 = 0.2 * rng.normal(size=T)  # steps inside lma.MAX_DISPARITY_STEP
        self.D0 = rng.uniform(1, 3, T)
        self.g = None
        self.D = None

    def _e(self):
        return np.array([self.g[k][s] for s in range(S) for k in lma.KEYS])

    def setGeometry(self, g):
        self.g = copy.deepcopy(g)

    def setFullFrameImages(self, D, tile_op=None):
        self.D = np.asarray(D, np.float64)

    def process(self):
        self.d = self.r0 + self.A @ self._e() + self.b * (self.D - self.D0)

    def getDisparity(self):
        out = np.full((T, 9), np.nan, np.float32)
        out[:, 1] = self.d
        return out

    def backward(self):
        return None

    def getDisparityJacobian(self):
        return (self.A.reshape(T, S, 4).astype(np.float32), self.b.astype(np.float32), self.d.astype(np.float32))


def _geom():
    return {k: [0.0] * S for k in lma.KEYS}


def test_step_equals_full_normal_equations():
    rng = np.random.default_rng(1)
    tp = LinearProcessor(rng)
    lam = 0.3
    g0, D0 = _geom(), tp.D0.copy()
    g1, D1, hist = lma.refine(tp, g0, D0, iterations=1, lam=lam, expand=False, coarse=0)
    # full system: [A b] with damping lam * diag(J^T J)
    J = np.concatenate([tp.A, np.diag(tp.b)], axis=1)
    r = tp.r0
    JtJ = J.T @ J
    step = np.linalg.solve(JtJ + lam * np.diag(np.diag(JtJ)), -J.T @ r)
    de = np.array([g1[k][s] for s in range(S) for k in lma.KEYS])
    assert np.abs(step[S * 4:]).max() < lma.MAX_DISPARITY_STEP
    assert np.allclose(de, step[:S * 4], atol=2e-5)
    assert np.allclose(D1 - D0, step[S * 4:], atol=2e-5)
    assert hist[1] < hist[0]


def test_disparity_step_is_clipped():
    """A tile whose residual barely depends on its disparity would take an unbounded step."""
    rng = np.random.default_rng(3)
    tp = LinearProcessor(rng)
    tp.b[4] = 1e-4
    tp.r0[4] = 0.5
    g1, D1, hist = lma.refine(tp, _geom(), tp.D0.copy(), iterations=1, lam=0.3, expand=False, coarse=0)
    assert np.abs(D1 - tp.D0).max() <= lma.MAX_DISPARITY_STEP
    assert abs(D1[4] - tp.D0[4]) == lma.MAX_DISPARITY_STEP


def test_iterations_reduce_cost_fixed_disparity():
    rng = np.random.default_rng(2)
    tp = LinearProcessor(rng)
    g, D, hist = lma.refine(tp, _geom(), tp.D0.copy(), iterations=8, free_disparity=False, coarse=0)
    assert all(b <= a for a, b in zip(hist, hist[1:]))
    e = np.array([g[k][s] for s in range(S) for k in lma.KEYS])
    best = np.linalg.lstsq(tp.A, -tp.r0, rcond=None)[0]
    assert np.allclose(e, best, atol=1e-3)


class WeakResponseProcessor(LinearProcessor):
    """The measured residual moves 5x less than the reported Jacobian says (a saturated peak)."""

    def process(self):
        self.d = self.r0 + 0.2 * (self.A @ self._e()) + self.b * (self.D - self.D0)


def test_step_expansion_recovers_a_short_gauss_newton_step():
    rng = np.random.default_rng(4)
    tp = WeakResponseProcessor(rng)
    _, _, h0 = lma.refine(tp, _geom(), tp.D0.copy(), iterations=3, free_disparity=False, expand=False, coarse=0)
    _, _, h1 = lma.refine(tp, _geom(), tp.D0.copy(), iterations=3, free_disparity=False, coarse=0)
    e = np.linalg.lstsq(tp.A, -tp.r0, rcond=None)[0]
    floor = float(np.sum((tp.r0 + tp.A @ e) ** 2))  # the least-squares minimum of the cost
    assert h1[-1] - floor < 0.2 * (h0[-1] - floor)


class DroppingProcessor(LinearProcessor):
    """Tiles whose residual exceeds 1 px lose their peak (NaN), as smeared correlation peaks do."""

    def getDisparity(self):
        out = super().getDisparity()
        out[np.abs(self.d) > 1.0, 1] = np.nan
        return out


def test_lost_tiles_count_in_the_cost():
    rng = np.random.default_rng(5)
    tp = DroppingProcessor(rng)
    tp.setGeometry(_geom())
    tp.setFullFrameImages(tp.D0 + 3.0)  # residual 3 b > 1: every tile without a peak
    tp.process()
    d, ok, cost = lma._evaluate(tp, _geom(), tp.D0 + 3.0, np.ones(T, np.int32), invalid_cost=2.0)
    assert not ok.any() and cost == 2.0 * T


def _blob(off, sigma=1.5):
    """a 15 x 15 surface (x right, y down) with a Gaussian maximum at off px from the centre"""
    y, x = np.mgrid[-7:8, -7:8]
    return np.exp(-((x - off[0]) ** 2 + (y - off[1]) ** 2) / (2 * sigma * sigma)).reshape(225)


def test_pair_peaks_subpixel():
    rng = np.random.default_rng(6)
    off = rng.uniform(-5, 5, (200, 2))
    got, strength = lma.pair_peaks(np.stack([_blob(o) for o in off]))
    assert np.abs(got - off).max() < 0.1
    assert (strength > 0.8).all()
    edge, _ = lma.pair_peaks(np.stack([_blob((7.0, 0.0)), np.full(225, np.nan)]))
    assert np.isnan(edge).all()


class PairPeakProcessor:
    """Port error of sensor s on tile t: J[t, s] (e - e_true, D_t - D_true_t), 2 x 5; every pair's
    surface a Gaussian at (error of cam1 - error of cam2), the sign of the correlation surfaces."""

    def __init__(self, rng, S=6, tx=5, ty=4):
        self.tilesX, self.tilesY, self.num_sensors = tx, ty, S
        self.T = tx * ty
        self.J = rng.normal(0, 0.5, (self.T, S, 2, 5))
        self.J[..., :4] *= 400.0  # px per rad
        e = rng.normal(0, 3e-3, (S, 4))
        self.e_true = (e - e.mean(axis=0)).reshape(S * 4)  # sums over the sensors 0, as the start's
        self.D_true = rng.uniform(1, 3, self.T)
        self.pairs = [(a, b, 4, 1) for a in range(S) for b in range(a + 1, S)]
        self.num_pairs = len(self.pairs)

    def setGeometry(self, g):
        self.e = np.array([g[k][s] for s in range(self.num_sensors) for k in lma.KEYS])

    def setFullFrameImages(self, D, tile_op=None):
        self.D = np.asarray(D, np.float64)

    def _err(self):
        de = (self.e - self.e_true).reshape(self.num_sensors, 4)
        return np.einsum("tsik,sk->tsi", self.J[..., :4], de) + self.J[..., 4] * (self.D - self.D_true)[:, None, None]

    def process(self):
        err = self._err()
        self.corr = np.stack([np.stack([_blob(err[t, a] - err[t, b]) for (a, b, _k, _i) in self.pairs])
                              for t in range(self.T)]).astype(np.float32)

    def backward(self):
        return None

    def getPortDerivatives(self):
        return self.J.copy()

    def getTaskTiles(self):
        t = np.arange(self.T)
        return ((t // self.tilesX) << 16) | (t % self.tilesX)

    def getPairMaxima(self):
        off, st = lma.pair_peaks(self.corr.reshape(-1, 225))
        return np.concatenate([off, st[:, None]], axis=1).reshape(self.T, self.num_pairs, 3).astype(np.float32)


def _geom_of(e, S):
    return {k: [float(e[s * 4 + i]) for s in range(S)] for i, k in enumerate(lma.KEYS)}


def test_coarse_stage_finds_extrinsics_from_pair_peaks():
    rng = np.random.default_rng(7)
    tp = PairPeakProcessor(rng)
    S = tp.num_sensors
    g0 = _geom_of(np.zeros(S * 4), S)
    tp.setGeometry(g0)
    tp.setFullFrameImages(tp.D_true)
    assert np.abs(tp._err()).max() > 3.0  # port errors of several px at the start
    g, D, costs = lma._coarse_stage(tp, g0, tp.D_true.copy(), None, 6, False, None)
    e = np.array([g[k][s] for s in range(S) for k in lma.KEYS])
    assert all(b < a for a, b in zip(costs, costs[1:]))
    assert np.abs(e - tp.e_true).max() < 1e-3 * np.abs(tp.e_true).max()
    assert np.abs(e.reshape(S, 4).sum(axis=0)).max() < 1e-7  # the sums over the sensors held


def test_coarse_stage_with_free_disparity():
    rng = np.random.default_rng(8)
    tp = PairPeakProcessor(rng)
    S = tp.num_sensors
    D0 = tp.D_true + rng.uniform(-0.5, 0.5, tp.T)
    g, D, costs = lma._coarse_stage(tp, _geom_of(np.zeros(S * 4), S), D0, None, 6, True, None)
    e = np.array([g[k][s] for s in range(S) for k in lma.KEYS])
    assert np.abs(e - tp.e_true).max() < 1e-3 * np.abs(tp.e_true).max()
    assert np.abs(D - tp.D_true).max() < 1e-3
