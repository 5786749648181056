"""Levenberg-Marquardt refinement of per-sensor extrinsics (azimuth, tilt,
roll, zoom) and per-tile target disparities on the analytic Jacobian of the
measured residual disparity (tp_backward).

The residual of tile t is its centroid disparity d_t (the measured correction
to the tile's target disparity, ImageDtt.java:2244); the cost is sum d_t^2
over tiles with a correlation peak.  Each iteration runs the forward and the
adjoint on the device, reads back the Jacobian rows (dd/d extrinsics of every
sensor, dd/d target disparity) and solves the damped normal equations on the
host with the per-tile disparity block eliminated (it is diagonal).  This is
the role of the reference's extrinsic fitting (AlignmentCorrection, which
solves for the CorrVector with finite-difference-free analytic port
derivatives, GeometryCorrection.java:2159-2314); here the correlation chain
itself is differentiated as well.

Note on observability: with only the combined disparity per tile, a change
of the per-tile target disparities can absorb any residual, so the
extrinsics move only as far as the damping of the disparity block lets them;
with free_disparity=False the target disparities stay fixed and the
extrinsics alone are fitted.

Two things make the iteration robust far from the solution, where ports are
off by a pixel or more:
- A tile without a correlation peak (NaN disparity) counts invalid_cost px^2
  in the cost, so a step cannot lower the cost by losing tiles; and a tile's
  d^2 counts at most invalid_cost (a truncated square), with the tiles past it
  left out of the normal equations.  Without the cap a tile whose peak is on
  the edge of existing, with a residual of a few pixels, makes every step a
  dead end: the smallest move (1e-9 rad was measured) brings its peak back and
  adds its d^2 to the cost.
- There the measured disparity responds more weakly than its local
  derivative says (the smeared peak of the combined strip saturates), and the
  Gauss-Newton step falls short. An accepted step is therefore doubled while
  the cost keeps falling, up to 8 times its length (expand).
"""
import copy

import numpy as np

KEYS = ("azimuth", "tilt", "roll", "zoom")


def _evaluate(tp, geometry, disparity, tile_op, invalid_cost=None):
    """(d, ok, cost): cost = sum over the tiles with a peak of d^2, capped at invalid_cost, plus
    invalid_cost per tile without a peak (invalid_cost None: plain sum of d^2 over the tiles with one)"""
    tp.setGeometry(geometry)
    tp.setFullFrameImages(disparity, tile_op=tile_op)
    tp.process()
    d = tp.getDisparity()[:, 1].astype(np.float64)
    ok = np.isfinite(d) & (tile_op != 0)
    if invalid_cost is None:
        return d, ok, float(np.sum(np.where(ok, d * d, 0.0)))
    lost = int(np.count_nonzero((tile_op != 0) & ~ok))
    return d, ok, float(np.sum(np.where(ok, np.minimum(d * d, invalid_cost), 0.0))) + invalid_cost * lost


# largest change of a tile's target disparity in one step, px: beyond about a pixel the
# linearisation no longer holds (window corners and the integer maximum switch)
MAX_DISPARITY_STEP = 1.0


def _moved(g, D, de, dd, scale):
    g_try = copy.deepcopy(g)
    S = len(g[KEYS[0]])
    for s in range(S):
        for k, key in enumerate(KEYS):
            g_try[key][s] = float(g_try[key][s] + scale * de[s * 4 + k])
    return g_try, D + np.clip(scale * dd, -MAX_DISPARITY_STEP, MAX_DISPARITY_STEP)


# damping range of one iteration; past LAM_MAX no damping found a lower cost
LAM_MIN, LAM_MAX, LAM_RESTART = 1e-7, 1e6, 1e-2
# lengths tried for the undamped step when no damping lowers the cost
STALL_SCALES = (2.0, 4.0, 8.0, 0.5, 0.25)


def refine(tp, geometry, disparity, tile_op=None, iterations=20, lam=LAM_RESTART, free_disparity=True,
           fixed_sensor=None, callback=None, invalid_cost=1.0, expand=True):
    """Runs `iterations` LM steps; returns (geometry, disparity, history) where history
    holds the cost (sum over tiles with a peak of min(d^2, invalid_cost), plus invalid_cost per
    tile without one) before each step and after the last; it never increases.  The per-tile disparity steps are
    clipped to +-MAX_DISPARITY_STEP (a tile whose disparity derivative is close to zero would
    otherwise take an unbounded step).  With expand an accepted step is doubled while that lowers
    the cost, up to 8 times its length.  The cost is only piecewise smooth (window corners move
    by whole pixels, peaks appear and vanish), so a point can be a dead end for every damping:
    then the undamped step is tried at other lengths (STALL_SCALES), the best that lowers the cost
    is taken, and the damping starts again from LAM_RESTART."""
    T = tp.tilesY * tp.tilesX
    S = tp.num_sensors
    g = copy.deepcopy(geometry)
    D = np.asarray(disparity, dtype=np.float64).reshape(T).copy()
    op = np.ones(T, np.int32) if tile_op is None else np.asarray(tile_op, np.int32).reshape(T)
    d, ok, cost = _evaluate(tp, g, D.astype(np.float32), op, invalid_cost)
    history = [cost]
    for it in range(iterations):
        tp.backward()
        je, jd, dv = tp.getDisparityJacobian()
        ok = np.isfinite(dv) & (op != 0)
        if invalid_cost is not None:  # past the cap the truncated square is flat
            ok &= np.where(ok, dv, 0.0) ** 2 < invalid_cost
        r = np.where(ok, dv, 0.0).astype(np.float64)
        A = np.where(ok[:, None], je.reshape(T, S * 4), 0.0).astype(np.float64)
        b = np.where(ok, jd, 0.0).astype(np.float64)
        if fixed_sensor is not None:  # gauge: keep one sensor's extrinsics
            A[:, fixed_sensor * 4:(fixed_sensor + 1) * 4] = 0.0
        JtJ = A.T @ A
        dA = np.diag(JtJ).copy()
        dA[dA == 0] = 1.0

        def solve(lm):
            if free_disparity:
                # disparity block diag(b^2 (1 + lm)), eliminated by its Schur complement
                hdd = b * b * (1.0 + lm)
                inv = np.where(hdd > 0, 1.0 / np.maximum(hdd, 1e-30), 0.0)
                M = JtJ + lm * np.diag(dA) - A.T @ (A * (b * b * inv)[:, None])
                rhs = -(A.T @ r) + A.T @ (b * b * inv * r)
                de = np.linalg.solve(M + 1e-12 * np.eye(S * 4), rhs)
                return de, -inv * b * (r + A @ de)
            de = np.linalg.solve(JtJ + lm * np.diag(dA) + 1e-12 * np.eye(S * 4), -(A.T @ r))
            return de, np.zeros(T)

        def cost_at(scale, de, dd):
            g_x, D_x = _moved(g, D, de, dd, scale)
            return _evaluate(tp, g_x, D_x.astype(np.float32), op, invalid_cost)[2], g_x, D_x

        best = None  # (cost, geometry, disparity) of the step taken
        while lam <= LAM_MAX:
            de, dd = solve(lam)
            c1, g1, D1 = cost_at(1.0, de, dd)
            if c1 < cost:
                best = (c1, g1, D1)
                scale = 1.0
                while expand and scale < 8.0:
                    scale *= 2.0
                    cx = cost_at(scale, de, dd)
                    if not cx[0] < best[0]:
                        break
                    best = cx
                lam = max(lam / 3.0, LAM_MIN)
                break
            lam *= 4.0
        if best is None:  # a dead end for every damping
            de, dd = solve(LAM_RESTART)
            for scale in STALL_SCALES:
                cx = cost_at(scale, de, dd)
                if cx[0] < cost and (best is None or cx[0] < best[0]):
                    best = cx
            lam = LAM_RESTART
        if best is not None:
            cost, g, D = best
        # the next backward differentiates the accepted point: the last forward was a trial
        _evaluate(tp, g, D.astype(np.float32), op, invalid_cost)
        history.append(cost)
        if callback:
            callback(it, cost, lam)
    return g, D, history
