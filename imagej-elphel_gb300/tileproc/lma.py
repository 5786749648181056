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
- A tile without a correlation peak (NaN disparity) counts a cap (px^2) in
  the cost, so a step cannot lower the cost by losing tiles; and a tile's d^2
  counts at most the cap (a truncated square), with the tiles past it left out
  of the normal equations.  Without the cap a tile whose peak is on the edge
  of existing, with a residual of a few pixels, makes every step a dead end:
  the smallest move (1e-9 rad was measured) brings its peak back and adds its
  d^2 to the cost.  The cap narrows from 9 to 4 to invalid_cost (1) over the
  iterations (ANNEAL), so that while the extrinsics are far off the tiles a
  pixel or two off still pull; with the narrow cap from the start one run in
  four stopped with a hundred tiles lost.
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


# caps of the first and the second quarter of the iterations (px^2): the truncated square starts
# wide and narrows to invalid_cost, so tiles a pixel or two off still pull while the extrinsics
# are far off, and none of them can hold the iteration at a dead end later
ANNEAL = (9.0, 4.0)


def refine_stages(iterations, invalid_cost=1.0, anneal=ANNEAL):
    """[(iterations, cap)] of the stages refine runs: iterations / (2 len(anneal)) under each cap of
    anneal in turn, the rest (at least half) under invalid_cost"""
    if invalid_cost is None or not anneal:
        return [(iterations, invalid_cost)]
    q = iterations // (2 * len(anneal))
    return [(q, a) for a in anneal] + [(iterations - q * len(anneal), invalid_cost)]


def refine(tp, geometry, disparity, tile_op=None, iterations=20, lam=LAM_RESTART, free_disparity=True,
           fixed_sensor=None, callback=None, invalid_cost=1.0, expand=True, anneal=ANNEAL):
    """Runs `iterations` LM steps; returns (geometry, disparity, history) where history holds the
    cost before each step and after the last: the sum over tiles with a peak of min(d^2, cap),
    plus cap per tile without one, with the cap of the step's stage (refine_stages: anneal[0] for
    the first quarter of the iterations, anneal[1] for the second, invalid_cost for the rest;
    each stage's first entry is its start point under its own cap).  It never increases: within a
    stage no step that raises the cost is taken, and the caps only narrow.  The per-tile disparity steps are clipped to +-MAX_DISPARITY_STEP (a tile
    whose disparity derivative is close to zero would otherwise take an unbounded step).  With
    expand an accepted step is doubled while that lowers the cost, up to 8 times its length.  The
    cost is only piecewise smooth (window corners move by whole pixels, peaks appear and vanish),
    so a point can be a dead end for every damping: then the undamped step is tried at other
    lengths (STALL_SCALES), the best that lowers the cost is taken, and the damping starts again
    from LAM_RESTART.  callback(iteration, cost, damping, geometry) follows every iteration."""
    g, D, history, done = geometry, disparity, [], 0
    for its, cap in refine_stages(iterations, invalid_cost, anneal):
        if its <= 0:
            continue
        g, D, h = _refine_stage(tp, g, D, tile_op, its, lam, free_disparity, fixed_sensor, callback, cap, expand,
                                done)
        history += h
        done += its
    if not history:
        history = [_evaluate(tp, copy.deepcopy(geometry), np.asarray(disparity, np.float32),
                             np.ones(tp.tilesY * tp.tilesX, np.int32) if tile_op is None else tile_op,
                             invalid_cost)[2]]
    return g, D, history


def _refine_stage(tp, geometry, disparity, tile_op, iterations, lam, free_disparity, fixed_sensor, callback,
                  invalid_cost, expand, it0):
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
            callback(it0 + it, cost, lam, g)
    return g, D, history
