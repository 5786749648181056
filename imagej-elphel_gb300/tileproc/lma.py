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
"""
import copy

import numpy as np

KEYS = ("azimuth", "tilt", "roll", "zoom")


def _evaluate(tp, geometry, disparity, tile_op):
    tp.setGeometry(geometry)
    tp.setFullFrameImages(disparity, tile_op=tile_op)
    tp.process()
    d = tp.getDisparity()[:, 1].astype(np.float64)
    ok = np.isfinite(d) & (tile_op != 0)
    return d, ok, float(np.sum(np.where(ok, d * d, 0.0)))


# largest change of a tile's target disparity in one step, px: beyond about a pixel the
# linearisation no longer holds (window corners and the integer maximum switch)
MAX_DISPARITY_STEP = 1.0


def refine(tp, geometry, disparity, tile_op=None, iterations=20, lam=1e-2, free_disparity=True,
           fixed_sensor=None, callback=None):
    """Runs `iterations` LM steps; returns (geometry, disparity, history) where history
    holds the cost (sum d^2 over tiles with a peak) before each step and after the last.
    The per-tile disparity steps are clipped to +-MAX_DISPARITY_STEP (a tile whose
    disparity derivative is close to zero would otherwise take an unbounded step)."""
    T = tp.tilesY * tp.tilesX
    S = tp.num_sensors
    g = copy.deepcopy(geometry)
    D = np.asarray(disparity, dtype=np.float64).reshape(T).copy()
    op = np.ones(T, np.int32) if tile_op is None else np.asarray(tile_op, np.int32).reshape(T)
    d, ok, cost = _evaluate(tp, g, D.astype(np.float32), op)
    history = [cost]
    for it in range(iterations):
        tp.backward()
        je, jd, dv = tp.getDisparityJacobian()
        ok = np.isfinite(dv) & (op != 0)
        r = np.where(ok, dv, 0.0).astype(np.float64)
        A = np.where(ok[:, None], je.reshape(T, S * 4), 0.0).astype(np.float64)
        b = np.where(ok, jd, 0.0).astype(np.float64)
        if fixed_sensor is not None:  # gauge: keep one sensor's extrinsics
            A[:, fixed_sensor * 4:(fixed_sensor + 1) * 4] = 0.0
        JtJ = A.T @ A
        dA = np.diag(JtJ).copy()
        dA[dA == 0] = 1.0
        while True:
            if free_disparity:
                # disparity block diag(b^2 (1 + lam)), eliminated by its Schur complement
                hdd = b * b * (1.0 + lam)
                inv = np.where(hdd > 0, 1.0 / np.maximum(hdd, 1e-30), 0.0)
                M = JtJ + lam * np.diag(dA) - A.T @ (A * (b * b * inv)[:, None])
                rhs = -(A.T @ r) + A.T @ (b * b * inv * r)
                de = np.linalg.solve(M + 1e-12 * np.eye(S * 4), rhs)
                dd = np.clip(-inv * b * (r + A @ de), -MAX_DISPARITY_STEP, MAX_DISPARITY_STEP)
            else:
                de = np.linalg.solve(JtJ + lam * np.diag(dA) + 1e-12 * np.eye(S * 4), -(A.T @ r))
                dd = np.zeros(T)
            g_try = copy.deepcopy(g)
            for s in range(S):
                for k, key in enumerate(KEYS):
                    g_try[key][s] = float(g_try[key][s] + de[s * 4 + k])
            D_try = D + dd
            d_try, ok_try, c_try = _evaluate(tp, g_try, D_try.astype(np.float32), op)
            if c_try < cost or lam > 1e8:
                g, D, cost = g_try, D_try, c_try
                lam = max(lam / 3.0, 1e-7)
                break
            lam *= 4.0
        history.append(cost)
        if callback:
            callback(it, cost, lam)
    return g, D, history
