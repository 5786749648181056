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
extrinsics alone are fitted.  The pairs' 2D maxima of the coarse stage see
each pair's offset across its baseline as well, so there free disparities
cost little: measured on the 16 x 640 x 512 scene with target disparities
also off by N(0, 0.3) px, the coarse stage reaches 1e-5 rad and a median
disparity error of 0.14 px (from 0.20), while the 20 adjoint-driven
iterations after it, whose disparities absorb the residual, drift to 1e-4 ..
5e-4 rad and 0.30 px.

Far from the solution, with ports off by a pixel or more, each pair's peak lies
off its strip line, the combined strip is smeared and the combined disparity
answers the extrinsics weakly and only near the start point: from extrinsics off
by N(0, 3e-3) rad on the 16 x 640 x 512 scene the iteration alone reached the
solution from two of six seeded starts.  A coarse stage therefore runs first
(_coarse_stage, COARSE iterations): Gauss-Newton on every pair's own 2D
correlation maximum, which stays measurable over +-6 px.  Measured on that
scene from 18 seeded starts (N(0, 1e-3), N(0, 2e-3), N(0, 3e-3) rad, six each)
it reaches 3e-5 rad (azimuth, tilt) and 1e-5 (roll, zoom) from every one in 3
to 5 steps; the adjoint-driven iterations then settle at the minimum of their
own cost, the combined disparity's, about 1e-4 rad from the truth (a cost of
435-437 px^2 there against 467 at the truth).  Two things keep the
adjoint-driven iteration robust:
- A tile without a correlation peak (NaN disparity) counts a cap (px^2) in
  the cost, so a step cannot lower the cost by losing tiles; and a tile's d^2
  counts at most the cap (a truncated square), with the tiles past it left out
  of the normal equations.  Without the cap a tile whose peak is on the edge
  of existing, with a residual of a few pixels, makes every step a dead end:
  the smallest move (1e-9 rad was measured) brings its peak back and adds its
  d^2 to the cost.  The cap narrows from 9 to 4 to 2 to invalid_cost (1) over
  the iterations (ANNEAL), so that while the extrinsics are far off the tiles a
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


# caps of the first sixths of the iterations (px^2): the truncated square starts wide and narrows
# to invalid_cost, so tiles a pixel or two off still pull while the extrinsics are far off, and
# none of them can hold the iteration at a dead end later
ANNEAL = (9.0, 4.0, 2.0)


def refine_stages(iterations, invalid_cost=1.0, anneal=ANNEAL):
    """[(iterations, cap)] of the stages refine runs: iterations / (2 len(anneal)) under each cap of
    anneal in turn, the rest (at least half) under invalid_cost"""
    if invalid_cost is None or not anneal:
        return [(iterations, invalid_cost)]
    q = iterations // (2 * len(anneal))
    return [(q, a) for a in anneal] + [(iterations - q * len(anneal), invalid_cost)]


# ---- coarse stage: every pair's own 2D correlation maximum ----
# Iterations of the coarse stage refine runs first, px scale of its Huber weights, and the offset
# a lost peak counts in its cost (the surface's half width)
COARSE = 6
HUBER_PX = 1.0
LOST_PX = 7.0


def pair_peaks(corr):
    """corr [n][225] (15 x 15 surfaces) -> offsets [n][2] (x right, y down, px from the centre) and
    strength [n]: the integer maximum refined by a parabola through it and its two neighbours on
    each axis; NaN offsets where the maximum is on the border or not finite.  The host statement
    of tp_get_pair_maxima, which the coarse stage reads (the parity test compares the two)."""
    c = np.asarray(corr, np.float32).reshape(-1, 225)
    filled = np.where(np.isnan(c), -np.inf, c)
    i = np.argmax(filled, axis=1)
    iy, ix = i // 15, i % 15
    n = np.arange(len(c))
    v0 = filled[n, i]
    ok = (ix >= 1) & (ix <= 13) & (iy >= 1) & (iy <= 13) & np.isfinite(v0)
    ixc, iyc = np.clip(ix, 1, 13), np.clip(iy, 1, 13)
    v = lambda y, x: filled[n, y * 15 + x]  # noqa: E731
    out = np.full((len(c), 2), np.nan)
    with np.errstate(invalid="ignore", divide="ignore"):
        for k, (m, p_) in enumerate(((v(iyc, ixc - 1), v(iyc, ixc + 1)), (v(iyc - 1, ixc), v(iyc + 1, ixc)))):
            den = m.astype(np.float64) - 2.0 * v(iyc, ixc) + p_
            frac = np.where(den < 0, 0.5 * (m - p_) / den, 0.0)
            frac = np.clip(np.nan_to_num(frac, nan=0.0, posinf=0.0, neginf=0.0), -0.5, 0.5)
            out[:, k] = np.where(ok, (ixc if k == 0 else iyc) - 7 + frac, np.nan)
    return out, np.where(ok, v0, 0.0)


def _coarse_weights(rn, st, huber):
    """Huber weights of scale huber px times (strength / median strength)^2, at most 1: the
    maximum of a pair whose windows barely overlap is weak and pulled towards the centre"""
    ref = np.median(st[st > 0]) if np.any(st > 0) else 1.0
    return np.minimum(1.0, huber / np.maximum(rn, 1e-12)) * np.minimum(1.0, np.maximum(st, 0.0) / ref) ** 2


def _huber(r, k=HUBER_PX):
    return np.where(r <= k, 0.5 * r * r, k * (r - 0.5 * k))


def _pair_measure(tp, g, D, op, pairs, huber):
    """forward at (g, D): (task tiles, port derivatives [n][S][2][5], pair offsets [n][P][2],
    Huber cost with LOST_PX per lost peak)"""
    tp.setGeometry(g)
    tp.setFullFrameImages(D.astype(np.float32), tile_op=op)
    tp.process()
    tp.backward()  # the FP64 port derivatives of this forward
    J = tp.getPortDerivatives()  # [n][S][2][5]: d(x, y) / d(azimuth, tilt, roll, zoom, disparity)
    txy = tp.getTaskTiles()
    tiles = (txy >> 16) * tp.tilesX + (txy & 0xFFFF)
    pm = tp.getPairMaxima()[tiles].astype(np.float64)  # [n][P][3]: dx, dy, strength
    r, st = pm[..., :2], pm[..., 2]
    ok = np.isfinite(r).all(axis=2)
    rn = np.where(ok, np.hypot(r[..., 0], r[..., 1]), 0.0)
    cost = float(np.sum(np.where(ok, _huber(rn, huber), 0.0)) + _huber(LOST_PX, huber) * np.count_nonzero(~ok))
    return tiles, J, r, cost, st


def _coarse_stage(tp, geometry, disparity, tile_op, iterations, free_disparity, fixed_sensor, huber=HUBER_PX):
    """Gauss-Newton on every pair's 2D correlation maximum.  A pair's surface peaks where its two
    windows align, at (port error of cam1) - (port error of cam2) px for the tile (a port error
    being the port's distance from where the scene puts it; plus the disparity error along the
    pair's baseline with free_disparity); the step moves the extrinsics (and disparities) so that
    the FP64 port derivatives (GeometryCorrection.getPortsCoordinatesAndDerivatives, recorded by
    tp_backward) cancel the measured offsets, with Huber weights of scale huber px times the
    squared relative strength of the maximum (_coarse_weights).
    This plays the part of the reference's lazy-eye measurement (per-pair peak offsets,
    clt_mismatch, ImageDtt.java:2340-2418) that its extrinsic fitting consumes
    (AlignmentCorrection).  The common azimuth, tilt, roll and zoom of all sensors move the
    offsets only through the lens distortion; left free, the steps drift along them (a 0.3 rad
    step was measured), so their sums over the sensors are held (or one sensor's parameters with
    fixed_sensor).  A step is taken at full, half or quarter length, the first that
    lowers the Huber cost (a lost peak counting LOST_PX); when none does the stage ends.  Returns
    (geometry, disparity, [cost of each point taken])."""
    T = tp.tilesY * tp.tilesX
    S = tp.num_sensors
    pairs = tp.pairs
    g = copy.deepcopy(geometry)
    D = np.asarray(disparity, dtype=np.float64).reshape(T).copy()
    op = np.ones(T, np.int32) if tile_op is None else np.asarray(tile_op, np.int32).reshape(T)
    tiles, J, r, cost, st = _pair_measure(tp, g, D, op, pairs, huber)
    costs = [cost]
    for _ in range(iterations):
        n = len(tiles)
        ok = np.isfinite(r).all(axis=2)
        rn = np.where(ok, np.hypot(r[..., 0], r[..., 1]), 0.0)
        w = np.where(ok, _coarse_weights(rn, st, huber), 0.0)
        rr = np.where(ok[..., None], r, 0.0)
        N = np.zeros((4 * S, 4 * S))
        gv = np.zeros(4 * S)
        U = np.zeros((n, 4 * S))  # disparity coupling per tile (free_disparity)
        hd = np.zeros(n)
        sd = np.zeros(n)
        ca = np.array([p[0] for p in pairs])
        cb = np.array([p[1] for p in pairs])
        Ja, Jb = J[:, ca, :, :4], J[:, cb, :, :4]  # [n][P][2][4]
        Naa = np.einsum("tp,tpik,tpil->pkl", w, Ja, Ja)
        Nbb = np.einsum("tp,tpik,tpil->pkl", w, Jb, Jb)
        Nab = np.einsum("tp,tpik,tpil->pkl", w, Ja, Jb)
        ga = np.einsum("tp,tpik,tpi->pk", w, Ja, rr)
        gb = np.einsum("tp,tpik,tpi->pk", w, Jb, rr)
        for k, (a, b) in enumerate(zip(ca, cb)):
            ia, ib = slice(4 * a, 4 * a + 4), slice(4 * b, 4 * b + 4)
            N[ia, ia] += Naa[k]
            N[ib, ib] += Nbb[k]
            N[ia, ib] -= Nab[k]
            N[ib, ia] -= Nab[k].T
            gv[ia] += ga[k]
            gv[ib] -= gb[k]
        if free_disparity:
            kd = J[:, ca][..., 4] - J[:, cb][..., 4]  # [n][P][2]
            hd = np.einsum("tp,tpi,tpi->t", w, kd, kd)
            sd = np.einsum("tp,tpi,tpi->t", w, kd, rr)
            ua = np.einsum("tp,tpik,tpi->tpk", w, Ja, kd)
            ub = np.einsum("tp,tpik,tpi->tpk", w, Jb, kd)
            for k, (a, b) in enumerate(zip(ca, cb)):
                U[:, 4 * a:4 * a + 4] += ua[:, k]
                U[:, 4 * b:4 * b + 4] -= ub[:, k]
        inv = np.where(hd > 0, 1.0 / np.maximum(hd, 1e-30), 0.0)
        if free_disparity:  # the per-tile disparities eliminated (their block is diagonal)
            N -= U.T @ (U * inv[:, None])
            gv -= U.T @ (sd * inv)
        if fixed_sensor is not None:
            fs = slice(4 * fixed_sensor, 4 * fixed_sensor + 4)
            N[fs, :] = 0.0
            N[:, fs] = 0.0
            gv[fs] = 0.0
        else:
            # the gauge: the common azimuth, tilt, roll and zoom of all sensors barely move the
            # offsets (only through lens distortion), so their sums over the sensors stay as they are
            Cg = np.tile(np.eye(4), (S, 1))
            N += 1e3 * np.abs(np.diag(N)).max() * (Cg @ Cg.T)
        dA = np.diag(N).copy()
        dA[dA == 0] = 1.0
        de = np.linalg.solve(N + 1e-6 * np.diag(dA) + 1e-12 * np.eye(4 * S), -gv)
        dd = np.zeros(T)
        if free_disparity:
            dd[tiles] = -inv * (sd + U @ de)
        for scale in (1.0, 0.5, 0.25):
            g1, D1 = _moved(g, D, de, dd, scale)
            m = _pair_measure(tp, g1, D1, op, pairs, huber)
            if m[3] < cost:
                g, D = g1, D1
                tiles, J, r, cost, st = m
                break
        else:
            break
        costs.append(cost)
    return g, D, costs


def refine(tp, geometry, disparity, tile_op=None, iterations=20, lam=LAM_RESTART, free_disparity=True,
           fixed_sensor=None, callback=None, invalid_cost=1.0, expand=True, anneal=ANNEAL, coarse=COARSE):
    """Runs `iterations` LM steps; returns (geometry, disparity, history) where history holds the
    cost before each step and after the last: the sum over tiles with a peak of min(d^2, cap),
    plus cap per tile without one, with the cap of the step's stage (refine_stages: each cap of
    anneal for 1 / (2 len(anneal)) of the iterations in turn, invalid_cost for the rest; each
    stage's first entry is its start point under its own cap).  With coarse > 0 the coarse stage
    (_coarse_stage, at most that many steps) runs first and history starts after it.  It never increases: within a
    stage no step that raises the cost is taken, and the caps only narrow.  The per-tile disparity steps are clipped to +-MAX_DISPARITY_STEP (a tile
    whose disparity derivative is close to zero would otherwise take an unbounded step).  With
    expand an accepted step is doubled while that lowers the cost, up to 8 times its length.  The
    cost is only piecewise smooth (window corners move by whole pixels, peaks appear and vanish),
    so a point can be a dead end for every damping: then the undamped step is tried at other
    lengths (STALL_SCALES), the best that lowers the cost is taken, and the damping starts again
    from LAM_RESTART.  callback(iteration, cost, damping, geometry) follows every iteration."""
    g, D, history, done = geometry, disparity, [], 0
    if coarse:
        g, D, _ = _coarse_stage(tp, g, D, tile_op, coarse, free_disparity, fixed_sensor)
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
