"""Finite-difference check of the adjoint's loss gradient on the full 16-sensor LWIR scene
(16 x 640x512, 5120 tiles, all 120 pairs), run once by hand on a GB300; the CPU oracle gives
the central differences.

    python tests/fd_check_c5.py [--extrinsic 40] [--tiles 160] [--out result.json]

The same construction as tests/test_gpu_adjoint.py::test_loss_gradient_matches_finite_differences
at the test's 160x128 crop, here at the full scene size: extrinsics perturbed by N(0, 1e-3) rad,
target disparities off the truth by N(0, 0.2) px, L = sum d^2 over the tiles' centroid
disparities, the adjoint driven with dL/dd = 2 d of the oracle.  40 extrinsic coordinates
(step 1e-6 rad) and 160 tile disparities (step 1e-4 px).

At this size a 1e-6 rad change of one sensor moves a window corner, an integer argmax or a
clipped combined-strip sample in some of the 5120 tiles almost every time, so the whole loss
jumps.  The check therefore splits the loss by tile: for an extrinsic coordinate it compares
the central difference of the sum over the tiles whose + and - evaluations have the same
corners, argmax and clipped samples (and a finite disparity) with the adjoint's per-tile
Jacobian rows (tp_get_disparity_jacobian) summed over the same tiles, and reports how many
tiles were set aside.  A tile-disparity coordinate moves only its own tile and is set aside
when that tile switches.  Every compared coordinate is held to 3 % of its finite difference
(with 1e-3 of the largest as the floor).  The sums over ~5000 tiles cancel (the output gives
|sum| / sum |terms|), so for the extrinsics the per-tile Jacobian entries dd_t/de are also
compared with each tile's own central difference (floor: 1 % of the coordinate's largest).
Prints one JSON line with the counts and the error statistics.
"""
import argparse
import copy
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path[:0] = [REPO, os.path.join(REPO, "imagej-elphel_gb300")]

W, H = 640, 512
T = (W // 8) * (H // 8)
KEYS = ("azimuth", "tilt", "roll", "zoom")


def oracle_run(O, sc, g, pairs, D, tile_op=None):
    op = np.ones(T, np.int32) if tile_op is None else tile_op
    P = O.make_pairs([(a, b, bx, by, kind) for (a, b, kind, _, bx, by) in pairs])
    r = O.run(W, H, sc["images"][:, None].astype(np.float64), op, np.asarray(D, np.float64), geometry=g, pairs=P,
              want=("disp", "int_tl", "diag"))
    rows = O.default_corr_params().corr_wndy_size
    combo = r["diag"][:, :15 * rows]
    return r["disp"][:, O.DISP_CM], r["int_tl"], r["disp"][:, O.DISP_IXY], (combo == 0.0) | np.isnan(combo)


def switched_tiles(a, b):
    """per tile: a window corner, the integer argmax or a clipped combined-strip sample differs"""
    tl = np.any(a[1] != b[1], axis=tuple(range(1, a[1].ndim)))
    ix = ~((a[2] == b[2]) | (np.isnan(a[2]) & np.isnan(b[2])))
    z = np.any(a[3] != b[3], axis=1)
    return tl | ix | z


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=31)
    ap.add_argument("--extrinsic", type=int, default=40)
    ap.add_argument("--tiles", type=int, default=160)
    ap.add_argument("--out", default="")
    a = ap.parse_args()
    from oracle import oracle as O
    from tileproc import GPUTileProcessor, synth

    sc = synth.make_scene("circle_lwir", seed=a.seed, width=W, height=H)
    rng = np.random.default_rng(a.seed + 1)
    g = copy.deepcopy(sc["geometry"])
    for k in KEYS:
        g[k] = (np.asarray(g[k]) + rng.normal(0, 1e-3, 16)).tolist()
    pairs = synth.circle_pairs(g)
    D = (sc["disparity_gt"].reshape(-1) + rng.normal(0, 0.2, T)).astype(np.float32)

    r0 = oracle_run(O, sc, g, pairs, D)
    d0 = r0[0]
    dl = np.where(np.isfinite(d0), 2 * d0, 0.0).astype(np.float32)
    tp = GPUTileProcessor(16, W, H)
    try:
        tp.setGeometry(g)
        tp.setBayerImages(sc["images"])
        tp.setCorrelation(pairs=pairs)
        tp.setFullFrameImages(D, tile_op=np.ones(T, np.int32))
        tp.process()
        ge, gd = tp.backward(dl_ddisp=dl)
        je = tp.getDisparityJacobian()[0].astype(np.float64)  # dd_t / d extrinsic [T][16][4]
    finally:
        tp.close()

    h, he = 1e-4, 1e-6
    rows = []
    set_aside = []
    cancel = []
    tile_err = []
    for flat in rng.choice(64, a.extrinsic, replace=False):
        s, k = flat // 4, flat % 4
        gp, gm = copy.deepcopy(g), copy.deepcopy(g)
        gp[KEYS[k]][s] += he
        gm[KEYS[k]][s] -= he
        rp, rm = oracle_run(O, sc, gp, pairs, D), oracle_run(O, sc, gm, pairs, D)
        keep = ~switched_tiles(rp, rm) & np.isfinite(rp[0]) & np.isfinite(rm[0]) & np.isfinite(d0)
        set_aside.append(int((~keep & np.isfinite(d0)).sum()))
        fd = float(np.sum(rp[0][keep] ** 2 - rm[0][keep] ** 2)) / (2 * he)
        terms = 2.0 * d0[keep] * je[keep, s, k]
        an = float(np.sum(terms))
        rows.append(("e", an, fd, False))
        cancel.append(abs(an) / max(float(np.sum(np.abs(terms))), 1e-300))
        # the Jacobian entry of every kept tile against its own central difference
        fdt = (rp[0][keep] - rm[0][keep]) / (2 * he)
        jt = je[keep, s, k]
        floor = 1e-2 * np.abs(fdt).max()
        tile_err.append(np.abs(jt - fdt) / np.maximum(np.abs(fdt), floor))
    valid = np.nonzero(np.isfinite(d0))[0]
    for t in rng.choice(valid, a.tiles, replace=False):
        op = np.zeros(T, np.int32)
        op[t] = 1
        Dp, Dm = D.astype(np.float64), D.astype(np.float64)
        Dp[t] += h
        Dm[t] -= h
        rp = oracle_run(O, sc, g, pairs, Dp, op)
        rm = oracle_run(O, sc, g, pairs, Dm, op)
        rows.append(("d", float(gd[t]), (rp[0][t] ** 2 - rm[0][t] ** 2) / (2 * h), bool(switched_tiles(rp, rm)[t])))
    got = np.array([r[1] for r in rows])
    fd = np.array([r[2] for r in rows])
    sw = np.array([r[3] for r in rows])
    kind = np.array([r[0] for r in rows])
    out = {"scene": "circle_lwir 16x%dx%d, %d tiles, 120 pairs" % (W, H, T), "seed": a.seed,
           "valid_tiles": int(np.isfinite(d0).sum()),
           "extrinsic_tiles_set_aside": {"median": float(np.median(set_aside)), "max": int(max(set_aside))}}
    ok_all = True
    for name, m in (("extrinsic", kind == "e"), ("disparity", kind == "d")):
        held = m & ~sw
        scale = np.abs(fd[held]).max()
        rel = np.abs(got - fd) / np.maximum(np.abs(fd), 1e-3 * scale)
        bad = held & (rel > 0.03)
        ok_all &= not bad.any()
        out[name] = {"coords": int(m.sum()), "straddle_switch": int((m & sw).sum()), "held": int(held.sum()),
                     "rel_err_median": float(np.median(rel[held])), "rel_err_max": float(rel[held].max()),
                     "outside_3pct": int(bad.sum())}
    te = np.concatenate(tile_err)
    out["extrinsic"]["sum_over_terms_median"] = float(np.median(cancel))  # |sum| / sum |terms|: cancellation
    out["extrinsic_per_tile"] = {"entries": int(te.size), "rel_err_median": float(np.median(te)),
                                 "rel_err_p99": float(np.percentile(te, 99)), "rel_err_max": float(te.max()),
                                 "within_3pct": float(np.mean(te <= 0.03))}
    out["pass"] = bool(ok_all)
    line = json.dumps(out)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")
    return 0 if ok_all else 1


if __name__ == "__main__":
    sys.exit(main())
