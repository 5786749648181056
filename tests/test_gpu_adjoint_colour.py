"""Adjoint of the forward chain for Bayer colour sensors (tp_backward on a quad colour handle),
checked by central finite differences of the FP64 oracle (needs a GB300).

Scene: 4 Bayer sensors (uint16 GR/BG) 128x96 with the quad geometry, per-sensor/colour CLT
kernels with their centre offsets and slopes, target disparities off the truth by N(0, 0.2) px.
The colour adjoint runs the pair chain back through the colour mix of the correlation (each
colour's own fat-zero normalisation and colour weight) and the forward-mode shift derivative
once per (sensor, colour) sub-tile on its sparse Bayer plane; a sensor's three colours share its
port, so their sensitivities add.

Tolerances and steps as in tests/test_gpu_adjoint.py: dd/dport to 2e-3 + 3 % of the central
difference (step 1e-3 px), the loss gradient to 3 % (1e-6 rad for the 16 extrinsics, 1e-4 px for
tile disparities), except the samples whose + and - evaluations differ in a window corner, an
integer argmax or a clipped combined-strip sample (the oracle lists them; for the extrinsics the
loss is split by tile and only those tiles are set aside).
"""
import copy

import numpy as np
import pytest

from helpers import make_gpu, run_oracle
from tileproc import synth

pytestmark = pytest.mark.gpu

W, H = 128, 96
T = (W // 8) * (H // 8)
KEYS = ("azimuth", "tilt", "roll", "zoom")


def _setup(seed=51):
    sc = synth.make_scene("quad_bayer", seed=seed, width=W, height=H)
    rng = np.random.default_rng(seed + 1)
    k, e = synth.random_clt_kernels(rng, 4, H // 16 + 2, W // 16 + 2, 3)
    D = (sc["disparity_gt"].reshape(-1) + rng.normal(0, 0.2, T)).astype(np.float32)
    return sc, k, e, D


def _oracle_run(O, sc, k, e, D, tile_op=None, ports_in=None, geometry=None):
    """(centroid disparity [T], integer corners, integer argmax [T], clipped combined-strip samples)"""
    s2 = dict(sc)
    if geometry is not None:
        s2["geometry"] = geometry
    r = run_oracle(O, s2, np.asarray(D, np.float64), kernels=k, kext=e, tile_op=tile_op, ports_in=ports_in)
    rows = r["cp"].corr_wndy_size
    combo = r["diag"][:, :15 * rows]
    return r["disp"][:, O.DISP_CM], r["int_tl"], r["disp"][:, O.DISP_IXY], (combo == 0.0) | np.isnan(combo)


def _switched(a, b, tiles=slice(None)):
    _, tl_a, ix_a, z_a = a
    _, tl_b, ix_b, z_b = b
    return (not np.array_equal(tl_a[tiles], tl_b[tiles])) or (
        not np.array_equal(ix_a[tiles], ix_b[tiles], equal_nan=True)) or (not np.array_equal(z_a[tiles], z_b[tiles]))


def _switched_tiles(a, b):
    """per tile: a window corner, the integer argmax or a clipped combined-strip sample differs"""
    tl = np.any(a[1] != b[1], axis=tuple(range(1, a[1].ndim)))
    ix = ~((a[2] == b[2]) | (np.isnan(a[2]) & np.isnan(b[2])))
    return tl | ix | np.any(a[3] != b[3], axis=1)


def _gpu(sc, k, e, D):
    tp = make_gpu(sc, k, e)
    tp.setCorrelation()
    tp.setFullFrameImages(D, tile_op=np.ones(T, np.int32))
    tp.process()
    return tp


def test_colour_port_sensitivities_match_finite_differences(oracle):
    sc, k, e, D = _setup()
    with _gpu(sc, k, e, D) as tp:
        tp.backward()
        sens = tp.getPortSensitivities()
        ports = tp.getPorts()
        txy = tp.getTaskTiles()
    d0 = _oracle_run(oracle, sc, k, e, D)[0]
    rng = np.random.default_rng(6)
    valid = np.nonzero(np.isfinite(d0))[0]
    h = 1e-3
    rows = []
    for t in rng.choice(valid, 12, replace=False):
        tile = (txy[t] >> 16) * (W // 8) + (txy[t] & 0xFFFF)
        op = np.zeros(T, np.int32)
        op[tile] = 1
        for s in range(4):
            for ax in range(2):
                pp = ports.copy()
                pp[t, s, ax] += h
                rp = _oracle_run(oracle, sc, k, e, D, op, pp)
                pp[t, s, ax] -= 2 * h
                rm = _oracle_run(oracle, sc, k, e, D, op, pp)
                fd = (rp[0][tile] - rm[0][tile]) / (2 * h)
                rows.append((sens[tile, s, ax], fd, _switched(rp, rm, tile)))
    got = np.array([r[0] for r in rows])
    fd = np.array([r[1] for r in rows])
    sw = np.array([r[2] for r in rows])
    bad = (np.abs(got - fd) > 2e-3 + 0.03 * np.abs(fd)) & ~sw
    print("colour dd/dport: max |fd| %.3g, max err %.3g, %d of %d samples straddle a switch" % (
        np.abs(fd).max(), np.abs(got - fd)[~sw].max(), sw.sum(), len(sw)))
    assert not bad.any(), list(zip(got[bad], fd[bad]))
    assert sw.mean() <= 0.2
    assert np.abs(fd[~sw]).max() > 0.05  # the sensitivities are not all trivially zero


def test_colour_loss_gradient_matches_finite_differences(oracle):
    """The 16 extrinsics and 40 tile disparities of L = sum d^2, the adjoint driven with the oracle's 2 d.
    A 1e-6 rad change of one sensor moves a corner of one of its 3 x 192 sub-tiles in most cases,
    so for the extrinsics the loss is split by tile: the central difference of the sum over the
    tiles whose + and - evaluations do not switch, against the adjoint's per-tile Jacobian rows
    (2 d dd/de) summed over the same tiles; every coordinate is compared."""
    sc, k, e, D = _setup()
    g = copy.deepcopy(sc["geometry"])
    d0 = _oracle_run(oracle, sc, k, e, D)[0]
    dl = np.where(np.isfinite(d0), 2 * d0, 0.0).astype(np.float32)
    with _gpu(sc, k, e, D) as tp:
        ge, gd = tp.backward(dl_ddisp=dl)
        je = tp.getDisparityJacobian()[0].astype(np.float64)  # [tiles][4][4]
    h, he = 1e-4, 1e-6
    rows = []
    for s in range(4):
        for kk, key in enumerate(KEYS):
            gp, gm = copy.deepcopy(g), copy.deepcopy(g)
            gp[key][s] += he
            gm[key][s] -= he
            rp = _oracle_run(oracle, sc, k, e, D, geometry=gp)
            rm = _oracle_run(oracle, sc, k, e, D, geometry=gm)
            keep = ~_switched_tiles(rp, rm) & np.isfinite(rp[0]) & np.isfinite(rm[0]) & np.isfinite(d0)
            fd = float(np.sum(rp[0][keep] ** 2 - rm[0][keep] ** 2)) / (2 * he)
            an = float(np.sum(2.0 * d0[keep] * je[keep, s, kk]))
            rows.append(("e", an, fd, False))
    rng = np.random.default_rng(7)
    for t in rng.choice(np.nonzero(np.isfinite(d0))[0], 40, replace=False):
        op = np.zeros(T, np.int32)
        op[t] = 1
        Dp, Dm = D.astype(np.float64), D.astype(np.float64)
        Dp[t] += h
        Dm[t] -= h
        rp = _oracle_run(oracle, sc, k, e, Dp, op)
        rm = _oracle_run(oracle, sc, k, e, Dm, op)
        rows.append(("d", gd[t], (rp[0][t] ** 2 - rm[0][t] ** 2) / (2 * h), _switched(rp, rm, t)))
    kind = np.array([r[0] for r in rows])
    got = np.array([r[1] for r in rows], np.float64)
    fd = np.array([r[2] for r in rows], np.float64)
    sw = np.array([r[3] for r in rows])
    held = ~sw
    rel = np.zeros(len(rows))
    for name in ("e", "d"):
        m = kind == name
        scale = np.abs(fd[m & held]).max()
        rel[m] = np.abs(got[m] - fd[m]) / np.maximum(np.abs(fd[m]), 1e-3 * scale)
    print("colour loss gradient: extrinsic rel err median %.3g max %.3g; disparity median %.3g max %.3g "
          "(%d of 40 straddle a switch)" % (
              np.median(rel[kind == "e"]), rel[kind == "e"].max(),
              np.median(rel[(kind == "d") & held]), rel[(kind == "d") & held].max(), sw[kind == "d"].sum()))
    bad = (rel > 0.03) & held
    assert not bad.any(), [(rows[i][0], got[i], fd[i]) for i in np.nonzero(bad)[0]]
    assert sw[kind == "d"].sum() <= 8


def test_colour_recompute_matches_stored_clt():
    """The adjoint with the CLT recomputed from the images (each Bayer colour as the dense fold of
    its sparse plane, where the forward takes the plane's symmetric shortcuts) against the adjoint
    on the stored CLT: the same gradients to 1e-4 of their largest, like the mono case."""
    sc, k, e, D = _setup()
    with _gpu(sc, k, e, D) as tp:
        ge0, gd0 = tp.backward()
        s0 = tp.getPortSensitivities()
        tp.setAdjointMode(recompute_clt=True)
        ge1, gd1 = tp.backward()
        s1 = tp.getPortSensitivities()
    assert np.abs(ge0).max() > 0 and np.isfinite(s0).any()
    assert np.allclose(ge1, ge0, rtol=1e-4, atol=1e-4 * np.abs(ge0).max())
    assert np.allclose(gd1, gd0, rtol=1e-4, atol=1e-4 * np.abs(gd0).max())
    m = np.isfinite(s0)
    assert np.array_equal(m, np.isfinite(s1))
    assert np.allclose(s1[m], s0[m], rtol=1e-4, atol=1e-4 * np.abs(s0[m]).max())


def test_colour_backward_is_deterministic():
    """The colour adjoint sums in a fixed order too: repeated passes agree bit for bit."""
    sc, k, e, D = _setup()
    with _gpu(sc, k, e, D) as tp:
        runs = []
        for _ in range(3):
            ge, gd = tp.backward()
            runs.append((ge, gd, tp.getPortSensitivities()) + tuple(tp.getDisparityJacobian()))
    assert np.isfinite(runs[0][2]).any()
    for r in runs[1:]:
        for a, b in zip(runs[0], r):
            assert np.array_equal(a, b, equal_nan=True)
