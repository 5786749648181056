"""Shared helpers: run the same seeded scene through the oracle and the GPU path."""
import numpy as np

from tileproc import synth


def rel_l2(a, b, axis):
    num = np.sqrt(np.sum((a - b) ** 2, axis=axis))
    den = np.sqrt(np.sum(b ** 2, axis=axis))
    return num / np.maximum(den, 1e-30)


def oracle_planes(scene, color_scales=(1.0, 1.0, 0.5)):
    """[S][C][H][W] float64 planes in the oracle's colour order (R, B, G)."""
    if scene["num_colors"] == 1:
        return scene["images"][:, None].astype(np.float64)
    return np.stack([synth.bayer_planes(m, scene["color_index"], color_scales) for m in scene["images"]])


def run_oracle(O, scene, target, kernels=None, kext=None, pairs=None, corr_params=None, tile_op=None,
               ports_in=None, corr=True, threads=None):
    W, H = scene["width"], scene["height"]
    T = (W // 8) * (H // 8)
    if tile_op is None:
        tile_op = np.ones(T, np.int32)
    kern = kx = None
    if kernels is not None:
        # oracle layout [S][C][kv][kh][4][64] from the product layout [S][kv][kh][C][4][64]
        kern = np.ascontiguousarray(np.moveaxis(kernels.astype(np.float64), 3, 1))
        kx = np.ascontiguousarray(np.moveaxis(kext.astype(np.float64), 3, 1))
    cp = corr_params if corr_params is not None else O.default_corr_params()
    ref = O.run(W, H, oracle_planes(scene), tile_op, np.broadcast_to(np.asarray(target, np.float64), (T,)),
                geometry=scene["geometry"], ports_in=ports_in, kernels=kern, kernel_ext=kx,
                pairs=pairs, corr_params=cp, corr=corr, num_threads=threads,
                want=("ports", "clt", "corr", "disp", "int_tl", "residual") + (("diag",) if corr else ()))
    ref["cp"] = cp
    ref["tile_op"] = np.asarray(tile_op)
    return ref


# The integer maxima (getMaxXYInt on the combined strip's row 0, getMaxXSOrtho on its profile) are
# discontinuous: where the oracle's two largest values differ by less than NEAR_TIE (relative), FP32
# rounding may pick the other one.  Such a tile passes only if the GPU's value equals the oracle's
# own FP64 value evaluated at the maximum the GPU picked.
NEAR_TIE = 1e-4
DISP_TOL = 0.005


def _first_max(v):
    """index of the first maximum over the non-NaN entries (14 when all are NaN), as getMaxXYInt"""
    imx = 0
    for i in range(1, len(v)):
        if np.isnan(v[imx]) or v[i] > v[imx]:
            imx = i
    return imx


def check_disparity_strict(O, d, ref, tiles=None, check_ortho=True):
    """Every tile the oracle processed: the centroid disparity (and with check_ortho the hor / vert
    disparities) within DISP_TOL px of the oracle, with no quantile; an integer maximum that differs
    from the oracle's only where the oracle's values at the two maxima are a near tie, and then the
    GPU's disparity equal (to DISP_TOL) to the oracle's evaluated at the GPU's maximum.  Returns
    a summary dict (tiles checked, ties used, max errors)."""
    r, dg, cp = ref["disp"], ref["diag"], ref["cp"]
    hw = int(cp.corr_strip_hight)
    if tiles is None:
        tiles = np.nonzero(ref["tile_op"] != 0)[0]
    out = {"tiles": len(tiles), "cm_ties": 0, "ortho_ties": 0, "cm_err": 0.0, "ortho_err": 0.0}
    bad = []
    for t in tiles:
        row0 = dg[t, :15]
        ixr, ixg = r[t, O.DISP_IXY], d[t, O.DISP_IXY]
        cmr, cmg = r[t, O.DISP_CM], d[t, O.DISP_CM]
        if np.isnan(ixr) and np.isnan(ixg):
            if not np.isnan(cmg):
                bad.append((t, "CM without an integer maximum"))
            continue
        if np.isnan(ixr) != np.isnan(ixg):
            # one side below min_corr: only where the oracle's maximum is at the threshold
            vmax = row0[_first_max(row0)]
            if not abs(vmax - cp.min_corr) <= NEAR_TIE * cp.min_corr:
                bad.append((t, "integer maximum found on one side only (max %.6g, min_corr %g)" % (vmax, cp.min_corr)))
            continue
        ir, ig = int(ixr) + 7, int(ixg) + 7
        want = cmr
        if ir != ig:
            top = row0[ir]
            if not (top - row0[ig] <= NEAR_TIE * abs(top)):
                bad.append((t, "integer maximum %d vs oracle %d, gap %.3g" % (ig - 7, ir - 7, (top - row0[ig]) / abs(top))))
                continue
            alt = O.cm_at(cp, dg[t, :15 * min(hw, O.DIAG_ROWS)], hw, ig - 7)
            want = np.nan if alt is None else -alt[0]
            out["cm_ties"] += 1
        if np.isnan(want) != np.isnan(cmg):
            bad.append((t, "centroid NaN on one side (GPU %g, oracle %g)" % (cmg, want)))
            continue
        if not np.isnan(want):
            e = abs(cmg - want)
            out["cm_err"] = max(out["cm_err"], e)
            if e > DISP_TOL:
                bad.append((t, "centroid %.5f vs oracle %.5f" % (cmg, want)))
        # strength = the combined strip at the integer maximum
        if abs(d[t, O.DISP_STRENGTH] - row0[ig]) > 1e-4 * np.nanmax(np.abs(row0)):
            bad.append((t, "strength %.6g vs oracle %.6g" % (d[t, O.DISP_STRENGTH], row0[ig])))
        if check_ortho:
            for k, ks, off in ((O.DISP_HOR, O.DISP_HOR_STRENGTH, O.DIAG_HOR), (O.DISP_VERT, O.DISP_VERT_STRENGTH,
                                                                              O.DIAG_VERT)):
                prof = dg[t, off:off + 15]
                if np.isnan(r[t, k]):  # no pairs of this orientation
                    if not np.isnan(d[t, k]):
                        bad.append((t, "ortho %d without pairs" % k))
                    continue
                if np.isnan(prof).any():
                    continue  # NaN surfaces: zero-contrast tiles are tested separately
                icr = int(np.argmax(prof))
                cands = [i for i in range(15) if prof[icr] - prof[i] <= NEAR_TIE * abs(prof[icr])]
                best = min(cands, key=lambda i: abs(d[t, k] + O.ortho_at(prof, i)[0]))
                alt = O.ortho_at(prof, best)
                e = abs(d[t, k] + alt[0])
                if best != icr:
                    out["ortho_ties"] += 1
                out["ortho_err"] = max(out["ortho_err"], e)
                if e > DISP_TOL:
                    bad.append((t, "ortho %d: %.5f vs oracle %.5f" % (k, d[t, k], -alt[0])))
                es = abs(d[t, ks] - alt[1])
                if es > 1e-4 * np.abs(prof).max() / 8:
                    bad.append((t, "ortho strength %d: %.6g vs oracle %.6g" % (ks, d[t, ks], alt[1])))
    assert not bad, "%d tiles fail: %s" % (len(bad), bad[:8])
    return out


def make_gpu(scene, kernels=None, kext=None):
    from tileproc import GPUTileProcessor
    S = scene["geometry"]["num_sensors"]
    C = scene["num_colors"]
    kv = kh = 0
    if kernels is not None:
        kv, kh = kernels.shape[1], kernels.shape[2]
    bayer = scene.get("bayer", (0, 1))
    tp = GPUTileProcessor(S, scene["width"], scene["height"], num_colors=C, kernels_hor=kh, kernels_vert=kv,
                          bayer_red_row=bayer[0], bayer_red_col=bayer[1])
    tp.setGeometry(scene["geometry"])
    tp.setBayerImages(scene["images"])
    if C == 3:
        tp.setColorScales([1.0, 1.0, 0.5])
    if kernels is not None:
        from tileproc import _lib
        tp.setConvolutionKernels(kernels, kext, layout=_lib.TP_KERNELS_CPU)
    return tp
