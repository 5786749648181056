"""ctypes wrapper around the FP64 oracle library (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check and time the GB300 path.  Nothing in the product imports this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

OR_MAX_SENSORS = 16
OR_MAX_PAIRS = 120
DISP_N = 9
DISP_INT, DISP_CM, DISP_STRENGTH, DISP_HOR, DISP_HOR_STRENGTH, DISP_VERT, DISP_VERT_STRENGTH, DISP_CM_S0, DISP_IXY = range(9)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Geometry(C.Structure):
    _fields_ = [("num_sensors", C.c_int), ("pixel_width", C.c_int), ("pixel_height", C.c_int),
                ("focal_length", C.c_double), ("pixel_size", C.c_double), ("distortion_radius", C.c_double),
                ("distortion", C.c_double * 7),
                ("rXY", (C.c_double * 2) * OR_MAX_SENSORS), ("pXY0", (C.c_double * 2) * OR_MAX_SENSORS),
                ("azimuth", C.c_double * OR_MAX_SENSORS), ("tilt", C.c_double * OR_MAX_SENSORS),
                ("roll", C.c_double * OR_MAX_SENSORS), ("zoom", C.c_double * OR_MAX_SENSORS)]


class Pairs(C.Structure):
    _fields_ = [("num_pairs", C.c_int), ("cam1", C.c_int * OR_MAX_PAIRS), ("cam2", C.c_int * OR_MAX_PAIRS),
                ("bx", C.c_double * OR_MAX_PAIRS), ("by", C.c_double * OR_MAX_PAIRS),
                ("kind", C.c_int * OR_MAX_PAIRS), ("combo_mask_lo", C.c_int), ("combo_mask_hi", C.c_int)]


class CorrParams(C.Structure):
    _fields_ = [("fat_zero", C.c_double), ("corr_sigma", C.c_double), ("corr_red", C.c_double),
                ("corr_blue", C.c_double), ("corr_offset", C.c_double), ("min_corr", C.c_double),
                ("corr_strip_hight", C.c_int), ("twice_diagonal", C.c_int), ("enhortho_width", C.c_int),
                ("enhortho_scale", C.c_double), ("corr_wndy_size", C.c_int), ("corr_wndy_hwidth", C.c_double),
                ("corr_wndy_blur", C.c_double), ("corr_wndx_size", C.c_int), ("corr_wndx_hwidth", C.c_double),
                ("corr_wndx_blur", C.c_double)]


class RunCfg(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("num_sensors", C.c_int), ("num_colors", C.c_int),
                ("kernels_hor", C.c_int), ("kernels_vert", C.c_int), ("kernel_step", C.c_int),
                ("num_threads", C.c_int), ("use_ports_in", C.c_int), ("corr", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.or_dct_iv8.argtypes = [_dp, _dp]
        L.or_dst_iv8.argtypes = [_dp, _dp]
        L.or_dct_ii8.argtypes = [_dp, _dp]
        L.or_dst_ii8.argtypes = [_dp, _dp]
        L.or_dtt24.argtypes = [_dp, _dp, C.c_int]
        L.or_dctiv_direct.argtypes = [_dp, _dp]
        for f in (L.or_dttt_iv, L.or_dttt_iie, L.or_dttt_iiie):
            f.argtypes = [_dp, _dp, C.c_int]
        L.or_hwindow.argtypes = [_dp]
        L.or_shifted_fold.argtypes = [C.c_double, C.c_double, _dp]
        L.or_fold_index.argtypes = [_ip]
        L.or_fold_tile.argtypes = [_dp, C.c_int, _dp, _dp]
        L.or_unfold_tile.argtypes = [_dp, C.c_int, _dp]
        L.or_corr_unfold_tile.argtypes = [_dp, _dp]
        L.or_win2d.argtypes = [_dp]
        L.or_extract_correct_tile.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int,
                                              C.c_double, C.c_double, _dp, _dp, _ip, _ip]
        L.or_convolve_tile.argtypes = [_dp, _dp]
        L.or_fract_shift.argtypes = [_dp, C.c_double, C.c_double]
        L.or_corr_lpf.argtypes = [C.c_double, _dp]
        L.or_clt_lpf.argtypes = [C.c_double, _dp]
        L.or_rot_matrices.argtypes = [C.POINTER(Geometry), _dp]
        L.or_rot_deriv_matrices.argtypes = [C.POINTER(Geometry), _dp]
        L.or_reverse_distortion_table.argtypes = [C.POINTER(Geometry), _dp, C.c_int]
        L.or_reverse_distortion_table.restype = C.c_int
        L.or_r_by_rdist.argtypes = [_dp, C.c_int, C.c_double]
        L.or_r_by_rdist.restype = C.c_double
        L.or_ports.argtypes = [C.POINTER(Geometry), _dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                               C.c_double, _dp, _dp]
        L.or_rig_aux_ports.argtypes = [C.POINTER(Geometry), C.POINTER(Geometry), C.POINTER(RigOffset), C.c_double,
                                       C.c_double, C.c_double, _dp]
        L.or_rig_rxy.argtypes = [C.POINTER(Geometry), C.POINTER(RigOffset), _dp]
        L.or_rig_matrix.argtypes = [C.POINTER(RigOffset), _dp]
        L.or_default_corr_params.argtypes = [C.POINTER(CorrParams)]
        L.or_quad_pairs.argtypes = [C.POINTER(Pairs)]
        L.or_correlate_pair.argtypes = [_dp, _dp, C.c_int, _dp, _dp, C.c_double, _dp]
        L.or_strip.argtypes = [_dp, C.c_double, C.c_double, C.c_int, C.c_int, _dp]
        L.or_combine_strips.argtypes = [_dp, _ip, C.c_int, _ip, C.c_int, C.c_double, C.c_int, _dp]
        L.or_max_xy_int_axis.argtypes = [_dp, C.c_int, C.c_double, _ip]
        L.or_max_xy_int_axis.restype = C.c_int
        L.or_half_flat_top_window.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, _dp]
        L.or_max_x_cm.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp]
        L.or_max_x_cm.restype = C.c_int
        L.or_ortho_notch.argtypes = [C.c_double, C.c_double, _dp]
        L.or_max_xs_ortho.argtypes = [_dp, _ip, C.c_int, C.c_double, C.c_int, _dp, _dp]
        L.or_max_xs_ortho.restype = C.c_int
        L.or_iclt_tile_add.argtypes = [_dp, C.c_double, C.c_int, C.c_int, _dp, C.c_int]
        L.or_calc_clt_kernel.argtypes = [_dp, C.c_int, _dp, _dp]
        L.or_fill_coord_corr.argtypes = [_dp, C.c_int, C.c_int, C.c_int]
        L.or_run.argtypes = [C.POINTER(RunCfg), C.POINTER(Geometry), _dp, C.POINTER(_dp), C.POINTER(_dp),
                             C.POINTER(_dp), _ip, _dp, C.POINTER(Pairs), C.POINTER(CorrParams),
                             _dp, _dp, _dp, _dp, _ip, _dp]
        L.or_run.restype = C.c_int
        L.or_run_diag.argtypes = L.or_run.argtypes + [_dp]
        L.or_run_diag.restype = C.c_int
        L.or_cm_at.argtypes = [C.POINTER(CorrParams), _dp, C.c_int, C.c_int, _dp]
        L.or_cm_at.restype = C.c_int
        L.or_ortho_at.argtypes = [_dp, C.c_int, _dp]
        L.or_ortho_at.restype = None
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---- DttRad2 ----
def _vec8(fn, x):
    x = _f64(x)
    y = np.zeros(8)
    fn(_d(x), _d(y))
    return y


def dct_iv8(x): return _vec8(lib().or_dct_iv8, x)
def dst_iv8(x): return _vec8(lib().or_dst_iv8, x)
def dct_ii8(x): return _vec8(lib().or_dct_ii8, x)
def dst_ii8(x): return _vec8(lib().or_dst_ii8, x)
def dctiv_direct(x): return _vec8(lib().or_dctiv_direct, x)


def _dttt(fn, x, mode):
    x = _f64(x).reshape(64)
    y = np.zeros(64)
    fn(_d(x), _d(y), int(mode))
    return y


def dttt_iv(x, mode): return _dttt(lib().or_dttt_iv, x, mode)
def dttt_iie(x, mode): return _dttt(lib().or_dttt_iie, x, mode)
def dttt_iiie(x, mode): return _dttt(lib().or_dttt_iiie, x, mode)


def dtt24_image(img, mode):
    """GPU_DTT24_DRV (dtt8x8.cuh:100-158) on a float image: every 8x8 block transformed in place
    (rows, then columns; mode 0-3 DCT-IV / DST-IV, 4-7 DCT-II / DST-II)"""
    a = _f64(img)
    h, w = a.shape
    out = np.zeros((h, w))
    fn = lib().or_dtt24
    for by in range(0, h, 8):
        for bx in range(0, w, 8):
            x = np.ascontiguousarray(a[by:by + 8, bx:bx + 8]).reshape(64)
            y = np.zeros(64)
            fn(_d(x), _d(y), int(mode))
            out[by:by + 8, bx:bx + 8] = y.reshape(8, 8)
    return out


def hwindow():
    y = np.zeros(8)
    lib().or_hwindow(_d(y))
    return y


def win2d():
    y = np.zeros(256)
    lib().or_win2d(_d(y))
    return y


def shifted_fold(sh, sv):
    y = np.zeros((4, 64, 4))
    lib().or_shifted_fold(float(sh), float(sv), _d(y))
    return y


def fold_index():
    y = np.zeros((64, 4), dtype=np.int32)
    lib().or_fold_index(_i(y))
    return y


def unfold_tile(x64, mode):
    x = _f64(x64).reshape(64)
    y = np.zeros(256)
    lib().or_unfold_tile(_d(x), int(mode), _d(y))
    return y


def corr_unfold_tile(q):
    q = _f64(q).reshape(4, 64)
    y = np.zeros(225)
    lib().or_corr_unfold_tile(_d(q), _d(y))
    return y


# ---- ImageDtt ----
def extract_correct_tile(image, cx, cy, kern=None, kext=None, kernel_step=16):
    image = _f64(image)
    h, w = image.shape
    clt = np.zeros((4, 64))
    res = np.zeros(2)
    tl = np.zeros(2, dtype=np.int32)
    kt = np.zeros(2, dtype=np.int32)
    if kern is not None:
        kern = _f64(kern)
        kext = _f64(kext)
        kv, kh = kern.shape[0], kern.shape[1]
        lib().or_extract_correct_tile(_d(image), w, h, _d(kern), _d(kext), kh, kv, kernel_step,
                                      float(cx), float(cy), _d(clt), _d(res), _i(tl), _i(kt))
    else:
        lib().or_extract_correct_tile(_d(image), w, h, None, None, 0, 0, kernel_step,
                                      float(cx), float(cy), _d(clt), _d(res), _i(tl), _i(kt))
    return clt, res, tl, kt


def fract_shift(clt, sx, sy):
    c = _f64(clt).reshape(4, 64).copy()
    lib().or_fract_shift(_d(c), float(sx), float(sy))
    return c


def convolve_tile(clt, kernel):
    c = _f64(clt).reshape(4, 64).copy()
    k = _f64(kernel).reshape(256)
    lib().or_convolve_tile(_d(c), _d(k))
    return c


def corr_lpf(sigma):
    y = np.zeros(64)
    lib().or_corr_lpf(float(sigma), _d(y))
    return y


def clt_lpf(sigma):
    y = np.zeros(64)
    lib().or_clt_lpf(float(sigma), _d(y))
    return y


def iclt_tile_add(clt, scale, tx, ty, frame):
    c = _f64(clt).reshape(4, 64)
    assert frame.dtype == np.float64 and frame.flags.c_contiguous
    lib().or_iclt_tile_add(_d(c), float(scale), int(tx), int(ty), _d(frame), frame.shape[1])


# ---- geometry ----
def make_geometry(g):
    """g: dict with keys num_sensors, width, height, focal_length, pixel_size,
    distortion_radius, distortion[7], rXY[S][2], pXY0[S][2], azimuth/tilt/roll/zoom[S]."""
    G = Geometry()
    S = int(g["num_sensors"])
    G.num_sensors = S
    G.pixel_width = int(g["width"])
    G.pixel_height = int(g["height"])
    G.focal_length = float(g["focal_length"])
    G.pixel_size = float(g["pixel_size"])
    G.distortion_radius = float(g["distortion_radius"])
    for i in range(7):
        G.distortion[i] = float(g["distortion"][i])
    for s in range(S):
        for k in range(2):
            G.rXY[s][k] = float(g["rXY"][s][k])
            G.pXY0[s][k] = float(g["pXY0"][s][k])
        G.azimuth[s] = float(g["azimuth"][s])
        G.tilt[s] = float(g["tilt"][s])
        G.roll[s] = float(g["roll"][s])
        G.zoom[s] = float(g["zoom"][s])
    return G


def rot_matrices(g):
    G = make_geometry(g)
    r = np.zeros((OR_MAX_SENSORS, 3, 3))
    lib().or_rot_matrices(C.byref(G), _d(r))
    return r[:G.num_sensors]


def rot_deriv_matrices(g):
    G = make_geometry(g)
    r = np.zeros((OR_MAX_SENSORS, 4, 3, 3))
    lib().or_rot_deriv_matrices(C.byref(G), _d(r))
    return r[:G.num_sensors]


def reverse_distortion_table(g):
    G = make_geometry(g)
    t = np.zeros(2100)
    n = lib().or_reverse_distortion_table(C.byref(G), _d(t), 2100)
    return t[:n]


def ports(g, px, py, disparity, deriv=False):
    G = make_geometry(g)
    S = G.num_sensors
    rots = np.zeros((OR_MAX_SENSORS, 3, 3))
    drots = np.zeros((OR_MAX_SENSORS, 4, 3, 3))
    lib().or_rot_matrices(C.byref(G), _d(rots))
    lib().or_rot_deriv_matrices(C.byref(G), _d(drots))
    tbl = np.zeros(2100)
    n = lib().or_reverse_distortion_table(C.byref(G), _d(tbl), 2100)
    out = np.zeros((OR_MAX_SENSORS, 2))
    dv = np.zeros((OR_MAX_SENSORS, 2, 4))
    lib().or_ports(C.byref(G), _d(rots), _d(drots), _d(tbl), n, float(px), float(py), float(disparity),
                   _d(out), _d(dv) if deriv else None)
    return (out[:S], dv[:S]) if deriv else out[:S]


class RigOffset(C.Structure):
    """GeometryCorrection.RigOffset of an auxiliary camera (GeometryCorrection.java:256-975)."""
    _fields_ = [("main_disparity_radius", C.c_double), ("aux_disparity_radius", C.c_double),
                ("baseline", C.c_double), ("aux_angle", C.c_double), ("aux_azimuth", C.c_double),
                ("aux_tilt", C.c_double), ("aux_roll", C.c_double), ("aux_zoom", C.c_double)]


def make_rig(r):
    """r: dict with the RigOffset fields above."""
    R = RigOffset()
    for name, _ in RigOffset._fields_:
        setattr(R, name, float(r[name]))
    return R


def rig_aux_ports(aux, main, rig, px, py, disparity_main):
    """ImageDtt.clt_bi_quad's auxiliary-camera ports (ImageDtt.java:8972-8996) -> [S][2]."""
    A, M, R = make_geometry(aux), make_geometry(main), make_rig(rig)
    out = np.zeros((OR_MAX_SENSORS, 2))
    lib().or_rig_aux_ports(C.byref(A), C.byref(M), C.byref(R), float(px), float(py), float(disparity_main),
                           _d(out))
    return out[:A.num_sensors]


def rig_rxy(aux, rig):
    """RigOffset.recalcRXY -> rXY_aux [S][2]."""
    A, R = make_geometry(aux), make_rig(rig)
    out = np.zeros((OR_MAX_SENSORS, 2))
    lib().or_rig_rxy(C.byref(A), C.byref(R), _d(out))
    return out[:A.num_sensors]


# ---- correlation ----
def default_corr_params(**kw):
    p = CorrParams()
    lib().or_default_corr_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def make_pairs(pairs=None):
    """pairs: None for the quad PAIRS[0..5], else list of (cam1, cam2, bx, by, kind)."""
    P = Pairs()
    if pairs is None:
        lib().or_quad_pairs(C.byref(P))
        return P
    P.num_pairs = len(pairs)
    for i, (a, b, bx, by, kind) in enumerate(pairs):
        P.cam1[i], P.cam2[i], P.bx[i], P.by[i], P.kind[i] = a, b, bx, by, kind
    P.combo_mask_lo = -1
    P.combo_mask_hi = -1
    return P


def correlate_pair(clt1, clt2, col_weights, lpf, fat_zero):
    clt1 = _f64(clt1)
    clt2 = _f64(clt2)
    nc = clt1.size // 256
    cw = _f64(col_weights) if col_weights is not None else np.ones(1)
    lp = _f64(lpf) if lpf is not None else None
    y = np.zeros(225)
    lib().or_correlate_pair(_d(clt1), _d(clt2), nc, _d(cw), _d(lp) if lp is not None else None,
                            float(fat_zero), _d(y))
    return y


def strip(corr225, bx, by, kind, hwidth=9):
    c = _f64(corr225)
    y = np.zeros(hwidth * 15)
    lib().or_strip(_d(c), float(bx), float(by), int(kind), int(hwidth), _d(y))
    return y


# ---- kernel preparation ----
def calc_clt_kernel(src64, normalize=True):
    s = _f64(src64).reshape(64 * 64)
    clt = np.zeros((4, 64))
    ext = np.zeros(8)
    lib().or_calc_clt_kernel(_d(s), int(normalize), _d(clt), _d(ext))
    return clt, ext


def fill_coord_corr(ext, kern_step=16):
    """ext: [kv][kh][8] float64, modified in place."""
    assert ext.dtype == np.float64 and ext.flags.c_contiguous
    kv, kh = ext.shape[:2]
    lib().or_fill_coord_corr(_d(ext), kh, kv, int(kern_step))
    return ext


# ---- full run ----
def run(width, height, images, tile_op, disparity, geometry=None, ports_in=None,
        kernels=None, kernel_ext=None, kernel_step=16, pairs=None, corr_params=None,
        num_threads=None, corr=True, want=("ports", "clt", "corr", "disp", "int_tl", "residual")):
    """images: float array [S][C][H][W] (sparse colour planes for Bayer).
    kernels: [S][C][kv][kh][4][64] CPU orientation or None; kernel_ext: [S][C][kv][kh][8]."""
    L = lib()
    images = _f64(images)
    S, Cn = images.shape[0], images.shape[1]
    T = (width // 8) * (height // 8)
    cfg = RunCfg()
    cfg.width, cfg.height, cfg.num_sensors, cfg.num_colors = width, height, S, Cn
    cfg.num_threads = num_threads or os.cpu_count() or 1
    cfg.corr = int(corr)
    img_ptrs = (_dp * (S * Cn))(*[_d(images[s, c]) for s in range(S) for c in range(Cn)])
    kern_ptrs = kext_ptrs = None
    if kernels is not None:
        kernels = _f64(kernels)
        kernel_ext = _f64(kernel_ext)
        cfg.kernels_vert, cfg.kernels_hor = kernels.shape[2], kernels.shape[3]
        cfg.kernel_step = kernel_step
        kern_ptrs = (_dp * S)(*[_d(kernels[s]) for s in range(S)])
        kext_ptrs = (_dp * S)(*[_d(kernel_ext[s]) for s in range(S)])
    G = make_geometry(geometry) if geometry is not None else Geometry()
    pin = None
    if ports_in is not None:
        ports_in = _f64(ports_in)
        cfg.use_ports_in = 1
        pin = ports_in
        G.num_sensors = S
    P = pairs if isinstance(pairs, Pairs) else make_pairs(pairs)
    cp = corr_params if corr_params is not None else default_corr_params()
    tile_op = np.ascontiguousarray(tile_op, dtype=np.int32).reshape(T)
    disparity = _f64(disparity).reshape(T)
    np_ = P.num_pairs
    out = {}
    out["ports"] = np.zeros((T, S, 2)) if "ports" in want else None
    out["clt"] = np.zeros((T, S, Cn, 4, 64)) if "clt" in want else None
    out["corr"] = np.zeros((T, np_, 225)) if ("corr" in want and corr) else None
    out["disp"] = np.zeros((T, DISP_N)) if ("disp" in want and corr) else None
    out["int_tl"] = np.zeros((T, S, Cn, 2), dtype=np.int32) if "int_tl" in want else None
    out["residual"] = np.zeros((T, S, Cn, 2)) if "residual" in want else None
    out["diag"] = np.full((T, DIAG_N), np.nan) if ("diag" in want and corr) else None
    nd = lambda k: _d(out[k]) if out[k] is not None else None
    rc = L.or_run_diag(C.byref(cfg), C.byref(G), _d(pin) if pin is not None else None, img_ptrs,
                       kern_ptrs, kext_ptrs, _i(tile_op), _d(disparity), C.byref(P), C.byref(cp),
                       nd("ports"), nd("clt"), nd("corr"), nd("disp"),
                       _i(out["int_tl"]) if out["int_tl"] is not None else None, nd("residual"), nd("diag"))
    if rc != 0:
        raise RuntimeError("or_run failed: %d" % rc)
    return {k: v for k, v in out.items() if v is not None}


# per-tile diagnostics of run(..., want=(..., "diag")): the combined strip rows [16][15]
# (the first min(corr_strip_hight, 16) rows filled), the horizontal and the vertical ortho profiles [15]
DIAG_ROWS = 16
DIAG_N = DIAG_ROWS * 15 + 30
DIAG_HOR, DIAG_VERT = DIAG_ROWS * 15, DIAG_ROWS * 15 + 15


def cm_at(corr_params, combo_rows, hwidth, ix):
    """getMaxXCm of a combined strip [rows][15] at the integer maximum ix: (x, s0, sigma) or None."""
    r = np.zeros(3)
    c = _f64(combo_rows).reshape(-1)
    ok = lib().or_cm_at(C.byref(corr_params), _d(c), int(hwidth), int(ix), _d(r))
    return r if ok else None


def ortho_at(c1d, icenter):
    """getMaxXSOrtho's (xcenter - 7, strength) of a 15-entry profile around the integer maximum icenter."""
    r = np.zeros(2)
    lib().or_ortho_at(_d(_f64(c1d).reshape(15)), int(icenter), _d(r))
    return r


def imclt_frames(clt, tilesX, tilesY, scale=0.25, lpf=None, present=None, num_threads=None):
    """ImageDtt.iclt_2d over all tiles of clt [tiles][S][C][4][64] -> [S][C][H+8][W+8]."""
    L = lib()
    if not getattr(L, "_imclt_set", False):
        L.or_imclt_frames.argtypes = [_dp, _ip, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int,
                                      C.c_int]
        L.or_imclt_frames.restype = C.c_int
        L._imclt_set = True
    clt = _f64(clt)
    S, Cn = clt.shape[1], clt.shape[2]
    out = np.zeros((S, Cn, tilesY * 8 + 8, tilesX * 8 + 8))
    lp = _f64(lpf).reshape(Cn, 64) if lpf is not None else None
    pr = np.ascontiguousarray(present, dtype=np.int32) if present is not None else None
    L.or_imclt_frames(_d(clt), _i(pr) if pr is not None else None, tilesX, tilesY, S, Cn, float(scale),
                      _d(lp) if lp is not None else None, _d(out), int(num_threads or os.cpu_count() or 1), 0)
    return out


class TexParams(C.Structure):
    _fields_ = [("min_shot", C.c_double), ("scale_shot", C.c_double), ("diff_sigma", C.c_double),
                ("diff_threshold", C.c_double), ("min_agree", C.c_double), ("dust_remove", C.c_int),
                ("keep_weights", C.c_int), ("corr_magic_scale", C.c_double)]


def texture_params(**kw):
    """CLTParameters defaults of the texture path, with keyword overrides."""
    p = TexParams(10.0, 3.0, 5.0, 1.5, 3.0, 1, 1, 0.85)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def texture_tile(clt, lpf, img_mask=0xf, col_weights=(0.25, 0.25, 0.5), extra_disparity=0.0, params=None,
                 diag=False, near_tie=1e-6):
    """ImageDtt texture branch (2662-2812) for one tile: clt [4][3][4][64] ->
    (rgba [12][256], aux [16] = max_diff[4], ports_rgb[12]) and with diag the per-tile
    diagnostics [3] (smallest relative margins of the second-port and dust-removal choices,
    smallest distance of a weight exponent from the double underflow of exp) and the tile
    [12][256] with every near-tie choice (0 < relative margin < near_tie) taken the other way."""
    L = lib()
    if not getattr(L, "_tex_set", False):
        L.or_texture_tile_diag.argtypes = [_dp, _dp, C.c_int, _dp, C.c_double, C.POINTER(TexParams), _dp, _dp,
                                           _dp, _dp, C.c_double]
        L.or_texture_tile_diag.restype = None
        L._tex_set = True
    c = _f64(clt).reshape(4, 3, 4, 64)
    lp = _f64(lpf).reshape(64)
    cw = _f64(col_weights).reshape(3)
    out = np.zeros((12, 256))
    aux = np.zeros(16)
    dg = np.zeros(3)
    alt = np.zeros((12, 256))
    L.or_texture_tile_diag(_d(c), _d(lp), int(img_mask), _d(cw), float(extra_disparity),
                           C.byref(params if params is not None else texture_params()), _d(out), _d(aux), _d(dg),
                           _d(alt) if diag else None, float(near_tie))
    return (out, aux, dg, alt) if diag else (out, aux)


def texture_tiles(clt, tiles, img_mask, lpf, col_weights=(0.25, 0.25, 0.5), extra=None, params=None,
                  num_threads=None):
    """texture_tile over `tiles` of clt [tiles][4][3][4][64] on a thread pool ->
    (rgba [n][12][256], aux [n][16])."""
    L = lib()
    if not getattr(L, "_texs_set", False):
        L.or_texture_tiles.argtypes = [_dp, _ip, _ip, _dp, C.c_int, _dp, _dp, C.POINTER(TexParams), _dp, _dp,
                                       C.c_int]
        L.or_texture_tiles.restype = C.c_int
        L._texs_set = True
    c = _f64(clt)
    assert c.shape[1:3] == (4, 3)
    t = np.ascontiguousarray(tiles, dtype=np.int32)
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(img_mask, dtype=np.int32), t.shape))
    n = len(t)
    ex = _f64(np.broadcast_to(np.asarray(extra, dtype=np.float64), t.shape)) if extra is not None else None
    out = np.zeros((n, 12, 256))
    aux = np.zeros((n, 16))
    L.or_texture_tiles(_d(c), _i(t), _i(m), _d(ex) if ex is not None else None, n, _d(_f64(lpf).reshape(64)),
                       _d(_f64(col_weights).reshape(3)), C.byref(params if params is not None else texture_params()),
                       _d(out), _d(aux), int(num_threads or os.cpu_count() or 1))
    return out, aux


def rig_tile(clt_main, clt_aux, corr_params=None, cm_max_normalization=0.55, no_int_x0=False):
    """clt_main [S][C][4][64], clt_aux [S'][C][4][64] -> (corr [225], rec [4])."""
    L = lib()
    if not getattr(L, "_rig_set", False):
        L.or_rig_tile.argtypes = [_dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(CorrParams), C.c_double, C.c_int,
                                  _dp, _dp]
        L.or_rig_tile.restype = None
        L._rig_set = True
    a = _f64(clt_main)
    b = _f64(clt_aux)
    cp = corr_params if corr_params is not None else default_corr_params()
    corr = np.zeros(225)
    rec = np.zeros(4)
    L.or_rig_tile(_d(a), a.shape[0], _d(b), b.shape[0], a.shape[1], C.byref(cp), float(cm_max_normalization),
                  int(bool(no_int_x0)), _d(corr), _d(rec))
    return corr, rec


class LmaParams(C.Structure):
    _fields_ = [("min_poly_strength", C.c_double), ("mix_corr_poly", C.c_int), ("ortho_vasw_pwr", C.c_double),
                ("cnvx_hwnd_size", C.c_int), ("cnvx_weight", C.c_double), ("cnvx_add3x3", C.c_int),
                ("adjust_wm", C.c_int), ("adjust_wy", C.c_int), ("adjust_wxy", C.c_int), ("adjust_ag", C.c_int),
                ("half_width", C.c_double), ("cost_wy", C.c_double), ("cost_wxy", C.c_double),
                ("lambda_initial", C.c_double), ("lambda_scale_good", C.c_double), ("lambda_scale_bad", C.c_double),
                ("lambda_max", C.c_double), ("rms_diff", C.c_double), ("num_iter", C.c_int), ("pair_mask", C.c_int)]


def _lma_lib():
    L = lib()
    if not getattr(L, "_lma_set", False):
        L.or_default_lma_params.argtypes = [C.POINTER(LmaParams)]
        L.or_default_lma_params.restype = None
        L.or_corr_lma.argtypes = [_dp, C.POINTER(C.c_int), C.c_int, C.c_double, C.POINTER(LmaParams), _dp,
                                  C.POINTER(C.c_int)]
        L.or_corr_lma.restype = C.c_int
        L.or_filter_convex.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp]
        L.or_filter_convex.restype = None
        L.or_rig_lma.argtypes = [_dp, C.POINTER(LmaParams), C.c_int, C.c_int, C.c_double, _dp]
        L.or_rig_lma.restype = C.c_int
        L._lma_set = True
    return L


def default_lma_params(**kw):
    p = LmaParams()
    _lma_lib().or_default_lma_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rig_lma(corr225, rec, params=None, use_poly=True, use_xy_poly=True, max_corr_radius=3.9):
    """The LMA branch of ImageDtt.tileInterCamCorrs (ImageDtt.java:7497-7560) on one rig tile:
    (converged, rec') with rec = {disparity, strength, dx, dy} of the centre-of-mass record."""
    r = np.array(rec, dtype=np.float64)
    p = params if params is not None else default_lma_params()
    ok = _lma_lib().or_rig_lma(_d(_f64(corr225).reshape(225)), C.byref(p), int(bool(use_poly)),
                               int(bool(use_xy_poly)), float(max_corr_radius), _d(r))
    return bool(ok), r


def filter_convex(corr225, hwin, x0c, y0c, add3x3=True, nc_cost=0.5):
    a = _f64(corr225)
    out = np.zeros(225)
    _lma_lib().or_filter_convex(_d(a), int(hwin), int(x0c), int(y0c), int(bool(add3x3)), float(nc_cost), _d(out))
    return out


def corr_lma(corrs, kinds, xcenter, params=None):
    """Correlation2d.corrLMA on one tile: corrs [np][225], quad pair kinds -> (ok, {disparity, strength,
    WM, WXY}, number of samples)."""
    a = _f64(corrs)
    k = np.ascontiguousarray(np.asarray(kinds, dtype=np.int32))
    p = params if params is not None else default_lma_params()
    out = np.zeros(4)
    ns = C.c_int(0)
    ok = _lma_lib().or_corr_lma(_d(a), k.ctypes.data_as(C.POINTER(C.c_int)), a.shape[0], float(xcenter),
                                C.byref(p), _d(out), C.byref(ns))
    return bool(ok), out, ns.value


class FoParams(C.Structure):
    _fields_ = [("fo_correct", C.c_int), ("fo_far", C.c_int), ("fo_ortho", C.c_int),
                ("fo_min_strength", C.c_double), ("fo_min_eff", C.c_double), ("fo_min_eff_ratio", C.c_double),
                ("fo_max_hwidth", C.c_double), ("fo_min_diff", C.c_double), ("fo_overcorrection", C.c_double),
                ("fo_lim_overcorr", C.c_double)]


def default_fo_params(**kw):
    L = _lma_lib()
    if not getattr(L, "_fo_set", False):
        L.or_default_fo_params.argtypes = [C.POINTER(FoParams)]
        L.or_default_fo_params.restype = None
        L.or_lma_tile.argtypes = [_dp, C.POINTER(C.c_int), C.c_int, C.POINTER(LmaParams), C.POINTER(FoParams), _dp,
                                  _dp]
        L.or_lma_tile.restype = C.c_int
        L._fo_set = True
    f = FoParams()
    L.or_default_fo_params(C.byref(f))
    for k, v in kw.items():
        setattr(f, k, v)
    return f


def lma_tile(corrs, kinds, cm, strength, params=None, fo=None):
    """The record update of ImageDtt.java:2254-2335 for one tile -> (ran, {CM, strength, POLY}, main LMA [4])."""
    fo = fo if fo is not None else default_fo_params()
    p = params if params is not None else default_lma_params()
    a = _f64(corrs)
    k = np.ascontiguousarray(np.asarray(kinds, dtype=np.int32))
    rec = np.array([cm, strength, np.nan], dtype=np.float64)
    lma = np.zeros(4)
    ran = _lma_lib().or_lma_tile(_d(a), k.ctypes.data_as(C.POINTER(C.c_int)), a.shape[0], C.byref(p), C.byref(fo),
                                 _d(rec), _d(lma))
    return bool(ran), rec, lma


class LyParams(C.Structure):
    """The mismatch measure (ImageDttParameters.java:50-52): ly_poly, ly_crazy_poly, ly_poly_backup."""
    _fields_ = [("ly_poly", C.c_int), ("ly_crazy_poly", C.c_double), ("ly_poly_backup", C.c_int)]


def lma_tile_mismatch(corrs, kinds, cm, strength, max_corr_radius=3.9, mismatch_max_diff=1.0, params=None, fo=None,
                      ly_poly=False, ly_crazy_poly=1.0, ly_poly_backup=True):
    """lma_tile with the lazy-eye mismatch -> (ran, {CM, strength, POLY}, main LMA [4], mismatch [np][3]);
    ly_poly selects mismatchPairs (quadric maxima) over mismatchPairsCM."""
    fo = fo if fo is not None else default_fo_params()
    p = params if params is not None else default_lma_params()
    L = _lma_lib()
    if not getattr(L, "_mism_set", False):
        L.or_lma_tile_mismatch_ly.argtypes = [_dp, C.POINTER(C.c_int), C.c_int, C.POINTER(LmaParams),
                                              C.POINTER(FoParams), C.c_double, C.c_double, C.POINTER(LyParams),
                                              _dp, _dp, _dp]
        L.or_lma_tile_mismatch_ly.restype = C.c_int
        L._mism_set = True
    ly = LyParams(int(bool(ly_poly)), float(ly_crazy_poly), int(bool(ly_poly_backup)))
    a = _f64(corrs)
    k = np.ascontiguousarray(np.asarray(kinds, dtype=np.int32))
    rec = np.array([cm, strength, np.nan], dtype=np.float64)
    lma = np.zeros(4)
    mism = np.zeros((a.shape[0], 3))
    ran = L.or_lma_tile_mismatch_ly(_d(a), k.ctypes.data_as(C.POINTER(C.c_int)), a.shape[0], C.byref(p),
                                    C.byref(fo), float(max_corr_radius), float(mismatch_max_diff), C.byref(ly),
                                    _d(rec), _d(lma), _d(mism))
    return bool(ran), rec, lma, mism


def quadratic_max(x, y, v, w):
    """Correlations2dLMA.getMaxXYPoly on samples: (ok, {x, y, value}) of the weighted quadric's maximum."""
    L = _lma_lib()
    if not getattr(L, "_qmax_set", False):
        L.or_quadratic_max.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp]
        L.or_quadratic_max.restype = C.c_int
        L._qmax_set = True
    xs, ys, vs, ws = (_f64(a) for a in (x, y, v, w))
    out = np.full(3, np.nan)
    ok = L.or_quadratic_max(_d(xs), _d(ys), _d(vs), _d(ws), len(xs), _d(out))
    return bool(ok), out
