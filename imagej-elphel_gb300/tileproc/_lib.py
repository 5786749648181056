"""ctypes binding of libtp.so (include/tp.h).

The library is built in-tree by imagej-elphel_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libtp.so")

TP_MAX_SENSORS = 16
TP_MAX_PAIRS = 120
TP_OK, TP_ERR_ARG, TP_ERR_CUDA, TP_ERR_STATE, TP_ERR_NOMEM, TP_ERR_TIMEOUT, TP_ERR_NOT_BUILT, TP_ERR_SCRATCH_LIMIT = range(8)
TP_COMPACT_MAX_TILES = 1024 * 1024
TP_F32, TP_U16 = 0, 1
TP_KERNELS_GPU, TP_KERNELS_CPU = 0, 1
DISP_N = 9
(DISP_INT, DISP_CM, DISP_STRENGTH, DISP_HOR, DISP_HOR_STRENGTH, DISP_VERT, DISP_VERT_STRENGTH,
 DISP_CM_S0, DISP_IXY) = range(9)


class TpConfig(C.Structure):
    _fields_ = [("num_sensors", C.c_int), ("num_colors", C.c_int), ("width", C.c_int), ("height", C.c_int),
                ("kernels_hor", C.c_int), ("kernels_vert", C.c_int), ("kernel_step", C.c_int),
                ("bayer_red_row", C.c_int), ("bayer_red_col", C.c_int), ("device", C.c_int)]


class TpGeometry(C.Structure):
    _fields_ = [("pixel_width", C.c_int), ("pixel_height", C.c_int), ("focal_length", C.c_double),
                ("pixel_size", C.c_double), ("distortion_radius", C.c_double), ("distortion", C.c_double * 7),
                ("rXY", (C.c_double * 2) * TP_MAX_SENSORS), ("pXY0", (C.c_double * 2) * TP_MAX_SENSORS),
                ("azimuth", C.c_double * TP_MAX_SENSORS), ("tilt", C.c_double * TP_MAX_SENSORS),
                ("roll", C.c_double * TP_MAX_SENSORS), ("zoom", C.c_double * TP_MAX_SENSORS)]


class TpRigOffset(C.Structure):
    _fields_ = [("main_disparity_radius", C.c_double), ("aux_disparity_radius", C.c_double),
                ("baseline", C.c_double), ("aux_angle", C.c_double), ("aux_azimuth", C.c_double),
                ("aux_tilt", C.c_double), ("aux_roll", C.c_double), ("aux_zoom", C.c_double)]


class TpPair(C.Structure):
    _fields_ = [("cam1", C.c_int), ("cam2", C.c_int), ("kind", C.c_int), ("in_combo", C.c_int),
                ("bx", C.c_float), ("by", C.c_float)]


class TpCorrParams(C.Structure):
    _fields_ = [("fat_zero", C.c_float), ("corr_sigma", C.c_float), ("corr_red", C.c_float),
                ("corr_blue", C.c_float), ("corr_offset", C.c_float), ("min_corr", C.c_float),
                ("corr_strip_hight", C.c_int), ("twice_diagonal", C.c_int), ("enhortho_width", C.c_float),
                ("enhortho_scale", C.c_float), ("corr_wndy_size", C.c_int), ("corr_wndy_hwidth", C.c_float),
                ("corr_wndy_blur", C.c_float), ("corr_wndx_size", C.c_int), ("corr_wndx_hwidth", C.c_float),
                ("corr_wndx_blur", C.c_float)]


class TpTextureParams(C.Structure):
    _fields_ = [("min_shot", C.c_float), ("scale_shot", C.c_float), ("diff_sigma", C.c_float),
                ("corr_magic_scale", C.c_float), ("dust_remove", C.c_int), ("keep_weights", C.c_int),
                ("corr_mode", C.c_int), ("aux", C.c_int)]


class TpLmaParams(C.Structure):
    _fields_ = [("min_poly_strength", C.c_float), ("mix_corr_poly", C.c_int), ("ortho_vasw_pwr", C.c_float),
                ("cnvx_hwnd_size", C.c_int), ("cnvx_weight", C.c_float), ("cnvx_add3x3", C.c_int),
                ("adjust_wm", C.c_int), ("adjust_wy", C.c_int), ("adjust_wxy", C.c_int), ("adjust_ag", C.c_int),
                ("half_width", C.c_float), ("cost_wy", C.c_float), ("cost_wxy", C.c_float),
                ("lambda_initial", C.c_float), ("lambda_scale_good", C.c_float), ("lambda_scale_bad", C.c_float),
                ("lambda_max", C.c_float), ("rms_diff", C.c_float), ("num_iter", C.c_int), ("pair_mask", C.c_int),
                ("fo_correct", C.c_int), ("fo_far", C.c_int), ("fo_ortho", C.c_int), ("fo_min_strength", C.c_float),
                ("fo_min_eff", C.c_float), ("fo_min_eff_ratio", C.c_float), ("fo_max_hwidth", C.c_float),
                ("fo_min_diff", C.c_float), ("fo_overcorrection", C.c_float), ("fo_lim_overcorr", C.c_float),
                ("mismatch", C.c_int), ("max_corr_radius", C.c_float), ("mismatch_max_diff", C.c_float),
                ("ly_poly", C.c_int), ("ly_crazy_poly", C.c_float), ("ly_poly_backup", C.c_int)]


_H = C.c_void_p
_vp = C.c_void_p

# name -> argtypes; every function returns tp_status (int)
PROTOTYPES = {
    "tp_create": [C.POINTER(TpConfig), C.POINTER(_H)],
    "tp_destroy": [_H],
    "tp_last_error": [_H, C.c_char_p, C.c_int],
    "tp_set_memory_limit": [C.c_size_t],
    "tp_get_memory_usage": [_H, C.POINTER(C.c_size_t)],
    "tp_default_corr_params": [C.POINTER(TpCorrParams)],
    "tp_default_texture_params": [C.POINTER(TpTextureParams)],
    "tp_quad_pairs": [C.POINTER(TpPair), C.POINTER(C.c_int)],
    "tp_set_geometry": [_H, C.POINTER(TpGeometry)],
    "tp_set_rig_geometry": [_H, C.POINTER(TpGeometry), C.POINTER(TpGeometry), C.POINTER(TpRigOffset)],
    "tp_set_kernels": [_H, C.c_int, _vp, _vp, C.c_int],
    "tp_set_image": [_H, C.c_int, _vp, C.c_int, C.c_size_t],
    "tp_set_image_async": [_H, C.c_int, _vp, C.c_int, C.c_size_t, _vp],
    "tp_set_color_scales": [_H, _vp],
    "tp_set_tasks": [_H, _vp, C.c_int],
    "tp_set_tile_ops": [_H, _vp, _vp],
    "tp_set_lpf": [_H, _vp],
    "tp_set_clt_lpf_mask": [_H, C.c_int],
    "tp_calc_kernels": [_H, C.c_int, _vp, C.c_int, C.c_int, C.c_int, _vp],
    "tp_dtt8x8": [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp],
    "tp_get_kernels": [_H, C.c_int, _vp, _vp],
    "tp_set_corr": [_H, C.POINTER(TpCorrParams), C.POINTER(TpPair), C.c_int],
    "tp_set_texture_params": [_H, C.POINTER(TpTextureParams)],
    "tp_ports": [_H, _vp],
    "tp_convert_correct": [_H, _vp],
    "tp_correlate": [_H, _vp],
    "tp_extract": [_H, _vp],
    "tp_imclt": [_H, _vp],
    "tp_textures": [_H, _vp],
    "tp_process": [_H, _vp],
    "tp_set_schedule": [_H, C.c_int, C.c_int],
    "tp_synchronize": [_H],
    "tp_get_num_tasks": [_H, C.POINTER(C.c_int)],
    "tp_get_ports": [_H, _vp],
    "tp_get_task_tiles": [_H, _vp],
    "tp_get_subtiles": [_H, _vp, _vp],
    "tp_get_clt": [_H, _vp],
    "tp_get_corr": [_H, _vp],
    "tp_get_disparity": [_H, _vp],
    "tp_get_rbg": [_H, C.c_int, _vp],
    "tp_get_rbg_async": [_H, C.c_int, _vp, _vp],
    "tp_get_disparity_async": [_H, _vp, _vp],
    "tp_get_textures": [_H, _vp],
    "tp_get_texture_aux": [_H, _vp],
    "tp_compact_tile_ops_noalloc": [_vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp],
    "tp_default_lma_params": [C.POINTER(TpLmaParams)],
    "tp_lma_refine": [_H, C.POINTER(TpLmaParams), _vp],
    "tp_get_lma": [_H, _vp],
    "tp_get_lma_mismatch": [_H, _vp],
    "tp_get_pair_maxima": [_H, _vp],
    "tp_rig_correlate": [_H, _H, C.c_float, C.c_int, _vp],
    "tp_get_rig": [_H, _vp, _vp],
    "tp_rig_lma": [_H, C.POINTER(TpLmaParams), C.c_int, C.c_int, _vp],
    "tp_batch_create": [C.POINTER(_H), C.c_int, C.POINTER(_H)],
    "tp_batch_destroy": [_H],
    "tp_batch_last_error": [_H, C.c_char_p, C.c_int],
    "tp_batch_process": [_H, C.c_int, _vp],
    "tp_batch_run_graph": [_H, _vp],
    "tp_batch_synchronize": [_H],
    "tp_backward": [_H, _vp, _vp, _vp, _vp],
    "tp_set_adjoint_mode": [_H, C.c_int],
    "tp_get_disparity_jacobian": [_H, _vp, _vp, _vp],
    "tp_get_port_sensitivities": [_H, _vp],
    "tp_get_port_derivatives": [_H, _vp],
}

_lib = None


def load():
    """Load libtp.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libtp.so is not built (%s); run imagej-elphel_gb300/build.py" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, args in PROTOTYPES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        _lib = L
    return _lib


class TpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("tp status %d: %s" % (status, msg))
        self.status = status
