"""Host-side mirror of com.elphel.imagej.gpu.GPUTileProcessor over libtp.so.

Method names follow the reference (GPUTileProcessor.java) so a caller of the
Java class finds the same calls; the data are numpy arrays and every call goes
through the C ABI of include/tp.h.  The ImageDtt-shaped one-shot call
(clt_aberrations_quad_corr) is `process()`.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class GPUTileProcessor:
    """One device context / buffer set for a fixed image geometry (GPUTileProcessor.java:243-360)."""

    def __init__(self, num_sensors, width, height, num_colors=1, kernels_hor=0, kernels_vert=0,
                 kernel_step=16, bayer_red_row=0, bayer_red_col=1, device=0):
        self._lib = L.load()
        cfg = L.TpConfig(num_sensors, num_colors, width, height, kernels_hor, kernels_vert, kernel_step,
                         bayer_red_row, bayer_red_col, device)
        h = C.c_void_p()
        st = self._lib.tp_create(C.byref(cfg), C.byref(h))
        if st != L.TP_OK:
            raise L.TpError(st, "tp_create failed")
        self.h = h
        self.num_sensors, self.num_colors = num_sensors, num_colors
        self.width, self.height = width, height
        self.tilesX, self.tilesY = width // 8, height // 8
        self.kernels_hor, self.kernels_vert = kernels_hor, kernels_vert
        self.num_pairs = 6 if num_sensors == 4 else 0

    # ---- plumbing ----
    def _ck(self, st, what):
        if st != L.TP_OK:
            buf = C.create_string_buffer(512)
            if self.h:
                self._lib.tp_last_error(self.h, buf, 512)
            raise L.TpError(st, "%s: %s" % (what, buf.value.decode(errors="replace")))

    def close(self):
        if getattr(self, "h", None):
            self._lib.tp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- inputs (GPUTileProcessor.java:363-527, 780-848) ----
    @staticmethod
    def _geometry(g, num_sensors):
        G = L.TpGeometry()
        G.pixel_width, G.pixel_height = int(g["width"]), int(g["height"])
        G.focal_length, G.pixel_size = float(g["focal_length"]), float(g["pixel_size"])
        G.distortion_radius = float(g["distortion_radius"])
        for i in range(7):
            G.distortion[i] = float(g["distortion"][i])
        for s in range(num_sensors):
            for k in range(2):
                G.rXY[s][k] = float(g["rXY"][s][k])
                G.pXY0[s][k] = float(g["pXY0"][s][k])
            G.azimuth[s], G.tilt[s] = float(g["azimuth"][s]), float(g["tilt"][s])
            G.roll[s], G.zoom[s] = float(g["roll"][s]), float(g["zoom"][s])
        return G

    def setGeometry(self, g):
        """g: dict with keys width, height, focal_length, pixel_size, distortion_radius,
        distortion[7], rXY[S][2], pXY0[S][2], azimuth/tilt/roll/zoom[S]."""
        G = self._geometry(g, self.num_sensors)
        self._ck(self._lib.tp_set_geometry(self.h, C.byref(G)), "tp_set_geometry")

    def setRigGeometry(self, aux, main, rig):
        """This camera as a rig's auxiliary one (GeometryCorrection.RigOffset; the ports of
        ImageDtt.clt_bi_quad): aux / main geometry dicts as setGeometry's (main with the main camera's
        sensor count), rig a dict of main_disparity_radius, aux_disparity_radius, baseline, aux_angle,
        aux_azimuth, aux_tilt, aux_roll, aux_zoom.  Task disparities are then the main camera's."""
        A = self._geometry(aux, self.num_sensors)
        M = self._geometry(main, int(main.get("num_sensors", self.num_sensors)))
        R = L.TpRigOffset(*[float(rig[name]) for name, _ in L.TpRigOffset._fields_])
        self._ck(self._lib.tp_set_rig_geometry(self.h, C.byref(A), C.byref(M), C.byref(R)), "tp_set_rig_geometry")

    def setConvolutionKernel(self, kernel, kernel_offsets, ncam, layout=L.TP_KERNELS_GPU):
        k = np.ascontiguousarray(kernel, dtype=np.float32)
        o = np.ascontiguousarray(kernel_offsets, dtype=np.float32)
        n = self.kernels_hor * self.kernels_vert * self.num_colors
        if k.size != n * 256 or o.size != n * 8:
            raise ValueError("kernel table size mismatch")
        self._ck(self._lib.tp_set_kernels(self.h, int(ncam), _ptr(k), _ptr(o), int(layout)), "tp_set_kernels")

    def setConvolutionKernels(self, kernels, kernel_offsets, layout=L.TP_KERNELS_CPU):
        """kernels: [S][kv][kh][C][4][64], offsets [S][kv][kh][C][8]."""
        for cam in range(self.num_sensors):
            self.setConvolutionKernel(kernels[cam], kernel_offsets[cam], cam, layout)

    def calcConvolutionKernels(self, psf, ncam, normalize=True, coord_corr=True, device_ptr=None, stream=None):
        """QuadCLT.calculateCLTKernel on the device: psf [kv][kh][C][64][64] float (host array), or
        device_ptr (an int address of the same layout in device memory)."""
        if device_ptr is not None:
            self._ck(self._lib.tp_calc_kernels(self.h, int(ncam), C.c_void_p(int(device_ptr)), 1, int(normalize),
                                               int(coord_corr), stream), "tp_calc_kernels")
            return
        p = np.ascontiguousarray(psf, dtype=np.float32)
        n = self.kernels_vert * self.kernels_hor * self.num_colors
        assert p.size == n * 4096, "psf must be [kernels_vert][kernels_hor][num_colors][64][64]"
        self._ck(self._lib.tp_calc_kernels(self.h, int(ncam), _ptr(p), 0, int(normalize), int(coord_corr), stream),
                 "tp_calc_kernels")

    def getConvolutionKernels(self, ncam):
        """(kernels [kv][kh][C][4][64], offsets [kv][kh][C][8]) of one sensor (TP_KERNELS_CPU layout)."""
        k = np.zeros((self.kernels_vert, self.kernels_hor, self.num_colors, 4, 64), dtype=np.float32)
        e = np.zeros((self.kernels_vert, self.kernels_hor, self.num_colors, 8), dtype=np.float32)
        self._ck(self._lib.tp_get_kernels(self.h, int(ncam), _ptr(k), _ptr(e)), "tp_get_kernels")
        return k, e

    def setBayerImage(self, image, ncam):
        img = np.ascontiguousarray(image)
        if img.shape != (self.height, self.width):
            raise ValueError("image shape %s != (%d, %d)" % (img.shape, self.height, self.width))
        dt = {np.dtype(np.float32): L.TP_F32, np.dtype(np.uint16): L.TP_U16}.get(img.dtype)
        if dt is None:
            raise ValueError("image dtype must be float32 or uint16")
        self._ck(self._lib.tp_set_image(self.h, int(ncam), _ptr(img), dt, 0), "tp_set_image")

    def setBayerImages(self, images):
        """One mosaic (or mono image) per sensor: [S][H][W] float32 or uint16."""
        for cam in range(self.num_sensors):
            self.setBayerImage(images[cam], cam)

    def setBayerPlanes(self, planes, force=True):
        """GPUTileProcessor.setBayerImages(double[][][] bayer_data, force) (GPUTileProcessor.java:
        452-468): per sensor the colour planes [C][H*W] (the EyesisCorrections.bayerToDoubleStack
        split, green already scaled) are summed into one float mosaic and uploaded; with force off
        a second call is skipped, as in the reference."""
        if getattr(self, "_planes_set", False) and not force:
            return
        for cam in range(self.num_sensors):
            p = np.asarray(planes[cam], dtype=np.float64).reshape(-1, self.height * self.width)
            mosaic = p.sum(axis=0).astype(np.float32).reshape(self.height, self.width)
            self.setBayerImage(mosaic, cam)
        self._planes_set = True

    def setColorScales(self, scales):
        s = np.ascontiguousarray(scales, dtype=np.float32)
        self._ck(self._lib.tp_set_color_scales(self.h, _ptr(s)), "tp_set_color_scales")

    def setTasks(self, packed_tasks):
        """packed_tasks: float32 [n][2 + 2S] in TpTask.asFloatArray layout."""
        t = np.ascontiguousarray(packed_tasks, dtype=np.float32)
        n = t.shape[0] if t.ndim == 2 else 0
        self._ck(self._lib.tp_set_tasks(self.h, _ptr(t), n), "tp_set_tasks")

    @staticmethod
    def packTasks(task, tx, ty, xy):
        """TpTask.asFloatArray (GPUTileProcessor.java:150-165) for arrays of tasks."""
        n = len(task)
        S = xy.shape[1]
        out = np.zeros((n, 2 + 2 * S), dtype=np.float32)
        out[:, 0] = np.asarray(task, dtype=np.int32).view(np.float32)
        out[:, 1] = (np.asarray(tx, dtype=np.int32) + (np.asarray(ty, dtype=np.int32) << 16)).view(np.float32)
        out[:, 2:] = np.asarray(xy, dtype=np.float32).reshape(n, 2 * S)
        return out

    def setFullFrameImages(self, target_disparities, tile_op=None):
        """Tasks for all tiles (or those with tile_op != 0) with device-side FP64 ports."""
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(target_disparities, dtype=np.float32),
                                                 (self.tilesY * self.tilesX,)))
        if tile_op is None:
            tile_op = np.ones(self.tilesY * self.tilesX, dtype=np.int32)
        op = np.ascontiguousarray(tile_op, dtype=np.int32).reshape(-1)
        self._ck(self._lib.tp_set_tile_ops(self.h, _ptr(op), _ptr(d)), "tp_set_tile_ops")

    def setLpfRbg(self, lpf):
        if lpf is None:
            self._ck(self._lib.tp_set_lpf(self.h, None), "tp_set_lpf")
            return
        l = np.ascontiguousarray(lpf, dtype=np.float32).reshape(self.num_colors, 64)
        self._ck(self._lib.tp_set_lpf(self.h, _ptr(l)), "tp_set_lpf")

    def setCltLpfMask(self, lpf_mask=7):
        """Store the CLT low-pass filtered as GPUTileProcessor.execConverCorrectTiles does (its
        lpf_mask = 7, GPUTileProcessor.java:547), with the filter of setLpfRbg; 0 = unfiltered."""
        self._ck(self._lib.tp_set_clt_lpf_mask(self.h, int(lpf_mask)), "tp_set_clt_lpf_mask")

    def setCorrelation(self, params=None, pairs=None, **kw):
        """params: TpCorrParams or None (reference defaults, overridable by keyword)."""
        if params is None:
            params = L.TpCorrParams()
            self._ck(self._lib.tp_default_corr_params(C.byref(params)), "tp_default_corr_params")
        for k, v in kw.items():
            setattr(params, k, v)
        if pairs is None:
            arr = (L.TpPair * 6)()
            n = C.c_int()
            self._ck(self._lib.tp_quad_pairs(arr, C.byref(n)), "tp_quad_pairs")
            np_ = n.value
        else:
            np_ = len(pairs)
            arr = (L.TpPair * max(np_, 1))()
            for i, (a, b, kind, in_combo, bx, by) in enumerate(pairs):
                arr[i] = L.TpPair(a, b, kind, in_combo, bx, by)
        self._ck(self._lib.tp_set_corr(self.h, C.byref(params), arr, np_), "tp_set_corr")
        self.num_pairs = np_
        self.pairs = [(arr[i].cam1, arr[i].cam2, arr[i].kind, arr[i].in_combo) for i in range(np_)]

    def setTextureParams(self, params=None, **kw):
        """Texture-tile settings: TpTextureParams or None (CLTParameters defaults), keyword overrides."""
        if params is None:
            params = L.TpTextureParams()
            self._ck(self._lib.tp_default_texture_params(C.byref(params)), "tp_default_texture_params")
        for k, v in kw.items():
            setattr(params, k, v)
        self._ck(self._lib.tp_set_texture_params(self.h, C.byref(params)), "tp_set_texture_params")
        self._tex_rows = 12 if params.keep_weights else 4

    # ---- execution ----
    def execPorts(self, stream=None):
        self._ck(self._lib.tp_ports(self.h, stream), "tp_ports")

    def execConverCorrectTiles(self, stream=None):
        self._ck(self._lib.tp_convert_correct(self.h, stream), "tp_convert_correct")

    def execCorrelate(self, stream=None):
        self._ck(self._lib.tp_correlate(self.h, stream), "tp_correlate")

    def execExtract(self, stream=None):
        self._ck(self._lib.tp_extract(self.h, stream), "tp_extract")

    def execImcltRbg(self, stream=None):
        self._ck(self._lib.tp_imclt(self.h, stream), "tp_imclt")

    def execTextures(self, stream=None):
        """Texture tiles (ImageDtt texture_tiles) of the current CLT and disparity."""
        self._ck(self._lib.tp_textures(self.h, stream), "tp_textures")

    def process(self, stream=None):
        self._ck(self._lib.tp_process(self.h, stream), "tp_process")

    def synchronize(self):
        self._ck(self._lib.tp_synchronize(self.h), "tp_synchronize")

    # ---- outputs ----
    def numTasks(self):
        n = C.c_int()
        self._ck(self._lib.tp_get_num_tasks(self.h, C.byref(n)), "tp_get_num_tasks")
        return n.value

    def getPorts(self):
        out = np.zeros((self.numTasks(), self.num_sensors, 2), dtype=np.float64)
        self._ck(self._lib.tp_get_ports(self.h, _ptr(out)), "tp_get_ports")
        return out

    def getTaskTiles(self):
        out = np.zeros(self.numTasks(), dtype=np.int32)
        self._ck(self._lib.tp_get_task_tiles(self.h, _ptr(out)), "tp_get_task_tiles")
        return out

    def getSubtiles(self):
        n = self.numTasks()
        tl = np.zeros((n, self.num_sensors, self.num_colors, 2), dtype=np.int32)
        res = np.zeros((n, self.num_sensors, self.num_colors, 2), dtype=np.float32)
        self._ck(self._lib.tp_get_subtiles(self.h, _ptr(tl), _ptr(res)), "tp_get_subtiles")
        return tl, res

    def getClt(self):
        out = np.zeros((self.tilesY * self.tilesX, self.num_sensors, self.num_colors, 4, 64), dtype=np.float32)
        self._ck(self._lib.tp_get_clt(self.h, _ptr(out)), "tp_get_clt")
        return out

    def getCorr(self):
        out = np.zeros((self.tilesY * self.tilesX, self.num_pairs, 225), dtype=np.float32)
        self._ck(self._lib.tp_get_corr(self.h, _ptr(out)), "tp_get_corr")
        return out

    def getDisparity(self):
        out = np.zeros((self.tilesY * self.tilesX, L.DISP_N), dtype=np.float32)
        self._ck(self._lib.tp_get_disparity(self.h, _ptr(out)), "tp_get_disparity")
        return out

    def getRBG(self, ncam):
        out = np.zeros((self.num_colors, self.height + 8, self.width + 8), dtype=np.float32)
        self._ck(self._lib.tp_get_rbg(self.h, int(ncam), _ptr(out)), "tp_get_rbg")
        return out

    # ---- LMA disparity ----
    def lmaRefine(self, params=None, stream=None, **kw):
        """Correlation2d.corrLMA on the last process(): returns [tiles][4] = {disparity, strength, WM, WXY}
        (NaN where not run); with mix_corr_poly (default) the disparity record's CM / strength take it."""
        if params is None:
            params = L.TpLmaParams()
            self._ck(self._lib.tp_default_lma_params(C.byref(params)), "tp_default_lma_params")
        for k, v in kw.items():
            setattr(params, k, v)
        self._ck(self._lib.tp_lma_refine(self.h, C.byref(params), stream), "tp_lma_refine")
        return self.getLma()

    def getLmaMismatch(self):
        """[tiles][pairs][3] lazy-eye mismatch {dx, dy, strength} of the last lmaRefine(mismatch=1)."""
        out = np.zeros((self.tilesY * self.tilesX, self.num_pairs, 3), dtype=np.float32)
        self._ck(self._lib.tp_get_lma_mismatch(self.h, _ptr(out)), "tp_get_lma_mismatch")
        return out

    def getPairMaxima(self):
        """[tiles][pairs][3] 2D maximum {dx, dy, strength} of every pair surface of the last process()."""
        out = np.zeros((self.tilesY * self.tilesX, self.num_pairs, 3), dtype=np.float32)
        self._ck(self._lib.tp_get_pair_maxima(self.h, _ptr(out)), "tp_get_pair_maxima")
        return out

    def getLma(self):
        out = np.zeros((self.tilesY * self.tilesX, 4), dtype=np.float32)
        self._ck(self._lib.tp_get_lma(self.h, _ptr(out)), "tp_get_lma")
        return out

    # ---- rig ----
    def rigCorrelate(self, aux, cm_max_normalization=0.55, no_int_x0=False, stream=None):
        """Inter-camera correlation with the auxiliary camera `aux` (another GPUTileProcessor on the
        same tile grid); returns (corr [tiles][225], rec [tiles][4] = disparity, strength, dx, dy)."""
        self._ck(self._lib.tp_rig_correlate(self.h, aux.h, float(cm_max_normalization), int(bool(no_int_x0)), stream),
                 "tp_rig_correlate")
        T = self.tilesY * self.tilesX
        corr = np.zeros((T, 225), dtype=np.float32)
        rec = np.zeros((T, 4), dtype=np.float32)
        self._ck(self._lib.tp_get_rig(self.h, _ptr(corr), _ptr(rec)), "tp_get_rig")
        return corr, rec

    def rigLma(self, use_poly=True, use_xy_poly=True, params=None, stream=None, **kw):
        """The LMA branch of the last rigCorrelate (ImageDtt.tileInterCamCorrs, ImageDtt.java:7497-7560,
        rig.use_poly / rig.use_xy_poly): returns the updated rec [tiles][4]."""
        if params is None:
            params = L.TpLmaParams()
            self._ck(self._lib.tp_default_lma_params(C.byref(params)), "tp_default_lma_params")
        for k, v in kw.items():
            setattr(params, k, v)
        self._ck(self._lib.tp_rig_lma(self.h, C.byref(params), int(bool(use_poly)), int(bool(use_xy_poly)), stream),
                 "tp_rig_lma")
        rec = np.zeros((self.tilesY * self.tilesX, 4), dtype=np.float32)
        self._ck(self._lib.tp_get_rig(self.h, None, _ptr(rec)), "tp_get_rig")
        return rec

    # ---- adjoint ----
    def setAdjointMode(self, recompute_clt=False):
        self._ck(self._lib.tp_set_adjoint_mode(self.h, int(bool(recompute_clt))), "tp_set_adjoint_mode")

    def backward(self, dl_ddisp=None, stream=None):
        """Adjoint of the last process(): returns (dL/d extrinsics [S][4], dL/d tile disparity [tiles])
        for L = sum l(d) with dl/dd = dl_ddisp (default 2 d)."""
        T = self.tilesY * self.tilesX
        ge = np.zeros((self.num_sensors, 4), dtype=np.float32)
        gd = np.zeros(T, dtype=np.float32)
        dl = None
        if dl_ddisp is not None:
            dl = np.ascontiguousarray(np.broadcast_to(np.asarray(dl_ddisp, dtype=np.float32), (T,)))
        self._ck(self._lib.tp_backward(self.h, _ptr(dl) if dl is not None else None, _ptr(ge), _ptr(gd), stream),
                 "tp_backward")
        return ge, gd

    def getDisparityJacobian(self):
        """(jac_extr [tiles][S][4], jac_disp [tiles], disparity [tiles]) of the last backward()."""
        T = self.tilesY * self.tilesX
        je = np.zeros((T, self.num_sensors, 4), dtype=np.float32)
        jd = np.zeros(T, dtype=np.float32)
        d = np.zeros(T, dtype=np.float32)
        self._ck(self._lib.tp_get_disparity_jacobian(self.h, _ptr(je), _ptr(jd), _ptr(d)), "tp_get_disparity_jacobian")
        return je, jd, d

    def getPortSensitivities(self):
        out = np.zeros((self.tilesY * self.tilesX, self.num_sensors, 2), dtype=np.float32)
        self._ck(self._lib.tp_get_port_sensitivities(self.h, _ptr(out)), "tp_get_port_sensitivities")
        return out

    def getPortDerivatives(self):
        out = np.zeros((self.numTasks(), self.num_sensors, 2, 5), dtype=np.float64)
        self._ck(self._lib.tp_get_port_derivatives(self.h, _ptr(out)), "tp_get_port_derivatives")
        return out

    def getTextures(self):
        """[tilesY * tilesX][4 or 12][256]: R, B, G, alpha (+ 4 port weights, 4 rms)."""
        rows = getattr(self, "_tex_rows", 12)
        out = np.zeros((self.tilesY * self.tilesX, rows, 256), dtype=np.float32)
        self._ck(self._lib.tp_get_textures(self.h, _ptr(out)), "tp_get_textures")
        return out

    def getTextureAux(self):
        """[tilesY * tilesX][16]: max_diff[4], ports_rgb[12] (colour * 4 + port)."""
        out = np.zeros((self.tilesY * self.tilesX, 16), dtype=np.float32)
        self._ck(self._lib.tp_get_texture_aux(self.h, _ptr(out)), "tp_get_texture_aux")
        return out

    def setSchedule(self, tiles_per_block=0, warps_per_block=0):
        """Fused-kernel schedule (0, 0 = defaults for the sensor/colour layout)."""
        self._ck(self._lib.tp_set_schedule(self.h, int(tiles_per_block), int(warps_per_block)), "tp_set_schedule")
