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
    return O.run(W, H, oracle_planes(scene), tile_op, np.broadcast_to(np.asarray(target, np.float64), (T,)),
                 geometry=scene["geometry"], ports_in=ports_in, kernels=kern, kernel_ext=kx,
                 pairs=pairs, corr_params=corr_params, corr=corr, num_threads=threads)


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
