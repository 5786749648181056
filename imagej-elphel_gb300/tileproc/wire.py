"""The reference's GPU-debug wire formats (little-endian float32 files written by
TwoQuadCLT.saveFloatKernels, TwoQuadCLT.java:1076-1178, and read by
TwoQuadCLT.getFloatsFromFile / showImageFromGPU, 1025-1074), so that dumps of a
real camera set can feed this processor and its outputs can be inspected with
the reference's own viewers.

  <prefix>_chn<N>[_transposed].kernel    [kv][kh][colour][4][64] CLT kernel tables
                                         (64 coefficients transposed in the _transposed file)
  <prefix>_chn<N>[_transposed].kernel_offsets  [kv][kh][colour][8] CltExtra records
  <prefix>_chn<N>.bayer                  [H][W] mosaic (sum of the colour planes)
  <prefix>_chn<N>.portsxy                [tiles][2] port x, y of sensor N
  *.rbg                                  [colours][(H + 8) * (W + 8)] IMCLT frames (getRBG)
"""
import numpy as np

_LE = "<f4"


def _transpose64(a):
    """Swap the two 8-index halves of the last axis (GPUTileProcessor.setConvolutionKernels 406-410)."""
    s = a.shape
    return np.ascontiguousarray(a.reshape(s[:-1] + (8, 8)).swapaxes(-1, -2).reshape(s))


def kernel_paths(prefix, chn, transposed=False):
    t = "_transposed" if transposed else ""
    return "%s_chn%d%s.kernel" % (prefix, chn, t), "%s_chn%d%s.kernel_offsets" % (prefix, chn, t)


def write_kernels(prefix, chn, kernels, offsets, transposed=False):
    """kernels [kv][kh][C][4][64] (ImageDtt coefficient order), offsets [kv][kh][C][8]."""
    kp, op = kernel_paths(prefix, chn, transposed)
    k = np.asarray(kernels, np.float64)
    if transposed:
        k = _transpose64(k)
    k.astype(_LE).tofile(kp)
    np.asarray(offsets, np.float64).astype(_LE).tofile(op)
    return kp, op


def read_kernels(prefix, chn, kernels_vert, kernels_hor, num_colors, transposed=False):
    """-> (kernels [kv][kh][C][4][64] in ImageDtt order, offsets [kv][kh][C][8]), float32."""
    kp, op = kernel_paths(prefix, chn, transposed)
    k = np.fromfile(kp, dtype=_LE).reshape(kernels_vert, kernels_hor, num_colors, 4, 64)
    if transposed:
        k = _transpose64(k)
    o = np.fromfile(op, dtype=_LE).reshape(kernels_vert, kernels_hor, num_colors, 8)
    return k.astype(np.float32), o.astype(np.float32)


def write_bayer(prefix, chn, mosaic):
    path = "%s_chn%d.bayer" % (prefix, chn)
    np.asarray(mosaic, np.float64).astype(_LE).tofile(path)
    return path


def read_bayer(prefix, chn, width, height):
    return np.fromfile("%s_chn%d.bayer" % (prefix, chn), dtype=_LE).reshape(height, width).astype(np.float32)


def write_portsxy(prefix, chn, ports):
    """ports [tiles][2] (x, y) of sensor chn."""
    path = "%s_chn%d.portsxy" % (prefix, chn)
    np.asarray(ports, np.float64).astype(_LE).tofile(path)
    return path


def read_portsxy(prefix, chn):
    return np.fromfile("%s_chn%d.portsxy" % (prefix, chn), dtype=_LE).reshape(-1, 2).astype(np.float32)


def write_rbg(path, rbg):
    """rbg [colours][H + 8][W + 8] as GPUTileProcessor.getRBG returns it."""
    np.asarray(rbg, np.float64).astype(_LE).tofile(path)
    return path


def read_rbg(path, width, height, num_colors=3):
    return np.fromfile(path, dtype=_LE).reshape(num_colors, height + 8, width + 8).astype(np.float32)
