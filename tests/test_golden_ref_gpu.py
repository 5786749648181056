"""Pin the oracle (CPU) and the GB300 path (GPU) to the reference's own CUDA kernels.

tests/golden/ref_gpu_128x96.npz holds the inputs and outputs of the reference
convert_correct_tiles / imclt_rbg kernels (TileProcessor.cuh), compiled from the
reference sources for sm_103a and run on a GB300 by
tests/golden/make_ref_gpu_golden.py.  Known, documented differences of that
kernel from the FP64 CPU path, and how the comparison handles them:
  * FP32 arithmetic with constants truncated to 6 significant digits
    (TileProcessor.cuh:240-244, dtt8x8.cuh:76-84): relative error floor
    ~1e-6, so the tolerance here is 5e-5 relative L2 per sub-tile;
  * rounding ties (floorf(x+0.5f) / lrintf vs Math.round): the golden task list
    keeps every corner and kernel index >= 2e-3 away from a tie;
  * CLT is stored with each 8x8 quadrant transposed relative to ImageDtt;
  * imclt_rbg folds the 0.25 of ImageDtt.iclt_2d into its half-amplitude
    window table HWINDOW2 and overwrites tile (0,0) with 100.0
    (TileProcessor.cuh:1259-1272): compared outside that 16x16 block.
"""
import os

import numpy as np
import pytest

from tileproc import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_128x96.npz")
TOL = 5e-5


def _load():
    if not os.path.exists(GOLD):
        pytest.skip("golden file not generated")
    g = dict(np.load(GOLD))
    W, H = int(g["width"]), int(g["height"])
    xo = (np.arange(W)[None, :] & 1) == 1
    yo = (np.arange(H)[:, None] & 1) == 0
    g["color_index"] = np.where(xo & yo, 0, np.where(~xo & ~yo, 1, 2))
    tasks = g["tasks"]
    txy = tasks[:, 1].view(np.int32)
    g["tx"], g["ty"] = txy & 0xFFFF, txy >> 16
    g["xy"] = tasks[:, 2:].reshape(-1, 4, 2).astype(np.float64)
    g["kernels"] = g["kernels_f16"].astype(np.float32)
    return g, W, H


def _oracle_clt(O, g, W, H):
    planes = np.stack([synth.bayer_planes(m, g["color_index"]) for m in g["mosaic_u16"]])
    n = len(g["tx"])
    out = np.zeros((n, 4, 3, 4, 64))
    kern = g["kernels"].astype(np.float64)
    kext = g["kext"].astype(np.float64)
    for t in range(n):
        for cam in range(4):
            for c in range(3):
                clt, res, tl, kt = O.extract_correct_tile(planes[cam, c], g["xy"][t, cam, 0], g["xy"][t, cam, 1],
                                                          kern=kern[cam, :, :, c], kext=kext[cam, :, :, c])
                out[t, cam, c] = O.fract_shift(clt, res[0], res[1])
    return out


def _ref_clt_cpu_orientation(g):
    r = g["ref_clt"].astype(np.float64)  # [n][4][3][4][64], quadrants transposed
    return r.reshape(r.shape[:-1] + (8, 8)).swapaxes(-1, -2).reshape(r.shape)


def test_oracle_matches_reference_gpu_clt(oracle):
    g, W, H = _load()
    want = _oracle_clt(oracle, g, W, H)
    got = _ref_clt_cpu_orientation(g)
    e = np.sqrt(((got - want) ** 2).sum((-2, -1)) / (want ** 2).sum((-2, -1)))
    assert e.max() < TOL, "reference GPU vs oracle CLT rel L2 max %.3g median %.3g" % (e.max(), np.median(e))


def test_oracle_matches_reference_gpu_imclt(oracle):
    g, W, H = _load()
    tX, tY = W // 8, H // 8
    clt = np.zeros((tX * tY, 4, 3, 4, 64))
    tiles = g["ty"] * tX + g["tx"]
    clt[tiles] = _ref_clt_cpu_orientation(g)
    want = oracle.imclt_frames(clt, tX, tY, scale=0.25)
    got = g["ref_rbg"].astype(np.float64)
    mask = np.ones(got.shape[-2:], bool)
    mask[:16, :16] = False
    err = np.abs(got - want)[..., mask].max() / np.abs(want).max()
    assert err < TOL, "reference imclt_rbg vs oracle iclt rel err %.3g" % err


@pytest.mark.gpu
def test_gb300_matches_reference_gpu(oracle, tp_lib):
    """Our kernels on the same inputs (reference task layout, float ports)."""
    g, W, H = _load()
    from tileproc import GPUTileProcessor, _lib
    kv, kh = g["kernels"].shape[1:3]
    with GPUTileProcessor(4, W, H, num_colors=3, kernels_hor=kh, kernels_vert=kv) as tp:
        tp.setColorScales([1.0, 1.0, 0.5])
        tp.setBayerImages(g["mosaic_u16"])
        tp.setConvolutionKernels(g["kernels"], g["kext"], layout=_lib.TP_KERNELS_CPU)
        tp.setTasks(g["tasks"])
        tp.setCorrelation()
        tp.process()
        tp.execImcltRbg()
        clt = tp.getClt()
        tiles = g["ty"] * (W // 8) + g["tx"]
        got = clt[tiles].astype(np.float64)
        ref = _ref_clt_cpu_orientation(g)
        e = np.sqrt(((got - ref) ** 2).sum((-2, -1)) / (ref ** 2).sum((-2, -1)))
        assert e.max() < TOL, "GB300 vs reference GPU CLT rel L2 max %.3g" % e.max()
        mask = np.ones((H + 8, W + 8), bool)
        mask[:16, :16] = False
        for cam in range(4):
            rbg = tp.getRBG(cam).astype(np.float64)
            ref_rbg = g["ref_rbg"][cam].astype(np.float64)
            err = np.abs(rbg - ref_rbg)[..., mask].max() / np.abs(ref_rbg).max()
            assert err < TOL, "cam %d IMCLT vs reference imclt_rbg rel err %.3g" % (cam, err)


GOLD_LPF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_128x96_lpf.npz")


def test_oracle_matches_reference_gpu_clt_lpf(oracle):
    """The reference convert_correct_tiles with lpf_mask = 7: the oracle's CLT times the module's
    lpf_data table (elementwise; the table is symmetric, so its orientation is the CLT's)."""
    if not os.path.exists(GOLD_LPF):
        pytest.skip("golden file not generated")
    g, W, H = _load()
    gl = dict(np.load(GOLD_LPF))
    lpf = gl["lpf_data"].astype(np.float64)  # [3][64]
    want = _oracle_clt(oracle, g, W, H) * lpf[None, None, :, None, :]
    got = gl["ref_clt"].astype(np.float64)
    got = got.reshape(got.shape[:-1] + (8, 8)).swapaxes(-1, -2).reshape(got.shape)
    e = np.sqrt(((got - want) ** 2).sum((-2, -1)) / (want ** 2).sum((-2, -1)))
    assert e.max() < TOL, "reference GPU low-pass CLT vs oracle rel L2 max %.3g" % e.max()


@pytest.mark.gpu
def test_gb300_lpf_mask_matches_reference_gpu(oracle, tp_lib):
    """The stored CLT with the reference GPU's lpf_mask = 7 (tp_set_clt_lpf_mask) and its lpf_data
    table set through tp_set_lpf, against the reference convert_correct_tiles run with that mask;
    the IMCLT frames do not change (the filter is not applied twice)."""
    if not os.path.exists(GOLD_LPF):
        pytest.skip("golden file not generated")
    g, W, H = _load()
    gl = dict(np.load(GOLD_LPF))
    assert np.array_equal(gl["tasks"], g["tasks"])
    from tileproc import GPUTileProcessor, _lib
    kv, kh = g["kernels"].shape[1:3]
    # the module's table is symmetric in its two frequency indices, so its orientation is the CLT's
    lpf = gl["lpf_data"].astype(np.float32)
    assert np.array_equal(lpf.reshape(3, 8, 8), lpf.reshape(3, 8, 8).swapaxes(-1, -2))
    with GPUTileProcessor(4, W, H, num_colors=3, kernels_hor=kh, kernels_vert=kv) as tp:
        tp.setColorScales([1.0, 1.0, 0.5])
        tp.setBayerImages(g["mosaic_u16"])
        tp.setConvolutionKernels(g["kernels"], g["kext"], layout=_lib.TP_KERNELS_CPU)
        tp.setTasks(g["tasks"])
        tp.setCorrelation()
        tp.setLpfRbg(lpf)
        tp.process()
        tp.execImcltRbg()
        rbg0 = [tp.getRBG(cam) for cam in range(4)]
        corr0 = tp.getCorr()
        tp.setCltLpfMask(7)
        tp.process()
        tp.execImcltRbg()
        tiles = g["ty"] * (W // 8) + g["tx"]
        got = tp.getClt()[tiles].astype(np.float64)
        ref = gl["ref_clt"].astype(np.float64)
        ref = ref.reshape(ref.shape[:-1] + (8, 8)).swapaxes(-1, -2).reshape(ref.shape)
        e = np.sqrt(((got - ref) ** 2).sum((-2, -1)) / (ref ** 2).sum((-2, -1)))
        assert e.max() < TOL, "GB300 vs reference GPU low-pass CLT rel L2 max %.3g" % e.max()
        for cam in range(4):
            assert np.allclose(tp.getRBG(cam), rbg0[cam], rtol=1e-5, atol=1e-5 * np.abs(rbg0[cam]).max())
        assert np.array_equal(tp.getCorr(), corr0)  # the correlation reads the unfiltered CLT
        with pytest.raises(_lib.TpError):
            tp.execTextures()


GOLD_DTT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_dtt24.npz")
DTT_TOL = 1e-5  # relative L2 per 8x8 block: the reference's 6-digit FP32 constants against FP64 / our FP32


def _load_dtt():
    if not os.path.exists(GOLD_DTT):
        pytest.skip("golden file not generated")
    return dict(np.load(GOLD_DTT))


def _block_rel_l2(got, want):
    h, w = want.shape
    g = got.reshape(h // 8, 8, w // 8, 8).swapaxes(1, 2).reshape(-1, 64).astype(np.float64)
    r = want.reshape(h // 8, 8, w // 8, 8).swapaxes(1, 2).reshape(-1, 64).astype(np.float64)
    return np.sqrt(((g - r) ** 2).sum(1) / (r ** 2).sum(1))


def test_oracle_matches_reference_gpu_dtt24(oracle):
    """The oracle's 2D transforms (DttRad2.dct_iv / dst_iv / dct_ii and the GPU's DST-II, rows then
    columns) against the reference GPU_DTT24_DRV in all eight modes."""
    g = _load_dtt()
    for mode in range(8):
        e = _block_rel_l2(oracle.dtt24_image(g["src"], mode), g["ref_dtt"][mode])
        assert e.max() < DTT_TOL, "mode %d: oracle vs reference GPU_DTT24_DRV rel L2 max %.3g" % (mode, e.max())


@pytest.mark.gpu
def test_gb300_dtt8x8_matches_reference_gpu(oracle, tp_lib):
    """tp_dtt8x8 (through the C ABI, device buffers) against the reference GPU_DTT24_DRV and the oracle
    in all eight modes, out of place and in place; sizes that are not multiples of 8 are refused."""
    import ctypes as C
    import torch
    from tileproc import _lib
    L = _lib.load()
    g = _load_dtt()
    src = torch.from_numpy(np.ascontiguousarray(g["src"])).cuda()
    h, w = src.shape
    for mode in range(8):
        dst = torch.zeros_like(src)
        assert L.tp_dtt8x8(C.c_void_p(dst.data_ptr()), C.c_void_p(src.data_ptr()), w, w, h, mode, None) == 0
        torch.cuda.synchronize()
        got = dst.cpu().numpy()
        e = _block_rel_l2(got, g["ref_dtt"][mode])
        assert e.max() < DTT_TOL, "mode %d: GB300 vs reference GPU_DTT24_DRV rel L2 max %.3g" % (mode, e.max())
        e = _block_rel_l2(got, oracle.dtt24_image(g["src"], mode))
        assert e.max() < DTT_TOL, "mode %d: GB300 vs oracle rel L2 max %.3g" % (mode, e.max())
        inplace = src.clone()
        assert L.tp_dtt8x8(C.c_void_p(inplace.data_ptr()), C.c_void_p(inplace.data_ptr()), w, w, h, mode, None) == 0
        torch.cuda.synchronize()
        assert np.array_equal(inplace.cpu().numpy(), got)
    dst = torch.zeros_like(src)
    assert L.tp_dtt8x8(C.c_void_p(dst.data_ptr()), C.c_void_p(src.data_ptr()), w, w - 4, h, 0, None) == _lib.TP_ERR_ARG
    assert L.tp_dtt8x8(C.c_void_p(dst.data_ptr()), C.c_void_p(src.data_ptr()), w, w, h, 8, None) == _lib.TP_ERR_ARG
