"""Aberration-kernel preparation on the GPU (tp_calc_kernels) vs the FP64 oracle
restatement of QuadCLT.calculateCLTKernel / ImageDtt.clt_fill_coord_corr on
seeded elliptical Gaussian PSFs.  Tolerances: integer window centre (CltExtra
data_x, data_y) exact; centroid offsets 1e-6 px; CLT kernel relative L2 per
kernel tile 1e-5 (FP32 downscale / DCT-IIIe vs FP64); centre slopes 1e-5
relative to their largest magnitude."""
import numpy as np
import pytest

from helpers import rel_l2
from tileproc import GPUTileProcessor, synth
from tileproc import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("normalize", [True, False])
def test_kernel_preparation_matches_oracle(oracle, normalize):
    rng = np.random.default_rng(17)
    W, H = 96, 64
    kh, kv, C = W // 16 + 2, H // 16 + 2, 3
    psf = synth.psf_kernels(rng, kv, kh, C)
    tp = GPUTileProcessor(4, W, H, num_colors=3, kernels_hor=kh, kernels_vert=kv)
    try:
        tp.calcConvolutionKernels(psf, 1, normalize=normalize, coord_corr=True)
        k, e = tp.getConvolutionKernels(1)
    finally:
        tp.close()
    want_k = np.zeros((kv, kh, C, 4, 64))
    want_e = np.zeros((C, kv, kh, 8))
    for ty in range(kv):
        for tx in range(kh):
            for c in range(C):
                ck, ce = oracle.calc_clt_kernel(psf[ty, tx, c].astype(np.float64), normalize=normalize)
                want_k[ty, tx, c] = ck
                want_e[c, ty, tx] = ce
    for c in range(C):
        oracle.fill_coord_corr(want_e[c], 16)
    want_e = np.moveaxis(want_e, 0, 2)
    assert np.array_equal(e[..., :2], want_e[..., :2].astype(np.float32))
    assert np.abs(e[..., 2:4] - want_e[..., 2:4]).max() <= 1e-6
    err = rel_l2(k.astype(np.float64), want_k, axis=(-2, -1))
    assert err.max() <= 1e-5, "kernel rel L2 max %.3g" % err.max()
    sl = np.abs(e[..., 4:] - want_e[..., 4:]).max() / np.abs(want_e[..., 4:]).max()
    assert sl <= 1e-5, "centre slope error %.3g" % sl


def test_kernel_preparation_from_device_memory(oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(18)
    W, H = 64, 48
    kh, kv = W // 16 + 2, H // 16 + 2
    psf = synth.psf_kernels(rng, kv, kh, 1)
    tp = GPUTileProcessor(4, W, H, num_colors=1, kernels_hor=kh, kernels_vert=kv)
    try:
        tp.calcConvolutionKernels(psf, 0)
        k_host, e_host = tp.getConvolutionKernels(0)
        d = torch.from_numpy(psf).cuda()
        tp.calcConvolutionKernels(None, 2, device_ptr=d.data_ptr())
        tp.synchronize()
        k_dev, e_dev = tp.getConvolutionKernels(2)
    finally:
        tp.close()
    assert np.array_equal(k_host, k_dev) and np.array_equal(e_host, e_dev)


def test_wire_kernel_files_through_both_layouts(tmp_path):
    """A transposed .kernel dump loaded with the GPUTileProcessor layout and the plain dump loaded
    with the ImageDtt layout give the same device table."""
    from tileproc import wire
    rng = np.random.default_rng(19)
    W, H = 64, 48
    kh, kv = W // 16 + 2, H // 16 + 2
    k = rng.standard_normal((kv, kh, 3, 4, 64)).astype(np.float32)
    e = rng.standard_normal((kv, kh, 3, 8)).astype(np.float32)
    prefix = str(tmp_path / "dump")
    wire.write_kernels(prefix, 0, k, e)
    wire.write_kernels(prefix, 0, k, e, transposed=True)
    kt = np.fromfile(wire.kernel_paths(prefix, 0, True)[0], dtype="<f4")
    kc, ec = wire.read_kernels(prefix, 0, kv, kh, 3)
    tp = GPUTileProcessor(4, W, H, num_colors=3, kernels_hor=kh, kernels_vert=kv)
    try:
        tp.setConvolutionKernel(kt, ec, 1, layout=L.TP_KERNELS_GPU)
        tp.setConvolutionKernel(kc, ec, 2, layout=L.TP_KERNELS_CPU)
        a, _ = tp.getConvolutionKernels(1)
        b, _ = tp.getConvolutionKernels(2)
    finally:
        tp.close()
    assert np.array_equal(a, b) and np.array_equal(b, k)
