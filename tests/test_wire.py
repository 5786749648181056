"""GPU-debug wire formats (tileproc.wire): byte layout (little-endian float32 in the
reference's loop order) and round trips, including the transposed kernel files."""
import numpy as np

from tileproc import wire


def test_kernel_files_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    kv, kh, C = 3, 4, 3
    k = rng.standard_normal((kv, kh, C, 4, 64)).astype(np.float32)
    e = rng.standard_normal((kv, kh, C, 8)).astype(np.float32)
    prefix = str(tmp_path / "main")
    kp, op = wire.write_kernels(prefix, 2, k, e)
    raw = np.fromfile(kp, dtype="<f4")
    # saveFloatKernels order: ty, tx, colour, quadrant, coefficient
    assert raw[((1 * kh + 2) * C + 1) * 256 + 3 * 64 + 17] == k[1, 2, 1, 3, 17]
    k2, e2 = wire.read_kernels(prefix, 2, kv, kh, C)
    assert np.array_equal(k2, k) and np.array_equal(e2, e)
    wire.write_kernels(prefix, 2, k, e, transposed=True)
    rawt = np.fromfile(wire.kernel_paths(prefix, 2, True)[0], dtype="<f4")
    i0 = 17
    assert rawt[((1 * kh + 2) * C + 1) * 256 + 3 * 64 + i0] == k[1, 2, 1, 3, ((i0 & 7) << 3) + (i0 >> 3)]
    k3, _ = wire.read_kernels(prefix, 2, kv, kh, C, transposed=True)
    assert np.array_equal(k3, k)


def test_image_ports_rbg_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    W, H = 32, 24
    mosaic = rng.uniform(0, 4095, (H, W)).astype(np.float32)
    prefix = str(tmp_path / "aux")
    wire.write_bayer(prefix, 1, mosaic)
    assert np.array_equal(wire.read_bayer(prefix, 1, W, H), mosaic)
    ports = rng.uniform(0, 100, (12, 2)).astype(np.float32)
    wire.write_portsxy(prefix, 3, ports)
    assert np.array_equal(wire.read_portsxy(prefix, 3), ports)
    rbg = rng.standard_normal((3, H + 8, W + 8)).astype(np.float32)
    p = wire.write_rbg(str(tmp_path / "x.rbg"), rbg)
    assert np.array_equal(wire.read_rbg(p, W, H), rbg)
    assert np.fromfile(p, dtype="<f4")[(W + 8) * (H + 8) + 5] == rbg[1, 0, 5]
