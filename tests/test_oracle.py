"""Self-consistency checks of the FP64 oracle (CPU only).

The reference ships no tests or fixtures for this path; its own cross-checks
(DttRad2 GPU-mirror methods, analytic vs finite-difference port derivatives in
AlignmentCorrection.java:2952-2990, GPU/CPU debug dumps) become these
automated checks.
"""
import numpy as np
import pytest

from tileproc import synth


def test_dct_iv_recursive_matches_direct(oracle):
    rng = np.random.default_rng(0)
    for _ in range(20):
        x = rng.standard_normal(8)
        assert np.abs(oracle.dct_iv8(x) - oracle.dctiv_direct(x)).max() < 1e-14


def test_dct_dst_iv_are_involutions(oracle):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(8)
    assert np.abs(oracle.dct_iv8(oracle.dct_iv8(x)) - x).max() < 1e-14
    assert np.abs(oracle.dst_iv8(oracle.dst_iv8(x)) - x).max() < 1e-14
    for mode in range(4):
        t = rng.standard_normal(64)
        y = oracle.dttt_iv(t, mode)
        # second application with the swapped mode undoes the transposed 2D transform
        swapped = ((mode << 1) & 2) | ((mode >> 1) & 1)
        assert np.abs(oracle.dttt_iv(y, swapped) - t).max() < 1e-13


def test_dst_iie_identity_used_by_gpu(oracle):
    """SIIe[j][k] = (-1)^k CIIe[7-j][k]: the GPU computes DST-IIe with the DCT-IIe matrix."""
    C = np.array([[np.sqrt(2 / 8) * np.cos(j * (2 * k + 1) * np.pi / 16) for k in range(8)] for j in range(8)])
    S = np.array([[np.sqrt(2 / 8) * np.sin((j + 1) * (2 * k + 1) * np.pi / 16) for k in range(8)] for j in range(8)])
    alt = np.array([(-1) ** k for k in range(8)])
    assert np.abs(S - (C[::-1, :] * alt[None, :])).max() < 1e-15


def test_mclt_perfect_reconstruction(oracle):
    """Forward MCLT of every tile + IMCLT overlap-add (x0.25) reproduces the image (Princen-Bradley)."""
    rng = np.random.default_rng(3)
    H, W = 64, 80
    img = rng.standard_normal((H, W))
    frame = np.zeros((H + 8, W + 8))
    for ty in range(H // 8):
        for tx in range(W // 8):
            clt, res, tl, _ = oracle.extract_correct_tile(img, tx * 8 + 4, ty * 8 + 4)
            assert tuple(tl) == (tx * 8 - 4, ty * 8 - 4) and np.all(res == 0)
            oracle.iclt_tile_add(clt, 0.25, tx, ty, frame)
    inner = frame[4:-4, 4:-4]
    assert np.abs(inner[8:-8, 8:-8] - img[8:-8, 8:-8]).max() < 1e-12


def test_fract_shift_is_a_rotation(oracle):
    rng = np.random.default_rng(4)
    c = rng.standard_normal((4, 64))
    s = oracle.fract_shift(c, 0.37, -0.21)
    assert abs(np.sum(s ** 2) - np.sum(c ** 2)) < 1e-12 * np.sum(c ** 2)
    back = oracle.fract_shift(s, -0.37, 0.21)
    assert np.abs(back - c).max() < 1e-13
    assert np.abs(oracle.fract_shift(c, 0.0, 0.0) - c).max() == 0


def test_fract_shift_moves_the_image(oracle):
    """A smooth image extracted at a fractional centre equals the integer-centre tile
    shifted in the CLT domain (the decomposition extract_correct_tile relies on)."""
    H = W = 64
    yy, xx = np.mgrid[0:H, 0:W]
    f = lambda x, y: np.sin(0.21 * x + 0.1) * np.cos(0.17 * y - 0.3) + 0.3 * np.sin(0.11 * (x + y))
    img = f(xx, yy)
    dx, dy = 0.3, -0.2
    frame = np.zeros((H + 8, W + 8))
    for ty in range(H // 8):
        for tx in range(W // 8):
            clt, res, tl, _ = oracle.extract_correct_tile(img, tx * 8 + 4 + dx, ty * 8 + 4 + dy)
            oracle.iclt_tile_add(oracle.fract_shift(clt, res[0], res[1]), 0.25, tx, ty, frame)
    got = frame[4:-4, 4:-4][12:-12, 12:-12]
    want = f(xx + dx, yy + dy)[12:-12, 12:-12]
    assert np.abs(got - want).max() < 0.02 * np.abs(want).max()


def test_convolve_identity_kernel(oracle):
    rng = np.random.default_rng(5)
    c = rng.standard_normal((4, 64))
    k = np.zeros((4, 64))
    k[0] = 1.0
    assert np.abs(oracle.convolve_tile(c, k) - c).max() == 0


def test_port_derivatives_match_finite_differences(oracle):
    """Analytic d(port)/d(azimuth, tilt, roll, zoom) vs central differences
    (the reference's own check, AlignmentCorrection.java:2952-2990)."""
    rng = np.random.default_rng(6)
    g = synth.circle_geometry(16, 640, 512, rng=rng, sigma=3e-3)
    g["distortion"] = [0.02, -0.01, 0.005, 0.0, 0.0, 0.0, 0.0]
    keys = ("azimuth", "tilt", "roll", "zoom")
    for _ in range(5):
        px, py, d = rng.uniform(50, 590), rng.uniform(50, 460), rng.uniform(0, 4)
        p0, dv = oracle.ports(g, px, py, d, deriv=True)
        for k, key in enumerate(keys):
            for s in (0, 5, 11):
                h = 1e-6
                gp = {kk: (list(vv) if isinstance(vv, list) else vv) for kk, vv in g.items()}
                gm = {kk: (list(vv) if isinstance(vv, list) else vv) for kk, vv in g.items()}
                gp[key][s] += h
                gm[key][s] -= h
                fd = (oracle.ports(gp, px, py, d)[s] - oracle.ports(gm, px, py, d)[s]) / (2 * h)
                an = dv[s, :, k]
                if key == "roll":
                    # the reference drops the radial-distortion term of d/droll (GeometryCorrection.java:2279-2280)
                    assert np.abs(an - fd).max() < 2e-2 * max(1.0, np.abs(fd).max())
                else:
                    assert np.abs(an - fd).max() < 1e-5 * max(1.0, np.abs(fd).max()), (key, s, an, fd)


def test_general_strip_reduces_to_reference(oracle):
    """The generalised (kind 4) strip sampler visits the reference's sample points for the quad directions."""
    rng = np.random.default_rng(7)
    corr = rng.standard_normal(225)
    for kind, b in ((0, (1, 0)), (1, (0, 1)), (2, (1, 1)), (3, (1, -1))):
        a = oracle.strip(corr, b[0], b[1], kind, 9)
        g = oracle.strip(corr, b[0], b[1], 4, 9)
        both = np.isfinite(a) & np.isfinite(g)
        assert np.array_equal(np.isnan(a), np.isnan(g)), kind
        assert np.abs(a[both] - g[both]).max() < 1e-14, kind


def test_constant_disparity_recovered(oracle):
    """Residual disparity sign and accuracy on constant-disparity synthetic scenes."""
    from helpers import run_oracle
    for gt, target in ((4.0, 4.0), (4.6, 4.0)):
        sc = synth.make_scene("quad_mono", seed=2, width=192, height=160, dmin=gt, dmax=gt)
        r = run_oracle(oracle, sc, target)
        d = r["disp"].reshape(20, 24, -1)[2:-2, 2:-2, oracle.DISP_CM]
        med = np.nanmedian(d)
        assert abs(med - (gt - target)) < 0.05 + 0.2 * abs(gt - target), med
        assert np.sign(med) == np.sign(gt - target) or gt == target


def test_kernel_chain_symmetric_kernel(oracle):
    """A centred symmetric PSF yields (near) zero antisymmetric CLT parts and zero centre offsets."""
    yy, xx = np.mgrid[-32:32, -32:32]
    src = np.exp(-(xx ** 2 + yy ** 2) / (2 * 2.0 ** 2))
    clt, ext = oracle.calc_clt_kernel(src)
    assert np.abs(clt[1:]).max() < 1e-12 * np.abs(clt[0]).max()
    assert np.abs(ext[:4]).max() < 1e-12
    # normalisation: kernel * window sums to 16 -> DC of the DCT-IIIe kernel
    assert np.isfinite(clt).all()


def test_fill_coord_corr_linear_field(oracle):
    kv, kh = 6, 7
    ext = np.zeros((kv, kh, 8))
    yy, xx = np.mgrid[0:kv, 0:kh]
    ext[..., 2] = 0.3 * xx - 0.1 * yy
    ext[..., 3] = 0.05 * xx + 0.2 * yy
    oracle.fill_coord_corr(ext, 16)
    assert np.allclose(ext[..., 4], 0.3 / 16) and np.allclose(ext[..., 5], -0.1 / 16)
    assert np.allclose(ext[..., 6], 0.05 / 16) and np.allclose(ext[..., 7], 0.2 / 16)


def _iclt_tile(oracle, clt4x64, lpf):
    """Full 16x16 IMCLT of one sub-tile (x0.25 x LPF), the texture branch's per-port tile."""
    out = np.zeros(256)
    for m in range(4):
        t = np.asarray(clt4x64[m]) * (0.25 * lpf)
        idct = ((m << 1) & 2) | ((m >> 1) & 1)
        out += oracle.unfold_tile(oracle.dttt_iv(t, idct), m)
    return out


def test_texture_identical_ports(oracle):
    """Identical ports: every port weight 1, alpha = window^2, RGB = the port's IMCLT tile, rms 0."""
    rng = np.random.default_rng(5)
    one = rng.normal(size=(3, 4, 64)) * 40.0
    clt = np.broadcast_to(one, (4, 3, 4, 64)).copy()
    lpf = oracle.corr_lpf(0.8)
    rgba, aux = oracle.texture_tile(clt, lpf)
    w2 = oracle.win2d() ** 2
    assert np.allclose(rgba[4:8], 1.0)
    assert np.allclose(rgba[3], w2)
    for c in range(3):
        assert np.allclose(rgba[c], _iclt_tile(oracle, one[c], lpf), rtol=1e-12, atol=1e-9)
    assert np.all(np.abs(rgba[8:12]) < 1e-6) or np.isnan(rgba[8:12]).any()
    assert np.allclose(aux[:4], 0.0)


def test_texture_single_port_and_forced(oracle):
    """One used port: its weight is 1, the others 0, RGB = that port's tile (tile_combine_rgba 2942-2950)."""
    rng = np.random.default_rng(6)
    clt = rng.normal(size=(4, 3, 4, 64)) * 30.0
    lpf = oracle.corr_lpf(0.8)
    rgba, _ = oracle.texture_tile(clt, lpf, img_mask=0x4)
    assert np.allclose(rgba[6], 1.0) and np.allclose(rgba[[4, 5, 7]], 0.0)
    for c in range(3):
        assert np.allclose(rgba[c], _iclt_tile(oracle, clt[2, c], lpf), rtol=1e-12, atol=1e-9)
    # the extra shift moves every port by disparity x port offset / corr_magic_scale
    shifted, _ = oracle.texture_tile(clt, lpf, img_mask=0x4, extra_disparity=0.85)
    c2 = clt[2].copy()
    for c in range(3):
        c2[c] = oracle.fract_shift(c2[c], -0.5, 0.5)
    for c in range(3):
        assert np.allclose(shifted[c], _iclt_tile(oracle, c2[c], lpf), rtol=1e-12, atol=1e-9)


def test_texture_outlier_port_is_suppressed(oracle):
    """A port that disagrees with the other three gets a small weight; dust_remove keeps the sum."""
    rng = np.random.default_rng(8)
    one = rng.normal(size=(3, 4, 64)) * 40.0
    clt = np.broadcast_to(one, (4, 3, 4, 64)).copy()
    clt[1] += rng.normal(size=(3, 4, 64)) * 400.0
    rgba, _ = oracle.texture_tile(clt, oracle.corr_lpf(0.8))
    centre = np.zeros((16, 16), bool)
    centre[4:12, 4:12] = True
    w = rgba[4:8].reshape(4, 16, 16)[:, centre]
    assert np.median(w[1]) < 0.2 and np.median(w[0]) > 0.9


def _rig(**kw):
    r = dict(main_disparity_radius=20.0, aux_disparity_radius=20.0, baseline=0.0, aux_angle=0.0, aux_azimuth=0.0,
             aux_tilt=0.0, aux_roll=0.0, aux_zoom=0.0)
    r.update(kw)
    return r


def test_rig_ports_reduce_to_the_camera_ports(oracle):
    """RigOffset with no offset, no rotation and equal radii: the auxiliary ports are the camera's own."""
    g = synth.make_scene("quad_mono", seed=3, width=128, height=96)["geometry"]
    for px, py, d in ((20.0, 12.0, 0.5), (100.0, 76.0, 3.25)):
        assert np.array_equal(oracle.rig_aux_ports(g, g, _rig(), px, py, d), oracle.ports(g, px, py, d))


def test_rig_baseline_is_a_lens_offset_at_the_scaled_disparity(oracle):
    """A pure baseline (recalcRXY): rXY_aux = rXY + baseline (cos, sin)(angle) / aux radius, and the main
    camera's disparity is scaled by aux / main radius (ImageDtt.java:8973)."""
    g = synth.make_scene("quad_mono", seed=3, width=128, height=96)["geometry"]
    rig = _rig(main_disparity_radius=25.0, aux_disparity_radius=20.0, baseline=8.0, aux_angle=0.6)
    shifted = dict(g)
    off = np.array([8.0 * np.cos(0.6), 8.0 * np.sin(0.6)]) / 20.0
    shifted["rXY"] = np.asarray(g["rXY"], np.float64) + off
    got = oracle.rig_aux_ports(g, g, rig, 64.0, 40.0, 2.0)
    want = oracle.ports(shifted, 64.0, 40.0, 2.0 * 20.0 / 25.0)
    assert np.allclose(got, want, atol=1e-12)
    rxy = oracle.rig_rxy(g, rig)
    assert np.allclose(rxy, shifted["rXY"], atol=1e-15)


def test_rig_roll_rotates_the_lens_offsets(oracle):
    g = synth.make_scene("quad_mono", seed=3, width=128, height=96)["geometry"]
    a = 0.3
    rxy = oracle.rig_rxy(g, _rig(aux_roll=a))
    r = np.asarray(g["rXY"], np.float64)
    want = np.stack([np.cos(a) * r[:, 0] + np.sin(a) * r[:, 1], -np.sin(a) * r[:, 0] + np.cos(a) * r[:, 1]], -1)
    assert np.allclose(rxy, want, atol=1e-15)
