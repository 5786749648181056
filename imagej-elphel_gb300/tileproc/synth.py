"""Seeded synthetic multi-sensor scenes for the tile processor.

The reference ships no sample data for this path, so inputs are generated:
  * quad_mono   -- 4 mono sensors (square quad, rXY = (+-0.5, +-0.5)), base image
                   = Gaussian-lowpassed noise (sigma 1.5 px, unit variance) plus
                   random axis-aligned rectangles of amplitude 0.5 covering ~10 %
                   of the frame; per-8x8-block disparity U[dmin, dmax].
  * quad_bayer  -- the same generator per colour plane (correlated R, G, B),
                   mosaicked (GR/BG by default) and quantised to 12-bit uint16.
  * circle_lwir -- 16 sensors on a circle with per-sensor extrinsic perturbations;
                   thermal-like 1/f^2 field plus N(0, 0.02) noise.
Each sensor image samples the base scene at the point the lens model maps to
that pixel for the block's disparity (inverse of the port model, solved by
fixed-point iteration), with cubic-spline interpolation.
"""
import numpy as np
from scipy import ndimage

QUAD_RXY = np.array([[-0.5, -0.5], [0.5, -0.5], [-0.5, 0.5], [0.5, 0.5]])


def quad_geometry(width, height, focal_length=4.5, pixel_size=2.2, distortion=None, extrinsics=None):
    g = {"num_sensors": 4, "width": width, "height": height, "focal_length": focal_length,
         "pixel_size": pixel_size, "distortion_radius": 2.8512,
         "distortion": list(distortion) if distortion is not None else [0.0] * 7,
         "rXY": QUAD_RXY.tolist(), "pXY0": [[width / 2.0, height / 2.0]] * 4,
         "azimuth": [0.0] * 4, "tilt": [0.0] * 4, "roll": [0.0] * 4, "zoom": [0.0] * 4}
    if extrinsics is not None:
        for k in ("azimuth", "tilt", "roll", "zoom"):
            g[k] = list(map(float, extrinsics[k]))
    return g


def circle_geometry(num_sensors=16, width=640, height=512, radius_mm=100.0, focal_length=4.9, pixel_size=12.0,
                    rng=None, sigma=1e-3):
    ang = 2 * np.pi * np.arange(num_sensors) / num_sensors
    # disparity normalised like the quad: disparityRadius = sqrt(2) * cameraRadius
    rxy = np.stack([np.cos(ang), np.sin(ang)], axis=1) / np.sqrt(2.0)
    g = {"num_sensors": num_sensors, "width": width, "height": height, "focal_length": focal_length,
         "pixel_size": pixel_size, "distortion_radius": 2.8512, "distortion": [0.0] * 7,
         "rXY": rxy.tolist(), "pXY0": [[width / 2.0, height / 2.0]] * num_sensors,
         "azimuth": [0.0] * num_sensors, "tilt": [0.0] * num_sensors, "roll": [0.0] * num_sensors,
         "zoom": [0.0] * num_sensors, "radius_mm": radius_mm}
    if rng is not None:
        for k in ("azimuth", "tilt", "roll", "zoom"):
            g[k] = (rng.standard_normal(num_sensors) * sigma).tolist()
    return g


def circle_pairs(geom):
    """All sensor pairs, strip direction b = rXY[cam2] - rXY[cam1] (kind 4)."""
    rxy = np.asarray(geom["rXY"])
    S = len(rxy)
    pairs = []
    for a in range(S):
        for b in range(a + 1, S):
            d = rxy[b] - rxy[a]
            pairs.append((a, b, 4, 1, float(d[0]), float(d[1])))
    return pairs


def _rot(geom, s):
    """CorrVector.getRotMatrices for one sensor (numpy, for rendering only)."""
    ca, sa = np.cos(geom["azimuth"][s]), np.sin(geom["azimuth"][s])
    ct, st = np.cos(geom["tilt"][s]), np.sin(geom["tilt"][s])
    z = 1.0 + geom["zoom"][s]
    cr, sr = np.cos(geom["roll"][s]) * z, np.sin(geom["roll"][s]) * z
    a_az = np.array([[ca, 0, -sa], [0, 1, 0], [sa, 0, ca]])
    a_t = np.array([[1, 0, 0], [0, ct, st], [0, -st, ct]])
    a_r = np.array([[cr, sr, 0], [-sr, cr, 0], [0, 0, 1]])
    return a_r @ (a_t @ a_az)


def port_map(geom, s, qx, qy, d):
    """Distortion-free port model: pixel of sensor s seeing centre-image point (qx, qy) at disparity d."""
    W, H = geom["width"], geom["height"]
    f = geom["focal_length"] / (0.001 * geom["pixel_size"])
    R = _rot(geom, s)
    vx = qx - 0.5 * W - d * geom["rXY"][s][0]
    vy = qy - 0.5 * H - d * geom["rXY"][s][1]
    rx = R[0, 0] * vx + R[0, 1] * vy + R[0, 2] * f
    ry = R[1, 0] * vx + R[1, 1] * vy + R[1, 2] * f
    rz = R[2, 0] * vx + R[2, 1] * vy + R[2, 2] * f
    return rx * f / rz + geom["pXY0"][s][0], ry * f / rz + geom["pXY0"][s][1]


def lowpass_noise(rng, h, w, sigma=1.5):
    f = ndimage.gaussian_filter(rng.standard_normal((h, w)), sigma, mode="wrap")
    return (f - f.mean()) / f.std()


def add_rectangles(rng, img, frac=0.1, amp=0.5, max_side=24):
    h, w = img.shape
    area = 0
    while area < frac * h * w:
        rw, rh = rng.integers(3, max_side, size=2)
        x0, y0 = rng.integers(0, w - rw), rng.integers(0, h - rh)
        img[y0:y0 + rh, x0:x0 + rw] += amp * (1 if rng.random() < 0.5 else -1)
        area += rw * rh
    return img


def thermal_field(rng, h, w):
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    f = np.sqrt(fx * fx + fy * fy)
    f[0, 0] = 1.0
    spec = (rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape)) / f
    spec[0, 0] = 0
    img = np.fft.irfft2(spec, s=(h, w))
    return (img - img.mean()) / img.std()


def block_disparity(rng, tiles_y, tiles_x, dmin, dmax):
    return rng.uniform(dmin, dmax, size=(tiles_y, tiles_x))


def _render(base, margin, geom, s, disp_blocks, xs, ys, iters=3):
    """Sample `base` (with `margin` px border) at the centre-image point seen by
    pixels (xs, ys) of sensor s, disparity piecewise constant on 8x8 blocks."""
    H, W = geom["height"], geom["width"]
    qx, qy = xs.astype(np.float64), ys.astype(np.float64)
    for _ in range(iters):
        bx = np.clip((qx // 8).astype(np.int64), 0, W // 8 - 1)
        by = np.clip((qy // 8).astype(np.int64), 0, H // 8 - 1)
        d = disp_blocks[by, bx]
        px, py = port_map(geom, s, qx, qy, d)
        qx = qx + (xs - px)
        qy = qy + (ys - py)
    return ndimage.map_coordinates(base, [qy + margin, qx + margin], order=3, mode="mirror")


def make_scene(kind, seed=1, width=None, height=None, dmin=0.0, dmax=8.0, noise=0.01,
               bayer_red_row=0, bayer_red_col=1):
    """Returns dict: images [S][H][W] (float32 mono or uint16 mosaic), geometry,
    disparity_gt [tilesY][tilesX], num_colors, and for Bayer the colour planes."""
    rng = np.random.default_rng(seed)
    if kind == "quad_mono":
        W, H = width or 512, height or 384
        geom = quad_geometry(W, H)
    elif kind == "quad_bayer":
        W, H = width or 2592, height or 1936
        geom = quad_geometry(W, H)
    elif kind == "circle_lwir":
        W, H = width or 640, height or 512
        geom = circle_geometry(16, W, H, rng=rng)
        if dmax == 8.0:
            dmax = 4.0
    else:
        raise ValueError(kind)
    S = geom["num_sensors"]
    tx, ty = W // 8, H // 8
    dgt = block_disparity(rng, ty, tx, dmin, dmax)
    margin = 32
    ys, xs = np.mgrid[0:H, 0:W]
    out = {"geometry": geom, "disparity_gt": dgt, "width": W, "height": H, "kind": kind, "seed": seed}
    if kind == "quad_mono":
        base = add_rectangles(rng, lowpass_noise(rng, H + 2 * margin, W + 2 * margin))
        imgs = np.zeros((S, H, W), dtype=np.float32)
        for s in range(S):
            v = _render(base, margin, geom, s, dgt, xs.ravel(), ys.ravel()).reshape(H, W)
            imgs[s] = (v + noise * rng.standard_normal((H, W))).astype(np.float32)
        out.update(images=imgs, num_colors=1)
    elif kind == "circle_lwir":
        base = thermal_field(rng, H + 2 * margin, W + 2 * margin)
        imgs = np.zeros((S, H, W), dtype=np.float32)
        for s in range(S):
            v = _render(base, margin, geom, s, dgt, xs.ravel(), ys.ravel()).reshape(H, W)
            imgs[s] = (v + 0.02 * rng.standard_normal((H, W))).astype(np.float32)
        out.update(images=imgs, num_colors=1)
    else:  # Bayer mosaic, colour planes correlated through a shared luminance
        lum = add_rectangles(rng, lowpass_noise(rng, H + 2 * margin, W + 2 * margin))
        planes = [lum + 0.3 * lowpass_noise(rng, H + 2 * margin, W + 2 * margin, 3.0),   # R
                  lum + 0.3 * lowpass_noise(rng, H + 2 * margin, W + 2 * margin, 3.0),   # B
                  lum]                                                                     # G
        xo = (xs & 1) == bayer_red_col
        yo = (ys & 1) == bayer_red_row
        col = np.where(xo & yo, 0, np.where(~xo & ~yo, 1, 2))
        imgs = np.zeros((S, H, W), dtype=np.uint16)
        for s in range(S):
            mosaic = np.zeros((H, W))
            for c in range(3):
                sel = col == c
                mosaic[sel] = _render(planes[c], margin, geom, s, dgt, xs[sel], ys[sel])
            mosaic += noise * rng.standard_normal((H, W))
            imgs[s] = np.clip(np.rint(2048 + 400 * mosaic), 0, 4095).astype(np.uint16)
        out.update(images=imgs, num_colors=3, bayer=(bayer_red_row, bayer_red_col), color_index=col)
    return out


def bayer_planes(mosaic, color_index, scales=(1.0, 1.0, 0.5)):
    """Sparse R, B, G planes of a mosaic (EyesisCorrections.bayerToDoubleStack with
    QuadCLT's green x0.5), float64 [3][H][W]."""
    m = mosaic.astype(np.float64)
    return np.stack([np.where(color_index == c, m * scales[c], 0.0) for c in range(3)])


def psf_kernels(rng, kv, kh, num_colors, sigma=(0.6, 1.4), offset=0.3):
    """Double-resolution (64x64, 0.5-px pitch) elliptical Gaussian PSFs for one sensor:
    [kv][kh][C][64][64] float32, sigma per axis uniform in `sigma` px, random orientation,
    centre offset uniform in +-`offset` px -- the input of QuadCLT.calculateCLTKernel."""
    n = kv * kh * num_colors
    sx = rng.uniform(*sigma, n) * 2.0
    sy = rng.uniform(*sigma, n) * 2.0
    th = rng.uniform(0, np.pi, n)
    cx = 32.0 + rng.uniform(-offset, offset, n) * 2.0
    cy = 32.0 + rng.uniform(-offset, offset, n) * 2.0
    yy, xx = np.mgrid[0:64, 0:64].astype(np.float64)
    out = np.empty((n, 64, 64), np.float32)
    for k in range(n):
        dx, dy = xx - cx[k], yy - cy[k]
        c, s_ = np.cos(th[k]), np.sin(th[k])
        u, v = c * dx + s_ * dy, -s_ * dx + c * dy
        g = np.exp(-0.5 * ((u / sx[k]) ** 2 + (v / sy[k]) ** 2))
        out[k] = (g / g.sum()).astype(np.float32)
    return out.reshape(kv, kh, num_colors, 64, 64)


def random_clt_kernels(rng, num_sensors, kv, kh, num_colors, strength=0.2, offset=0.5, grad=0.01):
    """Random CLT-domain kernel table ([S][kv][kh][C][4][64], CPU orientation) and
    CltExtra records ([S][kv][kh][C][8]) for exercising the aberration path."""
    k = strength * rng.standard_normal((num_sensors, kv, kh, num_colors, 4, 64))
    k[..., 0, :] += 1.0
    e = np.zeros((num_sensors, kv, kh, num_colors, 8))
    e[..., 0:2] = rng.uniform(-offset, offset, size=e[..., 0:2].shape)
    e[..., 2:4] = e[..., 0:2] + rng.uniform(-0.1, 0.1, size=e[..., 2:4].shape)
    e[..., 4:8] = rng.uniform(-grad, grad, size=e[..., 4:8].shape)
    return k.astype(np.float32), e.astype(np.float32)
