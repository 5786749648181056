"""Generate golden vectors by running the reference's own CUDA kernels.

Run on a GPU machine after `python oracle/build_ref_gpu.py` has produced
oracle/_ref/tp_ref_128x96.cubin on a machine that has the reference sources:

    python tests/golden/make_ref_gpu_golden.py OUT.npz

Scene: 4 Bayer sensors 128x96 (GR/BG), green scaled by 0.5 in the mosaic as
QuadCLT does before GPUTileProcessor.setBayerImages, per-sensor/colour CLT
kernels on the 16-px grid (10x8) with CltExtra offsets, and a task list of
interior tiles with fractional ports (the reference GPU kernel clamps borders
with swapped width/height, so border windows are avoided).  Ports are chosen
so that no window corner or kernel index sits within 2e-3 of a rounding tie
(the reference GPU rounds with floorf(x+0.5f)/lrintf in FP32, the CPU path
with Math.round in FP64).  Saved: the inputs, the reference GPU CLT of the
tasked tiles and the reference imclt_rbg frames (lpf_mask = 0).

    python tests/golden/make_ref_gpu_golden.py OUT.npz --lpf

writes the same inputs with the CLT of lpf_mask = 7, the mask GPUTileProcessor.
execConverCorrectTiles passes (GPUTileProcessor.java:547): each colour's stored
CLT multiplied by the module's lpf_data table (TileProcessor.cuh:1037-1061),
which is saved too.

    python tests/golden/make_ref_gpu_golden.py OUT.npz --dtt

runs the reference's transform test kernel GPU_DTT24_DRV (dtt8x8.cuh:100-158) on a seeded 64x32
image in its eight modes (DCT-IV / DST-IV and DCT-II / DST-II, rows then columns).
"""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "imagej-elphel_gb300"))

W, H = 128, 96
KH, KV = W // 16 + 2, H // 16 + 2


def java_round(x):
    f = np.floor(x)
    return np.where(x - f >= 0.5, f + 1, f)


def make_inputs(seed=2024):
    from tileproc import synth
    rng = np.random.default_rng(seed)
    sc = synth.make_scene("quad_bayer", seed=seed, width=W, height=H)
    scale = np.where(sc["color_index"] == 2, 0.5, 1.0)
    mosaics = (sc["images"].astype(np.float64) * scale[None]).astype(np.float32)
    k, e = synth.random_clt_kernels(rng, 4, KV, KH, 3)
    k = k.astype(np.float16).astype(np.float32)  # compact storage, exact in f32
    tx_all, ty_all = np.meshgrid(np.arange(2, W // 8 - 2), np.arange(2, H // 8 - 2))
    sel = rng.choice(tx_all.size, size=40, replace=False)
    txs, tys = tx_all.ravel()[sel], ty_all.ravel()[sel]
    xy = np.zeros((len(sel), 4, 2), np.float32)
    for n in range(len(sel)):
        for cam in range(4):
            while True:
                p = np.array([txs[n] * 8 + 4, tys[n] * 8 + 4]) + rng.uniform(-3, 3, 2)
                p = p.astype(np.float32).astype(np.float64)
                q = p / 16.0
                if np.any(np.abs(q - np.floor(q) - 0.5) < 2e-3):
                    continue
                kt = np.clip(java_round(q) + 1, 0, [KH - 1, KV - 1]).astype(int)
                ok = True
                for c in range(3):
                    ce = e[cam, kt[1], kt[0], c].astype(np.float64)
                    kd = p - (kt - 1 + 0.5) * 16
                    px = p[0] - 8 - (ce[0] + ce[4] * kd[0] + ce[5] * kd[1])
                    py = p[1] - 8 - (ce[1] + ce[6] * kd[0] + ce[7] * kd[1])
                    for v in (px, py):
                        if abs(v - np.floor(v) - 0.5) < 2e-3:
                            ok = False
                if ok:
                    xy[n, cam] = p
                    break
    from tileproc import GPUTileProcessor
    tasks = GPUTileProcessor.packTasks(np.ones(len(sel)), txs, tys, xy)
    return dict(mosaic_u16=sc["images"], color_index=sc["color_index"], mosaics=mosaics, kernels=k, kext=e,
                tasks=tasks, tx=txs, ty=tys, xy=xy)


def main_dtt(out):
    """GPU_DTT24_DRV, the reference's transform test kernel (dtt8x8.cuh:100-158), on a seeded
    64x32 image in all eight modes"""
    from oracle import build_ref_gpu
    from oracle.ref_gpu import RefGpu
    rng = np.random.default_rng(77)
    yy, xx = np.mgrid[0:32, 0:64]
    img = (rng.normal(size=(32, 64)) + np.sin(xx / 3.0) * np.cos(yy / 5.0) + 0.01 * xx).astype(np.float32)
    ref = RefGpu(build_ref_gpu.cubin_path(W, H), W, H)
    outs = np.stack([ref.dtt24(img, m) for m in range(8)])
    np.savez_compressed(out, src=img, ref_dtt=outs,
                        note="reference GPU_DTT24_DRV (dtt8x8.cuh) compiled for sm_103a, modes 0-7")
    print("wrote", out, "absmax", np.abs(outs).max())


def main(out, lpf=False):
    from oracle import build_ref_gpu
    from oracle.ref_gpu import RefGpu
    inp = make_inputs()
    # setConvolutionKernels uploads each 8x8 quadrant transposed (GPUTileProcessor.java:406-410)
    kg = inp["kernels"].reshape(4, KV, KH, 3, 4, 8, 8).swapaxes(-1, -2).reshape(4, KV, KH, 3, 4, 64)
    ref = RefGpu(build_ref_gpu.cubin_path(W, H), W, H)
    if lpf:
        clt, rbg = ref.run(inp["mosaics"], kg, inp["kext"], inp["tasks"], lpf_mask=7)
        ref_clt = clt[:, inp["ty"], inp["tx"]]
        np.savez_compressed(out, mosaic_u16=inp["mosaic_u16"], kernels_f16=inp["kernels"].astype(np.float16),
                            kext=inp["kext"], tasks=inp["tasks"], ref_clt=np.ascontiguousarray(ref_clt.swapaxes(0, 1)),
                            lpf_data=ref.get_global("lpf_data", 3 * 64).reshape(3, 64), width=W, height=H,
                            bayer=np.array([0, 1]), lpf_mask=7,
                            note="reference convert_correct_tiles (TileProcessor.cuh) compiled for sm_103a, lpf_mask 7")
        print("wrote", out, "tasks", len(inp["tx"]), "clt absmax", np.abs(ref_clt).max())
        return
    clt, rbg = ref.run(inp["mosaics"], kg, inp["kext"], inp["tasks"])
    ref_clt = clt[:, inp["ty"], inp["tx"]]  # [4][n][3][4][64]
    np.savez_compressed(out, mosaic_u16=inp["mosaic_u16"], kernels_f16=inp["kernels"].astype(np.float16),
                        kext=inp["kext"], tasks=inp["tasks"], ref_clt=np.ascontiguousarray(ref_clt.swapaxes(0, 1)),
                        ref_rbg=rbg, width=W, height=H, bayer=np.array([0, 1]), lpf_mask=0,
                        note="reference convert_correct_tiles/imclt_rbg (TileProcessor.cuh) compiled for sm_103a")
    print("wrote", out, "tasks", len(inp["tx"]), "clt absmax", np.abs(ref_clt).max(), "rbg absmax", np.abs(rbg).max())


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--dtt" in sys.argv:
        main_dtt(args[0] if args else "ref_gpu_dtt24.npz")
    else:
        main(args[0] if args else "ref_gpu_128x96.npz", lpf="--lpf" in sys.argv)
