"""Benchmark of the GB300 tile processor (one JSON line on rank 0).

Workload (default): 4 Bayer sensors 2592x1936 uint16 (12-bit), per-sensor /
per-colour CLT kernel tables on a 16-px grid (164x123), all 78,408 tiles:
stage 1 ports (FP64) -> stage 2 convert+correct -> 6-pair correlation ->
disparity extraction -> IMCLT colour frames -> RGBA texture tiles (with the
port weights and rms rows).  One step = one pass over one scene.  Inputs are seeded synthetic scenes (no public dataset exists for this
path); the per-step working set (~1.9 GB) exceeds the 129 MB L2, so no L2
flush is needed between steps.

  value : tiles/s with all inputs resident in HBM (CUDA events on the launch stream)
  e2e   : tiles/s through the public C ABI with host buffers: H2D of the 4 raw
          images and the tile ops + disparity from pinned memory, the step, and
          D2H of the disparity map and of every camera's RBG frames (what the
          reference's caller reads back), every step (host wall clock); the next
          frame's images go up on a copy stream while IMCLT / textures run, the
          frames come down on another during the textures and the next forward
  --impl reference : the reference CPU path (the FP64 C restatement of
          ImageDtt/Correlation2d, the Java reference cannot run here) on all
          host cores, a bounded tile sample per step.
Multi-GPU: replicas only (independent scenes per rank, no collective on the
data path); value = tiles of all ranks / max time over ranks.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "imagej-elphel_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "CLT tiles/s fwd & fwd+adjoint on 1 GB300 vs plain and CPU; err vs FP64 oracle"

CONFIGS = {
    # name: (kind, width, height, kernels, pairs)
    "c2_bayer_4x2592x1936": dict(kind="quad_bayer", width=2592, height=1936, kernels=True),
    # quarter-size Bayer scene for ncu captures (CLT 240 MB > L2, ~0.5 GB on the device)
    "c2q_bayer_4x1296x968": dict(kind="quad_bayer", width=1296, height=968, kernels=True),
    "c1_mono_4x512x384": dict(kind="quad_mono", width=512, height=384, kernels=False),
    "c3_lwir_16x640x512": dict(kind="circle_lwir", width=640, height=512, kernels=False),
}
DEFAULT_CONFIG = "c2_bayer_4x2592x1936"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)  # ~0.6 s timed: several clock samples
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default=DEFAULT_CONFIG, choices=sorted(CONFIGS))
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint / LM measurement")
    p.add_argument("--batch-scenes", type=int, default=64, help="scenes in the batched measurement (0 = skip)")
    p.add_argument("--batch-only", action="store_true", help="only the batched measurement (profiling)")
    p.add_argument("--adjoint-only", action="store_true",
                   help="only the 16-sensor forward / forward+adjoint / LM measurement (profiling)")
    p.add_argument("--cpu-sample-tiles", type=int, default=0, help="tiles per CPU sample (0 = auto)")
    p.add_argument("--schedule", default="", help="tiles_per_cta,warps_per_cta of the forward instead of the autotuner "
                                                  "(profiling)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, use_cuda):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend="nccl" if use_cuda else "gloo")
    return dist


def max_over_ranks(seconds, dist, device="cuda"):
    """The slowest rank's time (replicas: the job ends with its last rank); identity without dist."""
    if not dist:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(cfg_name, seed, rank=0):
    from tileproc import synth
    c = CONFIGS[cfg_name]
    sc = synth.make_scene(c["kind"], seed=seed + 1000 * rank, width=c["width"], height=c["height"])
    W, H = sc["width"], sc["height"]
    T = (W // 8) * (H // 8)
    rng = np.random.default_rng(seed + 7)
    S = sc["geometry"]["num_sensors"]
    k = e = None
    if c["kernels"]:
        k, e = synth.random_clt_kernels(rng, S, H // 16 + 2, W // 16 + 2, sc["num_colors"])
    if sc["num_colors"] == 3 or S == 4:
        target = np.full(T, 4.0, np.float32)
        pairs = None
    else:
        target = np.full(T, 2.0, np.float32)
        pairs = synth.circle_pairs(sc["geometry"])
    return dict(scene=sc, kernels=k, kext=e, target=target, pairs=pairs, T=T, W=W, H=H, S=S,
                C=sc["num_colors"], P=6 if pairs is None else len(pairs),
                KH=(W // 16 + 2) if k is not None else 0, KV=(H // 16 + 2) if k is not None else 0)


def algorithmic_bytes(w):
    """Each datum counted once (fixed per config): inputs + kernel tables + tasks + CLT +
    correlation surfaces + disparity + IMCLT frames."""
    S, C, T, P, W, H = w["S"], w["C"], w["T"], w["P"], w["W"], w["H"]
    b_in = 2 if w["scene"]["images"].dtype == np.uint16 else 4
    parts = {
        "images": S * W * H * b_in,
        "kernels": S * C * w["KH"] * w["KV"] * (1024 + 32),
        "tasks": T * (8 + 8 * S),
        "clt": T * S * C * 1024,
        "corr": T * P * 900,
        "disparity": T * 8,
        "imclt": S * C * (W + 8) * (H + 8) * 4,
    }
    tex = S == 4 and C == 3
    if tex:
        parts["textures"] = T * (12 * 1024 + 64)
    stage = {  # per-launch algorithmic bytes of each kernel
        "ports": T * 8 + T * S * 16 + T * S * C * (20 + 32),
        # fused: images + kernel tables + plan in, CLT + correlation surfaces + disparity out
        "forward": parts["images"] + S * C * w["KH"] * w["KV"] * 1024 + T * S * C * 20 + parts["clt"]
        + parts["corr"] + T * 36,
        "imclt": parts["clt"] + parts["imclt"],
    }
    if tex:  # CLT + task + disparity in, 12 texture rows + 16 aux floats out
        stage["textures"] = parts["clt"] + T * 12 + parts["textures"]
    return sum(parts.values()), parts, stage


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel, cfg_name):
    """dram bytes per launch of `kernel` from the committed ncu summary, if present."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        v = d.get(cfg_name, {}).get(kernel)
        if v is not None:
            return float(v)
    return None


def cpu_baseline(w, sample_tiles, threads):
    """Oracle (FP64 C restatement of the reference CPU path) on a bounded tile sample.
    Input conversion to the oracle's double planes/kernels happens once, outside the timing."""
    from oracle import oracle as O
    sc = w["scene"]
    T = w["T"]
    if "_cpu" not in w:
        if sc["num_colors"] == 3:
            from tileproc import synth
            planes = np.stack([synth.bayer_planes(m, sc["color_index"]) for m in sc["images"]])
        else:
            planes = sc["images"][:, None].astype(np.float64)
        kern = kx = None
        if w["kernels"] is not None:
            kern = np.ascontiguousarray(np.moveaxis(w["kernels"].astype(np.float64), 3, 1))
            kx = np.ascontiguousarray(np.moveaxis(w["kext"].astype(np.float64), 3, 1))
        pairs = None
        if w["pairs"] is not None:
            pairs = O.make_pairs([(a, b, bx, by, kind) for (a, b, kind, _, bx, by) in w["pairs"]])
        w["_cpu"] = (planes, kern, kx, pairs, w["target"].astype(np.float64))
    planes, kern, kx, pairs, target = w["_cpu"]
    step = max(1, T // max(sample_tiles, 1))
    op = np.zeros(T, np.int32)
    op[::step] = 1
    n = int(op.sum())
    t0 = time.perf_counter()
    r = O.run(w["W"], w["H"], planes, op, target, geometry=sc["geometry"], kernels=kern, kernel_ext=kx,
              pairs=pairs, num_threads=threads, want=("clt", "corr", "disp"))
    O.imclt_frames(r["clt"], w["W"] // 8, w["H"] // 8, present=op, num_threads=threads)
    if w["S"] == 4 and w["C"] == 3:
        tiles = np.nonzero(op)[0]
        g = 1.0 / (1.0 + 0.5 + 0.2)
        O.texture_tiles(r["clt"], tiles, 0xF, O.corr_lpf(0.8), (0.5 * g, 0.2 * g, g), num_threads=threads)
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def cpu_baseline_runs(w, sample_tiles, threads, warmup, steps):
    """cpu_baseline repeated: warm-up runs first (the oracle's first call also faults in its output
    arrays), then the timed ones; -> (tiles/s over the timed runs, tiles per run, seconds)."""
    runs = [cpu_baseline(w, sample_tiles, threads) for _ in range(warmup + steps)][warmup:]
    tiles, secs = sum(r[1] for r in runs), sum(r[2] for r in runs)
    return tiles / secs, runs[0][1], secs


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    w = make_workload(args.config, args.seed)
    threads = os.cpu_count() or 1
    sample = args.cpu_sample_tiles
    if not sample:
        # as large a sample as keeps the W + K runs near 90 s: one untimed run of the whole scene
        # gives the rate (a small sample would mostly time the oracle's per-call set-up)
        rate = cpu_baseline(w, w["T"], threads)[0]
        sample = int(min(w["T"], max(2000, rate * 90.0 / max(1, args.steps + args.warmup))))
    value, n_run, tot_t = cpu_baseline_runs(w, sample, threads, args.warmup, args.steps)
    line = {"metric": METRIC, "value": value, "unit": "tiles/s", "impl": "reference", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config, "tiles_per_scene": w["T"], "sample_tiles_per_step": n_run},
            "cpu_baseline": {"value": value, "unit": "tiles/s", "cores": threads, "kind": "port",
                             "sample": "%d of %d tiles per step (sized for about 90 s over the warm-up and timed "
                                       "steps from one untimed whole-scene run), stages 1-4%s, FP64 C restatement"
                                       % (n_run, w["T"], "b" if w["C"] == 3 else "a")},
            "e2e": {"value": value, "unit": "tiles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def measure_fwd_adjoint(seed, steps, warmup, lma_iterations=20):
    """16-sensor LWIR scene (640x512, 5120 tiles, 120 pairs): forward (ports + fused forward)
    vs forward + adjoint (tp_backward: plan with FP64 port derivatives, adjoint kernel,
    Jacobian contraction), CUDA events on the launch stream; then, from extrinsics perturbed by
    N(0, 3e-3) rad, the coarse stage and 20 LM iterations on the analytic Jacobian."""
    import copy
    import torch
    from tileproc import GPUTileProcessor, lma
    w = make_workload("c3_lwir_16x640x512", seed)
    sc = w["scene"]
    T, S = w["T"], w["S"]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = C.c_void_p(stream.cuda_stream)
    rng = np.random.default_rng(seed + 11)
    g0 = copy.deepcopy(sc["geometry"])
    for k in lma.KEYS:
        g0[k] = (np.asarray(g0[k]) + rng.normal(0, 3e-3, S)).tolist()
    D = sc["disparity_gt"].reshape(-1).astype(np.float32)
    tp = GPUTileProcessor(S, w["W"], w["H"])
    try:
        tp.setGeometry(g0)
        tp.setBayerImages(sc["images"])
        tp.setCorrelation(pairs=w["pairs"])
        tp.setFullFrameImages(D, tile_op=np.ones(T, np.int32))
        lib = tp._lib

        def fwd():
            tp._ck(lib.tp_ports(tp.h, sptr), "ports")
            tp._ck(lib.tp_process(tp.h, sptr), "process")

        def fwd_adj():
            fwd()
            tp._ck(lib.tp_backward(tp.h, None, None, None, sptr), "backward")

        out = {"workload": "c3_lwir_16x640x512", "tiles": T, "pairs": w["P"]}
        for name, fn in (("fwd", fwd), ("fwd_adjoint", fwd_adj)):
            for _ in range(warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            out[name + "_ms"] = ms
            out[name + "_tiles_per_s"] = T / (ms / 1000.0)
        out["adjoint_over_fwd"] = out["fwd_adjoint_ms"] / out["fwd_ms"]
        torch.cuda.synchronize()
        ones = np.ones(T, np.int32)
        # coarse stage (every pair's 2D correlation maximum, FP64 port derivatives), then the
        # adjoint-driven LM on the loss of the differentiation workload: sum over tiles of
        # (peak disparity - truth)^2, target disparities held at the scene truth, 64 extrinsics fitted
        t0 = time.perf_counter()
        gc, _, ccost = lma._coarse_stage(tp, g0, D, ones, lma.COARSE, False, None)
        secs_coarse = time.perf_counter() - t0
        t0 = time.perf_counter()
        g1, _, hist = lma.refine(tp, gc, D, iterations=lma_iterations, free_disparity=False, coarse=0)
        secs = time.perf_counter() - t0
        gt = sc["geometry"]
        # the same iteration run to 60 steps: where it converges; and the adjoint-driven iteration
        # alone from the perturbed start (no coarse stage)
        g2, _, hist2 = lma.refine(tp, gc, D, iterations=60, free_disparity=False, coarse=0)
        g3, _, _ = lma.refine(tp, g0, D, iterations=lma_iterations, free_disparity=False, coarse=0)
        valid = {name: int(lma._evaluate(tp, g, D, ones)[1].sum()) for name, g in (("start", g0), ("end", g1),
                                                                                   ("end60", g2))}
        cost_truth = lma._evaluate(tp, gt, D, ones, invalid_cost=1.0)[2]

        def rms(g, common):
            out_ = {}
            for k in lma.KEYS:
                e = np.asarray(g[k]) - np.asarray(gt[k])
                if common:
                    e = e - e.mean()
                out_[k] = float(np.sqrt(np.mean(e * e)))
            return out_

        cost1 = {name: lma._evaluate(tp, g, D, ones, invalid_cost=1.0)[2]
                 for name, g in (("start", g0), ("coarse", gc), ("end", g1), ("end60", g2), ("alone", g3))}
        out["lma"] = {"iterations": lma_iterations, "cost_start": cost1["start"], "cost_after_coarse": cost1["coarse"],
                      "cost_end": cost1["end"], "cost_at_truth": cost_truth,
                      "valid_tiles_start": valid["start"], "valid_tiles_end": valid["end"],
                      "cost": "sum over tiles of min(d^2, 1) (px^2), 1 px^2 for a tile without a correlation peak "
                              "(the iteration narrows its cap from 9 to 4 to 2 to 1 px^2)",
                      "seconds": secs,
                      "start": "extrinsics + N(0, 3e-3) rad on all 16 sensors, target disparity = scene truth "
                               "(held fixed: free_disparity=False)",
                      "gauge": "the coarse stage holds each parameter's sum over the 16 sensors; the common-mode "
                               "rows remove each parameter's mean (a rotation / zoom of the whole camera, which pair "
                               "disparities do not see)",
                      "coarse": {"steps": len(ccost) - 1, "seconds": secs_coarse,
                                 "what": "Gauss-Newton on every pair's 2D correlation maximum with the FP64 port "
                                         "derivatives, before the adjoint-driven iterations",
                                 "rms_error_end_common_removed": rms(gc, True)},
                      "rms_error_start": rms(g0, False), "rms_error_end": rms(g1, False),
                      "rms_error_start_common_removed": rms(g0, True),
                      "rms_error_end_common_removed": rms(g1, True),
                      "run_to_60": {"cost_end": cost1["end60"], "valid_tiles_end": valid["end60"],
                                    "rms_error_end": rms(g2, False),
                                    "rms_error_end_common_removed": rms(g2, True)},
                      "adjoint_alone_from_start": {"cost_end": cost1["alone"],
                                                   "rms_error_end_common_removed": rms(g3, True)}}
    finally:
        tp.close()
    return out


def measure_batch(seed, n_scenes, steps, warmup, types=("c2_bayer_4x2592x1936", "c3_lwir_16x640x512")):
    """C4: n_scenes scenes alternating over `types` (by default the 4x2592x1936 Bayer type and the
    16x640x512 LWIR type), each with its own seed-derived images, kernel table (Bayer) and extrinsics.  To keep the
    set-up short the per-scene inputs are seeded variations of one rendered scene per type
    (shifted mosaic + noise, scaled kernel table, perturbed extrinsics); the work per scene is
    unchanged.  Times one step (ports + forward of every scene) three ways on one stream:
    per-scene calls, one batched persistent launch, and the batch's CUDA graph."""
    import copy
    import torch
    from tileproc import GPUTileProcessor
    from tileproc import _lib as L
    from tileproc.batch import Batch
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = C.c_void_p(stream.cuda_stream)
    base = {t: make_workload(t, seed) for t in types}
    rng = np.random.default_rng(seed + 99)
    tps, tiles = [], 0
    try:
        for i in range(n_scenes):
            w = base[types[i % len(types)]]
            sc = w["scene"]
            g = copy.deepcopy(sc["geometry"])
            for k in ("azimuth", "tilt", "roll", "zoom"):
                g[k] = (np.asarray(g[k]) + rng.normal(0, 1e-3, w["S"])).tolist()
            shift = 2 * int(rng.integers(0, 8))
            imgs = np.roll(sc["images"], shift, axis=2)
            if imgs.dtype == np.uint16:
                imgs = np.clip(imgs.astype(np.int32) + rng.integers(-2, 3, imgs.shape), 0, 4095).astype(np.uint16)
            else:
                imgs = (imgs + rng.normal(0, 0.01, imgs.shape)).astype(np.float32)
            tp = GPUTileProcessor(w["S"], w["W"], w["H"], num_colors=w["C"], kernels_hor=w["KH"],
                                  kernels_vert=w["KV"])
            tps.append(tp)
            tp.setGeometry(g)
            if w["kernels"] is not None:
                f = np.float32(1.0 + 0.02 * rng.standard_normal())
                tp.setConvolutionKernels(w["kernels"] * f, w["kext"], layout=L.TP_KERNELS_CPU)
            if w["C"] == 3:
                tp.setColorScales([1.0, 1.0, 0.5])
            tp.setBayerImages(imgs)
            tp.setCorrelation(pairs=w["pairs"])
            tp.setFullFrameImages(w["target"], tile_op=np.full(w["T"], 0xF, np.int32))
            tiles += w["T"]
        lib = tps[0]._lib
        # the autotuner's schedule per scene type, picked on the type's first scene and set on all
        from tileproc.autotune import autotune
        picks = {}
        for i, t in enumerate(types[:n_scenes]):
            best, ms = autotune(tps[i], reps=3, warmup=1)
            picks[t] = {"pick": "%d,%d" % best, "ms": {"%d,%d" % k: round(v, 4) for k, v in ms.items()}}
            for tp in tps[i::len(types)]:
                tp.setSchedule(*best)

        def plain_of(sel):
            def fn():
                for tp in sel:
                    tp._ck(lib.tp_ports(tp.h, sptr), "ports")
                    tp._ck(lib.tp_process(tp.h, sptr), "process")
            return fn

        b = Batch(tps)
        out = {"workload": "%d scenes alternating %s" % (n_scenes, " / ".join(types)), "tiles_per_step": tiles,
               "autotune": picks}
        runs = [("plain", plain_of(tps)), ("batched", lambda: b.process(True, sptr)),
                ("graph", lambda: b.run_graph(sptr))]
        # the per-scene step split by scene type: what each type costs inside the plain step
        runs += [("plain_" + t, plain_of(tps[i::len(types)])) for i, t in enumerate(types[:n_scenes])]
        for name, fn in runs:
            for _ in range(warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            out[name + "_ms"] = ms
            if not name.startswith("plain_"):
                out[name + "_tiles_per_s"] = tiles / (ms / 1000.0)
        out["batched_over_plain"] = out["plain_ms"] / out["batched_ms"]
        out["graph_over_plain"] = out["plain_ms"] / out["graph_ms"]
        b.close()
    finally:
        for tp in tps:
            tp.close()
    return out


def prepare_psf_kernels(torch, tp, w, seed):
    """Renders each sensor's double-resolution PSF table on the device (torch, synthetic data) and
    runs tp_calc_kernels on it; the prepared tables replace w's kernels (the CPU baseline uses them)."""
    S, C, KV, KH = w["S"], w["C"], w["KV"], w["KH"]
    n = KV * KH * C
    g = torch.Generator(device="cuda").manual_seed(seed)
    yy, xx = torch.meshgrid(torch.arange(64, device="cuda", dtype=torch.float32),
                            torch.arange(64, device="cuda", dtype=torch.float32), indexing="ij")
    psf = torch.empty((n, 64, 64), device="cuda", dtype=torch.float32)
    kernels, kext, ms = [], [], 0.0
    for s in range(S):
        for a in range(0, n, 8192):
            b = min(n, a + 8192)
            m = b - a
            r = torch.rand((5, m, 1, 1), generator=g, device="cuda")
            sx, sy = (0.6 + 0.8 * r[0]) * 2.0, (0.6 + 0.8 * r[1]) * 2.0
            th = r[2] * np.pi
            cx, cy = 32.0 + (r[3] - 0.5) * 1.2, 32.0 + (r[4] - 0.5) * 1.2
            dx, dy = xx - cx, yy - cy
            u, v = torch.cos(th) * dx + torch.sin(th) * dy, -torch.sin(th) * dx + torch.cos(th) * dy
            q = torch.exp(-0.5 * ((u / sx) ** 2 + (v / sy) ** 2))
            psf[a:b] = q / q.sum(dim=(1, 2), keepdim=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tp.calcConvolutionKernels(None, s, device_ptr=psf.data_ptr())
        tp.synchronize()
        ms += 1000.0 * (time.perf_counter() - t0)
        k, e = tp.getConvolutionKernels(s)
        kernels.append(k)
        kext.append(e)
    del psf
    w["kernels"], w["kext"] = np.stack(kernels), np.stack(kext)
    return {"kernel_tiles": n * S, "psf": "64x64 double-resolution elliptical Gaussians", "ms": ms,
            "kernel_tiles_per_s": n * S / (ms / 1000.0)}


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    assert torch.cuda.is_available(), "bench.py needs a CUDA GPU"
    torch.cuda.set_device(local)
    dist = dist_init(world, True)
    import build as tp_build
    tp_build.build()
    from tileproc import GPUTileProcessor
    from tileproc import _lib as L
    w = make_workload(args.config, args.seed, rank)
    sc = w["scene"]
    T, S, Cn = w["T"], w["S"], w["C"]
    # a dedicated stream: the C ABI treats a NULL stream as "the handle's own stream",
    # so the events must be recorded on the stream handed to the launches
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = C.c_void_p(stream.cuda_stream)
    assert sptr.value, "need a non-default stream"
    tp = GPUTileProcessor(S, w["W"], w["H"], num_colors=Cn, kernels_hor=w["KH"], kernels_vert=w["KV"],
                          device=local)
    tp.setGeometry(sc["geometry"])
    kernel_prep = None
    if w["kernels"] is not None:
        # per-sensor / per-colour kernel tables from elliptical Gaussian PSFs (sigma 0.6..1.4 px,
        # random orientation, +-0.3 px offsets) through the QuadCLT kernel chain on the device
        kernel_prep = prepare_psf_kernels(torch, tp, w, args.seed + 1000 * rank)
    if Cn == 3:
        tp.setColorScales([1.0, 1.0, 0.5])
    tp.setBayerImages(sc["images"])
    tp.setCorrelation(pairs=w["pairs"])
    tile_op = np.full(T, 0xF, np.int32)  # all four ports (ImageDtt image mask), all tiles
    tp.setFullFrameImages(w["target"], tile_op=tile_op)
    lib = tp._lib
    # ports: stage 1 (FP64) + window plan; forward: fused convert+correct / correlate / extract;
    # imclt: inverse CLT into the colour frames; textures: RGBA texture tiles (quad colour only)
    stages = ["ports", "forward", "imclt"]
    fns = [lib.tp_ports, lib.tp_process, lib.tp_imclt]
    # schedule of the fused forward picked by the project's autotuner on this scene (outside the timing)
    if args.schedule:
        sched = tuple(int(v) for v in args.schedule.split(","))
        sched_ms = {}
        tp.setSchedule(*sched)
    else:
        from tileproc.autotune import autotune
        sched, sched_ms = autotune(tp, reps=5, warmup=2)
    with_tex = S == 4 and Cn == 3
    if with_tex:
        tp.setTextureParams()
        stages.append("textures")
        fns.append(lib.tp_textures)

    def step(evs=None):
        for i, f in enumerate(fns):
            if evs is not None:
                evs[i].record(stream)
            st = f(tp.h, sptr)
            if st != 0:
                tp._ck(st, stages[i])
        if evs is not None:
            evs[-1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(len(fns) + 1)] for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for k in range(args.steps):
            step(evs[k])
        t1.record(stream)
        torch.cuda.synchronize()
    elapsed = t0.elapsed_time(t1) / 1000.0
    elapsed = max_over_ranks(elapsed, dist)
    stage_ms = {s: statistics.mean(evs[k][i].elapsed_time(evs[k][i + 1]) for k in range(args.steps))
                for i, s in enumerate(stages)}
    value = world * T * args.steps / elapsed
    total_b, parts, stage_b = algorithmic_bytes(w)
    dom = max(stage_ms, key=stage_ms.get)
    peak, peak_kind = measured_peaks()
    ach = stage_b[dom] / (stage_ms[dom] / 1000.0) / 1e9
    traffic = ncu_traffic(dom, args.config)

    # ---- LMA disparity pass (Correlation2d.corrLMA with the far/foreground correction, the
    # reference's default disparity) after the forward, quad pair layouts.  The pass rewrites the
    # disparity record, so every repetition follows its own forward; only the pass is timed.
    lma_line = None
    if w["pairs"] is None:
        prm = L.TpLmaParams()
        tp._ck(lib.tp_default_lma_params(C.byref(prm)), "lma params")
        n_lma = max(3, min(args.steps, 20))
        lev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_lma)]
        for k in range(3 + n_lma):
            tp._ck(lib.tp_process(tp.h, sptr), "process")
            if k >= 3:
                lev[k - 3][0].record(stream)
            tp._ck(lib.tp_lma_refine(tp.h, C.byref(prm), sptr), "lma")
            if k >= 3:
                lev[k - 3][1].record(stream)
        torch.cuda.synchronize()
        lma_ms = statistics.mean(a.elapsed_time(b) for a, b in lev)
        lma = tp.getLma()
        fitted = int(np.isfinite(lma[:, 0]).sum())
        lma_line = {"ms": lma_ms, "tiles_per_s": T / (lma_ms / 1000.0), "fitted_tiles": fitted, "tiles": T,
                    "settings": "ImageDttParameters defaults: mix_corr_poly, fo_correct (4 orientation fits)",
                    "note": "separate pass after the forward, not in the step"}

    # ---- e2e through the public API with host buffers ----
    pin_imgs = [torch.from_numpy(np.ascontiguousarray(sc["images"][s])).pin_memory() for s in range(S)]
    pin_op = torch.from_numpy(tile_op).pin_memory()
    pin_disp = torch.from_numpy(w["target"].copy()).pin_memory()
    # results of two frames in flight: the disparity record and every camera's colour frames, as
    # the reference's caller reads them (GPUTileProcessor.getRBG), into page-locked buffers
    out_disp = [torch.empty((T, L.DISP_N), dtype=torch.float32).pin_memory() for _ in range(2)]
    out_rbg = [[torch.empty((Cn, w["H"] + 8, w["W"] + 8), dtype=torch.float32).pin_memory() for _ in range(S)]
               for _ in range(2)]
    np_imgs = [p.numpy() for p in pin_imgs]
    np_op, np_disp = pin_op.numpy(), pin_disp.numpy()
    np_out = [o.numpy() for o in out_disp]
    np_rbg = [[o.numpy() for o in f] for f in out_rbg]
    h2d = sum(a.nbytes for a in np_imgs) + np_op.nbytes + np_disp.nbytes
    d2h = np_out[0].nbytes + sum(a.nbytes for a in np_rbg[0])

    # Frames are double-buffered the way a camera loop would run them: the sensor images are read
    # only by the forward, so the next frame's pinned images go up on a copy stream while this
    # frame's IMCLT and textures run.  Every step still uploads one frame of images and its tile
    # ops and reads its disparity back; the first frame's images go up before the loop.
    copy_stream = torch.cuda.Stream()
    cptr = C.c_void_p(copy_stream.cuda_stream)
    up_done, fwd_done = torch.cuda.Event(), torch.cuda.Event()
    # frame k's colour frames go down on their own stream during frame k's textures and frame
    # k+1's forward; frame k+1's IMCLT (which rewrites them) waits for that copy
    down_stream = torch.cuda.Stream()
    dptr = C.c_void_p(down_stream.cuda_stream)
    rbg_done = torch.cuda.Event()

    def upload_images():
        for s in range(S):
            tp._ck(lib.tp_set_image_async(tp.h, s, C.c_void_p(np_imgs[s].ctypes.data), 1 if Cn == 3 else 0, 0, cptr),
                   "img")
        up_done.record(copy_stream)

    # the host reads frame k's results once frame k + 2 is enqueued (their buffers then take frame k + 2's)
    out_done = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_step(k):
        # tile ops first (uploaded after the previous frame's work, no host round trip), the forward
        # after this frame's image upload, the next frame's upload after the forward, the results
        # read back on the download stream; nothing here waits for the device
        b = k & 1
        out_done[b].synchronize()  # the host has frame k - 2's results: their buffers take frame k's
        tp._ck(lib.tp_set_tile_ops(tp.h, C.c_void_p(np_op.ctypes.data), C.c_void_p(np_disp.ctypes.data)), "ops")
        stream.wait_event(up_done)
        tp._ck(lib.tp_process(tp.h, sptr), "process")
        fwd_done.record(stream)
        copy_stream.wait_event(fwd_done)
        upload_images()
        stream.wait_event(rbg_done)
        tp._ck(lib.tp_imclt(tp.h, sptr), "imclt")
        for s in range(S):
            tp._ck(lib.tp_get_rbg_async(tp.h, s, C.c_void_p(np_rbg[b][s].ctypes.data), dptr), "rbg")
        rbg_done.record(down_stream)
        if with_tex:
            tp._ck(lib.tp_textures(tp.h, sptr), "textures")
        tp._ck(lib.tp_get_disparity_async(tp.h, C.c_void_p(np_out[b].ctypes.data), dptr), "disp")
        out_done[b].record(down_stream)

    upload_images()
    for k in range(min(args.warmup, 3)):
        e2e_step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    te = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - te
    e2e_t = max_over_ranks(e2e_t, dist)
    e2e_val = world * T * args.steps / e2e_t

    batched = batched_small = None
    if rank == 0 and args.batch_scenes > 0:
        nb_steps = max(3, min(args.steps // 4, 10))
        batched = measure_batch(args.seed, args.batch_scenes, nb_steps, min(args.warmup, 3))
        batched_small = measure_batch(args.seed, args.batch_scenes, nb_steps, min(args.warmup, 3),
                                      types=("c1_mono_4x512x384",))
        torch.cuda.set_stream(stream)

    fwd_adj = None
    colour_adj = None
    if rank == 0 and not args.no_adjoint:
        fwd_adj = measure_fwd_adjoint(args.seed, max(3, min(args.steps // 2, 50)), args.warmup)
        torch.cuda.set_stream(stream)
        if Cn == 3:
            # the colour adjoint on this workload's own handle: forward (ports + fused forward) vs
            # forward + tp_backward (the Bayer planes' colour mix reversed, ports' FP64 derivatives)
            def fwd_only():
                tp._ck(lib.tp_ports(tp.h, sptr), "ports")
                tp._ck(lib.tp_process(tp.h, sptr), "process")

            def fwd_bwd():
                fwd_only()
                tp._ck(lib.tp_backward(tp.h, None, None, None, sptr), "backward")

            colour_adj = {"workload": args.config, "tiles": T}
            n_c = max(3, min(args.steps // 2, 50))
            for name, fn in (("fwd", fwd_only), ("fwd_adjoint", fwd_bwd)):
                for _ in range(max(args.warmup, 3)):
                    fn()
                torch.cuda.synchronize()
                c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                c0.record(stream)
                for _ in range(n_c):
                    fn()
                c1.record(stream)
                torch.cuda.synchronize()
                colour_adj[name + "_ms"] = c0.elapsed_time(c1) / n_c
            colour_adj["adjoint_over_fwd"] = colour_adj["fwd_adjoint_ms"] / colour_adj["fwd_ms"]

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the reference arm's own measurement, in a fresh process: this one holds the CUDA context,
        # torch's thread pools and the timing threads, which slowed the oracle's threads by ~2.5x.
        # The whole scene per run, 3 timed runs: about 5-10 s of CPU work.
        sample = args.cpu_sample_tiles or T
        env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--impl", "reference", "--config", args.config,
                            "--seed", str(args.seed), "--steps", "3", "--warmup", "1", "--cpu-sample-tiles",
                            str(sample)], env=env, capture_output=True, text=True, check=True)
        ref_line = json.loads(r.stdout.strip().splitlines()[-1])
        cb = ref_line["cpu_baseline"]
        cpu = {"value": cb["value"], "unit": "tiles/s", "cores": cb["cores"], "kind": "port",
               "sample": "%d of %d tiles (every %d-th) per run, 1 warm-up + 3 timed runs (%.1f s), stages 1-4%s, "
                         "FP64 C restatement, in a separate process (bench.py --impl reference)" % (
                             ref_line["config"]["sample_tiles_per_step"], T, max(1, T // sample),
                             ref_line["ms_per_step"] * 3 / 1000.0, "b" if with_tex else "a")}
    # plan, tile map, disparity init, fused forward, imclt, textures; the staged-window forward of u16
    # Bayer quads hands the serial half of its extraction to a second kernel
    win = Cn == 3 and S <= 4 and w["scene"]["images"].dtype == np.uint16
    launches_per_step = 5 + int(with_tex) + int(win)
    line = {
        "metric": METRIC, "value": value, "unit": "tiles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.config, "tiles_per_scene": T, "sensors": S, "colors": Cn, "pairs": w["P"],
                   "kernels": ("%dx%d from PSFs" % (w["KH"], w["KV"])) if w["KH"] else "identity",
                   "kernel_prep": kernel_prep,
                   "stages": "ports(fp64)+fused(convert_correct,correlate,extract)+imclt" + (
                       "+textures(12 rows)" if with_tex else ""),
                   "l2": "per-step working set %.2f GB > 129 MB L2, no flush" % (total_b / 1e9),
                   "schedule": {"tiles_per_cta": sched[0], "warps_per_cta": sched[1],
                                "autotune_ms": {"%d,%d" % k: round(v, 4) for k, v in sched_ms.items()}},
                   "parallelism": "replicas" if world > 1 else "single"},
        "stage_ms": {k: round(v, 4) for k, v in stage_ms.items()},
        "algorithmic_bytes_per_step": total_b,
        "algorithmic_gbs": total_b / (elapsed / args.steps) / 1e9,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "traffic": traffic, "peak_source": peak_kind,
                     "bytes_per_launch": stage_b[dom]},
        "e2e": {"value": e2e_val, "unit": "tiles/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "reads_back": "disparity record + every camera's RBG frames (getRBG), pinned host buffers, two frames "
                             "in flight",
                "pipeline": "next frame's images uploaded on a copy stream during IMCLT and textures; RBG frames "
                            "and the disparity record read back on a download stream during textures and the next "
                            "forward; tile ops uploaded without a host round trip; the host waits only for the "
                            "results of the frame two back"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "fwd_adjoint": fwd_adj,
        "fwd_adjoint_colour": colour_adj,
        "lma_disparity": lma_line,
        "batched": batched,
        "batched_small_scenes": batched_small,
    }
    tp.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse_args()
    if args.batch_only:
        import torch
        import build as tp_build
        tp_build.build()
        torch.cuda.set_device(0)
        print(json.dumps(measure_batch(args.seed, args.batch_scenes, args.steps, args.warmup)))
        print(json.dumps(measure_batch(args.seed, args.batch_scenes, args.steps, args.warmup,
                                       types=("c1_mono_4x512x384",))))
        return 0
    if args.adjoint_only:
        import torch
        import build as tp_build
        tp_build.build()
        torch.cuda.set_device(0)
        print(json.dumps(measure_fwd_adjoint(args.seed, args.steps, args.warmup)))
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
