"""Schedule autotuner for the fused forward kernel.

Candidates (tp_set_schedule), spanning tiles per CTA x warps per tile x register
budget:
  (1, 1), (2, 2), (4, 4)  one warp per tile, 1 / 2 / 4 tiles per CTA, up to 128
                          registers (4 CTAs of 4 warps per SM); for u16 Bayer quads
                          with staged image windows;
  (1, 2), (1, 4)          one tile per CTA, its colour items and pairs split over 2 / 4
                          warps sharing the tile's CLT, up to 128 registers;
  (1, 3)                  one tile per CTA of 3 warps (one colour item, then two pairs
                          per warp for a quad colour scene), 80 registers for 8 CTAs
                          (24 warps) per SM.
The reference fixes its launch shape at compile time (TILES_PER_BLOCK,
THREADS_PER_TILE, GPUTileProcessor.java:92-93); here every candidate is timed on
the caller's own scene and the fastest is kept, per (sensors, colours, pairs,
size) key.
"""
import time

SCHEDULES = ((1, 1), (2, 2), (4, 4), (1, 2), (1, 3), (1, 4))

_cache = {}


def key_of(tp):
    return (tp.num_sensors, tp.num_colors, tp.num_pairs, tp.width, tp.height)


def picks():
    """{(sensors, colours, pairs, width, height): (schedule, {schedule: ms})} of every scene tuned so far"""
    return {k: (v[0], dict(v[1])) for k, v in _cache.items()}


def autotune(tp, reps=5, warmup=2, schedules=SCHEDULES, use_cache=True):
    """Times tp.process() under each schedule (wall clock around synchronised repetitions),
    leaves the fastest one set and returns (best, {schedule: ms})."""
    k = key_of(tp)
    if use_cache and k in _cache:
        best, times = _cache[k]
        tp.setSchedule(*best)
        return best, dict(times)
    times = {}
    for sch in schedules:
        tp.setSchedule(*sch)
        for _ in range(warmup):
            tp.process()
        tp.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            tp.process()
        tp.synchronize()
        times[sch] = 1000.0 * (time.perf_counter() - t0) / reps
    best = min(times, key=times.get)
    tp.setSchedule(*best)
    _cache[k] = (best, dict(times))
    return best, times
