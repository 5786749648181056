"""Schedule autotuner (tileproc.autotune) on a fake processor whose process() time
depends on the schedule: the fastest schedule is chosen, set, and cached per key."""
import time

from tileproc import autotune as at


class FakeTP:
    num_sensors, num_colors, num_pairs, width, height = 4, 3, 6, 64, 48

    def __init__(self, cost):
        self.cost = cost
        self.sched = None
        self.calls = 0

    def setSchedule(self, tpb, nw):
        self.sched = (tpb, nw)

    def process(self):
        self.calls += 1
        time.sleep(self.cost[self.sched])

    def synchronize(self):
        pass


def test_picks_fastest_and_caches():
    at._cache.clear()
    cost = {s: 0.004 for s in at.SCHEDULES}
    cost[(1, 2)] = 0.0005
    tp = FakeTP(cost)
    best, times = at.autotune(tp, reps=3, warmup=1)
    assert best == (1, 2) and tp.sched == (1, 2)
    assert set(times) == set(at.SCHEDULES)
    n = tp.calls
    tp2 = FakeTP(cost)
    best2, _ = at.autotune(tp2, reps=3, warmup=1)
    assert best2 == (1, 2) and tp2.calls == 0 and tp2.sched == (1, 2)
    assert n == len(at.SCHEDULES) * 4
