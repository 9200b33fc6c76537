"""The schedule autotuner's search and cache, on the CPU (simulated timings)."""
import types

from conehead_gb300 import _native as N
from conehead_gb300.autotune import CANDIDATES, autotune, signature


class FakeEngine:
    def __init__(self):
        self.tuning = None
        self.calls = 0

    def set_tuning(self, **t):
        self.tuning = dict(t)


def _jobs(sizes, crop=(500, 500)):
    out = []
    for n in sizes:
        g = N.grid_struct((n, n, n), (0.0, 0.0, 0.0), (0.25, 0.25, 0.25))
        b = N.Beam()
        b.block_rows, b.block_cols = crop
        out.append(types.SimpleNamespace(grid=g, beam=b))
    return out


def test_autotune_picks_the_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tuning.json")
    eng = FakeEngine()
    cost = lambda t: 10.0 + abs(t["dir_group"] - 32) + 3 * t["unit_order"] + abs(t["terma_ctas_per_sm"] - 4) / 10

    def timer(e, jobs):
        e.calls += 1
        return cost(e.tuning)

    jobs = _jobs([64, 96, 128, 160] * 16)
    r = autotune(eng, jobs, path=path, timer=timer, device_name="GB300")
    assert not r["cached"] and eng.calls == len(CANDIDATES)
    assert r["tuning"] == {"dir_group": 32, "unit_order": 0, "terma_ctas_per_sm": 3, "cone_method": 1} == eng.tuning
    eng2 = FakeEngine()
    r2 = autotune(eng2, _jobs([160, 128, 96, 64] * 16), path=path, timer=timer, device_name="GB300")
    assert r2["cached"] and eng2.calls == 0 and eng2.tuning == r["tuning"]
    # another device or a different workload is tuned afresh
    r3 = autotune(FakeEngine(), jobs, path=path, timer=timer, device_name="other")
    assert not r3["cached"]
    r4 = autotune(FakeEngine(), _jobs([32] * 3), path=path, timer=timer, device_name="GB300")
    assert not r4["cached"]


def test_signature_buckets():
    a = signature("d", _jobs([64, 128] * 10))
    b = signature("d", _jobs([128, 64] * 10))
    c = signature("d", _jobs([64, 128] * 10, crop=(2000, 2000)))
    assert a == b and a != c
