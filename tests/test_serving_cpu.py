"""Admission and continuous batching of the dose server, on the CPU.

The scheduler (conehead_gb300.serving.DoseServer) runs against a simulated
executor with a virtual clock: a batch of b beams occupies its slot for
``overhead + b * per_beam`` seconds, scratch grows with the batch, and the
memory it reports follows the same rules as the GPU executor's (fixed
tables, per-slot arenas that only grow, admitted outputs).
"""
import types

import numpy as np
import pytest

from conehead_gb300.serving import DoseServer, Request


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    def __init__(self, clock, n_slots=2, plan_bytes=100, per_beam=1.0, overhead=0.5, scratch_per_beam=10,
                 fail_phantom=None):
        self.clock = clock
        self.n_slots = n_slots
        self.plan_bytes = plan_bytes
        self.arena = [0] * n_slots
        self.finish = [None] * n_slots
        self.items = [None] * n_slots
        self.per_beam, self.overhead, self.spb = per_beam, overhead, scratch_per_beam
        self.sizes = {}
        self.launches = []          # (time, slot, items)
        self.fail_phantom = fail_phantom
        self.max_arena = 0

    def fixed_bytes(self):
        return self.n_slots * self.plan_bytes

    def scratch_bytes(self, slot):
        return self.arena[slot]

    def default_scratch_cap(self, max_wave_beams):
        return self.spb * max_wave_beams

    def output_bytes(self, req):
        return self.sizes[req.phantom] * len(req.beams)

    def wave_key(self, req):
        return req.settings.get("spacing", 0.25)

    def scratch_total(self, items):
        return self.spb * len(items)

    def scratch_growth(self, slot, items):
        return max(0, self.scratch_total(items) - self.arena[slot])

    def launch(self, slot, items):
        assert self.finish[slot] is None
        self.arena[slot] = max(self.arena[slot], self.spb * len(items))
        self.max_arena = max(self.max_arena, self.arena[slot])
        self.finish[slot] = self.clock() + self.overhead + self.per_beam * len(items)
        self.items[slot] = items
        self.launches.append((self.clock(), slot, list(items)))

    def done(self, slot):
        return self.finish[slot] is not None and self.clock() >= self.finish[slot]

    def collect(self, slot):
        items = self.items[slot]
        self.finish[slot] = None
        self.items[slot] = None
        for req, b in items:
            req.doses[b] = ("dose", req.rid, b)
        if any(req.phantom == self.fail_phantom for req, _ in items):
            raise RuntimeError("no intersection or line is within plane")

    def release(self, req):
        pass

    def trim(self, slot):
        self.arena[slot] = 0


def run_events(server, clock, arrivals, make, dt=0.05, limit=10000.0):
    """Submit make(i) at arrivals[i] on the virtual clock, step until drained."""
    reqs, i = [], 0
    while i < len(arrivals) or not server.idle():
        while i < len(arrivals) and arrivals[i] <= clock.t:
            reqs.append(server.submit(make(i)))
            i += 1
        server.step()
        clock.t += dt
        assert clock.t < limit
    return reqs


def _settings(spacing=0.25):
    return {"spacing": spacing}


def test_all_requests_finish_fifo_admission_and_budget_holds():
    clock = Clock()
    ex = FakeExecutor(clock)
    ex.sizes = {"a": 5, "b": 20}
    # plans 200 + pools 80: outputs get 220, one 8-beam request of "b" at most
    server = DoseServer(ex, budget_bytes=500, max_wave_beams=8, scratch_cap=40, clock=clock)
    rng = np.random.default_rng(0)
    arrivals = np.cumsum(rng.exponential(0.3, 60))
    names = rng.choice(["a", "b"], 60)
    nbeams = rng.integers(1, 9, 60)
    reqs = run_events(server, clock, arrivals, lambda i: Request(names[i], [None] * nbeams[i], _settings()))
    assert all(r.done and r.error is None for r in reqs)
    assert all(all(d is not None for d in r.doses) for r in reqs)
    admits = [r.t_admit for r in reqs]
    assert admits == sorted(admits)                      # first in, first admitted
    assert server.peak_used <= server.budget
    assert ex.max_arena <= server.cap                    # batches cut to the pool: at most 4 beams
    assert server.reserved == 0
    assert max(server.waves) <= 4
    st = server.stats()
    assert st["requests"] == 60 and st["beams"] == int(nbeams.sum())
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_batches_overlap_and_late_arrivals_join_the_next_batch():
    clock = Clock()
    ex = FakeExecutor(clock, per_beam=1.0, overhead=0.0)
    ex.sizes = {"a": 1}
    server = DoseServer(ex, budget_bytes=10 ** 9, max_wave_beams=16, clock=clock)
    first = server.submit(Request("a", [None] * 4, _settings()))
    server.step()                                        # slot 0: 4 beams, busy until t = 4
    clock.t = 1.0
    second = server.submit(Request("a", [None] * 2, _settings()))
    server.step()                                        # slot 1 takes it while slot 0 runs
    assert [s for _, s, _ in ex.launches] == [0, 1]
    assert ex.launches[1][0] < ex.finish[0]
    clock.t = 1.5
    late = [server.submit(Request("a", [None] * 3, _settings())) for _ in range(3)]
    server.step()                                        # both slots busy: the 9 beams wait
    assert len(ex.launches) == 2
    clock.t = 3.0
    server.step()                                        # slot 1 done: the 9 beams go as one batch
    assert len(ex.launches) == 3 and len(ex.launches[2][2]) == 9
    while not server.idle():
        clock.t += 0.25
        server.step()
    assert first.done and second.done and all(r.done for r in late)
    assert second.t_done < first.t_done                  # the later, shorter request was not held back


def test_requests_split_across_batches_and_keys_never_mix():
    clock = Clock()
    ex = FakeExecutor(clock)
    ex.sizes = {"a": 1}
    server = DoseServer(ex, budget_bytes=10 ** 9, max_wave_beams=5, clock=clock)
    reqs = [server.submit(Request("a", [None] * 7, _settings(0.25))),
            server.submit(Request("a", [None] * 3, _settings(0.4))),
            server.submit(Request("a", [None] * 2, _settings(0.25)))]
    while not server.idle():
        server.step()
        clock.t += 0.1
    for _, _, items in ex.launches:
        keys = {it[0].settings["spacing"] for it in items}
        assert len(keys) == 1 and len(items) <= 5
    assert all(r.done for r in reqs)
    # the 7-beam request spans two batches
    assert sum(1 for _, _, items in ex.launches if any(r is reqs[0] for r, _ in items)) >= 2


def test_oversized_request_is_refused_and_the_rest_run():
    clock = Clock()
    ex = FakeExecutor(clock)
    ex.sizes = {"small": 10, "huge": 10 ** 6}
    server = DoseServer(ex, budget_bytes=1000, clock=clock)
    reqs = [server.submit(Request("small", [None] * 2, _settings())),
            server.submit(Request("huge", [None], _settings())),
            server.submit(Request("small", [None] * 3, _settings()))]
    for _ in range(200):
        server.step()
        clock.t += 0.1
        if server.idle():
            break
    assert isinstance(reqs[1].error, MemoryError)
    assert reqs[0].done and reqs[2].done and reqs[0].error is None and reqs[2].error is None


def test_memory_pressure_waits_instead_of_overcommitting():
    clock = Clock()
    ex = FakeExecutor(clock, scratch_per_beam=50)
    ex.sizes = {"a": 40}
    # plans 200 + two pools of 60 = 320: room for one 2-beam request's outputs (80)
    server = DoseServer(ex, budget_bytes=400, max_wave_beams=8, scratch_cap=60, clock=clock)
    reqs = [server.submit(Request("a", [None] * 2, _settings())) for _ in range(6)]
    seen_busy = 0
    for _ in range(10000):
        server.step()
        seen_busy = max(seen_busy, len(server.busy))
        assert server.held() <= server.used() <= server.budget
        clock.t += 0.05
        if server.idle():
            break
    assert all(r.done and r.error is None for r in reqs)
    assert seen_busy == 2                                # the two beams of a request run on both slots
    assert all(len(items) == 1 for _, _, items in ex.launches)
    # requests are served one after another: admissions never overlap in time
    spans = sorted((r.t_admit, r.t_done) for r in reqs)
    assert all(a[1] <= b[0] + 1e-9 for a, b in zip(spans, spans[1:]))


def test_scratch_cap_refuses_beams_too_big_for_a_pool():
    clock = Clock()
    ex = FakeExecutor(clock, scratch_per_beam=50)
    ex.sizes = {"a": 1}
    server = DoseServer(ex, budget_bytes=10 ** 6, scratch_cap=40, clock=clock)
    r = server.submit(Request("a", [None], _settings()))
    server.step()
    assert isinstance(r.error, MemoryError) and "scratch" in str(r.error)


def test_failed_batch_reports_its_requests_only():
    clock = Clock()
    ex = FakeExecutor(clock, fail_phantom="bad")
    ex.sizes = {"good": 1, "bad": 1}
    server = DoseServer(ex, budget_bytes=10 ** 9, max_wave_beams=1, clock=clock)
    good = server.submit(Request("good", [None], _settings()))
    bad = server.submit(Request("bad", [None], _settings()))
    while not server.idle():
        server.step()
        clock.t += 0.1
    assert good.error is None and isinstance(bad.error, RuntimeError)
    assert server.stats()["requests"] == 1


def test_poisson_workload_shapes():
    from conehead_gb300.serving import poisson_workload
    rng = np.random.default_rng(3)
    arrivals, specs = poisson_workload(rng, ["p64", "p96"], rate=100.0, n_requests=50)
    assert arrivals[0] == 0 and np.all(np.diff(arrivals) >= 0)
    assert 0.2 < arrivals[-1] < 1.0                      # ~49 gaps of 10 ms
    assert all(1 <= len(b) <= 8 for _, b in specs)
    src, blk = specs[0][1][0]
    assert 0 <= src.gantry < 360 and blk.device_rect() == (1750, 2250, 1750, 2250)
