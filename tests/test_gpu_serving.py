"""GPU: the continuous-batching dose server.

* A request's dose is the same served alone and served inside a mix of
  requests on phantoms of other sizes that arrive while it is on the GPU
  (within 1e-5 of Dmax: only the float order of the dose accumulation
  differs), and every served dose equals ``Conehead.calculate`` of that beam.
* Under a budget with room for one request's outputs at a time, every
  request still completes and the server never holds more than its budget.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    return torch


def _executor(settings, sizes, n_slots=2):
    from conehead_gb300.phantoms import slab_phantom
    from conehead_gb300.serving import GpuExecutor
    ex = GpuExecutor(0, n_slots=n_slots)
    phantoms = {}
    for n in sizes:
        ph = slab_phantom(n, 0.25, seed=n, n_inserts=4)
        ex.add_phantom(f"p{n}", ph)
        phantoms[f"p{n}"] = ph
    ex.prepare(settings, (0.25, 0.25, 0.25), (max(sizes),) * 3)
    return ex, phantoms


def test_result_alone_equals_result_in_the_mix(gpu, settings):
    from conehead_gb300 import Conehead
    from conehead_gb300.phantoms import random_beam
    from conehead_gb300.serving import DoseServer, Request, drive
    ex, phantoms = _executor(settings, (32, 48, 64))
    rng = np.random.default_rng(31)
    probe_beams = [random_beam(rng, rect=(3.0, 8.0), collimator=True) for _ in range(3)]
    server = DoseServer(ex, budget_bytes=8 << 30, max_wave_beams=16)
    alone = server.submit(Request("p48", probe_beams, settings))
    server.run()
    assert alone.error is None
    alone_doses = [d.numpy().copy() for d in alone.doses]

    # the mix: 12 requests on all three phantoms arriving every 2 ms, the
    # probe request in the middle
    arrivals = np.arange(13) * 2e-3
    specs = []
    for i in range(13):
        if i == 6:
            specs.append(("p48", probe_beams))
        else:
            name = ["p32", "p48", "p64"][i % 3]
            specs.append((name, [random_beam(rng, rect=(2.0, 10.0), collimator=True)
                                 for _ in range(int(rng.integers(1, 5)))]))
    server2 = DoseServer(ex, budget_bytes=8 << 30, max_wave_beams=16)
    reqs = drive(server2, arrivals, specs, settings)
    assert all(r.error is None for r in reqs)
    assert max(server2.waves) > 1                         # beams of several requests shared a batch
    probe = reqs[6]
    for a, b in zip(alone_doses, probe.doses):
        b = b.numpy()
        assert a.max() > 0
        assert np.abs(a - b).max() <= TOL * a.max()
    # every served dose equals the drop-in call on that beam
    ch = Conehead()
    for req in reqs[::4]:
        for (src, blk), d in zip(req.beams, req.doses):
            ref = ch.calculate(src, blk, phantoms[req.phantom], settings)
            assert np.abs(d.numpy() - ref).max() <= TOL * max(ref.max(), 1e-30)
    ex.close()


def test_budget_admits_one_request_at_a_time(gpu, settings):
    from conehead_gb300.phantoms import random_beam
    from conehead_gb300.serving import DoseServer, Request
    ex, phantoms = _executor(settings, (48,))
    rng = np.random.default_rng(5)
    out_bytes = 4 * 48 ** 3 * 3
    cap = ex.default_scratch_cap(3)
    budget = ex.fixed_bytes() + 2 * cap + out_bytes          # room for one 3-beam request's outputs
    server = DoseServer(ex, budget_bytes=budget, max_wave_beams=3, scratch_cap=cap)
    reqs = [server.submit(Request("p48", [random_beam(rng) for _ in range(3)], settings)) for _ in range(5)]
    max_admitted = 0
    while not server.idle():
        server.step()
        max_admitted = max(max_admitted, sum(1 for r in reqs if r.t_admit is not None and not r.done))
        assert server.held() <= server.budget
    assert all(r.error is None for r in reqs)
    assert max_admitted == 1
    assert all(all(d.numpy().max() > 0 for d in r.doses) for r in reqs)
    ex.close()
