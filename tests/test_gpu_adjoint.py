"""GPU: the cone operator, its transpose and the beamlet-weight gradient.

* ``ch_cone`` applied to a beam's TERMA gives that beam's dose, and its
  transpose passes the adjoint identity <C^T r, t> = <r, C t> at 64^3 and
  128^3.
* The gradient of L = sum (dose - target)^2 (target 2 inside a sphere, 0
  elsewhere) with respect to beamlet weights, computed by the adjoint on the
  GPU in float32, agrees with FP64 central finite differences (h = 1e-4) of
  the FP64 oracle on 50 random beamlets (40^3 heterogeneous phantom,
  10 x 10 beamlets of 1 cm).
* At the full configuration (128^3 heterogeneous phantom, 40 x 40 beamlets
  of 0.5 cm, weights U[0, 1], 4 cm target sphere) the gradient agrees on all
  1600 beamlets with the exact FP64 gradient of the FP64 oracle (its forward,
  its transposed cone of 2 (dose - target) on the TERMA support, and the
  chain through blocked^2, conehead/conehead.py:360 and :377), and with a
  central difference of the plain forward along a random direction.
* The autograd path returns the adjoint's gradient and a descent step
  lowers the objective.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.conehead import engine
    return engine(0)


def _beam(gantry, collimator):
    from conehead_gb300 import Source
    src = Source()
    src.gantry = gantry
    src.collimator = collimator
    return src


def test_cone_operator_reproduces_the_dose_stage(eng, settings):
    import torch
    from conehead_gb300 import Block, Conehead
    from conehead_gb300.adjoint import cone
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(64, 0.25, seed=2, n_inserts=6)
    blk = Block()
    blk.set_rect(-3.0, 4.0, -2.5, 3.5)
    out = Conehead().calculate(_beam(40.0, 10.0), blk, ph, settings, return_intermediates=True)
    T = torch.from_numpy(out["terma"]).cuda()
    d = cone(eng, ph.size, ph.spacing, T).cpu().numpy()
    ref = out["dose"]
    assert ref.max() > 0
    assert np.abs(d - ref).max() <= 1e-5 * ref.max()


@pytest.mark.parametrize("n", [64, 128])
def test_transpose_identity(eng, settings, n):
    import torch
    from conehead_gb300 import Block, Conehead
    from conehead_gb300.adjoint import cone
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(n, 0.25, seed=n, n_inserts=8)
    blk = Block()
    blk.set_square(6.0)
    T = Conehead().calculate(_beam(100.0, 0.0), blk, ph, settings, return_intermediates=True)["terma"]
    g = torch.Generator().manual_seed(n)
    r = torch.rand(tuple(ph.size), generator=g).cuda()
    t = torch.from_numpy(T).cuda()
    ct = cone(eng, ph.size, ph.spacing, t).double()
    ctr = cone(eng, ph.size, ph.spacing, r, transpose=True).double()
    lhs = float((ctr * t.double()).sum())
    rhs = float((r.double() * ct).sum())
    print(f"{n}^3: <C^T r, t> = {lhs:.9e}, <r, C t> = {rhs:.9e}, rel {abs(lhs - rhs) / abs(rhs):.2e}")
    assert abs(lhs - rhs) <= 2e-6 * abs(rhs)
    # a random (non-TERMA) t as well: the operator is the same for any input
    t2 = torch.rand(tuple(ph.size), generator=g).cuda() * (torch.rand(tuple(ph.size), generator=g).cuda() > 0.97)
    lhs = float((ctr * t2.double()).sum())
    rhs = float((r.double() * cone(eng, ph.size, ph.spacing, t2).double()).sum())
    assert abs(lhs - rhs) <= 2e-6 * abs(rhs)


def test_transpose_matches_the_oracle_voxelwise(eng, settings, oracle_lib):
    import torch
    from conehead_gb300.adjoint import cone
    from conehead_gb300.kernel import poly_kernel_tables
    size = (20, 26, 17)
    spacing = (0.5, 0.5, 0.5)
    rng = np.random.default_rng(9)
    r = rng.random(size).astype(np.float32)
    r[rng.random(size) > 0.3] = 0.0
    eng.set_kernel(settings["energy_weights"])
    got = cone(eng, size, spacing, torch.from_numpy(r).cuda(), transpose=True).cpu().numpy()
    K, th, ph = poly_kernel_tables(settings["energy_weights"])
    ref = oracle_lib.cone_transpose(r, size, spacing, K, th, ph, oracle_lib.MODE_F32)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"C^T vs oracle transpose, 20x26x17: {err:.2e} of max")
    assert err <= 2e-6


def _objective_np(dose, target):
    d = dose.astype(np.float64) - target
    return float((d * d).sum())


def test_gradient_matches_fp64_finite_differences(eng, settings, oracle_lib):
    import torch
    from conehead_gb300.adjoint import BeamletDose, BeamletGrid, MapBlock, beamlet_dose, sphere_target
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(40, 0.5, seed=13, n_inserts=5)
    src = _beam(20.0, 0.0)
    bl = BeamletGrid.square(10, 1.0)
    rng = np.random.default_rng(17)
    w = rng.uniform(0.0, 1.0, bl.shape).astype(np.float32)
    target = sphere_target(ph, (0.5, 1.0, -0.5), 2.0)
    op = BeamletDose(eng, ph, src, bl, settings)
    wt = torch.tensor(w, device="cuda", requires_grad=True)
    dose = beamlet_dose(wt, op)
    tg = torch.from_numpy(target).cuda()
    loss = ((dose.double() - tg.double()) ** 2).sum()
    loss.backward()
    grad = wt.grad.cpu().numpy().astype(np.float64)

    def L64(weights):
        d = oracle_lib.calculate(src, MapBlock(bl.host_map(weights)), ph, settings, oracle_lib.MODE_F64)["dose"]
        return _objective_np(d, target)

    h = 1e-4
    flat = [(i, j) for i in range(bl.rows) for j in range(bl.cols)]
    picks = [flat[k] for k in rng.choice(len(flat), 50, replace=False)]
    fd, ad = [], []
    for i, j in picks:
        wp, wm = w.copy(), w.copy()
        wp[i, j] = np.float32(w[i, j] + h)
        wm[i, j] = np.float32(w[i, j] - h)
        step = float(wp[i, j]) - float(wm[i, j])          # the perturbation the float32 map holds
        fd.append((L64(wp) - L64(wm)) / step)
        ad.append(grad[i, j])
    fd, ad = np.array(fd), np.array(ad)
    scale = np.abs(fd).max()
    err = np.abs(ad - fd) / scale
    rel = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    print(f"adjoint vs FP64 central differences, 50 beamlets: max |diff| = {err.max():.2e} of max |grad|, "
          f"relative L2 {rel:.2e}")
    assert scale > 0
    assert err.max() <= 1e-3 and rel <= 1e-3


def test_full_size_directional_derivative(eng, settings):
    import torch
    from conehead_gb300.adjoint import BeamletDose, BeamletGrid, beamlet_dose, sphere_target
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(128, 0.25, seed=0)
    rng = np.random.default_rng(5)
    centre = tuple(rng.uniform(-3.0, 3.0, 3))
    target = torch.from_numpy(sphere_target(ph, centre, 2.0)).cuda().double()
    bl = BeamletGrid.square(40, 0.5)
    op = BeamletDose(eng, ph, _beam(float(rng.uniform(0, 360)), 0.0), bl, settings)
    w = torch.tensor(rng.uniform(0, 1, bl.shape).astype(np.float32), device="cuda", requires_grad=True)
    loss = ((beamlet_dose(w, op).double() - target) ** 2).sum()
    loss.backward()
    g = w.grad.double()
    delta = torch.tensor(rng.standard_normal(bl.shape), device="cuda")
    delta /= delta.norm()
    h = 1e-2
    with torch.no_grad():
        lp = float(((op.forward((w + h * delta).float()).double() - target) ** 2).sum())
        lm = float(((op.forward((w - h * delta).float()).double() - target) ** 2).sum())
    fd = (lp - lm) / (2 * h)
    ad = float((g * delta).sum())
    print(f"128^3, 40x40 beamlets: <grad, d> = {ad:.6e}, central difference {fd:.6e}, rel {abs(ad - fd) / abs(fd):.2e}")
    assert abs(ad - fd) <= 5e-4 * abs(fd)


def test_full_size_gradient_matches_the_fp64_gradient(eng, settings, oracle_lib):
    """128^3 slab phantom, 40 x 40 beamlets of 0.5 cm, weights U[0, 1], target
    2 inside a seeded 4 cm sphere: the GPU's float32 adjoint against the FP64
    chain-rule gradient of the oracle (one FP64 forward and one FP64
    transposed cone for all beamlets; about a minute of host time)."""
    import time

    import torch
    from conehead_gb300.adjoint import BeamletDose, BeamletGrid, beamlet_dose, sphere_target
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(128, 0.25, seed=0)
    rng = np.random.default_rng(5)
    centre = tuple(rng.uniform(-3.0, 3.0, 3))
    target = sphere_target(ph, centre, 2.0)
    src = _beam(float(rng.uniform(0, 360)), 0.0)
    bl = BeamletGrid.square(40, 0.5)
    w = rng.uniform(0, 1, bl.shape).astype(np.float32)
    op = BeamletDose(eng, ph, src, bl, settings)
    wt = torch.tensor(w, device="cuda", requires_grad=True)
    loss = ((beamlet_dose(wt, op).double() - torch.from_numpy(target).cuda().double()) ** 2).sum()
    loss.backward()
    g_gpu = wt.grad.cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    g64, _ = oracle_lib.beamlet_gradient_f64(src, bl, w, ph, settings, target)
    t_cpu = time.perf_counter() - t0
    scale = np.abs(g64).max()
    err = np.abs(g_gpu - g64) / scale
    rel = np.linalg.norm(g_gpu - g64) / np.linalg.norm(g64)
    picks = rng.choice(g64.size, 50, replace=False)
    print(f"128^3, 40x40 beamlets of 0.5 cm: GPU gradient vs FP64 chain-rule gradient: max |diff| "
          f"{err.max():.2e} of max |grad| over all 1600 beamlets ({err.reshape(-1)[picks].max():.2e} on 50 "
          f"random ones), relative L2 {rel:.2e}; FP64 oracle {t_cpu:.0f} s on {oracle_lib.num_threads()} threads")
    assert scale > 0
    assert err.max() <= 1e-3 and rel <= 1e-3


def test_autograd_matches_backward_and_descends(eng, settings):
    import torch
    from conehead_gb300.adjoint import BeamletDose, BeamletGrid, beamlet_dose, sphere_target
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(48, 0.4, seed=3, n_inserts=4)
    bl = BeamletGrid.square(12, 1.0)
    op = BeamletDose(eng, ph, _beam(0.0, 0.0), bl, settings)
    target = torch.from_numpy(sphere_target(ph, (0.0, 0.0, 0.0), 3.0, value=1.0)).cuda()
    w = torch.full(bl.shape, 0.5, device="cuda", requires_grad=True)
    dose = beamlet_dose(w, op)
    scale = float(target.max() / dose.detach().max())
    loss = ((dose * scale - target) ** 2).sum()
    loss.backward()
    direct = op.backward(2 * scale * (dose.detach() * scale - target), weights=w.detach())
    assert torch.allclose(w.grad, direct, rtol=1e-5, atol=1e-6 * float(direct.abs().max()))
    # a small step along -grad lowers the objective
    with torch.no_grad():
        step = 1e-3 / float(w.grad.abs().max())
        w2 = (w - step * w.grad).clamp(min=0)
        loss2 = ((op.forward(w2) * scale - target) ** 2).sum()
    assert float(loss2) < float(loss.detach())
