"""The prologue's whole-line rejection never drops a candidate voxel (CPU).

The cull pass tests every voxel of an (x, y) grid line against the beam's
frustum widened by a margin (a voxel whose projection onto the blocking
plane falls outside the widened jaw opening cannot receive fluence), and
before that rejects a whole line from its two end voxels: along a line the
projected coordinates are ratios of linear functions of z and so monotone,
and the per-voxel margin is bounded by its largest end values
(conehead_gb300/csrc/prologue.cu, ``line_outside`` and ``cull_line``).

This file restates both tests in float32 numpy with the beam constants the
library derives (``make_beam_dev`` in conehead_gb300/csrc/capi.cu) and
checks, on seeded grids, beams (gantry, collimator, asymmetric jaws) and
grids that reach close to the source plane, that no rejected line holds a
voxel the per-voxel test keeps, and that the rejection does take out most
lines of a small field.  It also checks the per-voxel margin itself: a
voxel any of whose S^3 blocking sub-samples projects into the jaw opening
is always kept (the margin is the farthest sub-sample's offset,
r = sqrt(3) s_max (S - 1) / (2 S), magnified to the blocking plane, with
r / (1 - r / dmin) bounding r d / (d - r) over the depths d > dmin = 0.2 |K|
that the cull tests).
"""
import numpy as np
import pytest

from conehead_gb300.source import Source

F = np.float32


def beam_consts(src, jaws, spacing, samples=3):
    """Cull constants of one beam, as the library computes them in float64
    and stores in float32.  jaws = (xlo, xhi, zlo, zhi) in cm at the
    blocking plane (already clipped to the 40 cm map); samples = sub-samples
    per axis of the blocking test (fluenceResampling)."""
    pos = np.asarray(src.position, dtype=np.float64)
    vy = np.asarray(src.v_y, dtype=np.float64)
    T = np.asarray(src.transform, dtype=np.float64)
    m0, m2 = T[0], T[2]
    w = pos.astype(np.float32).astype(np.float64)
    vyw = (vy[0] * w[0] + vy[1] * w[1]) + vy[2] * w[2]
    nS = float(vy @ pos)
    c = dict(
        vyf=vy.astype(F), m0f=m0.astype(F), m2f=m2.astype(F),
        a_nS=F(nS), a_m0S=F(m0 @ pos), a_m2S=F(m2 @ pos), a_K=F(-vyw),
        a_c0=F(m0 @ w), a_c2=F(m2 @ w),
        cx_lo=F(jaws[0]), cx_hi=F(jaws[1]), cz_lo=F(jaws[2]), cz_hi=F(jaws[3]),
        enable=(-nS > 0.0 and jaws[0] <= jaws[1] and jaws[2] <= jaws[3]),
    )
    r = np.sqrt(3.0) * max(spacing) * (samples - 1) / (2.0 * samples)
    dmin = 0.2 * abs(float(c["a_K"]))
    c["k"] = F(r / (1.0 - r / dmin)) if r < 0.1 * dmin else F(0)
    c["enable"] = c["enable"] and r < 0.1 * dmin
    return c


def project(c, px, py, pz):
    """Float32 projection of points: (depth, xb, zb, inv, lat)."""
    np_ = c["vyf"][0] * px + c["vyf"][1] * py + c["vyf"][2] * pz
    m0p = c["m0f"][0] * px + c["m0f"][1] * py + c["m0f"][2] * pz
    m2p = c["m2f"][0] * px + c["m2f"][1] * py + c["m2f"][2] * pz
    depth = (np_ - c["a_nS"]).astype(F)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        inv = (F(1) / depth).astype(F)
        si = (-c["a_K"] * inv).astype(F)
        xb = (c["a_c0"] + si * (c["a_m0S"] - m0p)).astype(F)
        zb = (c["a_c2"] + si * (c["a_m2S"] - m2p)).astype(F)
        lat = (np.maximum(np.abs(c["a_m0S"] - m0p), np.abs(c["a_m2S"] - m2p)) * inv).astype(F)
    return depth, xb, zb, inv, lat


def voxel_candidates(c, px, py, pz):
    """The per-voxel test of cull_line: True = the voxel stays listed."""
    depth, xb, zb, inv, lat = project(c, px, py, pz)
    kk = np.abs(c["a_K"])
    near = ~(depth > F(0.2) * kk)
    with np.errstate(invalid="ignore", over="ignore"):
        margin = (c["k"] * kk * inv * (F(1) + lat) + F(0.01)).astype(F)
        out = (xb < c["cx_lo"] - margin) | (xb > c["cx_hi"] + margin) | \
              (zb < c["cz_lo"] - margin) | (zb > c["cz_hi"] + margin)
    return near | ~out


def line_outside(c, px, py, z_first, z_last):
    """line_outside of prologue.cu for lines (px, py) [arrays] from voxel
    centre z_first to z_last."""
    kk = np.abs(c["a_K"])
    xs, zs, invs, lats, ok = [], [], [], [], np.ones(px.shape, bool)
    for pz in (z_first, z_last):
        depth, xb, zb, inv, lat = project(c, px, py, np.full(px.shape, pz, F))
        ok &= depth > F(0.2) * kk
        xs.append(xb), zs.append(zb), invs.append(inv), lats.append(lat)
    with np.errstate(invalid="ignore", over="ignore"):
        M = (c["k"] * kk * np.maximum(*invs) * (F(1) + np.maximum(*lats)) + F(0.02)).astype(F)
        xlo, xhi = np.minimum(*xs), np.maximum(*xs)
        zlo, zhi = np.minimum(*zs), np.maximum(*zs)
        rej = (xhi < c["cx_lo"] - M) | (xlo > c["cx_hi"] + M) | (zhi < c["cz_lo"] - M) | (zlo > c["cz_hi"] + M)
    return ok & rej


def grid_case(rng, n, spacing, origin, gantry, coll, jaws):
    src = Source()
    src.gantry = gantry
    src.collimator = coll
    c = beam_consts(src, jaws, spacing)
    idx = [np.arange(k) for k in n]
    cen = [(F(o) + F(s) * i.astype(F)).astype(F) for o, s, i in zip(origin, spacing, idx)]
    X, Y = np.meshgrid(cen[0], cen[1], indexing="ij")
    px, py = X.ravel(), Y.ravel()
    rej = line_outside(c, px, py, cen[2][0], cen[2][-1]) if c["enable"] else np.zeros(px.shape, bool)
    cand = voxel_candidates(c, px[:, None], py[:, None], cen[2][None, :])
    return rej, cand.any(axis=1)


def test_rejected_lines_hold_no_candidates():
    rng = np.random.default_rng(11)
    total = rejected = 0
    for case in range(60):
        n = tuple(int(v) for v in rng.integers(12, 56, 3))
        spacing = tuple(float(v) for v in rng.uniform(0.2, 0.6, 3))
        ext = [a * b for a, b in zip(n, spacing)]
        origin = [-e / 2 + rng.uniform(-4, 4) for e in ext]
        if case % 10 == 9:
            origin[1] = -100.0 + rng.uniform(-5, 25)     # grid reaching the source plane (y = -SAD)
        gantry = float(rng.uniform(0, 360))
        coll = float(rng.uniform(0, 90))
        if case % 3 == 0:
            a, b = sorted(rng.uniform(-20, 20, 2)), sorted(rng.uniform(-20, 20, 2))
        else:
            h = rng.uniform(0.5, 10, 2)
            off = rng.uniform(-3, 3, 2)
            a, b = (off[0] - h[0], off[0] + h[0]), (off[1] - h[1], off[1] + h[1])
        jaws = (max(a[0], -20.0), min(a[1], 20.0), max(b[0], -20.0), min(b[1], 20.0))
        rej, any_cand = grid_case(rng, n, spacing, origin, gantry, coll, jaws)
        bad = rej & any_cand
        assert not bad.any(), (case, int(bad.sum()))
        total += rej.size
        rejected += int(rej.sum())
    assert rejected > 0.3 * total, rejected / total


@pytest.mark.parametrize("gantry", [0.0, 37.0, 90.0, 211.0])
def test_small_field_rejects_most_lines(gantry):
    """128^3 at 0.25 cm centred on the isocentre, 5 x 5 cm field: most lines
    are rejected whole, and every line with a candidate is kept."""
    rng = np.random.default_rng(12)
    n, sp = (128, 128, 128), (0.25, 0.25, 0.25)
    origin = [-16.0, -16.0, -16.0]
    rej, any_cand = grid_case(rng, n, sp, origin, gantry, 0.0, (-2.5, 2.5, -2.5, 2.5))
    assert not (rej & any_cand).any()
    assert rej.mean() > 0.6, rej.mean()
    # lines the test keeps but that hold no candidate: the price of the bound
    assert (~rej & ~any_cand).mean() < 0.1


@pytest.mark.parametrize("samples", [1, 2, 3, 5])
def test_margin_keeps_every_voxel_with_an_open_sample(samples):
    rng = np.random.default_rng(20 + samples)
    n_needed = n_kept = 0
    for case in range(12):
        n = tuple(int(v) for v in rng.integers(16, 40, 3))
        spacing = np.array(rng.uniform(0.15, 0.6, 3))
        ext = np.array(n) * spacing
        src = Source()
        src.gantry = float(rng.uniform(0, 360))
        src.collimator = float(rng.uniform(0, 90))
        centre = rng.uniform(-3, 3, 3)
        if case % 4 == 3:
            # on the beam axis 25-40 cm from the source: depths from below
            # 0.2 SAD (always kept) up, magnifications up to 5
            centre = np.asarray(src.position, float) + np.asarray(src.v_y, float) * rng.uniform(25, 40)
        origin = centre - ext / 2
        h = rng.uniform(0.2, 6, 2)
        off = rng.uniform(-2, 2, 2)
        jaws = (round(off[0] - h[0], 2), round(off[0] + h[0], 2), round(off[1] - h[1], 2), round(off[1] + h[1], 2))
        c = beam_consts(src, jaws, tuple(spacing), samples)
        # voxel centres (float32 as the kernels hold them)
        idx = np.stack(np.meshgrid(*[np.arange(k) for k in n], indexing="ij"), -1).reshape(-1, 3)
        cen = (origin[None, :].astype(F) + spacing[None, :].astype(F) * idx.astype(F)).astype(F)
        keep = voxel_candidates(c, cen[:, 0], cen[:, 1], cen[:, 2])
        # every sub-sample, projected in float64 through the source onto the
        # blocking plane (v_y . (p - S) = -v_y . S, i.e. the isocentre plane)
        S_ = np.asarray(src.position, dtype=np.float64)
        vy = np.asarray(src.v_y, dtype=np.float64)
        T = np.asarray(src.transform, dtype=np.float64)
        o = (2 * np.arange(samples) + 1 - samples) / (2.0 * samples)
        offs = np.stack(np.meshgrid(o, o, o, indexing="ij"), -1).reshape(-1, 3) * spacing[None, :]
        pts = cen.astype(np.float64)[:, None, :] + offs[None, :, :]
        r = pts - S_
        si = -(vy @ S_) / (r @ vy)
        hit = S_ + si[..., None] * r
        xb, zb = hit @ T[0], hit @ T[2]
        front = (r @ vy) > 0
        open_ = front & (xb >= jaws[0]) & (xb < jaws[1]) & (zb >= jaws[2]) & (zb < jaws[3])
        needed = open_.any(axis=1)
        missed = needed & ~keep
        assert not missed.any(), (samples, case, int(missed.sum()))
        n_needed += int(needed.sum())
        n_kept += int(keep.sum())
    # the check saw voxels at the field edges, and the margin is not vacuous
    assert 0 < n_needed <= n_kept
