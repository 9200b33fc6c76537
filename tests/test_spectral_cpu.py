"""The fact the spectral cone stage rests on, checked on the CPU oracle.

The reference's cone stage (conehead/conehead.py:385-488) walks every TERMA
voxel's cones from the voxel centre and stops each walk where it leaves the
grid; the walks' offsets and weights do not depend on the start voxel.  So
the stage is one linear convolution, dose(v) = sum_s T(s) S(v - s), with a
stencil S that the dose of a unit impulse shows: on a (2n - 1)-per-axis grid
the impulse at the centre gives S at every offset two voxels of an n grid can
have.  The oracle's dose of any TERMA on the n grid then equals that
convolution, directly and through circular FFTs of period M >= 2n - 1 (the
spectral path's embedding).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def tables(settings):
    from conehead_gb300.kernel import poly_kernel_tables
    return poly_kernel_tables(settings["energy_weights"])


def _stencil(oracle_lib, tables, n, spacing):
    K, th, ph = tables
    big = [2 * k - 1 for k in n]
    imp = np.zeros(big)
    c = tuple(k - 1 for k in n)
    imp[c] = 1.0
    return oracle_lib.cone(imp, big, spacing, K, th, ph, oracle_lib.MODE_F64), c


@pytest.mark.parametrize("n,spacing", [((9, 11, 8), (0.5, 0.4, 0.6)), ((12, 7, 10), (0.25, 0.25, 0.25))])
def test_cone_stage_is_a_linear_convolution(oracle_lib, tables, n, spacing):
    K, th, ph = tables
    S, c = _stencil(oracle_lib, tables, n, spacing)
    rng = np.random.default_rng(sum(n))
    T = rng.random(n) * (rng.random(n) > 0.6)
    dose = oracle_lib.cone(T, list(n), list(spacing), K, th, ph, oracle_lib.MODE_F64)
    assert dose.max() > 0
    conv = np.zeros(n)
    for s in zip(*np.nonzero(T)):
        lo = [c[k] - s[k] for k in range(3)]
        conv += T[s] * S[lo[0]:lo[0] + n[0], lo[1]:lo[1] + n[1], lo[2]:lo[2] + n[2]]
    assert np.abs(conv - dose).max() <= 1e-12 * dose.max()
    # the same through circular FFTs of power-of-two period >= 2n - 1
    M = [16 if 2 * k - 1 <= 16 else 32 for k in n]
    circ = np.zeros(M)
    for o in np.ndindex(*S.shape):
        off = [o[k] - c[k] for k in range(3)]
        circ[off[0] % M[0], off[1] % M[1], off[2] % M[2]] += S[o]
    Tp = np.zeros(M)
    Tp[:n[0], :n[1], :n[2]] = T
    fft = np.real(np.fft.ifftn(np.fft.fftn(Tp) * np.fft.fftn(circ)))[:n[0], :n[1], :n[2]]
    assert np.abs(fft - dose).max() <= 1e-12 * dose.max()


def test_the_transpose_is_a_correlation(oracle_lib, tables):
    """C^T r = sum_v r(v) S(v - s): the conjugate spectrum."""
    K, th, ph = tables
    n, spacing = (9, 10, 8), (0.5, 0.5, 0.5)
    S, c = _stencil(oracle_lib, tables, n, spacing)
    rng = np.random.default_rng(8)
    r = rng.random(n)
    ct = oracle_lib.cone_transpose(r, list(n), list(spacing), K, th, ph, oracle_lib.MODE_F64)
    M = [32, 32, 16]
    circ = np.zeros(M)
    for o in np.ndindex(*S.shape):
        off = [o[k] - c[k] for k in range(3)]
        circ[off[0] % M[0], off[1] % M[1], off[2] % M[2]] += S[o]
    rp = np.zeros(M)
    rp[:n[0], :n[1], :n[2]] = r
    got = np.real(np.fft.ifftn(np.fft.fftn(rp) * np.conj(np.fft.fftn(circ))))[:n[0], :n[1], :n[2]]
    assert np.abs(got - ct).max() <= 1e-12 * np.abs(ct).max()


def _swz16(i, c, z_lines):
    """The period-256 passes' shared-memory slot of element (row i, line c)."""
    return i * 16 + (c ^ ((i ^ (i >> 4)) if z_lines else i) & 15)


def test_period_256_schedule_and_layouts():
    """Period 256 as two radix-16 stages with butterfly j of a line reading
    rows j + 16 r: stage 1 (no twiddles) leaves X1[j][q] at row 16 j + q,
    stage 2 reads rows j + 16 r, multiplies by tw[r j] and its outputs land at
    rows j + 16 q, the very rows stage 1 of a following transform of
    butterfly j reads.  Both shared-memory layouts are permutations of the
    4096 slots, and the 16 lanes of a stage access (16 lines at one j, or 16
    j at one line on lines along z) fall in 16 different banks of 8 bytes."""
    rng = np.random.default_rng(256)
    x = rng.standard_normal((16, 256)) + 1j * rng.standard_normal((16, 256))
    j = np.arange(16)
    r = np.arange(16)
    stage1 = np.fft.fft(x[:, j[:, None] + 16 * r[None, :]], axis=2)          # [line][j][q]
    rows = np.empty((16, 256), complex)
    rows[:, (16 * j[:, None] + r[None, :]).ravel()] = stage1.reshape(16, -1)
    tw = np.exp(-2j * np.pi * np.arange(256) / 256)
    z = rows[:, j[:, None] + 16 * r[None, :]] * tw[(r[None, :] * j[:, None])]   # [line][j][r]
    out = np.fft.fft(z, axis=2)                                                # [line][j][q]
    ref = np.fft.fft(x, axis=1)
    got = ref[:, j[:, None] + 16 * r[None, :]]
    assert np.abs(out - got).max() <= 1e-12 * np.abs(ref).max()
    i, c = np.meshgrid(np.arange(256), np.arange(16), indexing="ij")
    for zl in (False, True):
        slots = _swz16(i, c, zl)
        assert sorted(slots.ravel().tolist()) == list(range(4096))
        for q in range(16):
            for fixed in range(16):
                if zl:   # 16 lanes share the line, j varies
                    w = _swz16(16 * j + q, fixed, zl) % 16
                    rd = _swz16(j + 16 * q, fixed, zl) % 16
                else:    # 16 lanes share j, the line varies
                    w = _swz16(16 * fixed + q, j, zl) % 16
                    rd = _swz16(fixed + 16 * q, j, zl) % 16
                assert len(set(w.tolist())) == 16 and len(set(rd.tolist())) == 16


@pytest.mark.parametrize("n2", [8, 12, 24])
def test_period_16xn2_schedule(n2):
    """Periods 16 N2 = 128, 192 and 384 as 16 x N2 (spec_x16n_kernel,
    spec_y16n_kernel): forward with n = N2 n1 + n2 -- thread (line, n2) takes
    a 16-point DFT over n1 of rows N2 n1 + n2 with only n1 < 8 non-zero (the
    padded input), twiddled by exp(-2 pi i n2 k1 / M) into exchange row
    N2 k1 + n2; thread (line, k1) takes an N2-point DFT over n2 of rows
    N2 k1 + n2 and holds X[k1 + 16 k2].  Times S^ there, then the inverse
    with n = n2 + N2 n1 in the same thread (N2-point DFT over k2, twiddled by
    exp(+2 pi i n2 k1 / M), into exchange row 16 n2 + k1) and thread
    (line, n2) takes the 16-point DFT over k1 of rows 16 n2 + k1 into rows
    n2 + N2 n1, n1 < 8.  The N2-point DFT is three DFT(N2/3)s over the rows
    3 m + n3, twiddles exp(-+2 pi i n3 k / N2), DFT3s into k + (N2/3) k3
    (N2 = 12, 24), or one DFT8.
    Both exchange maps fill the M rows once."""
    M = 16 * n2
    rng = np.random.default_rng(M)
    nx = M // 2 - 15
    x = np.zeros((16, M), complex)
    x[:, :nx] = rng.standard_normal((16, nx)) + 1j * rng.standard_normal((16, nx))
    s = rng.standard_normal((16, M)) + 1j * rng.standard_normal((16, M))
    tw = np.exp(-2j * np.pi * np.arange(M) / M)
    k1 = np.arange(16)
    j2 = np.arange(n2)
    n1 = np.arange(16)
    q = n2 // 3

    def dftn(a, inv):
        # a[..., N2] along the last axis, the kernels' 3 x (N2 / 3) split
        # (N2 = 8: one DFT8)
        if n2 % 3:
            return np.fft.ifft(a, axis=-1) * n2 if inv else np.fft.fft(a, axis=-1)
        sign = 1 if inv else -1
        b = np.stack([np.fft.ifft(a[..., n3::3], axis=-1) * q if inv else np.fft.fft(a[..., n3::3], axis=-1)
                      for n3 in range(3)], axis=-2)                        # [..., n3, k]
        b = b * np.exp(sign * 2j * np.pi * np.arange(3)[:, None] * np.arange(q)[None, :] / n2)
        y = np.fft.ifft(b, axis=-2) * 3 if inv else np.fft.fft(b, axis=-2)  # [..., k3, k]
        return y.reshape(*a.shape[:-1], n2)                                 # index k + q k3

    # forward stage 1 into the exchange (rows N2 k1 + n2)
    assert not x[:, n2 * n1[8:, None] + j2[None, :]].any()
    y1 = np.fft.fft(x[:, n2 * n1[:, None] + j2[None, :]], axis=1)             # [line][k1][n2]
    y1 = y1 * tw[(k1[:, None] * j2[None, :]) % M]
    rows = np.full((16, M), np.nan + 0j)
    rows[:, (n2 * k1[:, None] + j2[None, :]).ravel()] = y1.reshape(16, -1)
    assert not np.isnan(rows).any()
    # forward stage 2: X[k1 + 16 k2] per thread (line, k1)
    z = dftn(rows[:, n2 * k1[:, None] + j2[None, :]], False)                 # [line][k1][k2]
    X = np.fft.fft(x, axis=1)
    assert np.abs(z - X[:, k1[:, None] + 16 * j2[None, :]]).max() <= 1e-12 * np.abs(X).max()
    # product, inverse stage A into the exchange (rows 16 n2 + k1)
    u = z * s[:, k1[:, None] + 16 * j2[None, :]]
    v = dftn(u, True) * np.conj(tw[(k1[:, None] * j2[None, :]) % M])        # [line][k1][n2]
    rows = np.full((16, M), np.nan + 0j)
    rows[:, (16 * j2[None, :] + k1[:, None]).ravel()] = v.reshape(16, -1)
    assert not np.isnan(rows).any()
    # inverse stage B: rows n2 + N2 n1
    out = np.fft.ifft(rows[:, 16 * j2[:, None] + k1[None, :]], axis=2) * 16  # [line][n2][n1]
    got = np.empty((16, M), complex)
    got[:, (j2[:, None] + n2 * n1[None, :]).ravel()] = out.reshape(16, -1)
    ref = np.fft.ifft(X * s, axis=1) * M
    assert np.abs(got[:, :nx] - ref[:, :nx]).max() <= 1e-11 * np.abs(ref).max()


@pytest.mark.parametrize("n2", [8, 12, 24])
def test_period_16xn2_z_exchange_layout(n2):
    """The z passes' exchange (spec_z16n_*_kernel): line c, row r at
    c (M + M/16) + r + r/16.  The slots of the 16 lines are distinct and
    inside the buffer, and the four access patterns -- 16 lanes at
    consecutive k1 of one line (rows 16 n2 + k1) and 16 lanes at consecutive
    n2 running on into the next line (rows 16 n2 + q) -- fall in 16
    different banks of 8 bytes."""
    M = 16 * n2
    slot = lambda r, c: c * (17 * n2) + r + (r >> 4)
    slots = [slot(r, c) for c in range(16) for r in range(M)]
    assert len(set(slots)) == len(slots) and max(slots) < 16 * 17 * n2
    for q in range(16):
        # lanes along n2 (thread t -> n2 = t mod N2, line t / N2), one warp half at a time
        for h0 in range(0, 16 * n2, 16):
            banks = {slot(16 * (t % n2) + q, t // n2) % 16 for t in range(h0, h0 + 16)}
            assert len(banks) == 16
    for r2 in range(n2):
        # lanes along k1 (thread t -> k1 = t mod 16, line t / 16)
        for c in range(16):
            banks = {slot(16 * r2 + k1, c) % 16 for k1 in range(16)}
            assert len(banks) == 16
