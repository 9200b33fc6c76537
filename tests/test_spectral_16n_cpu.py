"""A scalar restatement of the 16 x N2 pass kernels (CPU).

conehead_gb300/csrc/spectral.cu runs the x, y and z passes at FFT periods
M = 16 N2 = 128, 192 and 384 in spec_x16n_kernel, spec_y16n_kernel and
spec_z16n_{forward,inverse}_kernel.  This file restates, thread by thread,
what those kernels compute and where they read and write: the DFT formulas
as the kernels write them (DFT4, the 4 x 4 DFT16 with its rotation
constants, the half-input DFT16, DFT8 as two DFT4s, DFT3, and DFT12 / DFT24
as three DFT4s / DFT8s, twiddles and DFT3s), the exchange slots, the
twiddle-table indices and every global index.  It checks, on small seeded
blocks, that each exchange slot is written exactly once before it is read,
that every global read and write stays inside its array, that every output
row is written once, and that the results equal numpy.fft (x pass: forward,
times S^, inverse, rows < nx; y passes: forward to all M rows and back;
z passes: TERMA pair to A and A back to the dose pair, with lines that hold
no TERMA read as zeros).
"""
import math

import numpy as np
import pytest

C1, S1, R2 = 0.92387953251128674, 0.38268343236508977, 0.70710678118654752


def rot(v, c, s, inv):
    sn = s if inv else -s
    return complex(v.real * c - v.imag * sn, v.real * sn + v.imag * c)


def mi(v, inv):                      # times -i (forward) or +i (inverse)
    return complex(-v.imag, v.real) if inv else complex(v.imag, -v.real)


def dft4(a, inv):
    a0, a1, a2, a3 = a
    s02, d02, s13, d13 = a0 + a2, a0 - a2, a1 + a3, a1 - a3
    m = mi(d13, inv)
    return [s02 + s13, d02 + m, s02 - s13, d02 - m]


def dft16(v, inv, half_in=False):
    """Output X[k1 + 4 k2] in slot 4 k1 + k2, as the kernels' dft16."""
    v = list(v)
    for b in range(4):
        if half_in:
            a0, a1 = v[b], v[4 + b]
            m = mi(a1, inv)
            v[b], v[4 + b], v[8 + b], v[12 + b] = a0 + a1, a0 + m, a0 - a1, a0 - m
        else:
            v[b], v[4 + b], v[8 + b], v[12 + b] = dft4([v[b], v[4 + b], v[8 + b], v[12 + b]], inv)
    v[5] = rot(v[5], C1, S1, inv)
    v[9] = rot(v[9], R2, R2, inv)
    v[13] = rot(v[13], S1, C1, inv)
    v[6] = rot(v[6], R2, R2, inv)
    v[10] = mi(v[10], inv)
    v[14] = rot(v[14], -R2, R2, inv)
    v[7] = rot(v[7], S1, C1, inv)
    v[11] = rot(v[11], -R2, R2, inv)
    v[15] = rot(v[15], -C1, -S1, inv)
    for k1 in range(4):
        v[4 * k1:4 * k1 + 4] = dft4(v[4 * k1:4 * k1 + 4], inv)
    return v


def x16(v, m):                        # X[m] of a dft16 result
    return v[4 * (m & 3) + (m >> 2)]


def dft8(a, inv):
    e = dft4([a[0], a[2], a[4], a[6]], inv)
    o = dft4([a[1], a[3], a[5], a[7]], inv)
    o[1] = rot(o[1], R2, R2, inv)
    o[2] = mi(o[2], inv)
    o[3] = rot(o[3], -R2, R2, inv)
    return [e[k] + o[k] for k in range(4)] + [e[k] - o[k] for k in range(4)]


def dft3(a, b, c, inv):
    h = 0.86602540378443865
    s, d = b + c, b - c
    t = a - 0.5 * s
    u = complex(-h * d.imag, h * d.real) if inv else complex(h * d.imag, -h * d.real)
    return a + s, t + u, t - u


def dft_3xq(a, inv):
    """DFT12 / DFT24: three DFT4s / DFT8s over rows 3 m + n3, twiddles of
    30 / 15 degree multiples, DFT3s; natural order in and out."""
    q = len(a) // 3
    sub = dft4 if q == 4 else dft8
    b = [sub([a[3 * m + n3] for m in range(q)], inv) for n3 in range(3)]
    x = [0j] * len(a)
    for k in range(q):
        t0, t1, t2 = b[0][k], b[1][k], b[2][k]
        if k:
            a1, a2 = 2 * math.pi * k / len(a), 4 * math.pi * k / len(a)
            t1 = rot(t1, math.cos(a1), math.sin(a1), inv)
            t2 = rot(t2, math.cos(a2), math.sin(a2), inv)
        x[k], x[k + q], x[k + 2 * q] = dft3(t0, t1, t2, inv)
    return x


def dft_n2(a, inv):
    return dft8(a, inv) if len(a) == 8 else dft_3xq(a, inv)


class Exchange:
    """Shared memory that must be written once before each read."""

    def __init__(self, n):
        self.v = [None] * n

    def put(self, i, x):
        assert 0 <= i < len(self.v) and self.v[i] is None
        self.v[i] = x

    def get(self, i):
        assert self.v[i] is not None
        return self.v[i]


@pytest.mark.parametrize("n2", [8, 12, 24])
def test_x16n_pass(n2):
    M, T = 16 * n2, max(16 * n2, 256)
    rng = np.random.default_rng(n2)
    tw = np.exp(-2j * np.pi * np.arange(M) / M)
    My, Mz = 2, 16
    xs = My * Mz
    for nx in (M // 2 - 7, M // 2):
        B = rng.standard_normal(nx * xs) + 1j * rng.standard_normal(nx * xs)
        Sh = rng.standard_normal(M * xs) + 1j * rng.standard_normal(M * xs)
        out = B.copy()
        written = set()
        for ky in range(My):
            for kz0 in range(0, Mz, 16):
                off = ky * Mz + kz0
                sb = Exchange(M * 16)
                for t in range(T):                         # cp.async S^ rows
                    for q in range(8 * M // T):
                        e = t + q * T
                        i, cp = e >> 3, (e & 7) * 2
                        for h in range(2):
                            assert off + i * xs + cp + h < Sh.size
                            sb.put(i * 16 + cp + h, Sh[off + i * xs + cp + h])
                xb = Exchange(M * 16)
                for t in range(16 * n2):                   # forward stage 1
                    c, h = t & 15, t >> 4
                    v = [0j] * 16
                    for n1 in range(8):
                        x = n2 * n1 + h
                        if x < nx:
                            assert off + x * xs + c < B.size
                            v[n1] = B[off + x * xs + c]
                    v = dft16(v, False, half_in=True)
                    for m in range(16):
                        y = x16(v, m) * (tw[h * m] if m else 1)
                        xb.put((m * n2 + h) * 16 + c, y)
                z = {}
                for t in range(256):                       # stage 2, S^, stage A
                    c, h = t & 15, t >> 4
                    zz = dft_n2([xb.get((h * n2 + j) * 16 + c) for j in range(n2)], False)
                    z[t] = dft_n2([zz[k2] * sb.get((h + 16 * k2) * 16 + c) for k2 in range(n2)], True)
                xb = Exchange(M * 16)
                for t in range(256):
                    c, h = t & 15, t >> 4
                    for j in range(n2):
                        y = z[t][j] * (np.conj(tw[j * h]) if j else 1)
                        xb.put((j * 16 + h) * 16 + c, y)
                for t in range(16 * n2):                   # inverse stage B
                    c, h = t & 15, t >> 4
                    v = dft16([xb.get((h * 16 + q) * 16 + c) for q in range(16)], True)
                    for m in range(8):
                        x = h + n2 * m
                        if x < nx:
                            a = off + x * xs + c
                            assert a < B.size and a not in written
                            written.add(a)
                            out[a] = x16(v, m)
        assert len(written) == nx * xs
        full = np.zeros((M, xs), complex)
        full[:nx] = B.reshape(nx, xs)
        ref = np.fft.ifft(np.fft.fft(full, axis=0) * Sh.reshape(M, xs), axis=0)[:nx] * M
        assert np.abs(out.reshape(nx, xs) - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n2", [8, 12, 24])
def test_y16n_passes(n2):
    M = 16 * n2
    rng = np.random.default_rng(100 + n2)
    tw = np.exp(-2j * np.pi * np.arange(M) / M)
    nxg, Mz = 2, 16
    ny = M // 2 - 5
    A = rng.standard_normal(nxg * ny * Mz) + 1j * rng.standard_normal(nxg * ny * Mz)
    Bm = [None] * (nxg * M * Mz)
    for bx in range(nxg * (Mz >> 4)):
        x, kz0 = bx // (Mz >> 4), (bx % (Mz >> 4)) << 4
        src, dst = x * ny * Mz + kz0, x * M * Mz + kz0
        xb = Exchange(M * 16)
        for t in range(16 * n2):
            c, h = t & 15, t >> 4
            v = [A[src + (n2 * n1 + h) * Mz + c] if n2 * n1 + h < ny else 0j for n1 in range(8)] + [0j] * 8
            v = dft16(v, False, half_in=True)
            for m in range(16):
                xb.put((m * n2 + h) * 16 + c, x16(v, m) * (tw[h * m] if m else 1))
        for t in range(256):
            c, h = t & 15, t >> 4
            zz = dft_n2([xb.get((h * n2 + j) * 16 + c) for j in range(n2)], False)
            for k2 in range(n2):
                a = dst + (h + 16 * k2) * Mz + c
                assert Bm[a] is None
                Bm[a] = zz[k2]
    assert all(b is not None for b in Bm)
    Bm = np.array(Bm)
    full = np.zeros((nxg, M, Mz), complex)
    full[:, :ny] = A.reshape(nxg, ny, Mz)
    X = np.fft.fft(full, axis=1)
    assert np.abs(Bm.reshape(nxg, M, Mz) - X).max() <= 1e-12 * np.abs(X).max()
    A2 = [None] * A.size
    for bx in range(nxg * (Mz >> 4)):
        x, kz0 = bx // (Mz >> 4), (bx % (Mz >> 4)) << 4
        src, dst = x * M * Mz + kz0, x * ny * Mz + kz0
        xb = Exchange(M * 16)
        for t in range(256):
            c, h = t & 15, t >> 4
            zz = dft_n2([Bm[src + (h + 16 * k2) * Mz + c] for k2 in range(n2)], True)
            for j in range(n2):
                xb.put((j * 16 + h) * 16 + c, zz[j] * (np.conj(tw[j * h]) if j else 1))
        for t in range(16 * n2):
            c, h = t & 15, t >> 4
            v = dft16([xb.get((h * 16 + q) * 16 + c) for q in range(16)], True)
            for m in range(8):
                y = h + n2 * m
                if y < ny:
                    a = dst + y * Mz + c
                    assert A2[a] is None
                    A2[a] = x16(v, m)
    assert all(a is not None for a in A2)
    assert np.abs(np.array(A2) / M - A).max() <= 1e-12 * np.abs(A).max()


@pytest.mark.parametrize("n2", [8, 12, 24])
def test_z16n_passes(n2):
    M = 16 * n2
    rng = np.random.default_rng(200 + n2)
    slot = lambda r, c: c * (17 * n2) + r + (r >> 4)        # noqa: E731
    nz, nl = M // 2 - 3, 21                                # a partial last block of 16 lines
    zp = (nz + 3) // 4 * 4
    t1 = rng.standard_normal(nl * zp)
    t2 = rng.standard_normal(nl * zp)
    f1 = rng.random(nl) < 0.6
    f2 = rng.random(nl) < 0.6
    f1[16:] = f2[16:] = False                              # the second block of lines holds no TERMA
    # forward: the per-CTA twiddle table at m N2 + j holds exp(-2 pi i j m / M)
    twf = [np.exp(-2j * np.pi * (i % n2) * (i // n2) / M) for i in range(M)]
    A = [None] * (nl * M)
    for bx in range((nl + 15) // 16):
        l0 = bx * 16
        if not any(f1[l0:l0 + 16]) and not any(f2[l0:l0 + 16]):
            for e in range(min(16, nl - l0) * M):
                assert A[l0 * M + e] is None
                A[l0 * M + e] = 0j
            continue
        xb = Exchange(16 * 17 * n2)
        for t in range(16 * n2):
            j, c = t % n2, t // n2
            l = l0 + c
            v = [0j] * 16
            for n1 in range(8):
                z = n2 * n1 + j
                if l < nl and z < nz:
                    v[n1] = complex(t1[l * zp + z] if f1[l] else 0.0, t2[l * zp + z] if f2[l] else 0.0)
            v = dft16(v, False, half_in=True)
            for m in range(16):
                xb.put(slot(16 * j + m, c), x16(v, m) * (twf[m * n2 + j] if m else 1))
        for t in range(256):
            k1, c = t & 15, t >> 4
            l = l0 + c
            zz = dft_n2([xb.get(slot(16 * j + k1, c)) for j in range(n2)], False)
            if l < nl:
                for k2 in range(n2):
                    assert A[l * M + k1 + 16 * k2] is None
                    A[l * M + k1 + 16 * k2] = zz[k2]
    assert all(a is not None for a in A)
    A = np.array(A).reshape(nl, M)
    lines = np.zeros((nl, M), complex)
    for l in range(nl):
        lines[l, :nz] = (t1[l * zp:l * zp + nz] if f1[l] else 0) + 1j * (t2[l * zp:l * zp + nz] if f2[l] else 0)
    assert np.abs(A - np.fft.fft(lines, axis=1)).max() <= 1e-12 * np.abs(A).max()
    # inverse: the per-CTA table at 16 j + k1 holds exp(-2 pi i j k1 / M)
    twa = [np.exp(-2j * np.pi * (i >> 4) * (i & 15) / M) for i in range(M)]
    d1 = [None] * (nl * nz)
    d2 = [None] * (nl * nz)
    for bx in range((nl + 15) // 16):
        l0 = bx * 16
        xb = Exchange(16 * 17 * n2)
        for t in range(256):
            k1, c = t & 15, t >> 4
            l = l0 + c
            a = [A[l, k1 + 16 * k2] if l < nl else 0j for k2 in range(n2)]
            zz = dft_n2(a, True)
            for j in range(n2):
                xb.put(slot(16 * j + k1, c), zz[j] * (np.conj(twa[16 * j + k1]) if j else 1))
        for t in range(16 * n2):
            j, c = t % n2, t // n2
            l = l0 + c
            v = dft16([xb.get(slot(16 * j + q, c)) for q in range(16)], True)
            if l < nl:
                for m in range(8):
                    z = j + n2 * m
                    if z < nz:
                        assert d1[l * nz + z] is None
                        d1[l * nz + z], d2[l * nz + z] = x16(v, m).real, x16(v, m).imag
    assert all(d is not None for d in d1)
    assert np.abs(np.array(d1) / M - np.where(np.repeat(f1, nz), np.concatenate([t1[l * zp:l * zp + nz] for l in range(nl)]), 0)).max() < 1e-12
    assert np.abs(np.array(d2) / M - np.where(np.repeat(f2, nz), np.concatenate([t2[l * zp:l * zp + nz] for l in range(nl)]), 0)).max() < 1e-12
