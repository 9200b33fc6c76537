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
