# cython: language_level=3
# Test-only shim: exposes conehead's own nogil Cython DDA (conehead/dda_3d_c.pyx,
# compiled unmodified from the reference sources by oracle/build_ref.py) to
# Python so the oracle's and the GPU's DDA traces can be pinned against it.
cimport numpy as cnp
from conehead.dda_3d_c cimport dda_3d_c, result
from conehead.vector cimport vector_init, vector_get, vector_free


def trace(direction, shape, start, spacing):
    """Run dda_3d_c once; return (voxels list of (x, y, z), t-values list)."""
    cdef cnp.float64_t d[3]
    cdef cnp.int32_t n[3]
    cdef cnp.int32_t s[3]
    cdef cnp.float64_t sp[3]
    cdef result r
    cdef int i
    cdef cnp.int32_t* v
    for i in range(3):
        d[i] = direction[i]
        n[i] = shape[i]
        s[i] = start[i]
        sp[i] = spacing[i]
    vector_init(&r.intersection_t_values)
    vector_init(&r.voxels_traversed)
    dda_3d_c(d, n, s, sp, &r)
    voxels = []
    tvals = []
    for i in range(r.voxels_traversed.size):
        v = <cnp.int32_t*>vector_get(&r.voxels_traversed, i)
        voxels.append((v[0], v[1], v[2]))
        tvals.append((<cnp.float64_t*>vector_get(&r.intersection_t_values, i))[0])
    vector_free(&r.intersection_t_values)
    vector_free(&r.voxels_traversed)
    return voxels, tvals
