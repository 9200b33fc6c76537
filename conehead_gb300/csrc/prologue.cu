// Fused beam prologue: voxel blocking -> radiological depth -> off-axis
// distance -> fluence -> softening/horn -> TERMA, one thread per voxel.
//
// Follows conehead/conehead.py:71-120 (cuda_hit_test), :209-254
// (cuda_d_eff with cuda_dda_3d :123-206), :286-314 (cuda_oad), :320-360
// (cuda_fluence), :641-655 (softening/horn, host numpy float32) and
// :364-377 (cuda_terma).  The reference runs these as six launches with a
// host round trip after each; here they are one pass over the grid that
// writes only TERMA (plus the intermediates when asked).
//
// Exactness: blocked, d_eff, oad, f_soften and f_horn reproduce the
// reference's rounding bit for bit (float32 with float64 where Numba
// promotes, no FMA contraction).  Blocking samples are classified with a
// float32 projection first; a sample whose block cell is ambiguous within
// the float32 error bound (SAMPLE_DELTA cells) is recomputed with the exact
// float64 mirror, so GB300's low float64 rate is only paid at field edges.
// Fluence and TERMA run in float32 (reference: float64 fluence, float32
// TERMA) and are compared with a tolerance.

#include <algorithm>
#include <cstdio>

#include "ch_internal.cuh"

namespace ch {

constexpr float SAMPLE_DELTA = 0.05f;   // cells (0.1 mm) of float32 slack

// partial sums 0, 1/27, 1/27+1/27, ... accumulated in float64 as the
// reference does for a block value of exactly 1.0 and 3x3x3 samples
__constant__ double c_unit_partial[28];

// --------------------------------------------------------- block lookup --
// cell index i = floor(100 x) (x in cm, beam coordinates); the reference
// reads block_values[i + 1999] after checking i + 2000 in [0, 3999]; index
// -1 wraps to the last row/column.
__device__ __forceinline__ float cell_value(const BeamDev& b, int fi, int fk) {
  const int c0 = fi + 2000, c1 = fk + 2000;
  if (c0 < 0 || c0 > 3999 || c1 < 0 || c1 > 3999) return 0.0f;
  int r = c0 - 1, c = c1 - 1;
  if (r < 0) r += b.full_rows;
  if (c < 0) c += b.full_cols;
  r -= b.br0;
  c -= b.bc0;
  if (r < 0 || r >= b.brows || c < 0 || c >= b.bcols) return 0.0f;
  if (b.uniform) return 1.0f;
  return __ldg(b.block + (size_t)r * b.bcols + c);
}

// floor of a float32 cell coordinate as the reference stores it; values far
// outside the map (and NaN) land outside [-2000, 1999], where every cell reads 0
__device__ __forceinline__ int floor_cell(float v) {
  if (!(v == v)) return 1 << 24;
  return (int)floorf(fminf(fmaxf(v, -1.0e7f), 1.0e7f));
}

// Exact projection, float64 source arrays (conehead.py:25-47 + :109-116).
__device__ __forceinline__ bool project_exact_mixed(const BeamDev& b, const float* rd, float& px,
                                                    float& pz) {
  const double ndotu =
      dadd(dadd(dmul(b.vy[0], (double)rd[0]), dmul(b.vy[1], (double)rd[1])), dmul(b.vy[2], (double)rd[2]));
  if (fabs(ndotu) < 1e-6) return false;
  const double si = ddiv(-b.vyw, ndotu);
  float pp[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) pp[k] = d2f(dadd(dadd((double)b.srcf[k], dmul(si, (double)rd[k])), 0.0));
  px = d2f(dadd(dadd(dmul(b.m0[0], (double)pp[0]), dmul(b.m0[1], (double)pp[1])), dmul(b.m0[2], (double)pp[2])));
  pz = d2f(dadd(dadd(dmul(b.m2[0], (double)pp[0]), dmul(b.m2[1], (double)pp[1])), dmul(b.m2[2], (double)pp[2])));
  return true;
}

// Exact projection, float32 source arrays (all float32 arithmetic).
__device__ __forceinline__ bool project_exact_f32(const BeamDev& b, const float* rd, float& px,
                                                  float& pz) {
  const float ndotu = fadd(fadd(fmul(b.vyf[0], rd[0]), fmul(b.vyf[1], rd[1])), fmul(b.vyf[2], rd[2]));
  if (fabs((double)ndotu) < 1e-6) return false;
  const float si = fdiv(-b.vywf, ndotu);
  float pp[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) pp[k] = fadd(fadd(b.srcf[k], fmul(si, rd[k])), 0.0f);
  px = fadd(fadd(fmul(b.m0f[0], pp[0]), fmul(b.m0f[1], pp[1])), fmul(b.m0f[2], pp[2]));
  pz = fadd(fadd(fmul(b.m2f[0], pp[0]), fmul(b.m2f[1], pp[1])), fmul(b.m2f[2], pp[2]));
  return true;
}

// reference ray vector source - p, rounded to float32
__device__ __forceinline__ void ray_to_source(const BeamDev& b, const float* p, float* rd) {
  if (b.geom_f32) {
#pragma unroll
    for (int k = 0; k < 3; ++k) rd[k] = fsub(b.srcf[k], p[k]);
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) rd[k] = d2f(dsub(b.src[k], (double)p[k]));
  }
}

__device__ __forceinline__ bool project_exact(const BeamDev& b, const float* rd, float& px, float& pz) {
  return b.geom_f32 ? project_exact_f32(b, rd, px, pz) : project_exact_mixed(b, rd, px, pz);
}

// Exact transmission of one sub-sample (reference path end to end).  Kept
// out of line: it is rare, and inlining it at every sample site would bloat
// the kernel past the instruction cache.
// Block cell (floor(100 px), floor(100 pz)) of one sub-sample by the exact
// reference arithmetic; false (and bad = 1) for a ray parallel to the plane.
__device__ __forceinline__ bool sample_cell_exact(const BeamDev& b, const GridDev& g, const float* pos,
                                                  const float* off, int ix, int iy, int iz, int& bad, int& fi,
                                                  int& fk) {
  const int ii[3] = {ix, iy, iz};
  float ps[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // ((pos - s/2) + off/2) + off*i, exact in float64, one rounding
    const double v = dadd(dadd(dsub((double)pos[k], (double)g.spacing[k] * 0.5), (double)off[k] * 0.5),
                          dmul((double)off[k], (double)ii[k]));
    ps[k] = d2f(v);
  }
  float rd[3];
  ray_to_source(b, ps, rd);
  float px, pz;
  if (!project_exact(b, rd, px, pz)) {
    bad = 1;
    return false;
  }
  fi = floor_cell(fmul(px, 100.0f));
  fk = floor_cell(fmul(pz, 100.0f));
  return true;
}

__device__ __noinline__ float sample_exact(const BeamDev& b, const GridDev& g, const float* pos, const float* off,
                              int ix, int iy, int iz, int& bad) {
  int fi, fk;
  if (!sample_cell_exact(b, g, pos, off, ix, iy, iz, bad, fi, fk)) return 0.0f;
  return cell_value(b, fi, fk);
}

// ------------------------------------------------------------ blocking --
// Transmission of sub-sample (ix, iy, iz) at pos + (rx, ry, rz): float32
// projection, exact float64 mirror only when the block cell is ambiguous
// within SAMPLE_DELTA.
__device__ __forceinline__ float sample_value(const BeamDev& b, const GridDev& g, const float* pos,
                                              const float* off, float rx, float ry, float rz, int ix, int iy,
                                              int iz, int& bad) {
  const float p0 = pos[0] + rx, p1 = pos[1] + ry, p2 = pos[2] + rz;
  const float np_ = b.vyf[0] * p0 + b.vyf[1] * p1 + b.vyf[2] * p2;
  const float m0p = b.m0f[0] * p0 + b.m0f[1] * p1 + b.m0f[2] * p2;
  const float m2p = b.m2f[0] * p0 + b.m2f[1] * p1 + b.m2f[2] * p2;
  const float ndr = b.a_nS - np_;
  // the float32 error bound assumes a magnification SAD/depth below 5; closer
  // to the source plane (or behind it) take the exact path, which also
  // reports rays parallel to the blocking plane as the reference does
  if (!(fabsf(ndr) > 0.2f * fabsf(b.a_K))) return sample_exact(b, g, pos, off, ix, iy, iz, bad);
  const float si = __fdividef(b.a_K, ndr);
  const float ux = (b.a_c0 + si * (b.a_m0S - m0p)) * 100.0f;
  const float uz = (b.a_c2 + si * (b.a_m2S - m2p)) * 100.0f;
  const int i0 = floor_cell(ux - SAMPLE_DELTA), i1 = floor_cell(ux + SAMPLE_DELTA);
  const int k0 = floor_cell(uz - SAMPLE_DELTA), k1 = floor_cell(uz + SAMPLE_DELTA);
  float v = cell_value(b, i0, k0);
  if (i0 != i1 || k0 != k1) {
    const float v1 = cell_value(b, i1, k0), v2 = cell_value(b, i0, k1), v3 = cell_value(b, i1, k1);
    if (v1 != v || v2 != v || v3 != v) v = sample_exact(b, g, pos, off, ix, iy, iz, bad);
  }
  return v;
}

// General blocked fraction: any sample count, float32 source arrays, or
// transmission values other than 0 and 1 (float64, reference order
// acc = acc + v / S^3 over ix, iy, iz).
__device__ __noinline__ double blocked_general(const BeamDev& b, const GridDev& g, int S, const float* pos,
                                               int& bad) {
  float off[3];
  // f32(f64(s) / S) == fdiv(s, S): double rounding is innocuous for float32 operands
  for (int k = 0; k < 3; ++k) off[k] = fdiv(g.spacing[k], (float)S);
  const bool exact_all = b.geom_f32 != 0;
  double acc = 0.0;
  const double denom = (double)S * (double)S * (double)S;
  float last_v = -1.0f;
  double last_q = 0.0;
  for (int ix = 0; ix < S; ++ix)
    for (int iy = 0; iy < S; ++iy)
      for (int iz = 0; iz < S; ++iz) {
        float v;
        if (exact_all) {
          v = sample_exact(b, g, pos, off, ix, iy, iz, bad);
        } else {
          const float rx = off[0] * ((float)ix + 0.5f) - g.spacing[0] * 0.5f;
          const float ry = off[1] * ((float)iy + 0.5f) - g.spacing[1] * 0.5f;
          const float rz = off[2] * ((float)iz + 0.5f) - g.spacing[2] * 0.5f;
          v = sample_value(b, g, pos, off, rx, ry, rz, ix, iy, iz, bad);
        }
        if (v != last_v) {
          last_v = v;
          last_q = ddiv((double)v, denom);
        }
        acc = dadd(acc, last_q);
      }
  return acc;
}

// Blocked fraction of one voxel where it is decided without classifying the
// 3x3x3 samples one by one (returns false when they are needed): the general
// sum (other sample counts, float32 source arrays), and for a uniform jaw
// crop a voxel wholly inside or wholly outside the opening.
__device__ __forceinline__ bool blocked_quick(const BeamDev& b, const GridDev& g, int S, const float* pos, int& bad,
                                              double& out) {
  if (S != 3 || b.geom_f32) {
    out = blocked_general(b, g, S, pos, bad);
    return true;
  }
  float off[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) off[k] = fdiv(g.spacing[k], 3.0f);
  if (b.uniform) {
    // Fast test for a voxel wholly inside a jaw opening.  The samples lie in
    // the box of the extreme ones (offsets -s/3 and +s/3 per axis).  On the
    // source's side of the plane the projection through the source maps
    // segments to segments, so every sample's cell lies in the cell box of
    // the 8 corner projections, widened by the same float32 error bound as a
    // single sample.  The open cells of a uniform crop form a rectangle (the
    // -1 wrap at index -2000 excluded), so when both extreme cells of the box
    // are open every sample is open: blocked is the reference's sum of 27
    // ones.  Otherwise the samples are classified one by one.
    float umin = 3.0e38f, umax = -3.0e38f, wmin = 3.0e38f, wmax = -3.0e38f;
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float rx = off[0] * ((c & 1) ? 2.5f : 0.5f) - g.spacing[0] * 0.5f;
      const float ry = off[1] * ((c & 2) ? 2.5f : 0.5f) - g.spacing[1] * 0.5f;
      const float rz = off[2] * ((c & 4) ? 2.5f : 0.5f) - g.spacing[2] * 0.5f;
      const float p0 = pos[0] + rx, p1 = pos[1] + ry, p2 = pos[2] + rz;
      const float np_ = b.vyf[0] * p0 + b.vyf[1] * p1 + b.vyf[2] * p2;
      const float m0p = b.m0f[0] * p0 + b.m0f[1] * p1 + b.m0f[2] * p2;
      const float m2p = b.m2f[0] * p0 + b.m2f[1] * p1 + b.m2f[2] * p2;
      const float ndr = b.a_nS - np_;
      ok = ok && fabsf(ndr) > 0.2f * fabsf(b.a_K);
      const float si = __fdividef(b.a_K, ndr);
      const float ux = (b.a_c0 + si * (b.a_m0S - m0p)) * 100.0f;
      const float uz = (b.a_c2 + si * (b.a_m2S - m2p)) * 100.0f;
      umin = fminf(umin, ux);
      umax = fmaxf(umax, ux);
      wmin = fminf(wmin, uz);
      wmax = fmaxf(wmax, uz);
    }
    if (ok) {
      const int i0 = floor_cell(umin - SAMPLE_DELTA), i1 = floor_cell(umax + SAMPLE_DELTA);
      const int k0 = floor_cell(wmin - SAMPLE_DELTA), k1 = floor_cell(wmax + SAMPLE_DELTA);
      if (i0 > -2000 && k0 > -2000) {
        if (cell_value(b, i0, k0) == 1.0f && cell_value(b, i1, k1) == 1.0f) {
          out = c_unit_partial[27];
          return true;
        }
        // Wholly closed: the box misses the open rectangle of cells
        // i in [br0 - 1999, br0 + brows - 2000], k likewise (within the map's
        // [-1999, 1999]; the wrapped index -2000 is outside the box), so
        // every sample reads 0 and blocked is the reference's sum of zeros.
        const int oi0 = max(b.br0 - 1999, -1999), oi1 = min(b.br0 + b.brows - 2000, 1999);
        const int ok0 = max(b.bc0 - 1999, -1999), ok1 = min(b.bc0 + b.bcols - 2000, 1999);
        if (i1 < oi0 || i0 > oi1 || k1 < ok0 || k0 > ok1) {
          out = c_unit_partial[0];
          return true;
        }
      }
    }
  }
  return false;
}

// sample sidx = 9 ix + 3 iy + iz of the 3x3x3 set: its float32 offset from
// the voxel centre
__device__ __forceinline__ float sample_of(const BeamDev& b, const GridDev& g, const float* pos, const float* off,
                                           int sidx, int& bad) {
  const int ix = sidx / 9, iy = (sidx / 3) % 3, iz = sidx % 3;
  const float rx = off[0] * ((float)ix + 0.5f) - g.spacing[0] * 0.5f;
  const float ry = off[1] * ((float)iy + 0.5f) - g.spacing[1] * 0.5f;
  const float rz = off[2] * ((float)iz + 0.5f) - g.spacing[2] * 0.5f;
  return sample_value(b, g, pos, off, rx, ry, rz, ix, iy, iz, bad);
}

// blocked fraction of one voxel; the 3x3x3 jaw case (values 0 and 1 only)
// counts open samples and sums through the precomputed float64 partial sums
// (the reference's float64 sum of n ones and 27 - n zeros, in any order)
__device__ double blocked_fraction(const BeamDev& b, const GridDev& g, int S, const float* pos, int& bad) {
  double quick;
  if (blocked_quick(b, g, S, pos, bad, quick)) return quick;
  float off[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) off[k] = fdiv(g.spacing[k], 3.0f);
  int n_one = 0;
  bool other = false;
  // a rolled loop: one copy of the sample code keeps the kernel inside the
  // instruction cache (the float32 offsets only steer the classification,
  // whose ambiguous samples are recomputed exactly from ix, iy, iz)
#pragma unroll 1
  for (int sidx = 0; sidx < 27; ++sidx) {
    const float v = sample_of(b, g, pos, off, sidx, bad);
    n_one += v == 1.0f ? 1 : 0;
    other |= v != 0.0f && v != 1.0f;
  }
  if (!other) return c_unit_partial[n_one];
  return blocked_general(b, g, 3, pos, bad);
}

// blocked_fraction for the voxels of a converged warp: the quick decisions
// per lane, then, for each voxel that needs its samples classified, lanes
// 0..26 classify one sample each (a warp's field-edge voxels cost one sample
// time each instead of the whole warp running 27).  have: the lane holds a
// voxel at pos.
__device__ __forceinline__ double blocked_fraction_warp(const BeamDev& b, const GridDev& g, int S, bool have,
                                                        const float* pos, int& bad) {
  double out = 0.0;
  const bool need = have && !blocked_quick(b, g, S, pos, bad, out);
  unsigned m = __ballot_sync(0xffffffffu, need);
  if (!m) return out;
  const int lane = threadIdx.x & 31;
  float off[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) off[k] = fdiv(g.spacing[k], 3.0f);
  int n_one = 0;
  bool other = false;
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    float p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = __shfl_sync(0xffffffffu, pos[k], src);
    int sbad = 0;
    const float v = lane < 27 ? sample_of(b, g, p, off, lane, sbad) : 0.0f;
    const unsigned ones = __ballot_sync(0xffffffffu, v == 1.0f);
    const unsigned oth = __ballot_sync(0xffffffffu, v != 0.0f && v != 1.0f);
    const unsigned bd = __ballot_sync(0xffffffffu, sbad != 0);
    if (lane == src) {
      n_one = __popc(ones);
      other = oth != 0;
      if (bd) bad = 1;
    }
  }
  if (need) out = other ? blocked_general(b, g, 3, pos, bad) : c_unit_partial[n_one];
  return out;
}

// ------------------------------------------------------------------ DDA --
// radiological depth from voxel (x, y, z) toward the source (cuda_d_eff).
// The walk is generated UNROLL steps at a time so their density loads are
// in flight together; the float32 accumulation keeps the reference order.
constexpr int DDA_UNROLL = 8;

__device__ float radiological_depth(const float* __restrict__ rho, const GridDev& g, int x, int y, int z,
                                    const float* rd) {
  const float mag = __fsqrt_rn(fadd(fadd(fmul(rd[0], rd[0]), fmul(rd[1], rd[1])), fmul(rd[2], rd[2])));
  int s0, s1, s2;
  float t0, t1, t2, d0, d1, d2;
  dda_axis(fdiv(rd[0], mag), g.spacing[0], s0, t0, d0);
  dda_axis(fdiv(rd[1], mag), g.spacing[1], s1, t1, d1);
  dda_axis(fdiv(rd[2], mag), g.spacing[2], s2, t2, d2);
  const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
  // linear index of the density the reference reads at (x, y, z) and its
  // step along each grid axis (x and y swapped when swap_xy)
  // (volumes are limited to < 2^31 voxels by the host, so 32-bit indices)
  const int st0 = g.swap_xy ? n2 : n1 * n2;
  const int st1 = g.swap_xy ? n0 * n2 : n2;
  int idx = g.swap_xy ? (y * n0 + x) * n2 + z : (x * n1 + y) * n2 + z;
  const int dx = s0 * st0, dy = s1 * st1, dz = s2;
  // steps each axis may still take before the walk leaves the grid
  int left0 = s0 > 0 ? n0 - 1 - x : x, left1 = s1 > 0 ? n1 - 1 - y : y, left2 = s2 > 0 ? n2 - 1 - z : z;
  float deff = 0.0f, tprev = 0.0f;   // the first step adds rho * (t - 0), i.e. rho * t exactly
  bool inside = true;
  while (inside) {
    int vi[DDA_UNROLL];
    float tv[DDA_UNROLL];
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < DDA_UNROLL; ++q) {
      if (inside) {
        vi[q] = idx;
        const bool a01 = t0 < t1, s0 = a01 && t0 < t2, s1 = !a01 && t1 < t2;
        tv[q] = s0 ? t0 : (s1 ? t1 : t2);
        if (s0) {
          t0 = fadd(t0, d0);
          idx += dx;
          inside = --left0 >= 0;
        } else if (s1) {
          t1 = fadd(t1, d1);
          idx += dy;
          inside = --left1 >= 0;
        } else {
          t2 = fadd(t2, d2);
          idx += dz;
          inside = --left2 >= 0;
        }
        cnt = q + 1;
      }
    }
    float r[DDA_UNROLL];
#pragma unroll
    for (int q = 0; q < DDA_UNROLL; ++q) r[q] = q < cnt ? __ldg(rho + vi[q]) : 0.0f;
#pragma unroll
    for (int q = 0; q < DDA_UNROLL; ++q) {
      if (q < cnt) {
        deff = fadd(deff, fmul(r[q], fsub(tv[q], tprev)));
        tprev = tv[q];
      }
    }
  }
  return deff;
}

// ------------------------------------------------------------ kernels --
// Whole-line rejection for the cull.  Along an (x, y) line the voxel centres
// lie on one segment.  While the depth stays positive, the projected
// coordinates xb(z), zb(z) and the lateral ratio are ratios of linear
// functions of z without a pole, hence monotone: their ranges over the line
// are spanned by the two end voxels, and 1/depth and the lateral ratio (and
// so the per-voxel margin) are bounded by their largest end values.  Depth
// is linear, so its minimum is at an end too.  True only when no voxel of
// the line can pass the per-voxel test below; 0.01 cm on top of the margin
// covers the float32 rounding of both tests (about 1e-5 cm here).
__device__ __forceinline__ bool line_outside(const GridDev& g, const BeamDev& b, float px, float py) {
  // every lane of the warp tests the same line: even lanes project its first
  // voxel, odd lanes its last, and one shuffle step combines the two
  const unsigned full = 0xffffffffu;
  const int e = threadIdx.x & 1;
  const float kk = fabsf(b.a_K);
  const float pz = voxel_centre(g.origin[2], g.spacing[2], e ? g.n[2] - 1 : 0);
  const float np_ = b.vyf[0] * px + b.vyf[1] * py + b.vyf[2] * pz;
  const float m0p = b.m0f[0] * px + b.m0f[1] * py + b.m0f[2] * pz;
  const float m2p = b.m2f[0] * px + b.m2f[1] * py + b.m2f[2] * pz;
  const float depth = np_ - b.a_nS;
  const bool ok = depth > 0.2f * kk;
  // near or behind the source plane at either end: test per voxel
  if (!(ok && __shfl_xor_sync(full, (int)ok, 1))) return false;
  const float inv = 1.0f / depth;
  const float si = -b.a_K * inv;
  const float xb = b.a_c0 + si * (b.a_m0S - m0p);
  const float zb = b.a_c2 + si * (b.a_m2S - m2p);
  const float lat = fmaxf(fabsf(b.a_m0S - m0p), fabsf(b.a_m2S - m2p)) * inv;
  const float xb2 = __shfl_xor_sync(full, xb, 1), zb2 = __shfl_xor_sync(full, zb, 1);
  const float inv_max = fmaxf(inv, __shfl_xor_sync(full, inv, 1));
  const float lat_max = fmaxf(lat, __shfl_xor_sync(full, lat, 1));
  const float xlo = fminf(xb, xb2), xhi = fmaxf(xb, xb2), zlo = fminf(zb, zb2), zhi = fmaxf(zb, zb2);
  const float M = b.cull_margin_k * kk * inv_max * (1.0f + lat_max) + 0.02f;
  return xhi < b.cx_lo - M || xlo > b.cx_hi + M || zhi < b.cz_lo - M || zlo > b.cz_hi + M;
}

// Pass 1, every voxel: zero TERMA and keep the voxels the beam may reach
// (all voxels when intermediates are requested) on a compact list, so the
// blocking/depth/TERMA pass runs on full warps.
// One warp per (x, y) line of the grid, lanes along z: the index arithmetic
// runs once per line and the zeroing of TERMA is coalesced.
// zero_all = 0: TERMA is zeroed only on lines with listed voxels, and
// line_any (if set) records which lines those are.
__device__ __forceinline__ void cull_line(const GridDev& g, const BeamDev& b, float* __restrict__ T,
                                          const Inter& inter, int all_voxels, int* __restrict__ list_count,
                                          int* __restrict__ list_v, int line, unsigned char* line_any = nullptr,
                                          int zero_all = 1) {
  // volumes hold fewer than 2^31 voxels (checked on the host)
  if (line >= g.n[0] * g.n[1]) return;   // whole warp
  const int lane = threadIdx.x & 31;
  const int x = line / g.n[1], y = line - x * g.n[1];
  const float px = voxel_centre(g.origin[0], g.spacing[0], x);
  const float py = voxel_centre(g.origin[1], g.spacing[1], y);
  float* Tl = T + ((size_t)x * g.n[1] + y) * g.zp;
  // a line the beam cannot reach lists nothing (intermediates of every voxel
  // are written by the per-voxel loop, so it runs whenever they are asked)
  const bool no_inter = !inter.blocked && !inter.d_eff && !inter.oad && !inter.fluence && !inter.f_soften &&
                        !inter.f_horn && !inter.terma;
  if (b.cull_enable && !all_voxels && no_inter && line_outside(g, b, px, py)) {
    if (zero_all)
      for (int z = lane; z < g.n[2]; z += 32) Tl[z] = 0.0f;
    if (line_any && lane == 0) line_any[line] = 0;
    return;
  }
  bool any = false;
  for (int z0 = 0; z0 < g.n[2]; z0 += 32) {
    const int z = z0 + lane;
    const bool live = z < g.n[2];
    const int v = line * g.n[2] + z;
    bool keep = false;
    if (live) {
      float pos[3];
      pos[0] = px;
      pos[1] = py;
      pos[2] = voxel_centre(g.origin[2], g.spacing[2], z);
      bool candidate = true;
      if (b.cull_enable) {
        const float np_ = b.vyf[0] * pos[0] + b.vyf[1] * pos[1] + b.vyf[2] * pos[2];
        const float m0p = b.m0f[0] * pos[0] + b.m0f[1] * pos[1] + b.m0f[2] * pos[2];
        const float m2p = b.m2f[0] * pos[0] + b.m2f[1] * pos[1] + b.m2f[2] * pos[2];
        const float ndr = b.a_nS - np_;   // n . (S - p) = -depth
        const float depth = -ndr;
        if (depth > 0.2f * fabsf(b.a_K)) {
          // one fast reciprocal: its ~2 ulp error is far inside the 0.01 cm
          // margin, so the candidate set stays a superset of the beam
          const float inv_depth = __fdividef(1.0f, depth);
          const float si = -b.a_K * inv_depth;
          const float xb = b.a_c0 + si * (b.a_m0S - m0p);
          const float zb = b.a_c2 + si * (b.a_m2S - m2p);
          const float lat = fmaxf(fabsf(b.a_m0S - m0p), fabsf(b.a_m2S - m2p)) * inv_depth;
          const float margin = b.cull_margin_k * fabsf(b.a_K) * inv_depth * (1.0f + lat) + 0.01f;
          if (xb < b.cx_lo - margin || xb > b.cx_hi + margin || zb < b.cz_lo - margin ||
              zb > b.cz_hi + margin)
            candidate = false;
        }
      }
      keep = candidate || all_voxels;
      if (zero_all) Tl[z] = 0.0f;
      if (!keep) {
        if (inter.blocked) inter.blocked[v] = 0.0;
        if (inter.d_eff) inter.d_eff[v] = 0.0f;
        if (inter.oad) inter.oad[v] = 0.0f;
        if (inter.fluence) inter.fluence[v] = 0.0f;
        if (inter.f_soften) inter.f_soften[v] = 1.0f;
        if (inter.f_horn) inter.f_horn[v] = 1.0f;
        if (inter.terma) inter.terma[v] = 0.0f;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (m) {
      any = true;
      int base = 0;
      if (lane == 0) base = atomicAdd(list_count, __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (keep) list_v[base + __popc(m & ((1u << lane) - 1u))] = v;
    }
  }
  if (!zero_all && any)
    for (int z = lane; z < g.n[2]; z += 32) Tl[z] = 0.0f;
  if (line_any && lane == 0) line_any[line] = any ? 1 : 0;
}

__global__ void __launch_bounds__(256) cull_kernel(GridDev g, BeamDev b, float* __restrict__ T, Inter inter,
                                                   int all_voxels, int* __restrict__ list_count,
                                                   int* __restrict__ list_v) {
  cull_line(g, b, T, inter, all_voxels, list_count, list_v, (blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

// this CTA's beam record (blockIdx.y) copied into shared memory
__device__ __forceinline__ void load_record(const PrologueBeam* __restrict__ recs, PrologueBeam& R) {
  static_assert(sizeof(PrologueBeam) % 4 == 0 && sizeof(PrologueBeam) <= 4 * 1024, "record copy");
  const int* src = reinterpret_cast<const int*>(recs + blockIdx.y);
  int* dst = reinterpret_cast<int*>(&R);
  for (int i = threadIdx.x; i < (int)(sizeof(PrologueBeam) / 4); i += blockDim.x) dst[i] = __ldg(src + i);
  __syncthreads();
}

// every beam of a batch in one launch: blockIdx.y = beam
__global__ void __launch_bounds__(256) cull_batch_kernel(const PrologueBeam* __restrict__ recs) {
  __shared__ PrologueBeam R;
  load_record(recs, R);
  cull_line(R.g, R.b, R.T, Inter{}, 0, R.aabb + 6, R.list_v, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
            R.line_any, R.zero_all);
}

// Pass 2, listed voxels: blocked fraction, then (where the beam is not
// fully blocked, or for every voxel when intermediates are requested)
// radiological depth, oad, fluence, softening/horn and TERMA; TERMA support
// box for the cone stage.
// Entry e of a beam's list of count voxels; every lane of the warp calls it
// (the blocking classification and the box reduction are warp-wide).
__device__ __forceinline__ void terma_entry(const float* __restrict__ rho, const GridDev& g, const BeamDev& b,
                                            const SettingsDev& s, float* __restrict__ T, const Inter& inter,
                                            int all_voxels, int count, int e, const int* __restrict__ list_v,
                                            int* __restrict__ aabb, int* __restrict__ flags) {
  {
    const bool live = e < count;
    int x = 0, y = 0, z = 0, bad = 0, v = 0;
    float Tv = 0.0f;
    float pos[3] = {0.0f, 0.0f, 0.0f};
    if (live) {
      v = list_v[e];
      z = v % g.n[2];
      const int r = v / g.n[2];
      y = r % g.n[1];
      x = r / g.n[1];
      pos[0] = voxel_centre(g.origin[0], g.spacing[0], x);
      pos[1] = voxel_centre(g.origin[1], g.spacing[1], y);
      pos[2] = voxel_centre(g.origin[2], g.spacing[2], z);
    }
    // (every lane of the warp: the sample classification is shared)
    const double blocked = blocked_fraction_warp(b, g, s.samples, live, pos, bad);
    if (live) {
      if (inter.blocked) inter.blocked[v] = blocked;
      if (blocked == 0.0 && !all_voxels) {
        if (inter.terma) inter.terma[v] = 0.0f;
        goto next;
      }
      {
      float rd[3];
      ray_to_source(b, pos, rd);
      // ---- radiological depth (float32, exact mirror)
      const float deff = radiological_depth(rho, g, x, y, z, rd);
      // ---- off-axis distance (exact mirror)
      float px = 0.0f, pz = 0.0f;
      if (!project_exact(b, rd, px, pz)) bad = 1;
      const float oad = __fsqrt_rn(fadd(fmul(px, px), fmul(pz, pz)));
      // ---- fluence (float32 evaluation of the reference's float64 formula)
      const float mag = __fsqrt_rn(fadd(fadd(fmul(rd[0], rd[0]), fmul(rd[1], rd[1])), fmul(rd[2], rd[2])));
      const float sad = (float)b.sad;
      const float ratio = sad / mag;
      const float fpoint = s.sPri * (ratio * ratio);
      const float r_ann = oad * s.zAnn / sad;
      float fann = 0.0f;
      if (r_ann >= s.rInner && r_ann <= s.rOuter) {
        const float a = sad - s.zAnn, c = mag - s.zAnn;
        fann = s.sAnn * (a * a) / (c * c);
      }
      const float oadc = oad < 2.0f ? 2.0f : oad;
      const float r_exp = oadc * s.zExp / sad;
      const float ae = sad - s.zExp, ce = mag - s.zExp;
      const float fexp = s.sExp / r_exp * expf(-s.kExp * r_exp) * (ae * ae) / (ce * ce);
      const float fluence = (float)((double)(fpoint + fann + fexp) * blocked);
      // ---- softening and horn (reference host numpy, float32)
      float fs = 1.0f;
      if (oad < s.softLimit) fs = fdiv(1.0f, fsub(1.0f, fmul(s.softRatio, oad)));
      const float fh = fadd(1.0f, fmul(oad, s.hornRatio));
      // ---- TERMA (float32, reference order)
      float terma = 0.0f;
      for (int i = 0; i < s.n_energy; ++i) {
        const float ex = expf(fmul(fmul(-s.mu[i], fs), deff));
        terma = fadd(terma, fmul(fmul(fmul(fmul(fmul(s.w[i], fluence), ex), s.E[i]), s.mu[i]), fh));
      }
      Tv = d2f(dmul((double)terma, blocked));
      T[((size_t)x * g.n[1] + y) * g.zp + z] = Tv;
      if (inter.d_eff) inter.d_eff[v] = deff;
      if (inter.oad) inter.oad[v] = oad;
      if (inter.fluence) inter.fluence[v] = fluence;
      if (inter.f_soften) inter.f_soften[v] = fs;
      if (inter.f_horn) inter.f_horn[v] = fh;
      if (inter.terma) inter.terma[v] = Tv;
      }
    }
  next:
    // ---- support box of T != 0 (the reference skips T == 0 sources)
    const bool nz_ = live && Tv != 0.0f;
    const unsigned m = __ballot_sync(0xffffffffu, nz_);
    if (m) {
      int lo0 = nz_ ? x : INT_MAX, hi0 = nz_ ? x : INT_MIN;
      int lo1 = nz_ ? y : INT_MAX, hi1 = nz_ ? y : INT_MIN;
      int lo2 = nz_ ? z : INT_MAX, hi2 = nz_ ? z : INT_MIN;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lo0 = min(lo0, __shfl_xor_sync(0xffffffffu, lo0, o));
        hi0 = max(hi0, __shfl_xor_sync(0xffffffffu, hi0, o));
        lo1 = min(lo1, __shfl_xor_sync(0xffffffffu, lo1, o));
        hi1 = max(hi1, __shfl_xor_sync(0xffffffffu, hi1, o));
        lo2 = min(lo2, __shfl_xor_sync(0xffffffffu, lo2, o));
        hi2 = max(hi2, __shfl_xor_sync(0xffffffffu, hi2, o));
      }
      if ((threadIdx.x & 31) == 0) {
        atomicMin(aabb + 0, lo0); atomicMax(aabb + 1, hi0);
        atomicMin(aabb + 2, lo1); atomicMax(aabb + 3, hi1);
        atomicMin(aabb + 4, lo2); atomicMax(aabb + 5, hi2);
      }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, FLAG_PARALLEL_RAY);
  }
}

// The listed voxels of one beam, taken by n_ctas CTAs (this one is cta) in
// rounds of n_ctas * blockDim.x.
__device__ __forceinline__ void terma_body(const float* __restrict__ rho, const GridDev& g, const BeamDev& b,
                                           const SettingsDev& s, float* __restrict__ T, const Inter& inter,
                                           int all_voxels, const int* __restrict__ list_count,
                                           const int* __restrict__ list_v, int* __restrict__ aabb,
                                           int* __restrict__ flags, int cta, int n_ctas) {
  const int count = *list_count;
  const int rounds = (count + blockDim.x * n_ctas - 1) / (blockDim.x * n_ctas);
  for (int it = 0; it < rounds; ++it)
    terma_entry(rho, g, b, s, T, inter, all_voxels, count, (it * n_ctas + cta) * blockDim.x + threadIdx.x,
                list_v, aabb, flags);
}

__global__ void __launch_bounds__(256) terma_kernel(const float* __restrict__ rho, GridDev g, BeamDev b,
                                                    SettingsDev s, float* __restrict__ T, Inter inter,
                                                    int all_voxels, const int* __restrict__ list_count,
                                                    const int* __restrict__ list_v, int* __restrict__ aabb,
                                                    int* __restrict__ flags) {
  terma_body(rho, g, b, s, T, inter, all_voxels, list_count, list_v, aabb, flags, blockIdx.x, gridDim.x);
}

// Every beam's listed voxels in one launch, in chunks of 32 (one per lane)
// that warps claim from one counter: claim c is chunk c - base of the beam
// whose chunks cover c, where base counts the chunks of the beams before it
// (entries 32 (c - base) .. 32 (c - base) + 31 of its list).  A warp that finishes
// early takes the next chunk of any beam, so the SMs end together however
// unequal the beams' lists and ray lengths are (a static share per CTA left
// the SMs idle for a sixth of the launch).  Each warp keeps the record of
// its current beam in its own shared slot and copies the next one when the
// claimed chunk moves on to another beam; the claims of one warp increase,
// so the beam search walks forward only.
constexpr int TERMA_WARPS = 8;   // 256 threads

__global__ void __launch_bounds__(256, 3) terma_batch_kernel(const PrologueBeam* __restrict__ recs, int n_beams,
                                                          int* __restrict__ flags, int* __restrict__ work) {
  __shared__ PrologueBeam Rw[TERMA_WARPS];
  static_assert(sizeof(PrologueBeam) % 4 == 0, "record copy");
  const int lane = threadIdx.x & 31;
  PrologueBeam& R = Rw[threadIdx.x >> 5];
  int cur = -1, beam = 0, base = 0, count = 0;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    // chunks of beam b: ceil(list count / 32); the counts were written by the cull launch
    while (beam < n_beams) {
      count = recs[beam].aabb[6];
      const int chunks = (count + 31) >> 5;
      if (c < base + chunks) break;
      base += chunks;
      ++beam;
    }
    if (beam >= n_beams) break;   // whole warp
    if (beam != cur) {
      __syncwarp();
      const int* src = reinterpret_cast<const int*>(recs + beam);
      int* dst = reinterpret_cast<int*>(&R);
      for (int i = lane; i < (int)(sizeof(PrologueBeam) / 4); i += 32) dst[i] = __ldg(src + i);
      __syncwarp();
      cur = beam;
    }
    terma_entry(R.rho, R.g, R.b, R.s, R.T, Inter{}, 0, count, ((c - base) << 5) + lane, R.list_v, R.aabb, flags);
  }
}

// ----------------------------------------------------- beamlet adjoint --
// Beamlet holding block cell (fi, fk) under the lookup rule of cell_value
// (cell + 1999, index -1 wrapping to the last row/column), or -1.
__device__ __forceinline__ int beamlet_of(const BeamDev& b, const BeamletDev& bl, int fi, int fk) {
  const int c0 = fi + 2000, c1 = fk + 2000;
  if (c0 < 0 || c0 > 3999 || c1 < 0 || c1 > 3999) return -1;
  int r = c0 - 1, c = c1 - 1;
  if (r < 0) r += b.full_rows;
  if (c < 0) c += b.full_cols;
  r -= bl.r0;
  c -= bl.c0;
  if (r < 0 || c < 0 || r >= bl.rows * bl.cell_rows || c >= bl.cols * bl.cell_cols) return -1;
  return (r / bl.cell_rows) * bl.cols + c / bl.cell_cols;
}

// Beamlet of sub-sample (ix, iy, iz): the float32 projection decides when
// every cell within SAMPLE_DELTA of it lies in one beamlet, otherwise the
// exact float64 mirror finds the reference's cell.  (The forward pass may
// settle a sample on value alone; the derivative needs the beamlet.)
__device__ int sample_beamlet(const BeamDev& b, const BeamletDev& bl, const GridDev& g, const float* pos,
                              const float* off, float rx, float ry, float rz, int ix, int iy, int iz, int& bad) {
  if (!b.geom_f32) {
    const float p0 = pos[0] + rx, p1 = pos[1] + ry, p2 = pos[2] + rz;
    const float np_ = b.vyf[0] * p0 + b.vyf[1] * p1 + b.vyf[2] * p2;
    const float m0p = b.m0f[0] * p0 + b.m0f[1] * p1 + b.m0f[2] * p2;
    const float m2p = b.m2f[0] * p0 + b.m2f[1] * p1 + b.m2f[2] * p2;
    const float ndr = b.a_nS - np_;
    if (fabsf(ndr) > 0.2f * fabsf(b.a_K)) {
      const float si = __fdividef(b.a_K, ndr);
      const float ux = (b.a_c0 + si * (b.a_m0S - m0p)) * 100.0f;
      const float uz = (b.a_c2 + si * (b.a_m2S - m2p)) * 100.0f;
      const int i0 = floor_cell(ux - SAMPLE_DELTA), i1 = floor_cell(ux + SAMPLE_DELTA);
      const int k0 = floor_cell(uz - SAMPLE_DELTA), k1 = floor_cell(uz + SAMPLE_DELTA);
      const int id = beamlet_of(b, bl, i0, k0);
      if ((i0 == i1 && k0 == k1) ||
          (beamlet_of(b, bl, i1, k0) == id && beamlet_of(b, bl, i0, k1) == id && beamlet_of(b, bl, i1, k1) == id))
        return id;
    }
  }
  int fi, fk;
  if (!sample_cell_exact(b, g, pos, off, ix, iy, iz, bad, fi, fk)) return -1;
  return beamlet_of(b, bl, fi, fk);
}

// dL/dw for blocked(v) = sum_s w[beamlet(s)] / S^3 and T = blocked^2 * H
// (fluence and TERMA each carry one factor of blocked): over the voxels of
// the prologue's list with T != 0, g(v) = tbar(v) * 2 T(v) / blocked(v) is
// spread over the beamlets of its S^3 sub-samples.  Per-CTA float64
// histograms in shared memory, one global float64 add per touched beamlet.
__global__ void __launch_bounds__(256) blocked_adjoint_kernel(GridDev g, BeamDev b, BeamletDev bl, int S,
                                                              const float* __restrict__ T,
                                                              const float* __restrict__ tbar,
                                                              const int* __restrict__ list_count,
                                                              const int* __restrict__ list_v,
                                                              double* __restrict__ wbar, int* __restrict__ flags) {
  extern __shared__ double hist[];
  const int nb = bl.rows * bl.cols;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const int count = *list_count;
  int bad = 0;
  float off[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) off[k] = fdiv(g.spacing[k], (float)S);
  const double inv = 1.0 / ((double)S * (double)S * (double)S);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const int v = list_v[e];
    const int z = v % g.n[2];
    const int r = v / g.n[2];
    const int y = r % g.n[1];
    const int x = r / g.n[1];
    const float t = T[((size_t)x * g.n[1] + y) * g.zp + z];
    const float tb = tbar[v];
    if (t == 0.0f || tb == 0.0f) continue;
    float pos[3];
    pos[0] = voxel_centre(g.origin[0], g.spacing[0], x);
    pos[1] = voxel_centre(g.origin[1], g.spacing[1], y);
    pos[2] = voxel_centre(g.origin[2], g.spacing[2], z);
    const double blocked = blocked_fraction(b, g, S, pos, bad);
    if (!(blocked > 0.0)) continue;
    const double gv = (double)tb * 2.0 * (double)t / blocked * inv;
    for (int ix = 0; ix < S; ++ix)
      for (int iy = 0; iy < S; ++iy)
        for (int iz = 0; iz < S; ++iz) {
          const float rx = off[0] * ((float)ix + 0.5f) - g.spacing[0] * 0.5f;
          const float ry = off[1] * ((float)iy + 0.5f) - g.spacing[1] * 0.5f;
          const float rz = off[2] * ((float)iz + 0.5f) - g.spacing[2] * 0.5f;
          const int id = sample_beamlet(b, bl, g, pos, off, rx, ry, rz, ix, iy, iz, bad);
          if (id >= 0) atomicAdd(hist + id, gv);
        }
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, FLAG_PARALLEL_RAY);
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    if (hist[i] != 0.0) atomicAdd(wbar + i, hist[i]);
}

cudaError_t launch_blocked_adjoint(const GridDev& g, const BeamDev& b, const BeamletDev& bl, int S, const float* T,
                                   const float* tbar, const int* list_count, const int* list_v, double* wbar,
                                   int n_sm, int* flags, cudaStream_t st) {
  const size_t smem = (size_t)bl.rows * bl.cols * sizeof(double);
  if (smem > (48u << 10)) {
    // per device and cheap: set it on every launch that needs it
    cudaError_t e = cudaFuncSetAttribute(blocked_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  blocked_adjoint_kernel<<<n_sm * 2, 256, smem, st>>>(g, b, bl, S, T, tbar, list_count, list_v, wbar, flags);
  return cudaGetLastError();
}

void upload_unit_partials() {
  double p[28];
  p[0] = 0.0;
  const double q = 1.0 / 27.0;
  for (int i = 1; i < 28; ++i) p[i] = p[i - 1] + q;
  cudaMemcpyToSymbol(c_unit_partial, p, sizeof(p));
}

void launch_prologue(const float* rho, const GridDev& g, const BeamDev& b, const SettingsDev& s, float* T,
                     const Inter& inter, int all_voxels, int* aabb, int* list_v, int n_sm, int* flags,
                     cudaStream_t st, int ctas_per_sm) {
  const long long N = (long long)g.n[0] * g.n[1] * g.n[2];
  const int threads = 256;
  const long long lines = (long long)g.n[0] * g.n[1];
  int* list_count = aabb + 6;
  cull_kernel<<<(unsigned)((lines + 7) / 8), threads, 0, st>>>(g, b, T, inter, all_voxels, list_count, list_v);
  const long long want = (N + threads - 1) / threads;
  const long long cap = (long long)n_sm * ctas_per_sm;
  const int grid = (int)(want < cap ? want : cap);
  terma_kernel<<<grid > 0 ? grid : 1, threads, 0, st>>>(rho, g, b, s, T, inter, all_voxels, list_count, list_v,
                                                        aabb, flags);
}

// Batched prologue (no intermediates): one cull launch over every beam's grid
// and one TERMA launch in which each beam's list is shared by the same number
// of CTAs, so all beams run together and no beam leaves a tail.
void launch_prologue_batch(const PrologueBeam* recs, int n_beams, long long max_voxels, long long max_lines,
                           int n_sm, int* flags, int* work, cudaStream_t st, int ctas_per_sm) {
  const int threads = 256;
  cull_batch_kernel<<<dim3((unsigned)((max_lines + 7) / 8), n_beams), threads, 0, st>>>(recs);
  // persistent: at most the resident CTAs (3 per SM at 80 registers), fewer
  // for small batches; the warps share all beams' chunks
  const long long want = ((long long)n_beams * max_voxels + threads - 1) / threads;
  const long long cap = (long long)n_sm * std::min(ctas_per_sm, 3);
  terma_batch_kernel<<<(unsigned)std::max(1ll, std::min(cap, want)), threads, 0, st>>>(recs, n_beams, flags, work);
}

__global__ void init_scratch_kernel(int* aabb, int n_beams, int* counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // per beam: lo/hi pairs of the TERMA box, then the prologue list count
  if (i < n_beams * 8) aabb[i] = (i % 8 >= 6) ? 0 : ((i % 2 == 0) ? INT_MAX : INT_MIN);
  if (i < 8) counters[i] = 0;
}

void launch_init_scratch(int* aabb, int n_beams, int* counters, cudaStream_t st) {
  const int n = n_beams * 8 > 8 ? n_beams * 8 : 8;
  init_scratch_kernel<<<(n + 255) / 256, 256, 0, st>>>(aabb, n_beams, counters);
}

}  // namespace ch
