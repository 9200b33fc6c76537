// Collapsed-cone stage as a spectral convolution (replaces the per-voxel
// scatter of conehead/conehead.py:385-488 by the same linear operator).
//
// Every walk from a voxel centre visits the same offsets O_u[m] with the same
// weights w_u[m], so the cone stage is one linear convolution with a fixed
// stencil:
//     dose(v) = sum_s T(s) S(v - s),   S(o) = sum_u sum_m w_u[m] [O_u[m] = o].
// Walks stop where they leave the grid, i.e. only |o_k| <= n_k - 1 connects
// two voxels of the grid, so a circular convolution of period
// M_k >= 2 n_k - 1 on each axis equals the linear one on the grid:
//     dose = IFFT( FFT(T) . S^ ),   S^ = FFT(S) / (Mx My Mz),
// with S^ computed once per grid shape and kernel.  Two beams share one
// complex transform: TERMA of one is the real part, of the other the
// imaginary part; S is real, so their doses come back as the two parts.
//
// Each of the five passes over a pair of beams is a batch of 1-D FFTs of
// period M = 2^a or 3 * 2^a (the smallest >= 2n - 1, at least 16) along one
// axis.  A CTA holds up to 4096 complex values (L lines, L the largest power
// of two with L M <= 4096) in shared memory, element (i, line c) at
// i * L + (c ^ (i mod L)) so that both line-major and index-major sweeps are
// free of bank conflicts, and runs Stockham stages of radix 16, 3, 4 and 2
// with twiddles from a host-built table.  The passes skip the zero padding:
//   z forward  TERMA pair [nx][ny][nz] (pitch zp)  -> A [nx][ny][Mz]
//   y forward  A (y < ny)                          -> B [nx][My][Mz]
//   x          B (x < nx): forward, times S^, inverse, x < nx kept (in place)
//   y inverse  B                                   -> A (y < ny)
//   z inverse  A                                   -> dose pair [nx][ny][nz]
// Every global sweep is coalesced: lines along z are read and written along
// z, lines along y and x are taken in blocks of L consecutive kz.

#include <algorithm>
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "ch_internal.cuh"

namespace ch {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ int swz(int i, int c, int L) { return i * L + (c ^ (i & (L - 1))); }

// 4-point DFT in place (forward: X1 = d02 - i d13; inverse: d02 + i d13)
template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 s02 = make_float2(a0.x + a2.x, a0.y + a2.y), d02 = make_float2(a0.x - a2.x, a0.y - a2.y);
  const float2 s13 = make_float2(a1.x + a3.x, a1.y + a3.y), d13 = make_float2(a1.x - a3.x, a1.y - a3.y);
  const float2 mi = INV ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
  a0 = make_float2(s02.x + s13.x, s02.y + s13.y);
  a1 = make_float2(d02.x + mi.x, d02.y + mi.y);
  a2 = make_float2(s02.x - s13.x, s02.y - s13.y);
  a3 = make_float2(d02.x - mi.x, d02.y - mi.y);
}

// v times exp(-+i theta) given (cos theta, sin theta)
template <bool INV>
__device__ __forceinline__ float2 rot(float2 v, float c, float s) {
  const float sn = INV ? s : -s;
  return make_float2(v.x * c - v.y * sn, v.x * sn + v.y * c);
}

// 16-point DFT in place as 4 x 4: element r = 4a + b, output k = k1 + 4 k2.
// DFT4 over a for each b, times exp(-+2 pi i b k1 / 16), DFT4 over b for each
// k1; X[k1 + 4 k2] ends in v[4 k1 + k2].
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&v)[16]) {
  constexpr float C1 = 0.92387953251128674f;   // cos(pi/8)
  constexpr float S1 = 0.38268343236508977f;   // sin(pi/8)
  constexpr float R2 = 0.70710678118654752f;   // cos(pi/4)
#pragma unroll
  for (int b = 0; b < 4; ++b) dft4<INV>(v[b], v[4 + b], v[8 + b], v[12 + b]);
  v[5] = rot<INV>(v[5], C1, S1);     // b k1 = 1
  v[9] = rot<INV>(v[9], R2, R2);     // 2
  v[13] = rot<INV>(v[13], S1, C1);   // 3
  v[6] = rot<INV>(v[6], R2, R2);     // 2
  v[10] = INV ? make_float2(-v[10].y, v[10].x) : make_float2(v[10].y, -v[10].x);   // times -+i   // 4
  v[14] = rot<INV>(v[14], -R2, R2);  // 6
  v[7] = rot<INV>(v[7], S1, C1);     // 3
  v[11] = rot<INV>(v[11], -R2, R2);  // 6
  v[15] = rot<INV>(v[15], -C1, -S1); // 9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// dft16 with v[8..15] = 0 (the upper half of a zero-padded input): the first
// DFT4s see two inputs
template <bool INV>
__device__ __forceinline__ void dft16_half_in(float2 (&v)[16]) {
  constexpr float C1 = 0.92387953251128674f;
  constexpr float S1 = 0.38268343236508977f;
  constexpr float R2 = 0.70710678118654752f;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const float2 a0 = v[b], a1 = v[4 + b];
    const float2 mi = INV ? make_float2(-a1.y, a1.x) : make_float2(a1.y, -a1.x);   // -+i a1
    v[b] = make_float2(a0.x + a1.x, a0.y + a1.y);
    v[4 + b] = make_float2(a0.x + mi.x, a0.y + mi.y);
    v[8 + b] = make_float2(a0.x - a1.x, a0.y - a1.y);
    v[12 + b] = make_float2(a0.x - mi.x, a0.y - mi.y);
  }
  v[5] = rot<INV>(v[5], C1, S1);
  v[9] = rot<INV>(v[9], R2, R2);
  v[13] = rot<INV>(v[13], S1, C1);
  v[6] = rot<INV>(v[6], R2, R2);
  v[10] = INV ? make_float2(-v[10].y, v[10].x) : make_float2(v[10].y, -v[10].x);   // times -+i
  v[14] = rot<INV>(v[14], -R2, R2);
  v[7] = rot<INV>(v[7], S1, C1);
  v[11] = rot<INV>(v[11], -R2, R2);
  v[15] = rot<INV>(v[15], -C1, -S1);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// 3-point DFT in place: X0 = a + s, X1,2 = a - s/2 -+ i (sqrt 3 / 2) d with
// s = b + c, d = b - c (forward sign -, inverse +)
template <bool INV>
__device__ __forceinline__ void dft3(float2& a, float2& b, float2& c) {
  constexpr float H = 0.86602540378443865f;   // sqrt(3) / 2
  const float2 s = make_float2(b.x + c.x, b.y + c.y), d = make_float2(b.x - c.x, b.y - c.y);
  const float2 t = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
  const float2 u = INV ? make_float2(-H * d.y, H * d.x) : make_float2(H * d.y, -H * d.x);
  a = make_float2(a.x + s.x, a.y + s.y);
  b = make_float2(t.x + u.x, t.y + u.y);
  c = make_float2(t.x - u.x, t.y - u.y);
}

// One Stockham stage from src to dst (element (i, line c) layout above) on L
// lines of period M; Ns is the product of the radices done so far, tw[k] =
// exp(-2 pi i k / M).  Butterfly j of a line reads j + r M/R, multiplies by
// tw[r k M/(Ns R)] with k = j mod Ns, and writes (j - k) R + k + r Ns.  A
// thread takes one butterfly at a time.
// hin: the first stage of a transform whose input's upper half is zero (it
// reads only r < 8); hout: the last stage of one whose output's upper half
// is not wanted (it writes only the lower half).
template <bool INV>
__device__ __forceinline__ void stage16(const float2* src, float2* dst, int M, int L, int logL, int Ns,
                                        const float2* __restrict__ tw, bool hin, bool hout) {
  const int MR = M / 16, nb = L * MR, step = M / (Ns * 16);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j % Ns;
    float2 v[16];
    if (hin) {
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = src[swz(j + r * MR, c, L)];
      dft16_half_in<INV>(v);     // first stage: k = 0, no twiddles
      const int o = j << 4;
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) dst[swz(o + (k1 + 4 * k2) * Ns, c, L)] = v[4 * k1 + k2];
      continue;
    }
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = src[swz(j + r * MR, c, L)];
    if (k) {
#pragma unroll
      for (int r = 1; r < 16; ++r) {
        float2 w = __ldg(tw + r * k * step);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft16<INV>(v);
    const int o = (j - k) * 16 + k;
    if (hout) {
      // outputs o + q Ns with q = k1 + 4 k2 < 8 are the lower half
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 2; ++k2) dst[swz(o + (k1 + 4 * k2) * Ns, c, L)] = v[4 * k1 + k2];
    } else {
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) dst[swz(o + (k1 + 4 * k2) * Ns, c, L)] = v[4 * k1 + k2];
    }
  }
}

template <bool INV>
__device__ __forceinline__ void stage3(const float2* src, float2* dst, int M, int L, int logL, int Ns,
                                       const float2* __restrict__ tw) {
  const int MR = M / 3, nb = L * MR, step = M / (Ns * 3);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j % Ns;
    float2 v0 = src[swz(j, c, L)], v1 = src[swz(j + MR, c, L)], v2 = src[swz(j + 2 * MR, c, L)];
    float2 w1 = __ldg(tw + k * step), w2 = __ldg(tw + 2 * k * step);
    if (INV) {
      w1.y = -w1.y;
      w2.y = -w2.y;
    }
    v1 = cmul(v1, w1);
    v2 = cmul(v2, w2);
    dft3<INV>(v0, v1, v2);
    const int o = (j - k) * 3 + k;
    dst[swz(o, c, L)] = v0;
    dst[swz(o + Ns, c, L)] = v1;
    dst[swz(o + 2 * Ns, c, L)] = v2;
  }
}

template <bool INV>
__device__ __forceinline__ void stage4(const float2* src, float2* dst, int M, int L, int logL, int Ns,
                                       const float2* __restrict__ tw, bool hout) {
  const int MR = M / 4, nb = L * MR, step = M / (Ns * 4);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j % Ns;
    float2 v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) v[r] = src[swz(j + r * MR, c, L)];
#pragma unroll
    for (int r = 1; r < 4; ++r) {
      float2 w = __ldg(tw + r * k * step);
      if (INV) w.y = -w.y;
      v[r] = cmul(v[r], w);
    }
    dft4<INV>(v[0], v[1], v[2], v[3]);
    const int o = (j - k) * 4 + k;
    if (hout) {
      dst[swz(o, c, L)] = v[0];
      dst[swz(o + Ns, c, L)] = v[1];
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r) dst[swz(o + r * Ns, c, L)] = v[r];
    }
  }
}

template <bool INV>
__device__ __forceinline__ void stage2(const float2* src, float2* dst, int M, int L, int logL, int Ns,
                                       const float2* __restrict__ tw, bool hout) {
  const int MR = M / 2, nb = L * MR, step = M / (Ns * 2);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j % Ns;
    float2 w = __ldg(tw + k * step);
    if (INV) w.y = -w.y;
    const float2 a0 = src[swz(j, c, L)], a1 = cmul(src[swz(j + MR, c, L)], w);
    const int o = (j - k) * 2 + k;
    dst[swz(o, c, L)] = make_float2(a0.x + a1.x, a0.y + a1.y);
    if (!hout) dst[swz(o + Ns, c, L)] = make_float2(a0.x - a1.x, a0.y - a1.y);
  }
}

// factors of two of a period (compile time)
__host__ __device__ constexpr int twos_of(int m) { return (m & 1) ? 0 : 1 + twos_of(m >> 1); }

// FFT of the L lines of period M (2^a or 3 * 2^a, a >= 4) held in src,
// ping-ponging with dst; returns the buffer holding the result.  INV uses
// the conjugate twiddles (no 1/M scale).  Stages: radix 16, then radix 3 for
// a period with a factor 3, then radix 16 while four or more factors of two
// remain, then radix 4 and 2 (256 points take two stages, 384 four); every
// stage ends with one barrier.  The caller has synchronised after filling
// src.  MP > 0 (and LL >= 0) fix the period (and log2 L) at compile time:
// the stages unroll and the shared-memory addresses fold; otherwise they are
// read at run time.  half_in: the input's upper half is zero; half_out: only
// the output's lower half is wanted (the upper half of the result buffer is
// then left stale; a period of 48 ends on its radix-3 stage, which writes
// everything).
template <bool INV, int MP, int LL>
__device__ __forceinline__ float2* fft_block(float2* src, float2* dst, int M_rt, int logL_rt,
                                             const float2* __restrict__ tw, bool half_in, bool half_out) {
  const int M = MP > 0 ? MP : M_rt;
  const int logL = LL >= 0 ? LL : logL_rt, L = 1 << logL;
  const int a = MP > 0 ? twos_of(MP) : __ffs(M) - 1;
  const bool three = (M >> a) == 3;
  int twos = a - 4, Ns = 16;
  stage16<INV>(src, dst, M, L, logL, 1, tw, half_in, half_out && M == 16);
  __syncthreads();
  {
    float2* t = src;
    src = dst;
    dst = t;
  }
  if (three) {
    stage3<INV>(src, dst, M, L, logL, Ns, tw);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    Ns *= 3;
  }
#pragma unroll
  for (int st = 0; st < (MP > 0 ? (twos_of(MP > 0 ? MP : 1) - 4) / 4 : 2); ++st) {
    if (MP <= 0 && twos < 4) break;
    stage16<INV>(src, dst, M, L, logL, Ns, tw, false, half_out && twos == 4);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    Ns *= 16;
    twos -= 4;
  }
  if (twos >= 2) {
    stage4<INV>(src, dst, M, L, logL, Ns, tw, half_out && twos == 2);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    Ns *= 4;
    twos -= 2;
  }
  if (twos >= 1) {
    stage2<INV>(src, dst, M, L, logL, Ns, tw, half_out);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// ------------------------------------- period 256 with 16 lines per CTA --
// 256 = 16 x 16 and 16 lines x 16 butterflies = SPEC_THREADS: each thread
// takes butterfly j of line c in both stages (passes along y and x: c = t
// mod 16, j = t / 16; along z, where lines are contiguous: j = t mod 16,
// c = t / 16).  Stage 1 reads rows j + 16 r of the line (straight from
// global memory); stage 2 ends with rows j + 16 q, q = k1 + 4 k2, in
// v[4 k1 + k2] - the rows a first stage of butterfly j reads, so a transform
// that follows on the same line starts from registers, and the last stage
// stores to global memory: one shared-memory exchange and one barrier per
// transform.  Element (i, c) sits at 16 i + (c ^ (i mod 16)) when 16 lanes
// share j (the layout of the other periods) and at 16 i + (c ^ ((i ^ i / 16)
// mod 16)) when they share c: either way the stage-1 writes (rows 16 j + q)
// and stage-2 reads (rows j + 16 r) of 16 lanes fall in 16 different banks.
constexpr int R16_LINES = 16;
static_assert(R16_LINES * 16 == SPEC_THREADS, "one butterfly per thread and stage");
template <bool ZL>
__device__ __forceinline__ int swz16(int i, int c) {
  return i * 16 + (c ^ ((ZL ? i ^ (i >> 4) : i) & 15));
}

// stage 1 (no twiddles) of the rows in v (v[8..15] zero with hin), out to sm
template <bool INV, bool ZL>
__device__ __forceinline__ void r16_first(float2 (&v)[16], bool hin, float2* sm, int j, int c) {
  if (hin)
    dft16_half_in<INV>(v);
  else
    dft16<INV>(v);
  const int o = j << 4;
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) sm[swz16<ZL>(o + k1 + 4 * k2, c)] = v[4 * k1 + k2];
}

// stage 2 from sm: twiddles tw[r j] (conjugate for INV), then the DFT
template <bool INV, bool ZL>
__device__ __forceinline__ void r16_second(const float2* sm, float2 (&v)[16], int j, int c,
                                           const float2* __restrict__ tw) {
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = sm[swz16<ZL>(j + 16 * r, c)];
#pragma unroll
  for (int r = 1; r < 16; ++r) {
    float2 w = __ldg(tw + r * j);
    if (INV) w.y = -w.y;
    v[r] = cmul(v[r], w);
  }
  dft16<INV>(v);
}

// ------------------------------------------------- line block transfers --
// L lines of a pass along y or x: element (i, c) at base + i * stride + c
// (the lines are L consecutive kz).  Two adjacent lines move in one 16-byte
// access (stride, base and c are even); every load of a thread is issued
// before its shared-memory stores.  Rows i >= n are zero (the padding).
__device__ __forceinline__ void load_lines(const float2* __restrict__ base, size_t stride, int n, int M, int L,
                                           int logL, float2* sm) {
  if (L >= 2) {
    float4 v[SPEC_ELEMS / SPEC_THREADS / 2];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS / 2; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int c = (e & (L / 2 - 1)) * 2, i = e >> (logL - 1);
      v[q] = i < n ? __ldg(reinterpret_cast<const float4*>(base + (size_t)i * stride + c))
                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS / 2; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int c = (e & (L / 2 - 1)) * 2, i = e >> (logL - 1);
      if (i < M) {
        sm[swz(i, c, L)] = make_float2(v[q].x, v[q].y);
        sm[swz(i, c + 1, L)] = make_float2(v[q].z, v[q].w);
      }
    }
  } else {
    for (int i = threadIdx.x; i < M; i += SPEC_THREADS)
      sm[swz(i, 0, L)] = i < n ? base[(size_t)i * stride] : make_float2(0.0f, 0.0f);
  }
}

__device__ __forceinline__ void store_lines(const float2* res, float2* __restrict__ base, size_t stride, int n,
                                            int L, int logL) {
  if (L >= 2) {
    for (int e = threadIdx.x; e < n * L / 2; e += SPEC_THREADS) {
      const int c = (e & (L / 2 - 1)) * 2, i = e >> (logL - 1);
      const float2 a = res[swz(i, c, L)], b = res[swz(i, c + 1, L)];
      *reinterpret_cast<float4*>(base + (size_t)i * stride + c) = make_float4(a.x, a.y, b.x, b.y);
    }
  } else {
    for (int i = threadIdx.x; i < n; i += SPEC_THREADS) base[(size_t)i * stride] = res[swz(i, 0, L)];
  }
}

// ---------------------------------------------------------------- passes --
// Every pass is a template on MP, its period, and LL, log2 of its lines per
// CTA: MP > 0 fixes both at compile time, MP = -1 reads them from the launch
// (P.g.M and P.g.logL).  Lines per CTA: the largest power of two L with
// L M <= 4096 for lines along z; lines along y and x are taken in blocks of L
// consecutive kz, so L also divides Mz.
// z forward: lines (x, y), TERMA pair in, A out.  One CTA per L lines and pair.
// Shared memory of a five-pass kernel: two buffers of its CTA's lines.  A
// compile-time period and line count take only what they use, so period 96
// (3072 values per CTA, 48 KB) runs four CTAs per SM, the others (4096
// values, 64 KB) three.
template <int MP, int LL>
constexpr int spec_elems() {
  static_assert(MP <= 0 || (MP << (LL > 0 ? LL : 0)) <= SPEC_ELEMS, "lines of a CTA");
  return MP > 0 ? (MP << (LL > 0 ? LL : 0)) : SPEC_ELEMS;
}
template <int MP, int LL>
constexpr int spec_smem() { return 2 * spec_elems<MP, LL>() * 8; }
template <int MP, int LL>
constexpr int spec_ctas() { return spec_smem<MP, LL>() <= 48 * 1024 ? 4 : SPEC_CTAS_PER_SM; }

template <int MP, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, spec_ctas<MP, LL>()) spec_z_forward_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + spec_elems<MP, LL>();
  const SpecPair& pr = P.p[blockIdx.y];
  const int Mz = MP > 0 ? MP : P.g.M[2];
  const int logL = MP > 0 ? LL : P.g.logL[2], L = 1 << logL;
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * L;
  // lines of each beam that may hold TERMA (the others are zero and are not
  // read); a block without any transforms to zero
  // (both flags fetched together; one barrier publishes them and tells
  // whether the block holds any)
  __shared__ unsigned char zf[2][SPEC_ELEMS / SPEC_MIN_PERIOD];
  bool mine = false;
  for (int c = threadIdx.x; c < L; c += SPEC_THREADS) {
    const int l = l0 + c, lc = l < nl ? l : nl - 1;
    const unsigned a1 = pr.l1 ? (unsigned)__ldg(pr.l1 + lc) : 1u;
    const unsigned a2 = (pr.t2 && pr.l2) ? (unsigned)__ldg(pr.l2 + lc) : 1u;
    const bool f1 = l < nl && a1 != 0u;
    const bool f2 = l < nl && pr.t2 && a2 != 0u;
    zf[0][c] = f1;
    zf[1][c] = f2;
    mine = mine || f1 || f2;
  }
  if (!__syncthreads_or(mine)) {
    // L Mz float2 of consecutive lines, 16 bytes per store (Mz is even)
    float4* a4 = reinterpret_cast<float4*>(pr.a + (size_t)l0 * Mz);
    const int lines = min(L, nl - l0);
    for (int e = threadIdx.x; e < lines * Mz / 2; e += SPEC_THREADS) a4[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  if constexpr (MP == 256 && LL == 4) {
    // TERMA rows z < nz <= 128 (the upper half is zero) straight from global
    // memory; A written from the last stage
    const int j = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
    const bool ok = l < nl, f1 = zf[0][c], f2 = zf[1][c];
    const size_t o = (size_t)(ok ? l : 0) * P.g.zp;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int i = j + 16 * r;
      v[r] = make_float2(0.0f, 0.0f);
      if (r < 8 && i < nz) {
        if (f1) v[r].x = __ldg(pr.t1 + o + i);
        if (f2) v[r].y = __ldg(pr.t2 + o + i);
      }
    }
    r16_first<false, true>(v, true, sm, j, c);
    __syncthreads();
    r16_second<false, true>(sm, v, j, c, P.g.tw[2]);
    if (ok) {
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) pr.a[(size_t)l * Mz + j + 16 * (k1 + 4 * k2)] = v[4 * k1 + k2];
    }
  } else {
    {
      // every load of the thread first, then the shared-memory stores
      float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
      for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
        const int e = threadIdx.x + q * SPEC_THREADS;
        const int c = e / Mz, i = e - c * Mz, l = l0 + c;
        v[q] = make_float2(0.0f, 0.0f);
        if (c < L && l < nl && i < nz) {
          const size_t o = (size_t)l * P.g.zp + i;
          if (zf[0][c]) v[q].x = __ldg(pr.t1 + o);
          if (zf[1][c]) v[q].y = __ldg(pr.t2 + o);
        }
      }
#pragma unroll
      for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
        const int e = threadIdx.x + q * SPEC_THREADS;
        const int c = e / Mz, i = e - c * Mz;
        if (c < L) sm[swz(i, c, L)] = v[q];
      }
    }
    __syncthreads();
    const float2* res = fft_block<false, MP, LL>(sm, sm2, Mz, logL, P.g.tw[2], 2 * nz <= Mz, false);
    for (int e = threadIdx.x; e < L * Mz; e += SPEC_THREADS) {
      const int c = e / Mz, i = e - c * Mz, l = l0 + c;
      if (l < nl) pr.a[(size_t)l * Mz + i] = res[swz(i, c, L)];
    }
  }
}

// y forward (A -> B) or inverse (B -> A): lines (x, kz) in blocks of L kz.
template <bool INV, int MP, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, spec_ctas<MP, LL>()) spec_y_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + spec_elems<MP, LL>();
  const SpecPair& pr = P.p[blockIdx.y];
  const int My = MP > 0 ? MP : P.g.M[1], Mz = P.g.M[2];
  const int logL = MP > 0 ? LL : P.g.logL[1], L = 1 << logL;
  const int nkb = Mz >> logL;
  const int x = blockIdx.x / nkb, kz0 = (blockIdx.x - x * nkb) << logL;
  const int ny = P.g.n[1];
  const int n_in = INV ? My : ny, n_out = INV ? ny : My;
  const float2* src = INV ? pr.b + (size_t)x * My * Mz : pr.a + (size_t)x * ny * Mz;
  float2* dst = INV ? pr.a + (size_t)x * ny * Mz : pr.b + (size_t)x * My * Mz;
  src += kz0;
  dst += kz0;
  if constexpr (MP == 256 && LL == 4) {
    // rows of the forward input y < ny <= 128: the upper half is zero
    const int c = threadIdx.x & (R16_LINES - 1), j = threadIdx.x >> 4;
    const float2* sl = src + c;
    float2* dl = dst + c;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int i = j + 16 * r;
      if (INV)
        v[r] = __ldg(sl + (size_t)i * Mz);
      else
        v[r] = (r < 8 && i < ny) ? __ldg(sl + (size_t)i * Mz) : make_float2(0.0f, 0.0f);
    }
    r16_first<INV, false>(v, !INV, sm, j, c);
    __syncthreads();
    r16_second<INV, false>(sm, v, j, c, P.g.tw[1]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < (INV ? 2 : 4); ++k2) {
        const int i = j + 16 * (k1 + 4 * k2);
        if (!INV || i < ny) dl[(size_t)i * Mz] = v[4 * k1 + k2];
      }
    return;
  }
  load_lines(src, Mz, n_in, My, L, logL, sm);
  __syncthreads();
  const float2* res = fft_block<INV, MP, LL>(sm, sm2, My, logL, P.g.tw[1], !INV && 2 * ny <= My,
                                             INV && 2 * ny <= My);
  store_lines(res, dst, Mz, n_out, L, logL);
}

// x pass on B, lines (ky, kz) in blocks of L kz; consecutive CTAs take the
// same lines of consecutive pairs, so each block of S^ is read from L2.
// CONV: forward, times S^ (or its conjugate), inverse, x < nx kept;
// otherwise forward only over the full period (building S^).
template <bool CONV, int MP, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, spec_ctas<MP, LL>()) spec_x_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + spec_elems<MP, LL>();
  const int pair = blockIdx.x % P.n_pairs, blk = blockIdx.x / P.n_pairs;
  const SpecPair& pr = P.p[pair];
  const int Mx = MP > 0 ? MP : P.g.M[0], My = P.g.M[1], Mz = P.g.M[2];
  const int logL = MP > 0 ? LL : P.g.logL[0], L = 1 << logL;
  const int nkb = Mz >> logL;
  const int ky = blk / nkb, kz0 = (blk - ky * nkb) << logL;
  const size_t xs = (size_t)My * Mz, off = (size_t)ky * Mz + kz0;
  float2* b = pr.b + off;
  const int nx = CONV ? P.g.n[0] : Mx;
  if constexpr (CONV && MP == 256 && LL == 4) {
    // forward (input rows x < nx <= 128), times S^, inverse (rows x < nx
    // kept); forward stage 2, the product and inverse stage 1 in registers
    const int c = threadIdx.x & (R16_LINES - 1), j = threadIdx.x >> 4;
    float2* bl = b + c;
    {
      // S^ of the CTA's lines, copied to sm2 while the forward transform
      // runs: two adjacent lines per 16-byte copy, element (i, c) at
      // 16 i + (c ^ (i & 14)) (pairs stay adjacent; the reads below of 16
      // lines at one row fall in 16 banks)
      const float2* sh = P.g.shat + off;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = threadIdx.x + q * SPEC_THREADS, i = e >> 3, cp = (e & 7) * 2;
        const unsigned d = (unsigned)__cvta_generic_to_shared(sm2 + i * 16 + (cp ^ (i & 14)));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(sh + (size_t)i * xs + cp));
      }
      asm volatile("cp.async.commit_group;\n" ::);
    }
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int i = j + 16 * r;
      v[r] = (r < 8 && i < nx) ? __ldg(bl + (size_t)i * xs) : make_float2(0.0f, 0.0f);
    }
    r16_first<false, false>(v, true, sm, j, c);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();   // stage 1 and every thread's S^ copies are in shared memory
    r16_second<false, false>(sm, v, j, c, P.g.tw[0]);

    const float cs = P.g.conj ? -1.0f : 1.0f;
    float2 u[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) {
        const int q = k1 + 4 * k2;
        const int i = j + 16 * q;
        const float2 s = sm2[i * 16 + (c ^ (i & 14))];
        u[q] = cmul(v[4 * k1 + k2], make_float2(s.x, cs * s.y));
      }
    __syncthreads();   // every read of sm (stage 2) and sm2 (S^) done
    r16_first<true, false>(u, false, sm, j, c);
    __syncthreads();
    r16_second<true, false>(sm, u, j, c, P.g.tw[0]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 2; ++k2) {
        const int i = j + 16 * (k1 + 4 * k2);
        if (i < nx) bl[(size_t)i * xs] = u[4 * k1 + k2];
      }
    return;
  }
  load_lines(b, xs, nx, Mx, L, logL, sm);
  __syncthreads();
  float2* res = fft_block<false, MP, LL>(sm, sm2, Mx, logL, P.g.tw[0], 2 * nx <= Mx, false);
  if (CONV) {
    const float2* sh = P.g.shat + off;
    float2 sv[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      sv[q] = (e >> logL) < Mx ? __ldg(sh + (size_t)(e >> logL) * xs + (e & (L - 1))) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      if ((e >> logL) < Mx) {
        float2 s = sv[q];
        if (P.g.conj) s.y = -s.y;
        const int k = swz(e >> logL, e & (L - 1), L);
        res[k] = cmul(res[k], s);
      }
    }
    __syncthreads();
    res = fft_block<true, MP, LL>(res, res == sm ? sm2 : sm, Mx, logL, P.g.tw[0], false, 2 * nx <= Mx);
  }
  store_lines(res, b, xs, nx, L, logL);
}

// ----------------------------------------------- period 384 along x --
// 8-point DFT in place, natural order in and out (radix 2 over two DFT4s).
template <bool INV>
__device__ __forceinline__ void dft8(float2 (&a)[8]) {
  constexpr float R2 = 0.70710678118654752f;
  float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6], o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  o1 = rot<INV>(o1, R2, R2);
  o2 = INV ? make_float2(-o2.y, o2.x) : make_float2(o2.y, -o2.x);   // times -+i
  o3 = rot<INV>(o3, -R2, R2);
  a[0] = make_float2(e0.x + o0.x, e0.y + o0.y);
  a[4] = make_float2(e0.x - o0.x, e0.y - o0.y);
  a[1] = make_float2(e1.x + o1.x, e1.y + o1.y);
  a[5] = make_float2(e1.x - o1.x, e1.y - o1.y);
  a[2] = make_float2(e2.x + o2.x, e2.y + o2.y);
  a[6] = make_float2(e2.x - o2.x, e2.y - o2.y);
  a[3] = make_float2(e3.x + o3.x, e3.y + o3.y);
  a[7] = make_float2(e3.x - o3.x, e3.y - o3.y);
}

// 24-point DFT, natural order in (a) and out (x): n = 3 n8 + n3, three DFT8s
// over n8, twiddles exp(-+2 pi i n3 k8 / 24), eight DFT3s over n3, output
// k8 + 8 k3.
template <bool INV>
__device__ __forceinline__ void dft24(const float2 (&a)[24], float2 (&x)[24]) {
  // cos and sin of 15 m degrees, m = 0..14
  constexpr float C[15] = {1.0f,  0.96592582628906829f,  0.86602540378443865f,  0.70710678118654752f,
                           0.5f,  0.25881904510252076f,  0.0f,                 -0.25881904510252076f,
                           -0.5f, -0.70710678118654752f, -0.86602540378443865f, -0.96592582628906829f,
                           -1.0f, -0.96592582628906829f, -0.86602540378443865f};
  constexpr float S[15] = {0.0f, 0.25881904510252076f, 0.5f, 0.70710678118654752f, 0.86602540378443865f,
                           0.96592582628906829f, 1.0f, 0.96592582628906829f, 0.86602540378443865f,
                           0.70710678118654752f, 0.5f, 0.25881904510252076f, 0.0f,
                           -0.25881904510252076f, -0.5f};
  float2 b[3][8];
#pragma unroll
  for (int n3 = 0; n3 < 3; ++n3) {
#pragma unroll
    for (int n8 = 0; n8 < 8; ++n8) b[n3][n8] = a[3 * n8 + n3];
    dft8<INV>(b[n3]);
  }
#pragma unroll
  for (int k8 = 0; k8 < 8; ++k8) {
    float2 t0 = b[0][k8], t1 = b[1][k8], t2 = b[2][k8];
    if (k8 > 0) {
      t1 = rot<INV>(t1, C[k8], S[k8]);
      t2 = rot<INV>(t2, C[2 * k8], S[2 * k8]);
    }
    dft3<INV>(t0, t1, t2);
    x[k8] = t0;
    x[k8 + 8] = t1;
    x[k8 + 16] = t2;
  }
}

// 12-point DFT, natural order in (a) and out (x): n = 3 n4 + n3, three DFT4s
// over n4, twiddles exp(-+2 pi i n3 k4 / 12), four DFT3s over n3, output
// k4 + 4 k3.
template <bool INV>
__device__ __forceinline__ void dft12(const float2 (&a)[12], float2 (&x)[12]) {
  constexpr float C[7] = {1.0f, 0.86602540378443865f, 0.5f, 0.0f, -0.5f, -0.86602540378443865f, -1.0f};
  constexpr float S[7] = {0.0f, 0.5f, 0.86602540378443865f, 1.0f, 0.86602540378443865f, 0.5f, 0.0f};
  float2 b[3][4];
#pragma unroll
  for (int n3 = 0; n3 < 3; ++n3) {
#pragma unroll
    for (int n4 = 0; n4 < 4; ++n4) b[n3][n4] = a[3 * n4 + n3];
    dft4<INV>(b[n3][0], b[n3][1], b[n3][2], b[n3][3]);
  }
#pragma unroll
  for (int k4 = 0; k4 < 4; ++k4) {
    float2 t0 = b[0][k4], t1 = b[1][k4], t2 = b[2][k4];
    if (k4 > 0) {
      t1 = rot<INV>(t1, C[k4], S[k4]);
      t2 = rot<INV>(t2, C[2 * k4], S[2 * k4]);
    }
    dft3<INV>(t0, t1, t2);
    x[k4] = t0;
    x[k4 + 4] = t1;
    x[k4 + 8] = t2;
  }
}

template <bool INV, int N2>
__device__ __forceinline__ void dft_n2(const float2 (&a)[N2], float2 (&x)[N2]) {
  if constexpr (N2 == 24) {
    dft24<INV>(a, x);
  } else if constexpr (N2 == 12) {
    dft12<INV>(a, x);
  } else {
    static_assert(N2 == 8, "16 x N2 periods: 128, 192, 384");
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = a[i];
    dft8<INV>(x);
  }
}

// The x and y passes at periods 16 N2 = 384 (N2 = 24, grids of 129-192
// voxels along the axis), 192 (N2 = 12, 65-96 voxels) and 128 (N2 = 8,
// 49-64 voxels), 16 lines
// (consecutive kz, 128-byte rows) per CTA:
//   forward, n = N2 n1 + n2, k = k1 + 16 k2:
//     stage 1, thread (c, n2): 16-point DFT over n1 (n1 < 8 nonzero: the
//       upper half of the padded input) of row N2 n1 + n2, times
//       exp(-2 pi i n2 k1 / (16 N2)), out to shared memory row N2 k1 + n2;
//     stage 2, thread (c, k1): N2-point DFT over n2 -> X[k1 + 16 k2] in
//       registers;
//   inverse, k = k1 + 16 k2, n = n2 + N2 n1:
//     stage A, thread (c, k1): N2-point DFT over k2 -> n2, times
//       exp(+2 pi i n2 k1 / (16 N2)), out to shared memory row 16 n2 + k1;
//     stage B, thread (c, n2): 16-point DFT over k1 -> rows n2 + N2 n1,
//       n1 < 8, written where < n.
// The x pass chains forward, the product with S^ (the CTA's 16 N2 x 16
// block staged in shared memory by cp.async during stage 1) and inverse:
// stage 2, the product and stage A in the same thread's registers, two
// exchanges for the transform pair instead of the generic kernel's six to
// eight stages.  The forward y pass writes all 16 N2 rows of B from stage 2;
// the inverse starts with stage A on rows k1 + 16 k2 of B.  A row of 16
// lines is 128 bytes, one half-warp access: no swizzle is needed.  Stages
// 1 and B use 16 N2 threads, stages 2 and A 256.
template <int N2>
constexpr int r16n_threads() { return 16 * N2 > 256 ? 16 * N2 : 256; }
template <int N2>
constexpr int r16n_ctas() { return N2 == 24 ? 2 : 4; }
template <int N2>
constexpr int r16n_smem(bool conv) { return ((conv ? 2 : 1) * 16 * N2 * 16 + 16 * N2) * 8; }

template <int N2>
__global__ void __launch_bounds__(r16n_threads<N2>(), r16n_ctas<N2>()) spec_x16n_kernel(SpecLaunch P) {
  constexpr int M = 16 * N2, T = r16n_threads<N2>();
  extern __shared__ float2 spec_sm[];
  float2* const xb = spec_sm;                 // exchange, row r at 16 r
  float2* const sb = spec_sm + M * 16;        // S^ block, row kx at 16 kx
  float2* const twb = spec_sm + 2 * M * 16;   // exp(-2 pi i k / M)
  const int pair = blockIdx.x % P.n_pairs, blk = blockIdx.x / P.n_pairs;
  const SpecPair& pr = P.p[pair];
  const int My = P.g.M[1], Mz = P.g.M[2];
  const int nkb = Mz >> 4;
  const int ky = blk / nkb, kz0 = (blk - ky * nkb) << 4;
  const size_t xs = (size_t)My * Mz, off = (size_t)ky * Mz + kz0;
  float2* const b = pr.b + off;
  const int nx = P.g.n[0];
  const int c = threadIdx.x & 15, h = threadIdx.x >> 4;   // h: n2 (stages 1, B) or k1 (stages 2, A)
  {
    // S^ rows of the CTA's 16 lines: M x 128 bytes, 16 bytes per copy
    const float2* sh = P.g.shat + off;
#pragma unroll
    for (int q = 0; q < 8 * M / T; ++q) {
      const int e = threadIdx.x + q * T, i = e >> 3, cp = (e & 7) * 2;
      const unsigned d = (unsigned)__cvta_generic_to_shared(sb + i * 16 + cp);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(sh + (size_t)i * xs + cp));
    }
    asm volatile("cp.async.commit_group;\n" ::);
    if (threadIdx.x < M) twb[threadIdx.x] = __ldg(P.g.tw[0] + threadIdx.x);
  }
  __syncthreads();   // twiddle table
  if (threadIdx.x < 16 * N2) {
    // forward stage 1, thread (c, n2 = h): rows N2 n1 + n2, n1 < 8
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int x = N2 * n1 + h;
      v[n1] = (n1 < 8 && x < nx) ? __ldg(b + (size_t)x * xs + c) : make_float2(0.0f, 0.0f);
    }
    dft16_half_in<false>(v);
    // X[m] of the DFT16 sits in v[4 (m mod 4) + m / 4]
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      float2 y = v[4 * (m & 3) + (m >> 2)];
      if (m > 0) y = cmul(y, twb[h * m]);
      xb[(m * N2 + h) * 16 + c] = y;
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();   // exchange written, S^ landed
  float2 z[N2];
  if (threadIdx.x < 256) {
    // forward stage 2, thread (c, k1 = h); the product; inverse stage A
    float2 a[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) a[n2] = xb[(h * N2 + n2) * 16 + c];
    dft_n2<false, N2>(a, z);
    const float cs = P.g.conj ? -1.0f : 1.0f;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const float2 sv = sb[(h + 16 * k2) * 16 + c];
      a[k2] = cmul(z[k2], make_float2(sv.x, cs * sv.y));
    }
    dft_n2<true, N2>(a, z);
  }
  __syncthreads();   // every read of the exchange done
  if (threadIdx.x < 256) {
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) {
      float2 y = z[n2];
      if (n2 > 0) {
        float2 w = twb[n2 * h];
        w.y = -w.y;
        y = cmul(y, w);
      }
      xb[(n2 * 16 + h) * 16 + c] = y;
    }
  }
  __syncthreads();
  if (threadIdx.x < 16 * N2) {
    // inverse stage B, thread (c, n2 = h): rows n2 + N2 n1
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = xb[(h * 16 + q) * 16 + c];
    dft16<true>(v);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int x = h + N2 * m;
      if (x < nx) b[(size_t)x * xs + c] = v[4 * (m & 3) + (m >> 2)];
    }
  }
}

template <bool INV, int N2>
__global__ void __launch_bounds__(r16n_threads<N2>(), r16n_ctas<N2>()) spec_y16n_kernel(SpecLaunch P) {
  constexpr int M = 16 * N2;
  extern __shared__ float2 spec_sm[];
  float2* const xb = spec_sm;                 // exchange, row r at 16 r
  float2* const twb = spec_sm + M * 16;       // exp(-2 pi i k / M)
  const SpecPair& pr = P.p[blockIdx.y];
  const int Mz = P.g.M[2], ny = P.g.n[1];
  const int nkb = Mz >> 4;
  const int x = blockIdx.x / nkb, kz0 = (blockIdx.x - x * nkb) << 4;
  const float2* const src = (INV ? pr.b + (size_t)x * M * Mz : pr.a + (size_t)x * ny * Mz) + kz0;
  float2* const dst = (INV ? pr.a + (size_t)x * ny * Mz : pr.b + (size_t)x * M * Mz) + kz0;
  const int c = threadIdx.x & 15, h = threadIdx.x >> 4;   // h: n2 (stages 1, B) or k1 (stages 2, A)
  if (threadIdx.x < M) twb[threadIdx.x] = __ldg(P.g.tw[1] + threadIdx.x);
  __syncthreads();   // twiddle table
  if (!INV) {
    if (threadIdx.x < 16 * N2) {
      // stage 1, thread (c, n2 = h)
      float2 v[16];
#pragma unroll
      for (int n1 = 0; n1 < 16; ++n1) {
        const int y = N2 * n1 + h;
        v[n1] = (n1 < 8 && y < ny) ? __ldg(src + (size_t)y * Mz + c) : make_float2(0.0f, 0.0f);
      }
      dft16_half_in<false>(v);
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        float2 t = v[4 * (m & 3) + (m >> 2)];
        if (m > 0) t = cmul(t, twb[h * m]);
        xb[(m * N2 + h) * 16 + c] = t;
      }
    }
    __syncthreads();
    if (threadIdx.x < 256) {
      // stage 2, thread (c, k1 = h)
      float2 a[N2], z[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) a[n2] = xb[(h * N2 + n2) * 16 + c];
      dft_n2<false, N2>(a, z);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) dst[(size_t)(h + 16 * k2) * Mz + c] = z[k2];
    }
  } else {
    if (threadIdx.x < 256) {
      // stage A, thread (c, k1 = h)
      float2 a[N2], z[N2];
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) a[k2] = __ldg(src + (size_t)(h + 16 * k2) * Mz + c);
      dft_n2<true, N2>(a, z);
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) {
        float2 t = z[n2];
        if (n2 > 0) {
          float2 w = twb[n2 * h];
          w.y = -w.y;
          t = cmul(t, w);
        }
        xb[(n2 * 16 + h) * 16 + c] = t;
      }
    }
    __syncthreads();
    if (threadIdx.x < 16 * N2) {
      // stage B, thread (c, n2 = h)
      float2 v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = xb[(h * 16 + q) * 16 + c];
      dft16<true>(v);
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int y = h + N2 * m;
        if (y < ny) dst[(size_t)y * Mz + c] = v[4 * (m & 3) + (m >> 2)];
      }
    }
  }
}

// The z passes at periods 16 N2 = 384, 192 and 128, 16 lines (x, y) per CTA.
// Lines along z are contiguous, so lanes run along z: thread (n2, line)
// with n2 fastest in the 16-point stages (consecutive z: the TERMA reads and
// dose writes are coalesced), thread (k1, line) with k1 fastest in the
// N2-point stages (consecutive k: 128-byte runs of A).  The exchange holds
// each line's M rows with one slot of padding after every 16 (line c, row r
// at c (M + M/16) + r + r/16), and both transforms use rows 16 n2 + k1, so
// that 16 lanes at consecutive k1 (one row step) and at consecutive n2 (17
// slots apart) fall in 16 different banks.
//   forward: stage 1, thread (n2, c): 16-point DFT over n1 of z = N2 n1 + n2
//     (n1 < 8), twiddled by exp(-2 pi i n2 k1 / M), into rows 16 n2 + k1;
//     stage 2, thread (k1, c): N2-point DFT over n2 -> A[k1 + 16 k2];
//   inverse: stage A, thread (k1, c): N2-point DFT over k2 of A[k1 + 16 k2],
//     twiddled by exp(+2 pi i n2 k1 / M), into rows 16 n2 + k1; stage B,
//     thread (n2, c): 16-point DFT over k1 -> z = n2 + N2 n1 < nz.
template <int N2>
constexpr int r16n_zsmem() { return (16 * (16 * N2 + N2) + 16 * N2) * 8; }
template <int N2>
__device__ __forceinline__ int zslot(int r, int c) { return c * (17 * N2) + r + (r >> 4); }

template <int N2>
__global__ void __launch_bounds__(r16n_threads<N2>(), r16n_ctas<N2>()) spec_z16n_forward_kernel(SpecLaunch P) {
  constexpr int M = 16 * N2, T = r16n_threads<N2>();
  extern __shared__ float2 spec_sm[];
  float2* const xb = spec_sm;
  float2* const twb = spec_sm + 16 * 17 * N2;
  const SpecPair& pr = P.p[blockIdx.y];
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * 16;
  __shared__ unsigned char zf[2][16];
  bool mine = false;
  if (threadIdx.x < 16) {
    const int c = threadIdx.x, l = l0 + c, lc = l < nl ? l : nl - 1;
    const unsigned a1 = pr.l1 ? (unsigned)__ldg(pr.l1 + lc) : 1u;
    const unsigned a2 = (pr.t2 && pr.l2) ? (unsigned)__ldg(pr.l2 + lc) : 1u;
    zf[0][c] = l < nl && a1 != 0u;
    zf[1][c] = l < nl && pr.t2 && a2 != 0u;
    mine = zf[0][c] || zf[1][c];
  }
  // stage-1 twiddles exp(-2 pi i n2 m / M) at m N2 + n2: lanes at consecutive
  // n2 read consecutive slots
  for (int i = threadIdx.x; i < M; i += T) twb[i] = __ldg(P.g.tw[2] + (i % N2) * (i / N2));
  if (!__syncthreads_or(mine)) {
    // no TERMA on these lines: zeros, two values per 16-byte store
    const int lines = min(16, nl - l0);
    float4* a4 = reinterpret_cast<float4*>(pr.a + (size_t)l0 * M);
    for (int e = threadIdx.x; e < lines * M / 2; e += T) a4[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  if (threadIdx.x < 16 * N2) {
    const int n2 = threadIdx.x % N2, c = threadIdx.x / N2, l = l0 + c;
    const bool f1 = zf[0][c], f2 = zf[1][c];
    const size_t o = (size_t)(l < nl ? l : 0) * P.g.zp;
    float2 v[16];
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const int z = N2 * n1 + n2;
      v[n1] = make_float2(0.0f, 0.0f);
      if (n1 < 8 && z < nz) {
        if (f1) v[n1].x = __ldg(pr.t1 + o + z);
        if (f2) v[n1].y = __ldg(pr.t2 + o + z);
      }
    }
    dft16_half_in<false>(v);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      float2 y = v[4 * (m & 3) + (m >> 2)];
      if (m > 0) y = cmul(y, twb[m * N2 + n2]);
      xb[zslot<N2>(16 * n2 + m, c)] = y;
    }
  }
  __syncthreads();
  if (threadIdx.x < 256) {
    const int k1 = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
    float2 a[N2], z[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) a[n2] = xb[zslot<N2>(16 * n2 + k1, c)];
    dft_n2<false, N2>(a, z);
    if (l < nl) {
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) pr.a[(size_t)l * M + k1 + 16 * k2] = z[k2];
    }
  }
}

template <int N2>
__global__ void __launch_bounds__(r16n_threads<N2>(), r16n_ctas<N2>()) spec_z16n_inverse_kernel(SpecLaunch P) {
  constexpr int M = 16 * N2;
  extern __shared__ float2 spec_sm[];
  float2* const xb = spec_sm;
  float2* const twb = spec_sm + 16 * 17 * N2;
  const SpecPair& pr = P.p[blockIdx.y];
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * 16;
  // stage-A twiddles exp(-2 pi i n2 k1 / M) at 16 n2 + k1: lanes at
  // consecutive k1 read consecutive slots
  for (int i = threadIdx.x; i < M; i += r16n_threads<N2>()) twb[i] = __ldg(P.g.tw[2] + (i >> 4) * (i & 15));
  __syncthreads();   // twiddle table
  if (threadIdx.x < 256) {
    const int k1 = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
    const float2* al = pr.a + (size_t)(l < nl ? l : 0) * M;
    float2 a[N2], z[N2];
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) a[k2] = l < nl ? __ldg(al + k1 + 16 * k2) : make_float2(0.0f, 0.0f);
    dft_n2<true, N2>(a, z);
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) {
      float2 y = z[n2];
      if (n2 > 0) {
        float2 w = twb[16 * n2 + k1];
        w.y = -w.y;
        y = cmul(y, w);
      }
      xb[zslot<N2>(16 * n2 + k1, c)] = y;
    }
  }
  __syncthreads();
  if (threadIdx.x < 16 * N2) {
    const int n2 = threadIdx.x % N2, c = threadIdx.x / N2, l = l0 + c;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = xb[zslot<N2>(16 * n2 + q, c)];
    dft16<true>(v);
    if (l < nl) {
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int z = n2 + N2 * m;
        if (z < nz) {
          const float2 d = v[4 * (m & 3) + (m >> 2)];
          pr.d1[(size_t)l * nz + z] = d.x;
          if (pr.d2) pr.d2[(size_t)l * nz + z] = d.y;
        }
      }
    }
  }
}

// z inverse: lines (x, y), A in, dose pair out (real part, imaginary part).
template <int MP, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, spec_ctas<MP, LL>()) spec_z_inverse_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + spec_elems<MP, LL>();
  const SpecPair& pr = P.p[blockIdx.y];
  const int Mz = MP > 0 ? MP : P.g.M[2];
  const int logL = MP > 0 ? LL : P.g.logL[2], L = 1 << logL;
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * L;
  if constexpr (MP == 256 && LL == 4) {
    // all of A's line in; rows z < nz <= 128 of the result out
    const int j = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
    const bool ok = l < nl;
    const float2* al = pr.a + (size_t)(ok ? l : 0) * Mz;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = ok ? __ldg(al + j + 16 * r) : make_float2(0.0f, 0.0f);
    r16_first<true, true>(v, false, sm, j, c);
    __syncthreads();
    r16_second<true, true>(sm, v, j, c, P.g.tw[2]);
    if (ok) {
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 2; ++k2) {
          const int i = j + 16 * (k1 + 4 * k2);
          if (i < nz) {
            pr.d1[(size_t)l * nz + i] = v[4 * k1 + k2].x;
            if (pr.d2) pr.d2[(size_t)l * nz + i] = v[4 * k1 + k2].y;
          }
        }
    }
  } else {
    {
      float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
      for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
        const int e = threadIdx.x + q * SPEC_THREADS;
        const int c = e / Mz, i = e - c * Mz, l = l0 + c;
        v[q] = (c < L && l < nl) ? pr.a[(size_t)l * Mz + i] : make_float2(0.0f, 0.0f);
      }
#pragma unroll
      for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
        const int e = threadIdx.x + q * SPEC_THREADS;
        const int c = e / Mz, i = e - c * Mz;
        if (c < L) sm[swz(i, c, L)] = v[q];
      }
    }
    __syncthreads();
    const float2* res = fft_block<true, MP, LL>(sm, sm2, Mz, logL, P.g.tw[2], false, 2 * nz <= Mz);
    for (int e = threadIdx.x; e < L * Mz; e += SPEC_THREADS) {
      const int c = e / Mz, i = e - c * Mz, l = l0 + c;
      if (l < nl && i < nz) {
        const float2 v = res[swz(i, c, L)];
        pr.d1[(size_t)l * nz + i] = v.x;
        if (pr.d2) pr.d2[(size_t)l * nz + i] = v.y;
      }
    }
  }
}

// ------------------------------------------------------------ plane path --
// The z passes of the plane path use one exchange buffer (16 lines of 256)
// and run more CTAs per SM than the five-pass kernels: more loads and
// stores in flight in passes that stream A (measured per 16 pairs at 128^3:
// z forward 137 / 117 / 104 / 102 us at 3 / 4 / 5 / 6 CTAs per SM, z
// inverse 155 / 149 / 153 / 187 us).
constexpr int SPEC_ZFWD_CTAS_PER_SM = 5;
constexpr int SPEC_ZINV_CTAS_PER_SM = 4;
constexpr int SPEC_ZPLANE_SMEM = R16_LINES * 256 * 8;
// Periods of 256 on all three axes.  The y and x transforms of one kz plane
// (with the S^ product and both inverses) run in one kernel on the plane's
// spectrum held on chip, so the intermediate B [nx][My][Mz] of the five-pass
// path never reaches memory; A is laid out plane-major, A[kz][l] with
// l = x ny + y and plane pitch lp, so a plane is one contiguous block.
//
// z forward into plane-major A: stage 1 with lanes along z (the TERMA rows
// are read coalesced), stage 2 with lanes across the CTA's 16 lines (one kz
// of 16 consecutive lines is one 128-byte store).  Both stages address the
// exchange buffer with the z layout swz16<true>; either lane mapping reads
// or writes 16 distinct banks per half warp there.
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_ZFWD_CTAS_PER_SM) spec_z_forward_plane_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  const SpecPair& pr = P.p[blockIdx.y];
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2], lp = P.g.lp;
  const int l0 = blockIdx.x * R16_LINES;
  __shared__ unsigned char zf[2][R16_LINES];
  bool mine = false;
  if (threadIdx.x < R16_LINES) {
    const int c = threadIdx.x, l = l0 + c, lc = l < nl ? l : nl - 1;
    const unsigned a1 = pr.l1 ? (unsigned)__ldg(pr.l1 + lc) : 1u;
    const unsigned a2 = (pr.t2 && pr.l2) ? (unsigned)__ldg(pr.l2 + lc) : 1u;
    zf[0][c] = l < nl && a1 != 0u;
    zf[1][c] = l < nl && pr.t2 && a2 != 0u;
    mine = zf[0][c] || zf[1][c];
  }
  if (!__syncthreads_or(mine)) {
    // no TERMA on these 16 lines: zeros in every plane, two lines per
    // aligned 16-byte store (lp is a multiple of 32, l0 of 16)
    for (int e = threadIdx.x; e < SPEC_PLANE_M * (R16_LINES / 2); e += SPEC_THREADS) {
      const int kz = e >> 3, c2 = (e & 7) * 2;
      *reinterpret_cast<float4*>(pr.a + (size_t)kz * lp + l0 + c2) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    return;
  }
  {
    const int j = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
    const bool f1 = zf[0][c], f2 = zf[1][c];
    const size_t o = (size_t)(l < nl ? l : 0) * P.g.zp;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int i = j + 16 * r;
      v[r] = make_float2(0.0f, 0.0f);
      if (r < 8 && i < nz) {
        if (f1) v[r].x = __ldg(pr.t1 + o + i);
        if (f2) v[r].y = __ldg(pr.t2 + o + i);
      }
    }
    r16_first<false, true>(v, true, sm, j, c);
  }
  __syncthreads();
  const int c = threadIdx.x & 15, j = threadIdx.x >> 4, l = l0 + c;
  float2 v[16];
  r16_second<false, true>(sm, v, j, c, P.g.tw[2]);
  if (l < nl) {
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) pr.a[(size_t)(j + 16 * (k1 + 4 * k2)) * lp + l] = v[4 * k1 + k2];
  }
}

// z inverse from plane-major A: stage 1 with lanes across the 16 lines
// (coalesced loads of one kz), stage 2 with lanes along z (coalesced dose
// rows).
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_ZINV_CTAS_PER_SM) spec_z_inverse_plane_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  const SpecPair& pr = P.p[blockIdx.y];
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2], lp = P.g.lp;
  const int l0 = blockIdx.x * R16_LINES;
  {
    const int c = threadIdx.x & 15, j = threadIdx.x >> 4, l = l0 + c;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = l < nl ? __ldg(pr.a + (size_t)(j + 16 * r) * lp + l) : make_float2(0.0f, 0.0f);
    r16_first<true, true>(v, false, sm, j, c);
  }
  __syncthreads();
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4, l = l0 + c;
  float2 v[16];
  r16_second<true, true>(sm, v, j, c, P.g.tw[2]);
  if (l < nl) {
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 2; ++k2) {
        const int i = j + 16 * (k1 + 4 * k2);
        if (i < nz) {
          pr.d1[(size_t)l * nz + i] = v[4 * k1 + k2].x;
          if (pr.d2) pr.d2[(size_t)l * nz + i] = v[4 * k1 + k2].y;
        }
      }
  }
}

// ---- plane kernel helpers: one warp transforms two lines of 256 (lanes
// 0-15 the first, 16-31 the second; lane j of a line holds butterfly j) with
// an exchange buffer of its own, so only __syncwarp orders the two stages.
// A 64-bit shared access is served per half warp, i.e. per line here: each
// line has its own 256 elements, element i at i ^ ((i / 16) mod 16), so that
// the stage-1 writes (rows 16 j + q) and the stage-2 reads (rows j + 16 r)
// of a line's 16 lanes fall in 16 different banks.
__device__ __forceinline__ int wx(int i, int c) { return c * 256 + (i ^ ((i >> 4) & 15)); }

template <bool INV>
__device__ __forceinline__ void w16_first(float2 (&v)[16], bool hin, float2* wb, int j, int c) {
  if (hin)
    dft16_half_in<INV>(v);
  else
    dft16<INV>(v);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) wb[wx(16 * j + k1 + 4 * k2, c)] = v[4 * k1 + k2];
}

// stage 2 with the twiddles exp(-2 pi i r j / 256), r = 0..15, of butterfly
// j from a shared table row twj = tws + 18 j (rows padded to 144 bytes), two
// twiddles per 16-byte load: the 16 lanes of a line then read 8 distinct
// 16-byte bank groups, two wavefronts, the minimum for 256 bytes (every
// transform of the plane kernel has period 256)
constexpr int PLANE_TW_ROW = 18;
template <bool INV>
__device__ __forceinline__ void w16_second(const float2* wb, float2 (&v)[16], int j, int c, const float2* twj) {
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = wb[wx(j + 16 * r, c)];
  const float4* tw4 = reinterpret_cast<const float4*>(twj);
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const float4 t = tw4[m];
    if (m > 0) v[2 * m] = cmul(v[2 * m], make_float2(t.x, INV ? -t.y : t.y));
    v[2 * m + 1] = cmul(v[2 * m + 1], make_float2(t.z, INV ? -t.w : t.w));
  }
  dft16<INV>(v);
}

// distributed shared memory: the partner CTA's copy of a shared address
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
  uint32_t out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"((uint32_t)__cvta_generic_to_shared(p)),
               "r"(rank));
  return out;
}
__device__ __forceinline__ void st_cluster(uint32_t a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float2 ld_cluster(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}
// split cluster barrier: release/acquire where one CTA reads what the other
// wrote, relaxed where it only orders running and exiting
__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// One kz plane of one beam pair per cluster of two CTAs.  CTA r of the
// cluster holds the ky in [128 r, 128 r + 128) of the plane's spectrum,
// Y[x][ky - 128 r] (x < nx <= 128; 128 KB), in its shared memory, element
// (x, k) at x * 128 + (k ^ (x mod 16)) so that a row (lanes along ky) and a
// column (lanes along x) are both conflict-free:
//   1. y forward: CTA r transforms rows x in [64 r, 64 r + 64) of A (y < ny,
//      the upper half zero; rows without TERMA in either beam skip the
//      transform) and stores each output ky into the CTA that holds it (its
//      own shared memory or its partner's);
//   2. per ky column of its half: x forward (x < nx), times S^[kz][ky][kx]
//      (or its conjugate), x inverse (x < nx kept), in place;
//   3. y inverse of its rows: the 256 ky of a row come half from each CTA;
//      rows y < ny go back to A.
// Every warp owns two lines at a time (rows in 1 and 3, columns in 2) with
// its own exchange buffer, so warps never wait for each other inside a
// phase.  The next pair's rows of A (phase 1) are loaded while the current
// pair transforms, the S^ values of a column pair while its forward
// transform runs.  Cluster barriers start the kernel (the partner is
// running before its shared memory is written; waited on just before the
// first stores), separate the phases (release/acquire) and end it (the
// partner has read this CTA's half before it exits); every thread reaches
// each of them once.  Consecutive clusters take the same kz of consecutive
// pairs, so that plane of S^ comes from L2 after the first.
constexpr int PLANE_THREADS = 512;
constexpr int PLANE_WARPS = PLANE_THREADS / 32;
static_assert(SPEC_PLANE_SMEM >= (128 * 128 + PLANE_WARPS * 2 * 256 + 16 * PLANE_TW_ROW) * 8,
              "plane kernel shared memory");

template <int R>
__device__ __forceinline__ void plane_store_rows(float2* Y, uint32_t peer, int x, int jx, const float2 (&v)[16]) {
  // outputs ky = j + 16 q, q = k1 + 4 k2: q < 8 in CTA 0, q >= 8 in CTA 1
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      const int off = x * 128 + jx + 16 * (k1 + 4 * (k2 & 1));
      if ((k2 >> 1) == R)
        Y[off] = v[4 * k1 + k2];
      else
        st_cluster(peer + 8u * (uint32_t)off, v[4 * k1 + k2]);
    }
}

template <int R>
__device__ __forceinline__ void plane_load_row(const float2* Y, uint32_t peer, int x, int jx, float2 (&v)[16]) {
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int off = x * 128 + jx + 16 * (q & 7);
    v[q] = (q >> 3) == R ? Y[off] : ld_cluster(peer + 8u * (uint32_t)off);
  }
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PLANE_THREADS, 1) spec_plane_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  constexpr int H = SPEC_PLANE_M / 2;              // ky per CTA, and the largest nx
  float2* const Y = spec_sm;                         // [H][H], swizzled
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = lane & 15, c = lane >> 4;            // butterfly, line of the warp
  float2* const wb = spec_sm + H * H + warp * 2 * SPEC_PLANE_M;
  const int r = (int)cluster_rank();
  const uint32_t peer = cluster_addr(Y, (uint32_t)(r ^ 1));
  const int nx = P.g.n[0], ny = P.g.n[1];
  const float cs = P.g.conj ? -1.0f : 1.0f;
  // stage-2 twiddles of every butterfly (period 256): [j][r], rows of 18
  float2* const tws = spec_sm + H * H + PLANE_WARPS * 2 * SPEC_PLANE_M;
  if (threadIdx.x < 256) {
    const int tj = threadIdx.x >> 4, tr = threadIdx.x & 15;
    tws[PLANE_TW_ROW * tj + tr] = __ldg(P.g.tw[0] + tr * tj);
  }
  __syncthreads();
  const float2* const tw = tws + PLANE_TW_ROW * j;
  constexpr int ROWS = H / 2 / (2 * PLANE_WARPS);    // row pairs per warp in phases 1 and 3
  constexpr int COLS = H / (2 * PLANE_WARPS);        // column pairs per warp in phase 2
  const int pair = blockIdx.x >> 1, kz = blockIdx.y;
  float2* const plane = P.p[pair].a + (size_t)kz * P.g.lp;
  const float2* const sh = P.g.shat + (size_t)kz * SPEC_PLANE_M * SPEC_PLANE_M + (size_t)H * r * SPEC_PLANE_M;
  auto row_of = [&](int it) { return (H / 2) * r + 2 * (PLANE_WARPS * it + warp) + c; };
  auto load_a = [&](int it, float2 (&v)[8]) {        // rows of A: y < ny, the upper half zero
    const int x = row_of(it);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int y = j + 16 * q;
      v[q] = (x < nx && y < ny) ? __ldg(plane + (size_t)x * ny + y) : make_float2(0.0f, 0.0f);
    }
  };
  auto col_of = [&](int it) { return 2 * (PLANE_WARPS * it + warp) + c; };

  cluster_arrive_relaxed();
  float2 pa[8];
  load_a(0, pa);

  // ---- 1. y forward
  for (int it = 0; it < ROWS; ++it) {
    const int x = row_of(it);
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = pa[q];
      v[q + 8] = make_float2(0.0f, 0.0f);
    }
    if (it + 1 < ROWS) load_a(it + 1, pa);
    // two rows without TERMA in either beam (a beam lights a band of the
    // plane): their spectra are zero, the transform is skipped
    bool nz = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) nz = nz || v[q].x != 0.0f || v[q].y != 0.0f;
    if (__any_sync(0xffffffffu, nz)) {
      w16_first<false>(v, true, wb, j, c);
      __syncwarp();
      w16_second<false>(wb, v, j, c, tw);
      __syncwarp();
    }
    if (it == 0) cluster_wait();                      // the partner runs: its half may be written
    if (x < nx) {
      if (r == 0)
        plane_store_rows<0>(Y, peer, x, j ^ (x & 15), v);
      else
        plane_store_rows<1>(Y, peer, x, j ^ (x & 15), v);
    }
  }
  cluster_arrive_release();
  cluster_wait();

  // ---- 2. x forward, times S^, x inverse, on the CTA's ky columns
  for (int it = 0; it < COLS; ++it) {
    const int k = col_of(it);
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int x = j + 16 * q;
      v[q] = (q < 8 && x < nx) ? Y[x * H + (k ^ j)] : make_float2(0.0f, 0.0f);
    }
    float2 sv[16];                        // S^[kz][ky][kx = j + 16 q], in flight during the forward transform
    {
      const float2* row = sh + (size_t)k * SPEC_PLANE_M + j;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        sv[q] = __ldg(row + 16 * q);
        sv[q].y *= cs;
      }
    }
    w16_first<false>(v, true, wb, j, c);
    __syncwarp();
    w16_second<false>(wb, v, j, c, tw);
    __syncwarp();
    float2 u[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) u[k1 + 4 * k2] = cmul(v[4 * k1 + k2], sv[k1 + 4 * k2]);
    w16_first<true>(u, false, wb, j, c);
    __syncwarp();
    w16_second<true>(wb, u, j, c, tw);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 2; ++k2) {
        const int x = j + 16 * (k1 + 4 * k2);
        if (x < nx) Y[x * H + (k ^ j)] = u[4 * k1 + k2];
      }
  }
  cluster_arrive_release();
  cluster_wait();

  // ---- 3. y inverse: the 256 ky of a row, half from each CTA
  for (int it = 0; it < ROWS; ++it) {
    const int x = row_of(it);
    float2 v[16];
    if (x < nx) {
      if (r == 0)
        plane_load_row<0>(Y, peer, x, j ^ (x & 15), v);
      else
        plane_load_row<1>(Y, peer, x, j ^ (x & 15), v);
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = make_float2(0.0f, 0.0f);
    }
    w16_first<true>(v, false, wb, j, c);
    __syncwarp();
    w16_second<true>(wb, v, j, c, tw);
    __syncwarp();
    if (x < nx) {
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 2; ++k2) {
          const int y = j + 16 * (k1 + 4 * k2);
          if (y < ny) plane[(size_t)x * ny + y] = v[4 * k1 + k2];
        }
    }
  }
  // the partner's loads of this CTA's half have all returned (their values
  // were used above) before it arrives: relaxed suffices
  cluster_arrive_relaxed();
  cluster_wait();
}

// S^ [Mx][My][Mz] -> [Mz][My][Mx]: 32 x 32 (kx, kz) tiles through shared
// memory, one ky per blockIdx.z
__global__ void spec_transpose_kernel(const float2* __restrict__ in, float2* __restrict__ out, int Mx, int My,
                                      int Mz) {
  __shared__ float2 t[32][33];
  const int ky = blockIdx.z, kx0 = blockIdx.y * 32, kz0 = blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int kx = kx0 + i, kz = kz0 + threadIdx.x;
    if (kx < Mx && kz < Mz) t[i][threadIdx.x] = in[((size_t)kx * My + ky) * Mz + kz];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int kz = kz0 + i, kx = kx0 + threadIdx.x;
    if (kx < Mx && kz < Mz) out[((size_t)kz * My + ky) * Mx + kx] = t[threadIdx.x][i];
  }
}

__global__ void spec_scatter_kernel(const long long* __restrict__ idx, const float* __restrict__ val, int n,
                                    float* __restrict__ S) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) S[idx[k]] = val[k];
}

// ---------------------------------------------------------------- host --
// Periods: 2^a and 3 * 2^a (a >= 4) up to SPEC_MAX_PERIOD, ascending.
std::vector<int> spec_periods() {
  std::vector<int> p;
  for (int m = SPEC_MIN_PERIOD; m <= SPEC_MAX_PERIOD; m *= 2) {
    p.push_back(m);
    if (3 * m <= SPEC_MAX_PERIOD) p.push_back(3 * m);
  }
  std::sort(p.begin(), p.end());
  return p;
}

int spec_period(int n) {
  for (int m : spec_periods())
    if (m >= 2 * n - 1) return m;
  return 0;
}

std::vector<float2> spec_twiddles() {
  std::vector<float2> t;
  for (int M : spec_periods())
    for (int k = 0; k < M; ++k) {
      const double a = -2.0 * 3.14159265358979323846 * (double)k / (double)M;
      t.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
    }
  return t;
}

size_t spec_twiddle_offset(int M) {
  size_t o = 0;
  for (int m : spec_periods()) {
    if (m == M) return o;
    o += m;
  }
  return o;
}

// log2 of the lines per CTA of a pass of period M: the largest power of two
// L with L M <= SPEC_ELEMS, for passes along y and x also dividing Mz
int spec_lines_log2(int M) {
  int l = 0;
  while ((2 << l) * M <= SPEC_ELEMS) ++l;
  return l;
}
int spec_pass_lines_log2(int M, int Mz) {
  int t = 0;
  while (((Mz >> t) & 1) == 0) ++t;
  return std::min(spec_lines_log2(M), t);
}

// Compile-time periods for the common shapes (grids of 17 to 256 voxels per
// axis): a pass is specialised when its lines per CTA are the natural ones.
// (periods 128, 192 and 384 take the 16 x N2 kernels on every axis)
#define SPEC_FOR_PERIODS(X) X(64, 6) X(96, 5) X(256, 4) X(512, 3)

template <int MP, int LL>
cudaError_t set_smem() {
  cudaError_t e = cudaSuccess;
  for (const void* f : {(const void*)spec_z_forward_kernel<MP, LL>, (const void*)spec_y_kernel<false, MP, LL>,
                        (const void*)spec_y_kernel<true, MP, LL>, (const void*)spec_x_kernel<false, MP, LL>,
                        (const void*)spec_x_kernel<true, MP, LL>, (const void*)spec_z_inverse_kernel<MP, LL>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, spec_smem<MP, LL>());
  return e;
}

cudaError_t setup_spec_kernels() {
  cudaError_t e = set_smem<-1, -1>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(spec_z_forward_plane_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPEC_ZPLANE_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(spec_z_inverse_plane_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPEC_ZPLANE_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(spec_plane_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SPEC_PLANE_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_x16n_kernel<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<24>(true));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_x16n_kernel<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<12>(true));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<false, 24>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<24>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<true, 24>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<24>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<false, 12>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<12>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<true, 12>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<12>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_forward_kernel<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<24>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_forward_kernel<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<12>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_inverse_kernel<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<24>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_inverse_kernel<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<12>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_x16n_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<8>(true));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<false, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<8>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_y16n_kernel<true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_smem<8>(false));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_forward_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<8>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(spec_z16n_inverse_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, r16n_zsmem<8>());
#define SPEC_SET(mp, ll) \
  if (e == cudaSuccess) e = set_smem<mp, ll>();
  SPEC_FOR_PERIODS(SPEC_SET)
#undef SPEC_SET
  return e;
}

// Each pass is launched specialised when (period, lines) is one of
// SPEC_FOR_PERIODS, generic otherwise.
void launch_spec_transpose(const float2* in, float2* out, int Mx, int My, int Mz, cudaStream_t st) {
  spec_transpose_kernel<<<dim3((Mz + 31) / 32, (Mx + 31) / 32, My), dim3(32, 8), 0, st>>>(in, out, Mx, My, Mz);
}

void launch_spec_pairs(const SpecLaunch& L, cudaStream_t st) {
  const SpecGrid& g = L.g;
  const int nl = g.n[0] * g.n[1];
  if (g.plane) {
    const dim3 gz((nl + R16_LINES - 1) / R16_LINES, L.n_pairs);
    spec_z_forward_plane_kernel<<<gz, SPEC_THREADS, SPEC_ZPLANE_SMEM, st>>>(L);
    // clusters of two along x: consecutive clusters take the same kz plane of
    // consecutive pairs
    spec_plane_kernel<<<dim3(2 * L.n_pairs, SPEC_PLANE_M), PLANE_THREADS, SPEC_PLANE_SMEM, st>>>(L);
    spec_z_inverse_plane_kernel<<<gz, SPEC_THREADS, SPEC_ZPLANE_SMEM, st>>>(L);
    return;
  }
  const int Lz = 1 << g.logL[2], Ly = 1 << g.logL[1], Lx = 1 << g.logL[0];
  const dim3 gz((nl + Lz - 1) / Lz, L.n_pairs), gy(g.n[0] * (g.M[2] / Ly), L.n_pairs);
  const unsigned gx = g.M[1] * (g.M[2] / Lx) * L.n_pairs;
  bool z_done = false, y_done = false, x_done = false;
#define SPEC_Z(mp, ll) \
  if (!z_done && g.M[2] == mp && g.logL[2] == ll) { spec_z_forward_kernel<mp, ll><<<gz, SPEC_THREADS, (spec_smem<mp, ll>()), st>>>(L); z_done = true; }
#define SPEC_Y(mp, ll) \
  if (!y_done && g.M[1] == mp && g.logL[1] == ll) { spec_y_kernel<false, mp, ll><<<gy, SPEC_THREADS, (spec_smem<mp, ll>()), st>>>(L); y_done = true; }
#define SPEC_X(mp, ll) \
  if (!x_done && g.M[0] == mp && g.logL[0] == ll) { spec_x_kernel<true, mp, ll><<<gx, SPEC_THREADS, (spec_smem<mp, ll>()), st>>>(L); x_done = true; }
  // periods 384 and 192 along z: the 16 x N2 kernels
  const int nz2 = 2 * g.n[2] <= g.M[2] ? (g.M[2] == 384 ? 24 : g.M[2] == 192 ? 12 : g.M[2] == 128 ? 8 : 0) : 0;
  const dim3 gz16((nl + 15) / 16, L.n_pairs);
  if (nz2 == 24) spec_z16n_forward_kernel<24><<<gz16, r16n_threads<24>(), r16n_zsmem<24>(), st>>>(L);
  if (nz2 == 12) spec_z16n_forward_kernel<12><<<gz16, r16n_threads<12>(), r16n_zsmem<12>(), st>>>(L);
  if (nz2 == 8) spec_z16n_forward_kernel<8><<<gz16, r16n_threads<8>(), r16n_zsmem<8>(), st>>>(L);
  z_done = nz2 != 0;
  SPEC_FOR_PERIODS(SPEC_Z)
  if (!z_done) spec_z_forward_kernel<-1, -1><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  // periods 384 and 192 along y and x: the 16 x N2 kernels (16 lines per CTA)
  const int ny2 = g.M[2] % 16 == 0 && 2 * g.n[1] <= g.M[1] ? (g.M[1] == 384 ? 24 : g.M[1] == 192 ? 12 : g.M[1] == 128 ? 8 : 0) : 0;
  const int nx2 = g.M[2] % 16 == 0 && 2 * g.n[0] <= g.M[0] ? (g.M[0] == 384 ? 24 : g.M[0] == 192 ? 12 : g.M[0] == 128 ? 8 : 0) : 0;
  const dim3 gy16(g.n[0] * (g.M[2] / 16), L.n_pairs);
  const unsigned gx16 = g.M[1] * (g.M[2] / 16) * L.n_pairs;
  if (ny2 == 24) spec_y16n_kernel<false, 24><<<gy16, r16n_threads<24>(), r16n_smem<24>(false), st>>>(L);
  if (ny2 == 12) spec_y16n_kernel<false, 12><<<gy16, r16n_threads<12>(), r16n_smem<12>(false), st>>>(L);
  if (ny2 == 8) spec_y16n_kernel<false, 8><<<gy16, r16n_threads<8>(), r16n_smem<8>(false), st>>>(L);
  y_done = ny2 != 0;
  SPEC_FOR_PERIODS(SPEC_Y)
  if (!y_done) spec_y_kernel<false, -1, -1><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  if (nx2 == 24) spec_x16n_kernel<24><<<gx16, r16n_threads<24>(), r16n_smem<24>(true), st>>>(L);
  if (nx2 == 12) spec_x16n_kernel<12><<<gx16, r16n_threads<12>(), r16n_smem<12>(true), st>>>(L);
  if (nx2 == 8) spec_x16n_kernel<8><<<gx16, r16n_threads<8>(), r16n_smem<8>(true), st>>>(L);
  x_done = nx2 != 0;
  SPEC_FOR_PERIODS(SPEC_X)
  if (!x_done) spec_x_kernel<true, -1, -1><<<gx, SPEC_THREADS, SPEC_SMEM, st>>>(L);
#undef SPEC_Z
#undef SPEC_Y
#undef SPEC_X
  y_done = z_done = false;
#define SPEC_YI(mp, ll) \
  if (!y_done && g.M[1] == mp && g.logL[1] == ll) { spec_y_kernel<true, mp, ll><<<gy, SPEC_THREADS, (spec_smem<mp, ll>()), st>>>(L); y_done = true; }
#define SPEC_ZI(mp, ll) \
  if (!z_done && g.M[2] == mp && g.logL[2] == ll) { spec_z_inverse_kernel<mp, ll><<<gz, SPEC_THREADS, (spec_smem<mp, ll>()), st>>>(L); z_done = true; }
  if (ny2 == 24) spec_y16n_kernel<true, 24><<<gy16, r16n_threads<24>(), r16n_smem<24>(false), st>>>(L);
  if (ny2 == 12) spec_y16n_kernel<true, 12><<<gy16, r16n_threads<12>(), r16n_smem<12>(false), st>>>(L);
  if (ny2 == 8) spec_y16n_kernel<true, 8><<<gy16, r16n_threads<8>(), r16n_smem<8>(false), st>>>(L);
  y_done = ny2 != 0;
  SPEC_FOR_PERIODS(SPEC_YI)
  if (!y_done) spec_y_kernel<true, -1, -1><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  if (nz2 == 24) spec_z16n_inverse_kernel<24><<<gz16, r16n_threads<24>(), r16n_zsmem<24>(), st>>>(L);
  if (nz2 == 12) spec_z16n_inverse_kernel<12><<<gz16, r16n_threads<12>(), r16n_zsmem<12>(), st>>>(L);
  if (nz2 == 8) spec_z16n_inverse_kernel<8><<<gz16, r16n_threads<8>(), r16n_zsmem<8>(), st>>>(L);
  z_done = nz2 != 0;
  SPEC_FOR_PERIODS(SPEC_ZI)
  if (!z_done) spec_z_inverse_kernel<-1, -1><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L);
#undef SPEC_YI
#undef SPEC_ZI
}

void launch_spec_build(const SpecLaunch& L, const long long* idx, const float* val, int n_val, float* s_real,
                       cudaStream_t st) {
  const SpecGrid& g = L.g;
  const int nl = g.n[0] * g.n[1];
  const int Lz = 1 << g.logL[2], Ly = 1 << g.logL[1], Lx = 1 << g.logL[0];
  if (n_val > 0) spec_scatter_kernel<<<(n_val + 255) / 256, 256, 0, st>>>(idx, val, n_val, s_real);
  spec_z_forward_kernel<-1, -1><<<dim3((nl + Lz - 1) / Lz, 1), SPEC_THREADS, SPEC_SMEM, st>>>(L);
  spec_y_kernel<false, -1, -1><<<dim3(g.n[0] * (g.M[2] / Ly), 1), SPEC_THREADS, SPEC_SMEM, st>>>(L);
  spec_x_kernel<false, -1, -1><<<g.M[1] * (g.M[2] / Lx), SPEC_THREADS, SPEC_SMEM, st>>>(L);
}

}  // namespace ch
