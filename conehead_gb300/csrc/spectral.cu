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
// power-of-two length M along one axis.  A CTA holds 4096 complex values
// (L = 4096 / M lines) in shared memory, element (i, line c) at
// i * L + (c ^ (i mod L)) so that both line-major and index-major sweeps are
// free of bank conflicts, and runs radix-4 Stockham stages (one radix-2 stage
// when log2 M is odd) with twiddles from a host-built table.  The passes skip
// the zero padding:
//   z forward  TERMA pair [nx][ny][nz] (pitch zp)  -> A [nx][ny][Mz]
//   y forward  A (y < ny)                          -> B [nx][My][Mz]
//   x          B (x < nx): forward, times S^, inverse, x < nx kept (in place)
//   y inverse  B                                   -> A (y < ny)
//   z inverse  A                                   -> dose pair [nx][ny][nz]
// Every global sweep is coalesced: lines along z are read and written along
// z, lines along y and x are taken in blocks of L consecutive kz.

#include <cmath>
#include <vector>

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
  v[10] = rot<INV>(v[10], 0.0f, 1.0f);   // 4
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
  v[10] = rot<INV>(v[10], 0.0f, 1.0f);
  v[14] = rot<INV>(v[14], -R2, R2);
  v[7] = rot<INV>(v[7], S1, C1);
  v[11] = rot<INV>(v[11], -R2, R2);
  v[15] = rot<INV>(v[15], -C1, -S1);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// One Stockham stage from src to dst (element (i, line c) layout above) on L
// lines of period M; Ns = 2^logNs is the sub-transform size done so far and
// tw[k] = exp(-2 pi i k / M).  A thread takes one butterfly at a time.
// hin: the first stage of a transform whose input's upper half is zero (it
// reads only r < 8); hout: the last stage of one whose output's upper half
// is not wanted (it writes only the lower half).
template <bool INV>
__device__ __forceinline__ void stage16(const float2* src, float2* dst, int M, int L, int logL, int logNs,
                                        const float2* __restrict__ tw, bool hin, bool hout) {
  const int Ns = 1 << logNs, MR = M >> 4, nb = L * MR, step = M >> (logNs + 4);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j & (Ns - 1);
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
    const int o = ((j - k) << 4) + k;
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
__device__ __forceinline__ void stage4(const float2* src, float2* dst, int M, int L, int logL, int logNs,
                                       const float2* __restrict__ tw, bool hout) {
  const int Ns = 1 << logNs, MR = M >> 2, nb = L * MR, step = M >> (logNs + 2);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j & (Ns - 1);
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
    const int o = ((j - k) << 2) + k;
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
__device__ __forceinline__ void stage2(const float2* src, float2* dst, int M, int L, int logL, int logNs,
                                       const float2* __restrict__ tw, bool hout) {
  const int Ns = 1 << logNs, MR = M >> 1, nb = L * MR, step = M >> (logNs + 1);
  for (int bf = threadIdx.x; bf < nb; bf += SPEC_THREADS) {
    const int c = bf & (L - 1), j = bf >> logL, k = j & (Ns - 1);
    float2 w = __ldg(tw + k * step);
    if (INV) w.y = -w.y;
    const float2 a0 = src[swz(j, c, L)], a1 = cmul(src[swz(j + MR, c, L)], w);
    const int o = ((j - k) << 1) + k;
    dst[swz(o, c, L)] = make_float2(a0.x + a1.x, a0.y + a1.y);
    if (!hout) dst[swz(o + Ns, c, L)] = make_float2(a0.x - a1.x, a0.y - a1.y);
  }
}

// FFT of the L lines of period M held in src, ping-ponging with dst; returns
// the buffer holding the result.  INV uses the conjugate twiddles (no 1/M
// scale).  Stockham stages of radix 16 while four or more factors of two
// remain, then radix 4 and 2 (256 points take two stages); every stage ends
// with one barrier.  The caller has synchronised after filling src.
// LM, LL >= 0 fix log2 M and log2 L at compile time (the stages unroll and
// the shared-memory addresses fold); -1 takes them at run time.  half_in:
// the input's upper half is zero; half_out: only the output's lower half is
// wanted (the upper half of the result buffer is then left stale).
template <bool INV, int LM, int LL>
__device__ __forceinline__ float2* fft_block(float2* src, float2* dst, int logM_rt, int logL_rt,
                                             const float2* __restrict__ tw, bool half_in, bool half_out) {
  const int logM = LM >= 0 ? LM : logM_rt, logL = LL >= 0 ? LL : logL_rt;
  const int M = 1 << logM, L = 1 << logL;
  int logNs = 0;
#pragma unroll
  for (int st = 0; st < (LM >= 0 ? LM / 4 : 3); ++st) {
    if (LM < 0 && logM - logNs < 4) break;
    stage16<INV>(src, dst, M, L, logL, logNs, tw, half_in && logNs == 0, half_out && logNs + 4 == logM);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    logNs += 4;
  }
  if (logM - logNs >= 2) {
    stage4<INV>(src, dst, M, L, logL, logNs, tw, half_out && logNs + 2 == logM);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
    logNs += 2;
  }
  if (logM - logNs >= 1) {
    stage2<INV>(src, dst, M, L, logL, logNs, tw, half_out);
    __syncthreads();
    float2* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// ---------------------------------------------------------------- passes --
// Every pass is a template on LM = log2 of its period and LL = log2 of its
// lines per CTA: >= 0 fixes them at compile time, -1 reads them from the
// launch.
// z forward: lines (x, y), TERMA pair in, A out.  One CTA per L lines and pair.
template <int LM>
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_CTAS_PER_SM) spec_z_forward_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + SPEC_ELEMS;
  const SpecPair& pr = P.p[blockIdx.y];
  const int logMz = LM >= 0 ? LM : P.g.logM[2], Mz = 1 << logMz;
  const int logL = 12 - logMz, L = 1 << logL;
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * L;
  {
    // every load of the thread first, then the shared-memory stores
    float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int i = e & (Mz - 1), c = e >> logMz, l = l0 + c;
      v[q] = make_float2(0.0f, 0.0f);
      if (l < nl && i < nz) {
        const size_t o = (size_t)l * P.g.zp + i;
        v[q].x = __ldg(pr.t1 + o);
        if (pr.t2) v[q].y = __ldg(pr.t2 + o);
      }
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      sm[swz(e & (Mz - 1), e >> logMz, L)] = v[q];
    }
  }
  __syncthreads();
  const float2* res =
      fft_block<false, LM, (LM >= 0 ? 12 - LM : -1)>(sm, sm2, logMz, logL, P.g.tw[2], 2 * nz <= Mz, false);
  for (int e = threadIdx.x; e < SPEC_ELEMS; e += SPEC_THREADS) {
    const int i = e & (Mz - 1), c = e >> logMz, l = l0 + c;
    if (l < nl) pr.a[(size_t)l * Mz + i] = res[swz(i, c, L)];
  }
}

// y forward (A -> B) or inverse (B -> A): lines (x, kz) in blocks of L kz.
template <bool INV, int LM, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_CTAS_PER_SM) spec_y_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + SPEC_ELEMS;
  const SpecPair& pr = P.p[blockIdx.y];
  const int logMy = LM >= 0 ? LM : P.g.logM[1], My = 1 << logMy, Mz = P.g.M[2], logMz = P.g.logM[2];
  const int logL = LL >= 0 ? LL : min(12 - logMy, logMz), L = 1 << logL;
  const int nkb = Mz >> logL;
  const int x = blockIdx.x / nkb, kz0 = (blockIdx.x - x * nkb) << logL;
  const int ny = P.g.n[1];
  const int n_in = INV ? My : ny, n_out = INV ? ny : My;
  const float2* src = INV ? pr.b + (size_t)x * My * Mz : pr.a + (size_t)x * ny * Mz;
  float2* dst = INV ? pr.a + (size_t)x * ny * Mz : pr.b + (size_t)x * My * Mz;
  src += kz0;
  dst += kz0;
  {
    float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int c = e & (L - 1), i = e >> logL;
      v[q] = (e < (L << logMy) && i < n_in) ? src[(size_t)i * Mz + c] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      if (e < (L << logMy)) sm[swz(e >> logL, e & (L - 1), L)] = v[q];
    }
  }
  __syncthreads();
  const float2* res = fft_block<INV, LM, LL>(sm, sm2, logMy, logL, P.g.tw[1], !INV && 2 * ny <= My,
                                             INV && 2 * ny <= My);
  for (int e = threadIdx.x; e < n_out * L; e += SPEC_THREADS) {
    const int c = e & (L - 1), i = e >> logL;
    dst[(size_t)i * Mz + c] = res[swz(i, c, L)];
  }
}

// x pass on B, lines (ky, kz) in blocks of L kz; consecutive CTAs take the
// same lines of consecutive pairs, so each block of S^ is read from L2.
// CONV: forward, times S^ (or its conjugate), inverse, x < nx kept;
// otherwise forward only over the full period (building S^).
template <bool CONV, int LM, int LL>
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_CTAS_PER_SM) spec_x_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + SPEC_ELEMS;
  const int pair = blockIdx.x % P.n_pairs, blk = blockIdx.x / P.n_pairs;
  const SpecPair& pr = P.p[pair];
  const int logMx = LM >= 0 ? LM : P.g.logM[0], Mx = 1 << logMx, My = P.g.M[1], Mz = P.g.M[2];
  const int logMz = P.g.logM[2];
  const int logL = LL >= 0 ? LL : min(12 - logMx, logMz), L = 1 << logL;
  const int nkb = Mz >> logL;
  const int ky = blk / nkb, kz0 = (blk - ky * nkb) << logL;
  const size_t xs = (size_t)My * Mz, off = (size_t)ky * Mz + kz0;
  float2* b = pr.b + off;
  const int nx = CONV ? P.g.n[0] : Mx;
  {
    float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int c = e & (L - 1), i = e >> logL;
      v[q] = (e < (L << logMx) && i < nx) ? b[(size_t)i * xs + c] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      if (e < (L << logMx)) sm[swz(e >> logL, e & (L - 1), L)] = v[q];
    }
  }
  __syncthreads();
  float2* res = fft_block<false, LM, LL>(sm, sm2, logMx, logL, P.g.tw[0], 2 * nx <= Mx, false);
  if (CONV) {
    const float2* sh = P.g.shat + off;
    float2 sv[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      sv[q] = e < (L << logMx) ? __ldg(sh + (size_t)(e >> logL) * xs + (e & (L - 1))) : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      if (e < (L << logMx)) {
        float2 s = sv[q];
        if (P.g.conj) s.y = -s.y;
        const int k = swz(e >> logL, e & (L - 1), L);
        res[k] = cmul(res[k], s);
      }
    }
    __syncthreads();
    res = fft_block<true, LM, LL>(res, res == sm ? sm2 : sm, logMx, logL, P.g.tw[0], false, 2 * nx <= Mx);
  }
  for (int e = threadIdx.x; e < nx * L; e += SPEC_THREADS) {
    const int c = e & (L - 1), i = e >> logL;
    b[(size_t)i * xs + c] = res[swz(i, c, L)];
  }
}

// z inverse: lines (x, y), A in, dose pair out (real part, imaginary part).
template <int LM>
__global__ void __launch_bounds__(SPEC_THREADS, SPEC_CTAS_PER_SM) spec_z_inverse_kernel(SpecLaunch P) {
  extern __shared__ float2 spec_sm[];
  float2* sm = spec_sm;
  float2* sm2 = spec_sm + SPEC_ELEMS;
  const SpecPair& pr = P.p[blockIdx.y];
  const int logMz = LM >= 0 ? LM : P.g.logM[2], Mz = 1 << logMz;
  const int logL = 12 - logMz, L = 1 << logL;
  const int nl = P.g.n[0] * P.g.n[1], nz = P.g.n[2];
  const int l0 = blockIdx.x * L;
  {
    float2 v[SPEC_ELEMS / SPEC_THREADS];
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      const int l = l0 + (e >> logMz);
      v[q] = l < nl ? pr.a[(size_t)l * Mz + (e & (Mz - 1))] : make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int q = 0; q < SPEC_ELEMS / SPEC_THREADS; ++q) {
      const int e = threadIdx.x + q * SPEC_THREADS;
      sm[swz(e & (Mz - 1), e >> logMz, L)] = v[q];
    }
  }
  __syncthreads();
  const float2* res =
      fft_block<true, LM, (LM >= 0 ? 12 - LM : -1)>(sm, sm2, logMz, logL, P.g.tw[2], false, 2 * nz <= Mz);
  for (int e = threadIdx.x; e < SPEC_ELEMS; e += SPEC_THREADS) {
    const int i = e & (Mz - 1), c = e >> logMz, l = l0 + c;
    if (l < nl && i < nz) {
      const float2 v = res[swz(i, c, L)];
      pr.d1[(size_t)l * nz + i] = v.x;
      if (pr.d2) pr.d2[(size_t)l * nz + i] = v.y;
    }
  }
}

__global__ void spec_scatter_kernel(const long long* __restrict__ idx, const float* __restrict__ val, int n,
                                    float* __restrict__ S) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) S[idx[k]] = val[k];
}

// ---------------------------------------------------------------- host --
int spec_period(int n) {
  int m = SPEC_MIN_PERIOD;
  while (m < 2 * n - 1) m <<= 1;
  return m;
}

std::vector<float2> spec_twiddles() {
  std::vector<float2> t;
  for (int M = SPEC_MIN_PERIOD; M <= SPEC_MAX_PERIOD; M <<= 1)
    for (int k = 0; k < M; ++k) {
      const double a = -2.0 * 3.14159265358979323846 * (double)k / (double)M;
      t.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
    }
  return t;
}

size_t spec_twiddle_offset(int M) { return (size_t)M - SPEC_MIN_PERIOD; }

// Compile-time periods for the common shapes (grids of 17 to 256 voxels per
// axis): a pass is specialised when its lines per CTA are 4096 / M.
#define SPEC_FOR_PERIODS(X) X(6, 6) X(7, 5) X(8, 4) X(9, 3)

template <int LM, int LL>
cudaError_t set_smem() {
  cudaError_t e = cudaSuccess;
  for (const void* f : {(const void*)spec_z_forward_kernel<LM>, (const void*)spec_y_kernel<false, LM, LL>,
                        (const void*)spec_y_kernel<true, LM, LL>, (const void*)spec_x_kernel<false, LM, LL>,
                        (const void*)spec_x_kernel<true, LM, LL>, (const void*)spec_z_inverse_kernel<LM>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, SPEC_SMEM);
  return e;
}

cudaError_t setup_spec_kernels() {
  cudaError_t e = set_smem<-1, -1>();
#define SPEC_SET(lm, ll) \
  if (e == cudaSuccess) e = set_smem<lm, ll>();
  SPEC_FOR_PERIODS(SPEC_SET)
#undef SPEC_SET
  return e;
}

// Each pass is launched specialised when (log2 M, log2 L) is one of
// SPEC_FOR_PERIODS, generic otherwise.
void launch_spec_pairs(const SpecLaunch& L, cudaStream_t st) {
  const SpecGrid& g = L.g;
  const int nl = g.n[0] * g.n[1];
  const int Lz = SPEC_ELEMS / g.M[2];
  const int Ly = std::min(SPEC_ELEMS / g.M[1], g.M[2]);
  const int Lx = std::min(SPEC_ELEMS / g.M[0], g.M[2]);
  const dim3 gz((nl + Lz - 1) / Lz, L.n_pairs), gy(g.n[0] * (g.M[2] / Ly), L.n_pairs);
  const unsigned gx = g.M[1] * (g.M[2] / Lx) * L.n_pairs;
  const int lz = g.logM[2], ly = g.logM[1], lx = g.logM[0];
  const bool sy = (SPEC_ELEMS / g.M[1]) == Ly, sx = (SPEC_ELEMS / g.M[0]) == Lx;
  bool z_done = false, y_done = false, x_done = false;
#define SPEC_Z(lm, ll) \
  if (!z_done && lz == lm) { spec_z_forward_kernel<lm><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L); z_done = true; }
#define SPEC_Y(lm, ll) \
  if (!y_done && sy && ly == lm) { spec_y_kernel<false, lm, ll><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L); y_done = true; }
#define SPEC_X(lm, ll) \
  if (!x_done && sx && lx == lm) { spec_x_kernel<true, lm, ll><<<gx, SPEC_THREADS, SPEC_SMEM, st>>>(L); x_done = true; }
  SPEC_FOR_PERIODS(SPEC_Z)
  if (!z_done) spec_z_forward_kernel<-1><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  SPEC_FOR_PERIODS(SPEC_Y)
  if (!y_done) spec_y_kernel<false, -1, -1><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  SPEC_FOR_PERIODS(SPEC_X)
  if (!x_done) spec_x_kernel<true, -1, -1><<<gx, SPEC_THREADS, SPEC_SMEM, st>>>(L);
#undef SPEC_Z
#undef SPEC_Y
#undef SPEC_X
  y_done = z_done = false;
#define SPEC_YI(lm, ll) \
  if (!y_done && sy && ly == lm) { spec_y_kernel<true, lm, ll><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L); y_done = true; }
#define SPEC_ZI(lm, ll) \
  if (!z_done && lz == lm) { spec_z_inverse_kernel<lm><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L); z_done = true; }
  SPEC_FOR_PERIODS(SPEC_YI)
  if (!y_done) spec_y_kernel<true, -1, -1><<<gy, SPEC_THREADS, SPEC_SMEM, st>>>(L);
  SPEC_FOR_PERIODS(SPEC_ZI)
  if (!z_done) spec_z_inverse_kernel<-1><<<gz, SPEC_THREADS, SPEC_SMEM, st>>>(L);
#undef SPEC_YI
#undef SPEC_ZI
}

void launch_spec_build(const SpecLaunch& L, const long long* idx, const float* val, int n_val, float* s_real,
                       cudaStream_t st) {
  const SpecGrid& g = L.g;
  const int nl = g.n[0] * g.n[1];
  const int Lz = SPEC_ELEMS / g.M[2];
  const int Ly = std::min(SPEC_ELEMS / g.M[1], g.M[2]);
  const int Lx = std::min(SPEC_ELEMS / g.M[0], g.M[2]);
  if (n_val > 0) spec_scatter_kernel<<<(n_val + 255) / 256, 256, 0, st>>>(idx, val, n_val, s_real);
  spec_z_forward_kernel<-1><<<dim3((nl + Lz - 1) / Lz, 1), SPEC_THREADS, SPEC_SMEM, st>>>(L);
  spec_y_kernel<false, -1, -1><<<dim3(g.n[0] * (g.M[2] / Ly), 1), SPEC_THREADS, SPEC_SMEM, st>>>(L);
  spec_x_kernel<false, -1, -1><<<g.M[1] * (g.M[2] / Lx), SPEC_THREADS, SPEC_SMEM, st>>>(L);
}

}  // namespace ch
