// Cone-direction stencils and the plain (scatter) cone path.
//
// Key fact used by the gather path (conehead/conehead.py:385-488): the DDA
// from a voxel *centre* along a fixed direction visits offsets O_d[m] and
// exit distances t_d[m] that do not depend on the start voxel; only the
// grid exit truncates the walk, and because every axis steps monotonically
// "source and target inside the grid" implies the whole walk is inside.
// So the reference's scatter equals
//     dose(v) = sum_d sum_m T(v - O_d[m]) * dK_d[m]
// with dK_d[m] = K[phi_d, idx_m] - K[phi_d, idx_{m-1}] (dK_d[0] = K[idx_0]),
// idx_m = |floor(100 t_m - 5)| clamped to 5995.
//
// stencil_kernel builds O_d, t_d and dK_d for every (theta_i, phi_j) with the
// reference's arithmetic (float64 trigonometry stored to float32, float32
// normalisation, the float32 DDA of cuda_dda_3d :123-206).

#include "ch_internal.cuh"

namespace ch {

__device__ __forceinline__ void cone_direction(float theta_deg, float phi_deg, float* d) {
  // theta * pi / 180 in float64 (float32 * math.pi promotes), trig in float64
  const double th = ddiv(dmul((double)theta_deg, 3.141592653589793), 180.0);
  const double ph = ddiv(dmul((double)phi_deg, 3.141592653589793), 180.0);
  const double ct = cos(th), st = sin(th), cp = cos(ph), sp = sin(ph);
  float d0 = d2f(dmul(ct, sp)), d1 = d2f(cp), d2 = d2f(dmul(st, sp));
  const float nrm = __fsqrt_rn(fadd(fadd(fmul(d0, d0), fmul(d1, d1)), fmul(d2, d2)));
  d[0] = fdiv(d0, nrm);
  d[1] = fdiv(d1, nrm);
  d[2] = fdiv(d2, nrm);
}

__device__ __forceinline__ int kernel_index(float t) {
  long long i = (long long)floor(dsub(dmul((double)t, 100.0), 5.0));
  if (i < 0) i = -i;
  if (i > 5995) i = 5995;
  return (int)i;
}

// One thread per (theta_i, phi_j).  Walks at most max_len taps and stops at
// the first tap that cannot fit in a grid of dims cap[] (|O_k| > cap_k - 1)
// or once the kernel index has saturated (all further dK are zero).
__global__ void stencil_kernel(const float* __restrict__ theta, int n_theta, const float* __restrict__ phi,
                               int n_phi, const double* __restrict__ K, int n_r, float sx, float sy, float sz,
                               int cap0, int cap1, int cap2, int max_len, short4* __restrict__ off_out,
                               float* __restrict__ t_out, float* __restrict__ dk_out,
                               int* __restrict__ len_out, float* __restrict__ dir_out, ConeFrame frame) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n_theta * n_phi) return;
  const int i = id / n_phi, j = id % n_phi;
  float d[3];
  cone_direction(theta[i], phi[j], d);
  if (frame.on) {
    // cones in the beam frame: d_room[k] = sum_i xform[i][k] d[i] (the rows of
    // the beam's world->beam rotation are its axes); float64, one rounding
    float r[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      r[k] = d2f(dadd(dadd(dmul(frame.m[k], (double)d[0]), dmul(frame.m[3 + k], (double)d[1])),
                      dmul(frame.m[6 + k], (double)d[2])));
    d[0] = r[0];
    d[1] = r[1];
    d[2] = r[2];
  }
  dir_out[3 * id + 0] = d[0];
  dir_out[3 * id + 1] = d[1];
  dir_out[3 * id + 2] = d[2];
  int s0, s1, s2;
  float t0, t1, t2, e0, e1, e2;
  dda_axis(d[0], sx, s0, t0, e0);
  dda_axis(d[1], sy, s1, t1, e1);
  dda_axis(d[2], sz, s2, t2, e2);
  int o0 = 0, o1 = 0, o2 = 0;
  const double* Kj = K + (size_t)j * n_r;
  int prev = -1;
  int m = 0;
  const size_t base = (size_t)id * max_len;
  for (; m < max_len; ++m) {
    if (abs(o0) > cap0 - 1 || abs(o1) > cap1 - 1 || abs(o2) > cap2 - 1) break;
    float tv;
    int ax;
    if (t0 < t1) {
      if (t0 < t2) { tv = t0; ax = 0; } else { tv = t2; ax = 2; }
    } else {
      if (t1 < t2) { tv = t1; ax = 1; } else { tv = t2; ax = 2; }
    }
    const int ki = kernel_index(tv);
    if (prev == 5995 && ki == 5995) break;  // dK == 0 from here on
    const double dk = prev < 0 ? Kj[ki] : dsub(Kj[ki], Kj[prev]);
    prev = ki;
    off_out[base + m] = make_short4((short)o0, (short)o1, (short)o2, (short)ax);
    t_out[base + m] = tv;
    dk_out[base + m] = d2f(dk);
    if (ax == 0) { t0 = fadd(t0, e0); o0 += s0; }
    else if (ax == 1) { t1 = fadd(t1, e1); o1 += s1; }
    else { t2 = fadd(t2, e2); o2 += s2; }
  }
  len_out[id] = m;
}

// New spectrum, same walks: tap weights w = mult * f32(K[row][ki] - K[row][prev])
// recomputed from the stored t values exactly as stencil_kernel forms them,
// written to the tap table and to the tap's slot in its run record.
// One thread per unique walk.
__global__ void reweight_kernel(const double* __restrict__ K, int n_r, int n_walks, const int* __restrict__ tap_base,
                                const int* __restrict__ tap_len, const float* __restrict__ tvals,
                                const int* __restrict__ walk_row, const int* __restrict__ walk_mult,
                                int4* __restrict__ taps, const int* __restrict__ tap_run, int4* __restrict__ runs) {
  int* run_words = reinterpret_cast<int*>(runs);
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n_walks) return;
  const double* Kj = K + (size_t)walk_row[u] * n_r;
  const float mult = (float)walk_mult[u];
  const int b = tap_base[u], L = tap_len[u];
  int prev = -1;
  for (int m = 0; m < L; ++m) {
    const int ki = kernel_index(tvals[b + m]);
    const double dk = prev < 0 ? Kj[ki] : dsub(Kj[ki], Kj[prev]);
    prev = ki;
    const int wbits = __float_as_int(__fmul_rn(d2f(dk), mult));
    taps[b + m].w = wbits;
    run_words[tap_run[b + m]] = wbits;
  }
}

void launch_reweight(const double* K, int n_r, int n_walks, const int* tap_base, const int* tap_len,
                     const float* tvals, const int* walk_row, const int* walk_mult, int4* taps, const int* tap_run,
                     int4* runs, cudaStream_t st) {
  reweight_kernel<<<(n_walks + 127) / 128, 128, 0, st>>>(K, n_r, n_walks, tap_base, tap_len, tvals, walk_row,
                                                         walk_mult, taps, tap_run, runs);
}

void launch_stencil(const float* theta, int n_theta, const float* phi, int n_phi, const double* K, int n_r,
                    const float* spacing, const int* cap, int max_len, short4* off, float* t, float* dk,
                    int* len, float* dirs, const ConeFrame& frame, cudaStream_t st) {
  const int n = n_theta * n_phi;
  stencil_kernel<<<(n + 127) / 128, 128, 0, st>>>(theta, n_theta, phi, n_phi, K, n_r, spacing[0], spacing[1],
                                                 spacing[2], cap[0], cap[1], cap[2], max_len, off, t, dk, len,
                                                 dirs, frame);
}

// ------------------------------------------------------------- DDA hook --
__global__ void dda_trace_kernel(int n0, int n1, int n2, float sx, float sy, float sz, int n_rays,
                                 const int* __restrict__ starts, const float* __restrict__ dirs, int cap,
                                 int* __restrict__ vox, float* __restrict__ tv, int* __restrict__ len) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  int s0, s1, s2;
  float t0, t1, t2, e0, e1, e2;
  dda_axis(dirs[3 * r + 0], sx, s0, t0, e0);
  dda_axis(dirs[3 * r + 1], sy, s1, t1, e1);
  dda_axis(dirs[3 * r + 2], sz, s2, t2, e2);
  int c0 = starts[3 * r + 0], c1 = starts[3 * r + 1], c2 = starts[3 * r + 2];
  int m = 0;
  while (c0 >= 0 && c0 < n0 && c1 >= 0 && c1 < n1 && c2 >= 0 && c2 < n2) {
    float t;
    const int v0 = c0, v1 = c1, v2 = c2;
    if (t0 < t1) {
      if (t0 < t2) { t = t0; t0 = fadd(t0, e0); c0 += s0; }
      else { t = t2; t2 = fadd(t2, e2); c2 += s2; }
    } else {
      if (t1 < t2) { t = t1; t1 = fadd(t1, e1); c1 += s1; }
      else { t = t2; t2 = fadd(t2, e2); c2 += s2; }
    }
    if (m < cap) {
      const size_t o = (size_t)r * cap + m;
      vox[3 * o + 0] = v0;
      vox[3 * o + 1] = v1;
      vox[3 * o + 2] = v2;
      tv[o] = t;
    }
    ++m;
  }
  len[r] = m;
}

void launch_dda_trace(const int* n, const float* sp, int n_rays, const int* starts, const float* dirs, int cap,
                      int* vox, float* t, int* len, cudaStream_t st) {
  dda_trace_kernel<<<(n_rays + 127) / 128, 128, 0, st>>>(n[0], n[1], n[2], sp[0], sp[1], sp[2], n_rays, starts,
                                                        dirs, cap, vox, t, len);
}

// ------------------------------------------------------- plain scatter --
// The reference's cone kernel structure: one thread per TERMA voxel, every
// direction walked to the grid edge, float32 atomic adds into the dose.
// Uses the deduplicated stencils (identical walks merged, dK scaled by the
// multiplicity) so it does the same arithmetic as the gather path.
__global__ void __launch_bounds__(128) scatter_kernel(const float* __restrict__ T, int n0, int n1, int n2,
                                                      int zp, int n_dirs, const int* __restrict__ tap_base,
                                                      const int* __restrict__ tap_len,
                                                      const short4* __restrict__ offs,
                                                      const int4* __restrict__ taps, float* __restrict__ dose) {
  const long long N = (long long)n0 * n1 * n2;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N) return;
  const int z = (int)(v % n2);
  const long long r = v / n2;
  const int y = (int)(r % n1), x = (int)(r / n1);
  const float Tv = T[((long long)x * n1 + y) * zp + z];
  if (Tv == 0.0f) return;
  for (int u = 0; u < n_dirs; ++u) {
    const int b = tap_base[u], L = tap_len[u];
    for (int m = 0; m < L; ++m) {
      const short4 o = offs[b + m];
      const int tx = x + o.x, ty = y + o.y, tz = z + o.z;
      if (tx < 0 || tx >= n0 || ty < 0 || ty >= n1 || tz < 0 || tz >= n2) break;
      atomicAdd(dose + ((long long)tx * n1 + ty) * n2 + tz, Tv * __int_as_float(taps[b + m].w));
    }
  }
}

// Radiological cone distance (an extension, CH_OPT_RADIOLOGICAL_DISTANCE):
// the same walks as scatter_kernel, but the kernel is read at the
// density-scaled path length from the source voxel centre,
//   r_m = sum_{k <= m} rho(v_k) * (t_k - t_{k-1}),   t_{-1} = 0,
// accumulated in float32 in walk order like the radiological depth of the
// TERMA pass (conehead/conehead.py:209-254).  With rho = 1 this is the
// geometric walk tap for tap.  Densities are read with the x/y convention
// of the prologue (swap_xy).  Each unique walk carries its multiplicity.
__global__ void __launch_bounds__(128) scatter_radiological_kernel(
    const float* __restrict__ T, const float* __restrict__ rho, int n0, int n1, int n2, int zp, int swap_xy,
    int n_dirs, const int* __restrict__ tap_base, const int* __restrict__ tap_len, const short4* __restrict__ offs,
    const float* __restrict__ tvals, const int* __restrict__ walk_row, const int* __restrict__ walk_mult,
    const double* __restrict__ K, int n_r, float* __restrict__ dose) {
  const long long N = (long long)n0 * n1 * n2;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N) return;
  const int z = (int)(v % n2);
  const long long r = v / n2;
  const int y = (int)(r % n1), x = (int)(r / n1);
  const float Tv = T[((long long)x * n1 + y) * zp + z];
  if (Tv == 0.0f) return;
  for (int u = 0; u < n_dirs; ++u) {
    const int b = tap_base[u], L = tap_len[u];
    const double* Kj = K + (size_t)walk_row[u] * n_r;
    const float mult = (float)walk_mult[u];
    float rad = 0.0f, tprev = 0.0f;
    int prev = -1;
    for (int m = 0; m < L; ++m) {
      const short4 o = offs[b + m];
      const int tx = x + o.x, ty = y + o.y, tz = z + o.z;
      if (tx < 0 || tx >= n0 || ty < 0 || ty >= n1 || tz < 0 || tz >= n2) break;
      const long long ri = swap_xy ? ((long long)ty * n0 + tx) * n2 + tz : ((long long)tx * n1 + ty) * n2 + tz;
      const float t = tvals[b + m];
      rad = fadd(rad, fmul(__ldg(rho + ri), fsub(t, tprev)));
      tprev = t;
      const int ki = kernel_index(rad);
      if (prev == 5995 && ki == 5995) break;
      const double dk = prev < 0 ? Kj[ki] : dsub(Kj[ki], Kj[prev]);
      prev = ki;
      atomicAdd(dose + ((long long)tx * n1 + ty) * n2 + tz, Tv * __fmul_rn(d2f(dk), mult));
    }
  }
}

void launch_scatter_radiological(const float* T, const float* rho, const int* n, int zp, int swap_xy, int n_dirs,
                                 const int* tap_base, const int* tap_len, const short4* offs, const float* tvals,
                                 const int* walk_row, const int* walk_mult, const double* K, int n_r, float* dose,
                                 cudaStream_t st) {
  const long long N = (long long)n[0] * n[1] * n[2];
  scatter_radiological_kernel<<<(unsigned)((N + 127) / 128), 128, 0, st>>>(
      T, rho, n[0], n[1], n[2], zp, swap_xy, n_dirs, tap_base, tap_len, offs, tvals, walk_row, walk_mult, K, n_r,
      dose);
}

void launch_scatter(const float* T, const int* n, int zp, int n_dirs, const int* tap_base, const int* tap_len,
                    const short4* offs, const int4* taps, float* dose, cudaStream_t st) {
  const long long N = (long long)n[0] * n[1] * n[2];
  scatter_kernel<<<(unsigned)((N + 127) / 128), 128, 0, st>>>(T, n[0], n[1], n[2], zp, n_dirs, tap_base, tap_len,
                                                              offs, taps, dose);
}

}  // namespace ch
