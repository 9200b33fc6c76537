// Jaw + MLCX block map rasterised on the device (conehead/block.py:87-215).
//
// The reference builds a float32 map of |leaf span| x 4000 cells (0.1 mm) on
// the host from the plan's leaf positions and copies it to the GPU on every
// dose call (conehead/conehead.py:555).  Here the host passes the leaf table
// (a few KB, by value as the kernel parameter) and the kernel writes only the
// window the dose path reads -- the jaw opening -- straight into the crop
// buffer that ch_beam.block points at.
//
// One CTA row per map row: the leaf pair covering the row is found once per
// CTA (binary search over row0[], a uniform constant-bank read), then the
// threads stream the row's columns with coalesced float stores.  The values
// are those of the reference's arithmetic: the leaf ramp is multiplied in
// float64 and rounded to float32 (numpy's in-place multiply of a float32
// array by float64 linspace values), then subtracted from 1 in float32.

#include "ch_internal.cuh"

namespace ch {
namespace {

// tongue-and-groove profile of row i of a leaf w rows high: the writes
// rows 0, 1, 2 = 0.2, 0.5, 0.75 then rows w-1, w-2, w-3 = 0.2, 0.5, 0.75,
// later writes winning where they meet (conehead/block.py:148-155)
__device__ __forceinline__ float leaf_profile(int i, int w) {
  float v = 1.0f;
  if (i == 0) v = 0.2f;
  if (i == 1) v = 0.5f;
  if (i == 2) v = 0.75f;
  if (i == w - 1) v = 0.2f;
  if (i == w - 2) v = 0.5f;
  if (i == w - 3) v = 0.75f;
  return v;
}

__device__ __forceinline__ float leaf_value(float profile, double ramp) {
  return __fsub_rn(1.0f, __double2float_rn(__dmul_rn((double)profile, ramp)));
}

__global__ void __launch_bounds__(256) mlc_raster_kernel(const ch_mlc m, float* __restrict__ out, int rows,
                                                         int cols, int r0, int c0) {
  const int rr = blockIdx.y;
  const int r = r0 + rr;
  const bool row_open = r >= m.open_r0 && r < m.open_r1;
  // leaf pair of this row: the last n with row0[n] <= r, if r lies inside it
  int pair = -1;
  if (row_open) {
    int lo = 0, hi = m.n_pairs - 1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      if (m.row0[mid] <= r) {
        pair = mid;
        lo = mid + 1;
      } else {
        hi = mid - 1;
      }
    }
    if (pair >= 0 && r >= m.row0[pair] + m.rows[pair]) pair = -1;
  }
  int i = 0, w = 0, a_end = 0, b_start = 0;
  if (pair >= 0) {
    i = r - m.row0[pair];
    w = m.rows[pair];
    a_end = m.a_end[pair];
    b_start = m.b_start[pair];
  }
  float* row = out + (size_t)rr * cols;
  for (int cc = blockIdx.x * blockDim.x + threadIdx.x; cc < cols; cc += gridDim.x * blockDim.x) {
    const int c = c0 + cc;
    float v = 0.0f;
    if (row_open && c >= m.open_c0 && c < m.open_c1) {
      v = 1.0f;
      if (pair >= 0) {
        if (c >= b_start && c < m.map_cols - 1) {
          // bank B: bank A's leaf turned by 180 degrees, tip at its first columns
          const int j = c - b_start;
          v = leaf_value(leaf_profile(w - 1 - i, w), j < CH_MLC_TIP_CELLS ? m.tip[CH_MLC_TIP_CELLS - 1 - j] : 1.0);
        } else if (c < a_end) {
          const int k = c - (a_end - CH_MLC_TIP_CELLS);
          v = leaf_value(leaf_profile(i, w), k >= 0 ? m.tip[k] : 1.0);
        }
      }
    }
    row[cc] = v;
  }
}

}  // namespace

void launch_mlc_raster(const ch_mlc& m, float* out, int rows, int cols, int r0, int c0, cudaStream_t st) {
  const int threads = 256;
  const int gx = (cols + threads - 1) / threads;
  mlc_raster_kernel<<<dim3(gx < 16 ? gx : 16, rows), threads, 0, st>>>(m, out, rows, cols, r0, c0);
}

}  // namespace ch
