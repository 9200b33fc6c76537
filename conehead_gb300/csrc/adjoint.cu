// Small kernels of the cone operator and the beamlet adjoint.
//
//   nonzero_box_kernel   bounding box of the nonzero voxels of a volume
//                        (the input box the tap ranges are cut against)
//   beamlet_fill_kernel  block-map crop of a beamlet grid: every map cell of
//                        beamlet (i, j) holds its weight
//   to_float_kernel      float64 beamlet gradient -> float32
//
// The transposed blocking itself lives with the forward blocking in
// prologue.cu, because it must classify sub-samples exactly as the forward
// does.

#include <climits>

#include "ch_internal.cuh"

namespace ch {
namespace {

__global__ void __launch_bounds__(256) nonzero_box_kernel(const float* __restrict__ x, int n0, int n1, int n2,
                                                          int* __restrict__ box) {
  // box: lo/hi pairs per axis, initialised to INT_MAX / INT_MIN
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
  const long long N = (long long)n0 * n1 * n2;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < N;
       v += (long long)gridDim.x * blockDim.x) {
    if (__ldg(x + v) != 0.0f) {
      const int z = (int)(v % n2);
      const long long r = v / n2;
      const int y = (int)(r % n1), xx = (int)(r / n1);
      const int c[3] = {xx, y, z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        lo[k] = min(lo[k], c[k]);
        hi[k] = max(hi[k], c[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0 && lo[0] != INT_MAX) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      atomicMin(box + 2 * k, lo[k]);
      atomicMax(box + 2 * k + 1, hi[k]);
    }
  }
}

__global__ void __launch_bounds__(256) beamlet_fill_kernel(const float* __restrict__ w, BeamletDev bl,
                                                           float* __restrict__ crop) {
  const int rows = bl.rows * bl.cell_rows, cols = bl.cols * bl.cell_cols;
  const long long n = (long long)rows * cols;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    crop[i] = __ldg(w + (r / bl.cell_rows) * bl.cols + c / bl.cell_cols);
  }
}

__global__ void to_float_kernel(const double* __restrict__ in, float* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

}  // namespace

void launch_nonzero_box(const float* x, int n0, int n1, int n2, int* box, cudaStream_t st) {
  const long long N = (long long)n0 * n1 * n2;
  long long blocks = (N + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  nonzero_box_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, st>>>(x, n0, n1, n2, box);
}

void launch_beamlet_fill(const float* w, const BeamletDev& bl, float* crop, cudaStream_t st) {
  const long long n = (long long)bl.rows * bl.cell_rows * bl.cols * bl.cell_cols;
  long long blocks = (n + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  beamlet_fill_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, st>>>(w, bl, crop);
}

void launch_to_float(const double* in, float* out, int n, cudaStream_t st) {
  to_float_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, out, n);
}

}  // namespace ch
