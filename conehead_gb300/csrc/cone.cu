// Collapsed-cone stage as an atomic-free stencil gather (replaces the
// per-voxel scatter of conehead/conehead.py:385-488).
//
//   dose(v) = sum_u sum_m T(v - O_u[m]) * w_u[m]
//
// u runs over the deduplicated cone directions, w_u = multiplicity * dK_u.
// Work is split into units = (beam, 32x16x8 output tile, group of 16
// directions).  range_kernel first bounds, for every (tile, direction), the
// taps m whose sources can hold TERMA: the source box of the tile must meet
// the TERMA bounding box (exact, per axis, on the monotone offsets) and the
// beam frustum widened by half a voxel plus the tile (conservative, through
// the continuous ray: |O_k[m] - t_m d_k / s_k| <= 1).  Every skipped tap
// therefore reads only zero TERMA, so the result is exact.
//
// cone_gather_kernel is persistent and warp specialised:
//   * warp 8 (producer) claims units from a global counter, splits each
//     direction's tap range into chunks whose sources fit a 48x24x16-float
//     shared-memory window, and fills the window with TMA tile loads
//     (cp.async.bulk.tensor.3d, 48x8x1 boxes, out-of-grid reads zero-filled)
//     into a two-slot mbarrier pipeline;
//   * warps 0-7 (consumers) each own one x-slice of the tile; a thread holds
//     16 outputs (its lane's z, 16 consecutive y) in registers and for every
//     tap does 16 shared-memory loads + FMAs; on the unit's last chunk the
//     accumulators are added to the dose with red.global.add.f32.
// Every mbarrier wait is bounded; on expiry the kernel records
// FLAG_TIMEOUT and returns.

#include <cuda.h>

#include "ch_internal.cuh"

namespace ch {

constexpr long long MBAR_LIMIT = 1ll << 22;
constexpr int DESC_LAST = 1, DESC_DONE = 2;

struct __align__(16) ChunkDesc {
  int u, a, b;
  int x0w, y0w, z0w;
  int tx0, ty0, tz0;
  int beam, flags, ex;
  int nyb, pad0, pad1, pad2;
};

// ------------------------------------------------------------- PTX glue --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < MBAR_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"((unsigned long long)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

// ----------------------------------------------------------- range pass --
// first m in [0, L) with key(m) >= x, for non-decreasing key
template <typename Key>
__device__ __forceinline__ int lower_bound(int L, float x, Key key) {
  int lo = 0, hi = L;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (key(mid) < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// first m in [0, L) with key(m) > x, for non-decreasing key
template <typename Key>
__device__ __forceinline__ int upper_bound(int L, float x, Key key) {
  int lo = 0, hi = L;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (key(mid) <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void range_kernel(const RangeBeam* __restrict__ rbs, ConeDirs D) {
  const RangeBeam& R = rbs[blockIdx.y];
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long long)R.n_tiles * D.n_dirs) return;
  const int tile = (int)(id / D.n_dirs), u = (int)(id % D.n_dirs);
  const int lo0 = R.aabb[0], hi0 = R.aabb[1], lo1 = R.aabb[2], hi1 = R.aabb[3], lo2 = R.aabb[4], hi2 = R.aabb[5];
  uint32_t out = RANGE_EMPTY;
  if (lo0 <= hi0) {
    const int tx = tile / (R.ntile[1] * R.ntile[2]);
    const int ty = (tile / R.ntile[2]) % R.ntile[1];
    const int tz = tile % R.ntile[2];
    const int vlo[3] = {tx * TX, ty * TY, tz * TZ};
    const int vhi[3] = {min(vlo[0] + TX, R.n[0]) - 1, min(vlo[1] + TY, R.n[1]) - 1, min(vlo[2] + TZ, R.n[2]) - 1};
    const int blo[3] = {lo0, lo1, lo2}, bhi[3] = {hi0, hi1, hi2};
    const int base = D.tap_base[u], L = D.tap_len[u];
    const short4* O = D.offs + base;
    const float* tv = D.tvals + base;
    const float* dir = D.dirs + 3 * u;
    int mlo = 0, mhi = L - 1;
    // TERMA box: vlo - bhi <= O_k[m] <= vhi - blo, O_k monotone
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float A = (float)(vlo[k] - bhi[k]), B = (float)(vhi[k] - blo[k]);
      const float s = dir[k] < 0.0f ? -1.0f : 1.0f;
      auto key = [&](int m) {
        const short4 o = O[m];
        const int c = k == 0 ? o.x : (k == 1 ? o.y : o.z);
        return s * (float)c;
      };
      const float klo = s > 0 ? A : -B, khi = s > 0 ? B : -A;
      mlo = max(mlo, lower_bound(L, klo, key));
      mhi = min(mhi, lower_bound(L, khi + 0.5f, key) - 1);
    }
    // beam frustum planes through the continuous ray
    for (int j = 0; j < R.n_planes && mlo <= mhi; ++j) {
      float minv = 0.0f, l1 = 0.0f, g = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float b = R.pa[j][k] * R.spacing[k];
        minv += fminf(b * (float)vlo[k], b * (float)vhi[k]);
        l1 += fabsf(b);
        g += R.pa[j][k] * dir[k];
      }
      const float h = minv + R.pk0[j] - l1 - 1e-3f * (l1 + 1.0f);
      auto tkey = [&](int m) { return tv[m]; };
      if (g > 0.0f) {
        mlo = max(mlo, lower_bound(L, h / g, tkey));
      } else if (g < 0.0f) {
        mhi = min(mhi, upper_bound(L, h / g, tkey) - 1);
      } else if (h > 0.0f) {
        mhi = -1;
      }
    }
    if (mlo <= mhi) out = (uint32_t)mlo | ((uint32_t)mhi << 16);
  }
  R.ranges[(long long)tile * D.n_dirs + u] = out;
}

// --------------------------------------------------------- gather pass --
__device__ __forceinline__ void producer(const ConeBeam* __restrict__ beams, int n_beams, const ConeDirs& D,
                                         int total_units, int* unit_counter, unsigned long long* updates,
                                         int* flags, float* win, ChunkDesc* desc, uint64_t* full,
                                         uint64_t* empty) {
  const int lane = threadIdx.x & 31;
  const int n_groups = (D.n_dirs + DIR_GROUP - 1) / DIR_GROUP;
  int k = 0;
  bool ok = true;
  ChunkDesc pend;
  bool have = false;
  auto emit = [&](const ChunkDesc& d) -> bool {
    const int s = k % N_SLOTS;
    const uint32_t ph = (uint32_t)(k / N_SLOTS) & 1u;
    if (!mbar_wait(&empty[s], ph ^ 1u)) return false;
    const bool done = (d.flags & DESC_DONE) != 0;
    const uint32_t bytes = done ? 0u : (uint32_t)(d.ex * d.nyb * BOX_BYTES);
    if (lane == 0) {
      desc[s] = d;
      mbar_arrive_expect_tx(&full[s], bytes);
    }
    __syncwarp();
    if (!done) {
      const CUtensorMap* map = &beams[d.beam].tmap;
      float* slot = win + (size_t)s * WIN_FLOATS;
      for (int q = lane; q < d.ex * d.nyb; q += 32) {
        const int xs = q / d.nyb, yb = q % d.nyb;
        tma_load_3d(slot + (xs * WY + yb * BOX_Y) * WZ, map, &full[s], d.z0w, d.y0w + yb * BOX_Y, d.x0w + xs);
      }
    }
    ++k;
    return true;
  };

  while (ok) {
    int unit = 0;
    if (lane == 0) unit = atomicAdd(unit_counter, 1);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= total_units) break;
    int bi = 0;
    while (bi + 1 < n_beams && beams[bi + 1].unit_begin <= unit) ++bi;
    const ConeBeam& B = beams[bi];
    const int lu = unit - B.unit_begin;
    const int tile = lu / n_groups, g = lu % n_groups;
    const int tx0 = (tile / (B.ntile[1] * B.ntile[2])) * TX;
    const int ty0 = ((tile / B.ntile[2]) % B.ntile[1]) * TY;
    const int tz0 = (tile % B.ntile[2]) * TZ;
    const int u_end = min(D.n_dirs, (g + 1) * DIR_GROUP);
    unsigned long long work = 0;
    for (int u = g * DIR_GROUP; u < u_end && ok; ++u) {
      const uint32_t r = __ldg(B.ranges + (long long)tile * D.n_dirs + u);
      if (r == RANGE_EMPTY) continue;
      const int mlo = (int)(r & 0xffffu), mhi = (int)(r >> 16);
      const int cb = D.chunk_base[u], nc = D.n_chunks[u], tb = D.tap_base[u], L = D.tap_len[u];
      for (int c = 0; c < nc && ok; ++c) {
        const int ca = D.chunk_start[cb + c];
        const int ce = (c + 1 < nc) ? D.chunk_start[cb + c + 1] - 1 : L - 1;
        if (ce < mlo) continue;
        if (ca > mhi) break;
        const int a = max(ca, mlo), b = min(ce, mhi);
        const short4 oa = D.offs[tb + a], ob = D.offs[tb + b];
        ChunkDesc d;
        d.u = u;
        d.a = a;
        d.b = b;
        d.x0w = tx0 - max((int)oa.x, (int)ob.x);
        d.y0w = ty0 - max((int)oa.y, (int)ob.y);
        d.z0w = (tz0 - max((int)oa.z, (int)ob.z)) & ~3;
        d.tx0 = tx0;
        d.ty0 = ty0;
        d.tz0 = tz0;
        d.beam = bi;
        d.flags = 0;
        d.ex = TX + abs((int)ob.x - (int)oa.x);
        d.nyb = (TY + abs((int)ob.y - (int)oa.y) + BOX_Y - 1) / BOX_Y;
        d.pad0 = d.pad1 = d.pad2 = 0;
        work += (unsigned long long)(b - a + 1);
        if (have) ok = emit(pend);
        pend = d;
        have = true;
      }
    }
    if (have && ok) {
      pend.flags = DESC_LAST;
      ok = emit(pend);
      have = false;
    }
    if (lane == 0 && work) atomicAdd(updates, work * (unsigned long long)TILE_VOX);
  }
  if (ok) {
    ChunkDesc d = {};
    d.flags = DESC_DONE;
    ok = emit(d);
  }
  if (!ok) {
    if (lane == 0) atomicOr(flags, FLAG_TIMEOUT);
    // let this CTA's own copies land before its shared memory goes away
    for (int j = max(0, k - N_SLOTS); j < k; ++j) mbar_wait(&full[j % N_SLOTS], (uint32_t)(j / N_SLOTS) & 1u);
  }
}

__device__ __forceinline__ void consumer(const ConeBeam* __restrict__ beams, const ConeDirs& D, int* flags,
                                         const float* win, const ChunkDesc* desc, uint64_t* full,
                                         uint64_t* empty) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[TY];
#pragma unroll
  for (int i = 0; i < TY; ++i) acc[i] = 0.0f;
  for (int k = 0;; ++k) {
    const int s = k % N_SLOTS;
    if (!mbar_wait(&full[s], (uint32_t)(k / N_SLOTS) & 1u)) {
      if (lane == 0) atomicOr(flags, FLAG_TIMEOUT);
      return;
    }
    const ChunkDesc d = desc[s];
    if (d.flags & DESC_DONE) break;
    const float* w = win + (size_t)s * WIN_FLOATS;
    const int base0 = ((d.tx0 + warp - d.x0w) * WY + (d.ty0 - d.y0w)) * WZ + (d.tz0 + lane - d.z0w);
    const int2* tp = D.taps + D.tap_base[d.u];
    for (int m = d.a; m <= d.b; ++m) {
      const int2 tap = __ldg(tp + m);
      const float wt = __int_as_float(tap.y);
      const float* src = w + (base0 - tap.x);
#pragma unroll
      for (int i = 0; i < TY; ++i) acc[i] = fmaf(wt, src[i * WZ], acc[i]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (d.flags & DESC_LAST) {
      const ConeBeam& B = beams[d.beam];
      const int x = d.tx0 + warp, z = d.tz0 + lane;
      if (x < B.n[0] && z < B.n[2]) {
        float* out = B.dose + ((long long)x * B.n[1] + d.ty0) * B.n[2] + z;
#pragma unroll
        for (int i = 0; i < TY; ++i)
          if (d.ty0 + i < B.n[1]) atomicAdd(out + (long long)i * B.n[2], acc[i]);
      }
#pragma unroll
      for (int i = 0; i < TY; ++i) acc[i] = 0.0f;
    }
  }
}

__global__ void __launch_bounds__(CONE_THREADS, 1)
    cone_gather_kernel(const ConeBeam* __restrict__ beams, int n_beams, ConeDirs D, int total_units,
                       int* unit_counter, unsigned long long* updates, int* flags) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-align the window slots
  const uint32_t base = smem_u32(smem_raw);
  unsigned char* sm = smem_raw + ((1024u - (base & 1023u)) & 1023u);
  float* win = reinterpret_cast<float*>(sm);
  ChunkDesc* desc = reinterpret_cast<ChunkDesc*>(sm + (size_t)N_SLOTS * WIN_FLOATS * 4);
  uint64_t* full = reinterpret_cast<uint64_t*>(desc + N_SLOTS);
  uint64_t* empty = full + N_SLOTS;
  if (threadIdx.x == 0) {
    for (int s = 0; s < N_SLOTS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CONE_CONSUMER_WARPS);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if ((threadIdx.x >> 5) == CONE_CONSUMER_WARPS)
    producer(beams, n_beams, D, total_units, unit_counter, updates, flags, win, desc, full, empty);
  else
    consumer(beams, D, flags, win, desc, full, empty);
}

size_t cone_smem_bytes() {
  return 1024 + (size_t)N_SLOTS * WIN_FLOATS * 4 + N_SLOTS * sizeof(ChunkDesc) + 2 * N_SLOTS * sizeof(uint64_t);
}

cudaError_t setup_cone_kernel() {
  return cudaFuncSetAttribute(cone_gather_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)cone_smem_bytes());
}

void launch_range(const RangeBeam* rbs_dev, int n_beams, int max_tiles, const ConeDirs& D, cudaStream_t st) {
  const long long n = (long long)max_tiles * D.n_dirs;
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)n_beams);
  range_kernel<<<grid, 256, 0, st>>>(rbs_dev, D);
}

void launch_gather(const ConeBeam* beams_dev, int n_beams, const ConeDirs& D, int total_units, int n_ctas,
                   int* unit_counter, unsigned long long* updates, int* flags, cudaStream_t st) {
  cone_gather_kernel<<<n_ctas, CONE_THREADS, cone_smem_bytes(), st>>>(beams_dev, n_beams, D, total_units,
                                                                      unit_counter, updates, flags);
}

}  // namespace ch
