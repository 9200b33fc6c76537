// Collapsed-cone stage as an atomic-free stencil gather (replaces the
// per-voxel scatter of conehead/conehead.py:385-488).
//
//   dose(v) = sum_u sum_m T(v - O_u[m]) * w_u[m]
//
// u runs over the deduplicated cone directions, w_u = multiplicity * dK_u.
// Work is split into units = (beam, 16^3 output tile, group of 16
// directions).  range_kernel first bounds, for every (tile, direction), the
// taps m whose sources can hold TERMA: the source box of the tile must meet
// the TERMA bounding box (exact, per axis, on the monotone offsets) and the
// beam frustum widened by half a voxel plus the tile (conservative, through
// the continuous ray: |O_k[m] - t_m d_k / s_k| <= 1/2).  Every skipped tap
// therefore reads only zero TERMA, so the result is exact.
//
// cone_gather_kernel is persistent and warp specialised:
//   * warp 8 (producer) claims units from a global counter, walks each
//     direction's tap range chunk by chunk (chunks are cut on the host so
//     their sources fit one of three window shapes in a 108 KiB slot: P z x
//     rows y x ex x floats with (P, rows) = (24, 32), (40, 24), (56, 24)),
//     and fills the window with ONE TMA box per chunk
//     (cp.async.bulk.tensor.3d through the tensor map of that shape and x
//     extent, out-of-grid reads zero-filled) plus a bulk copy of the chunk's
//     taps into a two-slot mbarrier pipeline;
//   * warps 0-7 (consumers): lanes cover 16 z x 2 y rows of the 16^3 tile and
//     a thread holds the 16 x outputs of its (y, z) column in registers;
//     every tap costs 16 shared-memory loads + FMAs per thread, with the next
//     tap's offsets and weight prefetched; on the unit's last chunk the
//     accumulators are added to the dose with red.global.add.f32.
// Every mbarrier wait is bounded; on expiry the kernel records
// FLAG_TIMEOUT, lets the producer's copies in flight land (a wait bounded by
// MBAR_LIMIT) and returns.  The pipeline waits take their bound from the
// launch (ConeDirs::wait_limit, MBAR_LIMIT unless the plan sets another).

#include <cuda.h>

#include "ch_internal.cuh"

namespace ch {

constexpr int DESC_LAST = 1, DESC_DONE = 2;

// one chunk as the producer hands it to the consumers: runs a..b of walk u
// (walk-local; tb = the walk's first run), its window origin and shape
struct __align__(16) ChunkDesc {
  int u, a, b;
  int x0w, y0w, z0w;
  int tx0, ty0, tz0;
  int beam, flags, ex;
  int axis, var, tb, pad;
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
// `limit` try_wait iterations at most; false when the wait gave up
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  for (long long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// 1-D bulk copy global -> shared (both 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"((unsigned long long)src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
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
  const int tx = tile / (R.ntile[1] * R.ntile[2]);
  const int ty = (tile / R.ntile[2]) % R.ntile[1];
  const int tz = tile % R.ntile[2];
  const int vlo[3] = {tx * TX, ty * TY, tz * TZ};
  const int vhi[3] = {min(vlo[0] + TX, R.n[0]) - 1, min(vlo[1] + TY, R.n[1]) - 1, min(vlo[2] + TZ, R.n[2]) - 1};
  bool wanted = lo0 <= hi0;
  if (R.out_aabb && wanted) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
      wanted = wanted && vhi[k] >= R.out_aabb[2 * k] && vlo[k] <= R.out_aabb[2 * k + 1];
  }
  for (int j = 0; j < R.n_out_planes && wanted; ++j) {
    // the planes hold p . (spacing * i) + k0 <= 0 for voxels that can be in
    // the beam; a tile whose minimum is above 0 is wholly outside
    float minv = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float b = R.opa[j][k] * R.spacing[k];
      minv += fminf(b * (float)vlo[k], b * (float)vhi[k]);
    }
    wanted = minv + R.opk0[j] <= 1e-3f;
  }
  if (wanted) {
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
    // beam frustum planes through the continuous ray.  t_m is the parameter
    // where the ray leaves voxel O[m], so the ray point lies on that voxel's
    // closed box: |O_k[m] - t_m d_k / s_k| <= 1/2 per axis, hence the slack of
    // half the plane's L1 weight (plus a float margin)
    for (int j = 0; j < R.n_planes && mlo <= mhi; ++j) {
      float minv = 0.0f, l1 = 0.0f, g = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float b = R.pa[j][k] * R.spacing[k];
        minv += fminf(b * (float)vlo[k], b * (float)vhi[k]);
        l1 += fabsf(b);
        g += R.pa[j][k] * dir[k];
      }
      const float h = minv + R.pk0[j] - 0.5f * l1 - 1e-3f * (l1 + 1.0f);
      auto tkey = [&](int m) { return tv[m]; };
      if (g > 0.0f) {
        mlo = max(mlo, lower_bound(L, h / g, tkey));
      } else if (g < 0.0f) {
        mhi = min(mhi, upper_bound(L, h / g, tkey) - 1);
      } else if (h > 0.0f) {
        mhi = -1;
      }
    }
    if (mlo <= mhi) {
      // runs holding the first and last tap (whole runs are applied: their
      // other taps read zero TERMA)
      const int rb = D.run_base[u];
      const int rlo = (D.tap_run[base + mlo] >> 3) - rb, rhi = (D.tap_run[base + mhi] >> 3) - rb;
      out = (uint32_t)rlo | ((uint32_t)rhi << 16);
      // chunks holding them
      const int* cs = D.chunk_start + D.chunk_base[u];
      const int nc = D.n_chunks[u];
      auto ckey = [&](int c) { return (float)cs[c]; };
      const int c_first = upper_bound(nc, (float)rlo, ckey) - 1;
      const int c_last = upper_bound(nc, (float)rhi, ckey) - 1;
      R.cranges[(long long)tile * D.n_dirs + u] = (uint32_t)c_first | ((uint32_t)c_last << 16);
    }
  }
  R.ranges[(long long)tile * D.n_dirs + u] = out;
}

// --------------------------------------------------------- gather pass --
__device__ __forceinline__ void producer(const ConeBeam* __restrict__ beams, int n_beams, const ConeDirs& D,
                                         int total_units, int* unit_counter, unsigned long long* updates,
                                         int* flags, float* win, int4* slot_runs, ChunkDesc* desc,
                                         uint64_t* full, uint64_t* empty) {
  const int lane = threadIdx.x & 31;
  // test hook: no window is issued, so every consumer's wait for one expires
  if (D.withhold == CH_WITHHOLD_WINDOWS) return;
  const int n_groups = (D.n_dirs + D.group - 1) / D.group;
  int k = 0;
  bool ok = true;
  ChunkDesc pend;
  bool have = false;
  auto emit = [&](const ChunkDesc& d) -> bool {
    const int s = k % N_SLOTS;
    const uint32_t ph = (uint32_t)(k / N_SLOTS) & 1u;
    if (!mbar_wait(&empty[s], ph ^ 1u, D.wait_limit)) return false;
    const bool done = (d.flags & DESC_DONE) != 0;
    const uint32_t run_bytes = done ? 0u : (uint32_t)(d.b - d.a + 1) * (uint32_t)(RUN_REC_INT4 * sizeof(int4));
    const uint32_t win_bytes = done ? 0u : (uint32_t)(var_p(d.var) * var_rows(d.var) * d.ex * 4);
    if (lane == 0) {
      desc[s] = d;
      mbar_arrive_expect_tx(&full[s], win_bytes + run_bytes);
      if (!done) {
        // the whole window in one TMA box, the chunk's run records in one bulk copy
        tma_load_3d(win + (size_t)s * WIN_FLOATS, &beams[d.beam].tmap[tmap_index(d.var, d.ex)], &full[s], d.z0w,
                    d.y0w, d.x0w);
        bulk_load(slot_runs + (size_t)s * MAX_CHUNK_RUNS * RUN_REC_INT4, D.runs + (size_t)(d.tb + d.a) * RUN_REC_INT4,
                  run_bytes, &full[s]);
      }
    }
    __syncwarp();
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
    const int tile = D.order == 0 ? lu / n_groups : lu % B.n_tiles;
    const int g = D.order == 0 ? lu % n_groups : lu / B.n_tiles;
    const int tx0 = (tile / (B.ntile[1] * B.ntile[2])) * TX;
    const int ty0 = ((tile / B.ntile[2]) % B.ntile[1]) * TY;
    const int tz0 = (tile % B.ntile[2]) * TZ;
    // the unit's directions, 32 at a time: lanes fetch their ranges in parallel
    const int u0 = g * D.group;
    const int u_end = min(u0 + D.group, D.n_dirs);
    unsigned long long work = 0;
    for (int ub = u0; ub < u_end && ok; ub += 32) {
      // lanes fetch, for their walks in parallel, the run and chunk ranges,
      // the first chunk's record (most ranges lie in one chunk) and the tap
      // count, so the serial loop below rarely waits on global memory
      uint32_t r = RANGE_EMPTY, cr = 0;
      int cb = 0, tb = 0, ax = 0;
      int4 f0 = make_int4(0, 0, 0, 0), f1 = make_int4(0, 0, 0, 0);
      unsigned taps = 0;
      if (ub + lane < u_end) {
        const long long ri = (long long)tile * D.n_dirs + ub + lane;
        r = __ldg(B.ranges + ri);
        if (r != RANGE_EMPTY) {
          cr = __ldg(B.cranges + ri);
          cb = __ldg(D.chunk_base + ub + lane);
          tb = __ldg(D.run_base + ub + lane);
          ax = __ldg(D.axis + ub + lane);
          const int cf = cb + (int)(cr & 0xffffu);
          f0 = __ldg(D.chunk_rec + 2 * cf);
          f1 = __ldg(D.chunk_rec + 2 * cf + 1);
          // runs rlo..rhi hold these taps
          taps = (unsigned)(__ldg(D.run_tap + tb + (int)(r >> 16) + 1) - __ldg(D.run_tap + tb + (int)(r & 0xffffu)));
        }
      }
      work += __reduce_add_sync(0xffffffffu, taps);
      unsigned act = __ballot_sync(0xffffffffu, r != RANGE_EMPTY);
      while (act && ok) {
        const int j = __ffs(act) - 1;
        act &= act - 1;
        const uint32_t rj = __shfl_sync(0xffffffffu, r, j), crj = __shfl_sync(0xffffffffu, cr, j);
        const int cbj = __shfl_sync(0xffffffffu, cb, j), tbj = __shfl_sync(0xffffffffu, tb, j);
        const int axj = __shfl_sync(0xffffffffu, ax, j);
        const int rlo = (int)(rj & 0xffffu), rhi = (int)(rj >> 16);
        const int c_first = (int)(crj & 0xffffu), c_last = (int)(crj >> 16);
        // one chunk {first run, last run, variant, spans}, {max O} -> descriptor
        auto add_chunk = [&](int4 r0, int4 r1) {
          ChunkDesc d;
          d.u = ub + j;
          d.a = max(r0.x, rlo);
          d.b = min(r0.y, rhi);
          // window of the whole chunk (covers the clipped runs too)
          d.x0w = tx0 - r1.x;
          d.y0w = ty0 - r1.y;
          d.z0w = (tz0 - r1.z) & ~3;
          d.tx0 = tx0;
          d.ty0 = ty0;
          d.tz0 = tz0;
          d.beam = bi;
          d.flags = 0;
          d.ex = TX + (r0.w & 0xffff);
          d.axis = axj;
          d.var = r0.z;
          d.tb = tbj;
          d.pad = 0;
          if (have) {
            // the consumers change their output layout with the run axis:
            // they flush the sums of the walks before the change
            if (pend.axis != d.axis) pend.flags |= DESC_LAST;
            ok = emit(pend);
          }
          pend = d;
          have = true;
        };
        add_chunk(make_int4(__shfl_sync(0xffffffffu, f0.x, j), __shfl_sync(0xffffffffu, f0.y, j),
                            __shfl_sync(0xffffffffu, f0.z, j), __shfl_sync(0xffffffffu, f0.w, j)),
                  make_int4(__shfl_sync(0xffffffffu, f1.x, j), __shfl_sync(0xffffffffu, f1.y, j),
                            __shfl_sync(0xffffffffu, f1.z, j), 0));
        for (int c0 = c_first + 1; c0 <= c_last && ok; c0 += 32) {
          // lanes fetch up to 32 further chunk records at once
          int4 r0 = make_int4(0, 0, 0, 0), r1 = make_int4(0, 0, 0, 0);
          if (c0 + lane <= c_last) {
            r0 = __ldg(D.chunk_rec + 2 * (cbj + c0 + lane));
            r1 = __ldg(D.chunk_rec + 2 * (cbj + c0 + lane) + 1);
          }
          const int nrec = min(32, c_last - c0 + 1);
          for (int q = 0; q < nrec && ok; ++q)
            add_chunk(make_int4(__shfl_sync(0xffffffffu, r0.x, q), __shfl_sync(0xffffffffu, r0.y, q),
                                __shfl_sync(0xffffffffu, r0.z, q), __shfl_sync(0xffffffffu, r0.w, q)),
                      make_int4(__shfl_sync(0xffffffffu, r1.x, q), __shfl_sync(0xffffffffu, r1.y, q),
                                __shfl_sync(0xffffffffu, r1.z, q), 0));
        }
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
    // (always the full MBAR_LIMIT: a copy in flight completes in
    // microseconds, whatever limit the pipeline waits were given)
    for (int j = max(0, k - N_SLOTS); j < k; ++j)
      mbar_wait(&full[j % N_SLOTS], (uint32_t)(j / N_SLOTS) & 1u, MBAR_LIMIT);
  }
}

// One run of N taps for one thread: the OUT_PER_THREAD - 1 + N window values
// of its line along the run axis (stride S floats), then OUT_PER_THREAD * N
// FMAs from registers.
template <int S, int N>
__device__ __forceinline__ void apply_run(const float* src, const float (&wt)[RUN_MAX], float* acc) {
  float line[OUT_PER_THREAD - 1 + N];
#pragma unroll
  for (int k = 0; k < OUT_PER_THREAD - 1 + N; ++k) line[k] = src[k * S];
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int i = 0; i < OUT_PER_THREAD; ++i) acc[i] = fmaf(wt[j], line[i + j], acc[i]);
}

// One chunk of runs for one thread: 16 outputs along run axis AX in window
// variant V (pitches fixed at compile time).  The records sit in shared
// memory next to the window; the next run's first half is read a run ahead,
// the second half (weights 2 and 3) only for runs of more than 2 taps.
template <int V, int AX>
__device__ __forceinline__ void consume_chunk(const float* w, const int4* rp, int n_runs, int base0, float* acc) {
  constexpr int S = AX == 0 ? var_rows(V) * var_p(V) : var_p(V);
  int4 next = rp[0];
  for (int r = 0; r < n_runs; ++r) {
    const int4 h = next;
    if (r + 1 < n_runs) next = rp[RUN_REC_INT4 * (r + 1)];
    const float* src = w + (base0 - h.x);
    float wt[RUN_MAX] = {__int_as_float(h.z), __int_as_float(h.w), 0.0f, 0.0f};
    if (h.y <= 2) {
      if (h.y == 1) apply_run<S, 1>(src, wt, acc);
      else apply_run<S, 2>(src, wt, acc);
    } else {
      const int4 t = rp[RUN_REC_INT4 * r + 1];
      wt[2] = __int_as_float(t.x);
      wt[3] = __int_as_float(t.y);
      if (h.y == 3) apply_run<S, 3>(src, wt, acc);
      else apply_run<S, 4>(src, wt, acc);
    }
  }
}

__device__ __forceinline__ void consumer(const ConeBeam* __restrict__ beams, const ConeDirs& D, int* flags,
                                         const float* win, const int4* slot_runs, const ChunkDesc* desc,
                                         uint64_t* full, uint64_t* empty) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wl = warp % (TY / 2);                                  // line pair of this warp
  const int first = (warp / (TY / 2)) * OUT_PER_THREAD;            // first output along the run axis
  const int zl = lane & 15;                                        // z within the tile
  const int row = (wl & 1) + 4 * (wl >> 1) + 2 * (lane >> 4);      // run axis x: this thread's y row
  const int slice = 2 * wl + (lane >> 4);                          // run axis y: this thread's x slice
  float acc[OUT_PER_THREAD];                                       // outputs first.. along the run axis
#pragma unroll
  for (int i = 0; i < OUT_PER_THREAD; ++i) acc[i] = 0.0f;
  for (int k = 0;; ++k) {
    const int s = k % N_SLOTS;
    if (!mbar_wait(&full[s], (uint32_t)(k / N_SLOTS) & 1u, D.wait_limit)) {
      if (lane == 0) atomicOr(flags, FLAG_TIMEOUT);
      return;
    }
    const ChunkDesc d = desc[s];
    if (d.flags & DESC_DONE) break;
    const float* w = win + (size_t)s * WIN_FLOATS;
    const int4* rp = slot_runs + (size_t)s * MAX_CHUNK_RUNS * RUN_REC_INT4;
    const int nr = d.b - d.a + 1;
    const int rows = var_rows(d.var), P = var_p(d.var);
    const int xl = d.axis == 0 ? first : slice, yl = d.axis == 0 ? row : first;
    const int base0 = ((d.tx0 + xl - d.x0w) * rows + (d.ty0 + yl - d.y0w)) * P + (d.tz0 + zl - d.z0w);
    if (d.axis == 0) {
      if (d.var == 0) consume_chunk<0, 0>(w, rp, nr, base0, acc);
      else if (d.var == 1) consume_chunk<1, 0>(w, rp, nr, base0, acc);
      else consume_chunk<2, 0>(w, rp, nr, base0, acc);
    } else {
      if (d.var == 0) consume_chunk<0, 1>(w, rp, nr, base0, acc);
      else if (d.var == 1) consume_chunk<1, 1>(w, rp, nr, base0, acc);
      else consume_chunk<2, 1>(w, rp, nr, base0, acc);
    }
    __syncwarp();
    // (test hook: a slot is never freed, so the producer's wait for one
    // expires with two windows in flight)
    if (lane == 0 && D.withhold != CH_WITHHOLD_SLOTS) mbar_arrive(&empty[s]);
    if (d.flags & DESC_LAST) {
      const ConeBeam& B = beams[d.beam];
      const int x = d.tx0 + xl, y = d.ty0 + yl, z = d.tz0 + zl;
      const long long xs = (long long)B.n[1] * B.n[2];
      const long long step = d.axis == 0 ? xs : (long long)B.n[2];
      const int lim = d.axis == 0 ? B.n[0] - x : B.n[1] - y;        // outputs inside the grid
      if (x < B.n[0] && y < B.n[1] && z < B.n[2]) {
        float* out = B.dose + ((long long)x * B.n[1] + y) * B.n[2] + z;
#pragma unroll
        for (int i = 0; i < OUT_PER_THREAD; ++i)
          if (i < lim) atomicAdd(out + i * step, acc[i]);
      }
#pragma unroll
      for (int i = 0; i < OUT_PER_THREAD; ++i) acc[i] = 0.0f;
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
  int4* slot_runs = reinterpret_cast<int4*>(sm + (size_t)N_SLOTS * WIN_FLOATS * 4);
  ChunkDesc* desc = reinterpret_cast<ChunkDesc*>(slot_runs + N_SLOTS * MAX_CHUNK_RUNS * RUN_REC_INT4);
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
    producer(beams, n_beams, D, total_units, unit_counter, updates, flags, win, slot_runs, desc, full, empty);
  else
    consumer(beams, D, flags, win, slot_runs, desc, full, empty);
}

size_t cone_smem_bytes() {
  return 1024 + (size_t)N_SLOTS * WIN_FLOATS * 4 + (size_t)N_SLOTS * MAX_CHUNK_RUNS * RUN_REC_INT4 * sizeof(int4) +
         N_SLOTS * sizeof(ChunkDesc) + 2 * N_SLOTS * sizeof(uint64_t);
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
