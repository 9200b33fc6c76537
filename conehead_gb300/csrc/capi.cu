// Host side of the C ABI declared in include/conehead_gb300.h: plans,
// stencil preparation, scratch management and launch sequencing.
//
// A plan owns the kernel tables, the per-spacing direction stencils and a
// grow-only scratch arena (TERMA volumes, tile ranges, per-beam launch
// records).  Caller buffers (densities, block maps, dose) are never
// allocated or freed here.  Calls are stream ordered and asynchronous;
// device-side failures (bounded waits that expired, rays parallel to the
// blocking plane) are reported by ch_plan_sync / ch_plan_stats.

#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "ch_internal.cuh"

using namespace ch;

namespace {

thread_local std::string g_last_error;

ch_status fail(ch_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

#define CH_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(e_ == cudaErrorMemoryAllocation ? CH_ERR_OOM : CH_ERR_DEVICE,        \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                 \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

}  // namespace

struct StencilSet {
  bool valid = false;
  float spacing[3] = {0, 0, 0};
  int cap[3] = {0, 0, 0};
  int n_dirs = 0;            // unique walks
  int n_raw = 0;             // theta x phi
  size_t total_taps = 0;
  DevBuf tap_base, tap_len, taps, offs, tvals, chunk_base, n_chunks, chunk_start, chunk_rec, dirs;
  DevBuf runs, run_base, tap_run, run_tap, axis;   // run records of the gather (ConeDirs)
  DevBuf raw_dirs;           // float [n_theta*n_phi][3] as the device computed them
  DevBuf walk_row, walk_mult;  // per unique walk: kernel row (cone polar angle) and multiplicity
  std::vector<DevBuf*> bufs() {
    return {&tap_base, &tap_len, &taps, &offs, &tvals, &chunk_base, &n_chunks, &chunk_start, &chunk_rec, &dirs,
            &runs, &run_base, &tap_run, &run_tap, &axis, &raw_dirs, &walk_row, &walk_mult};
  }
  size_t bytes() const {
    size_t b = 0;
    for (DevBuf* d : const_cast<StencilSet*>(this)->bufs()) b += d->bytes;
    return b;
  }
};

struct FrameStencils {
  ConeFrame frame{};
  StencilSet fwd, adj;
  uint64_t last_use = 0;
  ~FrameStencils() {
    for (StencilSet* S : {&fwd, &adj})
      for (DevBuf* b : S->bufs()) b->release();
  }
};

// S^ of one grid shape and stencil set (spectral cone stage)
struct SpecEntry {
  const StencilSet* set = nullptr;
  int n[3] = {0, 0, 0};
  DevBuf shat;               // float2 [Mx][My][Mz]
  uint64_t last_use = 0;
  ~SpecEntry() { shat.release(); }
};

struct ch_plan {
  int device = 0;
  int n_sm = 0;
  ch_tuning tuning{DIR_GROUP, 0, 8, CH_CONE_SPECTRAL};
  int live_batches = 0;      // captured batches reading this plan's stencils
  long long wait_limit = 0;  // gather pipeline waits (try_wait iterations); 0 = MBAR_LIMIT
  int withhold = 0;          // test hook of the expired-wait path (ch_plan_set_wait_limit)
  int reweights = 0;         // spectrum switches served by reweighting the stencils
  std::vector<std::unique_ptr<FrameStencils>> frames;   // beam-frame cone stencils by orientation
  uint64_t use_clock = 0;
  bool have_kernel = false;
  int n_phi = 0, n_r = 0, n_theta = 0;
  DevBuf K, theta, phi;
  std::vector<float> h_theta, h_phi;   // the direction tables the stencils were built from
  StencilSet st;
  StencilSet st_adj;         // the same walks mirrored (offsets and directions negated): the transposed cone
  std::vector<std::unique_ptr<SpecEntry>> spec;   // S^ by grid shape and stencil set
  DevBuf spec_tw;            // FFT twiddles of every period
  // scratch
  DevBuf T, aabb, counters, ranges, cranges, cone_beams, range_beams, list_v, spec_work, pro_beams;
  DevBuf adj_in, adj_out, adj_w;   // cone-operator input (padded), output, beamlet gradient (float64)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t last_stream = nullptr;
  ch_stats stats{};
  bool stats_pending = false;
  bool timed = false;
  // pinned staging of the per-beam launch records, double buffered, so
  // their upload is a true async copy; ev_rec[i] marks when the upload from
  // buffer i has read it
  void* h_rec[2] = {nullptr, nullptr};
  size_t h_rec_bytes[2] = {0, 0};
  cudaEvent_t ev_rec[2] = {nullptr, nullptr};
  bool rec_pending[2] = {false, false};
  int rec_next = 0;
  ~ch_plan() {
    for (int i = 0; i < 2; ++i)
      if (rec_pending[i] && ev_rec[i]) cudaEventSynchronize(ev_rec[i]);
    spec.clear();
    for (DevBuf* b : {&K, &theta, &phi, &T, &aabb, &counters, &ranges, &cranges, &cone_beams, &range_beams, &list_v,
                      &spec_work, &pro_beams, &spec_tw, &adj_in, &adj_out, &adj_w})
      b->release();
    for (StencilSet* S : {&st, &st_adj})
      for (DevBuf* b : S->bufs()) b->release();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (int i = 0; i < 2; ++i) {
      if (ev_rec[i]) cudaEventDestroy(ev_rec[i]);
      if (h_rec[i]) cudaFreeHost(h_rec[i]);
    }
  }
};

namespace {

// ------------------------------------------------------------ stencils --
ch_status assemble_stencils(ch_plan* P, StencilSet& S, int sign, int n_raw, int max_len,
                            const std::vector<short4>& h_off_in, const std::vector<float>& h_t,
                            const std::vector<float>& h_dk, const std::vector<int>& h_len,
                            const std::vector<float>& h_dir_in, const float* spacing, const int* cap,
                            cudaStream_t s);

// drop the S^ built from stencil set S (it is being rebuilt or freed)
void spec_forget(ch_plan* P, const StencilSet* S) {
  P->spec.erase(std::remove_if(P->spec.begin(), P->spec.end(),
                               [S](const std::unique_ptr<SpecEntry>& e) { return e->set == S; }),
                P->spec.end());
}

ch_status build_stencils(ch_plan* P, const float* spacing, const int* cap, cudaStream_t s,
                         const ConeFrame& frame, StencilSet& S, StencilSet& S_adj) {
  spec_forget(P, &S);
  spec_forget(P, &S_adj);
  const int n_raw = P->n_theta * P->n_phi;
  const int max_len = cap[0] + cap[1] + cap[2] + 2;
  DevBuf off, tv, dk, len;
  CH_CUDA(off.ensure((size_t)n_raw * max_len * sizeof(short4)));
  CH_CUDA(tv.ensure((size_t)n_raw * max_len * sizeof(float)));
  CH_CUDA(dk.ensure((size_t)n_raw * max_len * sizeof(float)));
  CH_CUDA(len.ensure((size_t)n_raw * sizeof(int)));
  CH_CUDA(S.raw_dirs.ensure((size_t)n_raw * 3 * sizeof(float)));
  launch_stencil(P->theta.as<float>(), P->n_theta, P->phi.as<float>(), P->n_phi, P->K.as<double>(), P->n_r,
                 spacing, cap, max_len, off.as<short4>(), tv.as<float>(), dk.as<float>(), len.as<int>(),
                 S.raw_dirs.as<float>(), frame, s);
  CH_CUDA(cudaGetLastError());
  std::vector<short4> h_off((size_t)n_raw * max_len);
  std::vector<float> h_t((size_t)n_raw * max_len), h_dk((size_t)n_raw * max_len), h_dir((size_t)n_raw * 3);
  std::vector<int> h_len(n_raw);
  CH_CUDA(cudaMemcpyAsync(h_off.data(), off.p, h_off.size() * sizeof(short4), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaMemcpyAsync(h_t.data(), tv.p, h_t.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaMemcpyAsync(h_dk.data(), dk.p, h_dk.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaMemcpyAsync(h_len.data(), len.p, h_len.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaMemcpyAsync(h_dir.data(), S.raw_dirs.p, h_dir.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaStreamSynchronize(s));
  off.release();
  tv.release();
  dk.release();
  len.release();

  ch_status st = assemble_stencils(P, S, +1, n_raw, max_len, h_off, h_t, h_dk, h_len, h_dir, spacing, cap, s);
  if (st != CH_OK) return st;
  return assemble_stencils(P, S_adj, -1, n_raw, max_len, h_off, h_t, h_dk, h_len, h_dir, spacing, cap, s);
}

// Tap tables, chunks and launch data of one stencil set from the raw walks.
// sign = -1 mirrors every walk (offsets -O[m], direction -d): the DDA from a
// voxel centre along -d visits exactly -O[m] at the same t (the tie rule
// compares the same t values), so the mirrored set gathers the transpose.
ch_status assemble_stencils(ch_plan* P, StencilSet& S, int sign, int n_raw, int max_len,
                            const std::vector<short4>& h_off_in, const std::vector<float>& h_t,
                            const std::vector<float>& h_dk, const std::vector<int>& h_len,
                            const std::vector<float>& h_dir_in, const float* spacing, const int* cap,
                            cudaStream_t s) {
  std::vector<short4> h_off(h_off_in);
  std::vector<float> h_dir(h_dir_in);
  if (sign < 0) {
    for (short4& o : h_off) {
      o.x = (short)-o.x;
      o.y = (short)-o.y;
      o.z = (short)-o.z;
    }
    for (float& d : h_dir) d = -d;
  }
  // merge identical walks (the 12 phi = 180 deg directions are one walk)
  // walks merge when their offsets and kernel row (cone polar angle) agree:
  // their weights then agree for every spectrum, so the merge, the chunks
  // and the windows do not depend on the kernel and a new spectrum only
  // reweights the taps (reweight_taps)
  struct Key {
    std::vector<short4> o;
    int row;
    bool operator<(const Key& k) const {
      if (row != k.row) return row < k.row;
      if (o.size() != k.o.size()) return o.size() < k.o.size();
      return std::memcmp(o.data(), k.o.data(), o.size() * sizeof(short4)) < 0;
    }
  };
  std::map<Key, int> seen;
  std::vector<int> uniq_first, mult;
  for (int d = 0; d < n_raw; ++d) {
    const int L = h_len[d];
    if (L <= 0) continue;
    Key k;
    k.o.assign(h_off.begin() + (size_t)d * max_len, h_off.begin() + (size_t)d * max_len + L);
    k.row = d % P->n_phi;
    auto it = seen.find(k);
    if (it == seen.end()) {
      seen.emplace(std::move(k), (int)uniq_first.size());
      uniq_first.push_back(d);
      mult.push_back(1);
    } else {
      mult[it->second] += 1;
    }
  }
  const int U = (int)uniq_first.size();
  // Run axis of each walk: the one of x and y whose runs (consecutive taps
  // stepping along it, at most RUN_MAX) cost the fewest shared-memory reads
  // (15 + n line values and one or two record reads per run).  Walks are
  // ordered x-axis first so that a work unit changes layout at most once.
  auto split_runs = [&](const short4* o, int L, int ax, std::vector<int>* starts) {
    long cost = 0;
    int m = 0;
    while (m < L) {
      int n = 1;
      while (m + n < L && n < RUN_MAX && (&o[m + n].x)[ax] != (&o[m + n - 1].x)[ax]) ++n;
      if (starts) starts->push_back(m);
      cost += 15 + n + (n > 2 ? 2 : 1);
      m += n;
    }
    return cost;
  };
  std::vector<int> walk_axis(U), order;
  for (int u = 0; u < U; ++u) {
    const int d = uniq_first[u];
    const short4* o = &h_off[(size_t)d * max_len];
    walk_axis[u] = split_runs(o, h_len[d], 1, nullptr) < split_runs(o, h_len[d], 0, nullptr) ? 1 : 0;
  }
  for (int ax = 0; ax < 2; ++ax)
    for (int u = 0; u < U; ++u)
      if (walk_axis[u] == ax) order.push_back(u);
  std::vector<int> tap_base(U), tap_len(U), chunk_base(U), n_chunks(U), chunk_start, run_base(U), axis(U);
  std::vector<int> umult(U), urow(U), tap_run, run_tap;
  std::vector<int4> chunk_rec, runs;
  std::vector<int4> taps;
  std::vector<short4> offs;
  std::vector<float> tvals, dirs((size_t)U * 3);
  // window variant that holds a chunk with these offset spreads (cheapest
  // staged volume), or -1
  auto pick_variant = [](int sx, int sy, int sz) {
    int best = -1;
    long best_vol = 0;
    for (int v = 0; v < N_VARIANTS; ++v) {
      if (sx > var_span_x(v) || sy > var_span_y(v) || sz > var_span_z(v)) continue;
      const long vol = (long)var_p(v) * var_rows(v) * (TX + sx);
      if (best < 0 || vol < best_vol) {
        best = v;
        best_vol = vol;
      }
    }
    return best;
  };
  auto toff = [](const short4& o, int v) { return ((int)o.x * var_rows(v) + (int)o.y) * var_p(v) + (int)o.z; };
  for (int u = 0; u < U; ++u) {
    const int src = order[u];
    const int d = uniq_first[src], L = h_len[d];
    const short4* o = &h_off[(size_t)d * max_len];
    const int ax = walk_axis[src];
    umult[u] = mult[src];
    urow[u] = d % P->n_phi;
    axis[u] = ax;
    tap_base[u] = (int)taps.size();
    tap_len[u] = L;
    for (int k = 0; k < 3; ++k) dirs[(size_t)u * 3 + k] = h_dir[(size_t)d * 3 + k];
    std::vector<float> w(L);
    for (int m = 0; m < L; ++m) {
      int4 t;
      int* tv4 = &t.x;
      for (int v = 0; v < N_VARIANTS; ++v) tv4[v] = toff(o[m], v);
      w[m] = h_dk[(size_t)d * max_len + m] * (float)mult[src];
      std::memcpy(&t.w, &w[m], 4);
      taps.push_back(t);
      offs.push_back(o[m]);
      tvals.push_back(h_t[(size_t)d * max_len + m]);
    }
    std::vector<int> rs;
    split_runs(o, L, ax, &rs);
    const int R = (int)rs.size();
    rs.push_back(L);
    // greedy chunks of whole runs: grow while some window variant still holds the sources
    chunk_base[u] = (int)chunk_start.size();
    run_base[u] = (int)(runs.size() / RUN_REC_INT4);
    std::vector<int> run_var(R);
    int ra = 0;
    while (ra < R) {
      int rb = ra;
      const int a = rs[ra];
      while (rb + 1 < R && rb + 1 - ra < MAX_CHUNK_RUNS) {
        const int e = rs[rb + 2] - 1;
        if (pick_variant(std::abs(o[e].x - o[a].x), std::abs(o[e].y - o[a].y), std::abs(o[e].z - o[a].z)) < 0) break;
        ++rb;
      }
      const int e = rs[rb + 1] - 1;
      const int sx = std::abs(o[e].x - o[a].x), sy = std::abs(o[e].y - o[a].y), sz = std::abs(o[e].z - o[a].z);
      const int var = pick_variant(sx, sy, sz);
      chunk_start.push_back(ra);
      chunk_rec.push_back(make_int4(ra, rb, var, sx | (sy << 16)));
      chunk_rec.push_back(make_int4(std::max<int>(o[a].x, o[e].x), std::max<int>(o[a].y, o[e].y),
                                    std::max<int>(o[a].z, o[e].z), 0));
      for (int r = ra; r <= rb; ++r) run_var[r] = var;
      ra = rb + 1;
    }
    n_chunks[u] = (int)chunk_start.size() - chunk_base[u];
    // run records: the base is the run's tap furthest along the axis, and
    // the tap c steps behind it takes weight slot c (it reads line value i + c)
    for (int r = 0; r < R; ++r) {
      const int m0 = rs[r], n = rs[r + 1] - rs[r];
      const int g = (int)(runs.size() / RUN_REC_INT4);
      int mb = m0;
      for (int m = m0; m < m0 + n; ++m)
        if ((&o[m].x)[ax] > (&o[mb].x)[ax]) mb = m;
      int words[8] = {toff(o[mb], run_var[r]), n, 0, 0, 0, 0, 0, 0};
      for (int m = m0; m < m0 + n; ++m) {
        const int c = (&o[mb].x)[ax] - (&o[m].x)[ax];
        std::memcpy(&words[2 + c], &w[m], 4);
        tap_run.push_back(g * 8 + 2 + c);
      }
      runs.push_back(make_int4(words[0], words[1], words[2], words[3]));
      runs.push_back(make_int4(words[4], words[5], words[6], words[7]));
      run_tap.push_back(tap_base[u] + m0);
    }
  }
  run_tap.push_back((int)taps.size());
  auto up = [&](DevBuf& b, const void* h, size_t n) -> cudaError_t {
    cudaError_t e = b.ensure(std::max<size_t>(n, 16));
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(b.p, h, n, cudaMemcpyHostToDevice, s);
  };
  CH_CUDA(up(S.tap_base, tap_base.data(), tap_base.size() * sizeof(int)));
  CH_CUDA(up(S.tap_len, tap_len.data(), tap_len.size() * sizeof(int)));
  CH_CUDA(up(S.taps, taps.data(), taps.size() * sizeof(int4)));
  CH_CUDA(up(S.offs, offs.data(), offs.size() * sizeof(short4)));
  CH_CUDA(up(S.tvals, tvals.data(), tvals.size() * sizeof(float)));
  CH_CUDA(up(S.runs, runs.data(), runs.size() * sizeof(int4)));
  CH_CUDA(up(S.run_base, run_base.data(), run_base.size() * sizeof(int)));
  CH_CUDA(up(S.tap_run, tap_run.data(), tap_run.size() * sizeof(int)));
  CH_CUDA(up(S.run_tap, run_tap.data(), run_tap.size() * sizeof(int)));
  CH_CUDA(up(S.axis, axis.data(), axis.size() * sizeof(int)));
  CH_CUDA(up(S.chunk_base, chunk_base.data(), chunk_base.size() * sizeof(int)));
  CH_CUDA(up(S.n_chunks, n_chunks.data(), n_chunks.size() * sizeof(int)));
  CH_CUDA(up(S.chunk_start, chunk_start.data(), chunk_start.size() * sizeof(int)));
  CH_CUDA(up(S.chunk_rec, chunk_rec.data(), chunk_rec.size() * sizeof(int4)));
  CH_CUDA(up(S.dirs, dirs.data(), dirs.size() * sizeof(float)));
  CH_CUDA(up(S.walk_row, urow.data(), urow.size() * sizeof(int)));
  CH_CUDA(up(S.walk_mult, umult.data(), umult.size() * sizeof(int)));
  CH_CUDA(cudaStreamSynchronize(s));
  S.valid = true;
  S.n_dirs = U;
  S.n_raw = n_raw;
  S.total_taps = taps.size();
  for (int k = 0; k < 3; ++k) {
    S.spacing[k] = spacing[k];
    S.cap[k] = cap[k];
  }
  return CH_OK;
}

ch_status ensure_stencils(ch_plan* P, const float* spacing, const int* dims, cudaStream_t s) {
  StencilSet& S = P->st;
  bool ok = S.valid;
  for (int k = 0; k < 3 && ok; ++k)
    ok = S.spacing[k] == spacing[k] && S.cap[k] >= dims[k];
  if (ok) return CH_OK;
  if (P->live_batches > 0)
    return fail(CH_ERR_INVALID_ARG, "the plan's stencils cannot be rebuilt while captured batches use them "
                                    "(ch_batch_destroy them, or prepare the plan for the largest grid first)");
  int cap[3];
  for (int k = 0; k < 3; ++k) cap[k] = std::max(dims[k], S.valid && S.spacing[k] == spacing[k] ? S.cap[k] : 0);
  ConeFrame room{};
  return build_stencils(P, spacing, cap, s, room, P->st, P->st_adj);
}

// Stencils of the cones rotated into one beam's frame (CH_OPT_CONES_IN_BEAM_FRAME),
// cached per orientation (least recently used out past kMaxFrames).
constexpr size_t kMaxFrames = 16;
ch_status frame_stencils(ch_plan* P, const float* spacing, const int* dims, const double* xform, cudaStream_t s,
                         StencilSet** out) {
  P->use_clock += 1;
  for (auto& f : P->frames) {
    bool ok = f->fwd.valid && std::memcmp(f->frame.m, xform, sizeof(f->frame.m)) == 0;
    for (int k = 0; k < 3 && ok; ++k) ok = f->fwd.spacing[k] == spacing[k] && f->fwd.cap[k] >= dims[k];
    if (ok) {
      f->last_use = P->use_clock;
      *out = &f->fwd;
      return CH_OK;
    }
  }
  if (P->live_batches > 0)
    return fail(CH_ERR_INVALID_ARG, "beam-frame stencils cannot be built while captured batches exist");
  if (P->frames.size() >= kMaxFrames) {
    auto lru = std::min_element(P->frames.begin(), P->frames.end(),
                                [](const std::unique_ptr<FrameStencils>& a, const std::unique_ptr<FrameStencils>& b) {
                                  return a->last_use < b->last_use;
                                });
    spec_forget(P, &(*lru)->fwd);
    spec_forget(P, &(*lru)->adj);
    P->frames.erase(lru);
  }
  std::unique_ptr<FrameStencils> f(new FrameStencils());
  f->frame.on = 1;
  std::memcpy(f->frame.m, xform, sizeof(f->frame.m));
  int cap[3] = {dims[0], dims[1], dims[2]};
  ch_status st = build_stencils(P, spacing, cap, s, f->frame, f->fwd, f->adj);
  if (st != CH_OK) return st;
  f->last_use = P->use_clock;
  *out = &f->fwd;
  P->frames.push_back(std::move(f));
  return CH_OK;
}

ConeDirs cone_dirs(const StencilSet& S, const ch_plan* P) {
  const ch_tuning& t = P->tuning;
  ConeDirs D;
  D.wait_limit = P->wait_limit > 0 ? P->wait_limit : MBAR_LIMIT;
  D.withhold = P->withhold;
  D.group = t.dir_group;
  D.order = t.unit_order;
  D.n_dirs = S.n_dirs;
  D.tap_base = S.tap_base.as<int>();
  D.tap_len = S.tap_len.as<int>();
  D.taps = S.taps.as<int4>();
  D.offs = S.offs.as<short4>();
  D.tvals = S.tvals.as<float>();
  D.runs = S.runs.as<int4>();
  D.run_base = S.run_base.as<int>();
  D.tap_run = S.tap_run.as<int>();
  D.run_tap = S.run_tap.as<int>();
  D.axis = S.axis.as<int>();
  D.chunk_base = S.chunk_base.as<int>();
  D.n_chunks = S.n_chunks.as<int>();
  D.chunk_start = S.chunk_start.as<int>();
  D.chunk_rec = S.chunk_rec.as<int4>();
  D.dirs = S.dirs.as<float>();
  return D;
}

// ---------------------------------------------------------- spectral S^ --
SpecGrid spec_grid(const ch_plan* P, const int* n, const int* M, int zp, int conj, const float2* shat) {
  SpecGrid g{};
  for (int k = 0; k < 3; ++k) {
    g.n[k] = n[k];
    g.M[k] = M[k];
    g.logL[k] = k == 2 ? spec_lines_log2(M[2]) : spec_pass_lines_log2(M[k], M[2]);
    g.tw[k] = P->spec_tw.as<float2>() + spec_twiddle_offset(M[k]);
  }
  g.zp = zp;
  g.conj = conj;
  g.shat = shat;
  g.plane = spec_plane_path(M) && n[0] <= SPEC_PLANE_M / 2 && n[1] <= SPEC_PLANE_M / 2 && n[2] <= SPEC_PLANE_M / 2;
  g.lp = g.plane ? spec_plane_pitch(n) : 0;
  return g;
}

// S^ of grid shape n for stencil set S: the current tap weights summed per
// offset o with |o_k| <= n_k - 1 (float64 sums in offset order, times
// 1/(Mx My Mz)), placed at o mod M, then three forward FFT passes.  Cached
// per (set, shape), least recently used out past kSpecEntries while no
// captured batch holds one.
constexpr size_t kSpecEntries = 8;
ch_status spec_shat(ch_plan* P, const StencilSet& S, const int* n, cudaStream_t s, const float2** out) {
  P->use_clock += 1;
  for (auto& e : P->spec)
    if (e->set == &S && e->n[0] == n[0] && e->n[1] == n[1] && e->n[2] == n[2]) {
      e->last_use = P->use_clock;
      *out = e->shat.as<float2>();
      return CH_OK;
    }
  if (!P->spec_tw.p) {
    const std::vector<float2> tw = spec_twiddles();
    CH_CUDA(P->spec_tw.ensure(tw.size() * sizeof(float2)));
    CH_CUDA(cudaMemcpy(P->spec_tw.p, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice));
  }
  if (P->spec.size() >= kSpecEntries && P->live_batches == 0) {
    auto lru = std::min_element(P->spec.begin(), P->spec.end(),
                                [](const std::unique_ptr<SpecEntry>& a, const std::unique_ptr<SpecEntry>& b) {
                                  return a->last_use < b->last_use;
                                });
    P->spec.erase(lru);
  }
  const int M[3] = {spec_period(n[0]), spec_period(n[1]), spec_period(n[2])};
  const size_t vol = (size_t)M[0] * M[1] * M[2];
  std::vector<int4> taps(S.total_taps);
  std::vector<short4> offs(S.total_taps);
  CH_CUDA(cudaMemcpyAsync(taps.data(), S.taps.p, taps.size() * sizeof(int4), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaMemcpyAsync(offs.data(), S.offs.p, offs.size() * sizeof(short4), cudaMemcpyDeviceToHost, s));
  CH_CUDA(cudaStreamSynchronize(s));
  std::vector<std::pair<long long, float>> ent;
  ent.reserve(taps.size());
  for (size_t t = 0; t < taps.size(); ++t) {
    const short4 o = offs[t];
    if (std::abs((int)o.x) > n[0] - 1 || std::abs((int)o.y) > n[1] - 1 || std::abs((int)o.z) > n[2] - 1) continue;
    const long long i = (((long long)(o.x + M[0]) % M[0]) * M[1] + (o.y + M[1]) % M[1]) * M[2] + (o.z + M[2]) % M[2];
    float w;
    std::memcpy(&w, &taps[t].w, 4);
    ent.emplace_back(i, w);
  }
  std::sort(ent.begin(), ent.end(),
            [](const std::pair<long long, float>& a, const std::pair<long long, float>& b) { return a.first < b.first; });
  std::vector<long long> idx;
  std::vector<float> val;
  const double scale = 1.0 / (double)vol;
  for (size_t k = 0; k < ent.size();) {
    double sum = 0.0;
    size_t e = k;
    for (; e < ent.size() && ent[e].first == ent[k].first; ++e) sum += (double)ent[e].second;
    idx.push_back(ent[k].first);
    val.push_back((float)(sum * scale));
    k = e;
  }
  std::unique_ptr<SpecEntry> E(new SpecEntry());
  E->set = &S;
  for (int k = 0; k < 3; ++k) E->n[k] = n[k];
  DevBuf d_idx, d_val, s_real, work;
  auto cleanup = [&]() {
    d_idx.release();
    d_val.release();
    s_real.release();
    work.release();
  };
  cudaError_t e = E->shat.ensure(vol * sizeof(float2));
  if (e == cudaSuccess) e = s_real.ensure(vol * sizeof(float));
  if (e == cudaSuccess) e = work.ensure(vol * sizeof(float2));
  if (e == cudaSuccess) e = d_idx.ensure(std::max<size_t>(idx.size(), 1) * sizeof(long long));
  if (e == cudaSuccess) e = d_val.ensure(std::max<size_t>(val.size(), 1) * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx.p, idx.data(), idx.size() * sizeof(long long), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_val.p, val.data(), val.size() * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(s_real.p, 0, vol * sizeof(float), s);
  if (e != cudaSuccess) {
    cleanup();
    return fail(CH_ERR_DEVICE, std::string("spectral stencil: ") + cudaGetErrorString(e));
  }
  SpecLaunch L{};
  L.g = spec_grid(P, M, M, M[2], 0, nullptr);
  L.n_pairs = 1;
  L.p[0] = SpecPair{s_real.as<float>(), nullptr, nullptr, nullptr, work.as<float2>(), E->shat.as<float2>(),
                    nullptr, nullptr};
  launch_spec_build(L, d_idx.as<long long>(), d_val.as<float>(), (int)idx.size(), s_real.as<float>(), s);
  if (spec_plane_path(M)) {
    // the plane path reads S^ plane by plane: [Mz][My][Mx], transposed into
    // the work buffer, which then becomes the cached S^ (the untransposed
    // copy is released with the other build buffers)
    launch_spec_transpose(E->shat.as<float2>(), work.as<float2>(), M[0], M[1], M[2], s);
    std::swap(E->shat, work);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return fail(CH_ERR_DEVICE, std::string("spectral stencil: ") + cudaGetErrorString(e));
  E->last_use = P->use_clock;
  *out = E->shat.as<float2>();
  P->spec.push_back(std::move(E));
  return CH_OK;
}

// --------------------------------------------------------- validation --
ch_status check_grid(const ch_grid* g) {
  if (!g) return fail(CH_ERR_INVALID_ARG, "grid is NULL");
  for (int k = 0; k < 3; ++k) {
    if (g->n[k] <= 0 || g->n[k] > 4096) return fail(CH_ERR_INVALID_ARG, "grid dimension out of range (1..4096)");
    if ((long long)g->n[0] * g->n[1] * g->n[2] >= (1ll << 31))
      return fail(CH_ERR_INVALID_ARG, "grid holds 2^31 voxels or more");
    if (!(g->spacing[k] > 0.0f) || !std::isfinite(g->spacing[k]))
      return fail(CH_ERR_INVALID_ARG, "grid spacing must be positive");
    if (!std::isfinite(g->origin[k])) return fail(CH_ERR_INVALID_ARG, "grid origin must be finite");
  }
  return CH_OK;
}

ch_status check_beam(const ch_beam* b) {
  if (!b) return fail(CH_ERR_INVALID_ARG, "beam is NULL");
  if ((!b->block && !b->block_uniform) || b->block_rows <= 0 || b->block_cols <= 0)
    return fail(CH_ERR_INVALID_ARG, "beam block map missing");
  if (b->full_rows < b->block_r0 + b->block_rows || b->full_cols < b->block_c0 + b->block_cols ||
      b->block_r0 < 0 || b->block_c0 < 0)
    return fail(CH_ERR_INVALID_ARG, "block crop lies outside the full map");
  const double nn = b->vy[0] * b->vy[0] + b->vy[1] * b->vy[1] + b->vy[2] * b->vy[2];
  if (!(nn > 0.0)) return fail(CH_ERR_INVALID_ARG, "beam v_y is zero");
  return CH_OK;
}

ch_status check_settings(const ch_settings* s) {
  if (!s) return fail(CH_ERR_INVALID_ARG, "settings is NULL");
  if (s->samples < 1 || s->samples > 16) return fail(CH_ERR_INVALID_ARG, "fluenceResampling out of range (1..16)");
  if (s->n_energy < 0 || s->n_energy > CH_MAX_ENERGY) return fail(CH_ERR_INVALID_ARG, "too many energy bins");
  if (s->options & ~(CH_OPT_RADIOLOGICAL_DISTANCE | CH_OPT_CONES_IN_BEAM_FRAME))
    return fail(CH_ERR_INVALID_ARG, "unknown physics option bits");
  return CH_OK;
}

// ------------------------------------------------------ beam prep --
// samples: sub-samples per axis of the blocking test (fluenceResampling)
BeamDev make_beam(const ch_beam& in, const ch_grid& g, int samples) {
  BeamDev b{};
  for (int k = 0; k < 3; ++k) {
    b.src[k] = in.src[k];
    b.vy[k] = in.vy[k];
    b.m0[k] = in.xform[k];
    b.m2[k] = in.xform[6 + k];
    b.srcf[k] = (float)in.src[k];
    b.vyf[k] = (float)in.vy[k];
    b.m0f[k] = (float)in.xform[k];
    b.m2f[k] = (float)in.xform[6 + k];
  }
  // v_y . w with w = float32(src), reference evaluation order
  const double w0 = b.srcf[0], w1 = b.srcf[1], w2 = b.srcf[2];
  b.vyw = (b.vy[0] * w0 + b.vy[1] * w1) + b.vy[2] * w2;
  b.vywf = (b.vyf[0] * b.srcf[0] + b.vyf[1] * b.srcf[1]) + b.vyf[2] * b.srcf[2];
  b.geom_f32 = in.geom_f32;
  const double nS = b.vy[0] * b.src[0] + b.vy[1] * b.src[1] + b.vy[2] * b.src[2];
  const double m0S = b.m0[0] * b.src[0] + b.m0[1] * b.src[1] + b.m0[2] * b.src[2];
  const double m2S = b.m2[0] * b.src[0] + b.m2[1] * b.src[1] + b.m2[2] * b.src[2];
  b.a_nS = (float)nS;
  b.a_m0S = (float)m0S;
  b.a_m2S = (float)m2S;
  b.a_K = (float)(-b.vyw);
  b.a_c0 = (float)(b.m0[0] * w0 + b.m0[1] * w1 + b.m0[2] * w2);
  b.a_c2 = (float)(b.m2[0] * w0 + b.m2[1] * w1 + b.m2[2] * w2);
  // map rows [r0, r1] are read for x in [(r0 - 1999)/100, (r1 - 1998)/100);
  // cell 0 wraps to the last row, i.e. x in [-20, -19.99)
  const int r0 = in.block_r0, r1 = in.block_r0 + in.block_rows - 1;
  const int c0 = in.block_c0, c1 = in.block_c0 + in.block_cols - 1;
  double xlo = (r0 - 1999) / 100.0, xhi = (r1 - 1998) / 100.0;
  double zlo = (c0 - 1999) / 100.0, zhi = (c1 - 1998) / 100.0;
  if (r1 == in.full_rows - 1) xlo = std::min(xlo, -20.0);
  if (c1 == in.full_cols - 1) zlo = std::min(zlo, -20.0);
  b.cx_lo = (float)std::max(xlo, -20.0);
  b.cx_hi = (float)std::min(xhi, 20.0);
  b.cz_lo = (float)std::max(zlo, -20.0);
  b.cz_hi = (float)std::min(zhi, 20.0);
  const float smax = std::max(g.spacing[0], std::max(g.spacing[1], g.spacing[2]));
  // The sub-samples of a voxel sit at s (2 i + 1 - S) / (2 S) from its
  // centre per axis, so the farthest lies r = sqrt(3) smax (S - 1) / (2 S)
  // away.  An offset r at depth d moves the projection by at most
  // |K| r / (d - r) (1 + lateral ratio at the centre), and the cull tests
  // centres deeper than dmin = 0.2 |K| (nearer ones are always kept), so
  // k = r / (1 - r / dmin) bounds r d / (d - r); the margin's 0.01 cm
  // covers float32 rounding.  Voxels a tenth of dmin across or larger
  // (never in practice) are not culled.
  const double r_s = std::sqrt(3.0) * (double)smax * (double)(samples - 1) / (2.0 * samples);
  const double dmin = 0.2 * std::fabs((double)b.a_K);
  b.cull_margin_k = r_s < 0.1 * dmin ? (float)(r_s / (1.0 - r_s / dmin)) : 0.0f;
  b.cull_enable = (-nS > 0.0 && b.cx_lo <= b.cx_hi && b.cz_lo <= b.cz_hi && r_s < 0.1 * dmin) ? 1 : 0;
  b.block = in.block;
  b.brows = in.block_rows;
  b.bcols = in.block_cols;
  b.br0 = in.block_r0;
  b.bc0 = in.block_c0;
  b.full_rows = in.full_rows;
  b.full_cols = in.full_cols;
  b.uniform = in.block_uniform;
  b.sad = in.sad;
  b.sad_f32 = in.sad_f32;
  return b;
}

SettingsDev make_settings(const ch_settings& s) {
  SettingsDev d{};
  d.sPri = (float)s.sPri;
  d.sAnn = (float)s.sAnn;
  d.zAnn = (float)s.zAnn;
  d.rInner = (float)s.rInner;
  d.rOuter = (float)s.rOuter;
  d.zExp = (float)s.zExp;
  d.sExp = (float)s.sExp;
  d.kExp = (float)s.kExp;
  d.softRatio = (float)s.softRatio;
  d.softLimit = (float)s.softLimit;
  d.hornRatio = (float)s.hornRatio;
  d.samples = s.samples;
  d.n_energy = s.n_energy;
  for (int i = 0; i < s.n_energy; ++i) {
    d.E[i] = s.E[i];
    d.w[i] = s.w[i];
    d.mu[i] = s.mu[i];
  }
  return d;
}

// Frustum planes a.(p - S) <= e bounding every voxel centre whose samples
// can project into the open block region (widened by half a voxel).
void make_planes(const ch_beam& in, const ch_grid& g, const BeamDev& b, RangeBeam& R) {
  R.n_planes = 0;
  const double* n = in.vy;
  const double* S = in.src;
  const double D = -(n[0] * S[0] + n[1] * S[1] + n[2] * S[2]);
  if (!(D > 0.0)) return;
  // every grid point (widened by a voxel) must lie in front of the source
  for (int c = 0; c < 8; ++c) {
    double p[3];
    for (int k = 0; k < 3; ++k) {
      const int hi = (c >> k) & 1;
      p[k] = (double)g.origin[k] + (hi ? (g.n[k] - 0.5) * g.spacing[k] : -1.5 * g.spacing[k]);
    }
    const double depth = n[0] * (p[0] - S[0]) + n[1] * (p[1] - S[1]) + n[2] * (p[2] - S[2]);
    if (!(depth > 0.05 * D)) return;
  }
  const double m0S = b.m0[0] * S[0] + b.m0[1] * S[1] + b.m0[2] * S[2];
  const double m2S = b.m2[0] * S[0] + b.m2[1] * S[1] + b.m2[2] * S[2];
  const double pad = 0.02;  // cm, covers cell-edge and float32 slack
  struct Pl { double a[3]; };
  std::vector<Pl> pls;
  auto add = [&](const double* m, double sgn, double X, double mS) {
    Pl p;
    // sgn = +1: x_b >= X  ->  ((X - mS) n - D m) . r <= 0
    // sgn = -1: x_b <= X  ->  (D m - (X - mS) n) . r <= 0
    for (int k = 0; k < 3; ++k) p.a[k] = sgn * ((X - mS) * n[k] - D * m[k]);
    pls.push_back(p);
  };
  add(b.m0, +1.0, b.cx_lo - pad, m0S);
  add(b.m0, -1.0, b.cx_hi + pad, m0S);
  add(b.m2, +1.0, b.cz_lo - pad, m2S);
  add(b.m2, -1.0, b.cz_hi + pad, m2S);
  for (size_t j = 0; j < pls.size() && j < 4; ++j) {
    double e = 0.0, aos = 0.0, scale = 0.0;
    for (int k = 0; k < 3; ++k) {
      e += std::fabs(pls[j].a[k]) * g.spacing[k] * 0.5;
      aos += pls[j].a[k] * ((double)g.origin[k] - S[k]);
      scale = std::max(scale, std::fabs(pls[j].a[k]));
    }
    if (!(scale > 0.0)) continue;
    // normalise so float32 in the range kernel keeps its precision
    for (int k = 0; k < 3; ++k) R.pa[R.n_planes][k] = (float)(pls[j].a[k] / scale);
    R.pk0[R.n_planes] = (float)((aos - e) / scale - 1e-3);
    ++R.n_planes;
  }
}

struct BeamJob {
  GridDev g;
  BeamDev b;
  SettingsDev s;
  const float* rho;
  float* dose;
  size_t t_off;        // float offset in the T arena
  size_t r_off;        // uint32 offset in the ranges arena
  size_t l_off;        // int offset of the beam's voxel list
  size_t f_off;        // int offset of its per-line flags (one byte per (x, y) line)
  int ntile[3];
  int n_tiles;
  int n_units;
  ch_grid grid;
  ch_beam beam;
};

// The TMA tensor maps of one padded [x][y][zp] volume: one per window
// shape and x extent (boxes P z x rows y x ex x, zero fill outside).
ch_status encode_windows(PFN_cuTensorMapEncodeTiled_v12000 enc, ConeBeam& C, float* vol, const GridDev& g) {
  cuuint64_t gdim[3] = {(cuuint64_t)g.n[2], (cuuint64_t)g.n[1], (cuuint64_t)g.n[0]};
  cuuint64_t gstride[2] = {(cuuint64_t)g.zp * 4, (cuuint64_t)g.zp * g.n[1] * 4};
  cuuint32_t estr[3] = {1, 1, 1};
  for (int v = 0; v < N_VARIANTS; ++v) {
    for (int ex = TX; ex <= var_max_ex(v); ++ex) {
      cuuint32_t box[3] = {(cuuint32_t)var_p(v), (cuuint32_t)var_rows(v), (cuuint32_t)ex};
      CUresult r = enc(&C.tmap[tmap_index(v, ex)], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)vol, gdim, gstride,
                       box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return fail(CH_ERR_DEVICE, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    }
  }
  return CH_OK;
}

// Upload launch records through the plan's double-buffered pinned staging
// (a true async copy, issued before the kernels that read them).
// One host array staged to a device buffer.
struct Seg {
  void* dst;
  const void* src;
  size_t bytes;
};

// Launch records go through pinned, double-buffered staging so their upload
// is a true asynchronous copy: the buffer used two calls ago is reused once
// its upload has been read.
ch_status stage_records(ch_plan* P, const std::vector<Seg>& segs, cudaStream_t s) {
  const int hb = P->rec_next;
  P->rec_next ^= 1;
  if (P->rec_pending[hb]) CH_CUDA(cudaEventSynchronize(P->ev_rec[hb]));
  P->rec_pending[hb] = false;
  size_t total = 0;
  for (const Seg& g : segs) total += (g.bytes + 255) / 256 * 256;
  if (total > P->h_rec_bytes[hb]) {
    if (P->h_rec[hb]) CH_CUDA(cudaFreeHost(P->h_rec[hb]));
    P->h_rec[hb] = nullptr;
    P->h_rec_bytes[hb] = 0;
    CH_CUDA(cudaMallocHost(&P->h_rec[hb], total));
    P->h_rec_bytes[hb] = total;
  }
  if (!P->ev_rec[hb]) CH_CUDA(cudaEventCreateWithFlags(&P->ev_rec[hb], cudaEventDisableTiming));
  char* h = static_cast<char*>(P->h_rec[hb]);
  for (const Seg& g : segs) {
    std::memcpy(h, g.src, g.bytes);
    CH_CUDA(cudaMemcpyAsync(g.dst, h, g.bytes, cudaMemcpyHostToDevice, s));
    h += (g.bytes + 255) / 256 * 256;
  }
  CH_CUDA(cudaEventRecord(P->ev_rec[hb], s));
  P->rec_pending[hb] = true;
  return CH_OK;
}

// ------------------------------------------------- spectral cone layout --
// Beams of one grid shape are paired in call order; a launch takes up to
// SPEC_MAX_PAIRS pairs of one shape, and the launches of a batch run one
// after another in one work arena (A and B of each pair of the launch).
struct SpecPlanPair {
  int j1, j2;                // beams (j2 = -1: the first alone)
  size_t a_off, b_off;       // float2 offsets in the work arena
};
struct SpecPlanLaunch {
  int n[3], M[3];
  const float2* shat = nullptr;
  std::vector<SpecPlanPair> pairs;
};
struct SpecLayout {
  std::vector<SpecPlanLaunch> launches;
  size_t arena = 0;          // float2
};

constexpr long long kSpecMaxVolume = 1ll << 28;   // largest Mx My Mz (S^ of 2 GiB)

bool spec_fits(const int* n) {
  long long v = 1;
  for (int k = 0; k < 3; ++k) {
    const int m = spec_period(n[k]);
    if (m == 0) return false;
    v *= m;
  }
  return v <= kSpecMaxVolume;
}

SpecLayout spec_layout(int n, const ch_grid* grids) {
  SpecLayout L;
  std::vector<char> done(n, 0);
  for (int i = 0; i < n; ++i) {
    if (done[i]) continue;
    std::vector<int> group;
    for (int j = i; j < n; ++j)
      if (!done[j] && grids[j].n[0] == grids[i].n[0] && grids[j].n[1] == grids[i].n[1] &&
          grids[j].n[2] == grids[i].n[2]) {
        group.push_back(j);
        done[j] = 1;
      }
    const int* d = grids[i].n;
    const int M[3] = {spec_period(d[0]), spec_period(d[1]), spec_period(d[2])};
    // the plane path keeps A plane-major (pitch spec_plane_pitch) and needs no B
    const bool plane = spec_plane_path(M);
    const size_t a_sz = plane ? (size_t)M[2] * spec_plane_pitch(d) : (size_t)d[0] * d[1] * M[2];
    const size_t b_sz = plane ? 0 : (size_t)d[0] * M[1] * M[2];
    for (size_t p = 0; p < group.size(); p += 2 * SPEC_MAX_PAIRS) {
      SpecPlanLaunch l;
      for (int k = 0; k < 3; ++k) {
        l.n[k] = d[k];
        l.M[k] = M[k];
      }
      size_t off = 0;
      const size_t end = std::min(group.size(), p + 2 * SPEC_MAX_PAIRS);
      for (size_t q = p; q < end; q += 2) {
        SpecPlanPair pr;
        pr.j1 = group[q];
        pr.j2 = q + 1 < end ? group[q + 1] : -1;
        pr.a_off = off;
        off += (a_sz + 31) / 32 * 32;
        pr.b_off = off;
        off += (b_sz + 31) / 32 * 32;
        l.pairs.push_back(pr);
      }
      L.arena = std::max(L.arena, off);
      L.launches.push_back(std::move(l));
    }
  }
  return L;
}

bool spec_batch(const ch_plan* P, int n, const ch_grid* grids) {
  if (P->tuning.cone_method != CH_CONE_SPECTRAL) return false;
  for (int i = 0; i < n; ++i)
    if (!spec_fits(grids[i].n)) return false;
  return true;
}

// Scratch arena sizes of one batch, in the order T, aabb, counters, ranges,
// cranges, cone_beams, range_beams, list_v (every beam's voxel list),
// spectral work, prologue records (the buffers run() grows); the gather's
// tables are empty for a spectral batch.
constexpr int N_SCRATCH = 10;
struct ScratchNeed {
  size_t bytes[N_SCRATCH];
};

ScratchNeed scratch_need(int n, const ch_grid* grids, int U, bool spectral = false) {
  if (spectral) U = 0;
  size_t t_total = 0, r_total = 0, l_total = 0;
  for (int i = 0; i < n; ++i) {
    const size_t zp = (size_t)round_up(grids[i].n[2], 4);
    t_total += (size_t)grids[i].n[0] * grids[i].n[1] * zp;
    t_total = (t_total + 63) / 64 * 64;
    const size_t tiles = (size_t)((grids[i].n[0] + TX - 1) / TX) * ((grids[i].n[1] + TY - 1) / TY) *
                         ((grids[i].n[2] + TZ - 1) / TZ);
    r_total += tiles * U;
    l_total += ((size_t)grids[i].n[0] * grids[i].n[1] * grids[i].n[2] + 63) / 64 * 64;
    l_total += ((size_t)grids[i].n[0] * grids[i].n[1] + 255) / 256 * 64;     // line flags
  }
  ScratchNeed r;
  r.bytes[0] = t_total * sizeof(float);
  r.bytes[1] = (size_t)n * 8 * sizeof(int);
  r.bytes[2] = 8 * sizeof(int);
  r.bytes[3] = std::max<size_t>(r_total, 1) * sizeof(uint32_t);
  r.bytes[4] = r.bytes[3];
  r.bytes[5] = (size_t)n * sizeof(ConeBeam);
  r.bytes[6] = (size_t)n * sizeof(RangeBeam);
  r.bytes[7] = std::max<size_t>(l_total, 1) * sizeof(int);
  r.bytes[8] = spectral ? spec_layout(n, grids).arena * sizeof(float2) : 0;
  r.bytes[9] = (size_t)n * sizeof(PrologueBeam);
  return r;
}

const DevBuf* scratch_bufs(const ch_plan* P, int k) {
  const DevBuf* b[N_SCRATCH] = {&P->T,          &P->aabb,        &P->counters, &P->ranges,    &P->cranges,
                                &P->cone_beams, &P->range_beams, &P->list_v,   &P->spec_work, &P->pro_beams};
  return b[k];
}

// A validated batch: per-beam device parameters and scratch offsets.
struct BatchPlan {
  std::vector<BeamJob> jobs;
  const StencilSet* set = nullptr;   // the stencils of every beam of the batch
  int U = 0;
  int total_units = 0;
  int max_tiles = 0;
  bool spectral = false;             // cone stage by FFT convolution (else the gather)
  SpecLayout spec;
};

// Scratch a batch runs in (the plan's arena, or a captured batch's own).
struct Scratch {
  float* T;
  int* aabb;
  int* counters;
  uint32_t* ranges;
  uint32_t* cranges;
  ConeBeam* cone_beams;
  RangeBeam* range_beams;
  int* list_v;
  float2* spec;           // spectral work arena
  PrologueBeam* pro;      // batched prologue records
};

ch_status plan_batch(ch_plan* P, int n, const ch_grid* grids, const float* const* rho, const int* swap_xy,
                     const ch_beam* beams, const ch_settings* settings, float* const* dose, cudaStream_t s,
                     BatchPlan& B, const StencilSet* set = nullptr) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  if (n <= 0) return fail(CH_ERR_INVALID_ARG, "no beams");
  if (!grids || !beams || !settings) return fail(CH_ERR_INVALID_ARG, "batch arrays missing");
  CH_CUDA(cudaSetDevice(P->device));
  B.jobs.assign(n, BeamJob{});
  int dims[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    ch_status st;
    if ((st = check_grid(&grids[i])) != CH_OK) return st;
    if ((st = check_beam(&beams[i])) != CH_OK) return st;
    if ((st = check_settings(&settings[i])) != CH_OK) return st;
    if (!rho || !rho[i] || !dose || !dose[i]) return fail(CH_ERR_INVALID_ARG, "density or dose pointer is NULL");
    const int sw = swap_xy ? swap_xy[i] : 0;
    if (sw && grids[i].n[0] != grids[i].n[1])
      return fail(CH_ERR_INVALID_ARG, "swap_xy needs a square x/y grid");
    for (int k = 0; k < 3; ++k) {
      if (grids[i].spacing[k] != grids[0].spacing[k])
        return fail(CH_ERR_INVALID_ARG, "all beams of one call must share the voxel spacing");
      dims[k] = std::max(dims[k], grids[i].n[k]);
    }
  }
  if (set) {
    B.set = set;                 // the caller prepared it (beam-frame cones)
  } else {
    ch_status st = ensure_stencils(P, grids[0].spacing, dims, s);
    if (st != CH_OK) return st;
    B.set = &P->st;
  }
  B.U = B.set->n_dirs;
  B.spectral = spec_batch(P, n, grids);
  if (B.spectral) {
    B.spec = spec_layout(n, grids);
    for (SpecPlanLaunch& l : B.spec.launches) {
      ch_status st = spec_shat(P, *B.set, l.n, s, &l.shat);
      if (st != CH_OK) return st;
    }
  }
  const int n_groups = (B.U + P->tuning.dir_group - 1) / P->tuning.dir_group;
  size_t t_total = 0, r_total = 0, l_total = 0;
  B.total_units = 0;
  B.max_tiles = 0;
  for (int i = 0; i < n; ++i) {
    BeamJob& J = B.jobs[i];
    J.grid = grids[i];
    J.beam = beams[i];
    for (int k = 0; k < 3; ++k) {
      J.g.n[k] = grids[i].n[k];
      J.g.origin[k] = grids[i].origin[k];
      J.g.spacing[k] = grids[i].spacing[k];
    }
    J.g.zp = round_up(grids[i].n[2], 4);
    J.g.swap_xy = swap_xy ? swap_xy[i] : 0;
    J.b = make_beam(beams[i], grids[i], settings[i].samples);
    J.s = make_settings(settings[i]);
    J.rho = rho[i];
    J.dose = dose[i];
    J.t_off = t_total;
    t_total += (size_t)J.g.n[0] * J.g.n[1] * J.g.zp;
    t_total = (t_total + 63) / 64 * 64;
    J.l_off = l_total;
    l_total += ((size_t)J.g.n[0] * J.g.n[1] * J.g.n[2] + 63) / 64 * 64;
    J.f_off = l_total;
    l_total += ((size_t)J.g.n[0] * J.g.n[1] + 255) / 256 * 64;
    J.ntile[0] = (J.g.n[0] + TX - 1) / TX;
    J.ntile[1] = (J.g.n[1] + TY - 1) / TY;
    J.ntile[2] = (J.g.n[2] + TZ - 1) / TZ;
    J.n_tiles = J.ntile[0] * J.ntile[1] * J.ntile[2];
    J.n_units = J.n_tiles * n_groups;
    J.r_off = r_total;
    r_total += (size_t)J.n_tiles * B.U;
    B.total_units += J.n_units;
    B.max_tiles = std::max(B.max_tiles, J.n_tiles);
  }
  return CH_OK;
}

// Launch records of every beam (tensor maps over its TERMA volume, tap
// ranges, beam frustum planes) pointing into scratch S.
ch_status make_records(const BatchPlan& B, const Scratch& S, std::vector<ConeBeam>& cb, std::vector<RangeBeam>& rb) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return fail(CH_ERR_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  const int n = (int)B.jobs.size();
  cb.assign(n, ConeBeam{});
  rb.assign(n, RangeBeam{});
  int unit_begin = 0;
  for (int i = 0; i < n; ++i) {
    const BeamJob& J = B.jobs[i];
    ConeBeam& C = cb[i];
    std::memset(&C, 0, sizeof(C));
    ch_status est = encode_windows(enc, C, S.T + J.t_off, J.g);
    if (est != CH_OK) return est;
    C.dose = J.dose;
    C.ranges = S.ranges + J.r_off;
    C.cranges = S.cranges + J.r_off;
    for (int k = 0; k < 3; ++k) {
      C.n[k] = J.g.n[k];
      C.ntile[k] = J.ntile[k];
    }
    C.n_tiles = J.n_tiles;
    C.unit_begin = unit_begin;
    C.n_units = J.n_units;
    unit_begin += J.n_units;
    RangeBeam& R = rb[i];
    std::memset(&R, 0, sizeof(R));
    for (int k = 0; k < 3; ++k) {
      R.n[k] = J.g.n[k];
      R.ntile[k] = J.ntile[k];
      R.origin[k] = J.g.origin[k];
      R.spacing[k] = J.g.spacing[k];
    }
    R.n_tiles = J.n_tiles;
    make_planes(J.beam, J.grid, J.b, R);
    R.aabb = S.aabb + 8 * i;
    R.ranges = S.ranges + J.r_off;
    R.cranges = S.cranges + J.r_off;
  }
  return CH_OK;
}

// Records of the batched prologue, pointing into scratch S.
std::vector<PrologueBeam> make_prologue_records(const BatchPlan& B, const Scratch& S) {
  std::vector<PrologueBeam> pb(B.jobs.size());
  for (size_t i = 0; i < B.jobs.size(); ++i) {
    const BeamJob& J = B.jobs[i];
    PrologueBeam& R = pb[i];
    std::memset(&R, 0, sizeof(R));
    R.g = J.g;
    R.b = J.b;
    R.s = J.s;
    R.rho = J.rho;
    R.T = S.T + J.t_off;
    R.aabb = S.aabb + 8 * i;
    R.list_v = S.list_v + J.l_off;
    R.line_any = reinterpret_cast<unsigned char*>(S.list_v + J.f_off);
    R.zero_all = B.spectral ? 0 : 1;
  }
  return pb;
}

// Device view of the optional intermediates; all = 1 when a per-voxel output
// other than blocked/TERMA is wanted (every voxel is then evaluated).
Inter make_inter(const ch_intermediates* inter, int& all) {
  Inter in{};
  all = 0;
  if (inter) {
    in.blocked = inter->blocked;
    in.d_eff = inter->d_eff;
    in.oad = inter->oad;
    in.fluence = inter->fluence;
    in.f_soften = inter->f_soften;
    in.f_horn = inter->f_horn;
    in.terma = inter->terma;
    all = (in.d_eff || in.oad || in.fluence || in.f_soften || in.f_horn) ? 1 : 0;
  }
  return in;
}

// The device work of a batch (records already on the device): reset,
// prologues, dose zeroing, tap ranges, one persistent gather.  Only kernel
// launches and memsets, so it can be captured into a CUDA graph.  ev (4
// events, or NULL) marks the stage boundaries.
ch_status enqueue_batch(ch_plan* P, const BatchPlan& B, const Scratch& S, const ch_intermediates* inter,
                        const cudaEvent_t* ev, cudaStream_t s) {
  const int n = (int)B.jobs.size();
  int* flags = S.counters + 1;
  unsigned long long* updates = reinterpret_cast<unsigned long long*>(S.counters + 2);
  if (ev) CH_CUDA(cudaEventRecord(ev[0], s));
  launch_init_scratch(S.aabb, n, S.counters, s);
  if (inter) {
    // intermediates wanted: the per-beam prologue writes them
    for (int i = 0; i < n; ++i) {
      const BeamJob& J = B.jobs[i];
      int all = 0;
      const Inter in = make_inter(inter, all);
      launch_prologue(J.rho, J.g, J.b, J.s, S.T + J.t_off, in, all, S.aabb + 8 * i, S.list_v + J.l_off, P->n_sm,
                      flags, s, P->tuning.terma_ctas_per_sm);
      CH_CUDA(cudaGetLastError());
    }
  } else {
    // every beam's prologue in one cull and one TERMA launch (records staged)
    long long max_vox = 1, max_lines = 1;
    for (const BeamJob& J : B.jobs) {
      max_vox = std::max(max_vox, (long long)J.g.n[0] * J.g.n[1] * J.g.n[2]);
      max_lines = std::max(max_lines, (long long)J.g.n[0] * J.g.n[1]);
    }
    // counters[4]: the TERMA chunk counter (zeroed by launch_init_scratch)
    launch_prologue_batch(S.pro, n, max_vox, max_lines, P->n_sm, flags, S.counters + 4, s,
                          P->tuning.terma_ctas_per_sm);
    CH_CUDA(cudaGetLastError());
  }
  if (ev) CH_CUDA(cudaEventRecord(ev[1], s));
  if (B.spectral) {
    // FFT convolution, launch after launch in the work arena; every dose
    // voxel is written
    if (ev) CH_CUDA(cudaEventRecord(ev[2], s));
    for (const SpecPlanLaunch& l : B.spec.launches) {
      SpecLaunch L{};
      const BeamJob& J0 = B.jobs[l.pairs[0].j1];
      L.g = spec_grid(P, l.n, l.M, J0.g.zp, 0, l.shat);
      L.n_pairs = (int)l.pairs.size();
      for (int q = 0; q < L.n_pairs; ++q) {
        const SpecPlanPair& pr = l.pairs[q];
        const BeamJob& J1 = B.jobs[pr.j1];
        const BeamJob* J2 = pr.j2 >= 0 ? &B.jobs[pr.j2] : nullptr;
        // line flags exist when the batched prologue ran (no intermediates)
        const unsigned char* f1 = inter ? nullptr : reinterpret_cast<const unsigned char*>(S.list_v + J1.f_off);
        const unsigned char* f2 =
            (inter || !J2) ? nullptr : reinterpret_cast<const unsigned char*>(S.list_v + J2->f_off);
        L.p[q] = SpecPair{S.T + J1.t_off, J2 ? S.T + J2->t_off : nullptr, f1, f2, S.spec + pr.a_off,
                          S.spec + pr.b_off, J1.dose, J2 ? J2->dose : nullptr};
      }
      launch_spec_pairs(L, s);
      CH_CUDA(cudaGetLastError());
    }
    if (ev) CH_CUDA(cudaEventRecord(ev[3], s));
    return CH_OK;
  }
  for (int i = 0; i < n; ++i)
    CH_CUDA(cudaMemsetAsync(B.jobs[i].dose, 0, (size_t)B.jobs[i].g.n[0] * B.jobs[i].g.n[1] * B.jobs[i].g.n[2] * 4,
                            s));
  const ConeDirs D = cone_dirs(*B.set, P);
  launch_range(S.range_beams, n, B.max_tiles, D, s);
  CH_CUDA(cudaGetLastError());
  if (ev) CH_CUDA(cudaEventRecord(ev[2], s));
  launch_gather(S.cone_beams, n, D, B.total_units, P->n_sm, S.counters, updates, flags, s);
  CH_CUDA(cudaGetLastError());
  if (ev) CH_CUDA(cudaEventRecord(ev[3], s));
  return CH_OK;
}

ch_status run_group(ch_plan* P, int n, const ch_grid* grids, const float* const* rho, const int* swap_xy,
                    const ch_beam* beams, const ch_settings* settings, float* const* dose,
                    const ch_intermediates* inter, bool scatter, bool radiological, const StencilSet* set,
                    cudaStream_t s) {
  BatchPlan B;
  ch_status st = plan_batch(P, n, grids, rho, swap_xy, beams, settings, dose, s, B, set);
  if (st != CH_OK) return st;
  const ScratchNeed need = scratch_need(n, grids, B.U, B.spectral && !scatter);
  for (int k = 0; k < N_SCRATCH; ++k) CH_CUDA(const_cast<DevBuf*>(scratch_bufs(P, k))->ensure(need.bytes[k]));
  const Scratch S{P->T.as<float>(),          P->aabb.as<int>(),           P->counters.as<int>(),
                  P->ranges.as<uint32_t>(),  P->cranges.as<uint32_t>(),   P->cone_beams.as<ConeBeam>(),
                  P->range_beams.as<RangeBeam>(), P->list_v.as<int>(),    P->spec_work.as<float2>(),
                  P->pro_beams.as<PrologueBeam>()};
  for (auto& e : P->ev)
    if (!e) CH_CUDA(cudaEventCreate(&e));
  P->stats = ch_stats{};
  P->stats.n_unique_dirs = B.U;
  P->stats_pending = true;
  P->last_stream = s;
  if (scatter) {
    // plain path: prologues, then one per-voxel scatter launch per beam
    int* flags = S.counters + 1;
    CH_CUDA(cudaEventRecord(P->ev[0], s));
    launch_init_scratch(S.aabb, n, S.counters, s);
    for (int i = 0; i < n; ++i) {
      const BeamJob& J = B.jobs[i];
      int all = 0;
      const Inter in = make_inter(inter, all);
      launch_prologue(J.rho, J.g, J.b, J.s, S.T + J.t_off, in, all, S.aabb + 8 * i, S.list_v + J.l_off, P->n_sm,
                      flags, s,
                      P->tuning.terma_ctas_per_sm);
      CH_CUDA(cudaGetLastError());
    }
    CH_CUDA(cudaEventRecord(P->ev[1], s));
    const ConeDirs D = cone_dirs(*B.set, P);
    for (int i = 0; i < n; ++i) {
      const BeamJob& J = B.jobs[i];
      CH_CUDA(cudaMemsetAsync(J.dose, 0, (size_t)J.g.n[0] * J.g.n[1] * J.g.n[2] * 4, s));
      if (radiological)
        launch_scatter_radiological(S.T + J.t_off, J.rho, J.g.n, J.g.zp, J.g.swap_xy, B.U, D.tap_base, D.tap_len,
                                    D.offs, D.tvals, B.set->walk_row.as<int>(), B.set->walk_mult.as<int>(),
                                    P->K.as<double>(), P->n_r, J.dose, s);
      else
        launch_scatter(S.T + J.t_off, J.g.n, J.g.zp, B.U, D.tap_base, D.tap_len, D.offs, D.taps, J.dose, s);
      CH_CUDA(cudaGetLastError());
    }
    CH_CUDA(cudaEventRecord(P->ev[2], s));
    CH_CUDA(cudaEventRecord(P->ev[3], s));
    return CH_OK;
  }
  const std::vector<PrologueBeam> pb = make_prologue_records(B, S);
  std::vector<Seg> segs;
  if (!inter) segs.push_back(Seg{S.pro, pb.data(), pb.size() * sizeof(PrologueBeam)});
  std::vector<ConeBeam> cb;
  std::vector<RangeBeam> rb;
  if (!B.spectral) {
    if ((st = make_records(B, S, cb, rb)) != CH_OK) return st;
    segs.push_back(Seg{S.cone_beams, cb.data(), cb.size() * sizeof(ConeBeam)});
    segs.push_back(Seg{S.range_beams, rb.data(), rb.size() * sizeof(RangeBeam)});
  }
  if (!segs.empty() && (st = stage_records(P, segs, s)) != CH_OK) return st;
  if ((st = enqueue_batch(P, B, S, inter, P->ev, s)) != CH_OK) return st;
  P->stats.n_units = B.spectral ? 0 : B.total_units;
  return CH_OK;
}

// Beams with physics options run one at a time, each with its own stencils
// (beam-frame cones) and path (radiological distance: the scatter); plain
// beams keep the fused batch.
ch_status run(ch_plan* P, int n, const ch_grid* grids, const float* const* rho, const int* swap_xy,
              const ch_beam* beams, const ch_settings* settings, float* const* dose, const ch_intermediates* inter,
              bool scatter, cudaStream_t s) {
  bool any = false;
  for (int i = 0; i < n && settings && beams; ++i) any |= settings[i].options != 0;
  if (!any) return run_group(P, n, grids, rho, swap_xy, beams, settings, dose, inter, scatter, false, nullptr, s);
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  if (!grids) return fail(CH_ERR_INVALID_ARG, "batch arrays missing");
  CH_CUDA(cudaSetDevice(P->device));
  for (int i = 0; i < n; ++i) {
    ch_status st = check_grid(&grids[i]);
    if (st != CH_OK) return st;
    if ((st = check_settings(&settings[i])) != CH_OK) return st;
    const int opt = settings[i].options;
    StencilSet* set = nullptr;
    if (opt & CH_OPT_CONES_IN_BEAM_FRAME) {
      if ((st = frame_stencils(P, grids[i].spacing, grids[i].n, beams[i].xform, s, &set)) != CH_OK) return st;
    }
    const bool radio = (opt & CH_OPT_RADIOLOGICAL_DISTANCE) != 0;
    st = run_group(P, 1, &grids[i], rho ? &rho[i] : nullptr, swap_xy ? &swap_xy[i] : nullptr, &beams[i],
                   &settings[i], dose ? &dose[i] : nullptr, n == 1 ? inter : nullptr, scatter || radio, radio, set,
                   s);
    if (st != CH_OK) return st;
  }
  return CH_OK;
}

}  // namespace

// ------------------------------------------------------ static scratch --
// Scratch of ch_dose_static: a fixed device array, so that call allocates
// nothing.  It holds one beam's TERMA volume, the prologue voxel list, the
// tile range tables and the launch records; 36 MiB covers grids up to
// about 160^3.
// The array belongs to this library's module and stays allocated on every
// GPU that uses it until the process exits.
#define CH_STATIC_SCRATCH_BYTES (36ull << 20)
static __device__ __align__(256) unsigned char g_static_scratch[CH_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
unsigned char* g_static_ptr[kMaxDevices] = {};

// Device address of the static scratch on the current device (host code
// cannot use the array's name as a device pointer).  Looked up once per
// device, on that device's first ch_dose_static call.
ch_status static_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return fail(CH_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fail(CH_ERR_DEVICE, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    g_static_ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_static_ptr[device];
  return CH_OK;
}

inline size_t align_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

// The launch records of ch_dose_static travel as one kernel parameter (the
// launch copies it), so the call reads no host memory after it returns and
// needs neither a copy engine nor a pinned buffer.
struct StaticRecordWords {
  unsigned int w[(sizeof(ConeBeam) + sizeof(RangeBeam)) / 4];
};
static_assert(sizeof(ConeBeam) % 4 == 0 && sizeof(RangeBeam) % 4 == 0, "records are whole words");
static_assert(sizeof(StaticRecordWords) <= 16384, "the records fit the kernel parameter space");

__global__ void write_static_records(const __grid_constant__ StaticRecordWords rec, unsigned int* cone_dst,
                                     unsigned int* range_dst) {
  constexpr int NC = (int)(sizeof(ConeBeam) / 4), NR = (int)(sizeof(RangeBeam) / 4);
  for (int i = threadIdx.x; i < NC + NR; i += blockDim.x) {
    if (i < NC) cone_dst[i] = rec.w[i];
    else range_dst[i - NC] = rec.w[i];
  }
}

}  // namespace

extern "C" {

ch_status ch_plan_create(ch_plan** plan, int device) {
  if (!plan) return fail(CH_ERR_INVALID_ARG, "plan out-pointer is NULL");
  *plan = nullptr;
  int count = 0;
  CH_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(CH_ERR_INVALID_ARG, "no such CUDA device");
  CH_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  CH_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) return fail(CH_ERR_DEVICE, "conehead_gb300 needs a Blackwell (sm_10x) GPU");
  CH_CUDA(setup_cone_kernel());
  CH_CUDA(setup_spec_kernels());
  upload_unit_partials();
  CH_CUDA(cudaGetLastError());
  ch_plan* P = new ch_plan();
  P->device = device;
  P->n_sm = prop.multiProcessorCount;
  *plan = P;
  return CH_OK;
}

void ch_plan_destroy(ch_plan* plan) {
  if (!plan) return;
  cudaSetDevice(plan->device);
  delete plan;
}

ch_status ch_plan_set_kernel(ch_plan* P, const ch_kernel* k) {
  if (!P || !k || !k->cum || !k->theta || !k->phi) return fail(CH_ERR_INVALID_ARG, "kernel tables missing");
  if (P->live_batches > 0) return fail(CH_ERR_INVALID_ARG, "kernel tables cannot change while captured batches exist");
  if (k->n_phi <= 0 || k->n_r < 2 || k->n_theta <= 0 || k->n_phi > 1024 || k->n_theta > 1024)
    return fail(CH_ERR_INVALID_ARG, "kernel table sizes out of range");
  if (k->n_r < 5996) return fail(CH_ERR_INVALID_ARG, "kernel table needs 5996 radial samples (0.05..60 cm)");
  CH_CUDA(cudaSetDevice(P->device));
  // same cone directions and radial sampling: the stencils stay, only their
  // tap weights change (a spectrum switch costs one small kernel, no rebuild)
  const bool same_dirs = P->have_kernel && k->n_theta == P->n_theta && k->n_phi == P->n_phi && k->n_r == P->n_r &&
                         std::equal(k->theta, k->theta + k->n_theta, P->h_theta.begin()) &&
                         std::equal(k->phi, k->phi + k->n_phi, P->h_phi.begin());
  CH_CUDA(P->K.ensure((size_t)k->n_phi * k->n_r * sizeof(double)));
  CH_CUDA(P->theta.ensure((size_t)k->n_theta * sizeof(float)));
  CH_CUDA(P->phi.ensure((size_t)k->n_phi * sizeof(float)));
  CH_CUDA(cudaDeviceSynchronize());   // no call of this plan may still read the old tables
  CH_CUDA(cudaMemcpy(P->K.p, k->cum, (size_t)k->n_phi * k->n_r * sizeof(double), cudaMemcpyHostToDevice));
  CH_CUDA(cudaMemcpy(P->theta.p, k->theta, (size_t)k->n_theta * sizeof(float), cudaMemcpyHostToDevice));
  CH_CUDA(cudaMemcpy(P->phi.p, k->phi, (size_t)k->n_phi * sizeof(float), cudaMemcpyHostToDevice));
  P->n_phi = k->n_phi;
  P->n_r = k->n_r;
  P->n_theta = k->n_theta;
  P->h_theta.assign(k->theta, k->theta + k->n_theta);
  P->h_phi.assign(k->phi, k->phi + k->n_phi);
  P->have_kernel = true;
  if (same_dirs && P->st.valid) {
    for (StencilSet* S : {&P->st, &P->st_adj}) {
      if (!S->valid) continue;
      launch_reweight(P->K.as<double>(), P->n_r, S->n_dirs, S->tap_base.as<int>(), S->tap_len.as<int>(),
                      S->tvals.as<float>(), S->walk_row.as<int>(), S->walk_mult.as<int>(), S->taps.as<int4>(),
                      S->tap_run.as<int>(), S->runs.as<int4>(), nullptr);
      CH_CUDA(cudaGetLastError());
    }
    CH_CUDA(cudaStreamSynchronize(nullptr));
    P->reweights += 1;
  } else {
    P->st.valid = false;
    P->st_adj.valid = false;
  }
  P->frames.clear();          // beam-frame stencils are rebuilt on demand
  P->spec.clear();            // S^ follows the tap weights
  return CH_OK;
}

ch_status ch_dose(ch_plan* P, const ch_grid* grid, const float* rho, int swap_xy, const ch_beam* beam,
                  const ch_settings* settings, float* dose, void* stream) {
  return run(P, 1, grid, &rho, &swap_xy, beam, settings, &dose, nullptr, false, (cudaStream_t)stream);
}

ch_status ch_dose_ex(ch_plan* P, const ch_grid* grid, const float* rho, int swap_xy, const ch_beam* beam,
                     const ch_settings* settings, float* dose, const ch_intermediates* inter, void* stream) {
  return run(P, 1, grid, &rho, &swap_xy, beam, settings, &dose, inter, false, (cudaStream_t)stream);
}

ch_status ch_dose_batch(ch_plan* P, int n, const ch_grid* grids, const float* const* rho, const int* swap_xy,
                        const ch_beam* beams, const ch_settings* settings, float* const* dose, void* stream) {
  if (!grids || !beams || !settings) return fail(CH_ERR_INVALID_ARG, "batch arrays missing");
  return run(P, n, grids, rho, swap_xy, beams, settings, dose, nullptr, false, (cudaStream_t)stream);
}

ch_status ch_dose_scatter(ch_plan* P, const ch_grid* grid, const float* rho, int swap_xy, const ch_beam* beam,
                          const ch_settings* settings, float* dose, void* stream) {
  return run(P, 1, grid, &rho, &swap_xy, beam, settings, &dose, nullptr, true, (cudaStream_t)stream);
}

ch_status ch_dose_static(ch_plan* P, const ch_grid* grid, const float* rho, int swap_xy, const ch_beam* beam,
                         const ch_settings* settings, float* dose, void* stream) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  ch_status st;
  if ((st = check_grid(grid)) != CH_OK) return st;
  if ((st = check_beam(beam)) != CH_OK) return st;
  if ((st = check_settings(settings)) != CH_OK) return st;
  if (!rho || !dose) return fail(CH_ERR_INVALID_ARG, "density or dose pointer is NULL");
  if (swap_xy && grid->n[0] != grid->n[1]) return fail(CH_ERR_INVALID_ARG, "swap_xy needs a square x/y grid");
  if (settings->options) return fail(CH_ERR_INVALID_ARG, "ch_dose_static runs the reference physics only (options = 0)");
  // everything that allocates must already exist on the plan
  const StencilSet& S = P->st;
  bool ready = S.valid && P->counters.p;
  for (int k = 0; k < 3 && ready; ++k) ready = S.spacing[k] == grid->spacing[k] && S.cap[k] >= grid->n[k];
  if (!ready)
    return fail(CH_ERR_INVALID_ARG,
                "plan not prepared for this grid: run one ch_dose with the same voxel spacing and a grid at "
                "least this large on the plan first");
  cudaStream_t s = (cudaStream_t)stream;
  CH_CUDA(cudaSetDevice(P->device));

  // layout of the static scratch for this grid
  GridDev g{};
  for (int k = 0; k < 3; ++k) {
    g.n[k] = grid->n[k];
    g.origin[k] = grid->origin[k];
    g.spacing[k] = grid->spacing[k];
  }
  g.zp = round_up(grid->n[2], 4);
  g.swap_xy = swap_xy;
  const size_t N = (size_t)g.n[0] * g.n[1] * g.n[2];
  const int ntile[3] = {(g.n[0] + TX - 1) / TX, (g.n[1] + TY - 1) / TY, (g.n[2] + TZ - 1) / TZ};
  const int n_tiles = ntile[0] * ntile[1] * ntile[2];
  const int U = S.n_dirs;
  const int n_units = n_tiles * ((U + P->tuning.dir_group - 1) / P->tuning.dir_group);
  size_t off = 0;
  const size_t o_T = off;
  off = align_up(off + (size_t)g.n[0] * g.n[1] * g.zp * sizeof(float), 256);
  const size_t o_lv = off;
  off = align_up(off + N * sizeof(int), 256);
  const size_t o_aabb = off;
  off = align_up(off + 8 * sizeof(int), 256);
  const size_t o_r = off;
  off = align_up(off + (size_t)n_tiles * U * sizeof(uint32_t), 256);
  const size_t o_cr = off;
  off = align_up(off + (size_t)n_tiles * U * sizeof(uint32_t), 256);
  const size_t o_cb = off;
  off = align_up(off + sizeof(ConeBeam), 256);
  const size_t o_rb = off;
  off = align_up(off + sizeof(RangeBeam), 256);
  if (off > CH_STATIC_SCRATCH_BYTES)
    return fail(CH_ERR_INVALID_ARG, "grid needs " + std::to_string(off) + " bytes of scratch; the static scratch of "
                                    "ch_dose_static holds " + std::to_string(CH_STATIC_SCRATCH_BYTES) +
                                    " (grids up to about 160^3)");
  unsigned char* base = nullptr;
  if ((st = static_scratch(P->device, &base)) != CH_OK) return st;
  float* T = reinterpret_cast<float*>(base + o_T);
  int* aabb = reinterpret_cast<int*>(base + o_aabb);
  int* counters = P->counters.as<int>();
  int* flags = counters + 1;
  unsigned long long* updates = reinterpret_cast<unsigned long long*>(counters + 2);

  const BeamDev b = make_beam(*beam, *grid, settings->samples);
  const SettingsDev sd = make_settings(*settings);
  // this call records no stage events: ch_plan_stats reports zeros for it
  // rather than an earlier call's timings
  P->stats_pending = false;
  P->stats = ch_stats{};
  // aabb and the list count must start from their reset values; TERMA is
  // rewritten in full by the prologue and the range tables by range_kernel
  launch_init_scratch(aabb, 1, counters, s);
  launch_prologue(rho, g, b, sd, T, Inter{}, 0, aabb, reinterpret_cast<int*>(base + o_lv), P->n_sm, flags, s,
                  P->tuning.terma_ctas_per_sm);
  CH_CUDA(cudaGetLastError());
  CH_CUDA(cudaMemsetAsync(dose, 0, N * sizeof(float), s));

  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return fail(CH_ERR_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  ConeBeam C;
  std::memset(&C, 0, sizeof(C));
  if ((st = encode_windows(enc, C, T, g)) != CH_OK) return st;
  C.dose = dose;
  C.ranges = reinterpret_cast<uint32_t*>(base + o_r);
  C.cranges = reinterpret_cast<uint32_t*>(base + o_cr);
  for (int k = 0; k < 3; ++k) {
    C.n[k] = g.n[k];
    C.ntile[k] = ntile[k];
  }
  C.n_tiles = n_tiles;
  C.unit_begin = 0;
  C.n_units = n_units;
  RangeBeam R;
  std::memset(&R, 0, sizeof(R));
  for (int k = 0; k < 3; ++k) {
    R.n[k] = g.n[k];
    R.ntile[k] = ntile[k];
    R.origin[k] = g.origin[k];
    R.spacing[k] = g.spacing[k];
  }
  R.n_tiles = n_tiles;
  make_planes(*beam, *grid, b, R);
  R.aabb = aabb;
  R.ranges = reinterpret_cast<uint32_t*>(base + o_r);
  R.cranges = reinterpret_cast<uint32_t*>(base + o_cr);
  StaticRecordWords rec;
  std::memcpy(rec.w, &C, sizeof(C));
  std::memcpy(reinterpret_cast<unsigned char*>(rec.w) + sizeof(C), &R, sizeof(R));
  write_static_records<<<1, 256, 0, s>>>(rec, reinterpret_cast<unsigned int*>(base + o_cb),
                                         reinterpret_cast<unsigned int*>(base + o_rb));
  CH_CUDA(cudaGetLastError());
  const ConeDirs D = cone_dirs(P->st, P);
  launch_range(reinterpret_cast<const RangeBeam*>(base + o_rb), 1, n_tiles, D, s);
  CH_CUDA(cudaGetLastError());
  launch_gather(reinterpret_cast<const ConeBeam*>(base + o_cb), 1, D, n_units, P->n_sm, counters, updates, flags, s);
  CH_CUDA(cudaGetLastError());
  return CH_OK;
}

// ------------------------------------------------- cone operator, adjoint --
namespace {

GridDev grid_dev(const ch_grid& grid, int swap_xy) {
  GridDev g{};
  for (int k = 0; k < 3; ++k) {
    g.n[k] = grid.n[k];
    g.origin[k] = grid.origin[k];
    g.spacing[k] = grid.spacing[k];
  }
  g.zp = round_up(grid.n[2], 4);
  g.swap_xy = swap_xy;
  return g;
}

// Apply the cone stage to `in_dense` ([x][y][z], copied into the padded
// operator buffer): out = C in (forward stencils) or C^T in (mirrored).
// Tap ranges are cut against the nonzero box of the input (box, computed
// here into box[0..5]) and, if out_box is set, only output tiles meeting
// out_box are computed.  No frustum: the input is arbitrary.  `box` and the
// counters must have been reset (launch_init_scratch) by the caller.
ch_status cone_operator(ch_plan* P, const ch_grid& grid, const float* in_dense, float* out, bool transpose,
                        int* box, const int* out_box, cudaStream_t s, const RangeBeam* out_planes = nullptr) {
  if (spec_batch(P, 1, &grid)) {
    // spectral: C in = IFFT(FFT(in) S^), C^T in = IFFT(FFT(in) conj(S^)) (S is
    // real, so the mirrored stencil's spectrum is the conjugate); every
    // output voxel is computed
    const float2* shat = nullptr;
    ch_status st = spec_shat(P, P->st, grid.n, s, &shat);
    if (st != CH_OK) return st;
    const SpecLayout L = spec_layout(1, &grid);
    CH_CUDA(P->spec_work.ensure(L.arena * sizeof(float2)));
    const SpecPlanLaunch& l = L.launches[0];
    SpecLaunch SL{};
    SL.g = spec_grid(P, l.n, l.M, grid.n[2], transpose ? 1 : 0, shat);
    SL.n_pairs = 1;
    float2* w = P->spec_work.as<float2>();
    SL.p[0] = SpecPair{in_dense, nullptr, nullptr, nullptr, w + l.pairs[0].a_off, w + l.pairs[0].b_off, out,
                       nullptr};
    launch_spec_pairs(SL, s);
    CH_CUDA(cudaGetLastError());
    return CH_OK;
  }
  const GridDev g = grid_dev(grid, 0);
  const StencilSet& S = transpose ? P->st_adj : P->st;
  const int U = S.n_dirs;
  const ScratchNeed need = scratch_need(1, &grid, U);
  CH_CUDA(P->ranges.ensure(need.bytes[3]));
  CH_CUDA(P->cranges.ensure(need.bytes[4]));
  CH_CUDA(P->cone_beams.ensure(need.bytes[5]));
  CH_CUDA(P->range_beams.ensure(need.bytes[6]));
  CH_CUDA(P->adj_in.ensure((size_t)g.n[0] * g.n[1] * g.zp * sizeof(float)));
  int* counters = P->counters.as<int>();
  int* flags = counters + 1;
  unsigned long long* updates = reinterpret_cast<unsigned long long*>(counters + 2);
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return fail(CH_ERR_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  const int ntile[3] = {(g.n[0] + TX - 1) / TX, (g.n[1] + TY - 1) / TY, (g.n[2] + TZ - 1) / TZ};
  const int n_tiles = ntile[0] * ntile[1] * ntile[2];
  const int n_units = n_tiles * ((U + P->tuning.dir_group - 1) / P->tuning.dir_group);
  ConeBeam C;
  std::memset(&C, 0, sizeof(C));
  ch_status st = encode_windows(enc, C, P->adj_in.as<float>(), g);
  if (st != CH_OK) return st;
  C.dose = out;
  C.ranges = P->ranges.as<uint32_t>();
  C.cranges = P->cranges.as<uint32_t>();
  for (int k = 0; k < 3; ++k) {
    C.n[k] = g.n[k];
    C.ntile[k] = ntile[k];
  }
  C.n_tiles = n_tiles;
  C.unit_begin = 0;
  C.n_units = n_units;
  RangeBeam R;
  std::memset(&R, 0, sizeof(R));
  for (int k = 0; k < 3; ++k) {
    R.n[k] = g.n[k];
    R.ntile[k] = ntile[k];
    R.origin[k] = g.origin[k];
    R.spacing[k] = g.spacing[k];
  }
  R.n_tiles = n_tiles;
  R.n_planes = 0;
  R.aabb = box;
  R.out_aabb = out_box;
  R.ranges = P->ranges.as<uint32_t>();
  R.cranges = P->cranges.as<uint32_t>();
  if (out_planes) {
    R.n_out_planes = out_planes->n_planes;
    for (int j = 0; j < 4; ++j) {
      for (int k = 0; k < 3; ++k) R.opa[j][k] = out_planes->pa[j][k];
      R.opk0[j] = out_planes->pk0[j];
    }
  }
  if ((st = stage_records(P, {Seg{P->cone_beams.p, &C, sizeof(C)}, Seg{P->range_beams.p, &R, sizeof(R)}}, s)) != CH_OK)
    return st;
  // input into the padded layout the window tensor maps read
  CH_CUDA(cudaMemcpy2DAsync(P->adj_in.p, (size_t)g.zp * sizeof(float), in_dense, (size_t)g.n[2] * sizeof(float),
                            (size_t)g.n[2] * sizeof(float), (size_t)g.n[0] * g.n[1], cudaMemcpyDeviceToDevice, s));
  launch_nonzero_box(in_dense, g.n[0], g.n[1], g.n[2], box, s);
  CH_CUDA(cudaGetLastError());
  CH_CUDA(cudaMemsetAsync(out, 0, (size_t)g.n[0] * g.n[1] * g.n[2] * sizeof(float), s));
  const ConeDirs D = cone_dirs(S, P);
  launch_range(P->range_beams.as<RangeBeam>(), 1, n_tiles, D, s);
  CH_CUDA(cudaGetLastError());
  launch_gather(P->cone_beams.as<ConeBeam>(), 1, D, n_units, P->n_sm, counters, updates, flags, s);
  CH_CUDA(cudaGetLastError());
  return CH_OK;
}

ch_status check_beamlets(const ch_beamlets* bl) {
  if (!bl) return fail(CH_ERR_INVALID_ARG, "beamlet grid is NULL");
  if (bl->rows < 1 || bl->cols < 1 || (long long)bl->rows * bl->cols > CH_MAX_BEAMLETS)
    return fail(CH_ERR_INVALID_ARG, "beamlet grid must hold 1.." + std::to_string(CH_MAX_BEAMLETS) + " beamlets");
  if (bl->cell_rows < 1 || bl->cell_cols < 1 || bl->r0 < 0 || bl->c0 < 0 ||
      (long long)bl->rows * bl->cell_rows > 65536 || (long long)bl->cols * bl->cell_cols > 65536)
    return fail(CH_ERR_INVALID_ARG, "beamlet cells out of range");
  return CH_OK;
}

}  // namespace

ch_status ch_cone(ch_plan* P, const ch_grid* grid, const float* in, float* out, int transpose, void* stream) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  ch_status st = check_grid(grid);
  if (st != CH_OK) return st;
  if (!in || !out) return fail(CH_ERR_INVALID_ARG, "input or output pointer is NULL");
  if (in == out) return fail(CH_ERR_INVALID_ARG, "input and output must be different buffers");
  cudaStream_t s = (cudaStream_t)stream;
  CH_CUDA(cudaSetDevice(P->device));
  if ((st = ensure_stencils(P, grid->spacing, grid->n, s)) != CH_OK) return st;
  CH_CUDA(P->aabb.ensure(8 * sizeof(int)));
  CH_CUDA(P->counters.ensure(8 * sizeof(int)));
  launch_init_scratch(P->aabb.as<int>(), 1, P->counters.as<int>(), s);
  st = cone_operator(P, *grid, in, out, transpose != 0, P->aabb.as<int>(), nullptr, s);
  if (st != CH_OK) return st;
  P->stats_pending = false;
  return CH_OK;
}

ch_status ch_block_from_beamlets(const ch_beamlets* bl, const float* weights, float* crop, void* stream) {
  ch_status st = check_beamlets(bl);
  if (st != CH_OK) return st;
  if (!weights || !crop) return fail(CH_ERR_INVALID_ARG, "weights or crop pointer is NULL");
  BeamletDev d{bl->rows, bl->cols, bl->cell_rows, bl->cell_cols, bl->r0, bl->c0};
  launch_beamlet_fill(weights, d, crop, (cudaStream_t)stream);
  CH_CUDA(cudaGetLastError());
  return CH_OK;
}

ch_status ch_dose_adjoint(ch_plan* P, const ch_grid* grid, const float* rho, int swap_xy, const ch_beam* beam,
                          const ch_beamlets* bl, const ch_settings* settings, const float* grad_dose,
                          float* grad_weights, float* grad_terma, void* stream) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  ch_status st;
  if ((st = check_grid(grid)) != CH_OK) return st;
  if ((st = check_beam(beam)) != CH_OK) return st;
  if ((st = check_settings(settings)) != CH_OK) return st;
  if ((st = check_beamlets(bl)) != CH_OK) return st;
  if (settings->options) return fail(CH_ERR_INVALID_ARG, "the adjoint covers the reference physics only (options = 0)");
  if (!rho || !grad_dose || !grad_weights) return fail(CH_ERR_INVALID_ARG, "density or gradient pointer is NULL");
  if (swap_xy && grid->n[0] != grid->n[1]) return fail(CH_ERR_INVALID_ARG, "swap_xy needs a square x/y grid");
  if (beam->block_r0 != bl->r0 || beam->block_c0 != bl->c0 || beam->block_rows != bl->rows * bl->cell_rows ||
      beam->block_cols != bl->cols * bl->cell_cols || beam->block_uniform)
    return fail(CH_ERR_INVALID_ARG, "the beam's block crop must be the beamlet grid (ch_block_from_beamlets)");
  cudaStream_t s = (cudaStream_t)stream;
  CH_CUDA(cudaSetDevice(P->device));
  if ((st = ensure_stencils(P, grid->spacing, grid->n, s)) != CH_OK) return st;
  const GridDev g = grid_dev(*grid, swap_xy);
  const size_t N = (size_t)g.n[0] * g.n[1] * g.n[2];
  const ScratchNeed need = scratch_need(1, grid, P->st.n_dirs);
  CH_CUDA(P->T.ensure(need.bytes[0]));
  CH_CUDA(P->aabb.ensure(16 * sizeof(int)));
  CH_CUDA(P->counters.ensure(need.bytes[2]));
  CH_CUDA(P->list_v.ensure(need.bytes[7]));
  CH_CUDA(P->adj_out.ensure(N * sizeof(float)));
  CH_CUDA(P->adj_w.ensure((size_t)bl->rows * bl->cols * sizeof(double)));
  int* box = P->aabb.as<int>();          // [0..7] TERMA box + list count, [8..15] input box
  int* counters = P->counters.as<int>();
  int* flags = counters + 1;
  const BeamDev b = make_beam(*beam, *grid, settings->samples);
  const SettingsDev sd = make_settings(*settings);
  launch_init_scratch(box, 2, counters, s);
  // forward prologue: TERMA, its box and the list of voxels the beam reaches
  launch_prologue(rho, g, b, sd, P->T.as<float>(), Inter{}, 0, box, P->list_v.as<int>(), P->n_sm, flags, s, P->tuning.terma_ctas_per_sm);
  CH_CUDA(cudaGetLastError());
  // transposed cone: dL/dT = C^T dL/dD, only where TERMA is nonzero
  float* tbar = grad_terma ? grad_terma : P->adj_out.as<float>();
  RangeBeam frustum;
  std::memset(&frustum, 0, sizeof(frustum));
  make_planes(*beam, *grid, b, frustum);
  if ((st = cone_operator(P, *grid, grad_dose, tbar, true, box + 8, box, s, &frustum)) != CH_OK) return st;
  // transposed blocking and fluence: dL/dw
  CH_CUDA(cudaMemsetAsync(P->adj_w.p, 0, (size_t)bl->rows * bl->cols * sizeof(double), s));
  const BeamletDev d{bl->rows, bl->cols, bl->cell_rows, bl->cell_cols, bl->r0, bl->c0};
  CH_CUDA(launch_blocked_adjoint(g, b, d, settings->samples, P->T.as<float>(), tbar, box + 6, P->list_v.as<int>(),
                                 P->adj_w.as<double>(), P->n_sm, flags, s));
  launch_to_float(P->adj_w.as<double>(), grad_weights, bl->rows * bl->cols, s);
  CH_CUDA(cudaGetLastError());
  P->stats_pending = false;
  P->last_stream = s;
  return CH_OK;
}

// ------------------------------------------------------- captured batch --
struct ch_batch {
  ch_plan* P = nullptr;
  int n = 0;
  int total_units = 0;
  DevBuf T, aabb, counters, ranges, cranges, cone_beams, range_beams, list_v, spec_work, pro_beams;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~ch_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (DevBuf* b : {&T, &aabb, &counters, &ranges, &cranges, &cone_beams, &range_beams, &list_v, &spec_work,
                      &pro_beams})
      b->release();
  }
};

ch_status ch_batch_create(ch_plan* P, int n, const ch_grid* grids, const float* const* rho, const int* swap_xy,
                          const ch_beam* beams, const ch_settings* settings, float* const* dose, void* stream,
                          ch_batch** out) {
  if (!out) return fail(CH_ERR_INVALID_ARG, "batch out-pointer is NULL");
  *out = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  for (int i = 0; settings && i < n; ++i)
    if (settings[i].options) return fail(CH_ERR_INVALID_ARG, "captured batches run the reference physics only (options = 0)");
  BatchPlan B;
  ch_status st = plan_batch(P, n, grids, rho, swap_xy, beams, settings, dose, s, B);
  if (st != CH_OK) return st;
  std::unique_ptr<ch_batch> bt(new ch_batch());
  bt->P = P;
  bt->n = n;
  bt->total_units = B.total_units;
  const ScratchNeed need = scratch_need(n, grids, B.U, B.spectral);
  DevBuf* bufs[N_SCRATCH] = {&bt->T,          &bt->aabb,        &bt->counters, &bt->ranges,    &bt->cranges,
                             &bt->cone_beams, &bt->range_beams, &bt->list_v,   &bt->spec_work, &bt->pro_beams};
  for (int k = 0; k < N_SCRATCH; ++k) CH_CUDA(bufs[k]->ensure(need.bytes[k]));
  const Scratch S{bt->T.as<float>(),          bt->aabb.as<int>(),          bt->counters.as<int>(),
                  bt->ranges.as<uint32_t>(),  bt->cranges.as<uint32_t>(),  bt->cone_beams.as<ConeBeam>(),
                  bt->range_beams.as<RangeBeam>(), bt->list_v.as<int>(),   bt->spec_work.as<float2>(),
                  bt->pro_beams.as<PrologueBeam>()};
  CH_CUDA(cudaStreamSynchronize(s));
  {
    // the records are fixed for the batch's life: uploaded once, outside the graph
    const std::vector<PrologueBeam> pb = make_prologue_records(B, S);
    CH_CUDA(cudaMemcpy(bt->pro_beams.p, pb.data(), pb.size() * sizeof(PrologueBeam), cudaMemcpyHostToDevice));
  }
  if (!B.spectral) {
    std::vector<ConeBeam> cb;
    std::vector<RangeBeam> rb;
    if ((st = make_records(B, S, cb, rb)) != CH_OK) return st;
    // the records are fixed for the batch's life: upload them once, outside the graph
    CH_CUDA(cudaMemcpy(bt->cone_beams.p, cb.data(), n * sizeof(ConeBeam), cudaMemcpyHostToDevice));
    CH_CUDA(cudaMemcpy(bt->range_beams.p, rb.data(), n * sizeof(RangeBeam), cudaMemcpyHostToDevice));
  }
  // capture the device work on a private stream
  cudaStream_t cs;
  CH_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    return fail(CH_ERR_DEVICE, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  }
  st = enqueue_batch(P, B, S, nullptr, nullptr, cs);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);
  cudaStreamDestroy(cs);
  if (st != CH_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return fail(CH_ERR_DEVICE, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  bt->graph = g;
  CH_CUDA(cudaGraphInstantiate(&bt->exec, g, 0));
  P->live_batches += 1;
  *out = bt.release();
  return CH_OK;
}

ch_status ch_batch_launch(ch_batch* bt, void* stream) {
  if (!bt || !bt->exec) return fail(CH_ERR_INVALID_ARG, "batch is NULL");
  CH_CUDA(cudaSetDevice(bt->P->device));
  CH_CUDA(cudaGraphLaunch(bt->exec, (cudaStream_t)stream));
  return CH_OK;
}

ch_status ch_batch_sync(ch_batch* bt, void* stream) {
  if (!bt) return fail(CH_ERR_INVALID_ARG, "batch is NULL");
  CH_CUDA(cudaSetDevice(bt->P->device));
  CH_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  int c[2];
  CH_CUDA(cudaMemcpy(c, bt->counters.p, sizeof(c), cudaMemcpyDeviceToHost));
  if (c[1] & FLAG_TIMEOUT) return fail(CH_ERR_TIMEOUT, "a bounded device wait expired in the cone stage");
  if (c[1] & FLAG_PARALLEL_RAY) return fail(CH_ERR_PARALLEL_RAY, "no intersection or line is within plane");
  return CH_OK;
}

void ch_batch_destroy(ch_batch* bt) {
  if (!bt) return;
  cudaSetDevice(bt->P->device);
  cudaDeviceSynchronize();      // no replay may still be reading the batch's buffers
  bt->P->live_batches -= 1;
  delete bt;
}

ch_status ch_block_from_mlc(const ch_mlc* m, float* out, int rows, int cols, int r0, int c0, void* stream) {
  if (!m || !out) return fail(CH_ERR_INVALID_ARG, "MLC table or output is NULL");
  if (rows < 1 || cols < 1 || rows > 65535) return fail(CH_ERR_INVALID_ARG, "window must be 1..65535 rows and >= 1 column");
  if (m->n_pairs < 1 || m->n_pairs > CH_MAX_LEAF_PAIRS)
    return fail(CH_ERR_INVALID_ARG, "n_pairs out of range (1.." + std::to_string(CH_MAX_LEAF_PAIRS) + ")");
  if (m->map_rows < 1 || m->map_cols < CH_MLC_TIP_CELLS + 1)
    return fail(CH_ERR_INVALID_ARG, "map size out of range");
  int prev_end = 0;
  for (int n = 0; n < m->n_pairs; ++n) {
    const std::string leaf = "leaf pair " + std::to_string(n) + ": ";
    if (m->rows[n] < 3) return fail(CH_ERR_INVALID_ARG, leaf + "fewer than 3 rows");
    if (m->row0[n] < prev_end) return fail(CH_ERR_INVALID_ARG, leaf + "rows overlap the previous pair or start below 0");
    if ((long long)m->row0[n] + m->rows[n] > m->map_rows) return fail(CH_ERR_INVALID_ARG, leaf + "rows run past the map");
    if (m->a_end[n] < CH_MLC_TIP_CELLS || m->a_end[n] > m->map_cols)
      return fail(CH_ERR_INVALID_ARG, leaf + "bank A leaf shorter than its 15-cell tip or past the map");
    if (m->b_start[n] < 0 || m->b_start[n] > m->map_cols - 1 - CH_MLC_TIP_CELLS)
      return fail(CH_ERR_INVALID_ARG, leaf + "bank B leaf shorter than its 15-cell tip or past the map");
    prev_end = m->row0[n] + m->rows[n];
  }
  if (m->open_r0 < 0 || m->open_r1 > m->map_rows || m->open_c0 < 0 || m->open_c1 > m->map_cols)
    return fail(CH_ERR_INVALID_ARG, "jaw opening lies outside the map");
  for (int k = 0; k < CH_MLC_TIP_CELLS; ++k)
    if (!std::isfinite(m->tip[k])) return fail(CH_ERR_INVALID_ARG, "leaf tip ramp is not finite");
  launch_mlc_raster(*m, out, rows, cols, r0, c0, (cudaStream_t)stream);
  CH_CUDA(cudaGetLastError());
  return CH_OK;
}

ch_status ch_dda_trace(const ch_grid* grid, int n_rays, const int* starts, const float* dirs, int cap, int* vox,
                       float* t, int* len, void* stream) {
  ch_status st = check_grid(grid);
  if (st != CH_OK) return st;
  if (n_rays <= 0 || cap < 0 || !starts || !dirs || !len || (cap > 0 && (!vox || !t)))
    return fail(CH_ERR_INVALID_ARG, "bad DDA trace arguments");
  launch_dda_trace(grid->n, grid->spacing, n_rays, starts, dirs, cap, vox, t, len, (cudaStream_t)stream);
  CH_CUDA(cudaGetLastError());
  return CH_OK;
}

ch_status ch_cone_directions(ch_plan* P, float* out, void* stream) {
  if (!P || !out) return fail(CH_ERR_INVALID_ARG, "plan or output is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  if (!P->st.valid) {
    const float sp[3] = {1.0f, 1.0f, 1.0f};
    const int dims[3] = {2, 2, 2};
    ch_status st = ensure_stencils(P, sp, dims, (cudaStream_t)stream);
    if (st != CH_OK) return st;
  }
  CH_CUDA(cudaMemcpyAsync(out, P->st.raw_dirs.p, (size_t)P->st.n_raw * 3 * sizeof(float),
                          cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return CH_OK;
}

ch_status ch_plan_set_tuning(ch_plan* P, const ch_tuning* t) {
  if (!P || !t) return fail(CH_ERR_INVALID_ARG, "plan or tuning is NULL");
  // (captured batches keep the schedule they were captured with)
  if (t->dir_group < 1 || t->dir_group > MAX_DIR_GROUP)
    return fail(CH_ERR_INVALID_ARG, "dir_group out of range (1.." + std::to_string(MAX_DIR_GROUP) + ")");
  if (t->unit_order != 0 && t->unit_order != 1) return fail(CH_ERR_INVALID_ARG, "unit_order must be 0 or 1");
  if (t->terma_ctas_per_sm < 1 || t->terma_ctas_per_sm > 32)
    return fail(CH_ERR_INVALID_ARG, "terma_ctas_per_sm out of range (1..32)");
  if (t->cone_method != CH_CONE_SPECTRAL && t->cone_method != CH_CONE_GATHER)
    return fail(CH_ERR_INVALID_ARG, "cone_method must be CH_CONE_SPECTRAL or CH_CONE_GATHER");
  P->tuning = *t;
  return CH_OK;
}

ch_status ch_plan_get_tuning(ch_plan* P, ch_tuning* t) {
  if (!P || !t) return fail(CH_ERR_INVALID_ARG, "plan or tuning is NULL");
  *t = P->tuning;
  return CH_OK;
}

ch_status ch_plan_prepare(ch_plan* P, const ch_grid* grid, void* stream) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (!P->have_kernel) return fail(CH_ERR_NO_KERNEL, "ch_plan_set_kernel has not been called");
  ch_status st = check_grid(grid);
  if (st != CH_OK) return st;
  CH_CUDA(cudaSetDevice(P->device));
  st = ensure_stencils(P, grid->spacing, grid->n, (cudaStream_t)stream);
  if (st != CH_OK || !spec_batch(P, 1, grid)) return st;
  const float2* shat = nullptr;
  return spec_shat(P, P->st, grid->n, (cudaStream_t)stream, &shat);
}

ch_status ch_plan_memory(ch_plan* P, size_t* tables, size_t* scratch) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  size_t b = P->K.bytes + P->theta.bytes + P->phi.bytes;
  for (const StencilSet* S : {&P->st, &P->st_adj}) b += S->bytes();
  for (const auto& e : P->spec) b += e->shat.bytes;
  b += P->spec_tw.bytes;
  for (const auto& f : P->frames)
    for (const StencilSet* S : {&f->fwd, &f->adj}) b += S->bytes();
  size_t a = P->adj_in.bytes + P->adj_out.bytes + P->adj_w.bytes;
  for (int k = 0; k < N_SCRATCH; ++k) a += scratch_bufs(P, k)->bytes;
  if (tables) *tables = b;
  if (scratch) *scratch = a;
  return CH_OK;
}

ch_status ch_batch_scratch_bytes(ch_plan* P, int n, const ch_grid* grids, size_t* growth, size_t* total) {
  if (!P || !grids || n <= 0) return fail(CH_ERR_INVALID_ARG, "plan, grids or count missing");
  for (int i = 0; i < n; ++i) {
    ch_status st = check_grid(&grids[i]);
    if (st != CH_OK) return st;
  }
  const int U = P->st.valid ? P->st.n_dirs : P->n_theta * P->n_phi > 0 ? P->n_theta * P->n_phi : 576;
  const ScratchNeed need = scratch_need(n, grids, U, spec_batch(P, n, grids));
  size_t g = 0, t = 0;
  for (int k = 0; k < N_SCRATCH; ++k) {
    const size_t cur = scratch_bufs(P, k)->bytes;
    t += need.bytes[k];
    if (need.bytes[k] > cur) g += need.bytes[k] - cur;
  }
  if (growth) *growth = g;
  if (total) *total = t;
  return CH_OK;
}

ch_status ch_plan_trim(ch_plan* P) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  CH_CUDA(cudaSetDevice(P->device));
  // cudaFree waits for the device, so no call of this plan is still reading the arena
  for (DevBuf* b : {&P->T, &P->aabb, &P->counters, &P->ranges, &P->cranges, &P->cone_beams, &P->range_beams,
                    &P->list_v, &P->spec_work, &P->pro_beams, &P->adj_in, &P->adj_out, &P->adj_w})
    b->release();
  P->stats_pending = false;
  return CH_OK;
}

ch_status ch_plan_set_wait_limit(ch_plan* P, long long iterations, int withhold) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  if (P->live_batches > 0) return fail(CH_ERR_INVALID_ARG, "the wait limit cannot change while captured batches exist");
  if (withhold != 0 && withhold != CH_WITHHOLD_WINDOWS && withhold != CH_WITHHOLD_SLOTS)
    return fail(CH_ERR_INVALID_ARG, "withhold must be 0, CH_WITHHOLD_WINDOWS or CH_WITHHOLD_SLOTS");
  P->wait_limit = iterations > 0 ? iterations : 0;
  P->withhold = withhold;
  return CH_OK;
}

ch_status ch_plan_sync(ch_plan* P, void* stream) {
  if (!P) return fail(CH_ERR_INVALID_ARG, "plan is NULL");
  CH_CUDA(cudaSetDevice(P->device));
  CH_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (!P->counters.p) return CH_OK;
  int c[4];
  CH_CUDA(cudaMemcpy(c, P->counters.p, sizeof(c), cudaMemcpyDeviceToHost));
  const int flags = c[1];
  if (flags & FLAG_TIMEOUT) return fail(CH_ERR_TIMEOUT, "a bounded device wait expired in the cone stage");
  if (flags & FLAG_PARALLEL_RAY) return fail(CH_ERR_PARALLEL_RAY, "no intersection or line is within plane");
  return CH_OK;
}

ch_status ch_plan_stats(ch_plan* P, ch_stats* out) {
  if (!P || !out) return fail(CH_ERR_INVALID_ARG, "plan or output is NULL");
  CH_CUDA(cudaSetDevice(P->device));
  if (P->stats_pending) {
    CH_CUDA(cudaEventSynchronize(P->ev[3]));
    CH_CUDA(cudaEventElapsedTime(&P->stats.ms_prologue, P->ev[0], P->ev[1]));
    CH_CUDA(cudaEventElapsedTime(&P->stats.ms_range, P->ev[1], P->ev[2]));
    CH_CUDA(cudaEventElapsedTime(&P->stats.ms_cone, P->ev[2], P->ev[3]));
    int c[4];
    CH_CUDA(cudaMemcpy(c, P->counters.p, sizeof(c), cudaMemcpyDeviceToHost));
    unsigned long long u;
    std::memcpy(&u, c + 2, sizeof(u));
    P->stats.updates = (double)u;
    P->stats_pending = false;
  }
  *out = P->stats;
  return CH_OK;
}

const char* ch_status_string(ch_status s) {
  switch (s) {
    case CH_OK: return "ok";
    case CH_ERR_INVALID_ARG: return "invalid argument";
    case CH_ERR_OOM: return "out of device memory";
    case CH_ERR_DEVICE: return "CUDA error";
    case CH_ERR_TIMEOUT: return "device wait timed out";
    case CH_ERR_PARALLEL_RAY: return "ray parallel to the blocking plane";
    case CH_ERR_NO_KERNEL: return "kernel tables not set";
  }
  return "unknown status";
}

const char* ch_last_error(void) { return g_last_error.c_str(); }

int ch_version(void) { return 1; }

}  // extern "C"
