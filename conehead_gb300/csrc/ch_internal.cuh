// Internal definitions shared by the conehead_gb300 CUDA sources.
#pragma once

#include <cstdint>
#include <vector>
#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/conehead_gb300.h"

namespace ch {

// ------------------------------------------------------------------ sizes --
// Cone gather tile: 16 (x) x 16 (y) x 16 (z) outputs.  The 16 outputs of a
// tile line along the "run axis" of the walks being summed (x or y, chosen
// per walk on the host) are split between OUT_SPLIT consumer warps, each
// thread holding 16 / OUT_SPLIT of them in registers:
//   run axis x: half a warp covers 16 consecutive z of one y row, the other
//     half the same z two rows further (y + 2); 8 warps cover the 16 rows;
//   run axis y: half a warp covers 16 consecutive z of one x slice, the other
//     half the next slice (x + 1); 8 warps cover the 16 slices.
// More warps hide more shared-memory latency; every warp reads the run
// records and its own line ends.
constexpr int TZ = 16, TY = 16, TX = 16;
constexpr int TILE_VOX = TZ * TY * TX;
#ifndef CH_OUT_SPLIT
#define CH_OUT_SPLIT 2
#endif
constexpr int OUT_SPLIT = CH_OUT_SPLIT;
constexpr int OUT_PER_THREAD = 16 / OUT_SPLIT;
// A run is up to RUN_MAX consecutive taps of one walk whose steps all lie
// along the walk's run axis: its n taps read one line of 15 + n window values
// along that axis, so a thread loads each value once for up to n taps.
constexpr int RUN_MAX = 4;
// Shared-memory window of a chunk: [x][row][z] with z pitch P and `rows` y
// rows per x slice.  Three shapes ("variants") trade z reach for x and y reach
// in one fixed slot; the chunker picks the cheapest that holds the chunk.
// Every P is 8 mod 16, so 2P = 16 mod 32: the half-warps of the x layout
// (rows y and y + 2) hit disjoint banks.  Every `rows` is 2 mod 4, so the
// slice pitch rows * P is 16 mod 32: the half-warps of the y layout (slices x
// and x + 1) hit disjoint banks too.
constexpr int N_VARIANTS = 3;
__host__ __device__ constexpr int var_p(int v) { return v == 0 ? 24 : (v == 1 ? 40 : 56); }
__host__ __device__ constexpr int var_rows(int v) { return v == 0 ? 34 : (v == 1 ? 26 : 22); }
static_assert((2 * var_p(0)) % 32 == 16 && (2 * var_p(1)) % 32 == 16 && (2 * var_p(2)) % 32 == 16,
              "x layout: rows y and y + 2 must fall in disjoint banks");
static_assert((var_rows(0) * var_p(0)) % 32 == 16 && (var_rows(1) * var_p(1)) % 32 == 16 &&
                  (var_rows(2) * var_p(2)) % 32 == 16,
              "y layout: slices x and x + 1 must fall in disjoint banks");
constexpr int WIN_FLOATS = 27648;     // one pipeline slot (108 KiB)
__host__ __device__ constexpr int var_max_ex(int v) { return WIN_FLOATS / (var_p(v) * var_rows(v)); }
// largest tap-offset spread a chunk may have along each axis in variant v
// (z also absorbs the 4-float TMA alignment of the window origin)
__host__ __device__ constexpr int var_span_z(int v) { return var_p(v) - TZ - 3; }
__host__ __device__ constexpr int var_span_y(int v) { return var_rows(v) - TY; }
__host__ __device__ constexpr int var_span_x(int v) { return var_max_ex(v) - TX; }
// One TMA box loads a chunk's whole window: P x rows x ex floats, so every
// (variant, x extent) pair has its own tensor map.
__host__ __device__ constexpr int n_maps_before(int v) {
  return v == 0 ? 0 : (v == 1 ? var_max_ex(0) - TX + 1 : (var_max_ex(0) - TX + 1) + (var_max_ex(1) - TX + 1));
}
constexpr int N_TMAPS = n_maps_before(2) + (var_max_ex(2) - TX + 1);
__host__ __device__ constexpr int tmap_index(int v, int ex) { return n_maps_before(v) + (ex - TX); }
// Run record, two int4: {window offset of the run's base in its chunk's
// variant, n, w0, w1} and {w2, w3, 0, 0} (float bits).  The base is the tap
// furthest along the run axis; weight slot c belongs to the tap c steps
// behind it, which reads line value i + c for output i.
constexpr int RUN_REC_INT4 = 2;
constexpr int MAX_CHUNK_RUNS = 64;    // runs per chunk (their records are staged with the window)
constexpr int N_SLOTS = 2;
constexpr int CONE_CONSUMER_WARPS = (TY / 2) * OUT_SPLIT;
constexpr int CONE_THREADS = (CONE_CONSUMER_WARPS + 1) * 32;
constexpr int DIR_GROUP = 16;         // unique directions per work unit (default; ch_tuning.dir_group)
constexpr int MAX_DIR_GROUP = 1024;   // the producer walks a unit's directions 32 at a time

// Bounded device-side waits: try_wait iterations of an mbarrier wait before
// the gather gives up (its pipeline waits may be given a smaller bound per
// plan, ch_plan_set_wait_limit; the wait for its own copies in flight always
// has this one).
constexpr long long MBAR_LIMIT = 1ll << 22;

// device error flags (bit mask in Plan::d_flags[0])
constexpr int FLAG_TIMEOUT = 1;
constexpr int FLAG_PARALLEL_RAY = 2;
constexpr int FLAG_BAD_INDEX = 4;

// ---------------------------------------------------------- beam constants --
// Everything the per-voxel prologue needs about one beam, prepared on the
// host (float64 values mirrored from the reference's arrays, float32
// approximations for the fast blocking test).
struct BeamDev {
  // exact mirror inputs
  double src[3], vy[3], m0[3], m2[3];   // m0/m2: transform rows 0 and 2
  double vyw;                           // v_y . float32(src), reference order
  float srcf[3], vyf[3], m0f[3], m2f[3], vywf;  // float32 copies (geom_f32 path)
  int geom_f32;
  // fast approximate projection: xb ~ c0 + si * (m0.S - m0.p), si = K / (n.S - n.p)
  float a_c0, a_c2, a_m0S, a_m2S, a_nS, a_K;
  // cull box in beam coordinates (cm) for voxel centres (inclusive)
  float cx_lo, cx_hi, cz_lo, cz_hi;
  float cull_margin_k;   // margin = k * SAD/depth
  int cull_enable;
  // block crop
  const float* block;
  int brows, bcols, br0, bc0, full_rows, full_cols;
  int uniform;          // every crop value is 1.0
  // fluence / TERMA
  double sad;
  int sad_f32;
};

struct SettingsDev {
  float sPri, sAnn, zAnn, rInner, rOuter, zExp, sExp, kExp;
  float softRatio, softLimit, hornRatio;
  int samples;
  int n_energy;
  float E[CH_MAX_ENERGY], w[CH_MAX_ENERGY], mu[CH_MAX_ENERGY];
};

struct GridDev {
  int n[3];
  float origin[3];
  float spacing[3];
  int zp;             // padded z pitch of the internal TERMA volume
  int swap_xy;
};

// ------------------------------------------------------------ exact math --
// Reference arithmetic without FMA contraction (round after every op).
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float d2f(double a) { return __double2float_rn(a); }

// voxel centre: float32 store of f64(origin) + f64(spacing) * i.  The float64
// value is exact for any realistic grid, so one fused rounding equals it.
__device__ __forceinline__ float voxel_centre(float origin, float spacing, int i) {
  return __fmaf_rn(spacing, (float)i, origin);
}

// DDA initial t and increment for one axis (reference cuda_dda_3d):
// t0 = f32(f64(s/2) / f64(|d|)) == fdiv(s/2, |d|) (double rounding through
// float64 is innocuous for float32 operands), dt = s / |d| in float32.
__device__ __forceinline__ void dda_axis(float d, float s, int& step, float& t, float& dt) {
  step = d < 0.0f ? -1 : 1;
  float a = d < 0.0f ? -d : d;
  if (a == 0.0f) {
    t = 1000000000.0f;
    dt = 1000000000.0f;
  } else {
    t = fdiv(s * 0.5f, a);
    dt = fdiv(s, a);
  }
}

__device__ __forceinline__ int dda_pick(const float* t) {
  return (t[0] < t[1]) ? ((t[0] < t[2]) ? 0 : 2) : ((t[1] < t[2]) ? 1 : 2);
}

// ----------------------------------------------------- cone stage structs --
constexpr uint32_t RANGE_EMPTY = 0xffffffffu;

struct __align__(128) ConeBeam {
  CUtensorMap tmap[N_TMAPS];  // TERMA volume (dims nz, ny, nx; pitch zp), box P x rows x ex per map
  float* dose;
  const uint32_t* ranges; // [n_tiles][n_dirs]
  const uint32_t* cranges;
  int n[3];
  int ntile[3];
  int n_tiles;
  int unit_begin;
  int n_units;
  int pad[1];
};
static_assert(sizeof(ConeBeam) % 128 == 0, "ConeBeam must keep tensor maps aligned");

struct ConeDirs {
  int n_dirs;
  const int* tap_base;
  const int* tap_len;
  const int4* taps;        // window offset of O[m] in variants 0..2, float bits of w[m] (scatter path)
  const short4* offs;      // O[m] (x, y, z, step axis)
  const float* tvals;      // exit t of tap m
  const int4* runs;        // RUN_REC_INT4 per run, the runs of all walks back to back
  const int* run_base;     // first run of each walk
  const int* tap_run;      // per tap: its global run index * 8 + 2 + its weight slot (the word of its weight)
  const int* run_tap;      // per run: global index of its first tap (one trailing entry)
  const int* axis;         // per walk: run axis, 0 = x, 1 = y
  const int* chunk_base;
  const int* n_chunks;
  const int* chunk_start;  // first run of each chunk (walk-local)
  const int4* chunk_rec;   // 2 per chunk: {first run, last run, variant, span_x | span_y << 16},
                           //              {max O_x, max O_y, max O_z, 0} over the chunk's taps
  const float* dirs;       // unit direction (x, y, z)
  int group;               // unique directions per work unit (1..MAX_DIR_GROUP)
  int order;               // units: 0 = tile outer, group inner; 1 = group outer, tile inner
  long long wait_limit;    // try_wait iterations of a pipeline wait before the gather gives up
  int withhold;            // test hook: 0 = off; CH_WITHHOLD_WINDOWS / CH_WITHHOLD_SLOTS (the
                           // producer issues no window / the consumers free no slot)
};

struct RangeBeam {
  int n[3], ntile[3], n_tiles;
  float origin[3], spacing[3];
  int n_planes;
  float pa[4][3];
  float pk0[4];
  const int* aabb;          // box of the nonzero input (lo/hi pairs per axis)
  const int* out_aabb;      // if set, output tiles outside this box get no taps
  int n_out_planes;         // output tiles wholly outside one of these planes
  float opa[4][3];          // (the beam frustum, for the transposed cone of
  float opk0[4];            // the adjoint) get no taps either
  uint32_t* ranges;        // [n_tiles][n_dirs]: first | last run << 16 (walk-local), or RANGE_EMPTY
  uint32_t* cranges;       // [n_tiles][n_dirs]: first | last chunk << 16 (walk-local)
};

// Regular beamlet grid on the block map: beamlet (i, j) covers map rows
// r0 + i*cell_rows .. + cell_rows and columns c0 + j*cell_cols .. + cell_cols.
struct BeamletDev {
  int rows, cols, cell_rows, cell_cols, r0, c0;
};

struct Inter {
  double* blocked;
  float *d_eff, *oad, *fluence, *f_soften, *f_horn, *terma;
};

// ---------------------------------------------------- spectral cone stage --
// The cone stage as one circular convolution per grid shape (spectral.cu):
// periods M_k = the smallest 2^a or 3 * 2^a >= 2 n_k - 1 (at least
// SPEC_MIN_PERIOD), pairs of beams per complex transform.
constexpr int SPEC_THREADS = 256;
constexpr int SPEC_CTAS_PER_SM = 3;       // register budget of the passes (85 per thread)
constexpr int SPEC_ELEMS = 4096;          // complex values per CTA: 4096 / M lines of period M
constexpr int SPEC_MIN_PERIOD = 16, SPEC_MAX_PERIOD = 4096;
constexpr int SPEC_MAX_PAIRS = 16;        // beam pairs per launch (their work buffers coexist)
constexpr int SPEC_SMEM = 2 * SPEC_ELEMS * 8;   // two ping-pong buffers of float2 per CTA
struct SpecPair {
  const float* t1;   // TERMA of the first beam [nx][ny][zp]
  const float* t2;   // of the second (NULL: none)
  const unsigned char* l1;  // lines of t1 that may be nonzero (NULL: every line is read)
  const unsigned char* l2;  // of t2
  float2* a;         // [nx][ny][Mz]
  float2* b;         // [nx][My][Mz]
  float* d1;         // dose of the first beam [nx][ny][nz]
  float* d2;         // of the second (NULL: none)
};
struct SpecGrid {
  int n[3], M[3];
  int logL[3];             // log2 of the lines per CTA of the pass along x, y, z
  int zp;                  // z pitch of the TERMA volumes
  int conj;                // multiply by conj(S^): the transposed cone
  const float2* tw[3];     // twiddles exp(-2 pi i k / M_axis)
  const float2* shat;      // S^ [Mx][My][Mz], 1/(Mx My Mz) folded in; [Mz][My][Mx] on the plane path
  int plane;               // the plane path (spec_plane_path): A = [Mz][lp] plane-major, no B
  int lp;                  // plane pitch of A on the plane path (nx ny rounded up to 32)
};
struct SpecLaunch {
  SpecGrid g;
  int n_pairs;
  SpecPair p[SPEC_MAX_PAIRS];
};
int spec_period(int n);                  // 0 when no period up to SPEC_MAX_PERIOD holds 2n - 1
int spec_lines_log2(int M);
int spec_pass_lines_log2(int M, int Mz);
std::vector<float2> spec_twiddles();      // every period (ascending), back to back
size_t spec_twiddle_offset(int M);
cudaError_t setup_spec_kernels();        // allow SPEC_SMEM of dynamic shared memory
void launch_spec_pairs(const SpecLaunch& L, cudaStream_t st);
// The plane path: periods of 256 on every axis (grids of 97 to 128 voxels
// per axis).  z forward into plane-major A[kz][x y], one cluster of two CTAs
// per (pair, kz) plane for the y and x transforms, the S^ product and their
// inverses (the plane's spectrum held in the pair's shared memory), z
// inverse from A.  S^ is then kept as [Mz][My][Mx].
constexpr int SPEC_PLANE_M = 256;
// half the plane spectrum, an exchange buffer per warp, the twiddle table
constexpr int SPEC_PLANE_SMEM = (128 * 128 + 16 * 2 * 256 + 16 * 18) * 8;
inline bool spec_plane_path(const int* M) {
  return M[0] == SPEC_PLANE_M && M[1] == SPEC_PLANE_M && M[2] == SPEC_PLANE_M;
}
inline int spec_plane_pitch(const int* n) { return (n[0] * n[1] + 31) / 32 * 32; }
// S^ [Mx][My][Mz] -> [Mz][My][Mx]
void launch_spec_transpose(const float2* in, float2* out, int Mx, int My, int Mz, cudaStream_t st);
// S^ of one grid shape: scatter the stencil values into the real volume
// s_real (zeroed, [Mx][My][Mz] = L.p[0].t1), then three forward passes
// (L.g.n = M, L.p[0].a = work, L.p[0].b = S^)
void launch_spec_build(const SpecLaunch& L, const long long* idx, const float* val, int n_val, float* s_real,
                       cudaStream_t st);

// One beam of a batched prologue (device record).
struct PrologueBeam {
  GridDev g;
  BeamDev b;
  SettingsDev s;
  const float* rho;
  float* T;          // [nx][ny][zp]
  int* aabb;         // 8 ints: TERMA box, list count at [6]
  int* list_v;       // this beam's voxel list (nx ny nz entries)
  unsigned char* line_any;  // per (x, y) line: 1 when the line holds a listed voxel
  int zero_all;      // 1: zero TERMA on every line (the gather reads it anywhere);
                     // 0: only on lines with listed voxels (the spectral path reads line_any)
};

// ------------------------------------------------------------ launchers --
void upload_unit_partials();
// work: a zeroed int, the TERMA launch's chunk counter
void launch_prologue_batch(const PrologueBeam* recs, int n_beams, long long max_voxels, long long max_lines,
                           int n_sm, int* flags, int* work, cudaStream_t st, int ctas_per_sm);
void launch_prologue(const float* rho, const GridDev& g, const BeamDev& b, const SettingsDev& s, float* T,
                     const Inter& inter, int all_voxels, int* aabb, int* list_v, int n_sm, int* flags,
                     cudaStream_t st, int ctas_per_sm = 8);
// Frame of the cone directions: off = the room frame (the reference), on =
// rotated by a beam's world->beam matrix m (row major, xform of ch_beam).
struct ConeFrame {
  int on;
  double m[9];
};
void launch_stencil(const float* theta, int n_theta, const float* phi, int n_phi, const double* K, int n_r,
                    const float* spacing, const int* cap, int max_len, short4* off, float* t, float* dk,
                    int* len, float* dirs, const ConeFrame& frame, cudaStream_t st);
void launch_scatter_radiological(const float* T, const float* rho, const int* n, int zp, int swap_xy, int n_dirs,
                                 const int* tap_base, const int* tap_len, const short4* offs, const float* tvals,
                                 const int* walk_row, const int* walk_mult, const double* K, int n_r, float* dose,
                                 cudaStream_t st);
void launch_reweight(const double* K, int n_r, int n_walks, const int* tap_base, const int* tap_len,
                     const float* tvals, const int* walk_row, const int* walk_mult, int4* taps, const int* tap_run,
                     int4* runs, cudaStream_t st);
void launch_dda_trace(const int* n, const float* sp, int n_rays, const int* starts, const float* dirs, int cap,
                      int* vox, float* t, int* len, cudaStream_t st);
void launch_scatter(const float* T, const int* n, int zp, int n_dirs, const int* tap_base, const int* tap_len,
                    const short4* offs, const int4* taps, float* dose, cudaStream_t st);
size_t cone_smem_bytes();
cudaError_t setup_cone_kernel();
void launch_range(const RangeBeam* rbs_dev, int n_beams, int max_tiles, const ConeDirs& D, cudaStream_t st);
void launch_gather(const ConeBeam* beams_dev, int n_beams, const ConeDirs& D, int total_units, int n_ctas,
                   int* unit_counter, unsigned long long* updates, int* flags, cudaStream_t st);
void launch_init_scratch(int* aabb, int n_beams, int* counters, cudaStream_t st);
void launch_mlc_raster(const ch_mlc& m, float* out, int rows, int cols, int r0, int c0, cudaStream_t st);
void launch_nonzero_box(const float* x, int n0, int n1, int n2, int* box, cudaStream_t st);
void launch_beamlet_fill(const float* w, const BeamletDev& bl, float* crop, cudaStream_t st);
void launch_to_float(const double* in, float* out, int n, cudaStream_t st);
cudaError_t launch_blocked_adjoint(const GridDev& g, const BeamDev& b, const BeamletDev& bl, int S, const float* T,
                                   const float* tbar, const int* list_count, const int* list_v, double* wbar,
                                   int n_sm, int* flags, cudaStream_t st);

}  // namespace ch
