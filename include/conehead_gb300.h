/*
 * conehead_gb300 -- C ABI of the GB300 collapsed-cone dose engine.
 *
 * Plain C types only: grids, beams and settings are small structs of
 * numbers; volumes are raw device pointers (float32, C order [x][y][z],
 * z fastest, exactly the layout of the reference's numpy arrays); the
 * stream argument is a cudaStream_t passed as void*.  Every call returns a
 * ch_status; ch_last_error() gives a one-line message for the last failure
 * on the calling thread.
 *
 * Reference interfaces replaced (samuelpeet/conehead):
 *   ch_dose / ch_dose_ex  <- Conehead.calculate, conehead/conehead.py:522-738
 *                            (cuda_hit_test :71-120, cuda_d_eff :209-254,
 *                             cuda_oad :286-314, cuda_fluence :320-360,
 *                             softening/horn :641-655, cuda_terma :364-377,
 *                             cuda_dose :385-488)
 *   ch_plan_set_kernel    <- the polyenergetic kernel build,
 *                            conehead/conehead.py:685-706 (host tables in,
 *                            per-direction stencils built on the device)
 *   ch_dose_batch         <- a loop of Conehead.calculate calls, one launch
 *   ch_dose_scatter       <- cuda_dose's per-voxel scatter with float32
 *                            atomics, conehead/conehead.py:385-488 (kept as
 *                            the plain one-beam-per-launch GPU path)
 *   ch_dda_trace          <- cuda_dda_3d, conehead/conehead.py:123-206
 *                            (test hook for bit-exact DDA sequences)
 */
#ifndef CONEHEAD_GB300_H
#define CONEHEAD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CH_MAX_ENERGY 32

typedef enum {
  CH_OK = 0,
  CH_ERR_INVALID_ARG = 1,   /* bad sizes, null pointers, unsupported layout */
  CH_ERR_OOM = 2,           /* device allocation failed */
  CH_ERR_DEVICE = 3,        /* CUDA runtime error */
  CH_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
  CH_ERR_PARALLEL_RAY = 5,  /* a ray is parallel to the blocking plane
                               (the reference raises RuntimeError) */
  CH_ERR_NO_KERNEL = 6      /* ch_plan_set_kernel was not called */
} ch_status;

/* Dose grid: voxel centres at origin + spacing * index (cm). */
typedef struct {
  int n[3];
  float origin[3];
  float spacing[3];
} ch_grid;

/* One beam.  Geometry is given in float64 (float32 values convert
 * exactly); geom_f32 = 1 when the source's position/v_y/transform are
 * float32 arrays (a Source whose angles were never set), which changes the
 * arithmetic the reference performs.  The block map may be cropped:
 * `block` holds rows [block_r0, block_r0 + block_rows) and columns
 * [block_c0, block_c0 + block_cols) of a full_rows x full_cols map that is
 * zero outside the crop. */
typedef struct {
  double src[3];        /* source.position (cm) */
  double vy[3];         /* source.v_y, blocking-plane normal */
  double xform[9];      /* source.transform, row major */
  double sad;           /* source.sad */
  int geom_f32;
  int sad_f32;          /* 1 when source.sad is a float32 scalar */
  const float* block;   /* device pointer, row major [block_rows][block_cols] */
  int block_rows, block_cols;
  int block_r0, block_c0;
  int full_rows, full_cols;
  int block_uniform;    /* 1 when every value of the crop is 1.0 (a jaw
                           rectangle): lookups then read no memory, and
                           `block` may be NULL */
} ch_beam;

/* settings dict of Conehead.calculate (example.py:27-58) plus the spectrum
 * (energies, weights) and mu_water(E), all float32 as the reference uses. */
typedef struct {
  double sPri, sAnn, zAnn, rInner, rOuter, zExp, sExp, kExp;
  double softRatio, softLimit, hornRatio;
  int samples;          /* fluenceResampling */
  int n_energy;
  float E[CH_MAX_ENERGY];
  float w[CH_MAX_ENERGY];
  float mu[CH_MAX_ENERGY];
  int options;          /* 0 = the reference's physics; CH_OPT_* bits below */
} ch_settings;

/* Physics extensions, off by default (not in the reference, so no parity
 * claim; each equals the reference where it must, see the tests).
 *
 * CH_OPT_RADIOLOGICAL_DISTANCE: the kernel is read at the density-scaled
 *   path length along each cone line, r = sum rho(v) * (segment in v), from
 *   the source voxel centre, instead of the geometric distance.  Equal to the
 *   reference in water (rho = 1).  The weights then depend on the densities
 *   between source and target, so these beams run the per-source scatter
 *   path (ch_dose_scatter's structure), not the stencil gather.
 * CH_OPT_CONES_IN_BEAM_FRAME: the 12 x 48 cone directions are rotated with
 *   the beam (d = xform^T d_ref: the kernel's polar axis follows the central
 *   axis of the beam, the collimator turns the azimuths), instead of staying
 *   in the room frame (conehead/conehead.py:386 leaves source_transform
 *   unused).  Equal to the reference at gantry and collimator 0.  Stencils are
 *   built per beam orientation and cached in the plan. */
#define CH_OPT_RADIOLOGICAL_DISTANCE 1
#define CH_OPT_CONES_IN_BEAM_FRAME 2

/* Host tables of the polyenergetic kernel: cumulative K[n_phi][n_r]
 * (float64, radii 0.05 + 0.01 k cm), azimuths theta[n_theta] and cone polar
 * angles phi[n_phi] in degrees (float32). */
typedef struct {
  int n_phi, n_r, n_theta;
  const double* cum;
  const float* theta;
  const float* phi;
} ch_kernel;

/* Optional per-voxel intermediates (device pointers, any may be NULL). */
typedef struct {
  double* blocked;      /* float64 like the reference's device array */
  float* d_eff;
  float* oad;
  float* fluence;
  float* f_soften;
  float* f_horn;
  float* terma;
} ch_intermediates;

/* Stage timings (ms, CUDA events) and counters of the last dose call. */
typedef struct {
  float ms_prologue;
  float ms_range;
  float ms_cone;
  double updates;       /* voxel-direction updates issued by the cone stage */
  int n_unique_dirs;
  int n_units;
} ch_stats;

typedef struct ch_plan ch_plan;

ch_status ch_plan_create(ch_plan** plan, int device);
void ch_plan_destroy(ch_plan* plan);

/* Upload the kernel tables; stencils are rebuilt lazily per voxel spacing. */
ch_status ch_plan_set_kernel(ch_plan* plan, const ch_kernel* kernel);

/* Single beam: dose_dev (float32 [x][y][z]) is overwritten.  rho_dev holds
 * phantom.densities; swap_xy = 1 reproduces the reference's resampling step
 * (densities read transposed in x/y, which it does for square x/y grids). */
ch_status ch_dose(ch_plan* plan, const ch_grid* grid, const float* rho_dev, int swap_xy,
                  const ch_beam* beam, const ch_settings* settings, float* dose_dev,
                  void* stream);

/* As ch_dose, also writing the intermediates that are non-NULL (every voxel
 * is then evaluated, not just the ones the beam can reach). */
ch_status ch_dose_ex(ch_plan* plan, const ch_grid* grid, const float* rho_dev, int swap_xy,
                     const ch_beam* beam, const ch_settings* settings, float* dose_dev,
                     const ch_intermediates* inter, void* stream);

/* Many beams (each with its own grid/density/settings) in one pass: every
 * beam's prologue in one launch pair, then the cone stage over all beams
 * (one FFT launch group per grid shape, or one persistent gather). */
ch_status ch_dose_batch(ch_plan* plan, int n_beams, const ch_grid* grids,
                        const float* const* rho_dev, const int* swap_xy,
                        const ch_beam* beams, const ch_settings* settings,
                        float* const* dose_dev, void* stream);

/* Plain path: prologue + per-voxel scatter with float32 atomics, one beam
 * per launch (the reference's cuda_dose structure). */
ch_status ch_dose_scatter(ch_plan* plan, const ch_grid* grid, const float* rho_dev,
                          int swap_xy, const ch_beam* beam, const ch_settings* settings,
                          float* dose_dev, void* stream);

/* ch_dose without allocating: for callers that cannot call cudaMalloc
 * (e.g. inside a host framework that owns the device allocator, or in code
 * that must not allocate once set up).  No counterpart in the reference.
 * Same arguments and result as ch_dose, but the per-beam scratch lives in a
 * fixed 36 MiB device array inside this library (grids up to about 160^3;
 * larger grids return CH_ERR_INVALID_ARG with the size needed).  The plan must
 * already hold kernel tables and stencils for this voxel spacing and a grid
 * at least this large: run one ch_dose on it first.  The first call on a
 * device looks up the array's device address, so make that call before any
 * stream capture.  Every call shares the one array: calls whose work
 * overlaps on the GPU race, so serialise them (one stream, or events).  It
 * also uses the plan's own counters, so it must not overlap on the GPU with
 * any other call on the same plan either.  It records no stage timings:
 * ch_plan_stats reports zeros after it. */
ch_status ch_dose_static(ch_plan* plan, const ch_grid* grid, const float* rho_dev, int swap_xy,
                         const ch_beam* beam, const ch_settings* settings, float* dose_dev,
                         void* stream);

/* Jaw + MLCX block map of one static beam, in 0.1 mm map cells, as
 * Block._set_from_plan builds it (conehead/block.py:87-215).  The full map
 * is map_rows x map_cols (rows: leaf-boundary direction, map_rows =
 * |last - first leaf boundary|; columns: leaf travel, 4000).  Leaf pair n
 * covers rows [row0[n], row0[n] + rows[n]); its bank-A leaf covers columns
 * [0, a_end[n]) and its bank-B leaf [b_start[n], map_cols - 1).  A leaf's
 * transmission is 1 - profile(row) * ramp(column): the profile is 0.2, 0.5,
 * 0.75 on the three rows at each side (tongue and groove, later rows of that
 * list winning on narrow leaves) and 1 elsewhere; the ramp is tip[] over
 * the 15 columns at the leaf end and 1 elsewhere.  Bank B is bank A turned
 * by 180 degrees and is drawn over it.  Rows outside every pair read 1.
 * Everything outside the jaw opening [open_r0, open_r1) x [open_c0,
 * open_c1) reads 0.  The host fills this from the plan (conehead_gb300's
 * block.MLCField does, with the reference's rounding). */
#define CH_MAX_LEAF_PAIRS 256
#define CH_MLC_TIP_CELLS 15
typedef struct {
  int n_pairs;
  int map_rows, map_cols;
  int open_r0, open_r1, open_c0, open_c1;
  int reserved;
  int row0[CH_MAX_LEAF_PAIRS];
  int rows[CH_MAX_LEAF_PAIRS];
  int a_end[CH_MAX_LEAF_PAIRS];
  int b_start[CH_MAX_LEAF_PAIRS];
  double tip[CH_MLC_TIP_CELLS];   /* numpy.linspace(1, 0, 15) */
} ch_mlc;

/* Rasterise the window [r0, r0 + rows) x [c0, c0 + cols) of an MLC block
 * map into out_dev (float32, row major [rows][cols], device pointer) on the
 * device: no host map, no 64 MB upload.  Cells outside the map read 0.  Pass
 * the jaw opening as the window and the result is the cropped map that
 * ch_beam.block takes (block_r0 = open_r0, block_c0 = open_c0, full_rows =
 * map_rows, full_cols = map_cols).  Replaces building block_values on the
 * host and copying it to the device (conehead/block.py:87-215 and
 * conehead/conehead.py:555).  Leaf pairs must be ordered, disjoint and inside
 * the map, at least 3 rows high, with leaf lengths of at least 15 columns;
 * other tables give CH_ERR_INVALID_ARG. */
ch_status ch_block_from_mlc(const ch_mlc* mlc, float* out_dev, int rows, int cols, int r0, int c0,
                            void* stream);

/* ---------------------------------------------------------------- adjoint
 * Beamlet fluence: a rows x cols grid of beamlets on the block map, beamlet
 * (i, j) covering map rows r0 + i*cell_rows .. r0 + (i+1)*cell_rows - 1 and
 * columns c0 + j*cell_cols .. (0.1 mm cells; 0.5 cm beamlets are 50 x 50).
 * Its block crop holds weight w[i][j] in every cell of beamlet (i, j).  None
 * of this is in the reference; the dose of a beamlet map is exactly the
 * reference's dose for that block map. */
#define CH_MAX_BEAMLETS 16384
typedef struct {
  int rows, cols;
  int cell_rows, cell_cols;
  int r0, c0;
} ch_beamlets;

/* Fill the block crop ([rows*cell_rows][cols*cell_cols], device) of a
 * beamlet grid from weights_dev (float32 [rows][cols], device).  Pass it as
 * ch_beam.block with block_r0 = r0, block_c0 = c0. */
ch_status ch_block_from_beamlets(const ch_beamlets* beamlets, const float* weights_dev, float* crop_dev,
                                 void* stream);

/* The cone stage as an operator on any volume (device, float32 [x][y][z]):
 * out = C in, or out = C^T in with transpose = 1, where C maps TERMA to dose
 * exactly as ch_dose's cone stage does (conehead/conehead.py:385-488), by
 * the plan's cone method: spectral (the transpose multiplies by the
 * conjugate stencil spectrum) or gather (the transpose walks the mirrored
 * walks).  in and out must differ. */
ch_status ch_cone(ch_plan* plan, const ch_grid* grid, const float* in_dev, float* out_dev, int transpose,
                  void* stream);

/* Gradient of a dose objective with respect to beamlet weights: given
 * grad_dose = dL/d(dose) (device, [x][y][z]) for the dose ch_dose computes
 * from this beam (whose block crop is the beamlet grid's), writes
 * grad_weights = dL/dw (device, float32 [rows][cols]) and, if grad_terma is
 * not NULL, dL/d(TERMA) ([x][y][z]; exact where TERMA can be nonzero --
 * inside its box and the beam frustum -- and elsewhere the full C^T value
 * with the spectral cone method, 0 with the gather).  Steps: the
 * forward prologue, the transposed cone (C^T grad_dose on those voxels), and
 * the transposed blocking: blocked(v) = sum over the S^3 sub-samples of
 * w[beamlet] / S^3 and TERMA = blocked^2 * H(v) (fluence and TERMA each carry
 * one factor), so dL/dw gets 2 TERMA/blocked * dL/dTERMA / S^3 from every
 * sub-sample in its beamlet.  No counterpart in the reference. */
ch_status ch_dose_adjoint(ch_plan* plan, const ch_grid* grid, const float* rho_dev, int swap_xy,
                          const ch_beam* beam, const ch_beamlets* beamlets, const ch_settings* settings,
                          const float* grad_dose_dev, float* grad_weights_dev, float* grad_terma_dev,
                          void* stream);

/* Test hook: n_rays DDA traces on the device.  starts int32 [n][3],
 * dirs float32 [n][3] (used as given, no normalisation), grid dims/spacing
 * from `grid`.  Writes voxels int32 [n][cap][3], t float32 [n][cap] and
 * lengths int32 [n] (full length, even when > cap).  Device pointers. */
ch_status ch_dda_trace(const ch_grid* grid, int n_rays, const int* starts_dev,
                       const float* dirs_dev, int cap, int* voxels_dev, float* t_dev,
                       int* len_dev, void* stream);

/* Test hook: the cone directions the device computes for (theta_i, phi_j),
 * float32 [n_theta][n_phi][3] into out_dev. */
ch_status ch_cone_directions(ch_plan* plan, float* out_dev, void* stream);

/* Schedule of the cone and TERMA passes (results do not depend on it, up
 * to the float rounding of the dose sums).
 * cone_method: how the collapsed-cone stage (conehead/conehead.py:385-488)
 *   is evaluated.  CH_CONE_SPECTRAL (default): the stage is one linear
 *   convolution with the tap stencil of all cone walks, applied through
 *   forward and inverse 3-D FFTs of period >= 2n - 1 per axis (grids whose
 *   periods exceed the limit fall back to the gather).  CH_CONE_GATHER: the
 *   tap stencil is walked tile by tile (shared-memory windows, no atomics but
 *   one add per output and work unit).  Both give the reference's dose.
 * dir_group: unique directions per gather work unit, 1..1024 (default 16);
 * unit_order: 0 = a tile's direction groups are consecutive gather units
 * (default), 1 = a direction group's tiles are;
 * terma_ctas_per_sm: CTAs per SM of the TERMA pass, 1..32 (default 8); the
 * batched pass is persistent and holds at most 3 CTAs per SM (its register
 * budget), so values above 3 only change the single-beam pass.
 * Picked per workload by conehead_gb300.autotune. */
#define CH_CONE_SPECTRAL 0
#define CH_CONE_GATHER 1
typedef struct {
  int dir_group;
  int unit_order;
  int terma_ctas_per_sm;
  int cone_method;
} ch_tuning;

ch_status ch_plan_set_tuning(ch_plan* plan, const ch_tuning* tuning);
ch_status ch_plan_get_tuning(ch_plan* plan, ch_tuning* tuning);

/* A batch captured once into a CUDA graph and replayed with one launch.
 * ch_batch_create validates the beams like ch_dose_batch, builds every
 * launch record into device memory the batch owns (with its own scratch),
 * and captures the device work -- every beam's prologue and the cone stage
 * (FFT passes, or tap ranges and the persistent gather) -- into a graph.  Each ch_batch_launch
 * recomputes all doses from the current contents of the density and
 * block-map buffers (which may change in place between launches; the
 * geometry, settings, grids and schedule are fixed at capture).
 * ch_batch_sync waits on `stream` and reports device-side failures.  While
 * batches exist the plan's kernel tables and stencils are frozen: prepare the
 * plan for the largest grid first (ch_plan_prepare).  ch_batch_destroy waits
 * for the device.  No counterpart in the reference. */
typedef struct ch_batch ch_batch;
ch_status ch_batch_create(ch_plan* plan, int n_beams, const ch_grid* grids, const float* const* rho_dev,
                          const int* swap_xy, const ch_beam* beams, const ch_settings* settings,
                          float* const* dose_dev, void* stream, ch_batch** batch);
ch_status ch_batch_launch(ch_batch* batch, void* stream);
ch_status ch_batch_sync(ch_batch* batch, void* stream);
void ch_batch_destroy(ch_batch* batch);

/* Build the plan's direction stencils for this grid's voxel spacing and
 * size ahead of the first dose call (otherwise the first call that brings
 * a new spacing or a larger grid builds them), and, with the spectral cone
 * method, the stencil spectrum of exactly this grid shape (one per shape,
 * counted in ch_plan_memory's tables).  Serving code prepares each plan for
 * its grids once, so no request pays the build.  No counterpart in the
 * reference (it rebuilds everything per call, conehead/conehead.py:541-738). */
ch_status ch_plan_prepare(ch_plan* plan, const ch_grid* grid, void* stream);

/* Device bytes the plan holds: kernel tables and stencils (`tables`), and
 * its scratch arena (`scratch`).  Either pointer may be NULL. */
ch_status ch_plan_memory(ch_plan* plan, size_t* tables, size_t* scratch);

/* Scratch a ch_dose_batch call over these n grids needs: `total` is the
 * arena size it uses, `growth` how many bytes the plan's arena would grow
 * by (the arena only grows).  For admission control; no counterpart in the
 * reference.  Stencil tables (a few MB per spacing) are not included. */
ch_status ch_batch_scratch_bytes(ch_plan* plan, int n, const ch_grid* grids, size_t* growth, size_t* total);

/* Free the plan's scratch arena (kernel tables and stencils stay).  Waits
 * for all work on the device first. */
ch_status ch_plan_trim(ch_plan* plan);

/* Bound of the gather cone stage's pipeline waits, in mbarrier try_wait
 * iterations (iterations <= 0 restores the default, 2^22).  When a wait
 * gives up, the kernel records the failure, lets its own copies in flight
 * land and returns; ch_plan_sync then reports CH_ERR_TIMEOUT and the plan
 * stays usable.
 * withhold is the test hook of that failure path (0 in normal use): with
 * CH_WITHHOLD_WINDOWS the gather's producer issues no window, so the
 * consumers' waits for one expire; with CH_WITHHOLD_SLOTS the consumers never
 * free a window slot, so the producer's wait for one expires while its last
 * two window copies are in flight.  No counterpart in the reference (its
 * kernels have no device-side waits). */
#define CH_WITHHOLD_WINDOWS 1
#define CH_WITHHOLD_SLOTS 2
ch_status ch_plan_set_wait_limit(ch_plan* plan, long long iterations, int withhold);

/* Wait for the plan's work on `stream` and report device-side failures
 * (CH_ERR_TIMEOUT, CH_ERR_PARALLEL_RAY) of the last dose call. */
ch_status ch_plan_sync(ch_plan* plan, void* stream);

/* Stage timings and counters of the last dose call (waits for it). */
ch_status ch_plan_stats(ch_plan* plan, ch_stats* out);

const char* ch_status_string(ch_status status);
const char* ch_last_error(void);
int ch_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CONEHEAD_GB300_H */
