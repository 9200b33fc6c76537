// CPU oracle for the conehead dose path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, loop for loop, the reference's single-beam dose path
// (samuelpeet/conehead, conehead/conehead.py) so the GPU engine can be
// checked against it.  Nothing in the product links, loads or calls it: only
// the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
//
// Two precision modes:
//   mode 0 "fp32-mirrored": every intermediate has the type the Numba-compiled
//     reference gives it.  Local arrays are float32; float32 op float32 stays
//     float32; float32 op float64 (or op int64) is evaluated in float64 and
//     rounded only where it is stored into a float32 local/array.  No fused
//     multiply-add contraction (build with -ffp-contract=off).
//   mode 1 "fp64": the same algorithm with every local array, accumulator
//     and table lookup in float64 (an FP64 re-run of the method).
//
// Stages (reference file:line in conehead/conehead.py):
//   hit test / voxel blocking  :25-120   (27 sub-samples, 0.1 mm block map)
//   Amanatides-Woo 3D DDA      :123-206  (tie rule t0<t1 ? (t0<t2?x:z) : (t1<t2?y:z))
//   radiological depth d_eff   :209-254
//   off-axis distance          :286-314
//   three-source fluence       :320-360
//   softening / horn factors   :641-655  (host numpy, float32)
//   TERMA                      :364-377  (mu table float32 with current scipy)
//   collapsed-cone dose        :385-488  (scatter along 12 x 48 cone lines)
// The density array is read with the x/y swap the reference's resampling
// step produces (conehead.py:524-533,561-568 == densities.transpose(1,0,2)).
//
// Build: see oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

struct or_grid {
  int n[3];
  float origin[3];
  float spacing[3];
};

struct or_beam {
  double src[3];     // source.position
  double vy[3];      // source.v_y (blocking-plane normal)
  double xform[9];   // source.transform, row major
  double sad;        // source.sad
  int geom_f32;      // 1: position/v_y/transform are float32 arrays
  int sad_f32;       // 1: source.sad is a float32 scalar
  const float* block;  // block_values, row major [rows][cols]
  int block_rows, block_cols;
};

struct or_settings {
  double sPri, sAnn, zAnn, rInner, rOuter, zExp, sExp, kExp;
  double softRatio, softLimit, hornRatio;
  int samples;        // settings['fluenceResampling']
  int n_energy;
  const float* E;     // energies (MeV), float32
  const float* w;     // spectrum weights, float32
  const float* mu;    // mu_water(E), float32
};

}  // extern "C"

namespace {

inline int64_t idx3(const int* n, int x, int y, int z) {
  return ((int64_t)x * n[1] + y) * n[2] + z;
}

// density seen by the reference at dose-grid voxel (x, y, z)
inline float rho_at(const or_grid& g, const float* rho, int swap_xy, int x, int y, int z) {
  if (swap_xy) return rho[((int64_t)y * g.n[0] + x) * g.n[2] + z];
  return rho[idx3(g.n, x, y, z)];
}

// voxel centre coordinate: float32 store of f64(origin) + f64(spacing) * i
template <typename F>
inline F centre(float origin, float spacing, int i) {
  return (F)((double)origin + (double)spacing * (double)i);
}

// ---------------------------------------------------------------- DDA -----
// Amanatides & Woo from a voxel centre; records visited voxels and the exit
// t of each.  F is the type of the reference's local t/direction arrays.
template <typename F>
struct DdaStep { int v[3]; F t; };

template <typename F>
inline void dda_init(const F* dir_in, const float* spacing, int* step, F* t, F* dt) {
  for (int k = 0; k < 3; ++k) {
    F d = dir_in[k];
    step[k] = d < 0 ? -1 : 1;
    if (d < 0) d = -d;
    if (d == (F)0.0) {
      t[k] = (F)1000000000.0;
      dt[k] = (F)1000000000.0;
    } else {
      // (spacing / 2) / d is float64 arithmetic in Numba (float32 / int literal)
      t[k] = (F)(((double)spacing[k] / 2.0) / (double)d);
      dt[k] = (F)((F)spacing[k] / d);
    }
  }
}

template <typename F, typename Visit>
inline void dda_walk(const int* start, const F* dir, const float* spacing, const int* n,
                     Visit visit) {
  int step[3];
  F t[3], dt[3];
  dda_init<F>(dir, spacing, step, t, dt);
  int cur[3] = {start[0], start[1], start[2]};
  while (cur[0] >= 0 && cur[0] < n[0] && cur[1] >= 0 && cur[1] < n[1] &&
         cur[2] >= 0 && cur[2] < n[2]) {
    int ax;
    if (t[0] < t[1]) ax = (t[0] < t[2]) ? 0 : 2;
    else ax = (t[1] < t[2]) ? 1 : 2;
    visit(cur, t[ax]);
    t[ax] = (F)(t[ax] + dt[ax]);
    cur[ax] += step[ax];
  }
}

// --------------------------------------------------------- projection -----
// Project a point onto the isocentre plane along the line through the
// source (conehead.py:25-47) and rotate into beam coordinates (rows 0, 2 of
// the transform).  `rd` is the float32 ray vector source - point.
// Returns false for a ray parallel to the plane (the reference raises).
template <typename F>
bool project_f(const or_beam& b, const F* rd, F* out_x, F* out_z);

// float32 source arrays: all float32 arithmetic
template <>
bool project_f<float>(const or_beam& b, const float* rd, float* ox, float* oz) {
  float vy0 = (float)b.vy[0], vy1 = (float)b.vy[1], vy2 = (float)b.vy[2];
  float ndotu = vy0 * rd[0] + vy1 * rd[1] + vy2 * rd[2];
  if (std::fabs((double)ndotu) < 1e-6) return false;
  float w[3] = {(float)b.src[0], (float)b.src[1], (float)b.src[2]};
  float si = -(vy0 * w[0] + vy1 * w[1] + vy2 * w[2]) / ndotu;
  float pp[3];
  for (int k = 0; k < 3; ++k) pp[k] = (w[k] + si * rd[k]) + 0.0f;
  const double* m = b.xform;
  *ox = (float)m[0] * pp[0] + (float)m[1] * pp[1] + (float)m[2] * pp[2];
  *oz = (float)m[6] * pp[0] + (float)m[7] * pp[1] + (float)m[8] * pp[2];
  return true;
}

// float64 source arrays: float64 dot products, float32 stores
bool project_mixed(const or_beam& b, const float* rd, float* ox, float* oz) {
  double ndotu = b.vy[0] * (double)rd[0] + b.vy[1] * (double)rd[1] + b.vy[2] * (double)rd[2];
  if (std::fabs(ndotu) < 1e-6) return false;
  float w[3] = {(float)b.src[0], (float)b.src[1], (float)b.src[2]};
  double si = -(b.vy[0] * (double)w[0] + b.vy[1] * (double)w[1] + b.vy[2] * (double)w[2]) / ndotu;
  float pp[3];
  for (int k = 0; k < 3; ++k) pp[k] = (float)(((double)w[k] + si * (double)rd[k]) + 0.0);
  const double* m = b.xform;
  *ox = (float)(m[0] * (double)pp[0] + m[1] * (double)pp[1] + m[2] * (double)pp[2]);
  *oz = (float)(m[6] * (double)pp[0] + m[7] * (double)pp[1] + m[8] * (double)pp[2]);
  return true;
}

// FP64 re-run: everything float64
bool project_d(const or_beam& b, const double* rd, double* ox, double* oz) {
  double ndotu = b.vy[0] * rd[0] + b.vy[1] * rd[1] + b.vy[2] * rd[2];
  if (std::fabs(ndotu) < 1e-6) return false;
  const double* w = b.src;
  double si = -(b.vy[0] * w[0] + b.vy[1] * w[1] + b.vy[2] * w[2]) / ndotu;
  double pp[3];
  for (int k = 0; k < 3; ++k) pp[k] = w[k] + si * rd[k];
  const double* m = b.xform;
  *ox = m[0] * pp[0] + m[1] * pp[1] + m[2] * pp[2];
  *oz = m[6] * pp[0] + m[7] * pp[1] + m[8] * pp[2];
  return true;
}

// block-map lookup with the reference's cell rule (conehead.py:50-68):
// cell = floor(100 p) + 2000, outside [0, 3999] -> 0, else map[cell - 1]
// (cell 0 wraps to the last row/column, as Numba's negative indexing does).
inline int64_t floor_clamped(double v) {
  if (!(v == v)) return 0;  // NaN
  if (v > 1e12) return (int64_t)1e12;
  if (v < -1e12) return (int64_t)-1e12;
  return (int64_t)std::floor(v);
}

template <typename F>
float block_lookup(const or_beam& b, F px, F pz) {
  F c0, c1;
  if (sizeof(F) == 4) {
    c0 = (F)(float)floor_clamped((double)((float)px * 100.0f));
    c1 = (F)(float)floor_clamped((double)((float)pz * 100.0f));
    c0 = (F)((float)c0 + 2000.0f);
    c1 = (F)((float)c1 + 2000.0f);
  } else {
    c0 = (F)floor_clamped((double)px * 100.0) + 2000.0;
    c1 = (F)floor_clamped((double)pz * 100.0) + 2000.0;
  }
  if (c0 < 0 || c0 > 3999 || c1 < 0 || c1 > 3999) return 0.0f;
  int64_t r = (int64_t)c0 - 1, c = (int64_t)c1 - 1;
  if (r < 0) r += b.block_rows;
  if (c < 0) c += b.block_cols;
  // a map smaller than 4000 x 4000 is read past its end by the reference
  // (undefined); both implementations read 0 there
  if (r >= b.block_rows || c >= b.block_cols) return 0.0f;
  return b.block[r * b.block_cols + c];
}

struct Outputs {
  double* blocked;
  double* d_eff;
  double* oad;
  double* fluence;
  double* f_soften;
  double* f_horn;
  double* terma;
};

// ---------------------------------------------------------- prologue ------
int prologue_f32(const or_grid& g, const float* rho, int swap_xy, const or_beam& b,
                 const or_settings& s, Outputs o) {
  const int* n = g.n;
  const int S = s.samples;
  int bad = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : bad)
  for (int x = 0; x < n[0]; ++x)
    for (int y = 0; y < n[1]; ++y)
      for (int z = 0; z < n[2]; ++z) {
        const int id[3] = {x, y, z};
        const int64_t v = idx3(n, x, y, z);
        float pos[3], off[3];
        for (int k = 0; k < 3; ++k) {
          pos[k] = centre<float>(g.origin[k], g.spacing[k], id[k]);
          off[k] = (float)((double)g.spacing[k] / (double)S);
        }
        // --- hit test (blocked accumulates in float64)
        double acc = 0.0;
        for (int ix = 0; ix < S; ++ix)
          for (int iy = 0; iy < S; ++iy)
            for (int iz = 0; iz < S; ++iz) {
              const int ii[3] = {ix, iy, iz};
              float ps[3], rd[3];
              for (int k = 0; k < 3; ++k)
                ps[k] = (float)((((double)pos[k] - (double)g.spacing[k] / 2.0) +
                                 (double)off[k] / 2.0) + (double)off[k] * (double)ii[k]);
              float px, pz;
              bool ok;
              if (b.geom_f32) {
                for (int k = 0; k < 3; ++k) rd[k] = (float)b.src[k] - ps[k];
                ok = project_f<float>(b, rd, &px, &pz);
              } else {
                for (int k = 0; k < 3; ++k) rd[k] = (float)(b.src[k] - (double)ps[k]);
                ok = project_mixed(b, rd, &px, &pz);
              }
              if (!ok) { bad = 1; continue; }
              acc = acc + (double)block_lookup<float>(b, px, pz) / (double)(S * S * S);
            }
        const double blocked = acc;
        // --- ray vector to the source (shared by d_eff, oad and fluence)
        float rd[3];
        if (b.geom_f32) for (int k = 0; k < 3; ++k) rd[k] = (float)b.src[k] - pos[k];
        else for (int k = 0; k < 3; ++k) rd[k] = (float)(b.src[k] - (double)pos[k]);
        const float mag = std::sqrt(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]);
        // --- d_eff: DDA from the voxel toward the source
        float dir[3] = {rd[0] / mag, rd[1] / mag, rd[2] / mag};
        float deff = 0.0f;
        float tprev = 0.0f;
        bool first = true;
        dda_walk<float>(id, dir, g.spacing, n, [&](const int* c, float t) {
          const float r = rho_at(g, rho, swap_xy, c[0], c[1], c[2]);
          if (first) { deff = deff + r * t; first = false; }
          else deff = deff + r * (t - tprev);
          tprev = t;
        });
        // --- off-axis distance
        float px, pz;
        bool ok = b.geom_f32 ? project_f<float>(b, rd, &px, &pz) : project_mixed(b, rd, &px, &pz);
        if (!ok) { bad = 1; px = pz = 0.0f; }
        const float oad = std::sqrt(px * px + pz * pz);
        // --- fluence (float64 arithmetic, float32 store)
        const double sad = b.sad;
        double ratio = b.sad_f32 ? (double)((float)sad / mag) : sad / (double)mag;
        const double fpoint = s.sPri * (ratio * ratio);
        const double r_ann = (double)oad * s.zAnn / sad;
        double fann = 0.0;
        if (r_ann >= s.rInner && r_ann <= s.rOuter) {
          const double a = sad - s.zAnn, c = (double)mag - s.zAnn;
          fann = s.sAnn * (a * a) / (c * c);
        }
        const double oadc = oad < 2.0f ? 2.0 : (double)oad;
        const double r_exp = oadc * s.zExp / sad;
        const double ae = sad - s.zExp, ce = (double)mag - s.zExp;
        const double fexp = s.sExp / r_exp * std::exp(-s.kExp * r_exp) * (ae * ae) / (ce * ce);
        const float fluence = (float)((fpoint + fann + fexp) * blocked);
        // --- softening and horn (host numpy float32)
        float fs = 1.0f;
        if (oad < (float)s.softLimit) fs = 1.0f / (1.0f - (float)s.softRatio * oad);
        const float fh = 1.0f + oad * (float)s.hornRatio;
        // --- TERMA (float32, mu table float32)
        float terma = 0.0f;
        for (int i = 0; i < s.n_energy; ++i) {
          const float e = std::exp((-s.mu[i] * fs) * deff);
          terma = terma + ((((s.w[i] * fluence) * e) * s.E[i]) * s.mu[i]) * fh;
        }
        const float T = (float)((double)terma * blocked);
        if (o.blocked) o.blocked[v] = blocked;
        if (o.d_eff) o.d_eff[v] = deff;
        if (o.oad) o.oad[v] = oad;
        if (o.fluence) o.fluence[v] = fluence;
        if (o.f_soften) o.f_soften[v] = fs;
        if (o.f_horn) o.f_horn[v] = fh;
        o.terma[v] = T;
      }
  return bad ? 1 : 0;
}

int prologue_f64(const or_grid& g, const float* rho, int swap_xy, const or_beam& b,
                 const or_settings& s, Outputs o) {
  const int* n = g.n;
  const int S = s.samples;
  int bad = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : bad)
  for (int x = 0; x < n[0]; ++x)
    for (int y = 0; y < n[1]; ++y)
      for (int z = 0; z < n[2]; ++z) {
        const int id[3] = {x, y, z};
        const int64_t v = idx3(n, x, y, z);
        double pos[3], off[3];
        for (int k = 0; k < 3; ++k) {
          pos[k] = (double)g.origin[k] + (double)g.spacing[k] * id[k];
          off[k] = (double)g.spacing[k] / S;
        }
        double acc = 0.0;
        for (int ix = 0; ix < S; ++ix)
          for (int iy = 0; iy < S; ++iy)
            for (int iz = 0; iz < S; ++iz) {
              const int ii[3] = {ix, iy, iz};
              double ps[3], rd[3];
              for (int k = 0; k < 3; ++k) {
                ps[k] = pos[k] - (double)g.spacing[k] / 2.0 + off[k] / 2.0 + off[k] * ii[k];
                rd[k] = b.src[k] - ps[k];
              }
              double px, pz;
              if (!project_d(b, rd, &px, &pz)) { bad = 1; continue; }
              acc += (double)block_lookup<double>(b, px, pz) / (double)(S * S * S);
            }
        const double blocked = acc;
        double rd[3];
        for (int k = 0; k < 3; ++k) rd[k] = b.src[k] - pos[k];
        const double mag = std::sqrt(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]);
        double dir[3] = {rd[0] / mag, rd[1] / mag, rd[2] / mag};
        double deff = 0.0, tprev = 0.0;
        bool first = true;
        dda_walk<double>(id, dir, g.spacing, n, [&](const int* c, double t) {
          const double r = rho_at(g, rho, swap_xy, c[0], c[1], c[2]);
          deff += first ? r * t : r * (t - tprev);
          first = false;
          tprev = t;
        });
        double px, pz;
        if (!project_d(b, rd, &px, &pz)) { bad = 1; px = pz = 0.0; }
        const double oad = std::sqrt(px * px + pz * pz);
        const double sad = b.sad;
        const double ratio = sad / mag;
        const double fpoint = s.sPri * ratio * ratio;
        const double r_ann = oad * s.zAnn / sad;
        double fann = 0.0;
        if (r_ann >= s.rInner && r_ann <= s.rOuter) {
          const double a = sad - s.zAnn, c = mag - s.zAnn;
          fann = s.sAnn * (a * a) / (c * c);
        }
        const double oadc = oad < 2.0 ? 2.0 : oad;
        const double r_exp = oadc * s.zExp / sad;
        const double ae = sad - s.zExp, ce = mag - s.zExp;
        const double fexp = s.sExp / r_exp * std::exp(-s.kExp * r_exp) * (ae * ae) / (ce * ce);
        const double fluence = (fpoint + fann + fexp) * blocked;
        double fs = 1.0;
        if (oad < s.softLimit) fs = 1.0 / (1.0 - s.softRatio * oad);
        const double fh = 1.0 + oad * s.hornRatio;
        double terma = 0.0;
        for (int i = 0; i < s.n_energy; ++i) {
          const double mu = s.mu[i];
          terma += (double)s.w[i] * fluence * std::exp(-mu * fs * deff) * (double)s.E[i] * mu * fh;
        }
        if (o.blocked) o.blocked[v] = blocked;
        if (o.d_eff) o.d_eff[v] = deff;
        if (o.oad) o.oad[v] = oad;
        if (o.fluence) o.fluence[v] = fluence;
        if (o.f_soften) o.f_soften[v] = fs;
        if (o.f_horn) o.f_horn[v] = fh;
        o.terma[v] = terma * blocked;
      }
  return bad ? 1 : 0;
}

// ------------------------------------------------------------- cone -------
// Cone directions, computed as conehead.py:414-429 does per (theta, phi).
template <typename F>
void cone_direction(float theta_deg, float phi_deg, F* d) {
  const double th = (double)theta_deg * M_PI / 180.0;
  const double ph = (double)phi_deg * M_PI / 180.0;
  const double ct = std::cos(th), st = std::sin(th), cp = std::cos(ph), sp = std::sin(ph);
  d[0] = (F)(ct * sp);
  d[1] = (F)cp;
  d[2] = (F)(st * sp);
  const F nrm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  d[0] = d[0] / nrm;
  d[1] = d[1] / nrm;
  d[2] = d[2] / nrm;
}

inline int kernel_index(double t) {
  // abs(floor(t * 100 - 5)), clamped to the last kernel sample (conehead.py:457-461)
  int64_t i = (int64_t)std::floor(t * 100.0 - 5.0);
  if (i < 0) i = -i;
  if (i > 5995) i = 5995;
  return (int)i;
}

// Options of the physics extensions (not in the reference): rho != null reads
// the kernel at the radiological path length along each cone line
// (density-scaled distance); frame != null rotates the cone directions by a
// beam's world->beam matrix (cones in the beam frame).
struct ConeExt {
  const float* rho = nullptr;
  int swap_xy = 0;
  const double* frame = nullptr;   // row-major 3x3
};

template <typename F>
void rotate_direction(const double* m, F* d) {
  F r[3];
  for (int k = 0; k < 3; ++k) r[k] = (F)(m[k] * (double)d[0] + m[3 + k] * (double)d[1] + m[6 + k] * (double)d[2]);
  d[0] = r[0];
  d[1] = r[1];
  d[2] = r[2];
}

template <typename F>
void cone(const or_grid& g, const double* terma, const double* K, int n_r,
          const float* thetas, int n_theta, const float* phis, int n_phi, double* dose, const ConeExt& ext = {}) {
  const int* n = g.n;
  const int64_t N = (int64_t)n[0] * n[1] * n[2];
  std::vector<F> dirs((size_t)n_theta * n_phi * 3);
  for (int i = 0; i < n_theta; ++i)
    for (int j = 0; j < n_phi; ++j) {
      cone_direction<F>(thetas[i], phis[j], &dirs[((size_t)i * n_phi + j) * 3]);
      if (ext.frame) rotate_direction<F>(ext.frame, &dirs[((size_t)i * n_phi + j) * 3]);
    }
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  std::vector<std::vector<double>> priv((size_t)nthr);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double>& acc = priv[(size_t)tid];
    acc.assign((size_t)N, 0.0);
#pragma omp for collapse(2) schedule(dynamic, 1)
    for (int x = 0; x < n[0]; ++x)
      for (int y = 0; y < n[1]; ++y)
        for (int z = 0; z < n[2]; ++z) {
          const double Tv = terma[idx3(n, x, y, z)];
          if (Tv == 0.0) continue;
          const int start[3] = {x, y, z};
          for (int i = 0; i < n_theta; ++i)
            for (int j = 0; j < n_phi; ++j) {
              const F* d = &dirs[((size_t)i * n_phi + j) * 3];
              const double* Kj = K + (size_t)j * n_r;
              int prev_idx = -1;
              F rad = 0, tprev = 0;
              dda_walk<F>(start, d, g.spacing, n, [&](const int* c, F t) {
                F tk = t;
                if (ext.rho) {
                  // path length scaled by the density of each voxel crossed
                  const int64_t ri = ext.swap_xy ? ((int64_t)c[1] * n[0] + c[0]) * n[2] + c[2]
                                                 : ((int64_t)c[0] * n[1] + c[1]) * n[2] + c[2];
                  rad = rad + (F)ext.rho[ri] * (t - tprev);
                  tprev = t;
                  tk = rad;
                }
                const int ki = kernel_index((double)tk);
                const double dk = prev_idx < 0 ? Kj[ki] : Kj[ki] - Kj[prev_idx];
                prev_idx = ki;
                double contrib;
                if (sizeof(F) == 4) contrib = (double)(float)((double)(float)Tv * dk);
                else contrib = Tv * dk;
                acc[(size_t)idx3(n, c[0], c[1], c[2])] += contrib;
              });
            }
        }
  }
  for (int64_t v = 0; v < N; ++v) {
    double s = 0.0;
    for (int t = 0; t < nthr; ++t)
      if (!priv[(size_t)t].empty()) s += priv[(size_t)t][(size_t)v];
    dose[v] = s;
  }
}

// Transpose of cone(): out[s] = sum over directions and DDA steps m of the
// walk from s of dK_j[m] * r[v_m] -- the same walks as the scatter, reading
// where it writes.  It is the dL/dTERMA of the beamlet adjoint (no
// counterpart in the reference).  float64 sums in both modes.
// With `support` set, only voxels whose support value is nonzero are
// computed (the others are 0): the beamlet gradient needs dL/dTERMA only
// where TERMA is nonzero, and that bounds the walks to the forward's.
template <typename F>
void cone_transpose(const or_grid& g, const double* r, const double* K, int n_r, const float* thetas,
                    int n_theta, const float* phis, int n_phi, double* out, const double* support = nullptr) {
  const int* n = g.n;
  std::vector<F> dirs((size_t)n_theta * n_phi * 3);
  for (int i = 0; i < n_theta; ++i)
    for (int j = 0; j < n_phi; ++j)
      cone_direction<F>(thetas[i], phis[j], &dirs[((size_t)i * n_phi + j) * 3]);
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
  for (int x = 0; x < n[0]; ++x)
    for (int y = 0; y < n[1]; ++y)
      for (int z = 0; z < n[2]; ++z) {
        const int start[3] = {x, y, z};
        if (support && support[idx3(n, x, y, z)] == 0.0) {
          out[idx3(n, x, y, z)] = 0.0;
          continue;
        }
        double acc = 0.0;
        for (int i = 0; i < n_theta; ++i)
          for (int j = 0; j < n_phi; ++j) {
            const F* d = &dirs[((size_t)i * n_phi + j) * 3];
            const double* Kj = K + (size_t)j * n_r;
            int prev_idx = -1;
            dda_walk<F>(start, d, g.spacing, n, [&](const int* c, F t) {
              const int ki = kernel_index((double)t);
              const double dk = prev_idx < 0 ? Kj[ki] : Kj[ki] - Kj[prev_idx];
              prev_idx = ki;
              acc += dk * r[idx3(n, c[0], c[1], c[2])];
            });
          }
        out[idx3(n, x, y, z)] = acc;
      }
}

// Transposed blocking in float64 onto a beamlet grid (no counterpart in the
// reference; the test oracle of the beamlet-weight gradient).  blocked(v) is
// the mean over the voxel's S^3 sub-samples of the block map value of the
// cell each projects to (conehead.py:71-120); on a beamlet map that value is
// the weight of the beamlet holding the cell, so
//   d blocked(v) / d w_b = (sub-samples of v in beamlet b) / S^3,
// and grad[b] = sum_v coef[v] * d blocked(v) / d w_b for the caller's coef
// (dL/dTERMA * dTERMA/dblocked).  Sample positions, projection and cell rule
// are those of prologue_f64.  Beamlet (i, j) covers map rows
// r0 + i cell_rows .. and columns c0 + j cell_cols ..
int blocked_adjoint_f64(const or_grid& g, const or_beam& b, int S, const double* coef, int rows, int cols,
                        int cell_rows, int cell_cols, int r0, int c0, double* grad) {
  const int* n = g.n;
  const int nb = rows * cols;
  int bad = 0;
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  std::vector<std::vector<double>> priv((size_t)nthr, std::vector<double>((size_t)nb, 0.0));
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : bad)
  for (int x = 0; x < n[0]; ++x)
    for (int y = 0; y < n[1]; ++y) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      std::vector<double>& acc = priv[(size_t)tid];
      for (int z = 0; z < n[2]; ++z) {
        const double cv = coef[idx3(n, x, y, z)];
        if (cv == 0.0) continue;
        const int id[3] = {x, y, z};
        double pos[3], off[3];
        for (int k = 0; k < 3; ++k) {
          pos[k] = (double)g.origin[k] + (double)g.spacing[k] * id[k];
          off[k] = (double)g.spacing[k] / S;
        }
        for (int ix = 0; ix < S; ++ix)
          for (int iy = 0; iy < S; ++iy)
            for (int iz = 0; iz < S; ++iz) {
              const int ii[3] = {ix, iy, iz};
              double rd[3];
              for (int k = 0; k < 3; ++k)
                rd[k] = b.src[k] - (pos[k] - (double)g.spacing[k] / 2.0 + off[k] / 2.0 + off[k] * ii[k]);
              double px, pz;
              if (!project_d(b, rd, &px, &pz)) {
                bad = 1;
                continue;
              }
              const double cr = (double)floor_clamped(px * 100.0) + 2000.0;
              const double cc = (double)floor_clamped(pz * 100.0) + 2000.0;
              if (cr < 0 || cr > 3999 || cc < 0 || cc > 3999) continue;
              int64_t r = (int64_t)cr - 1, c = (int64_t)cc - 1;
              if (r < 0) r += b.block_rows;
              if (c < 0) c += b.block_cols;
              const int64_t i = r - r0, j = c - c0;
              if (i < 0 || j < 0 || i >= (int64_t)rows * cell_rows || j >= (int64_t)cols * cell_cols) continue;
              acc[(size_t)((i / cell_rows) * cols + j / cell_cols)] += cv / (double)(S * S * S);
            }
      }
    }
  for (int k = 0; k < nb; ++k) {
    double s = 0.0;
    for (int t = 0; t < nthr; ++t) s += priv[(size_t)t][(size_t)k];
    grad[k] = s;
  }
  return bad ? 1 : 0;
}

}  // namespace

extern "C" {

// Transposed cone computed only where support != 0 (0 elsewhere); see
// cone_transpose.
void or_cone_transpose_on(const or_grid* g, const double* r, const double* K, int n_r, const float* thetas,
                          int n_theta, const float* phis, int n_phi, int mode, const double* support,
                          double* out) {
  if (mode == 0) cone_transpose<float>(*g, r, K, n_r, thetas, n_theta, phis, n_phi, out, support);
  else cone_transpose<double>(*g, r, K, n_r, thetas, n_theta, phis, n_phi, out, support);
}

// Float64 transposed blocking onto a beamlet grid (see blocked_adjoint_f64);
// `grad` (rows * cols float64) is overwritten.  Returns 0, or 1 if a ray was
// parallel to the blocking plane.
int or_blocked_adjoint(const or_grid* g, const or_beam* b, int samples, const double* coef, int rows, int cols,
                       int cell_rows, int cell_cols, int r0, int c0, double* grad) {
  return blocked_adjoint_f64(*g, *b, samples, coef, rows, cols, cell_rows, cell_cols, r0, c0, grad);
}

// Cone stage with the physics extensions (see ConeExt): rho (float32, the
// phantom's densities, read with swap_xy like the TERMA pass) for the
// radiological distance, frame (3x3 row-major world->beam matrix) for cones
// in the beam frame; either may be null.
void or_cone_ext(const or_grid* g, const double* terma, const double* K, int n_r, const float* thetas,
                 int n_theta, const float* phis, int n_phi, int mode, const float* rho, int swap_xy,
                 const double* frame, double* dose) {
  ConeExt ext;
  ext.rho = rho;
  ext.swap_xy = swap_xy;
  ext.frame = frame;
  if (mode == 0) cone<float>(*g, terma, K, n_r, thetas, n_theta, phis, n_phi, dose, ext);
  else cone<double>(*g, terma, K, n_r, thetas, n_theta, phis, n_phi, dose, ext);
}

// Transposed collapsed-cone stage (see cone_transpose); `out` overwritten.
void or_cone_transpose(const or_grid* g, const double* r, const double* K, int n_r, const float* thetas,
                       int n_theta, const float* phis, int n_phi, int mode, double* out) {
  if (mode == 0) cone_transpose<float>(*g, r, K, n_r, thetas, n_theta, phis, n_phi, out);
  else cone_transpose<double>(*g, r, K, n_r, thetas, n_theta, phis, n_phi, out);
}

// Prologue: blocked, d_eff, oad, fluence, f_soften, f_horn and TERMA.
// All outputs are float64 arrays of n0*n1*n2 (any of the first six may be
// null).  Returns 0, or 1 if some ray was parallel to the blocking plane.
int or_prologue(const or_grid* g, const float* rho, int swap_xy, const or_beam* b,
                const or_settings* s, int mode, double* blocked, double* d_eff,
                double* oad, double* fluence, double* f_soften, double* f_horn,
                double* terma) {
  Outputs o{blocked, d_eff, oad, fluence, f_soften, f_horn, terma};
  if (mode == 0) return prologue_f32(*g, rho, swap_xy, *b, *s, o);
  return prologue_f64(*g, rho, swap_xy, *b, *s, o);
}

// Collapsed-cone scatter: dose[v] = sum over TERMA voxels s, directions
// (theta_i, phi_j) and DDA steps m of T(s) * dK_j[m].  K is the cumulative
// kernel [n_phi][n_r] (float64).  `dose` (float64, n0*n1*n2) is overwritten;
// contributions are summed in float64 (in mode 0 each contribution is first
// rounded to float32, as the reference's float32 atomic add does).
void or_cone(const or_grid* g, const double* terma, const double* K, int n_r,
             const float* thetas, int n_theta, const float* phis, int n_phi, int mode,
             double* dose) {
  if (mode == 0) cone<float>(*g, terma, K, n_r, thetas, n_theta, phis, n_phi, dose);
  else cone<double>(*g, terma, K, n_r, thetas, n_theta, phis, n_phi, dose);
}

// One DDA trace, for pinning against conehead's own dda_3d_c and the GPU
// trace hook.  Writes up to `cap` voxels (xyz triples) and exit t-values;
// returns the full path length.
int or_dda(const int* n, const float* spacing, const int* start, const double* dir,
           int mode, int cap, int* voxels, double* tvals) {
  int count = 0;
  auto rec = [&](const int* c, double t) {
    if (count < cap) {
      voxels[3 * count + 0] = c[0];
      voxels[3 * count + 1] = c[1];
      voxels[3 * count + 2] = c[2];
      tvals[count] = t;
    }
    ++count;
  };
  if (mode == 0) {
    float d[3] = {(float)dir[0], (float)dir[1], (float)dir[2]};
    dda_walk<float>(start, d, spacing, n, [&](const int* c, float t) { rec(c, (double)t); });
  } else {
    double d[3] = {dir[0], dir[1], dir[2]};
    dda_walk<double>(start, d, spacing, n, [&](const int* c, double t) { rec(c, t); });
  }
  return count;
}

// Cone direction (theta, phi in degrees) as the reference computes it.
void or_cone_direction(float theta, float phi, int mode, double* out) {
  if (mode == 0) {
    float d[3];
    cone_direction<float>(theta, phi, d);
    for (int k = 0; k < 3; ++k) out[k] = d[k];
  } else {
    cone_direction<double>(theta, phi, out);
  }
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
