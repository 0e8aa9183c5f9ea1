/*
 * sph_oracle.c -- TEST INFRASTRUCTURE ONLY (see sph_oracle.h).
 *
 * CPU restatement of the reference's SPH step.  Integer work (hash, sort,
 * cell starts) is exact; the floating-point stages come from
 * sph_oracle_core.inc in single and double precision.  Build with
 * -ffp-contract=off so that the single-precision forms round exactly as
 * written (oracle/Makefile).
 */
#include "sph_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- integer helpers shared by both precisions ------------------------ */

/* __mul24: product of the low 24 bits of each operand, sign-extended. */
static inline int32_t mul24(int32_t a, int32_t b) {
  int32_t sa = (int32_t)((uint32_t)a << 8) >> 8;
  int32_t sb = (int32_t)((uint32_t)b << 8) >> 8;
  return (int32_t)(uint32_t)((int64_t)sa * (int64_t)sb);
}

/* float -> int as the GPU converts it: saturating, NaN -> 0. */
static inline int32_t f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f < -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

/* calcGridPos (Kernel_Cell.cui:5-13): floor((p - worldMin) / cellSize),
   component-wise IEEE division. */
static inline void grid_pos(const SimParams* p, const float* pos4, int g[3]) {
  const float gx = (pos4[0] - p->worldMin.x) / p->cellSize.x;
  const float gy = (pos4[1] - p->worldMin.y) / p->cellSize.y;
  const float gz = (pos4[2] - p->worldMin.z) / p->cellSize.z;
  g[0] = f2i_sat(floorf(gx));
  g[1] = f2i_sat(floorf(gy));
  g[2] = f2i_sat(floorf(gz));
}

/* The same cell lookup for positions held in double (the double-precision
   trajectory): floor((p - worldMin) / cellSize) in double. */
static inline int32_t f2i_sat_d(double f) {
  if (f != f) return 0;
  if (f >= 2147483648.0) return INT32_MAX;
  if (f < -2147483648.0) return INT32_MIN;
  return (int32_t)f;
}
static inline void grid_pos_d(const SimParams* p, const double* pos4, int g[3]) {
  g[0] = f2i_sat_d(floor((pos4[0] - (double)p->worldMin.x) / (double)p->cellSize.x));
  g[1] = f2i_sat_d(floor((pos4[1] - (double)p->worldMin.y) / (double)p->cellSize.y));
  g[2] = f2i_sat_d(floor((pos4[2] - (double)p->worldMin.z) / (double)p->cellSize.z));
}

/* calcGridHash (Kernel_Cell.cui:15-19): z * (gx*gy) + y * gx + x with
   24-bit multiplies; out-of-grid coordinates wrap exactly as there. */
static inline uint32_t grid_hash(const SimParams* p, int x, int y, int z) {
  return (uint32_t)(mul24(z, (int32_t)p->gridSize_yx) + mul24(y, (int32_t)p->gridSize.x) + x);
}

/* FETCH(cellStart, h) through a texture bound to numCells entries: a fetch
   outside the array reads 0 (Params.cuh:5-14, System.cu:732). */
static inline uint32_t fetch_cell_start(const uint32_t* cs, uint32_t num_cells, uint32_t h) {
  const int32_t x = (int32_t)h;
  return (x >= 0 && (uint32_t)x < num_cells) ? cs[x] : 0u;
}

/* FETCH(particleHash, j).x through a texture bound to n entries.  The
   walks stop at j >= n: there the reference's texture returns a zero key and
   zero particle, which a walk of cell 0 would take for a particle at the
   origin (only when every particle sits in cell 0); the oracle and the
   product stop instead. */
static inline uint32_t fetch_key(const uint32_t* kv, uint32_t n, uint32_t j) {
  const int32_t x = (int32_t)j;
  return (x >= 0 && (uint32_t)x < n) ? kv[2 * (size_t)x] : 0u;
}

/* ---- floating-point stages, instantiated per precision ---------------- */
#define REAL float
#define PIN float
#define GRID_POS grid_pos
#define SFX(name) name##_f32
#define FMA(a, b, c) fmaf((a), (b), (c))
#define SQRT(a) sqrtf(a)
#define SIN(a) sinf(a)
#define COS(a) cosf(a)
#define ATAN(a) atanf(a)
#define FABS(a) fabsf(a)
#include "sph_oracle_core.inc"
#undef REAL
#undef SFX
#undef FMA
#undef SQRT
#undef SIN
#undef COS
#undef ATAN
#undef FABS
#undef PIN
#undef GRID_POS

#define REAL double
#define PIN float
#define GRID_POS grid_pos
#define SFX(name) name##_f64
#define FMA(a, b, c) fma((a), (b), (c))
#define SQRT(a) sqrt(a)
#define SIN(a) sin(a)
#define COS(a) cos(a)
#define ATAN(a) atan(a)
#define FABS(a) fabs(a)
#include "sph_oracle_core.inc"
#undef SFX
#undef PIN
#undef GRID_POS
#define PIN double
#define GRID_POS grid_pos_d
#define SFX(name) name##_d64
#include "sph_oracle_core.inc"
#undef REAL
#undef SFX
#undef PIN
#undef GRID_POS
#undef FMA
#undef SQRT
#undef SIN
#undef COS
#undef ATAN
#undef FABS

/* ---- public stages ----------------------------------------------------- */

void orc_calc_hash(const SimParams* p, const float* pos, uint32_t n, uint32_t* kv) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    int g[3];
    grid_pos(p, pos + 4 * i, g);
    kv[2 * i] = grid_hash(p, g[0], g[1], g[2]);
    kv[2 * i + 1] = (uint32_t)i;
  }
}

/* LSD radix sort on 8-bit digits, one stable counting pass per digit, like
   RadixSum / RadixPrefixSum / RadixAddOffsetsAndShuffle do per pass. */
void orc_sort_pairs(uint32_t* kv, uint32_t n, uint32_t bits) {
  if (n == 0) return;
  uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n);
  if (!tmp) abort();
  uint32_t* src = kv;
  uint32_t* dst = tmp;
  for (uint32_t shift = 0; shift < bits; shift += 8) {
    size_t count[257];
    memset(count, 0, sizeof(count));
    for (uint32_t i = 0; i < n; ++i) count[((src[2 * i] >> shift) & 0xff) + 1]++;
    for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
    for (uint32_t i = 0; i < n; ++i) {
      const size_t o = count[(src[2 * i] >> shift) & 0xff]++;
      dst[2 * o] = src[2 * i];
      dst[2 * o + 1] = src[2 * i + 1];
    }
    uint32_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != kv) memcpy(kv, src, sizeof(uint32_t) * 2 * (size_t)n);
  free(tmp);
}

void orc_reorder(const SimParams* p, const uint32_t* kv, const float* pos, const float* vel,
                 uint32_t n, float* sorted_pos, float* sorted_vel, uint32_t* cell_start) {
  memset(cell_start, 0xff, sizeof(uint32_t) * (size_t)p->numCells);
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t h = kv[2 * i];
    /* reorderD writes cellStart[hash] unchecked; hashes outside the grid
       would write outside the array there and are skipped here. */
    if ((i == 0 || h != kv[2 * (i - 1)]) && h < p->numCells) cell_start[h] = i;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const uint32_t j = kv[2 * i + 1];
    memcpy(sorted_pos + 4 * i, pos + 4 * (size_t)j, 16);
    memcpy(sorted_vel + 4 * i, vel + 4 * (size_t)j, 16);
  }
}

void orc_density_f32(const SimParams* p, const float* sorted_pos, const uint32_t* kv,
                     const uint32_t* cell_start, uint32_t n, float* density, float* pressure) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    density_one_f32(p, sorted_pos, kv, cell_start, n, (uint32_t)i, density + i, pressure + i, 0);
}

void orc_density_f64(const SimParams* p, const float* sorted_pos, const uint32_t* kv,
                     const uint32_t* cell_start, uint32_t n, double* density, double* pressure,
                     int32_t* nbr) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    density_one_f64(p, sorted_pos, kv, cell_start, n, (uint32_t)i, density + i, pressure + i,
                    nbr ? nbr + i : 0);
}

void orc_force_f32(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                   const float* density, const float* pressure, const uint32_t* kv,
                   const uint32_t* cell_start, uint32_t n, float* new_vel) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const uint32_t si = kv[2 * i + 1];
    force_one_f32(p, sorted_pos, sorted_vel, density, pressure, kv, cell_start, n, (uint32_t)i,
                  new_vel + 4 * (size_t)si, 0, 0);
  }
}

void orc_force_f64(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                   const double* density, const double* pressure, const uint32_t* kv,
                   const uint32_t* cell_start, uint32_t n, double* new_vel, double* scale) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const uint32_t si = kv[2 * i + 1];
    force_one_f64(p, sorted_pos, sorted_vel, density, pressure, kv, cell_start, n, (uint32_t)i,
                  new_vel + 4 * (size_t)si, 0, scale ? scale + si : 0);
  }
}

/* FETCH of a float4 array through a texture bound to n entries: zeros
   outside it. */
static inline void fetch4(const float* a, uint32_t n, uint32_t j, float out[4]) {
  const int32_t x = (int32_t)j;
  if (x >= 0 && (uint32_t)x < n) memcpy(out, a + 4 * (size_t)x, 16);
  else out[0] = out[1] = out[2] = out[3] = 0.f;
}

static inline float dot4(const float* a, const float* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

/* The trapped-air sum of the CLR_Vel foam estimate (System.cu:429-470):
   cells visited x outermost, then y, then z; each walk re-fetches the cell
   start (an empty cell reads 0xFFFFFFFF, so the walk starts at index -1,
   whose texture fetch returns zeros: for cell 0 that zero record is taken
   as a particle at the origin at rest); float4 normalise and dot include w;
   weight W(x, 3) = (1 - x) / 3. */
static float foam_vdiff(const SimParams* p, const float* spos, const float* svel,
                        const uint32_t* kv, const uint32_t* cs, uint32_t n, uint32_t index) {
  const float* pi = spos + 4 * (size_t)index;
  const float* vi = svel + 4 * (size_t)index;
  int g[3];
  grid_pos(p, pi, g);
  float vdiff = 0.0f;
  for (int x = -1; x < 2; ++x)
    for (int y = -1; y < 2; ++y)
      for (int z = -1; z < 2; ++z)
        for (uint32_t i = 0; i < p->maxParInCell; ++i) {
          const uint32_t gh = grid_hash(p, g[0] + x, g[1] + y, g[2] + z);
          const uint32_t start = fetch_cell_start(cs, p->numCells, gh);
          const uint32_t j = start + i;
          if (fetch_key(kv, n, j) != gh) break;
          if (j == index) continue;
          float v2[4], x2[4], sv[4], sx[4], dv[4], dx[4];
          fetch4(svel, n, j, v2);
          fetch4(spos, n, j, x2);
          for (int k = 0; k < 4; ++k) {
            sv[k] = vi[k] + v2[k];
            sx[k] = pi[k] + x2[k];
            dv[k] = vi[k] - v2[k];
            dx[k] = pi[k] - x2[k];
          }
          const float iv = 1.0f / sqrtf(dot4(sv, sv)), ix = 1.0f / sqrtf(dot4(sx, sx));
          for (int k = 0; k < 4; ++k) {
            sv[k] = sv[k] * iv;
            sx[k] = sx[k] * ix;
          }
          const float r = sqrtf(dot4(dx, dx));
          const float w = r <= 3.0f ? (1 - r) / 3.0f : 0.0f;
          vdiff = vdiff + sqrtf(dot4(dv, dv)) * (1.0f - dot4(sv, sx)) * w;
        }
  return vdiff;
}

static inline float phi_clamp(float I, float tmin, float tmax) {
  return (fminf(I, tmax) - fminf(I, tmin)) / (tmax - tmin);
}

/* Colour and dye of computeForceD (System.cu:405-546) for one particle.
   `add` is the velocity increment the force pass produced, `vdiff` the
   foam sum (CLR_Vel only). */
static void color_one(const SimParams* p, const float* pos4, const float* vel4, float dens,
                      R3_f32 add, float vdiff, float* dye, float* clr4) {
  float cx = 0.2f, cy = 0.5f, cz = 1.f, intens = 0.f;
  const float dt = p->timeStep;
  switch (p->clrType) {
    case SPH_CLR_NONE:
      return;
    case SPH_CLR_VEL: {
      const float v = 2.5f * len3_f32(r3_f32(vel4[0], vel4[1], vel4[2]));
      const float clrV = p->brightness + p->contrast * v;
      intens = clrV;
      const float trapped = phi_clamp(vdiff, 5.0f, 20.0f);
      const float kEnergy = (float)((double)(p->particleMass * 1000 * dot4(vel4, vel4)) * 0.5);
      const float kPot = phi_clamp(kEnergy, 0.1f, 1.0f);
      const float Nd = kPot * (3.0f * trapped + 3.0f * 0.0f);
      cx = cy = cz = Nd;
    } break;
    case SPH_CLR_VELACC: {
      const float v = 2.5f * len3_f32(r3_f32(vel4[0], vel4[1], vel4[2]));
      const float f = 0.02f * len3_f32(add) / dt;
      const float clrV = p->brightness + p->contrast * v;
      const float clrF = p->contrast * f;
      cx = cx * clrV + 0.7f * clrF;
      cy = cy * clrV + 0.35f * clrF;
      cz = cz * clrV + 0.f * clrF;
    } break;
    case SPH_CLR_DENSACC: {
      const float d = 4.f * (dens - p->restDensity) / p->restDensity;
      const float f = 0.02f * len3_f32(add) / dt;
      const float clrD = p->brightness + p->contrast * d;
      const float clrF = p->contrast * f;
      cx = cx * clrD + 0.7f * clrF;
      cy = cy * clrD + 0.7f * clrF;
      cz = cz * clrD + 0.f * clrF;
    } break;
    case SPH_CLR_VELRGB: {
      const float s = p->contrast * 2.5f;
      cx = 0.5f + s * vel4[0];
      cy = 0.5f + s * vel4[1];
      cz = 0.5f + s * vel4[2];
    } break;
    case SPH_CLR_ACCEL: {
      const float f = 0.02f * len3_f32(add) / dt;
      const float clrF = p->brightness + p->contrast * f;
      intens = clrF;
      cx *= clrF;
      cy *= clrF;
      cz *= clrF;
    } break;
    case SPH_CLR_DENS: {
      const float d = 4.f * (dens - p->restDensity) / p->restDensity;
      const float clrD = p->brightness + p->contrast * d;
      intens = clrD;
      cx *= clrD;
      cy *= clrD;
      cz *= clrD;
    } break;
    default:
      return;
  }
  if (p->iHue == 1) {
    cx = intens;
    cy = 0.f;
  }
  if (p->dyeClear > 0) {
    *dye = 0.f;
  } else if (p->dyeType > 0) {
    float dyeCl = *dye;
    const float rx = pos4[0] - p->dyePos.x, ry = pos4[1] - p->dyePos.y, rz = pos4[2] - p->dyePos.z;
    if (p->dyeType == 1) {
      if (fabsf(rx) < p->dyeSize.x && fabsf(ry) < p->dyeSize.y && fabsf(rz) < p->dyeSize.z) dyeCl = 1.f;
    } else if (p->dyeType == 2) {
      if (len3_f32(r3_f32(rx, ry, rz)) < p->dyeSize.y) dyeCl = 1.f;
    }
    dyeCl -= dt * p->dyeFade;
    if (dyeCl < 0.f) dyeCl = 0.f;
    if (dyeCl >= 0.f) *dye = dyeCl;
    if (p->iHue == 0) {
      cx += 0.9f * dyeCl;
      cy += 0.9f * dyeCl;
      cz += 1.f * dyeCl;
    } else {
      cy = dyeCl;
    }
  }
  clr4[0] = cx;
  clr4[1] = cy;
  clr4[2] = cz;
  clr4[3] = 1.f;
}

/* Force pass plus colour/dye, single precision, the whole computeForceD. */
void orc_force_color_f32(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                         const float* density, const float* pressure, const uint32_t* kv,
                         const uint32_t* cell_start, uint32_t n, float* new_vel, float* dye,
                         float* clr) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const uint32_t si = kv[2 * i + 1];
    R3_f32 add;
    force_one_f32(p, sorted_pos, sorted_vel, density, pressure, kv, cell_start, n, (uint32_t)i,
                  new_vel + 4 * (size_t)si, &add, 0);
    if (clr && dye) {
      const float vdiff = p->clrType == SPH_CLR_VEL
                              ? foam_vdiff(p, sorted_pos, sorted_vel, kv, cell_start, n, (uint32_t)i)
                              : 0.f;
      color_one(p, sorted_pos + 4 * i, sorted_vel + 4 * i, density[i], add, vdiff, dye + si,
                clr + 4 * (size_t)si);
    }
  }
}

/* ---- whole step (CPU baseline) ----------------------------------------- */

int orc_step_f32(const SimParams* p, float* pos, float* vel, uint32_t n, uint32_t steps,
                 int threads) {
#ifdef _OPENMP
  const int saved = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const size_t f4 = sizeof(float) * 4 * (size_t)n;
  float* npos = (float*)malloc(f4);
  float* nvel = (float*)malloc(f4);
  float* spos = (float*)malloc(f4);
  float* svel = (float*)malloc(f4);
  float* dens = (float*)malloc(sizeof(float) * (size_t)n);
  float* pres = (float*)malloc(sizeof(float) * (size_t)n);
  uint32_t* kv = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n);
  uint32_t* kv2 = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n);
  uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)p->numCells + 1));
  int rc = 0;
  if (!npos || !nvel || !spos || !svel || !dens || !pres || !kv || !kv2 || !cs) {
    rc = -1;
    goto done;
  }
  for (uint32_t s = 0; s < steps; ++s) {
    /* integrate (SPH_Update.cpp:39-47) */
    orc_integrate_f32(p, pos, vel, n, npos, nvel);
    memcpy(pos, npos, f4);
    memcpy(vel, nvel, f4);
    /* calcHash + sort (SPH_Update.cpp:56-58): a stable counting sort by
       cell gives the order the radix sort gives when every hash lies in
       the grid; otherwise the radix restatement runs. */
    orc_calc_hash(p, pos, n, kv);
    int in_grid = 1;
    for (uint32_t i = 0; i < n; ++i)
      if (kv[2 * i] >= p->numCells) in_grid = 0;
    if (in_grid) {
      memset(cs, 0, sizeof(uint32_t) * ((size_t)p->numCells + 1));
      for (uint32_t i = 0; i < n; ++i) cs[kv[2 * i] + 1]++;
      for (uint32_t c = 0; c < p->numCells; ++c) cs[c + 1] += cs[c];
      for (uint32_t i = 0; i < n; ++i) {
        const uint32_t o = cs[kv[2 * i]]++;
        kv2[2 * o] = kv[2 * i];
        kv2[2 * o + 1] = kv[2 * i + 1];
      }
      memcpy(kv, kv2, sizeof(uint32_t) * 2 * (size_t)n);
    } else {
      orc_sort_pairs(kv, n, p->numCells >= 65536 ? 32 : 16);
    }
    /* reorder, density, force (SPH_Update.cpp:65-80) */
    orc_reorder(p, kv, pos, vel, n, spos, svel, cs);
    orc_density_f32(p, spos, kv, cs, n, dens, pres);
    orc_force_f32(p, spos, svel, dens, pres, kv, cs, n, vel);
  }
done:
  free(npos); free(nvel); free(spos); free(svel); free(dens); free(pres);
  free(kv); free(kv2); free(cs);
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return rc;
}

/* cSPH::Update (SPH_Update.cpp:12-81) with the whole state in double:
   integrate, cell of each position (double, clamped into the grid), stable
   sort by (cell, index), reorder, density, force.  The reference trajectory
   a single-precision run is measured against; every arithmetic step is the
   restatement of the single-precision oracle evaluated in double.
   *mean_density (if not NULL) gets the mean of the last step's densities. */
int orc_step_d64(const SimParams* p, double* pos, double* vel, uint32_t n, uint32_t steps,
                 double* mean_density) {
  const size_t d4 = sizeof(double) * 4 * (size_t)n;
  double* npos = (double*)malloc(d4);
  double* nvel = (double*)malloc(d4);
  double* spos = (double*)malloc(d4);
  double* svel = (double*)malloc(d4);
  double* dens = (double*)malloc(sizeof(double) * (size_t)n);
  double* pres = (double*)malloc(sizeof(double) * (size_t)n);
  uint32_t* kv = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n);
  uint32_t* kv2 = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n);
  uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)p->numCells + 1));
  int rc = 0;
  if (!npos || !nvel || !spos || !svel || !dens || !pres || !kv || !kv2 || !cs) {
    rc = -1;
    goto done;
  }
  for (uint32_t s = 0; s < steps; ++s) {
    orc_integrate_d64(p, pos, vel, n, npos, nvel);
    memcpy(pos, npos, d4);
    memcpy(vel, nvel, d4);
    memset(cs, 0, sizeof(uint32_t) * ((size_t)p->numCells + 1));
    for (uint32_t i = 0; i < n; ++i) {
      int g[3];
      grid_pos_d(p, pos + 4 * (size_t)i, g);
      for (int k = 0; k < 3; ++k) {
        const int lim = (int)(k == 0 ? p->gridSize.x : (k == 1 ? p->gridSize.y : p->gridSize.z)) - 1;
        g[k] = g[k] < 0 ? 0 : (g[k] > lim ? lim : g[k]);
      }
      kv[2 * i] = grid_hash(p, g[0], g[1], g[2]);
      kv[2 * i + 1] = i;
      cs[kv[2 * i] + 1]++;
    }
    for (uint32_t c = 0; c < p->numCells; ++c) cs[c + 1] += cs[c];
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t o = cs[kv[2 * i]]++;
      kv2[2 * o] = kv[2 * i];
      kv2[2 * o + 1] = kv[2 * i + 1];
    }
    memcpy(kv, kv2, sizeof(uint32_t) * 2 * (size_t)n);
    memset(cs, 0xff, sizeof(uint32_t) * (size_t)p->numCells);
    for (uint32_t i = 0; i < n; ++i)
      if (i == 0 || kv[2 * i] != kv[2 * (i - 1)]) cs[kv[2 * i]] = i;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const uint32_t j = kv[2 * i + 1];
      memcpy(spos + 4 * i, pos + 4 * (size_t)j, 32);
      memcpy(svel + 4 * i, vel + 4 * (size_t)j, 32);
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)n; ++i)
      density_one_d64(p, spos, kv, cs, n, (uint32_t)i, dens + i, pres + i, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const uint32_t si = kv[2 * i + 1];
      force_one_d64(p, spos, svel, dens, pres, kv, cs, n, (uint32_t)i, vel + 4 * (size_t)si, 0, 0);
    }
    if (mean_density && s + 1 == steps) {
      double sum = 0;
      for (uint32_t i = 0; i < n; ++i) sum += dens[i];
      *mean_density = n ? sum / n : 0.0;
    }
  }
done:
  free(npos); free(nvel); free(spos); free(svel); free(dens); free(pres);
  free(kv); free(kv2); free(cs);
  return rc;
}

void orc_reduce(const SimParams* p, const float* vel, const float* density, uint32_t n,
                double* out2) {
  double ke = 0, rho = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const double vx = vel[4 * i], vy = vel[4 * i + 1], vz = vel[4 * i + 2];
    ke += 0.5 * (double)p->particleMass * (vx * vx + vy * vy + vz * vz);
    if (density) rho += density[i];
  }
  out2[0] = ke;
  out2[1] = n ? rho / n : 0.0;
}

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
