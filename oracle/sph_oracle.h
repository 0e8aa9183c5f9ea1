/*
 * sph_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * The oracle: a plain-C restatement of the reference's SPH step on the CPU,
 * used by tests/ as the parity checker, by __graft_entry__.smoke() as its
 * check, and by bench.py as the timed CPU baseline.  The product never links
 * or calls it.
 *
 * All arrays are host arrays.  Positions and velocities are float4 records
 * (x, y, z, w) stored as 4 consecutive floats; key/value pairs are (hash,
 * index) uint32 pairs, the reference's uint2 particleHash layout.
 *
 * Two arithmetic modes:
 *   _f32  single precision, every operation an explicit IEEE round-to-nearest
 *         step in a fixed order (built with -ffp-contract=off, fused
 *         multiply-adds only where fmaf() is written);
 *   _f64  double precision on the same float inputs, the accuracy reference
 *         for the GPU kernels' single-precision results.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>
#include "sph_params.h"

#ifdef __cplusplus
extern "C" {
#endif

/* calcGridPos/calcGridHash/calcHashD (Kernel_Cell.cui:5-34). */
void orc_calc_hash(const SimParams* p, const float* pos, uint32_t n, uint32_t* kv);

/* RadixSort (radixsort_kernel.cu:445-472): stable sort of (key, value)
   pairs by the low `bits` bits of the key (bits rounded up to whole bytes,
   as the reference loops shift = 0, 8, ... < bits). */
void orc_sort_pairs(uint32_t* kv, uint32_t n, uint32_t bits);

/* reorderD + memset (Kernel_Cell.cui:40-67, System.cu:689-713): cellStart of
   every cell (0xFFFFFFFF when empty) and pos/vel gathered to sorted order. */
void orc_reorder(const SimParams* p, const uint32_t* kv, const float* pos, const float* vel,
                 uint32_t n, float* sorted_pos, float* sorted_vel, uint32_t* cell_start);

/* computeDensityD (Kernel_Cell.cui:142-199), sorted order.  nbr (optional)
   receives, per particle, the number of pairs with r^2 < h^2. */
void orc_density_f32(const SimParams* p, const float* sorted_pos, const uint32_t* kv,
                     const uint32_t* cell_start, uint32_t n, float* density, float* pressure);
void orc_density_f64(const SimParams* p, const float* sorted_pos, const uint32_t* kv,
                     const uint32_t* cell_start, uint32_t n, double* density, double* pressure,
                     int32_t* nbr);

/* computeForceD core (System.cu:228-250, 374-402 with Kernel_Cell.cui:
   78-96, 210-261): new velocity of every particle written in original order
   through kv[i].y.  The _f64 form also returns, per particle, the sum of the
   magnitudes of the velocity increments that were added up (the scale a
   relative tolerance on the sum is stated against). */
void orc_force_f32(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                   const float* density, const float* pressure, const uint32_t* kv,
                   const uint32_t* cell_start, uint32_t n, float* new_vel);
void orc_force_f64(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                   const double* density, const double* pressure, const uint32_t* kv,
                   const uint32_t* cell_start, uint32_t n, double* new_vel, double* scale);

/* The whole computeForceD in single precision: orc_force_f32 plus the
   colour and dye outputs (System.cu:405-546, including the CLR_Vel foam
   estimate and its second neighbour walk), both in original order. */
void orc_force_color_f32(const SimParams* p, const float* sorted_pos, const float* sorted_vel,
                         const float* density, const float* pressure, const uint32_t* kv,
                         const uint32_t* cell_start, uint32_t n, float* new_vel, float* dye,
                         float* clr);

/* integrateD with boundary() (System.cu:41-205). */
void orc_integrate_f32(const SimParams* p, const float* pos, const float* vel, uint32_t n,
                       float* new_pos, float* new_vel);
void orc_integrate_f64(const SimParams* p, const float* pos, const float* vel, uint32_t n,
                       double* new_pos, double* new_vel);

/* One cSPH::Update (SPH_Update.cpp:12-81) per step, single precision, on
   pos/vel in original order (updated in place).  Internally a stable
   counting sort stands in for the radix sort (same order) and the particle
   loops run on `threads` OpenMP threads (<= 0: all).  Returns 0, or -1 when
   a work buffer could not be allocated. */
int orc_step_f32(const SimParams* p, float* pos, float* vel, uint32_t n, uint32_t steps,
                 int threads);

/* The same steps with positions and velocities held in double and every
   stage evaluated in double: the reference trajectory a single-precision run
   is measured against (kinetic energy and mean-density drift).
   *mean_density (if not NULL) gets the mean of the last step's densities.
   Returns 0, or -1 when a work buffer could not be allocated. */
int orc_step_d64(const SimParams* p, double* pos, double* vel, uint32_t n, uint32_t steps,
                 double* mean_density);

/* Number of OpenMP threads a parallel region would use. */
int orc_threads(void);

/* Kinetic energy sum(0.5 m |v|^2) and mean density, in double. */
void orc_reduce(const SimParams* p, const float* vel, const float* density, uint32_t n,
                double* out2);

#ifdef __cplusplus
}
#endif
#endif
