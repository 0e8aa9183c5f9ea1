/*
 * sph_params.h -- the simulation-parameter block shared by the host, the C ABI
 * and the device kernels.
 *
 * The struct is byte-for-byte the layout of the reference's `struct SimParams`
 * (source/CUDA/Params.cuh:53-114), so a caller that fills the reference struct
 * can hand the same bytes to this library.  Field names, order and types are
 * kept identical on purpose: this is an ABI, not a design choice.  Enumerations
 * (Params.cuh:24-41) are 32-bit integers here; the reference's enums are
 * 32-bit because each has a 0xFFFFFFFF sentinel member.
 *
 * Plain C: no CUDA headers are needed to include this file.
 */
#ifndef PIBITI_SPH_PARAMS_H
#define PIBITI_SPH_PARAMS_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__CUDACC__)
#include <vector_types.h>
typedef float3 sph_float3;
typedef float4 sph_float4;
typedef uint3 sph_uint3;
typedef int3 sph_int3;
typedef uint2 sph_uint2;
#else
typedef struct { float x, y, z; } sph_float3;
typedef struct __attribute__((aligned(16))) { float x, y, z, w; } sph_float4;
typedef struct { uint32_t x, y, z; } sph_uint3;
typedef struct { int32_t x, y, z; } sph_int3;
typedef struct __attribute__((aligned(8))) { uint32_t x, y; } sph_uint2;
#endif

/* BndType (Params.cuh:24) */
#define SPH_BND_BOX 0
#define SPH_BND_CYL_Y 1
#define SPH_BND_CYL_Z 2
#define SPH_BND_CYL_YZ 3
#define SPH_BND_SPHERE 4
#define SPH_BND_PUMP_Y 5
/* BndEff (Params.cuh:28) */
#define SPH_BND_EFF_NONE 0
#define SPH_BND_EFF_WRAP 1
#define SPH_BND_EFF_CYCLE 2
#define SPH_BND_EFF_WAVE 3
/* ClrType (Params.cuh:32) */
#define SPH_CLR_DENS 0
#define SPH_CLR_ACCEL 1
#define SPH_CLR_DENSACC 2
#define SPH_CLR_VEL 3
#define SPH_CLR_VELACC 4
#define SPH_CLR_VELRGB 5
#define SPH_CLR_NONE 6
/* AccType (Params.cuh:40) */
#define SPH_ACC_OFF 0
#define SPH_ACC_BOX 1
#define SPH_ACC_CYLY 2
#define SPH_ACC_CYLYSM 3

#define SPH_NUM_ACC 4 /* Params.cuh:50 */

/* struct Accel (Params.cuh:44-48) */
typedef struct {
  sph_float3 pos, size, acc;
  uint32_t type;
} SphAccel;

/* struct SimParams (Params.cuh:53-114), same field order and widths. */
typedef struct {
  /* simulation */
  float timeStep;
  uint32_t numParticles, maxParInCell;
  sph_float3 gravity;
  float globalDamping;
  /* grid */
  sph_uint3 gridSize;
  sph_float3 cellSize;
  uint32_t gridSize_yx, numCells;
  /* world */
  sph_float3 worldMin, worldMax, worldSize, worldMinD, worldMaxD, worldSizeD;
  /* SPH */
  float particleR, h, h2;
  float SpikyKern, LapKern, Poly6Kern;
  float particleMass, restDensity, stiffness, viscosity, minDens, minDist;
  /* boundary */
  float distBndHard, distBndSoft;
  float bndDamp, bndStiff, bndDampC;
  uint32_t bndType, bndEffZ;
  /* sphere collider */
  sph_float4 collPos;
  float collR;
  float spring, damping, shear;
  /* visual */
  uint32_t clrType;
  int32_t iHue;
  float brightness, contrast;
  /* dye */
  int32_t dyeType, dyeClear;
  float dyeFade;
  sph_float3 dyePos, dyeSize;
  /* accelerators */
  SphAccel acc[SPH_NUM_ACC];
  int32_t iHmap;
  /* pump */
  float angOut, hClose, radIn;
  float rVexit, rDexit, s1, s2, s3, s4, s5, s6;
  /* rotor */
  float rAngle, rTwist;
  int32_t rotType, rotBlades;
  sph_int3 rotSize;
  float rotR, rotSpc;
  float r2Dist, r2Angle, r2twist, ff2;
} SimParams;

/* Offsets of the reference layout, checked at compile time. */
#if defined(__cplusplus)
#define SPH_STATIC_ASSERT static_assert
#else
#define SPH_STATIC_ASSERT _Static_assert
#endif
SPH_STATIC_ASSERT(offsetof(SimParams, gravity) == 12, "SimParams.gravity");
SPH_STATIC_ASSERT(offsetof(SimParams, gridSize) == 28, "SimParams.gridSize");
SPH_STATIC_ASSERT(offsetof(SimParams, numCells) == 56, "SimParams.numCells");
SPH_STATIC_ASSERT(offsetof(SimParams, worldMin) == 60, "SimParams.worldMin");
SPH_STATIC_ASSERT(offsetof(SimParams, particleR) == 132, "SimParams.particleR");
SPH_STATIC_ASSERT(offsetof(SimParams, bndType) == 200, "SimParams.bndType");
SPH_STATIC_ASSERT(offsetof(SimParams, collPos) == 208, "SimParams.collPos");
SPH_STATIC_ASSERT(offsetof(SimParams, clrType) == 240, "SimParams.clrType");
SPH_STATIC_ASSERT(offsetof(SimParams, acc) == 292, "SimParams.acc");
SPH_STATIC_ASSERT(offsetof(SimParams, iHmap) == 452, "SimParams.iHmap");
SPH_STATIC_ASSERT(offsetof(SimParams, rotSize) == 516, "SimParams.rotSize");
SPH_STATIC_ASSERT(offsetof(SimParams, ff2) == 548, "SimParams.ff2");
SPH_STATIC_ASSERT(sizeof(SimParams) == 560, "SimParams size");

#ifdef __cplusplus
}
#endif
#endif /* PIBITI_SPH_PARAMS_H */
