/*
 * pibiti_sph.h -- C ABI of the GB300 SPH step (libpibiti_sph.so).
 *
 * Two layers, both plain C with no CUDA or torch types in the signatures
 * (streams are passed as `void*` holding a cudaStream_t; NULL means the
 * legacy default stream):
 *
 *  1. Stage entry points with the argument lists of the reference's own
 *     extern "C" wrappers (source/CUDA/System.cuh:1-38,
 *     source/CUDA/radixsort.cuh:30-32), with OpenGL buffer ids replaced by
 *     device pointers.  A program that called the reference's wrappers calls
 *     these in the same order (cSPH::Update, source/SPH/SPH_Update.cpp:12-81)
 *     and gets the same buffers back.  Device buffers belong to the caller.
 *
 *  2. A system handle (the replacement for cSPH, source/SPH/SPH.h:9-50)
 *     that owns its device buffers and runs whole steps with fused kernels:
 *     sph_create / sph_set_array / sph_get_array / sph_step / sph_destroy.
 *     One handle can hold many independent scenes (an ensemble) stepped
 *     together.
 *
 * Every function returns an int status (SPH_OK = 0).  The reference exits
 * the process on any CUDA error (cutil.h CUDA_SAFE_CALL); this library
 * returns SPH_ERR_CUDA instead and sph_last_error() describes it.
 * Calls are asynchronous on their stream unless stated otherwise.
 */
#ifndef PIBITI_SPH_H
#define PIBITI_SPH_H

#include <stddef.h>
#include <stdint.h>

#include "sph_params.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SPH_OK 0
#define SPH_ERR_CUDA 1        /* a CUDA call failed (context may be unusable) */
#define SPH_ERR_ARG 2         /* bad pointer, size or index */
#define SPH_ERR_PARAMS 3      /* SimParams inconsistent or outside what the kernels cover */
#define SPH_ERR_UNSUPPORTED 4 /* a reference feature this library does not implement */
#define SPH_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define SPH_ERR_NOMEM 6       /* device or host allocation failed */
#define SPH_ERR_STATE 7       /* call not valid in the current state */
#define SPH_ERR_XML 8         /* scene file missing or malformed */

/* Text of the last error raised on the calling host thread. */
const char* sph_last_error(void);
/* Library version string. */
const char* sph_version(void);

/* ======================================================================
 * 1. Stage entry points (reference wrappers)
 * ==================================================================== */

/* threadSync (System.cu:613): wait for all device work. */
int sph_threadSync(void);
/* allocateArray / freeArray (System.cu:616-617). */
int sph_allocateArray(void** devPtr, size_t size);
int sph_freeArray(void* devPtr);
/* copyFromDevice (System.cu:623-628) without the VBO id; copyToDevice
   (System.cu:629-632).  Synchronous, like the reference. */
int sph_copyFromDevice(void* host, const void* device, int size);
int sph_copyToDevice(void* device, const void* host, int offset, int size);

/* setParameters (System.cu:634-637): the parameters every following stage
   call uses (one set per process, like the reference's __constant__ par).
   Rejects parameter sets the kernels do not cover (SPH_ERR_PARAMS /
   SPH_ERR_UNSUPPORTED). */
int sph_setParameters(const SimParams* hostParams);
/* Stream for the stage calls (NULL: legacy default stream). */
int sph_setStageStream(void* stream);

/* integrate (System.cuh:24-25): integrateD + boundary() over all particles,
   old -> new position and velocity (float4, original order). */
int sph_integrate(const sph_float4* oldPos, sph_float4* newPos, const sph_float4* oldVel,
                  sph_float4* newVel, int numParticles);

/* calcHash (System.cuh:27): particleHash[i] = {cell hash of pos[i], i}. */
int sph_calcHash(const sph_float4* pos, sph_uint2* particleHash, int numParticles);

/* RadixSort (radixsort.cuh:30-32, radixsort_kernel.cu:445-472): stable sort
   of (key, value) pairs by the low `bits` bits of the key, 8 bits per pass,
   ping-ponging between pData0 and pData1.  After an even number of passes
   (bits = 16 or 32, the values cSPH::Update uses) the result is in pData0;
   after an odd number it is in pData1, exactly as with the reference. */
int sph_RadixSort(sph_uint2* pData0, sph_uint2* pData1, uint32_t elements, uint32_t bits);

/* The same sort without any device allocation; it has no counterpart in the
   reference.  For callers that must not call cudaMalloc/cudaFree while they
   run (a frame loop that cannot absorb cudaFree's device-wide wait, or a
   process whose device memory is held by another allocator).  Its scratch
   is a 2.0 MiB array inside the library that every GPU loading it keeps
   until exit, so at most 4,194,304 pairs (larger: SPH_ERR_ARG).  Each call
   outside a stream capture looks up the array's address on the current
   device (so a cudaDeviceReset in between is harmless); a call inside a
   capture uses the address of the last call on that device, so make one
   before capturing (else SPH_ERR_STATE).  Calls that overlap on the GPU
   share the array and race.
   Runs on the stage stream; result location as sph_RadixSort. */
int sph_RadixSort_noalloc(sph_uint2* pData0, sph_uint2* pData1, uint32_t elements, uint32_t bits);

/* reorder (System.cuh:29-30): cellStart[c] = first sorted index of cell c
   (0xFFFFFFFF when empty), pos/vel gathered into sorted order. */
int sph_reorder(const sph_float4* oldPos, const sph_float4* oldVel, sph_float4* sortedPos,
                sph_float4* sortedVel, const sph_uint2* particleHash, uint32_t* cellStart,
                uint32_t numParticles, uint32_t numCells);

/* collide (System.cuh:32-35) without the timer and GL ids: density pass
   (pressure, density in sorted order), then force pass writing
   newVel[particleHash[i].y].  clr (may be NULL) and dyeColor (may be NULL)
   receive the colour and dye outputs in original order; oldPos/newPos/
   oldVel are accepted for signature parity and not read, as in the
   reference's kernels. */
int sph_collide(const sph_float4* oldPos, sph_float4* newPos, sph_float4* clr,
                const sph_float4* sortedPos, const sph_float4* sortedVel, const sph_float4* oldVel,
                sph_float4* newVel, float* pressure, float* density, float* dyeColor,
                const sph_uint2* particleHash, const uint32_t* cellStart, uint32_t numParticles,
                uint32_t numCells);

/* ======================================================================
 * 2. System handle (cSPH replacement)
 * ==================================================================== */
typedef struct SphSystem SphSystem;

#define SPH_ARRAY_POS 0
#define SPH_ARRAY_VEL 1

/* Create a system for one scene of params->numParticles particles
   (cSPH::_InitMem, SPH_Mem.cpp:11-54).  Particles start at the origin with
   zero velocity until sph_set_array fills them. */
int sph_create(const SimParams* params, SphSystem** out);
/* Create one system holding `count` independent scenes, stepped together. */
int sph_create_ensemble(const SimParams* scenes, uint32_t count, SphSystem** out);
int sph_destroy(SphSystem* sys);
/* Stream used by every following call on this handle. */
int sph_set_stream(SphSystem* sys, void* stream);
/* Replace a scene's parameters between steps (the slider path of
   SPH_Update.cpp:19-26).  numParticles and the grid must not change. */
int sph_set_params(SphSystem* sys, uint32_t scene, const SimParams* params);
int sph_get_params(SphSystem* sys, uint32_t scene, SimParams* out);
uint32_t sph_num_scenes(const SphSystem* sys);
/* Total particles (all scenes) and the first particle index of a scene. */
uint32_t sph_num_particles(const SphSystem* sys);
uint32_t sph_scene_offset(const SphSystem* sys, uint32_t scene);

/* setArray (SPH_Util.cpp:59-71): write `count` float4 records, starting at
   original particle index `start` (indices run over all scenes), from host
   memory (src_on_device = 0) or device memory (1).  Synchronous for host
   sources.  A pinned host buffer (one the GPU can address) is read by the
   GPU directly in one pass; pageable memory goes through a device staging
   copy. */
int sph_set_array(SphSystem* sys, uint32_t which, const sph_float4* data, uint32_t start,
                  uint32_t count, int src_on_device);
/* getArray (SPH_Util.cpp:44-56): all particles in original order, to host
   (dst_on_device = 0, synchronous) or device memory.  `which` is an enum;
   the reference's inverted bool is not reproduced.  A pinned host buffer is
   written by the GPU directly, as in sph_set_array. */
int sph_get_array(SphSystem* sys, uint32_t which, sph_float4* out, int dst_on_device);

/* Update (SPH_Update.cpp:12-81) `steps` times: integrate, hash, sort,
   cell ranges, density, force.  Steps after the first replay a captured
   CUDA graph. */
int sph_step(SphSystem* sys, uint32_t steps);

/* Steps captured per CUDA graph (even, >= 2; default 2).  sph_step(sys, k)
   replays floor(k / steps_per_graph) graph launches and runs the rest
   directly, so a whole run of steps_per_graph steps is one launch. */
int sph_set_graph_steps(SphSystem* sys, uint32_t steps_per_graph);

/* Colour and dye from every following step, the output of the reference's
   collide() (vboClr, dDyeColor; System.cu:405-546): clr gets one float4
   per particle and dye one float per particle, both device buffers of
   sph_num_particles records in original order owned by the caller (the dye
   is read and written: it carries over from step to step, as in the
   reference).  The colour type and constants are SimParams' (clrType,
   brightness, contrast, iHue, dye*).  NULL clr turns the output off; dye
   may be NULL.  The step's velocity increment is taken as v_new - v_old,
   and the CLR_Vel foam sum skips neighbour cells beyond the grid edge
   (the reference wraps there); sph_collide keeps the reference's exact
   form of both. */
int sph_set_color_output(SphSystem* sys, sph_float4* clr, float* dye);

/* Persistent stepping: with on != 0, sph_step(sys, k) runs its k steps as
   one cooperative launch (all blocks resident, a grid barrier between the
   stages, the same per-particle code as the launch-per-stage path, so the
   same results bit for bit).  A barrier wait that does not end within its
   poll limit sets bit 2 (value 4) of sph_flags and the kernel returns
   early.  Needs the neighbour masks (maxParInCell <= 21) and a device with
   cooperative launch; not used while a colour output is set. */
int sph_set_persistent(SphSystem* sys, int on);
/* Test hook for that timeout: one persistent step in which block 0 leaves
   before the first barrier and each wait is bounded at 4096 polls, so the
   other blocks' waits run out and the kernel ends; *flags gets sph_flags
   (bit 2 set).  Only scratch arrays are written: the state does not advance
   and the handle stays usable.  Needs persistent stepping on. */
int sph_persistent_withheld(SphSystem* sys, uint32_t* flags);

/* Launch shape of the density and force walks: threads per block and the
   form of each walk (every shape gives the same bits).
     shape  threads  density                     force
       0      64     global memory               global, row masks
       1     128     global memory               global, row masks
       2     256     global memory               global, row masks
       3     128     staged in shared memory     staged in shared memory
       4     128     staged, interleaved pairs   global, one cell at a time
       5     256     staged, interleaved pairs   global, one cell at a time
       6     128     staged, interleaved pairs   global, row masks
       7     128     global memory               global, one cell at a time
       8      64     staged, interleaved pairs   global, one cell at a time
       9     128     staged, interleaved pairs   global, pairs evaluated by the warp
      10      64     staged, interleaved pairs   global, pairs evaluated by the warp
   "Staged": the candidates of the block's neighbour cells are copied to
   shared memory once per block (a block whose cells need more room, or
   whose particles belong to two scenes, walks global memory).  4 is the
   default.  Without neighbour masks (maxParInCell > 16) every shape walks
   global memory. */
#define SPH_WALK_SHAPES 11
int sph_set_walk_shape(SphSystem* sys, uint32_t shape);
int sph_get_walk_shape(SphSystem* sys, uint32_t* shape, uint32_t* threads_per_block);

/* Autotuner: times `trial_steps` steps with each walk shape on this
   handle's own scenes and keeps the fastest (written to *chosen; per-shape
   ms per step to ms_per_step[SPH_WALK_SHAPES] if not NULL).  The particle
   state is saved before and restored after, so tuning does not advance the
   simulation. */
int sph_autotune(SphSystem* sys, uint32_t trial_steps, float* ms_per_step, uint32_t* chosen);

/* One step with a CUDA event recorded on the handle's stream before the
   first stage and after each of the six stages (1: integrate + cell count,
   2: scan, 3: id scatter, 4: stable placement, 5: density, 6: force);
   stage_ms[k] receives stage k+1's time in ms.  Synchronous. */
int sph_step_timed(SphSystem* sys, float* stage_ms, uint32_t nstages);

/* The neighbour structures of the last step, in the reference's formats:
   sortedHash[i] = {cell hash, original index} (local to each scene),
   cellStart[c] (0xFFFFFFFF when empty) and cellEnd[c] (one past the last
   sorted index; 0xFFFFFFFF when empty), cells of all scenes concatenated.
   Any pointer may be NULL.  To host (synchronous) or device memory. */
int sph_get_cells(SphSystem* sys, sph_uint2* sortedHash, uint32_t* cellStart, uint32_t* cellEnd,
                  int dst_on_device);
/* Density and pressure of the last step, in sorted order (as the reference
   keeps dDensity/dPressure), to host or device memory. */
int sph_get_fields(SphSystem* sys, float* density, float* pressure, int dst_on_device);
uint32_t sph_num_cells(const SphSystem* sys);

/* Double-precision reductions of the current state, per scene:
   out[4*s + 0] kinetic energy, [1] mean density of the last step,
   [2] max |rho/rho0 - 1|, [3] number of non-finite position/velocity
   components.  Synchronous. */
int sph_stats(SphSystem* sys, double* out);

/* Error and counter flags raised on the device since the last call (and
   cleared by it): bit 0 a cell held more than maxParInCell particles (the
   walk truncated it, as the reference does), bit 1 a non-finite position. */
int sph_flags(SphSystem* sys, uint32_t* flags);

/* ======================================================================
 * 4. Learned corrector: a per-particle MLP 16 -> 64 -> 64 -> 3 (tanh) on the
 *    tensor cores, BF16 operands and FP32 accumulation.  No counterpart in
 *    the reference: it lets a step of 4x dt be corrected towards four steps
 *    of dt.  All pointers are device pointers.
 * ==================================================================== */
#define SPH_MLP_IN 16
#define SPH_MLP_HIDDEN 64
#define SPH_MLP_OUT 3

/* Number of FP32 parameters: W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3]
   b3[3], in that order (5443). */
int sph_mlp_param_count(void);
/* Bytes of the packed BF16 image the kernels read. */
int sph_mlp_packed_bytes(void);
/* FP32 parameters -> packed BF16 image. */
int sph_mlp_pack(const float* params, void* packed, void* stream);
/* y[n][3] = MLP(x[n][16]); x is BF16 (uint16 bit patterns), y FP32. */
int sph_mlp_forward(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream);
/* The same forward pass on the 5th-generation tensor cores (tcgen05.mma with
   the accumulators in tensor memory), with the same BF16 roundings: its
   outputs equal sph_mlp_forward's.  x must be 16-byte aligned.  Its waits
   for the tensor cores are bounded: a thread block whose wait runs out
   writes NaN to the rows it did not finish and sets bit 0 of a status word
   that sph_mlp_status reads and clears (synchronous).  The learned step
   uses this pass; its density check treats NaN as a failed coarse step. */
int sph_mlp_forward_tc(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream);
int sph_mlp_status(uint32_t* status);
/* Test hook for the timeout path of sph_mlp_forward_tc: the same launch
   with the tensor-core work withheld and each wait bounded at 1024 polls,
   so every thread block's first wait runs out: all n rows become NaN, status
   bit 0 is set, and the tensor memory is freed (a later pass runs normally). */
int sph_mlp_forward_tc_withheld(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream);
/* One pass over n samples of the loss mean((y - target)^2) (over all 3n
   outputs): adds d loss / d params to grad[5443] and the loss to *loss
   (both FP32, zeroed by the caller). */
int sph_mlp_train_pass(const void* packed, const uint16_t* x, const float* target, uint32_t n,
                       float* grad, float* loss, void* stream);
/* The same training pass on the 5th-generation tensor cores: forward,
   backward and weight-gradient products as tcgen05.mma with the
   accumulators in tensor memory (the weight gradients accumulate there over
   all of a thread block's 128-sample tiles), the same BF16 roundings as
   sph_mlp_train_pass; only the FP32 summation order differs.  x must be
   16-byte aligned.  Its waits for the tensor cores are bounded: a thread
   block whose wait runs out adds NaN to *loss, adds nothing to grad and sets
   bit 1 of the status word of sph_mlp_status. */
int sph_mlp_train_pass_tc(const void* packed, const uint16_t* x, const float* target, uint32_t n,
                          float* grad, float* loss, void* stream);
/* Test hook for the timeout path of sph_mlp_train_pass_tc: the tensor-core
   work withheld and each wait bounded at 1024 polls; *loss becomes NaN,
   grad is untouched, status bit 1 is set, and the tensor memory is freed. */
int sph_mlp_train_pass_tc_withheld(const void* packed, const uint16_t* x, const float* target,
                                   uint32_t n, float* grad, float* loss, void* stream);
/* Adam step `step` (1-based) on the FP32 parameters with moments m, v. */
int sph_mlp_adam(float* params, float* m, float* v, const float* grad, float lr, float beta1,
                 float beta2, float eps, uint32_t step, void* stream);

/* The learned step on a system handle.  A coarse step is one whole step
   with the time step multiplied by n = `substeps` whose force pass also
   writes 16 features per particle; then, per particle, with v0 the velocity
   the step started from, vs the velocity after gravity and the walls (the
   integrate part) and v1 after the force pass:
     dv_pre = vs - v0, dv_post = v1 - vs;
   an optional jerk correction jerk * ((dv_pre - dv_pre') - (dv_post -
   dv_post')) from the previous coarse step's increments (primes) of the
   same particle; the MLP's correction dv = y * out_scale * |g| * dt_coarse;
   and the drift correction of the position drift * dt_coarse * (v - vs -
   dv_pre) with v the corrected velocity.  drift = (n-1)/(2n) is the
   difference, for constant accelerations, between n steps of dt and one of
   n dt when gravity and walls kick before the drift and the SPH force
   after it; jerk = (n-1)/(2n) the same for accelerations linear in time.
   After every coarse step a density check runs: if any scene's mean
   density departs from the linear extrapolation of its last two accepted
   steps by more than `tol` times its last value, or any value is not
   finite, the state is restored and the scene set advances by `substeps`
   plain steps of the original time step instead (counted in *fallbacks). */
/* Model: FP32 parameters (host, sph_mlp_param_count() floats), feature
   mean[16] and 1/std[16] (host, 32 floats), out_scale[3]. */
int sph_learned_set_model(SphSystem* sys, const float* params, const float* feat_stats,
                          const float* out_scale);
int sph_learned_step(SphSystem* sys, uint32_t coarse_steps, uint32_t substeps, float tol,
                     uint32_t* fallbacks);
/* Factors of the drift and jerk corrections: < 0 selects (n-1)/(2n), 0
   turns the correction off (defaults: drift (n-1)/(2n), jerk off). */
int sph_learned_set_options(SphSystem* sys, float drift, float jerk);
/* Training data: one coarse step (no correction) that writes the raw FP32
   features (device, N x 16, sorted order) and the original index of each
   sorted slot (device, N); the state advances by that coarse step. */
int sph_features_step(SphSystem* sys, uint32_t substeps, float* feat_raw, uint32_t* ids);

/* ======================================================================
 * 3. Scenes (Scene / cSPH::LoadScenes replacement, host only)
 * ==================================================================== */

/* Init data of a scene that is not part of SimParams (Scene.h:22-62). */
typedef struct {
  char title[64];
  int32_t chapter, is_default;
  float cellSize;
  sph_float3 initMin, initMax;
  int32_t initType, initLast;
  float spacing, dropR;
  int32_t rain;
} SphSceneInfo;

/* Number of <Scene> elements under the root of a Scenes.xml file. */
int sph_scene_count(const char* path, int* count);
/* Scene `index` of the file: the reference's defaults (Scene.cpp:7-66),
   the XML attributes (Scene_Load.cpp:11-111) and the derived constants
   (Scene.cpp:69-113).  info may be NULL. */
int sph_scene_load(const char* path, int index, SimParams* out, SphSceneInfo* info);
/* The same for one <Scene .../> element given as text. */
int sph_scene_parse(const char* xml, SimParams* out, SphSceneInfo* info);
/* Scene() with no XML: defaults plus derivations. */
int sph_scene_default(SimParams* out, SphSceneInfo* info);
/* Index of the scene marked default="" (or def=""), else 0
   (SPH_Scenes.cpp:186). */
int sph_scene_default_index(const char* path, int* index);

/* cSPH::Reset (SPH_Init.cpp:23-79): the initial volume of a scene, written
   to host arrays of numParticles float4 each.  type 0 fills the init volume
   as a lattice (the reference's loop order); type 1 places particles
   uniformly at random from a seeded generator (the reference calls
   rand()).  Returns the number of particles placed in *placed. */
int sph_scene_reset(const SimParams* params, const SphSceneInfo* info, int type, uint64_t seed,
                    sph_float4* pos, sph_float4* vel, uint32_t* placed);

/* Emitters, rain and Drop (App/Update.cpp:9-97, SPH_Init.cpp:83-117): the
   reference computes the particles on the host and writes them with
   setArray at a running emit index; here the functions below compute them
   and the caller writes them with sph_set_array (the Python layer's
   `emit` helper wraps the index as App::emitId does, splitting a write
   that would run past the end, where the reference writes out of range). */
#define SPH_NUM_EMIT 4
typedef struct {
  sph_float3 pos, rot; /* rot in degrees (x: pitch, y: yaw) */
  float vel;
  int32_t size, size2; /* size2 0: square */
} SphEmitter;
typedef struct {
  SphEmitter emit[SPH_NUM_EMIT];
  float rVel, r2Vel; /* rotor speeds (RotorVel, Rotor2Vel / WaveSpeed) */
} SphSceneMotion;
/* Emitters and rotor speeds of scene `index` of a file (Scene_Load.cpp:44-54,
   98-105) / of one <Scene> element given as text. */
int sph_scene_load_motion(const char* path, int index, SphSceneMotion* out);
int sph_scene_parse_motion(const char* xml, SphSceneMotion* out);
/* One frame of one emitter: size x size2 particles on a lattice of `spacing`
   in the emitter's plane, rotated (glRotatef(rot.x, x) then glRotatef(-rot.y,
   y), applied transposed), placed at pos, moving at vel along the rotated z
   axis; pos.w = vel.w = 0.  Writes *count (0 when size is 0) particles; fails
   when capacity is smaller. */
int sph_emitter_particles(const SphEmitter* em, float spacing, sph_float4* pos, sph_float4* vel,
                          uint32_t capacity, uint32_t* count);
/* cSPH::Drop: a ball of radius dropR spacings at rest, centred in the box or
   (random != 0) at a random place near the top drawn from a seeded
   splitmix64 (the reference calls rand()); at most `capacity` particles. */
int sph_drop_particles(const SimParams* params, const SphSceneInfo* info, int random,
                       uint64_t seed, sph_float4* pos, sph_float4* vel, uint32_t capacity,
                       uint32_t* count);
/* The per-frame parameter updates of App::UpdateEmitter (Update.cpp:14-23):
   rotor angles advanced by one time step, the dye-clear countdown. */
int sph_scene_advance(SimParams* params, const SphSceneMotion* motion);

/* ======================================================================
 * 5. Headless screen-space rendering (no reference ABI counterpart: the
 *    reference renders through OpenGL, Graphics/render_particles.cpp)
 * ==================================================================== */

/* The reference's fluid pipeline in CUDA, into device buffers: point
   sprites into a depth and thickness G-buffer in draw order (Gbuffer.vs,
   Gbuffer.fs; depth test GL_LESS, blend SRC_ALPHA / ONE_MINUS_SRC_ALPHA),
   `iterations` passes of curvature flow (CurvatureFlow.fs, method 1) or of
   the bilateral filter (BilateralFilter.fs, method 2), then the shading of
   ScreenSpaceRender.fs.  The cube map and the scene behind the fluid are
   the constant colours env_color and background.  Depth is FP32 (the
   reference's depth textures are the driver's choice). */
#define SPH_RENDER_MAX_KERNEL_CENTER 16
typedef struct SphRenderer SphRenderer;
typedef struct {
  float modelview[16], projection[16]; /* GL column-major */
  float point_radius, point_scale;     /* m_ParRadius, m_ParScale (pixels at distance 1) */
  int32_t method;                      /* RenderMethod: 0 none, 1 curvature flow, 2 bilateral */
  int32_t iterations;                  /* nIter */
  int32_t kernel_center;               /* KernelC (bilateral), <= SPH_RENDER_MAX_KERNEL_CENTER */
  float sigma;                         /* DomainSigma (bilateral; the reference uses 0.01) */
  float env_color[3], background[3];
} SphRenderParams;
int sph_render_create(int width, int height, SphRenderer** out);
int sph_render_destroy(SphRenderer* renderer);
/* One frame of n particles (device float4 positions).  Outputs (device,
   width x height, row 0 at the bottom as GL's window coordinates; any may
   be NULL): the smoothed depth (1.0 where nothing was drawn), the
   thickness, the RGBA image.  *fragments (may be NULL) receives the number
   of sprite fragments.  A frame whose sprites reach 2^32 or more (sprite,
   16 x 16 pixel tile) pairs is refused with SPH_ERR_ARG.  Synchronous. */
int sph_render_frame(SphRenderer* renderer, const SphRenderParams* params, const sph_float4* pos,
                     uint32_t n, float* depth_out, float* thickness_out, sph_float4* rgba_out,
                     uint64_t* fragments);
/* The foam overlay SetFoam draws over the shaded frame (render_particles.cpp:
   306-334; Foam.vs, Foam.gs, Foam.fs): per particle, color[i].x is the foam
   value w (the colour array the reference binds, aliased to the shader's
   attribute 3); copy k = 0, 1 of the point is drawn at clip position
   gl_Position - k when k < w, with the particle's point size; the disc is cut
   to radius clamp(w / 0.05, 0, 1); the colour is (1, 1, 1, 1) for w >= 0.05,
   else (1, 1, 1, 1 - w / 0.05); blending off, depth test GL_ALWAYS, so each
   pixel keeps the last fragment in draw order.  rgba_inout (may be NULL) is
   the frame the fragments overwrite; foam_depth_out (may be NULL) receives
   their gl_FragDepth clamped to [0, 1], 1.0 where no foam was drawn.  Uses
   modelview, projection, point_radius and point_scale of params; n <= 2^30.
   Synchronous. */
int sph_render_foam(SphRenderer* renderer, const SphRenderParams* params, const sph_float4* pos,
                    const sph_float4* color, uint32_t n, sph_float4* rgba_inout, float* foam_depth_out);

#ifdef __cplusplus
}
#endif
#endif /* PIBITI_SPH_H */
