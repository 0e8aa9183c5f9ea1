// sph_stage.cu -- the stage entry points: the reference's extern "C"
// wrappers (System.cu:613-756, radixsort_kernel.cu:445-472) re-implemented
// over device pointers, plus the library's error reporting.
//
// The kernels here follow the reference's data flow one to one (original-
// order state, uint2 {hash, index} pairs, cellStart with 0xFFFFFFFF for empty
// cells and no cellEnd) and its neighbour walk exactly: 27 cells whose hashes
// wrap like calcGridHash, at most maxParInCell entries per cell, a cell ends
// where the sorted hash changes, and a cell outside the table reads as
// empty (the reference's texture fetch returns 0 there).  Every kernel guards
// its tail, so any particle count is accepted.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {

namespace {
thread_local char g_err[512] = "";
SimParams g_params;
bool g_params_set = false;
cudaStream_t g_stage_stream = nullptr;
std::mutex g_scratch_mu;
uint32_t* g_scratch = nullptr;
size_t g_scratch_words = 0;
}  // namespace

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

cudaStream_t stage_stream() { return g_stage_stream; }

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SPH_OK;
  return fail(e == cudaErrorMemoryAllocation ? SPH_ERR_NOMEM : SPH_ERR_CUDA, "%s: %s (%s)", what,
              cudaGetErrorString(e), cudaGetErrorName(e));
}

int validate_params(const SimParams& p, bool fused) {
  const uint32_t gx = p.gridSize.x, gy = p.gridSize.y, gz = p.gridSize.z;
  if (gx == 0 || gy == 0 || gz == 0) return fail(SPH_ERR_PARAMS, "grid has a zero dimension");
  if ((uint64_t)gx * gy != p.gridSize_yx || (uint64_t)gx * gy * gz != p.numCells)
    return fail(SPH_ERR_PARAMS, "gridSize_yx/numCells do not match gridSize");
  if (p.gridSize_yx >= (1u << 23) || gz >= (1u << 23) || p.numCells >= (1u << 31))
    return fail(SPH_ERR_PARAMS, "grid of %u cells is beyond the 24-bit cell hash", p.numCells);
  if (!(p.cellSize.x > 0.f && p.cellSize.y > 0.f && p.cellSize.z > 0.f))
    return fail(SPH_ERR_PARAMS, "cellSize must be positive");
  if (!(p.h > 0.f) || !(p.timeStep == p.timeStep))
    return fail(SPH_ERR_PARAMS, "h must be positive and timeStep finite");
  if (p.rotType > 3) return fail(SPH_ERR_PARAMS, "unknown rotType %d", p.rotType);
  if (p.rotType > 0 && p.rotBlades <= 0) return fail(SPH_ERR_PARAMS, "rotor needs rotBlades > 0");
  if ((p.iHmap > 0 || p.rotType > 0) && !(p.rotSpc > 0.f))
    return fail(SPH_ERR_PARAMS, "height map and rotor need rotSpc > 0");
  if (p.bndType > SPH_BND_PUMP_Y) return fail(SPH_ERR_PARAMS, "unknown bndType %u", p.bndType);
  if (fused) {
    // The fused kernels skip neighbour cells outside the grid.  The
    // reference instead wraps x and y coordinates into other rows of the
    // grid; those cells lie at least (g - 2) cells away, so skipping them
    // changes nothing as long as that distance exceeds h.
    const float dx = (float)((int)gx - 2) * p.cellSize.x, dy = (float)((int)gy - 2) * p.cellSize.y;
    if (!(dx > 1.001f * p.h) || !(dy > 1.001f * p.h))
      return fail(SPH_ERR_PARAMS,
                  "grid too small for the fused step: (gridSize-2)*cellSize must exceed h in x "
                  "and y (%u x %u cells of %g for h=%g); use the stage entry points",
                  gx, gy, (double)p.cellSize.x, (double)p.h);
  }
  return SPH_OK;
}

namespace {

constexpr int kBlock = 256;
inline unsigned grid_for(size_t n, int block) { return (unsigned)((n + block - 1) / block); }

__global__ void st_integrate(const SimParams p, const float4* __restrict__ old_pos,
                             float4* __restrict__ new_pos, const float4* __restrict__ old_vel,
                             float4* __restrict__ new_vel, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x4 = old_pos[i], v4 = old_vel[i];
  float3 x = make_float3(x4.x, x4.y, x4.z), v = make_float3(v4.x, v4.y, v4.z);
  integrate(p, x, v);
  new_pos[i] = make_float4(x.x, x.y, x.z, x4.w);
  new_vel[i] = make_float4(v.x, v.y, v.z, v4.w);
}

__global__ void st_calc_hash(const SimParams p, const float4* __restrict__ pos,
                             uint2* __restrict__ hash, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int3 g = grid_pos(p, pos[i]);
  hash[i] = make_uint2(grid_hash_raw(p, g.x, g.y, g.z), (uint32_t)i);
}

// reorderD (Kernel_Cell.cui:40-67): a cell starts where the sorted hash
// changes.  Hashes outside the table are not written (the reference writes
// them unchecked); out-of-range source indices gather zeros.
__global__ void st_reorder(const uint2* __restrict__ hash, uint32_t* __restrict__ cell_start,
                           const float4* __restrict__ old_pos, const float4* __restrict__ old_vel,
                           float4* __restrict__ sorted_pos, float4* __restrict__ sorted_vel,
                           uint32_t n, uint32_t num_cells) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint2 kv = hash[i];
  if ((i == 0 || kv.x != hash[i - 1].x) && kv.x < num_cells) cell_start[kv.x] = i;
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f), v = x;
  if (kv.y < n) {
    x = old_pos[kv.y];
    v = old_vel[kv.y];
  }
  sorted_pos[i] = x;
  sorted_vel[i] = v;
}

// First sorted index of the cell with hash gh as the reference's
// FETCH(cellStart, gh) sees it: 0 outside the table (texture border).
__device__ __forceinline__ uint32_t ref_cell_start(const uint32_t* cs, uint32_t num_cells, uint32_t gh) {
  return ((int)gh >= 0 && gh < num_cells) ? cs[gh] : 0u;
}
__device__ __forceinline__ uint32_t ref_key(const uint2* hash, uint32_t n, uint32_t j) {
  return ((int)j >= 0 && j < n) ? hash[j].x : 0u;
}

// computeDensityD (Kernel_Cell.cui:142-199).
__global__ void st_density(const SimParams p, const float4* __restrict__ spos,
                           const uint2* __restrict__ hash, const uint32_t* __restrict__ cs,
                           float* __restrict__ pressure, float* __restrict__ density, uint32_t n,
                           uint32_t num_cells) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = spos[i];
  const int3 g = grid_pos(p, xi);
  float sum = 0.f;
  int nbr = 0;
  for (int z = -1; z <= 1; ++z)
    for (int y = -1; y <= 1; ++y)
      for (int x = -1; x <= 1; ++x) {
        const uint32_t gh = grid_hash_raw(p, g.x + x, g.y + y, g.z + z);
        const uint32_t start = ref_cell_start(cs, num_cells, gh);
        if (start == kEmpty) continue;
        float cell = 0.f;
        for (uint32_t k = 0; k < p.maxParInCell; ++k) {
          const uint32_t j = start + k;
          // Past the last particle the reference's texture fetch reads a
          // zero key; only a walk of cell 0 could match it, so stop there.
          if (j >= n || ref_key(hash, n, j) != gh) break;
          if (j != i) cell = density_pair(xi, spos[j], p.h2, cell, nbr);
        }
        sum = __fadd_rn(sum, cell);
      }
  const float dens = __fmul_rn(__fmul_rn(sum, p.Poly6Kern), p.particleMass);
  pressure[i] = __fmul_rn(__fsub_rn(dens, p.restDensity), p.stiffness);
  density[i] = dens;
}

// computeForceD (System.cu:228-546): new velocity, colour (with the foam
// estimate) and dye in original order through hash[i].y.
__global__ void st_force(const SimParams p, const float4* __restrict__ spos,
                         const float4* __restrict__ svel, const float* __restrict__ pressure,
                         const float* __restrict__ density, const uint2* __restrict__ hash,
                         const uint32_t* __restrict__ cs, float4* __restrict__ new_vel,
                         float4* __restrict__ clr, float* __restrict__ dye, uint32_t n,
                         uint32_t num_cells) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = spos[i], vi = svel[i];
  const float pi = pressure[i], di = density[i], inv_di = __frcp_rn(di);
  const int3 g = grid_pos(p, xi);
  const ForceConsts k = force_consts(p);
  float3 F = make_float3(0.f, 0.f, 0.f);
  for (int z = -1; z <= 1; ++z)
    for (int y = -1; y <= 1; ++y)
      for (int x = -1; x <= 1; ++x) {
        const uint32_t gh = grid_hash_raw(p, g.x + x, g.y + y, g.z + z);
        const uint32_t start = ref_cell_start(cs, num_cells, gh);
        if (start == kEmpty) continue;
        float3 cell = make_float3(0.f, 0.f, 0.f);
        for (uint32_t q = 0; q < p.maxParInCell; ++q) {
          const uint32_t j = start + q;
          if (j >= n || ref_key(hash, n, j) != gh) break;
          if (j != i)
            force_pair(k, xi, vi, inv_di, pi, spos[j], svel[j], __frcp_rn(density[j]), pressure[j],
                       cell);
        }
        F.x = __fadd_rn(F.x, cell.x);
        F.y = __fadd_rn(F.y, cell.y);
        F.z = __fadd_rn(F.z, cell.z);
      }
  const float3 add = velocity_increment(p, F, xi, vi);
  const uint32_t si = hash[i].y;
  if (si >= n) return;
  new_vel[si] = make_float4(__fadd_rn(vi.x, add.x), __fadd_rn(vi.y, add.y), __fadd_rn(vi.z, add.z),
                            __fadd_rn(vi.w, 0.f));
  if (clr) {
    float vdiff = 0.f;
    if (p.clrType == SPH_CLR_VEL) {
      // the foam walk (System.cu:441-468): x outermost, the cell start
      // re-read per entry, an empty cell starting at index -1 (a zero record)
      for (int x = -1; x < 2; ++x)
        for (int y = -1; y < 2; ++y)
          for (int z = -1; z < 2; ++z)
            for (uint32_t q = 0; q < p.maxParInCell; ++q) {
              const uint32_t gh = grid_hash_raw(p, g.x + x, g.y + y, g.z + z);
              const uint32_t j = ref_cell_start(cs, num_cells, gh) + q;
              if (ref_key(hash, n, j) != gh) break;
              if (j == i) continue;
              const bool in = (int)j >= 0 && j < n;
              const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
              vdiff = __fadd_rn(vdiff, foam_term(xi, vi, in ? spos[j] : zero, in ? svel[j] : zero));
            }
    }
    float4 c;
    if (color_dye(p, xi, vi, di, add, vdiff, dye ? dye + si : nullptr, c)) clr[si] = c;
  }
}

int need_params() {
  if (!g_params_set) return fail(SPH_ERR_STATE, "sph_setParameters has not been called");
  return SPH_OK;
}

int stage_scratch(size_t words, uint32_t** out) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (words > g_scratch_words) {
    if (g_scratch) cudaFree(g_scratch);
    g_scratch = nullptr;
    g_scratch_words = 0;
    SPH_CUDA(cudaMalloc(&g_scratch, words * sizeof(uint32_t)), "RadixSort scratch");
    g_scratch_words = words;
  }
  *out = g_scratch;
  return SPH_OK;
}

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" {

const char* sph_last_error(void) { return g_err; }
const char* sph_version(void) { return "pibiti_gb300 0.1 (sm_103a)"; }

int sph_threadSync(void) { return cuda_check(cudaDeviceSynchronize(), "threadSync"); }

int sph_allocateArray(void** devPtr, size_t size) {
  if (!devPtr) return fail(SPH_ERR_ARG, "allocateArray: null pointer");
  return cuda_check(cudaMalloc(devPtr, size), "allocateArray");
}

int sph_freeArray(void* devPtr) { return cuda_check(cudaFree(devPtr), "freeArray"); }

int sph_copyFromDevice(void* host, const void* device, int size) {
  if (size < 0 || (!host && size)) return fail(SPH_ERR_ARG, "copyFromDevice: bad size/pointer");
  return cuda_check(cudaMemcpy(host, device, (size_t)size, cudaMemcpyDeviceToHost), "copyFromDevice");
}

int sph_copyToDevice(void* device, const void* host, int offset, int size) {
  if (size < 0 || offset < 0 || (!host && size)) return fail(SPH_ERR_ARG, "copyToDevice: bad size/pointer");
  return cuda_check(cudaMemcpy((char*)device + offset, host, (size_t)size, cudaMemcpyHostToDevice),
                    "copyToDevice");
}

int sph_setParameters(const SimParams* hostParams) {
  if (!hostParams) return fail(SPH_ERR_ARG, "setParameters: null");
  SPH_TRY(validate_params(*hostParams, false));
  g_params = *hostParams;
  g_params_set = true;
  return SPH_OK;
}

int sph_setStageStream(void* stream) {
  g_stage_stream = (cudaStream_t)stream;
  return SPH_OK;
}

int sph_integrate(const sph_float4* oldPos, sph_float4* newPos, const sph_float4* oldVel,
                  sph_float4* newVel, int numParticles) {
  SPH_TRY(need_params());
  if (numParticles < 0) return fail(SPH_ERR_ARG, "integrate: negative count");
  if (numParticles == 0) return SPH_OK;
  st_integrate<<<grid_for(numParticles, kBlock), kBlock, 0, g_stage_stream>>>(
      g_params, (const float4*)oldPos, (float4*)newPos, (const float4*)oldVel, (float4*)newVel,
      numParticles);
  return cuda_check(cudaGetLastError(), "integrate");
}

int sph_calcHash(const sph_float4* pos, sph_uint2* particleHash, int numParticles) {
  SPH_TRY(need_params());
  if (numParticles < 0) return fail(SPH_ERR_ARG, "calcHash: negative count");
  if (numParticles == 0) return SPH_OK;
  st_calc_hash<<<grid_for(numParticles, kBlock), kBlock, 0, g_stage_stream>>>(
      g_params, (const float4*)pos, (uint2*)particleHash, numParticles);
  return cuda_check(cudaGetLastError(), "calcHash");
}

int sph_RadixSort(sph_uint2* pData0, sph_uint2* pData1, uint32_t elements, uint32_t bits) {
  if (elements == 0) return SPH_OK;
  if (!pData0 || !pData1) return fail(SPH_ERR_ARG, "RadixSort: null buffer");
  uint32_t* scratch = nullptr;
  SPH_TRY(stage_scratch(radix_scratch_words(elements), &scratch));
  return radix_sort_pairs((uint2*)pData0, (uint2*)pData1, elements, bits, scratch, g_stage_stream);
}

int sph_reorder(const sph_float4* oldPos, const sph_float4* oldVel, sph_float4* sortedPos,
                sph_float4* sortedVel, const sph_uint2* particleHash, uint32_t* cellStart,
                uint32_t numParticles, uint32_t numCells) {
  SPH_CUDA(cudaMemsetAsync(cellStart, 0xff, (size_t)numCells * sizeof(uint32_t), g_stage_stream),
           "reorder: cellStart reset");
  if (numParticles == 0) return SPH_OK;
  st_reorder<<<grid_for(numParticles, kBlock), kBlock, 0, g_stage_stream>>>(
      (const uint2*)particleHash, cellStart, (const float4*)oldPos, (const float4*)oldVel,
      (float4*)sortedPos, (float4*)sortedVel, numParticles, numCells);
  return cuda_check(cudaGetLastError(), "reorder");
}

int sph_collide(const sph_float4* oldPos, sph_float4* newPos, sph_float4* clr,
                const sph_float4* sortedPos, const sph_float4* sortedVel, const sph_float4* oldVel,
                sph_float4* newVel, float* pressure, float* density, float* dyeColor,
                const sph_uint2* particleHash, const uint32_t* cellStart, uint32_t numParticles,
                uint32_t numCells) {
  (void)oldPos;
  (void)newPos;
  (void)oldVel;
  SPH_TRY(need_params());
  if (numParticles == 0) return SPH_OK;
  const unsigned grid = grid_for(numParticles, 64);
  st_density<<<grid, 64, 0, g_stage_stream>>>(g_params, (const float4*)sortedPos,
                                               (const uint2*)particleHash, cellStart, pressure,
                                               density, numParticles, numCells);
  st_force<<<grid, 64, 0, g_stage_stream>>>(g_params, (const float4*)sortedPos,
                                             (const float4*)sortedVel, pressure, density,
                                             (const uint2*)particleHash, cellStart, (float4*)newVel,
                                             (float4*)clr, dyeColor, numParticles, numCells);
  return cuda_check(cudaGetLastError(), "collide");
}

}  // extern "C"
