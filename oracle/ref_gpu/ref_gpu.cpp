/*
 * ref_gpu.cpp -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Runs the reference's own CUDA kernels on the GPU: the PTX that
 * build_ref_gpu.sh compiles from the reference tree is loaded through the
 * CUDA driver API, and the kernels are launched the way the reference's
 * wrappers launch them (System.cu:641-756, radixsort_kernel.cu:445-472): the
 * same grid and block sizes, the same dynamic shared memory, the same
 * cellStart memset, every wrapper ending with a device synchronisation as
 * its threadSync() does.  Nothing in the product loads this; the tests use
 * it to compare the fused step with the reference's GPU execution and to
 * time the reference's kernels on the same GPU.
 *
 * Texture bindings (System.cu:700, 729-732) are records {pointer, element
 * count} in the module (gpu_prelude.h); the reference's sizes in bytes are
 * passed here as element counts.
 */
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

namespace {

struct TexRecord {
  const void* ptr;
  long long count;
};
static_assert(sizeof(TexRecord) == 16, "texture record layout of gpu_prelude.h");

enum { T_POS, T_VEL, T_HASH, T_CELL, T_PRES, T_DENS, T_DYE, T_COUNT };
const char* const kTexNames[T_COUNT] = {"oldPosTex",   "oldVelTex",  "particleHashTex", "cellStartTex",
                                        "pressureTex", "densityTex", "dyeColorTex"};

// Kernel grid constants of radixsort_kernel.cu:13-44 (NUM_BLOCKS,
// NUM_THREADS_PER_BLOCK, PREFIX_NUM_BLOCKS, PREFIX_NUM_THREADS_PER_BLOCK)
// and the dynamic shared memory of each launch (GRFSIZE, PREFIX_GRFSIZE,
// SHUFFLE_GRFSIZE).
constexpr unsigned kSortBlocks = 48, kSortThreads = 64, kPrefixBlocks = 16, kPrefixThreads = 192;
constexpr unsigned kSumSmem = 4 * 256 * 4, kPrefixSmem = (3072 + 2 * 192) * 4, kShuffleSmem = (4 * 256 + 16) * 4;

CUcontext g_ctx = nullptr;
CUmodule g_sys = nullptr, g_radix = nullptr;
CUfunction f_integrate, f_hash, f_reorder, f_density, f_force, f_sum, f_prefix, f_shuffle;
CUdeviceptr g_par = 0, g_tex[T_COUNT] = {};
size_t g_par_bytes = 0;
char g_err[512] = "";

int fail(int code, const char* what) {
  snprintf(g_err, sizeof g_err, "%s", what);
  return code;
}
int fail_cu(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  snprintf(g_err, sizeof g_err, "%s: %s", what, s ? s : "unknown CUDA error");
  return 1;
}
#define CK(x, what)                                 \
  do {                                              \
    const CUresult r_ = (x);                        \
    if (r_ != CUDA_SUCCESS) return fail_cu(what, r_); \
  } while (0)

bool read_file(const char* path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// computeGridSize (System.cu:641-647)
void grid_size(unsigned n, unsigned block, unsigned& nb, unsigned& nt) {
  nt = n < block ? n : block;
  nb = n % nt != 0 ? n / nt + 1 : n / nt;
}

// The reference kernels have no tail guard: a launch covers whole blocks and
// every thread reads element `index`.  Sizes whose last block would be
// partial are refused (the reference's own host code needs N % 512 == 0).
bool size_ok(unsigned n) { return n > 0 && (n <= 64 || n % 512 == 0); }

int launch(CUfunction f, unsigned grid, unsigned block, unsigned smem, void** args) {
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, nullptr, args, nullptr), "kernel launch");
  return 0;
}
int sync_device() {
  CK(cuCtxSynchronize(), "synchronize");
  return 0;
}
int bind(int which, const void* ptr, long long count) {
  const TexRecord r{ptr, count};
  CK(cuMemcpyHtoD(g_tex[which], &r, sizeof r), "texture binding");
  return 0;
}
int unbind_all() {
  for (int k = 0; k < T_COUNT; ++k)
    if (int rc = bind(k, nullptr, 0)) return rc;
  return 0;
}

}  // namespace

extern "C" {

const char* ref_gpu_error(void) { return g_err; }

// Loads the two PTX modules and resolves the entries listed in `entries`
// (lines name=entry, as build_ref_gpu.sh writes them).
int ref_gpu_load(const char* system_ptx, const char* radix_ptx, const char* entries) {
  if (g_sys) return 0;
  CK(cuInit(0), "cuInit");
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0), "device 0");
  CK(cuDevicePrimaryCtxRetain(&g_ctx, dev), "primary context");
  CK(cuCtxSetCurrent(g_ctx), "current context");
  std::string sys, radix, names;
  if (!read_file(system_ptx, sys) || !read_file(radix_ptx, radix) || !read_file(entries, names))
    return fail(2, "reference PTX or entry list missing");
  CK(cuModuleLoadData(&g_sys, sys.c_str()), "load the reference's System.cu kernels");
  CK(cuModuleLoadData(&g_radix, radix.c_str()), "load the reference's radix sort kernels");
  struct {
    const char* name;
    CUmodule* mod;
    CUfunction* fn;
  } want[] = {{"integrateD", &g_sys, &f_integrate},
              {"calcHashD", &g_sys, &f_hash},
              {"reorderD", &g_sys, &f_reorder},
              {"computeDensityD", &g_sys, &f_density},
              {"computeForceD", &g_sys, &f_force},
              {"RadixSum", &g_radix, &f_sum},
              {"RadixPrefixSum", &g_radix, &f_prefix},
              {"RadixAddOffsetsAndShuffle", &g_radix, &f_shuffle}};
  for (auto& w : want) {
    const std::string key = std::string(w.name) + "=";
    const size_t at = names.find(key);
    if (at == std::string::npos || (at > 0 && names[at - 1] != '\n')) return fail(2, "entry list incomplete");
    const size_t end = names.find('\n', at);
    const std::string entry = names.substr(at + key.size(), end == std::string::npos ? end : end - at - key.size());
    CK(cuModuleGetFunction(w.fn, *w.mod, entry.c_str()), w.name);
  }
  CK(cuModuleGetGlobal(&g_par, &g_par_bytes, g_sys, "par"), "par");
  for (int k = 0; k < T_COUNT; ++k) {
    size_t bytes = 0;
    CK(cuModuleGetGlobal(&g_tex[k], &bytes, g_sys, kTexNames[k]), kTexNames[k]);
    if (bytes != sizeof(TexRecord)) return fail(2, "texture record size");
  }
  return unbind_all();
}

// Unloads the modules (to load the other build of the System.cu kernels).
int ref_gpu_unload(void) {
  if (g_sys) CK(cuModuleUnload(g_sys), "unload");
  if (g_radix) CK(cuModuleUnload(g_radix), "unload");
  g_sys = g_radix = nullptr;
  return 0;
}

unsigned long long ref_gpu_params_bytes(void) { return g_par_bytes; }

// setParameters (System.cu:632-637)
int ref_gpu_set_params(const void* params, unsigned long long bytes) {
  if (!g_sys) return fail(2, "not loaded");
  if (bytes != g_par_bytes) return fail(2, "SimParams size differs from the reference's");
  CK(cuMemcpyHtoD(g_par, params, bytes), "setParameters");
  return 0;
}

// integrate (System.cu:653-667)
int ref_gpu_integrate(void* old_pos, void* new_pos, void* old_vel, void* new_vel, unsigned n) {
  if (!size_ok(n)) return fail(3, "integrate: N must be <= 64 or a multiple of 512");
  unsigned nb, nt;
  grid_size(n, 256, nb, nt);
  void* args[] = {&new_pos, &new_vel, &old_pos, &old_vel};
  if (int rc = launch(f_integrate, nb, nt, 0, args)) return rc;
  return sync_device();
}

// calcHash (System.cu:671-685)
int ref_gpu_calc_hash(void* pos, void* hash, unsigned n) {
  if (!size_ok(n)) return fail(3, "calcHash: N must be <= 64 or a multiple of 512");
  unsigned nb, nt;
  grid_size(n, 2 * 256, nb, nt);
  void* args[] = {&pos, &hash};
  if (int rc = launch(f_hash, nb, nt, 0, args)) return rc;
  return sync_device();
}

// RadixSort (radixsort_kernel.cu:445-472): `bits / 8` passes, result in d0
// after an even number of passes.
int ref_gpu_radix_sort(void* d0, void* d1, unsigned elements, unsigned bits) {
  unsigned rounded = elements % 3072 == 0 ? elements : elements + (3072 - elements % 3072);
  for (unsigned shift = 0; shift < bits; shift += 8) {
    void* a_sum[] = {&d0, &elements, &rounded, &shift};
    if (int rc = launch(f_sum, kSortBlocks, kSortThreads, kSumSmem, a_sum)) return rc;
    if (int rc = launch(f_prefix, kPrefixBlocks, kPrefixThreads, kPrefixSmem, nullptr)) return rc;
    int ishift = (int)shift;
    void* a_shuffle[] = {&d0, &d1, &elements, &rounded, &ishift};
    if (int rc = launch(f_shuffle, kSortBlocks, kSortThreads, kShuffleSmem, a_shuffle)) return rc;
    void* t = d0;
    d0 = d1;
    d1 = t;
  }
  return sync_device();
}

// reorder (System.cu:689-713)
int ref_gpu_reorder(void* old_pos, void* old_vel, void* sorted_pos, void* sorted_vel, void* hash,
                    void* cell_start, unsigned n, unsigned num_cells) {
  if (!size_ok(n)) return fail(3, "reorder: N must be <= 64 or a multiple of 512");
  unsigned nb, nt;
  grid_size(n, 256, nb, nt);
  CK(cuMemsetD32((CUdeviceptr)cell_start, 0xffffffffu, num_cells), "cellStart memset");
  if (int rc = bind(T_POS, old_pos, n)) return rc;
  if (int rc = bind(T_VEL, old_vel, n)) return rc;
  void* args[] = {&hash, &cell_start, &old_pos, &old_vel, &sorted_pos, &sorted_vel};
  if (int rc = launch(f_reorder, nb, nt, 0, args)) return rc;
  if (int rc = sync_device()) return rc;
  return unbind_all();
}

// collide (System.cu:717-756): the density pass, a synchronisation, the
// force pass; newVel is written in original particle order.
int ref_gpu_collide(void* sorted_pos, void* sorted_vel, void* new_vel, void* clr, void* pressure,
                    void* density, void* dye, void* hash, void* cell_start, unsigned n, unsigned num_cells) {
  if (!size_ok(n)) return fail(3, "collide: N must be <= 64 or a multiple of 512");
  if (int rc = bind(T_POS, sorted_pos, n)) return rc;
  if (int rc = bind(T_PRES, pressure, n)) return rc;
  if (int rc = bind(T_VEL, sorted_vel, n)) return rc;
  if (int rc = bind(T_DENS, density, n)) return rc;
  if (int rc = bind(T_DYE, dye, n)) return rc;
  if (int rc = bind(T_HASH, hash, n)) return rc;
  if (int rc = bind(T_CELL, cell_start, num_cells)) return rc;
  unsigned nb, nt;
  grid_size(n, 64, nb, nt);
  void* a_dens[] = {&clr, &sorted_pos, &pressure, &density, &hash, &cell_start};
  if (int rc = launch(f_density, nb, nt, 0, a_dens)) return rc;
  if (int rc = sync_device()) return rc;
  void* new_pos = nullptr;  // computeForceD's newPos is not used (System.cu:260-548)
  void* a_force[] = {&new_pos, &new_vel, &sorted_pos, &sorted_vel, &clr, &pressure, &density, &dye, &hash, &cell_start};
  if (int rc = launch(f_force, nb, nt, 0, a_force)) return rc;
  if (int rc = sync_device()) return rc;
  return unbind_all();
}

}  // extern "C"
