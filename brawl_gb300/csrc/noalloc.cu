// noalloc.cu -- total_energy for callers that cannot allocate device memory.
//
// brawl_total_energy keeps one FP64 energy per site in scratch that the
// library allocates the first time it is needed.  Some callers cannot let a
// library allocate: a host program that hands all device memory to its own
// pool allocator at start-up, or one that records its GPU work into a CUDA
// graph and so must finish every allocation before recording starts.
// brawl_total_energy_noalloc gives them the same bit-identical total energy
// without any allocation: the caller passes device buffers for the inputs
// and the output, and the per-site scratch is a fixed array in this file.
//
// Scratch: g_noalloc_site_energy, kNoAllocMaxSites doubles (4 MiB), a
// file-scope __device__ array that every device loading the library holds
// until the process exits.  Each call writes every entry it later reads, so
// nothing has to be cleared between calls; calls that overlap on the GPU
// (on different streams) share the array and race.
//
// Set-up, once per CUDA context (the device's primary context for callers
// of the runtime API), on the first call made with that context current:
// the array's device address (host code may only name the symbol, which is
// not a device address), the kernels loaded (module loading is lazy by
// default, and loading code may allocate) and the SM count.  That first call
// should come before any stream capture.  A context created later for the
// same device (after cudaDeviceReset, or a driver-API context of the
// caller's) gets its own set-up.  The neighbour tables are constant memory
// initialised with the module image, so no copy is needed in any context.
#include <cuda.h>

#include <mutex>
#include <vector>

#include "api_internal.h"

namespace brawl {
namespace {

constexpr int kNoAllocMaxSites = 1 << 19;

static __device__ __align__(256) double g_noalloc_site_energy[kNoAllocMaxSites];

// Neighbour entries of every lattice (packed dx, dy, dz, shell, the order of
// lattice_tables.h) and the first entry of every shell.
struct EntryTables {
  uint32_t ents[3][kMaxZ];
  int16_t starts[3][11];
};

constexpr uint32_t pack_offset(int8_t dx, int8_t dy, int8_t dz, int sh) {
  return (uint32_t)(uint8_t)dx | ((uint32_t)(uint8_t)dy << 8) | ((uint32_t)(uint8_t)dz << 16) |
         ((uint32_t)sh << 24);
}

constexpr EntryTables make_entry_tables() {
  EntryTables t{};
  for (int sh = 0; sh < 2; ++sh)
    for (int k = kSCShellStart[sh]; k < kSCShellStart[sh + 1]; ++k)
      t.ents[kSimpleCubic][k] = pack_offset(kSCOffsets[k][0], kSCOffsets[k][1], kSCOffsets[k][2], sh);
  for (int sh = 0; sh < 10; ++sh)
    for (int k = kBCCShellStart[sh]; k < kBCCShellStart[sh + 1]; ++k)
      t.ents[kBcc][k] = pack_offset(kBCCOffsets[k][0], kBCCOffsets[k][1], kBCCOffsets[k][2], sh);
  for (int sh = 0; sh < 6; ++sh)
    for (int k = kFCCShellStart[sh]; k < kFCCShellStart[sh + 1]; ++k)
      t.ents[kFcc][k] = pack_offset(kFCCOffsets[k][0], kFCCOffsets[k][1], kFCCOffsets[k][2], sh);
  for (int sh = 0; sh <= 2; ++sh) t.starts[kSimpleCubic][sh] = kSCShellStart[sh];
  for (int sh = 0; sh <= 10; ++sh) t.starts[kBcc][sh] = kBCCShellStart[sh];
  for (int sh = 0; sh <= 6; ++sh) t.starts[kFcc][sh] = kFCCShellStart[sh];
  return t;
}

static __constant__ EntryTables c_tab = make_entry_tables();

// Site energies in the reference's order, read straight from the
// reference-layout grid config(1, 2n1, 2n2, 2n3); one thread per occupied
// site, indexed in z, y, x order (the order total_energy adds them).
__global__ void noalloc_site_energies(Geom g, const int8_t* __restrict__ cfg,
                                      const double* __restrict__ V, double* __restrict__ e_site) {
  const int lat = g.lattice;
  const int W1 = 2 * g.n1, W2 = 2 * g.n2;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.n_sites;
       idx += gridDim.x * blockDim.x) {
    int x, y, z;
    decode_site(g, idx, x, y, z);
    const int cs = cfg[x + W1 * (y + W2 * z)];
    double total = 0.0;
    for (int sh = 0; sh < g.nsh; ++sh) {
      double e = 0.0;
      for (int k = c_tab.starts[lat][sh]; k < c_tab.starts[lat][sh + 1]; ++k) {
        int dx, dy, dz, shk;
        unpack_entry(c_tab.ents[lat][k], dx, dy, dz, shk);
        const int nx = wrap_general(x, dx, g.W1), ny = wrap_general(y, dy, g.W2),
                  nz = wrap_general(z, dz, g.W3);
        const int s = cfg[nx + W1 * (ny + W2 * nz)];
        e = __dadd_rn(e, V[(cs - 1) + g.ns * ((s - 1) + g.ns * sh)]);
      }
      total = sh == 0 ? e : __dadd_rn(total, e);
    }
    e_site[idx] = total;
  }
}

// The ordered sum on one warp (the library's total-energy sum).
__global__ void __launch_bounds__(32) noalloc_sum_sites(int n, const double* __restrict__ e_site,
                                                        double* out) {
  const double energy = ordered_half_sum_warp(e_site, n, threadIdx.x);
  if (threadIdx.x == 0) *out = energy;
}

// What the set-up of one context found.
struct ContextScratch {
  unsigned long long ctx_id;
  double* scratch;
  int sms;
};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

std::mutex g_setup_mutex;
std::vector<ContextScratch> g_contexts;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int driver_entry(const char* name, void** fn) {
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  const cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*fn)
    return api_fail(BRAWL_ECUDA, std::string("driver entry point ") + name + " unavailable");
  return BRAWL_OK;
}

// The unique id of the context current on this thread (made current on
// device dev when the thread has none yet).
int current_context_id(int dev, unsigned long long* id) {
  if (!g_ctx_get_current) {
    void* f = nullptr;
    int rc = driver_entry("cuCtxGetCurrent", &f);
    if (rc != BRAWL_OK) return rc;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    rc = driver_entry("cuCtxGetId", &f);
    if (rc != BRAWL_OK) return rc;
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS)
    return api_fail(BRAWL_ECUDA, "cuCtxGetCurrent failed");
  if (!ctx) {
    // no context bound to this thread yet: bind the device's primary one
    const cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return api_fail(BRAWL_ECUDA, cudaGetErrorString(e));
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
      return api_fail(BRAWL_ECUDA, "no CUDA context current");
  }
  if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return api_fail(BRAWL_ECUDA, "cuCtxGetId failed");
  return BRAWL_OK;
}

// Once per context: the scratch array's device address, the kernels loaded,
// the SM count.
int setup_context(int dev, ContextScratch* out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long id = 0;
  int rc = current_context_id(dev, &id);
  if (rc != BRAWL_OK) return rc;
  for (const ContextScratch& c : g_contexts)
    if (c.ctx_id == id) {
      *out = c;
      return BRAWL_OK;
    }
  ContextScratch c{id, nullptr, 0};
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_site_energy);
  if (e != cudaSuccess)
    return api_fail(BRAWL_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  c.scratch = static_cast<double*>(p);
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, noalloc_site_energies);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, noalloc_sum_sites);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess)
    return api_fail(BRAWL_ECUDA, std::string("set-up: ") + cudaGetErrorString(e));
  if (c.sms < 1) c.sms = 1;
  g_contexts.push_back(c);
  *out = c;
  return BRAWL_OK;
}

}  // namespace
}  // namespace brawl

using namespace brawl;

extern "C" int brawl_total_energy_noalloc(const brawl_setup* setup, const double* d_V_ex,
                                          const int8_t* d_config, double* d_energy,
                                          void* stream) {
  if (!setup || !d_V_ex || !d_config || !d_energy)
    return api_fail(BRAWL_EINVAL, "brawl_total_energy_noalloc: null argument");
  Geom g;
  int rc = api_make_geom(*setup, g);
  if (rc != BRAWL_OK) return rc;
  if (g.n_sites > kNoAllocMaxSites)
    return api_fail(BRAWL_EINVAL, "brawl_total_energy_noalloc: " + std::to_string(g.n_sites) +
                                      " sites exceed the fixed scratch of " +
                                      std::to_string(kNoAllocMaxSites) + " sites");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return api_fail(BRAWL_ECUDA, cudaGetErrorString(e));
  ContextScratch cs;
  rc = setup_context(dev, &cs);
  if (rc != BRAWL_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // grid-stride over the sites, at most 8 blocks of 256 per SM
  int blocks = (g.n_sites + 255) / 256;
  if (blocks > 8 * cs.sms) blocks = 8 * cs.sms;
  noalloc_site_energies<<<blocks, 256, 0, s>>>(g, d_config, d_V_ex, cs.scratch);
  noalloc_sum_sites<<<1, 32, 0, s>>>(g.n_sites, cs.scratch, d_energy);
  e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(BRAWL_ECUDA, cudaGetErrorString(e));
  return BRAWL_OK;
}
