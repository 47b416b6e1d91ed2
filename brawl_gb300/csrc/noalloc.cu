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
#include <cstring>
#include <mutex>

#include "api_internal.h"

namespace brawl {
namespace {

constexpr int kNoAllocMaxSites = 1 << 19;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_site_energy[kNoAllocMaxSites];

// Neighbour entries of every lattice (packed dx, dy, dz, shell), filled once
// per device at set-up; constant memory needs no allocation.
static __constant__ uint32_t c_entries[3][kMaxZ];
static __constant__ int16_t c_starts[3][11];

std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Once per device, with that device current: the scratch array's device
// address (host code may not use the symbol itself as a device pointer) and
// the constant tables.
int setup_device(int dev, double** scratch) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev]) {
    *scratch = g_scratch_ptr[dev];
    return BRAWL_OK;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_site_energy);
  if (e != cudaSuccess)
    return api_fail(BRAWL_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  uint32_t ents[3][kMaxZ];
  int16_t starts[3][11];
  std::memset(ents, 0, sizeof(ents));
  std::memset(starts, 0, sizeof(starts));
  for (int lat = 0; lat < 3; ++lat) {
    const int8_t(*offs)[3] = shell_offsets(lat);
    const int16_t* st = shell_starts(lat);
    const int ns = max_shells(lat);
    for (int sh = 0; sh <= ns; ++sh) starts[lat][sh] = st[sh];
    for (int sh = 0; sh < ns; ++sh)
      for (int k = st[sh]; k < st[sh + 1]; ++k)
        ents[lat][k] = (uint32_t)(uint8_t)offs[k][0] | ((uint32_t)(uint8_t)offs[k][1] << 8) |
                       ((uint32_t)(uint8_t)offs[k][2] << 16) | ((uint32_t)sh << 24);
  }
  e = cudaMemcpyToSymbol(c_entries, ents, sizeof(ents));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_starts, starts, sizeof(starts));
  if (e != cudaSuccess)
    return api_fail(BRAWL_ECUDA, std::string("constant tables: ") + cudaGetErrorString(e));
  g_scratch_ptr[dev] = static_cast<double*>(p);
  *scratch = g_scratch_ptr[dev];
  return BRAWL_OK;
}

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
      for (int k = c_starts[lat][sh]; k < c_starts[lat][sh + 1]; ++k) {
        int dx, dy, dz, shk;
        unpack_entry(c_entries[lat][k], dx, dy, dz, shk);
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

__global__ void noalloc_sum_sites(int n, const double* __restrict__ e_site, double* out) {
  double energy = 0.0;
  for (int i = 0; i < n; ++i) energy = __dadd_rn(energy, e_site[i]);
  *out = __dmul_rn(0.5, energy);
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
  if (dev < 0 || dev >= kMaxDevices) return api_fail(BRAWL_ECUDA, "device index out of range");
  double* scratch = nullptr;
  rc = setup_device(dev, &scratch);
  if (rc != BRAWL_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int blocks = (g.n_sites + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  noalloc_site_energies<<<blocks, 256, 0, s>>>(g, d_config, d_V_ex, scratch);
  noalloc_sum_sites<<<1, 1, 0, s>>>(g.n_sites, scratch, d_energy);
  e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(BRAWL_ECUDA, cudaGetErrorString(e));
  return BRAWL_OK;
}
