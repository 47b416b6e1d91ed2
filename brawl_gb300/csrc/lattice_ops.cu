// lattice_ops.cu -- initial configurations, total energies and layout
// conversions for batches of chains.
#include "kernels.cuh"

namespace brawl {

// ---------------------------------------------------------------------------
// initial_setup (src/initialise.F90:434-617).  The reference visits the
// occupied sites in z, y, x order -- exactly the compact index order -- and
// for each draws u until a species with quota left contains u in its
// interval [sum(c(0:l-1)), sum(c(0:l))]; every species whose interval holds
// u and whose quota is open is written in turn (the last one wins) and each
// such write uses up one of its quota.  The interval tests are done exactly
// on the 32-bit word: lo <= u <=> w >= lo_w, u <= hi <=> w <= hi_w.
// One warp per chain; all lanes follow the same control flow so the whole
// warp can regenerate the mt19937ar block when needed.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) initial_setup_kernel(const InitJob* __restrict__ jobs) {
  __shared__ uint32_t mt[kMTN];
  __shared__ int64_t check[kMaxSpecies];
  const InitJob& J = jobs[blockIdx.x];
  const int lane = threadIdx.x;
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  int pos = (int)J.rng[kMTN];
  __syncwarp();
  unsigned long long draws = 0;
  if (!initial_setup_warp(J, J.lat, mt, pos, check, draws, lane)) {
    if (lane == 0) *J.status = kStatusBadSpecies;
    return;
  }
  __syncwarp();
  for (int i = lane; i < kMTN; i += 32) J.rng[i] = mt[i];
  if (lane == 0) {
    J.rng[kMTN] = (uint32_t)pos;
    J.counters[kCntDraws] += draws;
  }
}

void launch_initial_setup(const InitJob* d_jobs, int n_jobs, cudaStream_t stream) {
  BRAWL_CARVEOUT(initial_setup_kernel);
  if (n_jobs > 0) initial_setup_kernel<<<n_jobs, 32, 0, stream>>>(d_jobs);
}

__global__ void site_energies_kernel(const EnergyJob* __restrict__ jobs, int n_jobs,
                                     int64_t total_sites) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total_sites;
       t += (int64_t)gridDim.x * blockDim.x) {
    // locate the chain by binary search on the site prefix
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].site_offset <= t) lo = mid;
      else hi = mid - 1;
    }
    const EnergyJob& J = jobs[lo];
    const int idx = (int)(t - J.site_offset);
    int x, y, z;
    decode_site(J.g, idx, x, y, z);
    J.site_energy[idx] = site_energy_ref(J.g, J.lat, J.V, J.entries, J.shell_start, x, y, z);
  }
}

// energy = energy + e(site) over sites in order, then 0.5 * energy; one
// warp per chain (ordered_half_sum_warp).
constexpr int kSumWarps = 4;
__global__ void __launch_bounds__(32 * kSumWarps) sum_sites_kernel(const EnergyJob* __restrict__ jobs,
                                                                   int n_jobs) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * kSumWarps + (threadIdx.x >> 5);
  if (c >= n_jobs) return;  // the whole warp
  const EnergyJob& J = jobs[c];
  const double energy = ordered_half_sum_warp(J.site_energy, J.g.n_sites, lane);
  if (lane == 0) *J.out = energy;
}

void launch_total_energy(const EnergyJob* d_jobs, int n_jobs, int64_t total_sites,
                         cudaStream_t stream) {
  if (n_jobs <= 0) return;
  int64_t blocks = (total_sites + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  BRAWL_CARVEOUT(site_energies_kernel);
  site_energies_kernel<<<(int)blocks, 256, 0, stream>>>(d_jobs, n_jobs, total_sites);
  BRAWL_CARVEOUT(sum_sites_kernel);
  sum_sites_kernel<<<(n_jobs + kSumWarps - 1) / kSumWarps, 32 * kSumWarps, 0, stream>>>(d_jobs, n_jobs);
}

// One block row per job (blockIdx.y), the sites strided over the row's
// blocks.
__global__ void lattice_snapshot_kernel(const EnergyJob* __restrict__ src, const EnergyJob* __restrict__ dst) {
  const int c = blockIdx.y;
  const int n = src[c].g.n_sites;
  const int8_t* __restrict__ from = src[c].lat;
  int8_t* __restrict__ to = const_cast<int8_t*>(dst[c].lat);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) to[i] = from[i];
}

void launch_lattice_snapshot(const EnergyJob* d_src, const EnergyJob* d_dst, int n_jobs, int max_sites,
                             cudaStream_t stream) {
  if (n_jobs <= 0) return;
  BRAWL_CARVEOUT(lattice_snapshot_kernel);
  const int bx = std::min(8, (max_sites + 255) / 256);
  for (int base = 0; base < n_jobs; base += 65535)  // gridDim.y <= 65535
    lattice_snapshot_kernel<<<dim3(bx, std::min(65535, n_jobs - base)), 256, 0, stream>>>(d_src + base,
                                                                                        d_dst + base);
}

__global__ void one_site_energy_kernel(const EnergyJob* __restrict__ job, int x, int y, int z,
                                       double* out) {
  *out = site_energy_ref(job->g, job->lat, job->V, job->entries, job->shell_start, x, y, z);
}

void launch_site_energy(const EnergyJob* d_job, int x, int y, int z, double* out,
                        cudaStream_t stream) {
  BRAWL_CARVEOUT(one_site_energy_kernel);
  one_site_energy_kernel<<<1, 1, 0, stream>>>(d_job, x, y, z, out);
}

// ---------------------------------------------------------------------------
// Layout conversions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool occupied(const Geom& g, int x, int y, int z) {
  if (g.lattice == kBcc) return ((x & 1) == (z & 1)) && ((y & 1) == (z & 1));
  if (g.lattice == kFcc) return ((x + y + z) & 1) == 0;
  return true;
}

__global__ void pack_kernel(Geom g, const int8_t* __restrict__ grid, int8_t* __restrict__ lat,
                            int32_t* status) {
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3;
  const int64_t total = (int64_t)W1 * W2 * W3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % W1), y = (int)((t / W1) % W2), z = (int)(t / ((int64_t)W1 * W2));
    const int8_t s = grid[t];
    if (occupied(g, x, y, z)) {
      lat[compact_index(g, x, y, z)] = s;
      if (s < 1 || s > g.ns) *status = kStatusBadSpecies;
    } else if (s != 0) {
      *status = kStatusBadSpecies;
    }
  }
}

__global__ void unpack_kernel(Geom g, const int8_t* __restrict__ lat, int8_t* __restrict__ grid) {
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3;
  const int64_t total = (int64_t)W1 * W2 * W3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % W1), y = (int)((t / W1) % W2), z = (int)(t / ((int64_t)W1 * W2));
    grid[t] = occupied(g, x, y, z) ? lat[compact_index(g, x, y, z)] : (int8_t)0;
  }
}

void launch_pack(const Geom& g, const int8_t* d_grid, int8_t* d_lat, int32_t* d_status,
                 cudaStream_t stream) {
  const int64_t total = (int64_t)8 * g.n1 * g.n2 * g.n3;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  BRAWL_CARVEOUT(pack_kernel);
  pack_kernel<<<blocks, 256, 0, stream>>>(g, d_grid, d_lat, d_status);
}

void launch_unpack(const Geom& g, const int8_t* d_lat, int8_t* d_grid, cudaStream_t stream) {
  const int64_t total = (int64_t)8 * g.n1 * g.n2 * g.n3;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  BRAWL_CARVEOUT(unpack_kernel);
  unpack_kernel<<<blocks, 256, 0, stream>>>(g, d_lat, d_grid);
}

// Batch layout conversions: one row of blocks per chain (blockIdx.y), each
// thread four consecutive cells of the chain's grid (grids are multiples of
// 8 cells, 8-byte aligned), so the grids -- possibly page-locked host
// memory read or written in place -- stream through in 4-byte accesses.
__global__ void pack_batch_kernel(const GridJob* __restrict__ jobs, const int8_t* __restrict__ grids) {
  const GridJob& J = jobs[blockIdx.y];
  const int W1 = 2 * J.g.n1, W2 = 2 * J.g.n2;
  const int64_t quads = (int64_t)2 * J.g.n1 * J.g.n2 * J.g.n3;  // cells / 4
  const bool small = quads < ((int64_t)1 << 29);                  // 4 q fits in 32 bits
  const char4* src = reinterpret_cast<const char4*>(grids + J.grid_offset);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < quads;
       q += (int64_t)gridDim.x * blockDim.x) {
    const char4 v = src[q];
    const int8_t s4[4] = {v.x, v.y, v.z, v.w};
    const int row = small ? (int)(4 * q) / W1 : (int)((4 * q) / W1);  // < W2 * W3
    int x = (int)(4 * q - (int64_t)row * W1), y = row % W2, z = row / W2;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int8_t s = s4[k];
      if (occupied(J.g, x, y, z)) {
        J.lat[compact_index(J.g, x, y, z)] = s;
        if (s < 1 || s > J.g.ns) *J.status = kStatusBadSpecies;
      } else if (s != 0) {
        *J.status = kStatusBadSpecies;
      }
      if (++x == W1) {  // the quad runs on into the next row
        x = 0;
        if (++y == W2) {
          y = 0;
          ++z;
        }
      }
    }
  }
}

__global__ void unpack_batch_kernel(const GridJob* __restrict__ jobs, int8_t* __restrict__ grids) {
  const GridJob& J = jobs[blockIdx.y];
  const int W1 = 2 * J.g.n1, W2 = 2 * J.g.n2;
  const int64_t quads = (int64_t)2 * J.g.n1 * J.g.n2 * J.g.n3;
  const bool small = quads < ((int64_t)1 << 29);
  char4* dst = reinterpret_cast<char4*>(grids + J.grid_offset);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < quads;
       q += (int64_t)gridDim.x * blockDim.x) {
    int8_t s4[4];
    const int row = small ? (int)(4 * q) / W1 : (int)((4 * q) / W1);
    int x = (int)(4 * q - (int64_t)row * W1), y = row % W2, z = row / W2;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s4[k] = occupied(J.g, x, y, z) ? J.lat[compact_index(J.g, x, y, z)] : (int8_t)0;
      if (++x == W1) {
        x = 0;
        if (++y == W2) {
          y = 0;
          ++z;
        }
      }
    }
    dst[q] = make_char4(s4[0], s4[1], s4[2], s4[3]);
  }
}

// store_state (src/analytics.f90:43-64): every occupied site adds 1.0 to its
// species' count, one block row per chain (+1.0 sums of a few thousand
// samples are exact, so the order of the adds does not matter).
__global__ void alro_add_kernel(const GridJob* __restrict__ jobs, double* __restrict__ counts,
                                const int64_t* __restrict__ offsets) {
  const GridJob& J = jobs[blockIdx.y];
  double* c = counts + offsets[blockIdx.y];
  const int n = J.g.n_sites;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = J.lat[i];
    if (s >= 1 && s <= J.g.ns) c[(size_t)(s - 1) * n + i] += 1.0;
  }
}

void launch_alro_add(const GridJob* d_jobs, int n_jobs, double* d_counts, const int64_t* d_offsets,
                     cudaStream_t stream) {
  BRAWL_CARVEOUT(alro_add_kernel);
  if (n_jobs > 0) alro_add_kernel<<<dim3(8, n_jobs), 256, 0, stream>>>(d_jobs, d_counts, d_offsets);
}

// blocks per chain: enough threads for the largest grid's quads, at most 32
static dim3 batch_grid(int n_jobs, int64_t total_cells) {
  const int64_t per = total_cells / 4 / (n_jobs > 0 ? n_jobs : 1);
  int64_t bx = (per + 255) / 256;
  if (bx < 1) bx = 1;
  if (bx > 32) bx = 32;
  return dim3((unsigned)bx, (unsigned)n_jobs);
}

void launch_pack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells,
                       const int8_t* d_grids, cudaStream_t stream) {
  BRAWL_CARVEOUT(pack_batch_kernel);
  if (n_jobs > 0) pack_batch_kernel<<<batch_grid(n_jobs, total_cells), 256, 0, stream>>>(d_jobs, d_grids);
}

void launch_unpack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells, int8_t* d_grids,
                         cudaStream_t stream) {
  BRAWL_CARVEOUT(unpack_batch_kernel);
  if (n_jobs > 0) unpack_batch_kernel<<<batch_grid(n_jobs, total_cells), 256, 0, stream>>>(d_jobs, d_grids);
}

void preload_lattice_kernels() {
  cudaFuncAttributes a;
  cudaFuncGetAttributes(&a, initial_setup_kernel);
  cudaFuncGetAttributes(&a, site_energies_kernel);
  cudaFuncGetAttributes(&a, sum_sites_kernel);
  cudaFuncGetAttributes(&a, lattice_snapshot_kernel);
  cudaFuncGetAttributes(&a, pack_kernel);
  cudaFuncGetAttributes(&a, unpack_kernel);
  cudaFuncGetAttributes(&a, pack_batch_kernel);
  cudaFuncGetAttributes(&a, unpack_batch_kernel);
}

}  // namespace brawl
