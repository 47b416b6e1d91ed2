// kernels.cuh -- launch-side declarations shared by the kernel translation
// units and the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "chain_engine.cuh"

namespace brawl {

// Shared-memory layout of one chain's CTA, identical on host and device.
struct SmemLayout {
  uint32_t mt, F, V, ents, sstart, lat, total;
};

__host__ __device__ inline uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline SmemLayout smem_layout(const Geom& g, bool lattice_in_smem) {
  SmemLayout L;
  const uint32_t nsp = (uint32_t)g.ns + 1;
  L.mt = 0;
  L.F = L.mt + kMTN * 4;
  L.V = align_up(L.F + nsp * nsp * (uint32_t)g.nsh * 4, 16);
  L.ents = L.V + (uint32_t)(g.ns * g.ns * g.nsh) * 8;
  L.sstart = L.ents + (uint32_t)g.z * 4;
  L.lat = align_up(L.sstart + (uint32_t)(g.nsh + 1) * 2, 16);
  L.total = lattice_in_smem ? align_up(L.lat + (uint32_t)g.n_sites, 16) : L.lat;
  return L;
}

// Metropolis swap trials, one warp (CTA) per chain.
void launch_metropolis(const ChainJob* d_jobs, int n_jobs, bool lattice_in_smem,
                       uint32_t smem_bytes, cudaStream_t stream);

// initial_setup (src/initialise.F90:434-617) on the device, one warp per
// chain.  Per chain: counts[ns] species quotas, lo_w/hi_w[ns] the interval
// bounds in units of 2^-32 (w >= lo_w and w <= hi_w <=> lo <= u <= hi).
struct InitJob {
  int8_t* lat;
  uint32_t* rng;
  int32_t n_sites, ns;
  int64_t counts[kMaxSpecies];
  int64_t lo_w[kMaxSpecies];
  int64_t hi_w[kMaxSpecies];
  unsigned long long* counters;
  int32_t* status;
};
void launch_initial_setup(const InitJob* d_jobs, int n_jobs, cudaStream_t stream);

// total_energy (src/bw_hamiltonian.f90:58-81): per-site FP64 energies in the
// reference's order, then the sequential sum over sites in z, y, x order.
struct EnergyJob {
  Geom g;
  const int8_t* lat;
  const double* V;
  const uint32_t* entries;
  const int16_t* shell_start;
  double* site_energy;        // n_sites scratch
  double* out;                // total energy
  int64_t site_offset;        // prefix over chains (for the grid-stride map)
};
void launch_total_energy(const EnergyJob* d_jobs, int n_jobs, int64_t total_sites,
                         cudaStream_t stream);

// Site energy of one site (nbr_energy), one thread.
void launch_site_energy(const EnergyJob* d_job, int x, int y, int z, double* out,
                        cudaStream_t stream);

// Conversions between the reference's full doubled grid config(1,2n1,2n2,2n3)
// (x fastest) and the compact occupied-site array.
void launch_pack(const Geom& g, const int8_t* d_grid, int8_t* d_lat, int32_t* d_status,
                 cudaStream_t stream);
void launch_unpack(const Geom& g, const int8_t* d_lat, int8_t* d_grid, cudaStream_t stream);

// The same for every chain of a batch at once: grids concatenated in chain
// order starting at grid_offset[c].
struct GridJob {
  Geom g;
  int8_t* lat;
  int64_t grid_offset;
  int32_t* status;
};
void launch_pack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells,
                       const int8_t* d_grids, cudaStream_t stream);
void launch_unpack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells, int8_t* d_grids,
                         cudaStream_t stream);

}  // namespace brawl
