// wl_kernels.cuh -- device state of Wang-Landau walkers and their launches.
#pragma once

#include "kernels.cuh"

namespace brawl {

struct WlWalker {
  ChainJob job;          // geometry, tables, stream, counters, status, lattice
  double* lng;           // ln g over all bins (the reference's wl_logdos)
  double* hist;          // the window's histogram (mpi_wl_hist), end-start+1
  int32_t start, end;    // 1-based window bins
  int32_t bins;
  int32_t hist_period;   // INT(0.02*REAL(n_atoms))
  double e0;             // e_unswapped at entry: full_energy(config)
  double e_out;          // e_unswapped at exit
  double wl_f;
  double e1, range;      // bin_edges(1), bin_edges(bins+1) - bin_edges(1)
  int64_t n_trials;
  int64_t accepted;
};

// Walkers first..first+count-1 share a window and are averaged together.
struct WlGroup {
  int32_t first, count;
};

uint32_t wl_smem_bytes(const Geom& g, int nb);
void launch_wl_sweeps(WlWalker* d_walkers, int n, uint32_t smem, cudaStream_t stream);
void launch_wl_average(const WlGroup* d_groups, int n_groups, WlWalker* d_walkers, int bins,
                       cudaStream_t stream);

}  // namespace brawl
