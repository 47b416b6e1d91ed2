// wl_kernels.cuh -- device state of Wang-Landau walkers and their launches.
#pragma once

#include "kernels.cuh"

namespace brawl {

// The radial-density samples that sweeps() takes per bin
// (src/wang-landau.F90:566-586), shared by the walkers of a batch: the
// ASRO plan (packed offsets with their shell class, asro.cuh), the per-walker
// cap MAX(radial_samples / num_walkers, 1) and radial_record_bool.
struct WlRadial {
  const uint32_t* offsets;
  const unsigned long long* class_masks;
  const uint8_t* done;   // bins
  int32_t n_offsets, n_class;
  int32_t wc_range, cap;
};

struct WlWalker {
  ChainJob job;          // geometry, tables, stream, counters, status, lattice
  double* lng;           // ln g over all bins (the reference's wl_logdos)
  double* hist;          // the window's histogram (mpi_wl_hist), end-start+1
  int32_t start, end;    // 1-based window bins
  int32_t bins;
  int32_t hist_period;   // INT(0.02*REAL(n_atoms))
  const double* e0_src;  // full_energy(config) at entry, on the device
  double e0;             // e_unswapped at entry (when e0_src is null)
  double e_out;          // e_unswapped at exit
  double wl_f;
  double e1, range;      // bin_edges(1), bin_edges(bins+1) - bin_edges(1)
  int64_t n_trials;
  int64_t accepted;
  // A sweeps() call may run as several launches: i0 trials of the call are
  // done, and e_state (when set) carries e_unswapped between the launches.
  int64_t i0;
  double* e_state;
  int32_t S;             // fixed-point shift of the chain's F table
  int32_t lazy_cap;      // moves the deferred-energy log holds (>= 1)
  // radial-density samples (all null when off): the plan, this walker's
  // radial_record (bins), rho_of_E (bins x wc x ns x ns, rho(i, j, l, bin)
  // with i fastest) and radial_mc_steps
  const WlRadial* radial;
  int32_t* radial_record;
  double* rho_of_E;
  int32_t* radial_steps;
  int32_t rad_n_offsets, rad_n_class;  // the plan's sizes (shared memory)
  // configuration store (config_per_bin / config_store, null when off):
  // bins slots of n_sites bytes in the compact device layout, and one flag
  // per bin, set while the bin's slot is still open
  int8_t* store;
  uint8_t* store_open;
};

// enter_energy_window (src/wang-landau.F90:643-741) for one walker.
struct WlEnterJob {
  ChainJob job;          // lattice (compact), stream, V, entries, shell starts
  InitJob init;          // initial_setup of the redraws (and of the start)
  double min_e, max_e;   // the window's outer bin edges
  double sig2x2;         // 2 (0.0025 |E_max - E_min| n_atoms / (Ry_to_eV 1000))^2
  int64_t max_steps;
  double* site_e;        // n_sites scratch for full_energy
  int64_t steps;         // out: loop iterations, -1 when max_steps ran out
  double energy;         // out: the final full_energy
  int32_t initial;       // draw the starting configuration with initial_setup first
  int32_t pad;
};

uint32_t wl_enter_smem_bytes(const Geom& g);
void launch_wl_enter(WlEnterJob* d_jobs, int n, uint32_t smem, cudaStream_t stream);

// Walkers first..first+count-1 share a window and are averaged together.
struct WlGroup {
  int32_t first, count;
};

// Shared memory of a walker's sweep; lazy_cap 0 gives the bytes without the
// deferred-energy log; rad_bins > 0 adds the radial-sample scratch.
uint32_t wl_smem_bytes(const Geom& g, int nb, int lazy_cap, int rad_bins = 0, int rad_n_offsets = 0,
                       int rad_n_class = 0);
// max_z: the largest neighbour count of the walkers; all_D: every walker's
// difference table D is staged (walker_layout's use_D).
void launch_wl_sweeps(WlWalker* d_walkers, int n, uint32_t smem, int max_z, bool all_D,
                      cudaStream_t stream);
void launch_wl_average(const WlGroup* d_groups, int n_groups, WlWalker* d_walkers, int bins,
                       int with_hist, cudaStream_t stream);
uint32_t wl_exchange_smem_bytes(int per_window);
void launch_wl_exchange(WlWalker* d_walkers, const double* d_energy, const WlGroup* d_groups,
                        int n_windows, int per_window, int* d_ibin, int2* d_ov, int* d_partner,
                        int* d_exchanged, int* d_n_accepted, cudaStream_t stream);
void launch_wl_flatness(const WlWalker* d_walkers, int n, double* d_out, cudaStream_t stream);
void launch_wl_combine(WlWalker* d_walkers, int n, const WlGroup* d_groups, int n_groups, int bins,
                       double* d_out, int* d_status, cudaStream_t stream);
// merge_configs' copies: pick[bins] (device) names the walker whose slot each
// bin takes, or -1
void launch_wl_store_merge(const WlWalker* d_walkers, int n, int bins, const int* d_pick, cudaStream_t stream);

}  // namespace brawl
