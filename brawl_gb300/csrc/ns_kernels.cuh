// ns_kernels.cuh -- device state of a nested-sampling run and its launches.
#pragma once

#include "kernels.cuh"

namespace brawl {

struct NsRun {
  ChainJob job;        // geometry, tables, stream, counters, status
  InitJob init;        // initial_setup quotas and interval bounds
  int8_t* walkers;     // K * n_sites compact configurations
  double* energies;    // K
  uint32_t* rnde;      // K: the jitter word drawn after each initial_setup
  double* limits;      // n_iter ceilings written by the current launch
  int32_t K, n_steps;
  int32_t n_at;        // n_1*n_2*n_3*n_basis*n_species (nested_sampling.f90:82)
  int32_t half;        // int(K / 2.0) in single precision
  int32_t S;           // fixed-point shift of F
  int32_t extra_steps;
  int64_t n_acc;       // accepted steps of the latest walk
  int64_t iter;        // iterations done
  int32_t n_iter;      // iterations of the current launch
  int32_t lazy_cap;    // steps the deferred-energy log holds (>= 1)
};

// Shared memory of a run's walks; lazy_cap 0 gives the bytes without the
// deferred-energy log.
uint32_t ns_smem_bytes(const Geom& g, int lazy_cap);
void launch_ns_init(NsRun* d_runs, int n_runs, cudaStream_t stream);
void launch_ns_jitter(NsRun* d_runs, int n_runs, int max_K, cudaStream_t stream);
// max_z: the largest neighbour count of the runs; all_D: every run's
// difference table D is staged (walker_layout's use_D).
void launch_ns_iterate(NsRun* d_runs, int n_runs, uint32_t smem_bytes, int max_z, bool all_D,
                       cudaStream_t stream);

}  // namespace brawl
