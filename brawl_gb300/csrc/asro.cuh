// asro.cuh -- ASRO pair counts (radial_densities, src/analytics.f90:293-404)
// and the coordination-shell distances they are binned by (lattice_shells,
// src/analytics.f90:205-275).
#pragma once

#include <cstdint>
#include <vector>

#include "chain_engine.cuh"

namespace brawl {

// radial_densities visits, for every occupied site, the periodic offsets in
// [-m, m]^3 with m = min(n, 5) per axis, and adds one pair count to every
// shell l whose distance is within 1e-3 of the minimum-image distance.  That
// distance depends on the offset alone (for |d| = n both wraps give the same
// |dx|), so the host resolves each offset once: offsets that reach an empty
// sublattice or match no shell are dropped, and the rest are grouped by the
// set of shells they match ("class").  The kernel then only counts
// (species_i, species_j, class) triples, exactly, in integers.
struct AsroPlan {
  std::vector<uint32_t> offsets;  // packed (dx, dy, dz, class)
  std::vector<uint64_t> class_mask;
  int n_class = 0;
};

struct AsroJob {
  Geom g;
  const int8_t* lat;
  const uint32_t* offsets;
  int32_t n_offsets, n_class;
  unsigned long long* counts;          // (ns+1)^2 * n_class
  unsigned long long* species_counts;  // ns+1
};

int make_asro_plan(const Geom& g, int wc_range, const double* shells, AsroPlan& plan);
void launch_asro(const AsroJob* d_job, const Geom& g, int n_class, cudaStream_t stream);
// rho(i, j, l) = counts / particle_counts(i), column-major (ns, ns, wc).
void finish_asro(const Geom& g, int wc_range, const AsroPlan& plan,
                 const unsigned long long* counts, double* rho);
void lattice_shells_host(const Geom& g, int wc_range, double* shells);

}  // namespace brawl
