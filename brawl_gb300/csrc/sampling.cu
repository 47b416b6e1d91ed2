// sampling.cu -- the per-temperature sampling reductions of
// metropolis_simulated_annealing on the device, for every chain of a batch
// (src/metropolis.F90:360-430), and the ensemble averages of
// comms_reduce_metropolis_results (src/comms.F90:122-160).
//
// Per chain the device keeps what the reference keeps per process: the sums
// step_E and step_Esq of the sampled total energies (step_E + E and
// step_Esq + E**2, in sample order, FP64), the sum r_densities of the
// sampled radial densities, and the accepted-move count at the start of the
// sampling loop.  At the end of a temperature one launch forms
// energies_of_T = step_E / n_save / n_atoms, the heat capacity
// (step_Esq / n_save - (step_E / n_save)**2) / (sim_temp * temp) / n_atoms
// clamped at zero, acceptance_of_T = accepted / real(n_mc_steps) and
// rho_of_T = r_densities / n_save_asro, then every quantity's sum over the
// chains in chain order (the ranks' MPI_SUM in rank order) divided by
// real(p).  Every operation is a separately rounded FP64 operation in the
// reference's order, so the values are the host loop's bit for bit.
#include "kernels.cuh"

namespace brawl {

// step_E += E, step_Esq += E * E (src/metropolis.F90:363-367) when sums is
// set; the energy also copied to a trajectory row when traj is set
__global__ void energy_accumulate_kernel(const double* __restrict__ e, double* __restrict__ sums,
                                         double* __restrict__ traj, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double E = e[c];
  if (sums) {
    sums[c] = __dadd_rn(sums[c], E);
    sums[n + c] = __dadd_rn(sums[n + c], __dmul_rn(E, E));
  }
  if (traj) traj[c] = E;
}

// the accepted-move counters at the start of the sampling loop
__global__ void acceptance_snapshot_kernel(const unsigned long long* __restrict__ counters,
                                           unsigned long long* __restrict__ acc0, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) acc0[c] = counters[(size_t)c * kNumCounters + kCntAccepted];
}

// rho(i, j, l) = count / particle_count(i) for one chain (radial_densities'
// last step, src/analytics.f90:388-400), written to rho_out and added to
// the chain's sums (r_densities = r_densities + asro, :381-383)
__global__ void asro_finish_kernel(const unsigned long long* __restrict__ counts,
                                   const unsigned long long* __restrict__ class_mask, int n_class,
                                   int ns, int wc, double* __restrict__ rho_out,
                                   double* __restrict__ rho_sum) {
  const int nsp = ns + 1;
  const unsigned long long* pc = counts + (size_t)nsp * nsp * n_class;
  const int total = ns * ns * wc;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int i = t % ns + 1, j = (t / ns) % ns + 1, l = t / (ns * ns);
    unsigned long long c = 0;
    for (int k = 0; k < n_class; ++k)
      if ((class_mask[k] >> l) & 1ull) c += counts[(i * nsp + j) * n_class + k];
    const double r = __ddiv_rn((double)c, (double)(long long)pc[i]);
    if (rho_out) rho_out[t] = r;
    rho_sum[t] = __dadd_rn(rho_sum[t], r);
  }
}

// Per chain (one thread each): energies_of_T, C_of_T, acceptance_of_T
// (src/metropolis.F90:410-428); then thread 0 sums each over the chains in
// order and divides by real(p) (src/comms.F90:130-150).
__global__ void temperature_stats_kernel(int n, const double* __restrict__ sums,
                                         const unsigned long long* __restrict__ counters,
                                         const unsigned long long* __restrict__ acc0,
                                         const double* __restrict__ n_atoms, double n_save,
                                         double sim_temp, double temp, double n_mc_real,
                                         int with_energies, double* __restrict__ out) {
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    double e_T = 0.0, C = 0.0;
    if (with_energies) {
      const double sE = sums[c], sEsq = sums[n + c];
      e_T = __ddiv_rn(__ddiv_rn(sE, n_save), n_atoms[c]);
      const double mean = __ddiv_rn(sE, n_save);
      C = __ddiv_rn(__ddiv_rn(__dsub_rn(__ddiv_rn(sEsq, n_save), __dmul_rn(mean, mean)),
                              __dmul_rn(sim_temp, temp)),
                    n_atoms[c]);
      if (C < 0.0 || temp <= 0.0) C = 0.0;
    }
    const unsigned long long a = counters[(size_t)c * kNumCounters + kCntAccepted] - acc0[c];
    out[c] = e_T;
    out[n + c] = C;
    out[2 * n + c] = __ddiv_rn((double)(long long)a, n_mc_real);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double p = (double)(float)n;
    for (int q = 0; q < 3; ++q) {
      double s = out[q * n];
      for (int c = 1; c < n; ++c) s = __dadd_rn(s, out[q * n + c]);
      out[3 * n + q] = __ddiv_rn(s, p);
    }
  }
}

// rho_of_T = r_densities / real(n_save_asro) per chain, then the chains'
// sum in order divided by real(p) (src/comms.F90:152-158); m values each.
__global__ void asro_stats_kernel(int n, int m, const double* __restrict__ rho_sum,
                                  double n_save, double* __restrict__ out) {
  const double p = (double)(float)n;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < n; ++c) {
      const double r = __ddiv_rn(rho_sum[(size_t)c * m + t], n_save);
      out[(size_t)c * m + t] = r;
      s = c == 0 ? r : __dadd_rn(s, r);
    }
    out[(size_t)n * m + t] = __ddiv_rn(s, p);
  }
}

void launch_energy_accumulate(const double* d_e, double* d_sums, double* d_traj, int n, cudaStream_t s) {
  BRAWL_CARVEOUT(energy_accumulate_kernel);
  energy_accumulate_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_e, d_sums, d_traj, n);
}

void launch_acceptance_snapshot(const unsigned long long* d_counters, unsigned long long* d_acc0, int n,
                                cudaStream_t s) {
  BRAWL_CARVEOUT(acceptance_snapshot_kernel);
  acceptance_snapshot_kernel<<<(n + 127) / 128, 128, 0, s>>>(d_counters, d_acc0, n);
}

void launch_asro_finish(const unsigned long long* d_counts, const unsigned long long* d_mask, int n_class,
                        int ns, int wc, double* d_rho_out, double* d_rho_sum, cudaStream_t s) {
  BRAWL_CARVEOUT(asro_finish_kernel);
  const int total = ns * ns * wc;
  asro_finish_kernel<<<(total + 127) / 128, 128, 0, s>>>(d_counts, d_mask, n_class, ns, wc, d_rho_out,
                                                         d_rho_sum);
}

void launch_temperature_stats(int n, const double* d_sums, const unsigned long long* d_counters,
                              const unsigned long long* d_acc0, const double* d_n_atoms, double n_save,
                              double sim_temp, double temp, double n_mc_real, int with_energies,
                              double* d_out, cudaStream_t s) {
  BRAWL_CARVEOUT(temperature_stats_kernel);
  temperature_stats_kernel<<<1, 256, 0, s>>>(n, d_sums, d_counters, d_acc0, d_n_atoms, n_save, sim_temp,
                                             temp, n_mc_real, with_energies, d_out);
}

void launch_asro_stats(int n, int m, const double* d_rho_sum, double n_save, double* d_out, cudaStream_t s) {
  BRAWL_CARVEOUT(asro_stats_kernel);
  asro_stats_kernel<<<(m + 127) / 128, 128, 0, s>>>(n, m, d_rho_sum, n_save, d_out);
}

}  // namespace brawl
