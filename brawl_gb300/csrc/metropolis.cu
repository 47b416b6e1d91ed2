// metropolis.cu -- Metropolis-Kawasaki swap trials for a batch of chains.
//
// Each CTA is one warp and owns one chain for the whole launch: it stages the
// chain's lattice (compact uint8), its mt19937ar block and its interaction
// tables in shared memory, runs n_trials of monte_carlo_step_lattice
// (src/metropolis.F90:751-813) or monte_carlo_step_nbr (:829-891) in the
// reference's order, and writes the state back.  A batch of one chain is the
// plain one-chain-per-launch path; a batch of many is the batched path.
#include "kernels.cuh"

namespace brawl {

template <bool kSmemLat>
__global__ void __launch_bounds__(32) metropolis_kernel(const ChainJob* __restrict__ jobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const ChainJob J = jobs[blockIdx.x];
  const Geom g = J.g;
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(g, kSmemLat);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + L.mt);
  int32_t* F = reinterpret_cast<int32_t*>(smem + L.F);
  double* V = reinterpret_cast<double*>(smem + L.V);
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + L.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + L.sstart);
  int8_t* lat = kSmemLat ? reinterpret_cast<int8_t*>(smem + L.lat) : J.lat;

  // ---- stage state ------------------------------------------------------
  const int nsp = g.ns + 1;
  const int nF = nsp * nsp * g.nsh, nV = g.ns * g.ns * g.nsh;
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nF; i += 32) F[i] = J.F[i];
  for (int i = lane; i < nV; i += 32) V[i] = J.V[i];
  for (int i = lane; i < g.z; i += 32) ents[i] = J.entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = J.shell_start[i];
  if (kSmemLat) {
    const int n16 = g.n_sites >> 4;
    const uint4* src = reinterpret_cast<const uint4*>(J.lat);
    uint4* dst = reinterpret_cast<uint4*>(lat);
    for (int i = lane; i < n16; i += 32) dst[i] = src[i];
    for (int i = (n16 << 4) + lane; i < g.n_sites; i += 32) lat[i] = J.lat[i];
  }
  int pos = (int)J.rng[kMTN];
  __syncwarp();

  LaneEntries le;
  load_lane_entries(ents, g.z, lane, le);

  const int n_peek = J.nbr_swap ? 5 : 7;
  const int n_base = J.nbr_swap ? 4 : 6;
  unsigned long long c_eval = 0, c_draws = 0, c_acc = 0, c_exp = 0, c_exact = 0;
  DecideStats st = {0u, 0u};
  int status = kStatusOk;

  for (int64_t t = 0; t < J.n_trials; ++t) {
    const uint32_t w = mt_peek(mt, pos, n_peek, lane);
    const uint32_t w0 = __shfl_sync(kFull, w, 0), w1 = __shfl_sync(kFull, w, 1),
                   w2 = __shfl_sync(kFull, w, 2), w3 = __shfl_sync(kFull, w, 3);
    SitePair p;
    draw_site(g, w0, w1, w2, p.ax, p.ay, p.az);
    if (J.nbr_swap) {
      draw_nbr(g, w3, p.ax, p.ay, p.az, p.bx, p.by, p.bz);
    } else {
      const uint32_t w4 = __shfl_sync(kFull, w, 4), w5 = __shfl_sync(kFull, w, 5);
      draw_site(g, w3, w4, w5, p.bx, p.by, p.bz);
    }
    p.ai = compact_index(g, p.ax, p.ay, p.az);
    p.bi = compact_index(g, p.bx, p.by, p.bz);
    p.sa = lat[p.ai];
    p.sb = lat[p.bi];
    int consumed = n_base;
    int accept;
    if (p.sa == p.sb) {
      // same species: accepted without an energy evaluation or a draw
      accept = 1;
    } else {
      ++c_eval;
      const int dE = fixed_delta(g, lat, F, le, p);
      const uint32_t wu = __shfl_sync(kFull, w, n_base);
      accept = -1;
      if (dE < -J.band) {
        accept = 1;
      } else if (dE > J.band) {
        consumed = n_base + 1;
        accept = fast_exp_decision(J, dE, wu);
      }
      if (accept < 0) {
        // decision inside the band: the reference's FP64 sums, in its order
        ++c_exact;
        double e_un, e_sw;
        exact_pair_energies(g, lat, V, ents, sstart, p, lane, e_un, e_sw);
        const double delta_e = __dsub_rn(e_sw, e_un);
        if (delta_e < 0.0) {
          consumed = n_base;
          accept = 1;
        } else {
          consumed = n_base + 1;
          accept = u_lt_exp(wu, __dmul_rn(-J.beta, delta_e), st);
        }
      }
      if (consumed > n_base) ++c_exp;
      if (accept && lane == 0) {
        lat[p.ai] = (int8_t)p.sb;
        lat[p.bi] = (int8_t)p.sa;
      }
      __syncwarp();
    }
    c_acc += accept;
    c_draws += consumed;
    pos += consumed;
    if (pos < 0) status = kStatusRngInvariant;
  }

  // ---- write back ---------------------------------------------------------
  __syncwarp();
  if (pos < 0) pos = 0;
  for (int i = lane; i < kMTN; i += 32) J.rng[i] = mt[i];
  if (lane == 0) J.rng[kMTN] = (uint32_t)pos;
  if (kSmemLat) {
    const int n16 = g.n_sites >> 4;
    const uint4* src = reinterpret_cast<const uint4*>(lat);
    uint4* dst = reinterpret_cast<uint4*>(J.lat);
    for (int i = lane; i < n16; i += 32) dst[i] = src[i];
    for (int i = (n16 << 4) + lane; i < g.n_sites; i += 32) J.lat[i] = lat[i];
  }
  if (lane == 0) {
    unsigned long long* c = J.counters;
    c[kCntTrials] += (unsigned long long)J.n_trials;
    c[kCntEvaluated] += c_eval;
    c[kCntDraws] += c_draws;
    c[kCntAccepted] += c_acc;
    c[kCntExpTests] += c_exp;
    c[kCntExactPath] += c_exact;
    c[kCntExpFp64] += st.fp64;
    c[kCntExpCr] += st.cr;
    if (status != kStatusOk) *J.status = status;
  }
}

void launch_metropolis(const ChainJob* d_jobs, int n_jobs, bool lattice_in_smem,
                       uint32_t smem_bytes, cudaStream_t stream) {
  if (n_jobs <= 0) return;
  if (lattice_in_smem) {
    cudaFuncSetAttribute(metropolis_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes);
    metropolis_kernel<true><<<n_jobs, 32, smem_bytes, stream>>>(d_jobs);
  } else {
    cudaFuncSetAttribute(metropolis_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes);
    metropolis_kernel<false><<<n_jobs, 32, smem_bytes, stream>>>(d_jobs);
  }
}

}  // namespace brawl
