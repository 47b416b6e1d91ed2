// metropolis.cu -- Metropolis-Kawasaki swap trials for a batch of chains.
//
// Each CTA is one warp and owns one chain for the whole launch: it stages the
// chain's lattice (compact uint8), its mt19937ar block, its interaction
// tables and the per-axis wrap tables in shared memory, runs n_trials of
// monte_carlo_step_lattice (src/metropolis.F90:751-813) or
// monte_carlo_step_nbr (:829-891) in the reference's order, and writes the
// state back.  A batch of one chain is the plain one-chain-per-launch path; a
// batch of many is the batched path.
#include "kernels.cuh"

namespace brawl {

// The reference-order FP64 decision for one trial (rare: only when the
// fixed-point value is within the band).  Kept out of line so the hot loop
// stays small; reads the job from global memory.  Returns bit 0 accept,
// bit 1 the acceptance uniform was drawn, bit 2 the FP64 libm tier was
// needed, bit 3 the double-double tier.
__device__ __noinline__ int exact_decision(const ChainJob* __restrict__ Jg, const int8_t* lat,
                                           const double* V, const uint32_t* ents,
                                           const int16_t* sstart, int ax, int ay, int az, int ai,
                                           int bx, int by, int bz, int bi, int sa, int sb,
                                           int lane, uint32_t wu) {
  const Geom g = Jg->g;
  SitePair p;
  p.ax = ax; p.ay = ay; p.az = az; p.ai = ai;
  p.bx = bx; p.by = by; p.bz = bz; p.bi = bi;
  p.sa = sa; p.sb = sb;
  double e_un, e_sw;
  exact_pair_energies(g, CompactLat{lat}, V, ents, sstart, p, lane, e_un, e_sw);
  const double delta_e = __dsub_rn(e_sw, e_un);
  if (delta_e < 0.0) return 1;
  DecideStats st = {0u, 0u};
  const int acc = u_lt_exp(wu, __dmul_rn(-Jg->beta, delta_e), st);
  return acc | 2 | (st.fp64 ? 4 : 0) | (st.cr ? 8 : 0);
}

template <int NJ, bool kSmemLat, bool kUseD>
__global__ void __launch_bounds__(32) metropolis_kernel(const ChainJob* __restrict__ jobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const ChainJob J = jobs[blockIdx.x];
  if (J.status && *J.status != 0) return;  // the chain's input was flagged: no trial runs
  const Geom g = J.g;
  const int lane = threadIdx.x;
  __shared__ unsigned long long s_t_start;  // kept out of registers
  __shared__ unsigned long long* s_t_ns;
  if (lane == 0) {
    s_t_start = global_ns();
    s_t_ns = jobs[blockIdx.x].t_ns;
  }
  const SmemLayout L = smem_layout(g, kSmemLat);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + L.mt);
  int32_t* I = reinterpret_cast<int32_t*>(smem + L.I);
  double* V = reinterpret_cast<double*>(smem + L.V);
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + L.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + L.sstart);
  int8_t* lat = kSmemLat ? reinterpret_cast<int8_t*>(smem + L.lat) : J.lat;

  // ---- stage state ------------------------------------------------------
  const int nsp = g.ns + 1;
  const int nF = nsp * nsp * g.nsh * (L.use_D ? 1 + nsp : 1), nV = g.ns * g.ns * g.nsh;
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nF; i += 32) I[L.F_off + i] = J.F[i];
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
  AxisTables T;
  build_axis_tables(g, I, L.tab_len, lane, T);
  int pos = (int)J.rng[kMTN];
  __syncwarp();

  LanePlan<NJ> P;
  make_lane_plan<NJ>(g, ents, I, T, lane, P);
  const int lat_off = (int)L.lat, I_off = (int)(L.I / 4);
  // an entry can map a site onto itself only when a wrap period is within
  // the offsets' reach
  const bool self_map = g.W1 <= kHalo || g.W2 <= kHalo || g.W3 <= kHalo;

  const int n_peek = J.nbr_swap ? 5 : 7;
  const int n_base = J.nbr_swap ? 4 : 6;
  unsigned long long c_eval = 0, c_draws = 0, c_acc = 0, c_exp = 0, c_exact = 0;
  unsigned int c_fp64 = 0, c_cr = 0;
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
    int accept = 1;  // same species: accepted without an energy evaluation or a draw
    if (p.sa != p.sb) {
      ++c_eval;
      bool near;
      int dE = fixed_delta<NJ, kSmemLat, kUseD>(g, lat, lat_off, I_off, L.F_off, L.D_off, P, p,
                                                lane, near);
      if (near || self_map)
        dE = fixed_delta_general<kSmemLat>(g.lattice, g.ns, g.nsh, g.z, lat, lat_off, I_off,
                                           L.F_off, (int)L.ents,
                                           (int)L.tab_len[0], (int)L.tab_len[1],
                                           (int)L.tab_len[2], p.ax, p.ay, p.az, p.ai, p.bx, p.by,
                                           p.bz, p.bi, p.sa, p.sb, lane);
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
        const int r = exact_decision(jobs + blockIdx.x, lat, V, ents, sstart, p.ax, p.ay, p.az,
                                     p.ai, p.bx, p.by, p.bz, p.bi, p.sa, p.sb, lane, wu);
        accept = r & 1;
        consumed = (r & 2) ? n_base + 1 : n_base;
        c_fp64 += (r >> 2) & 1;
        c_cr += (r >> 3) & 1;
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
    c[kCntExpFp64] += c_fp64;
    c[kCntExpCr] += c_cr;
    if (status != kStatusOk) *J.status = status;
    if (s_t_ns) *s_t_ns = global_ns() - s_t_start;
  }
}

template <int NJ, bool kSmemLat, bool kUseD>
static void launch_one(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes,
                       cudaStream_t stream) {
  cudaFuncSetAttribute(metropolis_kernel<NJ, kSmemLat, kUseD>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  BRAWL_CARVEOUT(metropolis_kernel<NJ, kSmemLat, kUseD>);
  metropolis_kernel<NJ, kSmemLat, kUseD><<<n_jobs, 32, smem_bytes, stream>>>(d_jobs);
}

template <int NJ>
static void launch_nj(const ChainJob* d_jobs, int n_jobs, bool smem_lat, bool use_D,
                      uint32_t smem_bytes, cudaStream_t stream) {
  if (smem_lat) {
    if (use_D) launch_one<NJ, true, true>(d_jobs, n_jobs, smem_bytes, stream);
    else launch_one<NJ, true, false>(d_jobs, n_jobs, smem_bytes, stream);
  } else {
    if (use_D) launch_one<NJ, false, true>(d_jobs, n_jobs, smem_bytes, stream);
    else launch_one<NJ, false, false>(d_jobs, n_jobs, smem_bytes, stream);
  }
}

int lane_entries_for(int max_z) {
  const int nj = (max_z + 15) / 16;
  return nj <= 2 ? 2 : nj <= 4 ? 4 : nj <= 6 ? 6 : nj <= 8 ? 8 : 11;
}

void launch_metropolis(const ChainJob* d_jobs, int n_jobs, bool lattice_in_smem, bool use_D,
                       uint32_t smem_bytes, int max_z, cudaStream_t stream) {
  if (n_jobs <= 0) return;
  switch (lane_entries_for(max_z)) {
    case 2: launch_nj<2>(d_jobs, n_jobs, lattice_in_smem, use_D, smem_bytes, stream); break;
    case 4: launch_nj<4>(d_jobs, n_jobs, lattice_in_smem, use_D, smem_bytes, stream); break;
    case 6: launch_nj<6>(d_jobs, n_jobs, lattice_in_smem, use_D, smem_bytes, stream); break;
    case 8: launch_nj<8>(d_jobs, n_jobs, lattice_in_smem, use_D, smem_bytes, stream); break;
    default: launch_nj<11>(d_jobs, n_jobs, lattice_in_smem, use_D, smem_bytes, stream); break;
  }
}

// Loads every variant's code now (module loading is lazy by default, and a
// first launch that loads code waits for the kernels already running).
template <int NJ>
static void preload_nj(cudaFuncAttributes& a) {
  cudaFuncGetAttributes(&a, metropolis_kernel<NJ, true, true>);
  cudaFuncGetAttributes(&a, metropolis_kernel<NJ, true, false>);
  cudaFuncGetAttributes(&a, metropolis_kernel<NJ, false, true>);
  cudaFuncGetAttributes(&a, metropolis_kernel<NJ, false, false>);
}

void preload_metropolis_kernels() {
  cudaFuncAttributes a;
  preload_nj<2>(a);
  preload_nj<4>(a);
  preload_nj<6>(a);
  preload_nj<8>(a);
  preload_nj<11>(a);
}

}  // namespace brawl
