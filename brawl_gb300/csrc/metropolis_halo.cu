// metropolis_halo.cu -- Metropolis-Kawasaki swap trials for fcc/bcc chains
// staged with a periodic halo (see halo_engine.cuh): the batched path's
// kernel for every lattice that fits.  One warp (CTA) per chain; trials in
// the reference's order (monte_carlo_step_lattice / _nbr,
// src/metropolis.F90:751-891) on the chain's own mt19937ar stream.
#include <climits>

#include "halo_engine.cuh"
#include "kernels.cuh"

namespace brawl {

// Species of canonical compact site i through the halo layout.
struct HaloLat {
  int sz, sy, origin, SZ, SY, off;
  __device__ __forceinline__ int operator()(int i) const {
    extern __shared__ int8_t s_i8[];
    const int Z = i / sz, r = i - Z * sz, Y = r / sy, X = r - Y * sy;
    return s_i8[off + origin + Z * SZ + Y * SY + X];
  }
};

// Fixed-point delta for any pair (neighbouring sites included), from the
// canonical neighbour indices.  Out of line: only pairs within the
// interaction range come here.
__device__ __noinline__ int halo_delta_general(const ChainJob* __restrict__ Jg, int ents_off,
                                               int I_off, int F_off, HaloLat lat, int ax, int ay,
                                               int az, int ai, int bx, int by, int bz, int bi,
                                               int sa, int sb, int lane) {
  extern __shared__ int32_t s_i32[];
  extern __shared__ uint32_t s_u32[];
  const Geom g = Jg->g;
  const bool h = lane >= 16;
  const int cx = h ? bx : ax, cy = h ? by : ay, cz = h ? bz : az;
  const int own = h ? bi : ai, other = h ? ai : bi;
  const int so = h ? sb : sa, sn = h ? sa : sb;
  const int nsp = g.ns + 1;
  const int rowN = I_off + F_off + sn * g.nsh * nsp;
  const int rowO = I_off + F_off + so * g.nsh * nsp;
  int acc = 0;
  for (int k = lane & 15; k < g.z; k += 16) {
    int dx, dy, dz, sh;
    unpack_entry(s_u32[ents_off / 4 + k], dx, dy, dz, sh);
    const int ni = neighbour_index(g, cx, cy, cz, dx, dy, dz);
    const int s_before = lat(ni);
    const int s_after = ni == other ? so : (ni == own ? sn : s_before);
    acc += s_i32[rowN + sh * nsp + s_after] - s_i32[rowO + sh * nsp + s_before];
  }
  return __reduce_add_sync(kFull, acc);
}

// The reference-order FP64 decision (see metropolis.cu); returns bit 0
// accept, bit 1 uniform drawn, bit 2 FP64 libm tier, bit 3 double-double.
__device__ __noinline__ int halo_exact_decision(const ChainJob* __restrict__ Jg, HaloLat lat,
                                                const double* V, const uint32_t* ents,
                                                const int16_t* sstart, int ax, int ay, int az,
                                                int ai, int bx, int by, int bz, int bi, int sa,
                                                int sb, int lane, uint32_t wu) {
  const Geom g = Jg->g;
  SitePair p;
  p.ax = ax; p.ay = ay; p.az = az; p.ai = ai;
  p.bx = bx; p.by = by; p.bz = bz; p.bi = bi;
  p.sa = sa; p.sb = sb;
  double e_un, e_sw;
  exact_pair_energies(g, lat, V, ents, sstart, p, lane, e_un, e_sw);
  const double delta_e = __dsub_rn(e_sw, e_un);
  if (delta_e < 0.0) return 1;
  DecideStats st = {0u, 0u};
  const int acc = u_lt_exp(wu, __dmul_rn(-Jg->beta, delta_e), st);
  return acc | 2 | (st.fp64 ? 4 : 0) | (st.cr ? 8 : 0);
}

// The species of the neighbour at entry e of a site at padded index `base`
// (relative to the staged lattice) with parity par, through the halo's
// padded offsets (the plan's arithmetic, for any entry).
__device__ __forceinline__ int halo_nbr_species(uint32_t e, int base, int par, int SZ, int SY, bool bcc) {
  extern __shared__ int8_t s_i8[];
  int dx, dy, dz, sh;
  unpack_entry(e, dx, dy, dz, sh);
  const int ddx = (par + dx) >> 1;
  const int ddy = bcc ? ((par + dy) >> 1) : dy;
  return s_i8[base + dz * SZ + ddy * SY + ddx];
}

// halo_exact_decision for a pair that is not near (the pairs halo_delta
// takes): no neighbour of either site is the other, so every neighbour
// holds the same species before and after the swap and is read through
// the padded offsets.  Lane c < 4 nsh adds, in list order from 0.0, the
// terms of shell c % nsh of evaluation c / nsh (site 1 before, site 2
// before, site 1 after, site 2 after); the shell sums are then added in
// shell order and the two sites' energies summed (nbr_energy and
// pair_energy, src/bw_hamiltonian.f90:99-114) -- the values and order of
// exact_pair_energies, so the same doubles.  Each chain's loop is unrolled
// by four, so the loads of four terms issue ahead of their adds (measured
// faster than a hand-pipelined four-ahead loop with predicated adds: 644
// against 670 cycles per trial on a two-species chain whose exact tier
// decides 1.7% of the trials).
static __device__ __noinline__ int halo_exact_far(const ChainJob* __restrict__ Jg, const double* V,
                                                  const uint32_t* ents, const int16_t* sstart, int lat_off,
                                                  int SZ, int SY, int bcc, int ns, int nsh, int pa, int pb,
                                                  int par_a, int par_b, int sa, int sb, uint32_t wu, int lane) {
  const int nc = 4 * nsh;
  double part[2] = {0.0, 0.0};
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    const int c = lane + 32 * r;
    double sum = 0.0;
    if (c < nc) {
      const int ev = c / nsh, sh = c - ev * nsh;
      const bool on2 = ev & 1, after = ev >= 2;
      const int base = lat_off + (on2 ? pb : pa);
      const int par = on2 ? par_b : par_a;
      const int cs = (on2 != after) ? sb : sa;
      // Vr[ns * s] = V(cs, s, sh) for the neighbour species s (1-based)
      const double* Vr = V + (cs - 1) + ns * ns * sh - ns;
      const int k1 = sstart[sh + 1];
      // unrolled by four: the loads of four terms issue ahead of their adds
#pragma unroll 4
      for (int k = sstart[sh]; k < k1; ++k)
        sum = __dadd_rn(sum, Vr[ns * halo_nbr_species(ents[k], base, par, SZ, SY, bcc)]);
    }
    part[r] = sum;
  }
  double e_un, e_sw;
  combine_pair_energies(part, nsh, lane, e_un, e_sw);
  const double delta_e = __dsub_rn(e_sw, e_un);
  if (delta_e < 0.0) return 1;
  DecideStats st = {0u, 0u};
  const int acc = u_lt_exp(wu, __dmul_rn(-Jg->beta, delta_e), st);
  return acc | 2 | (st.fp64 ? 4 : 0) | (st.cr ? 8 : 0);
}

// Log-domain acceptance thresholds: the uphill decision as two integer
// compares of the fixed-point energy change against bounds taken from the
// acceptance word (no exponential of the change).  The reference accepts an uphill move iff u < exp(-beta dE_ref)
// (src/metropolis.F90:802), i.e. iff t > beta dE_ref log2(e) with
// t = -log2(u) = 32 - log2(w) for u = w 2^-32.  With k = beta 2^-S log2(e)
// and the fixed-point dE within band quanta of dE_ref 2^S, the move is
// certainly accepted when dE < (t - e)/k - band and certainly rejected when
// dE > (t + e)/k + band, where e = 1e-4 bounds the error of t as computed
// here (float conversion of w, lg2.approx, the subtraction: together below
// 2e-5 on [0, 32]) with room to spare.  The float products carry a further
// relative 1e-6 and the thresholds are rounded towards the undecided side.
// Between the two, and for w = 0, the exact tier decides.
struct AcceptThresholds {
  int acc_below;  // dE < acc_below: accepted
  int rej_above;  // dE > rej_above: rejected
};

__device__ __forceinline__ AcceptThresholds accept_thresholds(uint32_t w, float inv_k, float band_f) {
  AcceptThresholds T;
  float lw;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(lw) : "f"(__uint2float_rn(w)));
  const float t = 32.0f - lw;
  const float a = __fmul_rn(__fmul_rn(t - 1e-4f, inv_k), 1.0f - 1e-6f) - band_f - 1.0f;
  const float r = __fmul_rn(__fmul_rn(t + 1e-4f, inv_k), 1.0f + 1e-6f) + band_f + 1.0f;
  // fixed-point changes stay within +-2^30: clamp before converting
  T.acc_below = w == 0u ? INT_MIN : __float2int_rd(fminf(a, 1073741824.0f));
  T.rej_above = w == 0u ? INT_MAX : __float2int_ru(fminf(r, 2147483520.0f));
  return T;
}

template <int NJ, bool FULL>
__global__ void __launch_bounds__(32) metropolis_halo_kernel(const ChainJob* __restrict__ jobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  extern __shared__ uint32_t s_u32[];
  extern __shared__ int32_t s_i32[];
  extern __shared__ int8_t s_i8[];
  const ChainJob* Jg = jobs + blockIdx.x;
  if (Jg->status && *Jg->status != 0) return;  // the chain's input was flagged: no trial runs
  const Geom g = Jg->g;
  const HaloGeom H = Jg->hg;
  const int lane = threadIdx.x;
  __shared__ unsigned long long s_t_start;  // kept out of registers
  if (lane == 0) s_t_start = global_ns();
  const HaloLayout L = halo_layout(g, H);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + L.mt);
  uint32_t* tbuf = reinterpret_cast<uint32_t*>(smem + L.tbuf);
  int32_t* ptab = reinterpret_cast<int32_t*>(smem + L.ptab);
  int32_t* ctab = reinterpret_cast<int32_t*>(smem + L.ctab);
  double* V = reinterpret_cast<double*>(smem + L.V);
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + L.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + L.sstart);
  int32_t* I = reinterpret_cast<int32_t*>(smem + L.I);
  int8_t* lat = reinterpret_cast<int8_t*>(smem + L.lat);

  // ---- stage state ------------------------------------------------------
  const int nsp = g.ns + 1;
  const int nI = nsp * nsp * g.nsh * (1 + nsp), nV = g.ns * g.ns * g.nsh;
  const uint32_t* rng = Jg->rng;
  for (int i = lane; i < kMTN; i += 32) mt[i] = rng[i];
  for (int i = lane; i < nI; i += 32) I[i] = Jg->F[i];
  for (int i = lane; i < nV; i += 32) V[i] = Jg->V[i];
  for (int i = lane; i < g.z; i += 32) ents[i] = Jg->entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = Jg->shell_start[i];
  __syncwarp();
  halo_fill(g, H, Jg->lat, lat, lane);
  const SiteDraw S = make_site_draw(g, H);
  Ring R;
  ring_init_sites(mt, tbuf, ptab, ctab, S, (int)rng[kMTN], lane, R);
  HaloPlan<NJ> P;
  make_halo_plan<NJ>(g, H, ents, lane, P);
  __syncwarp();

  const int lat_off = (int)L.lat;
  const int tb = (int)(L.tbuf / 4);
  const int pt = (int)(L.ptab / 4), ct = (int)(L.ctab / 4);
  const int I_off = (int)(L.I / 4);
  const int D_abs = I_off + L.D_off;
  const HaloLat hl = {g.sz, g.sy, H.origin, H.SZ, H.SY, lat_off};
  const bool bcc = g.lattice == kBcc;
  const int ys = g.ys;
  const int nbr_swap = Jg->nbr_swap;
  const int band = Jg->band;
  const float inv_k = 1.0f / Jg->beta_q_l2, band_f = (float)band;
  const int64_t n_trials = Jg->n_trials;
  const int n_peek = nbr_swap ? 5 : 7;
  const int n_base = nbr_swap ? 4 : 6;
  // lanes 0-7 write site 1's cells of an accepted swap, lanes 8-15 site 2's
  const bool img_b = lane >= 8;
  // 32-bit tallies (a launch runs fewer than 2^31 trials per chain, see
  // launch_metropolis_halo); the words drawn follow from them: n_base per
  // trial plus the uniforms
  unsigned int b_eval = 0, b_acc = 0, b_exact = 0;
  unsigned int c_fp64 = 0, c_cr = 0;
  const int nt = (int)n_trials;
  // the uniforms drawn follow from the words consumed: n_base a trial plus
  // one per uniform, counted through the ring's generated blocks
  const int avail0 = R.avail;
  unsigned int gens = 0;

  for (int t = 0; t < nt; ++t) {
    gens += R.avail < n_peek ? 1u : 0u;
    ring_ensure_sites(mt, tbuf, ptab, ctab, S, R, n_peek, lane);
    const int wb = tb + R.idx;
    SitePair p;
    int Ya, Xa, Yb, Xb, pa, pb, ea = 0, eb = 0;
    if (nbr_swap) {
      draw_site_halo(g, bcc, s_u32[wb], s_u32[wb + 1], s_u32[wb + 2], p.ax, p.ay, p.az, Ya, Xa);
      draw_nbr(g, s_u32[wb + 3], p.ax, p.ay, p.az, p.bx, p.by, p.bz);
      Yb = p.by >> ys;
      Xb = p.bx >> 1;
      pa = H.origin + p.az * H.SZ + Ya * H.SY + Xa;
      pb = H.origin + p.bz * H.SZ + Yb * H.SY + Xb;
    } else {
      // the two sites from the site table: padded index and parity
      ea = s_i32[pt + R.idx];
      eb = s_i32[pt + R.idx + 3];
      pa = ea & kPadMask;
      pb = eb & kPadMask;
    }
    p.sa = s_i8[lat_off + pa];
    p.sb = s_i8[lat_off + pb];
    int consumed = n_base;
    int accept = 1;  // same species: accepted without an energy evaluation or a draw
    if (p.sa != p.sb) {
      ++b_eval;
      bool par_a, par_b;
      if (nbr_swap) {
        par_a = bcc ? (p.az & 1) : (p.ax & 1);
        par_b = bcc ? (p.bz & 1) : (p.bx & 1);
      } else {
        site_coords(s_i32[ct + R.idx], p.ax, p.ay, p.az);
        site_coords(s_i32[ct + R.idx + 3], p.bx, p.by, p.bz);
        Ya = p.ay >> ys;
        Xa = p.ax >> 1;
        Yb = p.by >> ys;
        Xb = p.bx >> 1;
        par_a = ea >> 30;
        par_b = eb >> 30;
      }
      // the fast-tier sum is issued first and the near test fills its loads'
      // latency; a neighbouring pair (which the fast sum assumes away) takes
      // the general sum instead
      int dE = halo_delta<NJ, FULL>(g, lat_off, D_abs, P, pa, pb, par_a, par_b, p.sa, p.sb, lane);
      const bool near = pair_near_flat(g, H, p.ax, p.ay, p.az, p.bx, p.by, p.bz);
      if (near) {
        dE = halo_delta_general(Jg, (int)L.ents, I_off, L.F_off, hl, p.ax, p.ay, p.az,
                                p.az * g.sz + Ya * g.sy + Xa, p.bx, p.by, p.bz,
                                p.bz * g.sz + Yb * g.sy + Xb, p.sa, p.sb, lane);
      }
      const uint32_t wu = s_u32[wb + n_base];
      accept = -1;
      if (dE < -band) {
        accept = 1;
      } else if (dE > band) {
        consumed = n_base + 1;
        const AcceptThresholds th = accept_thresholds(wu, inv_k, band_f);
        accept = dE < th.acc_below ? 1 : (dE > th.rej_above ? 0 : -1);
      }
      if (accept < 0) {
        ++b_exact;
        const int r = near ? halo_exact_decision(Jg, hl, V, ents, sstart, p.ax, p.ay, p.az,
                                                 p.az * g.sz + Ya * g.sy + Xa, p.bx, p.by, p.bz,
                                                 p.bz * g.sz + Yb * g.sy + Xb, p.sa, p.sb, lane, wu)
                           : halo_exact_far(Jg, V, ents, sstart, lat_off, H.SZ, H.SY, bcc, g.ns, g.nsh, pa,
                                            pb, par_a, par_b, p.sa, p.sb, wu, lane);
        accept = r & 1;
        consumed = (r & 2) ? n_base + 1 : n_base;
        c_fp64 += (r >> 2) & 1;
        c_cr += (r >> 3) & 1;
      }
      if (accept) {
        const int img = halo_image_index(H, lane, p.az, Ya, Xa, p.bz, Yb, Xb);
        if (img >= 0) s_i8[lat_off + img] = (int8_t)(img_b ? p.sa : p.sb);
        __syncwarp();
      }
    }
    b_acc += accept;
    ring_consume(R, consumed);
  }
  const unsigned long long words =
      (unsigned long long)(avail0 - R.avail) + (unsigned long long)kMTN * gens;
  const unsigned long long c_exp = words - (unsigned long long)n_base * (unsigned long long)nt;
  const unsigned long long c_eval = b_eval, c_acc = b_acc, c_exact = b_exact;
  const unsigned long long c_draws = (unsigned long long)n_base * (unsigned long long)n_trials + c_exp;

  // ---- write back ---------------------------------------------------------
  __syncwarp();
  halo_store(g, H, lat, Jg->lat, lane);
  ring_writeback(mt, tbuf, R, Jg->rng, lane);
  if (lane == 0) {
    unsigned long long* c = Jg->counters;
    c[kCntTrials] += (unsigned long long)n_trials;
    c[kCntEvaluated] += c_eval;
    c[kCntDraws] += c_draws;
    c[kCntAccepted] += c_acc;
    c[kCntExpTests] += c_exp;
    c[kCntExactPath] += c_exact;
    c[kCntExpFp64] += c_fp64;
    c[kCntExpCr] += c_cr;
    if (Jg->t_ns) *Jg->t_ns = global_ns() - s_t_start;
  }
}

template <int NJ, bool FULL>
static void launch_halo_nj(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes,
                           cudaStream_t stream) {
  cudaFuncSetAttribute(metropolis_halo_kernel<NJ, FULL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes);
  BRAWL_CARVEOUT((metropolis_halo_kernel<NJ, FULL>));
  metropolis_halo_kernel<NJ, FULL><<<n_jobs, 32, smem_bytes, stream>>>(d_jobs);
}

void launch_metropolis_halo(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int min_z,
                            int max_z, cudaStream_t stream) {
  if (n_jobs <= 0) return;
  const int nj = lane_entries_for(max_z);
  // every chain with z = 64 (bcc, 6 shells): no lane entry to mask
  const bool full = min_z == max_z && max_z == 16 * nj;
  switch (nj) {
    case 2: launch_halo_nj<2, false>(d_jobs, n_jobs, smem_bytes, stream); break;
    case 4:
      if (full) launch_halo_nj<4, true>(d_jobs, n_jobs, smem_bytes, stream);
      else launch_halo_nj<4, false>(d_jobs, n_jobs, smem_bytes, stream);
      break;
    case 6: launch_halo_nj<6, false>(d_jobs, n_jobs, smem_bytes, stream); break;
    case 8: launch_halo_nj<8, false>(d_jobs, n_jobs, smem_bytes, stream); break;
    default: launch_halo_nj<11, false>(d_jobs, n_jobs, smem_bytes, stream); break;
  }
}

void preload_halo_kernels() {
  cudaFuncAttributes a;
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<2, false>);
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<4, false>);
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<4, true>);
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<6, false>);
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<8, false>);
  cudaFuncGetAttributes(&a, metropolis_halo_kernel<11, false>);
}

}  // namespace brawl
