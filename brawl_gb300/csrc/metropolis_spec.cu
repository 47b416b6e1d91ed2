// metropolis_spec.cu -- speculative rounds of Metropolis-Kawasaki swap trials
// for fcc/bcc chains staged with a periodic halo.
//
// A chain's trials are sequential, and a trial's result depends on the
// previous ones in two ways only: where its six (or seven) mt19937ar words
// start, and the lattice it reads.  A trial draws six words (the two sites,
// monte_carlo_step_lattice, src/metropolis.F90:751-813) and a seventh only
// when the species differ and dE >= 0.  So trial d of a round starts at
// offset 6d + m, m being how many of the d earlier trials drew a seventh
// word (4d + m with nbr_swap).  A round of NC trials evaluates every
// candidate (d, m), 0 <= m <= d, at once, one warp each, all on the lattice
// as it stood at the start of the round.  The trials are then resolved in
// order: trial d takes candidate (d, m_d).  That candidate is valid unless an
// accepted swap of an earlier trial in the round lies within interaction
// range of one of its sites, i.e. the swap touched a site the candidate read.
// At the first such conflict the round stops, and the trial is re-evaluated
// in the next round on the updated lattice.  Resolved swaps touch disjoint
// sites and are written in parallel.  The result is the sequential kernel's:
// same words, same decisions, same lattice, same counters.
#include "halo_engine.cuh"
#include "kernels.cuh"

namespace brawl {

namespace {

// One candidate's outcome.  hdr: words consumed (bits 0-3), the trial's
// return value (bit 4), the lattice changes (bit 5), counters (bits 8-12:
// evaluated, seventh word, exact tier, FP64 exp, double-double exp).
// xy / zz: the two sites' doubled coordinates, 16 bits each (ax | ay << 16,
// bx | by << 16, az | bz << 16).  wr: the halo writes of an accepted swap,
// one per lane of the first half warp (padded index | species << 24, or -1).
struct __align__(16) SpecSlot {
  int32_t hdr;
  int32_t a_xy, b_xy, zz;
  int32_t wr[16];
};

// Whether an accepted swap at slot q touched a site that candidate s read:
// lanes 0-3 test the four (site of q, site of s) pairs, the warp votes.
__device__ __forceinline__ bool spec_conflict(const Geom& g, const HaloGeom& H, int4 q, int4 s, int lane) {
  const int c = lane & 3;
  const int qxy = (c & 2) ? q.z : q.y, sxy = (c & 1) ? s.z : s.y;
  const int qz = (c & 2) ? (q.w >> 16) : (q.w & 0xffff), sz = (c & 1) ? (s.w >> 16) : (s.w & 0xffff);
  const bool near = pair_near(g, H, qxy & 0xffff, qxy >> 16, qz, sxy & 0xffff, sxy >> 16, sz);
  return __ballot_sync(kFull, near && lane < 4) != 0u;
}

struct SpecLat {
  int sz, sy, origin, SZ, SY, off;
  __device__ __forceinline__ int operator()(int i) const {
    extern __shared__ int8_t s_i8[];
    const int Z = i / sz, r = i - Z * sz, Y = r / sy, X = r - Y * sy;
    return s_i8[off + origin + Z * SZ + Y * SY + X];
  }
};

__device__ __noinline__ int spec_delta_general(const ChainJob* __restrict__ Jg, int ents_off, int I_off,
                                               int F_off, SpecLat lat, int ax, int ay, int az, int ai,
                                               int bx, int by, int bz, int bi, int sa, int sb, int lane) {
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

__device__ __noinline__ int spec_exact_decision(const ChainJob* __restrict__ Jg, SpecLat lat, const double* V,
                                                const uint32_t* ents, const int16_t* sstart, int ax, int ay,
                                                int az, int ai, int bx, int by, int bz, int bi, int sa, int sb,
                                                int lane, uint32_t wu) {
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

// candidate index of (trial d, extra words m)
__host__ __device__ constexpr int spec_slot(int d, int m) { return d * (d + 1) / 2 + m; }

}  // namespace

template <int NJ, int NC>
__global__ void __launch_bounds__(32 * (NC * (NC + 1) / 2))
    metropolis_spec_kernel(const ChainJob* __restrict__ jobs) {
  constexpr int W = NC * (NC + 1) / 2;
  extern __shared__ __align__(16) unsigned char smem[];
  extern __shared__ uint32_t s_u32[];
  extern __shared__ int8_t s_i8[];
  __shared__ SpecSlot slots[W];
  __shared__ unsigned long long s_t_start;
  const ChainJob* Jg = jobs + blockIdx.x;
  if (Jg->status && *Jg->status != 0) return;  // the chain's input was flagged: no trial runs
  const Geom g = Jg->g;
  const HaloGeom H = Jg->hg;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_t_start = global_ns();
  const HaloLayout L = halo_layout(g, H);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + L.mt);
  uint32_t* tbuf = reinterpret_cast<uint32_t*>(smem + L.tbuf);
  double* V = reinterpret_cast<double*>(smem + L.V);
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + L.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + L.sstart);
  int32_t* I = reinterpret_cast<int32_t*>(smem + L.I);
  int8_t* lat = reinterpret_cast<int8_t*>(smem + L.lat);

  // ---- stage state ------------------------------------------------------
  const int nsp = g.ns + 1;
  const int nI = nsp * nsp * g.nsh * (1 + nsp), nV = g.ns * g.ns * g.nsh;
  const uint32_t* rng = Jg->rng;
  for (int i = tid; i < kMTN; i += 32 * W) mt[i] = rng[i];
  for (int i = tid; i < nI; i += 32 * W) I[i] = Jg->F[i];
  for (int i = tid; i < nV; i += 32 * W) V[i] = Jg->V[i];
  for (int i = tid; i < g.z; i += 32 * W) ents[i] = Jg->entries[i];
  for (int i = tid; i <= g.nsh; i += 32 * W) sstart[i] = Jg->shell_start[i];
  halo_fill(g, H, Jg->lat, lat, tid, 32 * W);
  __syncthreads();
  Ring R;
  if (warp == 0) {
    ring_init(mt, tbuf, (int)rng[kMTN], lane, R);
  } else {
    R.idx = (int)rng[kMTN];
    R.avail = kMTN - R.idx;
    R.next_half = 1;
  }
  HaloPlan<NJ> P;
  make_halo_plan<NJ>(g, H, ents, lane, P);
  __syncthreads();

  const int lat_off = (int)L.lat;
  const int tb = (int)(L.tbuf / 4);
  const int I_off = (int)(L.I / 4);
  const int D_abs = I_off + L.D_off;
  const SpecLat hl = {g.sz, g.sy, H.origin, H.SZ, H.SY, lat_off};
  const bool bcc = g.lattice == kBcc;
  const int ys = g.ys;
  const int nbr_swap = Jg->nbr_swap;
  const int band = Jg->band;
  const float bql2 = Jg->beta_q_l2, bband = Jg->beta_band;
  const int64_t n_trials = Jg->n_trials;
  const int n_peek = nbr_swap ? 5 : 7;
  const int n_base = nbr_swap ? 4 : 6;
  // this warp's candidate (d, m)
  int my_d = 0, my_m = 0;
#pragma unroll
  for (int d = 0; d < NC; ++d)
#pragma unroll
    for (int m = 0; m <= d; ++m)
      if (spec_slot(d, m) == warp) {
        my_d = d;
        my_m = m;
      }
  // 32-bit tallies (fewer than 2^31 trials per launch)
  unsigned int b_eval = 0, b_acc = 0, b_exp = 0, b_exact = 0;
  unsigned int c_fp64 = 0, c_cr = 0;

  int t = 0;
  const int nt = (int)n_trials;
  while (t < nt) {
    const int nd = min(NC, nt - t);
    const int need = n_base * (nd - 1) + (nd - 1) + n_peek;
    if (R.avail < need) {
      if (warp == 0) ring_generate(mt, tbuf, R.next_half, lane);
      R.avail += kMTN;
      R.next_half ^= 1;
      __syncthreads();
    }
    // ---- evaluate this warp's candidate on the round's lattice -----------
    if (my_d < nd) {
      const int wb = tb + R.idx + n_base * my_d + my_m;
      SitePair p;
      draw_site(g, s_u32[wb], s_u32[wb + 1], s_u32[wb + 2], p.ax, p.ay, p.az);
      if (nbr_swap) draw_nbr(g, s_u32[wb + 3], p.ax, p.ay, p.az, p.bx, p.by, p.bz);
      else draw_site(g, s_u32[wb + 3], s_u32[wb + 4], s_u32[wb + 5], p.bx, p.by, p.bz);
      const int Ya = p.ay >> ys, Xa = p.ax >> 1, Yb = p.by >> ys, Xb = p.bx >> 1;
      const int pa = H.origin + p.az * H.SZ + Ya * H.SY + Xa;
      const int pb = H.origin + p.bz * H.SZ + Yb * H.SY + Xb;
      p.sa = s_i8[lat_off + pa];
      p.sb = s_i8[lat_off + pb];
      int words = n_base, accept = 1, flags = 0;
      if (p.sa != p.sb) {
        flags = 1;
        const bool near = pair_near(g, H, p.ax, p.ay, p.az, p.bx, p.by, p.bz);
        p.ai = p.az * g.sz + Ya * g.sy + Xa;
        p.bi = p.bz * g.sz + Yb * g.sy + Xb;
        int dE;
        if (!near) {
          const bool par_a = bcc ? (p.az & 1) : (p.ax & 1);
          const bool par_b = bcc ? (p.bz & 1) : (p.bx & 1);
          dE = halo_delta<NJ>(g, lat_off, D_abs, P, pa, pb, par_a, par_b, p.sa, p.sb, lane);
        } else {
          dE = spec_delta_general(Jg, (int)L.ents, I_off, L.F_off, hl, p.ax, p.ay, p.az, p.ai, p.bx, p.by,
                                  p.bz, p.bi, p.sa, p.sb, lane);
        }
        const uint32_t wu = s_u32[wb + n_base];
        accept = -1;
        if (dE < -band) {
          accept = 1;
        } else if (dE > band) {
          words = n_base + 1;
          accept = fast_exp2_decision(bql2, bband, dE, wu);
        }
        if (accept < 0) {
          flags |= 4;
          const int r = spec_exact_decision(Jg, hl, V, ents, sstart, p.ax, p.ay, p.az, p.ai, p.bx, p.by,
                                            p.bz, p.bi, p.sa, p.sb, lane, wu);
          accept = r & 1;
          words = (r & 2) ? n_base + 1 : n_base;
          flags |= (r & 4) ? 8 : 0;
          flags |= (r & 8) ? 16 : 0;
        }
        if (words > n_base) flags |= 2;
      }
      const bool changed = accept && p.sa != p.sb;
      SpecSlot& S = slots[warp];
      if (lane == 0)
        *reinterpret_cast<int4*>(&S) = make_int4(words | (accept << 4) | ((changed ? 1 : 0) << 5) | (flags << 8),
                                                 p.ax | (p.ay << 16), p.bx | (p.by << 16), p.az | (p.bz << 16));
      if (changed && lane < 16) {
        // the halo writes of the swap: lanes 8k..8k+7 take site k through
        // the 8 combinations of images per axis
        const bool b = lane >= 8;
        const int combo = lane & 7;
        int Z = b ? p.bz : p.az, Y = b ? Yb : Ya, X = b ? Xb : Xa;
        const int sp = b ? p.sa : p.sb;
        bool ok = true;
        if (combo & 1) {
          if (X < H.hx) X += H.NX;
          else if (X >= H.NX - H.hx) X -= H.NX;
          else ok = false;
        }
        if (combo & 2) {
          if (Y < H.hy) Y += H.NY;
          else if (Y >= H.NY - H.hy) Y -= H.NY;
          else ok = false;
        }
        if (combo & 4) {
          if (Z < H.hz) Z += H.NZ;
          else if (Z >= H.NZ - H.hz) Z -= H.NZ;
          else ok = false;
        }
        S.wr[lane] = ok ? (halo_index(H, Z, Y, X) | (sp << 24)) : -1;
      }
    }
    __syncthreads();
    // ---- resolve in order (every warp, same result) -------------------------
    // trial d takes candidate (d, m); it stands unless an accepted swap of an
    // earlier trial of the round is within range of one of its sites
    int done = 0, m = 0, words = 0;
    int k_sel[NC];
    int4 h_sel[NC];
    bool go = true;
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      k_sel[d] = -1;
      h_sel[d] = make_int4(0, 0, 0, 0);
      if (go && d < nd) {
        const int k = spec_slot(d, m);
        const int4 h = *reinterpret_cast<const int4*>(&slots[k]);
        bool conflict = false;
#pragma unroll
        for (int e = 0; e < d; ++e)
          if ((h_sel[e].x >> 5) & 1) conflict = conflict || spec_conflict(g, H, h_sel[e], h, lane);
        if (conflict) {
          go = false;
        } else {
          k_sel[d] = k;
          h_sel[d] = h;
          done = d + 1;
          const int w = h.x & 15;
          words += w;
          m += w - n_base;
          const int f = h.x;
          b_acc += (f >> 4) & 1;
          b_eval += (f >> 8) & 1;
          b_exp += (f >> 9) & 1;
          b_exact += (f >> 10) & 1;
          c_fp64 += (f >> 11) & 1;
          c_cr += (f >> 12) & 1;
        }
      }
    }
    // ---- write the resolved swaps (disjoint sites), one warp each ----------
    int kw = -1, hw = 0;
#pragma unroll
    for (int d = 0; d < NC; ++d) {
      kw = warp == d ? k_sel[d] : kw;
      hw = warp == d ? h_sel[d].x : hw;
    }
    if (kw >= 0 && ((hw >> 5) & 1) && lane < 16) {
      const int v = slots[kw].wr[lane];
      if (v >= 0) lat[v & 0xFFFFFF] = (int8_t)(v >> 24);
    }
    __syncthreads();
    ring_consume(R, words);
    t += done;
  }

  const unsigned long long c_eval = b_eval, c_acc = b_acc, c_exp = b_exp, c_exact = b_exact;
  const unsigned long long c_draws = (unsigned long long)n_base * (unsigned long long)n_trials + c_exp;

  // ---- write back ---------------------------------------------------------
  halo_store(g, H, lat, Jg->lat, tid, 32 * W);
  if (warp == 0) ring_writeback(mt, tbuf, R, Jg->rng, lane);
  if (tid == 0) {
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

uint32_t spec_static_smem(int nc) { return (uint32_t)(nc * (nc + 1) / 2) * sizeof(SpecSlot) + 64; }

template <int NJ, int NC>
static void launch_spec(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, cudaStream_t stream) {
  cudaFuncSetAttribute(metropolis_spec_kernel<NJ, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes);
  BRAWL_CARVEOUT(metropolis_spec_kernel<NJ, NC>);
  metropolis_spec_kernel<NJ, NC><<<n_jobs, 32 * (NC * (NC + 1) / 2), smem_bytes, stream>>>(d_jobs);
}

template <int NC>
static void launch_spec_nc(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int max_z,
                           cudaStream_t stream) {
  switch (lane_entries_for(max_z)) {
    case 2: launch_spec<2, NC>(d_jobs, n_jobs, smem_bytes, stream); break;
    case 4: launch_spec<4, NC>(d_jobs, n_jobs, smem_bytes, stream); break;
    case 6: launch_spec<6, NC>(d_jobs, n_jobs, smem_bytes, stream); break;
    case 8: launch_spec<8, NC>(d_jobs, n_jobs, smem_bytes, stream); break;
    default: launch_spec<11, NC>(d_jobs, n_jobs, smem_bytes, stream); break;
  }
}

void launch_halo_chains(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int min_z, int max_z,
                        int nc, int max_optin, cudaStream_t stream) {
  if (nc >= 2 && smem_bytes + spec_static_smem(nc) <= (uint32_t)max_optin)
    launch_metropolis_spec(d_jobs, n_jobs, smem_bytes, max_z, nc, stream);
  else
    launch_metropolis_halo(d_jobs, n_jobs, smem_bytes, min_z, max_z, stream);
}

void launch_metropolis_spec(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int max_z, int nc,
                            cudaStream_t stream) {
  if (n_jobs <= 0) return;
  switch (nc) {
    case 2: launch_spec_nc<2>(d_jobs, n_jobs, smem_bytes, max_z, stream); break;
    case 3: launch_spec_nc<3>(d_jobs, n_jobs, smem_bytes, max_z, stream); break;
    default: launch_spec_nc<4>(d_jobs, n_jobs, smem_bytes, max_z, stream); break;
  }
}

}  // namespace brawl
