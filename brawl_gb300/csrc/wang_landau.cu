// wang_landau.cu -- Wang-Landau walker updates on the device
// (src/wang-landau.F90:515-632): sweeps() for every walker of a batch, then
// the in-window average of ln g and of the histogram that the reference
// does with MPI_Allreduce over the walkers of a window followed by a
// division by their number.
//
// One warp per walker.  Each trial's bins depend on the walker's running
// FP64 energy (e_swapped = e_unswapped - pair_unswapped + pair_swapped, the
// pair energies summed in the reference's order).  The kernel carries an
// interval that contains it: a trial's bin comes from the fixed-point delta
// when the interval lies in one bin, and accepted moves are logged and
// their FP64 sums run together later (lazy_exact.cuh); a bin the interval
// does not settle flushes the log and takes the exact sums.  The acceptance
// test log(genrand()) < lng(i) - lng(j) is decided in FP32 first
// (exact_fp.cuh).  The window's ln g and histogram slices are staged in
// shared memory.
#include "halo_engine.cuh"
#include "kernels.cuh"
#include "lazy_exact.cuh"
#include "wl_kernels.cuh"

namespace brawl {

// bin_index (src/wang-landau.F90:515-523): int() truncates toward zero.
// Values far outside the bin range (where int() would overflow) map to a
// bin that is in no window.
__device__ __forceinline__ int wl_bin_index(double E, double e1, double range, int bins) {
  const double t = __dmul_rn(__ddiv_rn(__dsub_rn(E, e1), range), (double)bins);
  if (!(t > -1.0e9 && t < 1.0e9)) return t < 0.0 ? -1000000000 : 1000000000;
  return (int)t + 1;
}

// The same bin, without the FP64 division when it cannot matter: with
// rf = float(bins / range), tf = float(E - e1) * rf is within
// |t| * 1.9e-7 of the reference's t (three single roundings and two
// double ones), so when tf -/+ that margin truncate to the same integer,
// so does t.  Otherwise (near a bin edge, far outside, NaN) the reference
// expression decides.
__device__ __forceinline__ int wl_bin_index_fast(double E, double e1, double range, int bins, float rf) {
  const double d = __dsub_rn(E, e1);
  const float tf = __fmul_rn(__double2float_rn(d), rf);
  const float M = fabsf(tf) * 2.5e-7f + 1.0e-30f;
  if (fabsf(tf) < 5.0e8f) {
    // rounded outwards, so [lo, hi] contains the exact interval
    const float lo = truncf(__fsub_rd(tf, M)), hi = truncf(__fadd_ru(tf, M));
    if (lo == hi) return (int)lo + 1;
  }
  return wl_bin_index(E, e1, range, bins);
}

// e_swapped as the reference forms it: e_unswapped - pair_unswapped +
// pair_swapped with the pair energies summed in its order.  Out of line: it
// runs only for accepted moves and for the rare undecided bins.
__device__ __noinline__ double wl_exact_e_sw(const Geom& g, const int8_t* lat, const double* V, const uint32_t* ents,
                                             const int16_t* sstart, const SitePair& p, int lane, double e_un,
                                             double* vbuf) {
  double p_un, p_sw;
  exact_pair_energies_staged(g, CompactLat{lat}, V, ents, sstart, p, lane, p_un, p_sw, vbuf);
  return __dadd_rn(__dsub_rn(e_un, p_un), p_sw);
}

// radial_densities (src/analytics.f90:293-404) of the staged lattice, added
// to rho_of_E(:, :, :, bin): the (species, species, shell class) pair counts
// through the ASRO plan (asro.cuh) in shared memory, then rho(i, j, l) =
// count / particle_counts(i) per element, each added to its own FP64 sum.
// Out of line: a sample is taken at most once every n_atoms trials.
__device__ __noinline__ void wl_radial_sample(const Geom& g, const int8_t* lat, const uint32_t* offs,
                                              const unsigned long long* masks, unsigned int* hist,
                                              int n_off, int n_class, int wc, double* rho_bin,
                                              int lane) {
  const int nsp = g.ns + 1;
  const int nh = nsp * nsp * n_class;
  unsigned int* pcs = hist + nh;
  for (int i = lane; i < nh + nsp; i += 32) hist[i] = 0u;
  __syncwarp();
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3;
  for (int site = lane; site < g.n_sites; site += 32) {
    int x, y, z;
    decode_site(g, site, x, y, z);
    const int si = lat[site];
    atomicAdd(&pcs[si], 1u);
    const int row = si * nsp;
    for (int o = 0; o < n_off; ++o) {
      int dx, dy, dz, cls;
      unpack_entry(offs[o], dx, dy, dz, cls);
      const int sj = lat[compact_index(g, wrap_general(x, dx, W1), wrap_general(y, dy, W2),
                                       wrap_general(z, dz, W3))];
      atomicAdd(&hist[(row + sj) * n_class + cls], 1u);
    }
  }
  __syncwarp();
  const int ns = g.ns, per = ns * ns * wc;
  for (int k = lane; k < per; k += 32) {
    const int i = k % ns + 1, j = (k / ns) % ns + 1, l = k / (ns * ns);
    unsigned int c = 0;
    for (int cl = 0; cl < n_class; ++cl)
      if ((masks[cl] >> l) & 1ull) c += hist[(i * nsp + j) * n_class + cl];
    rho_bin[k] = __dadd_rn(rho_bin[k], __ddiv_rn((double)c, (double)pcs[i]));
  }
  __syncwarp();
}

// config_per_bin(jbin, ...) = config: the warp copies the compact lattice
// to the bin's store slot, in words when the size and the slot allow.  Out
// of line: a bin is stored once.
__device__ __noinline__ void wl_store_config(const Geom& g, const int8_t* lat, int8_t* dst, int lane) {
  const int n = g.n_sites;
  if ((n & 3) == 0 && (reinterpret_cast<uintptr_t>(dst) & 3) == 0) {
    const uint32_t* s = reinterpret_cast<const uint32_t*>(lat);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (int i = lane; i < (n >> 2); i += 32) d[i] = s[i];
  } else {
    for (int i = lane; i < n; i += 32) dst[i] = lat[i];
  }
}

// Warps per walker: warp 0 walks; the others join only the deferred-energy
// flushes (each sub-partition of an SM has its own FP64 pipe).
constexpr int kWlWarps = 4;

template <int NJ, bool kUseD>
__global__ void __launch_bounds__(32 * kWlWarps, 1) wl_sweep_kernel(WlWalker* __restrict__ walkers) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_ctl[2];  // the flushes' command and move count (lazy_flush_block)
  WlWalker& W = walkers[blockIdx.x];
  const ChainJob& J = W.job;
  const Geom g = J.g;
  const int lane = threadIdx.x & 31;
  const int nthreads = blockDim.x;
  const unsigned long long t_start = global_ns();
  const int nV = g.ns * g.ns * g.nsh;
  const int nb = W.end - W.start + 1;
  const bool rad_on = W.radial_record != nullptr;
  const WalkerLayout WLy = walker_layout(g, nb, W.lazy_cap, rad_on ? W.bins : 0, W.rad_n_offsets,
                                         W.rad_n_class);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + WLy.mt);
  uint32_t* tbuf = reinterpret_cast<uint32_t*>(smem + WLy.tbuf);
  double* V = reinterpret_cast<double*>(smem + WLy.V);
  int32_t* I = reinterpret_cast<int32_t*>(smem + WLy.I);
  int32_t* F = I + WLy.F_off;
  double* lng = reinterpret_cast<double*>(smem + WLy.slices);
  double* hist = lng + nb;
  uint8_t* sopen = smem + WLy.sopen;  // the window's open store flags
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + WLy.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + WLy.sstart);
  int8_t* lat = reinterpret_cast<int8_t*>(smem + WLy.lat);
  double* vbuf = reinterpret_cast<double*>(smem + WLy.vbuf);
  const LazyLog LG = lazy_layout(g, smem + WLy.lazy, W.lazy_cap);
  if (threadIdx.x >= 32) {
    // a helper warp: flushes only, until warp 0 releases it
    lazy_helper_loop(g, V, sstart, LG, kFoldWangLandau, threadIdx.x, nthreads, s_ctl);
    return;
  }
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nV; i += 32) V[i] = J.V[i];
  for (int i = lane; i < WLy.nI - WLy.F_off; i += 32) F[i] = J.F[i];
  for (int i = lane; i < nb; i += 32) {
    lng[i] = W.lng[W.start - 1 + i];
    hist[i] = W.hist[i];
    sopen[i] = W.store ? W.store_open[W.start - 1 + i] : (uint8_t)0;
  }
  for (int i = lane; i < g.z; i += 32) ents[i] = J.entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = J.shell_start[i];
  for (int i = lane; i < g.n_sites; i += 32) lat[i] = J.lat[i];
  // radial samples: a bin is eligible while radial_record < cap and
  // radial_record_bool is unset
  uint32_t* elig = reinterpret_cast<uint32_t*>(smem + WLy.rad);
  uint32_t* r_offs = reinterpret_cast<uint32_t*>(smem + WLy.rad_offsets);
  unsigned long long* r_masks = reinterpret_cast<unsigned long long*>(smem + WLy.rad_masks);
  unsigned int* r_hist = reinterpret_cast<unsigned int*>(smem + WLy.rad_hist);
  int rsteps = 0, r_cap = 0, r_wc = 0;
  if (rad_on) {
    const WlRadial RP = *W.radial;
    r_cap = RP.cap;
    r_wc = RP.wc_range;
    rsteps = *W.radial_steps;
    for (int w = lane; w < (W.bins + 31) / 32; w += 32) {
      uint32_t bits = 0u;
      for (int b = 0; b < 32 && 32 * w + b < W.bins; ++b) {
        const int k = 32 * w + b;
        if (W.radial_record[k] < RP.cap && !RP.done[k]) bits |= 1u << b;
      }
      elig[w] = bits;
    }
    for (int i = lane; i < RP.n_offsets; i += 32) r_offs[i] = RP.offsets[i];
    for (int i = lane; i < RP.n_class; i += 32) r_masks[i] = RP.class_masks[i];
  }
  AxisTables T;
  build_axis_tables(g, I, WLy.tab_len, lane, T);
  __syncwarp();
  LanePlan<NJ> P;
  make_lane_plan<NJ>(g, ents, I, T, lane, P);
  const int lat_off = (int)WLy.lat, I_off = (int)(WLy.I / 4);
  const int log_off = (int)(LG.codes - smem);
  // an entry can map a site onto itself only when a wrap period is within
  // the offsets' reach
  const bool self_map = g.W1 <= kHalo || g.W2 <= kHalo || g.W3 <= kHalo;
  Ring ring;
  ring_init(mt, tbuf, (int)J.rng[kMTN], lane, ring);

  const double e1 = W.e1, range = W.range, f = W.wl_f;
  const int bins = W.bins, start = W.start, end = W.end;
  const double rbins = __ddiv_rn((double)bins, range);
  const float rf = __double2float_rn(rbins);
  const int period = W.hist_period;
  const int band = J.band;
  const double q = ldexp(1.0, -W.S);               // one fixed-point quantum
  // e_ex: the reference's e_unswapped before the n_log logged moves; after
  // them it lies in e_ex + [Dlo - Rs, Dhi + Rs] quanta (Rs: the roundings of
  // the logged updates), and bins follow from float offsets of t0, the bin
  // coordinate of e_ex, taken once per exact energy
  double e_ex = (W.i0 > 0 && W.e_state) ? *W.e_state : (W.e0_src ? *W.e0_src : W.e0);
  const float qrf = __double2float_rn(__dmul_rn(q, rbins));
  long long Dlo = 0, Dhi = 0, Rs = 0, Eq = 0;
  float t0 = 0.0f;
  auto rebase = [&]() {
    Eq = quanta_bound(e_ex, W.S);
    t0 = __double2float_rn(__dmul_rn(__dsub_rn(e_ex, e1), rbins));
    Dlo = Dhi = Rs = 0;
  };
  rebase();
  int n_log = 0;
  int ibin = wl_bin_index(e_ex, e1, range, bins);
  int status = (ibin < start || ibin > end) ? kStatusWalkerOutsideWindow : kStatusOk;
  unsigned int c_eval = 0, c_exp = 0, c_exact = 0, n_acc = 0;
  DecideStats st = {0u, 0u};
  // histogram ticks at trials i with i % period == 0
  long long until = period > 0 ? period - (W.i0 % period) : -1;
  // folds the logged moves into e_ex; their energy must be in the interval
  auto flush = [&]() {
    if (n_log == 0) return;
    const double e0 = e_ex;
    e_ex = lazy_flush_block(g, V, sstart, LG, n_log, e_ex, kFoldWangLandau, lane, nthreads, s_ctl);
    if (!in_quanta(e_ex, e0, Dlo - Rs, Dhi + Rs, q)) status = kStatusBandViolated;
    n_log = 0;
    rebase();
  };

  const int n_tr = (int)W.n_trials;
  // select_sites or select_sites_nbr (src/wang-landau.F90:1527-1539)
  const bool nbr = J.nbr_swap != 0;
  const int n_base = nbr ? 4 : 6;
  for (int it = 0; it < n_tr && status == kStatusOk; ++it) {
    ring_ensure(mt, tbuf, ring, n_base + 1, lane);
    const int wb = ring.idx;
    SitePair p;
    draw_site(g, tbuf[wb], tbuf[wb + 1], tbuf[wb + 2], p.ax, p.ay, p.az);
    if (nbr) draw_nbr(g, tbuf[wb + 3], p.ax, p.ay, p.az, p.bx, p.by, p.bz);
    else draw_site(g, tbuf[wb + 3], tbuf[wb + 4], tbuf[wb + 5], p.bx, p.by, p.bz);
    p.ai = compact_index(g, p.ax, p.ay, p.az);
    p.bi = compact_index(g, p.bx, p.by, p.bz);
    p.sa = lat[p.ai];
    p.sb = lat[p.bi];
    const bool differ = p.sa != p.sb;
    int jbin = ibin;
    bool exact_done = false;
    double e_sw = e_ex;
    long long r1 = 0;
    int dE = 0;
    uint8_t* rec = LG.codes + (size_t)n_log * 2 * g.z;
    if (differ) {
      ++c_eval;
      // The reference's e_swapped = (e_un - p_un) + p_sw lies within band
      // quanta of e_un + dE q plus the two roundings, each at most 2^-53 of
      // |e_un - p_un| <= |e_un| + 2^30 q or of |e_swapped|; its bin is
      // decided without the FP64 sums when that interval sits in one bin.
      bool near;
      dE = fixed_delta_rec<NJ, kUseD>(g, lat_off, I_off, WLy.F_off, WLy.D_off, P, p, lane,
                                      log_off + n_log * 2 * g.z, near);
      if (near || self_map) dE = compact_fixed_delta_rec(g, lat, F, ents, p, lane, rec);
      bool settled = false;
      for (int pass = 0; pass < 2 && !settled; ++pass) {
        const long long B = 2 * (Eq + max(llabs(Dlo), llabs(Dhi)) + Rs) + (1ll << 30) +
                            llabs((long long)dE) + band;
        r1 = Rs + (B >> 53) + 1;
        settled = bin_from_quanta(t0, qrf, Dlo + dE - band - r1, Dhi + dE + band + r1, jbin);
        if (!settled && pass == 0 && n_log > 0) {
          // the logged moves' exact energy may settle it; this move's codes
          // move to the log's first slot
          flush();
          lazy_copy_slot(g, rec, LG.codes, lane);
          rec = LG.codes;
        } else if (!settled) {
          break;
        }
      }
      if (!settled) {
        ++c_exact;
        exact_done = true;
        e_sw = wl_exact_e_sw(g, lat, V, ents, sstart, p, lane, e_ex, vbuf);
        jbin = wl_bin_index_fast(e_sw, e1, range, bins, rf);
      }
    }
    // a radial sample of the trial configuration (the swap applied), before
    // the decision, as the reference takes it
    bool swapped = false;
    if (rad_on && jbin >= 1 && jbin <= bins && ((elig[(jbin - 1) >> 5] >> ((jbin - 1) & 31)) & 1u)) {
      if (++rsteps >= g.n_sites) {
        rsteps = 0;
        if (differ && lane == 0) {
          lat[p.ai] = (int8_t)p.sb;
          lat[p.bi] = (int8_t)p.sa;
        }
        swapped = differ;
        __syncwarp();
        wl_radial_sample(g, lat, r_offs, r_masks, r_hist, W.rad_n_offsets, W.rad_n_class, r_wc,
                         W.rho_of_E + (size_t)(jbin - 1) * g.ns * g.ns * r_wc, lane);
        if (lane == 0) {
          const int rec = W.radial_record[jbin - 1] + 1;
          W.radial_record[jbin - 1] = rec;
          if (rec >= r_cap) elig[(jbin - 1) >> 5] &= ~(1u << ((jbin - 1) & 31));
        }
        __syncwarp();
      }
    }
    int consumed = n_base;
    if (jbin >= start && jbin <= end) {
      consumed = n_base + 1;
      ++c_exp;
      const uint32_t wu = tbuf[wb + n_base];
      const double d = __dsub_rn(lng[ibin - start], lng[jbin - start]);
      if (log_u_lt(wu, d, st)) {
        ++n_acc;
        if (differ) {
          if (exact_done) {
            e_ex = e_sw;  // the log is empty here
            rebase();
          } else {
            // logged: the energy after it is in e_ex + [Dlo - Rs, Dhi + Rs]
            if (lane == 0) {
              LG.spec[2 * n_log] = (int8_t)p.sa;
              LG.spec[2 * n_log + 1] = (int8_t)p.sb;
            }
            ++n_log;
            Dlo += (long long)dE - band;
            Dhi += (long long)dE + band;
            Rs = r1;
          }
          if (lane == 0) {
            lat[p.ai] = (int8_t)p.sb;
            lat[p.bi] = (int8_t)p.sa;
          }
        }
        ibin = jbin;
      } else {
        jbin = ibin;
        if (swapped && lane == 0) {  // the sampled swap undone
          lat[p.ai] = (int8_t)p.sa;
          lat[p.bi] = (int8_t)p.sb;
        }
      }
    } else {
      jbin = ibin;
      if (swapped && lane == 0) {
        lat[p.ai] = (int8_t)p.sa;
        lat[p.bi] = (int8_t)p.sb;
      }
    }
    if (--until == 0) {
      if (lane == 0) hist[jbin - start] = __dadd_rn(hist[jbin - start], 1.0);
      // config_per_bin(jbin) = config the first time the bin is sampled
      // (src/wang-landau.F90:605-610); the flag reads alike in every lane
      if (sopen[jbin - start]) {
        __syncwarp();
        wl_store_config(g, lat, W.store + (size_t)(jbin - 1) * (size_t)g.n_sites, lane);
        __syncwarp();
        if (lane == 0) sopen[jbin - start] = 0;
      }
      until = period;
    }
    if (lane == 0) lng[jbin - start] = __dadd_rn(lng[jbin - start], f);
    __syncwarp();
    if (n_log == LG.cap) flush();
    ring_consume(ring, consumed);
  }
  flush();
  lazy_helpers_release(lane, nthreads, s_ctl);
  const double e_un = e_ex;

  __syncwarp();
  for (int i = lane; i < nb; i += 32) {
    W.lng[W.start - 1 + i] = lng[i];
    W.hist[i] = hist[i];
    if (W.store) W.store_open[W.start - 1 + i] = sopen[i];
  }
  for (int i = lane; i < g.n_sites; i += 32) J.lat[i] = lat[i];
  ring_writeback(mt, tbuf, ring, J.rng, lane);
  if (lane == 0) {
    W.e_out = e_un;
    if (W.e_state) *W.e_state = e_un;
    if (rad_on) *W.radial_steps = rsteps;
    W.accepted = n_acc;
    unsigned long long* c = J.counters;
    c[kCntTrials] += (unsigned long long)W.n_trials;
    c[kCntEvaluated] += c_eval;
    c[kCntDraws] += (unsigned long long)n_base * (unsigned long long)W.n_trials + c_exp;
    c[kCntAccepted] += n_acc;
    c[kCntExpTests] += c_exp;
    c[kCntExactPath] += c_exact;
    c[kCntExpFp64] += st.fp64;
    c[kCntExpCr] += st.cr;
    if (status != kStatusOk) *J.status = status;
    if (J.t_ns) *J.t_ns = global_ns() - t_start;
  }
}

// full_energy (src/bw_hamiltonian.f90:58-81) of the staged lattice: the
// site energies in the reference's order, one lane per site, then their sum
// in site order on one lane and the half.  Returned in every lane.
__device__ double full_energy_warp(const Geom& g, const int8_t* lat, const double* V,
                                   const uint32_t* ents, const int16_t* sstart, double* site_e,
                                   int lane) {
  for (int i = lane; i < g.n_sites; i += 32) {
    int x, y, z;
    decode_site(g, i, x, y, z);
    site_e[i] = site_energy_ref(g, lat, V, ents, sstart, x, y, z);
  }
  __syncwarp();
  double e = 0.0;
  if (lane == 0) {
    for (int i = 0; i < g.n_sites; ++i) e = __dadd_rn(e, site_e[i]);
    e = __dmul_rn(0.5, e);
  }
  e = __shfl_sync(kFull, e, 0);
  __syncwarp();
  return e;
}

// enter_energy_window (src/wang-landau.F90:643-741), one warp per walker:
// the walk biased towards the middle of the window, log(u) < -delta_e with
// delta_e = ((e_sw - target)^2 - (e_un - target)^2) / sig2x2 decided from
// the reference-order pair energies, until full_energy lies inside the
// window's inner 80%; every n_atoms*250 steps initial_setup draws the
// configuration again (the running energy left as it is, as the reference
// leaves it).  Bounded by max_steps.
__global__ void __launch_bounds__(32, 1) wl_enter_kernel(WlEnterJob* __restrict__ jobs) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int64_t check[kMaxSpecies];
  WlEnterJob& E = jobs[blockIdx.x];
  const ChainJob& J = E.job;
  const Geom g = J.g;
  const int lane = threadIdx.x;
  const int nV = g.ns * g.ns * g.nsh;
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem);
  double* V = reinterpret_cast<double*>(smem + align_up(kMTN * 4, 16));
  uint32_t* ents = reinterpret_cast<uint32_t*>(V + nV);
  int16_t* sstart = reinterpret_cast<int16_t*>(ents + g.z);
  int8_t* lat = reinterpret_cast<int8_t*>(
      smem + align_up((uint32_t)(reinterpret_cast<unsigned char*>(sstart + g.nsh + 1) - smem), 16));
  double* vbuf = reinterpret_cast<double*>(
      smem + align_up((uint32_t)(reinterpret_cast<unsigned char*>(lat + g.n_sites) - smem), 16));
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nV; i += 32) V[i] = J.V[i];
  for (int i = lane; i < g.z; i += 32) ents[i] = J.entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = J.shell_start[i];
  for (int i = lane; i < g.n_sites; i += 32) lat[i] = J.lat[i];
  int pos = (int)J.rng[kMTN];
  __syncwarp();
  unsigned long long draws = 0;
  int status = kStatusOk;
  if (E.initial && !initial_setup_warp(E.init, lat, mt, pos, check, draws, lane)) status = kStatusBadSpecies;
  const double lo = E.min_e, hi = E.max_e;
  const double target = __ddiv_rn(__dadd_rn(lo, hi), 2.0);
  const double cond = __dmul_rn(fabs(__dsub_rn(hi, lo)), 0.1);
  const double in_hi = __dsub_rn(hi, cond), in_lo = __dadd_rn(lo, cond);
  const int64_t reinit = (int64_t)g.n_sites * 250;
  double e_un = status == kStatusOk ? full_energy_warp(g, lat, V, ents, sstart, E.site_e, lane) : 0.0;
  int64_t steps = -1, i_steps = 0;
  DecideStats st = {0u, 0u};
  for (int64_t it = 1; it <= E.max_steps && status == kStatusOk; ++it) {
    if (++i_steps % reinit == 0) {
      i_steps = 0;
      if (!initial_setup_warp(E.init, lat, mt, pos, check, draws, lane)) {
        status = kStatusBadSpecies;
        break;
      }
    }
    if (e_un < in_hi && e_un > in_lo) {
      e_un = full_energy_warp(g, lat, V, ents, sstart, E.site_e, lane);
      if (e_un < in_hi && e_un > in_lo) {
        steps = it;
        break;
      }
      continue;
    }
    const uint32_t w = mt_peek(mt, pos, 6, lane);
    SitePair p;
    draw_site(g, __shfl_sync(kFull, w, 0), __shfl_sync(kFull, w, 1), __shfl_sync(kFull, w, 2), p.ax,
              p.ay, p.az);
    draw_site(g, __shfl_sync(kFull, w, 3), __shfl_sync(kFull, w, 4), __shfl_sync(kFull, w, 5), p.bx,
              p.by, p.bz);
    pos += 6;
    p.ai = compact_index(g, p.ax, p.ay, p.az);
    p.bi = compact_index(g, p.bx, p.by, p.bz);
    p.sa = lat[p.ai];
    p.sb = lat[p.bi];
    if (p.sa != p.sb) {
      double p_un, p_sw;
      exact_pair_energies_staged(g, CompactLat{lat}, V, ents, sstart, p, lane, p_un, p_sw, vbuf);
      const double e_sw = __dadd_rn(__dsub_rn(e_un, p_un), p_sw);
      const double a = __dsub_rn(e_sw, target), b = __dsub_rn(e_un, target);
      const double d = __ddiv_rn(__dsub_rn(__dmul_rn(a, a), __dmul_rn(b, b)), E.sig2x2);
      const uint32_t wu = __shfl_sync(kFull, mt_peek(mt, pos, 1, lane), 0);
      pos += 1;
      if (log_u_lt(wu, -d, st)) {
        e_un = e_sw;
        if (lane == 0) {
          lat[p.ai] = (int8_t)p.sb;
          lat[p.bi] = (int8_t)p.sa;
        }
      }
      __syncwarp();
    }
  }
  __syncwarp();
  for (int i = lane; i < g.n_sites; i += 32) J.lat[i] = lat[i];
  for (int i = lane; i < kMTN; i += 32) J.rng[i] = mt[i];
  if (lane == 0) {
    J.rng[kMTN] = (uint32_t)(pos < 0 ? 0 : pos);
    E.steps = steps;
    E.energy = e_un;
    if (status != kStatusOk) *J.status = status;
  }
}

uint32_t wl_enter_smem_bytes(const Geom& g) {
  uint32_t b = align_up(kMTN * 4, 16) + (uint32_t)(g.ns * g.ns * g.nsh) * 8 + (uint32_t)g.z * 4 +
               (uint32_t)(g.nsh + 1) * 2;
  b = align_up(b, 16) + (uint32_t)g.n_sites;
  b = align_up(b, 16) + 4u * (uint32_t)g.z * 8;
  return align_up(b, 16);
}

void launch_wl_enter(WlEnterJob* d_jobs, int n, uint32_t smem, cudaStream_t stream) {
  cudaFuncSetAttribute(wl_enter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  BRAWL_CARVEOUT(wl_enter_kernel);
  if (n > 0) wl_enter_kernel<<<n, 32, smem, stream>>>(d_jobs);
}

// The window average: for every bin, the walkers' values summed in walker
// order and divided by their count (MPI_Allreduce SUM then /num_walkers,
// src/wang-landau.F90:628-631; dos_average, :1127-1133, averages ln g
// alone).  groups[k] lists the walkers of window k.
__global__ void wl_average_kernel(const WlGroup* __restrict__ groups, WlWalker* walkers,
                                  int bins, int with_hist) {
  const WlGroup G = groups[blockIdx.y];
  if (G.count <= 1) return;
  const double inv = (double)(float)G.count;
  const int nbins = walkers[G.first].bins;  // the bins argument (the largest) sizes the grid
  (void)bins;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
    double s = walkers[G.first].lng[b];
    for (int k = 1; k < G.count; ++k) s = __dadd_rn(s, walkers[G.first + k].lng[b]);
    const double a = __ddiv_rn(s, inv);
    for (int k = 0; k < G.count; ++k) walkers[G.first + k].lng[b] = a;
  }
  if (!with_hist) return;
  const int nb = walkers[G.first].end - walkers[G.first].start + 1;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    double s = walkers[G.first].hist[b];
    for (int k = 1; k < G.count; ++k) s = __dadd_rn(s, walkers[G.first + k].hist[b]);
    const double a = __ddiv_rn(s, inv);
    for (int k = 0; k < G.count; ++k) walkers[G.first + k].hist[b] = a;
  }
}

uint32_t wl_smem_bytes(const Geom& g, int nb, int lazy_cap, int rad_bins, int rad_n_offsets,
                       int rad_n_class) {
  return walker_layout(g, nb, lazy_cap, rad_bins, rad_n_offsets, rad_n_class).total;
}

template <int NJ, bool kUseD>
static void launch_wl_nj(WlWalker* d_walkers, int n, uint32_t smem, cudaStream_t stream) {
  cudaFuncSetAttribute(wl_sweep_kernel<NJ, kUseD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  BRAWL_CARVEOUT(wl_sweep_kernel<NJ, kUseD>);
  wl_sweep_kernel<NJ, kUseD><<<n, 32 * kWlWarps, smem, stream>>>(d_walkers);
}

template <bool kUseD>
static void launch_wl_d(WlWalker* d_walkers, int n, uint32_t smem, int max_z, cudaStream_t stream) {
  switch (lane_entries_for(max_z)) {
    case 2: launch_wl_nj<2, kUseD>(d_walkers, n, smem, stream); break;
    case 4: launch_wl_nj<4, kUseD>(d_walkers, n, smem, stream); break;
    case 6: launch_wl_nj<6, kUseD>(d_walkers, n, smem, stream); break;
    case 8: launch_wl_nj<8, kUseD>(d_walkers, n, smem, stream); break;
    default: launch_wl_nj<11, kUseD>(d_walkers, n, smem, stream); break;
  }
}

void launch_wl_sweeps(WlWalker* d_walkers, int n, uint32_t smem, int max_z, bool all_D,
                      cudaStream_t stream) {
  if (n <= 0) return;
  if (all_D) launch_wl_d<true>(d_walkers, n, smem, max_z, stream);
  else launch_wl_d<false>(d_walkers, n, smem, max_z, stream);
}

void launch_wl_average(const WlGroup* d_groups, int n_groups, WlWalker* d_walkers, int bins,
                       int with_hist, cudaStream_t stream) {
  if (n_groups <= 0) return;
  dim3 grid((bins + 255) / 256, n_groups);
  BRAWL_CARVEOUT(wl_average_kernel);
  wl_average_kernel<<<grid, 256, 0, stream>>>(d_groups, d_walkers, bins, with_hist);
}

// ---------------------------------------------------------------------------
// replica_exchange (src/wang-landau.F90:1392-1501) for walkers ordered by
// window, per_window each (walker w plays MPI rank w).  One warp: the bins
// and overlaps of every walker in parallel, then the reference's sequence --
// per adjacent pair of windows both candidate lists shuffled on walker 0's
// stream (shuffle_rows, :1513-1525), equal overlaps matched in list order,
// and every matched lower walker drawing genrand() < exp(lng(i) - lng(j))
// from its own stream, the pair's configurations swapped on acceptance.
// A stream is staged in shared memory (624 words + position, the layout the
// chains keep in global memory) while it is drawn from.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ void stream_load(uint32_t* s, const uint32_t* g, int lane) {
  for (int i = lane; i <= kMTN; i += 32) s[i] = g[i];
  __syncwarp();
}

__device__ __forceinline__ void stream_store(uint32_t* g, const uint32_t* s, int lane) {
  __syncwarp();
  for (int i = lane; i <= kMTN; i += 32) g[i] = s[i];
  __syncwarp();
}

// genrand_int32 on a staged stream; warp-collective, every lane gets the word.
__device__ __forceinline__ uint32_t stream_draw(uint32_t* s, int lane) {
  int pos = (int)s[kMTN];
  if (pos >= kMTN) {
    mt_twist_warp(s, lane);
    pos = 0;
  }
  const uint32_t w = mt_temper(s[pos]);
  __syncwarp();
  if (lane == 0) s[kMTN] = (uint32_t)(pos + 1);
  __syncwarp();
  return w;
}

// shuffle_rows: rows r = n..2 swap with MIN(1+int(genrand()*r), n);
// int(u*r) = floor(w*r / 2^32) exactly for r < 2^21.
__device__ void shuffle_rows(int2* rows, int n, uint32_t* s, int lane) {
  for (int r = n; r >= 2; --r) {
    const uint32_t w = stream_draw(s, lane);
    int k = 1 + (int)__umulhi(w, (uint32_t)r);
    k = k > n ? n : k;
    if (lane == 0) {
      const int2 t = rows[r - 1];
      rows[r - 1] = rows[k - 1];
      rows[k - 1] = t;
    }
    __syncwarp();
  }
}

}  // namespace

__global__ void __launch_bounds__(32) wl_exchange_kernel(WlWalker* __restrict__ W,
                                                         const double* __restrict__ energy,
                                                         const WlGroup* __restrict__ groups,
                                                         int n_windows, int per_window,
                                                         int* __restrict__ ibin,
                                                         int2* __restrict__ ov,
                                                         int* __restrict__ partner,
                                                         int* __restrict__ exchanged,
                                                         int* __restrict__ n_accepted) {
  extern __shared__ __align__(16) uint32_t sm[];
  uint32_t* st0 = sm;                        // walker 0's stream
  uint32_t* st1 = sm + 640;                  // a matched walker's stream
  int2* lo = reinterpret_cast<int2*>(sm + 1280);
  int2* up = lo + per_window;
  int2* pairs = up + per_window;
  int* s_np = reinterpret_cast<int*>(pairs + per_window);
  const int lane = threadIdx.x;
  const int n = n_windows * per_window;
  const double e1 = W[0].e1, range = W[0].range;
  const int bins = W[0].bins;

  for (int w = lane; w < n; w += 32) {
    const int idx = w / per_window + 1;
    const int ib = wl_bin_index(energy[w], e1, range, bins);
    bool lower = false, upper = false;
    if (idx > 1)
      lower = ib < W[groups[idx - 2].first].end + 1 && ib > W[groups[idx - 1].first].start - 1;
    if (idx < n_windows)
      upper = ib > W[groups[idx].first].start - 1 && ib < W[groups[idx - 1].first].end + 1;
    ibin[w] = ib;
    ov[w] = make_int2(w, upper ? idx : (lower ? idx - 1 : 0));
    partner[w] = -1;
    exchanged[w] = 0;
  }
  __syncwarp();
  stream_load(st0, W[0].job.rng, lane);
  int n_acc = 0;
  DecideStats st = {0u, 0u};
  for (int i = 1; i <= n_windows - 1; ++i) {
    for (int j = lane; j < per_window; j += 32) {
      lo[j] = ov[(i - 1) * per_window + j];
      up[j] = ov[i * per_window + j];
    }
    __syncwarp();
    shuffle_rows(lo, per_window, st0, lane);
    shuffle_rows(up, per_window, st0, lane);
    if (lane == 0) {
      int np = 0;
      for (int j = 0; j < per_window; ++j) {
        if (lo[j].y == 0) continue;
        for (int k = 0; k < per_window; ++k) {
          if (up[k].y == 0) continue;
          if (lo[j].y == up[k].y) {
            pairs[np++] = make_int2(lo[j].x, up[k].x);
            lo[j] = make_int2(0, 0);
            up[k] = make_int2(0, 0);
          }
        }
      }
      *s_np = np;
    }
    __syncwarp();
    const int np = *s_np;
    for (int p = 0; p < np; ++p) {
      const int a = pairs[p].x, b = pairs[p].y;
      const int jb = wl_bin_index(energy[b], e1, range, bins);
      uint32_t* s = a == 0 ? st0 : st1;
      if (a != 0) stream_load(st1, W[a].job.rng, lane);
      const uint32_t wu = stream_draw(s, lane);
      if (a != 0) stream_store(W[a].job.rng, st1, lane);
      const int ia = ibin[a];
      int acc = 0;
      if (ia >= 1 && ia <= bins && jb >= 1 && jb <= bins) {
        const double d = __dsub_rn(W[a].lng[ia - 1], W[a].lng[jb - 1]);
        acc = u_lt_exp(wu, d, st);
      }
      if (lane == 0) {
        partner[a] = b;
        partner[b] = a;
      }
      if (acc) {
        int8_t* la = W[a].job.lat;
        int8_t* lb = W[b].job.lat;
        for (int t = lane; t < W[a].job.g.n_sites; t += 32) {
          const int8_t x = la[t];
          la[t] = lb[t];
          lb[t] = x;
        }
        if (lane == 0) {
          exchanged[a] = 1;
          exchanged[b] = 1;
        }
        ++n_acc;
      }
      __syncwarp();
    }
  }
  stream_store(W[0].job.rng, st0, lane);
  if (lane == 0) *n_accepted = n_acc;
}

uint32_t wl_exchange_smem_bytes(int per_window) {
  return 1280u * 4u + 3u * (uint32_t)per_window * 8u + 16u;
}

void launch_wl_exchange(WlWalker* d_walkers, const double* d_energy, const WlGroup* d_groups,
                        int n_windows, int per_window, int* d_ibin, int2* d_ov, int* d_partner,
                        int* d_exchanged, int* d_n_accepted, cudaStream_t stream) {
  const uint32_t smem = wl_exchange_smem_bytes(per_window);
  cudaFuncSetAttribute(wl_exchange_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  BRAWL_CARVEOUT(wl_exchange_kernel);
  wl_exchange_kernel<<<1, 32, smem, stream>>>(d_walkers, d_energy, d_groups, n_windows, per_window,
                                              d_ibin, d_ov, d_partner, d_exchanged, d_n_accepted);
}

// flatness = minval(hist)/(sum(hist)/mpi_bins) (src/wang-landau.F90:222),
// one thread per walker summing its histogram in bin order.
__global__ void wl_flatness_kernel(const WlWalker* __restrict__ W, int n, double* __restrict__ out) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n) return;
  const int nb = W[w].end - W[w].start + 1;
  const double* h = W[w].hist;
  double mn = h[0], s = 0.0;
  for (int b = 0; b < nb; ++b) {
    const double v = h[b];
    mn = v < mn ? v : mn;
    s = __dadd_rn(s, v);
  }
  out[w] = __ddiv_rn(mn, __ddiv_rn(s, (double)nb));
}

void launch_wl_flatness(const WlWalker* d_walkers, int n, double* d_out, cudaStream_t stream) {
  BRAWL_CARVEOUT(wl_flatness_kernel);
  wl_flatness_kernel<<<(n + 127) / 128, 128, 0, stream>>>(d_walkers, n, d_out);
}

// dos_combine (src/wang-landau.F90:1147-1194) in one CTA: window by window,
// the first bin of the overlap where the slopes of the combined and the
// window's ln g differ least (the lowest such bin: the reference keeps the
// first strict improvement), then the window's ln g shifted onto the
// combined one from that bin to the window's end, exactly as the
// reference's sequential loop rounds it: the meeting bin becomes
// c' = (buf(k) + c(k)) - buf(k) and every later bin (buf(j) + c') - buf(k).
// Finally the minimum is subtracted.  status: 0, or 1 when no overlap bin
// was ever found (the reference would index bin 0).
constexpr int kCombineThreads = 256;
#define kInfD __longlong_as_double(0x7ff0000000000000LL)

__global__ void __launch_bounds__(kCombineThreads) wl_combine_kernel(
    const WlWalker* __restrict__ W, const WlGroup* __restrict__ groups, int n_groups,
    double* __restrict__ out, int* __restrict__ status) {
  __shared__ double red_d[kCombineThreads];
  __shared__ int red_j[kCombineThreads];
  __shared__ int s_beta;
  __shared__ double s_c;
  const int tid = threadIdx.x;
  const int bins = W[0].bins;
  const double* first = W[groups[0].first].lng;
  for (int b = tid; b < bins; b += kCombineThreads) out[b] = first[b];
  if (tid == 0) s_beta = 0;
  __syncthreads();
  for (int i = 1; i < n_groups; ++i) {
    const WlWalker& Wi = W[groups[i].first];
    const double* buf = Wi.lng;
    const int s = Wi.start, e = Wi.end;
    const int L = W[groups[i - 1].first].end - s;     // j = 0 .. L-1
    double best = kInfD;
    int bj = 0x7fffffff;
    for (int j = tid; j < L; j += kCombineThreads) {
      const double bo = __dsub_rn(out[s + j], out[s + j - 1]);
      const double bm = __dsub_rn(buf[s + j], buf[s + j - 1]);
      const double d = fabs(__dsub_rn(bo, bm));
      if (d < 1.7976931348623157e308 && (d < best || (d == best && j < bj))) {
        best = d;
        bj = j;
      }
    }
    red_d[tid] = best;
    red_j[tid] = bj;
    __syncthreads();
    for (int h = kCombineThreads / 2; h > 0; h >>= 1) {
      if (tid < h) {
        const double d2 = red_d[tid + h];
        const int j2 = red_j[tid + h];
        if (d2 < red_d[tid] || (d2 == red_d[tid] && j2 < red_j[tid])) {
          red_d[tid] = d2;
          red_j[tid] = j2;
        }
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (red_j[0] != 0x7fffffff) s_beta = s + red_j[0] + 1;
      if (s_beta >= 1) {
        const int k = s_beta;
        s_c = __dsub_rn(__dadd_rn(buf[k - 1], out[k - 1]), buf[k - 1]);
      }
    }
    __syncthreads();
    const int k = s_beta;
    if (k < 1) {
      if (tid == 0) *status = 1;
      return;
    }
    const double c = s_c, bk = buf[k - 1];
    for (int j = k + tid; j <= e; j += kCombineThreads)
      out[j - 1] = j == k ? c : __dsub_rn(__dadd_rn(buf[j - 1], c), bk);
    __syncthreads();
  }
  // minimum (NaN ignored), then subtract
  double mn = kInfD;
  bool have = false;
  for (int b = tid; b < bins; b += kCombineThreads) {
    const double v = out[b];
    if (v == v && (!have || v < mn)) {
      mn = v;
      have = true;
    }
  }
  red_d[tid] = have ? mn : kInfD;
  red_j[tid] = have ? 1 : 0;
  __syncthreads();
  for (int h = kCombineThreads / 2; h > 0; h >>= 1) {
    if (tid < h && red_j[tid + h]) {
      if (!red_j[tid] || red_d[tid + h] < red_d[tid]) red_d[tid] = red_d[tid + h];
      red_j[tid] = 1;
    }
    __syncthreads();
  }
  const double m = red_j[0] ? red_d[0] : 0.0;
  for (int b = tid; b < bins; b += kCombineThreads) out[b] = __dsub_rn(out[b], m);
  if (tid == 0) *status = 0;
}

// MPI_BCAST of the combined ln g: every walker's copy.
__global__ void wl_broadcast_kernel(WlWalker* __restrict__ W, const double* __restrict__ src) {
  const int bins = W[0].bins;
  double* dst = W[blockIdx.y].lng;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bins; b += gridDim.x * blockDim.x)
    dst[b] = src[b];
}

void launch_wl_combine(WlWalker* d_walkers, int n, const WlGroup* d_groups, int n_groups, int bins,
                       double* d_out, int* d_status, cudaStream_t stream) {
  BRAWL_CARVEOUT(wl_combine_kernel);
  wl_combine_kernel<<<1, kCombineThreads, 0, stream>>>(d_walkers, d_groups, n_groups, d_out, d_status);
  dim3 grid((bins + 255) / 256, n);
  BRAWL_CARVEOUT(wl_broadcast_kernel);
  wl_broadcast_kernel<<<grid, 256, 0, stream>>>(d_walkers, d_out);
}

// merge_configs (src/wang-landau.F90:1556-1615) after the host's draw: bin b
// of every walker's store takes walker pick[b]'s slot (walker 0's when no
// walker holds the bin, as rank 0's array is broadcast), and its flag is
// closed when a walker held it, open otherwise.  One block per (bin,
// walker stripe); the source slot is never written.
__global__ void wl_store_merge_kernel(const WlWalker* __restrict__ W, int n, const int* __restrict__ pick) {
  const int b = blockIdx.x;
  const int src = pick[b] >= 0 ? pick[b] : 0;
  const size_t n_sites = (size_t)W[src].job.g.n_sites;
  const int8_t* from = W[src].store + (size_t)b * n_sites;
  for (int w = blockIdx.y; w < n; w += gridDim.y) {
    if (w != src) {
      int8_t* to = W[w].store + (size_t)b * n_sites;
      for (size_t i = threadIdx.x; i < n_sites; i += blockDim.x) to[i] = from[i];
    }
    if (threadIdx.x == 0) W[w].store_open[b] = pick[b] >= 0 ? 0 : 1;
  }
}

void launch_wl_store_merge(const WlWalker* d_walkers, int n, int bins, const int* d_pick, cudaStream_t stream) {
  if (n <= 0 || bins <= 0) return;
  const dim3 grid((unsigned)bins, (unsigned)std::min(n, 64));
  wl_store_merge_kernel<<<grid, 256, 0, stream>>>(d_walkers, n, d_pick);
}

template <bool kUseD>
static void preload_wl_d(cudaFuncAttributes& a) {
  cudaFuncGetAttributes(&a, wl_sweep_kernel<2, kUseD>);
  cudaFuncGetAttributes(&a, wl_sweep_kernel<4, kUseD>);
  cudaFuncGetAttributes(&a, wl_sweep_kernel<6, kUseD>);
  cudaFuncGetAttributes(&a, wl_sweep_kernel<8, kUseD>);
  cudaFuncGetAttributes(&a, wl_sweep_kernel<11, kUseD>);
}

void preload_wl_kernels() {
  cudaFuncAttributes a;
  preload_wl_d<true>(a);
  preload_wl_d<false>(a);
  cudaFuncGetAttributes(&a, wl_average_kernel);
  cudaFuncGetAttributes(&a, wl_flatness_kernel);
}

}  // namespace brawl
