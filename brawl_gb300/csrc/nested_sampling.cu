// nested_sampling.cu -- nested sampling on the device
// (src/nested_sampling.f90:45-206): K walkers drawn by initial_setup from
// one stream, then per iteration the highest energy becomes the ceiling, a
// random walker is cloned over it and walks n_steps (+ adaptive extra steps)
// random swaps, each accepted iff E + dE stays below the ceiling.
//
// One warp per independent run.  The walkers live in HBM (compact, one byte
// per site); the active walker is staged in shared memory for its walk.  The
// walker's energy is carried in FP64 as the reference does; the kernel keeps
// an interval that contains it, and the fixed-point delta settles most
// steps: certainly over the ceiling (rejected) or certainly under it
// (accepted, logged, its FP64 sums run later with others, lazy_exact.cuh).
// A step the interval does not settle flushes the log and takes the
// reference-order FP64 sums.
#include "halo_engine.cuh"
#include "kernels.cuh"
#include "lazy_exact.cuh"
#include "ns_kernels.cuh"

namespace brawl {

// Walker initialisation: for each walker in order, initial_setup then one
// draw for the 1e-8 energy jitter (nested_sampling.f90:86-96).
__global__ void __launch_bounds__(32) ns_init_kernel(NsRun* __restrict__ runs) {
  __shared__ uint32_t mt[kMTN];
  __shared__ int64_t check[kMaxSpecies];
  NsRun& R = runs[blockIdx.x];
  const int lane = threadIdx.x;
  uint32_t* rng = R.job.rng;
  for (int i = lane; i < kMTN; i += 32) mt[i] = rng[i];
  int pos = (int)rng[kMTN];
  __syncwarp();
  unsigned long long draws = 0;
  const int n = R.job.g.n_sites;
  for (int w = 0; w < R.K; ++w) {
    if (!initial_setup_warp(R.init, R.walkers + (size_t)w * n, mt, pos, check, draws, lane)) {
      if (lane == 0) *R.job.status = kStatusBadSpecies;
      return;
    }
    const uint32_t u = __shfl_sync(kFull, mt_peek(mt, pos, 1, lane), 0);
    pos += 1;
    ++draws;
    if (lane == 0) R.rnde[w] = u;
  }
  __syncwarp();
  for (int i = lane; i < kMTN; i += 32) rng[i] = mt[i];
  if (lane == 0) {
    rng[kMTN] = (uint32_t)pos;
    R.job.counters[kCntDraws] += draws;
  }
}

// energies(w) = full_energy(walker w) + rnde * 1e-8 (the literal is single
// precision in the reference).
__global__ void ns_jitter_kernel(NsRun* __restrict__ runs, int n_runs) {
  const int r = blockIdx.y;
  if (r >= n_runs) return;
  NsRun& R = runs[r];
  const double c = (double)1.0e-8f;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < R.K; w += gridDim.x * blockDim.x) {
    const double u = __dmul_rn((double)R.rnde[w], 2.3283064365386963e-10);
    R.energies[w] = __dadd_rn(R.energies[w], __dmul_rn(u, c));
  }
}

// Order-preserving integer key of a double (larger double, larger key).
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Fixed-point lower bound of the room under the ceiling: Gdn <= (pred(limit)
// - E) * 2^S, pred(limit) the largest double below it; a step with
// dE + band <= Gdn certainly lands strictly below the ceiling.
__device__ __forceinline__ long long gap_dn(double limit, double E, int S) {
  const double gd = __dsub_rd(nextafter(limit, -__longlong_as_double(0x7ff0000000000000LL)), E);
  const double m = __dsub_rd(gd, __dmul_ru(fabs(gd), 8.881784197001252e-16));  // - |gd| 2^-50
  const double s = ldexp(m, S);
  if (!(s > -9.0e18)) return -0x7fffffffffffffffll;
  if (s > 9.0e18) return 0x7fffffffffffffffll;
  return (long long)floor(s);
}

// Fixed-point upper bound of the ceiling gap: Gup >= (limit - E) * 2^S.
__device__ __forceinline__ long long gap_up(double limit, double E, int S) {
  const double gd = __dsub_rn(limit, E);
  const double m = __dadd_rn(gd, __dmul_rn(fabs(gd), 8.881784197001252e-16));  // + |gd| 2^-50
  const double s = ldexp(m, S);
  if (!(s < 9.0e18)) return 0x7fffffffffffffffll;
  if (s < -9.0e18) return -0x7fffffffffffffffll;
  return (long long)ceil(s);
}


// site-2 redraws tried at once, one per lane (3 words each, within the
// ring's mirror)
constexpr int kRedraws = 32;
static_assert(3 * kRedraws <= kRingMirror, "redraw words must fit the ring's mirror");

// Warps per run: warp 0 walks; the others join only the deferred-energy
// flushes, whose FP64 sums are the step's largest cost (each sub-partition
// of an SM has its own FP64 pipe, so four warps sum four times as fast).
constexpr int kNsWarps = 4;

template <int NJ, bool kUseD>
__global__ void __launch_bounds__(32 * kNsWarps, 1) ns_iterate_kernel(NsRun* __restrict__ runs) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_ctl[2];  // the flushes' command and move count (lazy_flush_block)
  NsRun& R = runs[blockIdx.x];
  const ChainJob& J = R.job;
  const Geom g = J.g;
  const int lane = threadIdx.x & 31;
  const int nthreads = blockDim.x;
  const unsigned long long t_start = global_ns();
  const int n = g.n_sites;
  const int nV = g.ns * g.ns * g.nsh;
  const WalkerLayout WLy = walker_layout(g, 0, R.lazy_cap);
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem + WLy.mt);
  uint32_t* tbuf = reinterpret_cast<uint32_t*>(smem + WLy.tbuf);
  double* V = reinterpret_cast<double*>(smem + WLy.V);
  int32_t* I = reinterpret_cast<int32_t*>(smem + WLy.I);
  int32_t* F = I + WLy.F_off;
  uint32_t* ents = reinterpret_cast<uint32_t*>(smem + WLy.ents);
  int16_t* sstart = reinterpret_cast<int16_t*>(smem + WLy.sstart);
  int8_t* lat = reinterpret_cast<int8_t*>(smem + WLy.lat);
  double* vbuf = reinterpret_cast<double*>(smem + WLy.vbuf);
  const LazyLog LG = lazy_layout(g, smem + WLy.lazy, R.lazy_cap);
  if (threadIdx.x >= 32) {
    // a helper warp: flushes only, until warp 0 releases it
    lazy_helper_loop(g, V, sstart, LG, kFoldNested, threadIdx.x, nthreads, s_ctl);
    return;
  }
  const double q = ldexp(1.0, -R.S);
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nV; i += 32) V[i] = J.V[i];
  for (int i = lane; i < WLy.nI - WLy.F_off; i += 32) F[i] = J.F[i];
  for (int i = lane; i < g.z; i += 32) ents[i] = J.entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = J.shell_start[i];
  AxisTables T;
  build_axis_tables(g, I, WLy.tab_len, lane, T);
  __syncwarp();
  LanePlan<NJ> P;
  make_lane_plan<NJ>(g, ents, I, T, lane, P);
  const int lat_off = (int)WLy.lat, I_off = (int)(WLy.I / 4);
  const int log_off = (int)(LG.codes - smem);
  const bool self_map = g.W1 <= kHalo || g.W2 <= kHalo || g.W3 <= kHalo;
  Ring ring;
  ring_init(mt, tbuf, (int)J.rng[kMTN], lane, ring);

  const int K = R.K;
  const int half = R.half;
  const int S = R.S;
  const int band = J.band;
  int extra_steps = R.extra_steps;
  long long n_acc = R.n_acc;
  long long it = R.iter;
  unsigned long long c_steps = 0, c_draws = 0, c_acc = 0, c_exact = 0;
  int status = kStatusOk;

  for (int li = 0; li < R.n_iter; ++li) {
    ++it;
    // maxloc: first index of the largest energy
    unsigned long long best = 0;
    int bidx = 0x7fffffff;
    for (int w = lane; w < K; w += 32) {
      const unsigned long long k = dkey(R.energies[w]);
      if (k > best || (k == best && w < bidx)) {
        best = k;
        bidx = w;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(kFull, best, o);
      const int oi = __shfl_xor_sync(kFull, bidx, o);
      if (ok > best || (ok == best && oi < bidx)) {
        best = ok;
        bidx = oi;
      }
    }
    const int imax = bidx;
    const double limit = R.energies[imax];
    if (lane == 0) R.limits[li] = limit;
    // adaptive extra steps (nested_sampling.f90:129-144)
    if (half > 0 && (it % half) == 0) {
      if (((float)n_acc < (float)R.n_at * 0.05f) && (extra_steps < R.n_steps * 100))
        extra_steps += R.n_steps;
    }
    // clone: irnd = ceiling(rnd * K), 0 only when rnd == 0 (clamped to 1)
    ring_ensure(mt, tbuf, ring, 1, lane);
    const uint32_t wr = tbuf[ring.idx];
    ring_consume(ring, 1);
    ++c_draws;
    int irnd = (int)(((unsigned long long)wr * (unsigned long long)K + 0xffffffffull) >> 32);
    if (irnd < 1) irnd = 1;
    const int8_t* src = R.walkers + (size_t)(irnd - 1) * n;
    for (int i = lane; i < n; i += 32) lat[i] = src[i];
    // E: the walker's exact energy before the n_log logged steps; after
    // them it lies in E + [Dlo - Rs, Dhi + Rs] quanta (Rs: the roundings of
    // the logged updates), so the ceiling tests are integer compares against
    // gaps taken once per exact energy
    double E = R.energies[irnd - 1];
    long long Dlo = 0, Dhi = 0, Rs = 0, Eq = 0, gup = 0, gdn = 0;
    int n_log = 0;
    __syncwarp();
    auto rebase = [&]() {
      gup = gap_up(limit, E, S);
      gdn = gap_dn(limit, E, S);
      Eq = quanta_bound(E, S);
      Dlo = Dhi = Rs = 0;
    };
    rebase();
    auto flush = [&]() {
      if (n_log == 0) return;
      const double E0 = E;
      E = lazy_flush_block(g, V, sstart, LG, n_log, E, kFoldNested, lane, nthreads, s_ctl);
      if (!in_quanta(E, E0, Dlo - Rs, Dhi + Rs, q)) status = kStatusBandViolated;
      n_log = 0;
      rebase();
    };
    n_acc = 0;
    const long long steps = (long long)R.n_steps + extra_steps;
    for (long long st = 0; st < steps && status == kStatusOk; ++st) {
      ring_ensure(mt, tbuf, ring, 3, lane);
      SitePair p;
      draw_site(g, tbuf[ring.idx], tbuf[ring.idx + 1], tbuf[ring.idx + 2], p.ax, p.ay, p.az);
      ring_consume(ring, 3);
      p.ai = compact_index(g, p.ax, p.ay, p.az);
      p.sa = lat[p.ai];
      // site 2 is redrawn until its species differs from site 1's: the
      // redraws are consecutive word triples, so lane k tries the k-th next
      // one and the first lane that finds another species ends the loop
      // (kRedraws at a time)
      int tries = 0;
      for (;;) {
        ring_ensure(mt, tbuf, ring, 3 * kRedraws, lane);
        int bx = 0, by = 0, bz = 0, bi = 0, sb = 0;
        bool other = false;
        if (lane < kRedraws) {
          const int o = ring.idx + 3 * lane;
          draw_site(g, tbuf[o], tbuf[o + 1], tbuf[o + 2], bx, by, bz);
          bi = compact_index(g, bx, by, bz);
          sb = lat[bi];
          other = sb != p.sa;
        }
        const unsigned hit = __ballot_sync(kFull, other);
        const int used = hit ? __ffs(hit) : kRedraws;  // redraws consumed
        ring_consume(ring, 3 * used);
        c_draws += 3 * used;
        tries += used;
        if (hit) {
          const int k = used - 1;
          p.bx = __shfl_sync(kFull, bx, k);
          p.by = __shfl_sync(kFull, by, k);
          p.bz = __shfl_sync(kFull, bz, k);
          p.bi = __shfl_sync(kFull, bi, k);
          p.sb = __shfl_sync(kFull, sb, k);
          break;
        }
        if (tries > (1 << 24)) {
          status = kStatusBadSpecies;  // a single species: the reference loops forever
          break;
        }
      }
      if (status != kStatusOk) break;
      c_draws += 3;
      ++c_steps;
      uint8_t* rec = LG.codes + (size_t)n_log * 2 * g.z;
      bool near;
      int dE = fixed_delta_rec<NJ, kUseD>(g, lat_off, I_off, WLy.F_off, WLy.D_off, P, p, lane,
                                          log_off + n_log * 2 * g.z, near);
      if (near || self_map) dE = compact_fixed_delta_rec(g, lat, F, ents, p, lane, rec);
      // E + dE lies in E_exact + [lo, hi] quanta; rounding the sum to a double
      // keeps it on the same side of the ceiling (a double) or of the
      // double below it
      long long lo = Dlo - Rs + dE - band, hi = Dhi + Rs + dE + band;
      if (lo >= gup) continue;  // certainly at or over the ceiling: rejected
      bool logged = false;
      if (hi > gdn && n_log > 0) {
        // not settled with the logged steps' interval: their exact energy
        // may settle it; this step's codes move to the log's first slot
        __syncwarp();
        flush();
        lazy_copy_slot(g, rec, LG.codes, lane);
        lo = (long long)dE - band;
        hi = (long long)dE + band;
        if (lo >= gup) continue;
      }
      if (hi <= gdn) {
        // certainly below the ceiling: accepted, the FP64 sums deferred
        if (lane == 0) {
          LG.spec[2 * n_log] = (int8_t)p.sa;
          LG.spec[2 * n_log + 1] = (int8_t)p.sb;
        }
        ++n_log;
        Dlo += (long long)dE - band;
        Dhi += (long long)dE + band;
        // the update E + delta_e rounds by at most |E + delta_e| 2^-53
        const long long B = Eq + max(llabs(Dlo), llabs(Dhi)) + Rs;
        Rs += (B >> 53) + 1;
        logged = true;
      } else {
        // the exact step, as the reference takes it (the log is empty)
        ++c_exact;
        double e_un, e_sw;
        exact_pair_energies_staged(g, CompactLat{lat}, V, ents, sstart, p, lane, e_un, e_sw, vbuf);
        const double delta_e = __dsub_rn(e_sw, e_un);
        const double e_new = __dadd_rn(E, delta_e);
        if (!(e_new < limit)) continue;
        E = e_new;
        rebase();
      }
      ++n_acc;
      ++c_acc;
      if (lane == 0) {
        lat[p.ai] = (int8_t)p.sb;
        lat[p.bi] = (int8_t)p.sa;
      }
      __syncwarp();
      if (logged && n_log == LG.cap) flush();
    }
    flush();
    if (status != kStatusOk) break;
    int8_t* dst = R.walkers + (size_t)imax * n;
    for (int i = lane; i < n; i += 32) dst[i] = lat[i];
    if (lane == 0) R.energies[imax] = E;
    __syncwarp();
  }
  lazy_helpers_release(lane, nthreads, s_ctl);
  ring_writeback(mt, tbuf, ring, J.rng, lane);
  if (lane == 0) {
    R.extra_steps = extra_steps;
    R.n_acc = n_acc;
    R.iter = it;
    unsigned long long* c = J.counters;
    c[kCntTrials] += c_steps;
    c[kCntEvaluated] += c_steps;
    c[kCntDraws] += c_draws;
    c[kCntAccepted] += c_acc;
    c[kCntExactPath] += c_exact;
    if (status != kStatusOk) *J.status = status;
    if (J.t_ns) *J.t_ns = global_ns() - t_start;
  }
}

uint32_t ns_smem_bytes(const Geom& g, int lazy_cap) {
  return walker_layout(g, 0, lazy_cap).total;
}

void launch_ns_init(NsRun* d_runs, int n_runs, cudaStream_t stream) {
  BRAWL_CARVEOUT(ns_init_kernel);
  ns_init_kernel<<<n_runs, 32, 0, stream>>>(d_runs);
}

void launch_ns_jitter(NsRun* d_runs, int n_runs, int max_K, cudaStream_t stream) {
  dim3 grid((max_K + 255) / 256, n_runs);
  BRAWL_CARVEOUT(ns_jitter_kernel);
  ns_jitter_kernel<<<grid, 256, 0, stream>>>(d_runs, n_runs);
}

template <int NJ, bool kUseD>
static void launch_ns_nj(NsRun* d_runs, int n_runs, uint32_t smem_bytes, cudaStream_t stream) {
  cudaFuncSetAttribute(ns_iterate_kernel<NJ, kUseD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_bytes);
  BRAWL_CARVEOUT(ns_iterate_kernel<NJ, kUseD>);
  ns_iterate_kernel<NJ, kUseD><<<n_runs, 32 * kNsWarps, smem_bytes, stream>>>(d_runs);
}

template <bool kUseD>
static void launch_ns_d(NsRun* d_runs, int n_runs, uint32_t smem_bytes, int max_z, cudaStream_t stream) {
  switch (lane_entries_for(max_z)) {
    case 2: launch_ns_nj<2, kUseD>(d_runs, n_runs, smem_bytes, stream); break;
    case 4: launch_ns_nj<4, kUseD>(d_runs, n_runs, smem_bytes, stream); break;
    case 6: launch_ns_nj<6, kUseD>(d_runs, n_runs, smem_bytes, stream); break;
    case 8: launch_ns_nj<8, kUseD>(d_runs, n_runs, smem_bytes, stream); break;
    default: launch_ns_nj<11, kUseD>(d_runs, n_runs, smem_bytes, stream); break;
  }
}

void launch_ns_iterate(NsRun* d_runs, int n_runs, uint32_t smem_bytes, int max_z, bool all_D,
                       cudaStream_t stream) {
  if (n_runs <= 0) return;
  if (all_D) launch_ns_d<true>(d_runs, n_runs, smem_bytes, max_z, stream);
  else launch_ns_d<false>(d_runs, n_runs, smem_bytes, max_z, stream);
}

template <bool kUseD>
static void preload_ns_d(cudaFuncAttributes& a) {
  cudaFuncGetAttributes(&a, ns_iterate_kernel<2, kUseD>);
  cudaFuncGetAttributes(&a, ns_iterate_kernel<4, kUseD>);
  cudaFuncGetAttributes(&a, ns_iterate_kernel<6, kUseD>);
  cudaFuncGetAttributes(&a, ns_iterate_kernel<8, kUseD>);
  cudaFuncGetAttributes(&a, ns_iterate_kernel<11, kUseD>);
}

void preload_ns_kernels() {
  cudaFuncAttributes a;
  preload_ns_d<true>(a);
  preload_ns_d<false>(a);
  cudaFuncGetAttributes(&a, ns_init_kernel);
  cudaFuncGetAttributes(&a, ns_jitter_kernel);
}

}  // namespace brawl
