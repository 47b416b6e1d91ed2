// lazy_exact.cuh -- deferred reference-order energies for walkers that carry
// their energy in FP64 (Wang-Landau sweeps, nested-sampling walks).
//
// The reference updates a walker's energy on every accepted move from the
// two FP64 pair energies, each a chain of dependent FP64 adds in neighbour
// list order.  Most decisions only need an interval that contains that
// energy: the fixed-point delta gives one (band quanta wide per move), and a
// bin or a ceiling is usually far from its edges.  So an accepted move whose
// decision the interval settles is logged -- the species of the two sites
// and of their neighbours as they were at the move -- and the FP64 sums of
// the logged moves run later, together: one chain per (move, site, before or
// after, shell), several chains per lane so the FP64 adds overlap, then the
// walker's energy folded through the moves in order exactly as the
// reference does.  Same values, same order, same roundings: identical
// energies; only when they are computed changes.  A decision the interval
// does not settle flushes the log first and then takes the exact path.
#pragma once

#include "chain_engine.cuh"
#include "kernels.cuh"

namespace brawl {

constexpr int kLazyMaxCap = 64;
constexpr int kLazyPartner = 0x40;  // the neighbour is the other site of the pair
constexpr int kLazySelf = 0x80;     // the neighbour is the site itself (small lattices)

// Shared-memory bytes of a log of `cap` moves: neighbour codes (2 z bytes a
// move), the pair's species (2), the chain sums (4 nsh doubles) and the pair
// energies (2 doubles).
__host__ __device__ inline uint32_t lazy_bytes(const Geom& g, int cap) {
  const uint32_t c = (uint32_t)cap;
  uint32_t b = align_up(c * 2u * (uint32_t)g.z, 16);
  b += align_up(c * 2u, 16);
  b += c * 4u * (uint32_t)g.nsh * 8u;
  b += c * 2u * 8u;
  return align_up(b, 16);
}

// The largest log (a power of two, at most kLazyMaxCap) that fits beside
// `base` bytes within `limit`; 0 when not even one move fits.
inline int lazy_cap_for(const Geom& g, uint32_t base, uint32_t limit) {
  for (int cap = kLazyMaxCap; cap >= 1; cap >>= 1)
    if (base + lazy_bytes(g, cap) <= limit) return cap;
  return 0;
}

struct LazyLog {
  uint8_t* codes;  // [cap][2][z]: species | kLazyPartner | kLazySelf
  int8_t* spec;    // [cap][2]: species of site 1 and site 2 before the move
  double* part;    // [cap][4][nsh]: shell sums, then site energies
  double* pair;    // [cap][2]: pair energy before and after
  int cap;
};

__device__ inline LazyLog lazy_layout(const Geom& g, unsigned char* base, int cap) {
  LazyLog L;
  const uint32_t c = (uint32_t)cap;
  L.codes = base;
  base += align_up(c * 2u * (uint32_t)g.z, 16);
  L.spec = reinterpret_cast<int8_t*>(base);
  base += align_up(c * 2u, 16);
  L.part = reinterpret_cast<double*>(base);
  base += c * 4u * (uint32_t)g.nsh * 8u;
  L.pair = reinterpret_cast<double*>(base);
  L.cap = cap;
  return L;
}

// Shared memory of a walker kernel (a Wang-Landau walker's sweep, nested-
// sampling walks): the stream and its tempered ring, V, the int32 region I
// (axis tables, F, D when it fits, as in smem_layout), nb bins of ln g and of
// the histogram (Wang-Landau), the neighbour entries and shell starts, the
// compact lattice, the staged exact-sum terms (4 z doubles) and the log.
struct WalkerLayout {
  uint32_t mt, tbuf, V, I, slices, sopen, ents, sstart, lat, vbuf, lazy;
  uint32_t rad, rad_offsets, rad_masks, rad_hist, total;  // radial-sample scratch
  uint32_t tab_len[3];
  int32_t F_off, D_off, use_D, nI;
};

// rad_bins > 0: the radial-sample scratch follows the log -- one eligibility
// bit per bin, the ASRO plan's offsets and class masks, and the
// (species, species, class) and species counts.
__host__ __device__ inline WalkerLayout walker_layout(const Geom& g, int nb, int lazy_cap,
                                                      int rad_bins = 0, int rad_n_offsets = 0,
                                                      int rad_n_class = 0) {
  WalkerLayout L;
  const uint32_t nsp = (uint32_t)g.ns + 1;
  const uint32_t nF = nsp * (uint32_t)g.nsh * nsp;
  const uint32_t nD = nsp * nsp * (uint32_t)g.nsh * nsp;
  L.mt = 0;
  L.tbuf = kMTN * 4;
  L.V = align_up((kMTN + kTbufWords) * 4, 16);
  L.I = align_up(L.V + (uint32_t)(g.ns * g.ns * g.nsh) * 8, 16);
  L.tab_len[0] = 2 * (uint32_t)g.n1 + 2 * kHalo;
  L.tab_len[1] = 2 * (uint32_t)g.n2 + 2 * kHalo;
  L.tab_len[2] = 2 * (uint32_t)g.n3 + 2 * kHalo;
  const uint32_t ntab = 2 * (L.tab_len[0] + L.tab_len[1] + L.tab_len[2]);
  L.use_D = nD * 4 <= kMaxDBytes ? 1 : 0;
  L.F_off = (int32_t)ntab;
  L.D_off = (int32_t)(ntab + nF);
  L.nI = (int32_t)(ntab + nF + (L.use_D ? nD : 0));
  L.slices = align_up(L.I + (uint32_t)L.nI * 4, 16);
  // the window's ln g and histogram slices, then its open store flags
  L.sopen = L.slices + 2u * (uint32_t)nb * 8;
  L.ents = align_up(L.sopen + (uint32_t)nb, 4);
  L.sstart = L.ents + (uint32_t)g.z * 4;
  L.lat = align_up(L.sstart + (uint32_t)(g.nsh + 1) * 2, 16);
  L.vbuf = align_up(L.lat + (uint32_t)g.n_sites, 16);
  L.lazy = align_up(L.vbuf + 4u * (uint32_t)g.z * 8, 16);
  L.rad = L.lazy + (lazy_cap > 0 ? lazy_bytes(g, lazy_cap) : 0);
  L.rad_offsets = L.rad;
  L.rad_masks = L.rad;
  L.rad_hist = L.rad;
  L.total = L.rad;
  if (rad_bins > 0) {
    L.rad_offsets = align_up(L.rad + (((uint32_t)rad_bins + 31) / 32) * 4, 16);
    L.rad_masks = align_up(L.rad_offsets + (uint32_t)rad_n_offsets * 4, 16);
    L.rad_hist = L.rad_masks + (uint32_t)rad_n_class * 8;
    L.total = align_up(L.rad_hist + (nsp * nsp * (uint32_t)rad_n_class + nsp) * 4, 16);
  }
  return L;
}

// fixed_delta (chain_engine.cuh) on a compact lattice in shared memory, also
// writing each neighbour's species to the log slot at byte offset rec_off
// (site 1's entries first).  Valid when the pair is not near and no site is
// its own neighbour; otherwise the caller takes compact_fixed_delta_rec.
template <int NJ, bool kUseD>
__device__ __forceinline__ int fixed_delta_rec(const Geom& g, int lat_off, int I_off, int F_off,
                                               int D_off, const LanePlan<NJ>& P,
                                               const SitePair& p, int lane, int rec_off,
                                               bool& near) {
  extern __shared__ int32_t s_i32[];
  extern __shared__ int8_t s_i8[];
  extern __shared__ uint8_t s_u8[];
  const bool h = lane >= 16;
  const int cx = h ? p.bx : p.ax, cy = h ? p.by : p.ay, cz = h ? p.bz : p.az;
  const int other = h ? p.ai : p.bi;
  const int so = h ? p.sb : p.sa, sn = h ? p.sa : p.sb;
  const int nsp = g.ns + 1;
  const int rowD = I_off + D_off + (so * nsp + sn) * g.nsh * nsp;
  const int rowN = I_off + F_off + sn * g.nsh * nsp;
  const int rowO = I_off + F_off + so * g.nsh * nsp;
  const int bx = I_off + cx, by = I_off + cy, bz = I_off + cz;
  const int out = rec_off + (h ? g.z : 0) + (lane & 15);
  int acc = 0;
  bool hit = false;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int ni = s_i32[P.ax[j] + bx] + s_i32[P.ay[j] + by] + s_i32[P.az[j] + bz];
    const int s_before = (int)s_i8[lat_off + ni];
    const int t = kUseD ? s_i32[rowD + P.shp[j] + s_before]
                        : s_i32[rowN + P.shp[j] + s_before] - s_i32[rowO + P.shp[j] + s_before];
    hit |= ni == other;
    const bool v = (P.valid >> j) & 1u;
    if (v) s_u8[out + 16 * j] = (uint8_t)s_before;
    acc += v ? t : 0;
  }
  near = __any_sync(kFull, hit);
  return __reduce_add_sync(kFull, acc);
}

// compact_fixed_delta, also writing the neighbour codes of both sites to
// rec[0, 2z) (site 1's entries first).
__device__ __forceinline__ int compact_fixed_delta_rec(const Geom& g, const int8_t* lat,
                                                       const int32_t* F, const uint32_t* ents,
                                                       const SitePair& p, int lane, uint8_t* rec) {
  const bool h = lane >= 16;
  const int cx = h ? p.bx : p.ax, cy = h ? p.by : p.ay, cz = h ? p.bz : p.az;
  const int own = h ? p.bi : p.ai, other = h ? p.ai : p.bi;
  const int so = h ? p.sb : p.sa, sn = h ? p.sa : p.sb;
  const int nsp = g.ns + 1;
  const int rowN = sn * g.nsh * nsp, rowO = so * g.nsh * nsp;
  uint8_t* out = rec + (h ? g.z : 0);
  int acc = 0;
  for (int k = lane & 15; k < g.z; k += 16) {
    int dx, dy, dz, sh;
    unpack_entry(ents[k], dx, dy, dz, sh);
    const int ni = neighbour_index(g, cx, cy, cz, dx, dy, dz);
    const int sb = lat[ni];
    const int sa = ni == other ? so : (ni == own ? sn : sb);
    out[k] = (uint8_t)(sb | (ni == other ? kLazyPartner : 0) | (ni == own ? kLazySelf : 0));
    acc += F[rowN + sh * nsp + sa] - F[rowO + sh * nsp + sb];
  }
  return __reduce_add_sync(kFull, acc);
}

// Copies a move's codes between log slots (all lanes).
__device__ __forceinline__ void lazy_copy_slot(const Geom& g, const uint8_t* from, uint8_t* to,
                                               int lane) {
  for (int k = lane; k < 2 * g.z; k += 32) to[k] = from[k];
  __syncwarp();
}

// An upper bound of |E| in quanta 2^-S (saturated far below overflow).
__device__ __forceinline__ long long quanta_bound(double E, int S) {
  const double s = ldexp(fabs(E), S);
  return s < 1.0e18 ? (long long)ceil(s) + 1 : 1000000000000000000ll;
}

// E lies in E0 + [lo, hi] quanta (the check of a deferred energy).
__device__ __forceinline__ bool in_quanta(double E, double E0, long long lo, long long hi, double q) {
  const double a = __dadd_rd(E0, __dmul_rd(__ll2double_rd(lo), q));
  const double b = __dadd_ru(E0, __dmul_ru(__ll2double_ru(hi), q));
  return E >= a && E <= b;
}

// The bin (int(t) + 1, as bin_index) of every energy in E0 + [lo, hi]
// quanta, from t0 = float((E0 - e1) * bins / range) and qrf = float(q * bins /
// range), when one bin holds them all.  t0 is within 6e-8 |t0| of the exact
// coordinate, the offsets within 1.8e-7 |offset| (three roundings), their
// sums within 6e-8 |t|, and the reference's own t within 5e-16 |t|; m
// doubles that.  Far outside (|t| >= 5e8) is left to the exact path.
__device__ __forceinline__ bool bin_from_quanta(float t0, float qrf, long long lo, long long hi,
                                                int& bin) {
  const float plo = __fmul_rn(__ll2float_rn(lo), qrf), phi = __fmul_rn(__ll2float_rn(hi), qrf);
  const float tlo = __fadd_rn(t0, plo), thi = __fadd_rn(t0, phi);
  if (!(fabsf(tlo) < 5.0e8f && fabsf(thi) < 5.0e8f)) return false;
  const float m = (fabsf(t0) + fmaxf(fabsf(tlo), fabsf(thi))) * 1.2e-7f +
                  fmaxf(fabsf(plo), fabsf(phi)) * 3.6e-7f + 1.0e-30f;
  const float blo = truncf(__fsub_rd(tlo, m)), bhi = truncf(__fadd_ru(thi, m));
  if (blo != bhi) return false;
  bin = (int)blo + 1;
  return true;
}

enum LazyFold : int {
  kFoldWangLandau = 0,  // e = (e - pair_before) + pair_after
  kFoldNested = 1,      // e = e + (pair_after - pair_before)
};

constexpr int kLazyIlp = 8;  // chains per lane in flight

// The species a chain's logged neighbour holds at its evaluation (before or
// after the move).
__device__ __forceinline__ int lazy_species(const LazyLog& L, int at, int s_before, int s_after,
                                            bool after) {
  const int code = (int)L.codes[at];
  int s = code & 0x3f;
  if (after) {
    if (code & kLazyPartner) s = s_before;  // the partner now holds our old species
    else if (code & kLazySelf) s = s_after;
  }
  return s;
}

// One logged neighbour's term V(cs, s, shell) of a chain (0 for a lane's
// chain slot past the last chain: adding 0.0 to the unused sums).
__device__ __forceinline__ double lazy_term(const LazyLog& L, const double* Vsh, int at, int cs,
                                            int s_before, int s_after, bool after, bool on, int ns) {
  if (!on) return 0.0;
  return Vsh[(cs - 1) + ns * (lazy_species(L, at, s_before, s_after, after) - 1)];
}

// bar.sync on named barrier `id` for `count` threads (a multiple of 32):
// the warps of a block that share a deferred-energy log meet there.
__device__ __forceinline__ void named_barrier(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// The site energies of the n logged moves, summed by `nthreads` threads
// (this one is tid), ILP chains per thread in flight.  Chain c = 4 m + ev is
// evaluation ev of move m (site 1 before, site 2 before, site 1 after, site
// 2 after); it adds each shell's terms in list order from 0.0 and the shell
// sums left to right (nbr_energy).  The four chains of a move sit in four
// neighbouring lanes (c = tid mod 4), so the pair energies site 1 + site 2
// (pair_energy) are taken through shuffles and written to L.pair[2 m +
// after]; for the nested fold the differences pair_after - pair_before go to
// L.part[m].
template <int ILP>
__device__ __forceinline__ void lazy_sites(const Geom& g, const double* V, const int16_t* sstart,
                                           const LazyLog& L, int n, int fold, int tid, int nthreads) {
  const int z = g.z, nsh = g.nsh, ns = g.ns;
  const int nch = 4 * n;
  for (int c0 = 0; c0 < nch; c0 += nthreads * ILP) {
    int row[ILP], cs[ILP], s_before[ILP], s_after[ILP];
    bool on[ILP], after[ILP];
    double site[ILP];
#pragma unroll
    for (int i = 0; i < ILP; ++i) {
      const int c = c0 + nthreads * i + tid;
      on[i] = c < nch;
      const int m = on[i] ? c >> 2 : 0, ev = c & 3;
      const bool site2 = ev & 1;
      after[i] = ev >= 2;
      const int sa = L.spec[2 * m], sb = L.spec[2 * m + 1];
      s_before[i] = site2 ? sb : sa;  // the site's own species before the move
      s_after[i] = site2 ? sa : sb;
      cs[i] = after[i] ? s_after[i] : s_before[i];
      row[i] = m * 2 * z + (site2 ? z : 0);
      site[i] = 0.0;
    }
    for (int sh = 0; sh < nsh; ++sh) {
      const int k0 = sstart[sh], len = sstart[sh + 1] - k0;
      const double* Vsh = V + ns * ns * sh;
      double sum[ILP];
#pragma unroll
      for (int i = 0; i < ILP; ++i) sum[i] = 0.0;
      int k = 0;
      // the terms of four neighbours of every chain are loaded before
      // their adds, so the loads overlap and the adds issue back to back;
      // each chain still adds its terms in list order
      for (; k + 4 <= len; k += 4) {
        double t[ILP][4];
#pragma unroll
        for (int i = 0; i < ILP; ++i)
#pragma unroll
          for (int u = 0; u < 4; ++u)
            t[i][u] = lazy_term(L, Vsh, row[i] + k0 + k + u, cs[i], s_before[i], s_after[i], after[i], on[i], ns);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int i = 0; i < ILP; ++i) sum[i] = __dadd_rn(sum[i], t[i][u]);
      }
      for (; k < len; ++k) {
#pragma unroll
        for (int i = 0; i < ILP; ++i)
          sum[i] = __dadd_rn(sum[i], lazy_term(L, Vsh, row[i] + k0 + k, cs[i], s_before[i], s_after[i],
                                               after[i], on[i], ns));
      }
      // site energy: shell 1 + shell 2 + ... left to right
#pragma unroll
      for (int i = 0; i < ILP; ++i) site[i] = sh == 0 ? sum[i] : __dadd_rn(site[i], sum[i]);
    }
#pragma unroll
    for (int i = 0; i < ILP; ++i) {
      const int c = c0 + nthreads * i + tid;
      const int ev = c & 3;
      const double pr = __dadd_rn(site[i], __shfl_down_sync(kFull, site[i], 1));  // site 1 + site 2
      if (on[i] && (ev & 1) == 0) L.pair[2 * (c >> 2) + (ev >> 1)] = pr;
      const double pr_after = __shfl_down_sync(kFull, pr, 2);
      if (fold == kFoldNested && on[i] && ev == 0) L.part[c >> 2] = __dsub_rn(pr_after, pr);
    }
  }
}

// lazy_sites with as many chains per thread as the log needs (1 to MaxIlp
// in flight; more chains loop).  Out of line: flushes are rare next to the
// steps.  One warp wants 8 chains per lane to keep its FP64 pipe busy;
// four warps need no more than 4 (fewer registers).
template <int MaxIlp>
static __device__ __noinline__ void lazy_sites_any(const Geom& g, const double* V, const int16_t* sstart,
                                                   LazyLog L, int n, int fold, int tid, int nthreads) {
  const int per = (4 * n + nthreads - 1) / nthreads;
  if (per <= 1) lazy_sites<1>(g, V, sstart, L, n, fold, tid, nthreads);
  else if (per <= 2 || MaxIlp == 2) lazy_sites<2>(g, V, sstart, L, n, fold, tid, nthreads);
  else if (per <= 4 || MaxIlp == 4) lazy_sites<4>(g, V, sstart, L, n, fold, tid, nthreads);
  else lazy_sites<MaxIlp>(g, V, sstart, L, n, fold, tid, nthreads);
}

// The walker's energy e folded with the n moves' pair energies (one warp;
// every lane returns the same value).
static __device__ __noinline__ double lazy_fold(LazyLog L, int n, double e, int fold) {
  if (fold == kFoldWangLandau) {
    // e = (e - pair_before) + pair_after, two dependent adds per move
    for (int m = 0; m < n; ++m) e = __dadd_rn(__dsub_rn(e, L.pair[2 * m]), L.pair[2 * m + 1]);
  } else {
    // e = e + (pair_after - pair_before): the differences were taken in
    // parallel, so the chain is one add per move
    for (int m = 0; m < n; ++m) e = __dadd_rn(e, L.part[m]);
  }
  __syncwarp();
  return e;
}

// The exact energies of the n logged moves folded into e (the walker's
// exact energy before the first of them), by one warp.  All lanes; returns
// the same value in every lane.
__device__ __forceinline__ double lazy_flush(const Geom& g, const double* V, const int16_t* sstart,
                                             const LazyLog& L, int n, double e, int fold, int lane) {
  lazy_sites_any<kLazyIlp>(g, V, sstart, L, n, fold, lane, 32);
  __syncwarp();
  return lazy_fold(L, n, e, fold);
}

// The same with the helper warps of the block: warp 0 posts the move count
// in ctl[1] and meets the helpers at barrier 1, every thread sums its share
// of the chains, barrier 2 closes, and warp 0 folds.  With one warp
// (nthreads = 32) it is lazy_flush.
__device__ __forceinline__ double lazy_flush_block(const Geom& g, const double* V, const int16_t* sstart,
                                                   const LazyLog& L, int n, double e, int fold, int lane,
                                                   int nthreads, volatile int* ctl) {
  if (nthreads == 32) return lazy_flush(g, V, sstart, L, n, e, fold, lane);
  if (lane == 0) {
    ctl[0] = 1;
    ctl[1] = n;
  }
  named_barrier(1, nthreads);
  lazy_sites_any<4>(g, V, sstart, L, n, fold, lane, nthreads);
  named_barrier(2, nthreads);
  return lazy_fold(L, n, e, fold);
}

// The helper warps' side of lazy_flush_block (threads tid >= 32): wait at
// barrier 1 for a flush (ctl[0] = 1) or the end (ctl[0] = 0), sum this
// thread's chains, meet at barrier 2.
__device__ __forceinline__ void lazy_helper_loop(const Geom& g, const double* V, const int16_t* sstart,
                                                 const LazyLog& L, int fold, int tid, int nthreads,
                                                 volatile int* ctl) {
  for (;;) {
    named_barrier(1, nthreads);
    if (ctl[0] == 0) return;
    lazy_sites_any<4>(g, V, sstart, L, ctl[1], fold, tid, nthreads);
    named_barrier(2, nthreads);
  }
}

// Warp 0's end of the helpers' loop.
__device__ __forceinline__ void lazy_helpers_release(int lane, int nthreads, volatile int* ctl) {
  if (nthreads == 32) return;
  if (lane == 0) ctl[0] = 0;
  named_barrier(1, nthreads);
}

}  // namespace brawl
