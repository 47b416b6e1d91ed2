// chain_engine.cuh -- the per-chain, warp-cooperative pieces of BraWl's
// sampling hot path on sm_103a.
//
// One chain (replica, walker) is owned by one warp.  Its lattice lives as a
// compact uint8 array of occupied sites (shared memory when it fits), its
// mt19937ar state as 624 words in shared memory, and every trial follows the
// reference's sequential proposal order on that chain's own stream:
//
//   * site draws        -- *_random_site, src/random_site.f90:74-193
//                          (z, x, y for fcc/bcc; x, y, z for simple cubic),
//                          computed exactly with integer multiply-high
//   * swap energy       -- pair_energy before/after the swap,
//                          src/bw_hamiltonian.f90:99-114
//   * decision          -- monte_carlo_step_lattice, src/metropolis.F90:751-813
//
// Energies are decided in two tiers.  The fast tier sums the swap's energy
// change as exact int32 fixed point (V_ex scaled by 2^S and rounded), spread
// over the 32 lanes and reduced with one redux.sync; its distance from the
// reference's FP64 value is bounded by `band` quanta (fixed-point rounding
// plus the worst-case rounding of the reference's own FP64 sums).  Only when
// a decision falls inside that band does the warp recompute the four site
// energies in the reference's exact FP64 order (one lane per shell sum,
// neighbours added in list order, shells added left to right, then
// site1 + site2 and e_swapped - e_unswapped).
#pragma once

#include <cstdint>

#include "exact_fp.cuh"
#include "lattice_tables.h"

// Every kernel asks for the largest shared-memory carveout once, so kernels
// of all sizes from concurrent streams can share an SM without it being
// reconfigured between them.
#define BRAWL_CARVEOUT(...)                                                              \
  do {                                                                                   \
    static bool carveout_set_ = false;                                                   \
    if (!carveout_set_) {                                                                \
      cudaFuncSetAttribute(__VA_ARGS__, cudaFuncAttributePreferredSharedMemoryCarveout,  \
                           (int)cudaSharedmemCarveoutMaxShared);                         \
      carveout_set_ = true;                                                              \
    }                                                                                    \
  } while (0)

namespace brawl {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMTN = 624;
// Words mirrored past the end of a ring of tempered words (halo_engine.cuh),
// so that up to this many consecutive words can be read without wrapping.
constexpr int kRingMirror = 96;
// trials per speculative round of the halo Metropolis kernel (1: one trial
// at a time); brawl_batch_set_speculation overrides it per batch
constexpr int kDefaultSpeculation = 1;
constexpr int kMTM = 397;
constexpr int kMaxZ = 168;           // neighbour entries of bcc with 10 shells
constexpr int kMaxLaneEntries = 11;  // ceil(2 * kMaxZ / 32)
constexpr int kMaxSpecies = 15;      // species codes 1..15 (int8 storage)

enum Counter : int {
  kCntTrials = 0,    // monte_carlo_step calls (or WL/NS steps)
  kCntEvaluated,     // trials whose two species differed
  kCntDraws,         // 32-bit words consumed from the chain's stream
  kCntAccepted,      // accept == 1
  kCntExpTests,      // trials that drew the acceptance uniform
  kCntExactPath,     // trials decided with the FP64 reference-order sums
  kCntExpFp64,       // exp/log decisions that needed the FP64 libm value
  kCntExpCr,         // ... and the double-double value
  kNumCounters
};

enum Status : int {
  kStatusOk = 0,
  kStatusRngInvariant = 1,   // stream position left its block (internal error)
  kStatusBadSpecies = 2,     // a species code outside 1..ns was met
  kStatusWalkerOutsideWindow = 3,  // a Wang-Landau walker's energy left its window
  kStatusBandViolated = 4,   // an exact value fell outside its fixed-point bound (internal error)
};

struct Geom {
  int32_t lattice, n1, n2, n3;
  int32_t nsh, ns, n_sites, z;
  int32_t sy, sz, xs, ys;     // compact index: z*sz + (y>>ys)*sy + (x>>xs)
  int32_t W1, W2, W3;         // neighbour wrap modulus per axis
  int32_t fast_wrap;          // one conditional add/sub wraps every offset
  int32_t nbr_k;              // nearest-neighbour count (6/8/12)
  int32_t pad;
};

// Halo layout of an fcc/bcc lattice staged in shared memory (see
// halo_engine.cuh).
struct HaloGeom {
  int32_t NX, NY, NZ;     // compact extents
  int32_t hx, hy, hz;     // halo widths
  int32_t SY, SZ;         // padded strides (x stride 1)
  int32_t padded;         // padded byte count
  int32_t origin;         // hz*SZ + hy*SY + hx
  int32_t dmx, dmy, dmz;  // largest |offset| component per axis (doubled grid)
  int32_t pad;
};

// One chain's work order for a launch.  Plain data, shared with the host.
struct ChainJob {
  Geom g;
  HaloGeom hg;
  int32_t nbr_swap;
  int32_t band;               // decision band of the fixed-point tier, quanta
  double beta;
  float beta_q;               // beta * 2^-S (float)
  float beta_band;            // beta * band * 2^-S, rounded up (float)
  float beta_q_l2;            // beta * 2^-S * log2(e) (float)
  int32_t halo;               // 1: staged with a halo (halo kernel)
  int64_t n_trials;
  int8_t* lat;                // compact species array, n_sites bytes
  uint32_t* rng;              // mt[624], then the stream position
  const double* V;            // V_ex(a, b, shell), a fastest, ns*ns*nsh
  const int32_t* F;           // fixed-point F then D tables (see fixed_delta)
  const uint32_t* entries;    // z packed neighbour entries (dx,dy,dz,shell)
  const int16_t* shell_start; // nsh + 1 entry offsets
  unsigned long long* counters;
  int32_t* status;
  unsigned long long* t_ns;   // when set: the CTA's device time (ns) is written here
};

// Device clock in ns (%globaltimer), for the per-chain timings a scheduler
// uses to size the next launch's work.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------------------
// mt19937ar (src/mt19937ar.c:82-125), warp-cooperative
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

__device__ __forceinline__ uint32_t mt_mix(uint32_t a, uint32_t b, uint32_t c) {
  // c ^ (y >> 1) ^ mag01[y & 1] with y = (a & UPPER) | (b & LOWER)
  uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  return c ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// Regenerates the 624-word block in place with the whole warp, in three
// phases that respect the recurrence's dependencies: words [0,227) read
// only old words, [227,454) read new words of the first phase, and
// [454,624) read new words of the second phase (word 623 also reads the new
// word 0, as the reference's last step does).  Each phase reads all of its
// inputs before any lane writes.
static __device__ __noinline__ void mt_twist_warp(uint32_t* mt, int lane) {
  const int bounds[4] = {0, kMTN - kMTM, 2 * (kMTN - kMTM), kMTN};
#pragma unroll
  for (int ph = 0; ph < 3; ++ph) {
    const int lo = bounds[ph], hi = bounds[ph + 1];
    uint32_t nv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int k = lo + lane + 32 * i;
      nv[i] = 0;
      if (k < hi) {
        int k1 = k + 1 == kMTN ? 0 : k + 1;
        int km = k + kMTM;
        km = km >= kMTN ? km - kMTN : km;
        nv[i] = mt_mix(mt[k], mt[k1], mt[km]);
      }
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int k = lo + lane + 32 * i;
      if (k < hi) mt[k] = nv[i];
    }
    __syncwarp();
  }
}

// Makes n words (n <= 32) available at positions pos..pos+n-1 and returns
// word pos+lane in lanes < n.  When fewer than n words remain in the block
// the remaining ones are captured first, the block is regenerated and pos
// becomes negative (the captured words sit at negative positions).  The
// caller must then consume at least the captured words, which holds for
// every caller: a trial never consumes fewer than n-1 of n peeked words and
// a block is only regenerated when at most n-1 remain.
__device__ __forceinline__ uint32_t mt_peek(uint32_t* mt, int& pos, int n, int lane) {
  int avail = kMTN - pos;
  uint32_t w = 0;
  if (avail >= n) {
    if (lane < n) w = mt_temper(mt[pos + lane]);
  } else {
    if (lane < avail) w = mt_temper(mt[pos + lane]);
    __syncwarp();
    mt_twist_warp(mt, lane);
    if (lane >= avail && lane < n) w = mt_temper(mt[lane - avail]);
    pos -= kMTN;
  }
  return w;
}

// ---------------------------------------------------------------------------
// lattice addressing
// ---------------------------------------------------------------------------
__device__ __forceinline__ int compact_index(const Geom& g, int x, int y, int z) {
  return z * g.sz + (y >> g.ys) * g.sy + (x >> g.xs);
}

// inverse of compact_index
__device__ __forceinline__ void decode_site(const Geom& g, int idx, int& x, int& y, int& z) {
  if (g.lattice == kBcc) {
    z = idx / g.sz;
    int r = idx - z * g.sz;
    int yh = r / g.sy, xh = r - yh * g.sy;
    int p = z & 1;
    y = 2 * yh + p;
    x = 2 * xh + p;
  } else if (g.lattice == kFcc) {
    z = idx / g.sz;
    int r = idx - z * g.sz;
    y = r / g.sy;
    int xh = r - y * g.sy;
    x = 2 * xh + ((y + z) & 1);
  } else {
    z = idx / g.sz;
    int r = idx - z * g.sz;
    y = r / g.sy;
    x = r - y * g.sy;
  }
}

__device__ __forceinline__ int wrap_fast(int c, int W) {
  c = c < 0 ? c + W : c;
  return c >= W ? c - W : c;
}

// General rule: an axis with a zero offset keeps the site's own index (the
// reference uses site_i directly there), otherwise modulo(i + d, W).
__device__ __forceinline__ int wrap_general(int c, int d, int W) {
  if (d == 0) return c;
  int t = (c + d) % W;
  return t < 0 ? t + W : t;
}

__device__ __forceinline__ int neighbour_index(const Geom& g, int x, int y, int z, int dx,
                                               int dy, int dz) {
  int nx, ny, nz;
  if (g.fast_wrap) {
    nx = wrap_fast(x + dx, g.W1);
    ny = wrap_fast(y + dy, g.W2);
    nz = wrap_fast(z + dz, g.W3);
  } else {
    nx = wrap_general(x, dx, g.W1);
    ny = wrap_general(y, dy, g.W2);
    nz = wrap_general(z, dz, g.W3);
  }
  return compact_index(g, nx, ny, nz);
}

__device__ __forceinline__ uint32_t umulhi32(uint32_t w, uint32_t k) { return __umulhi(w, k); }

// floor(u * k) for u = w * 2^-32 and small k is exactly (w * k) >> 32.
__device__ __forceinline__ void draw_site(const Geom& g, uint32_t w0, uint32_t w1, uint32_t w2,
                                          int& x, int& y, int& z) {
  if (g.lattice == kBcc) {
    z = (int)umulhi32(w0, 2u * g.n3);
    int p = z & 1;
    x = 2 * (int)umulhi32(w1, (uint32_t)g.n1) + p;
    y = 2 * (int)umulhi32(w2, (uint32_t)g.n2) + p;
  } else if (g.lattice == kFcc) {
    z = (int)umulhi32(w0, 2u * g.n3);
    x = (int)umulhi32(w1, 2u * g.n1);
    y = 2 * (int)umulhi32(w2, (uint32_t)g.n2) + ((x + z) & 1);
  } else {
    x = (int)umulhi32(w0, 2u * g.n1);
    y = (int)umulhi32(w1, 2u * g.n2);
    z = (int)umulhi32(w2, 2u * g.n3);
  }
}

// Nearest-neighbour vectors of the nbr_swap proposals (the reference's
// sc_nbrs, bcc_nbrs and fcc_nbrs, src/random_site.f90:29-61), by lattice code.
static __constant__ int8_t cNbrSwap[3][12][3] = {
    {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 0, -1}, {0, -1, 0}, {-1, 0, 0}},
    {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1},
     {-1, -1, -1}},
    {{0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {1, 1, 0}, {1, -1, 0}, {1, 0, 1},
     {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0}, {-1, 0, 1}, {-1, 0, -1}}};

// Nearest neighbour chosen by one draw, n = floor(k*u)
// (src/random_site.f90:97-225); wraps on the doubled grid for every lattice.
__device__ __forceinline__ void draw_nbr(const Geom& g, uint32_t w, int x, int y, int z,
                                         int& nx, int& ny, int& nz) {
  const int k = (int)umulhi32(w, (uint32_t)g.nbr_k);
  const int8_t* v = cNbrSwap[g.lattice][k];
  nx = wrap_general(x, v[0], 2 * g.n1);
  ny = wrap_general(y, v[1], 2 * g.n2);
  nz = wrap_general(z, v[2], 2 * g.n3);
}

__device__ __forceinline__ void unpack_entry(uint32_t e, int& dx, int& dy, int& dz, int& sh) {
  dx = (int)(int8_t)(e & 0xffu);
  dy = (int)(int8_t)((e >> 8) & 0xffu);
  dz = (int)(int8_t)((e >> 16) & 0xffu);
  sh = (int)(e >> 24);
}

struct SitePair {
  int ax, ay, az, ai;  // site 1 (rdm1)
  int bx, by, bz, bi;  // site 2 (rdm2)
  int sa, sb;          // species before the swap
};

// ---------------------------------------------------------------------------
// Fast tier: exact fixed-point energy change of swapping the two sites.
//
// Lanes 0-15 work on site 1 and lanes 16-31 on site 2; lane l owns the
// site's neighbour entries (l & 15) + 16 j.  Neighbour addresses come from
// three small per-axis tables in shared memory that map an unwrapped
// coordinate t in [-kHalo, 2n + kHalo) straight to its wrapped contribution
// to the compact index, so one neighbour costs three table loads and two
// adds whatever the lattice and however far it wraps.  (For simple cubic an
// axis with a zero offset keeps the site's own index, which the reference's
// modulo-n wrap does not; those entries read identity tables instead.)
// ---------------------------------------------------------------------------
constexpr int kHalo = 6;  // every neighbour offset component is within +-5

struct AxisTables {
  const int32_t* tx[2];  // [0] wrapping, [1] identity (simple-cubic zero offsets)
  const int32_t* ty[2];
  const int32_t* tz[2];
};

// Fixed-point tables of the fast tier, in one int32 region of shared memory
// (all indices below are element offsets into it):
//   F[(a * nsh + shell) * (ns+1) + b]        = round(V_ex(a, b, shell) * 2^S)
//   D[((so * (ns+1) + sn) * nsh + shell) * (ns+1) + b]
//                                            = F(sn, b, shell) - F(so, b, shell)
// D is the change of one neighbour term when its centre changes from so to
// sn; only the partner site (whose own species changes too) needs F.
template <int NJ>
struct LanePlan {
  int32_t ax[NJ], ay[NJ], az[NJ];  // element offsets of the entry's axis-table slot
  int32_t shp[NJ];                 // shell * (ns + 1)
  uint32_t valid;                  // bit j: entry j exists
};

template <int NJ>
__device__ __forceinline__ void make_lane_plan(const Geom& g, const uint32_t* ents,
                                               const int32_t* tabs_base, const AxisTables& T,
                                               int lane, LanePlan<NJ>& P) {
  const int sub = lane & 15;
  const int nsp = g.ns + 1;
  P.valid = 0;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int k = sub + 16 * j;
    int dx = 0, dy = 0, dz = 0, sh = 0;
    if (k < g.z) {
      unpack_entry(ents[k], dx, dy, dz, sh);
      P.valid |= 1u << j;
    }
    const bool sc = g.lattice == kSimpleCubic;
    const int ix = sc && dx == 0 ? 1 : 0;
    const int iy = sc && dy == 0 ? 1 : 0;
    const int iz = sc && dz == 0 ? 1 : 0;
    P.ax[j] = (int32_t)(T.tx[ix] - tabs_base) + dx + kHalo;
    P.ay[j] = (int32_t)(T.ty[iy] - tabs_base) + dy + kHalo;
    P.az[j] = (int32_t)(T.tz[iz] - tabs_base) + dz + kHalo;
    P.shp[j] = sh * nsp;
  }
}

// Sum over this lane's entries of the change of its neighbour terms; the
// warp total (returned in every lane) is the fixed-point swap delta.
// Shared memory is addressed through the dynamic shared-memory symbols
// themselves (element offsets, not pointers), so every access is a plain
// 32-bit shared load the compiler can schedule freely.  I_off is the start
// of the int32 region (axis tables, F, D) in int32 units; lat_off the byte
// offset of the staged lattice (used when kSmemLat).
//
// This tier assumes neither site is a neighbour of the other (nor of
// itself): `near` returns whether any lane met the partner, and the caller
// then recomputes the trial with fixed_delta_general.
template <int NJ, bool kSmemLat, bool kUseD>
__device__ __forceinline__ int fixed_delta(const Geom& g, const int8_t* lat_g, int lat_off,
                                           int I_off, int F_off, int D_off,
                                           const LanePlan<NJ>& P, const SitePair& p, int lane,
                                           bool& near) {
  extern __shared__ int32_t s_i32[];
  extern __shared__ int8_t s_i8[];
  const bool h = lane >= 16;
  const int cx = h ? p.bx : p.ax, cy = h ? p.by : p.ay, cz = h ? p.bz : p.az;
  const int other = h ? p.ai : p.bi;
  const int so = h ? p.sb : p.sa, sn = h ? p.sa : p.sb;
  const int nsp = g.ns + 1;
  const int rowD = I_off + D_off + (so * nsp + sn) * g.nsh * nsp;
  const int rowN = I_off + F_off + sn * g.nsh * nsp;
  const int rowO = I_off + F_off + so * g.nsh * nsp;
  const int bx = I_off + cx, by = I_off + cy, bz = I_off + cz;
  int acc = 0;
  bool hit = false;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int ni = s_i32[P.ax[j] + bx] + s_i32[P.ay[j] + by] + s_i32[P.az[j] + bz];
    const int s_before = kSmemLat ? (int)s_i8[lat_off + ni] : (int)lat_g[ni];
    const int t = kUseD ? s_i32[rowD + P.shp[j] + s_before]
                        : s_i32[rowN + P.shp[j] + s_before] - s_i32[rowO + P.shp[j] + s_before];
    hit |= ni == other;
    acc += ((P.valid >> j) & 1u) ? t : 0;
  }
  near = __any_sync(kFull, hit);
  return __reduce_add_sync(kFull, acc);
}

// The same sum for any pair, including neighbouring sites and sites that
// are their own neighbours on tiny lattices (the partner's term uses its new
// species, a site's own term its new species).  Out of line and rebuilt
// from the entry table so the hot loop's registers stay where they are.
// tl0..tl2 are the axis-table lengths (the tables sit at the start of I).
template <bool kSmemLat>
__device__ __noinline__ int fixed_delta_general(int lattice, int ns, int nsh, int z,
                                                const int8_t* lat_g, int lat_off,
                                                int I_off, int F_off, int ents_off, int tl0,
                                                int tl1, int tl2, int ax, int ay, int az, int ai,
                                                int bx_, int by_, int bz_, int bi, int sa, int sb,
                                                int lane) {
  extern __shared__ int32_t s_i32[];
  extern __shared__ int8_t s_i8[];
  extern __shared__ uint32_t s_u32[];
  const bool h = lane >= 16;
  const int cx = h ? bx_ : ax, cy = h ? by_ : ay, cz = h ? bz_ : az;
  const int own = h ? bi : ai, other = h ? ai : bi;
  const int so = h ? sb : sa, sn = h ? sa : sb;
  const int nsp = ns + 1;
  const int rowN = I_off + F_off + sn * nsh * nsp;
  const int rowO = I_off + F_off + so * nsh * nsp;
  const bool sc = lattice == kSimpleCubic;
  const int xw = I_off, xi = I_off + tl0;
  const int yw = I_off + 2 * tl0, yi = yw + tl1;
  const int zw = I_off + 2 * (tl0 + tl1), zi = zw + tl2;
  int acc = 0;
  for (int k = lane & 15; k < z; k += 16) {
    int dx, dy, dz, sh;
    unpack_entry(s_u32[ents_off / 4 + k], dx, dy, dz, sh);
    const int tx = (sc && dx == 0) ? xi : xw;
    const int ty = (sc && dy == 0) ? yi : yw;
    const int tz = (sc && dz == 0) ? zi : zw;
    const int ni = s_i32[tx + cx + dx + kHalo] + s_i32[ty + cy + dy + kHalo] +
                   s_i32[tz + cz + dz + kHalo];
    const int s_before = kSmemLat ? (int)s_i8[lat_off + ni] : (int)lat_g[ni];
    const int s_after = ni == other ? so : (ni == own ? sn : s_before);
    acc += s_i32[rowN + sh * nsp + s_after] - s_i32[rowO + sh * nsp + s_before];
  }
  return __reduce_add_sync(kFull, acc);
}

// ---------------------------------------------------------------------------
// Exact tier: the reference's FP64 pair energies before and after the swap.
// Chain c in [0, 4*nsh): evaluation c / nsh (0: site 1 before, 1: site 2
// before, 2: site 1 after, 3: site 2 after), shell c % nsh.
// ---------------------------------------------------------------------------
// Lattice accessors: species of canonical compact site i.
struct CompactLat {
  const int8_t* p;
  __device__ __forceinline__ int operator()(int i) const { return p[i]; }
};

// The pair energies from the (evaluation, shell) partial sums, sum c = ev
// * nsh + sh in lane c of part[0] (c < 32) or lane c - 32 of part[1]: lane
// ev < 4 adds the shell sums of evaluation ev in shell order (site 1
// before, site 2 before, site 1 after, site 2 after; nbr_energy's shell 1 +
// shell 2 + ...), all four at once, then e_un = e(site 1) + e(site 2)
// before and e_sw the same after (pair_energy).  Every lane returns both.
__device__ __forceinline__ void combine_pair_energies(const double part[2], int nsh, int lane, double& e_un,
                                                      double& e_sw) {
  const int ev = lane & 3;
  double acc = 0.0;
  for (int sh = 0; sh < nsh; ++sh) {
    const int c = ev * nsh + sh;
    const double v0 = __shfl_sync(kFull, part[0], c & 31);
    const double v1 = __shfl_sync(kFull, part[1], c & 31);
    const double v = c < 32 ? v0 : v1;
    acc = sh == 0 ? v : __dadd_rn(acc, v);
  }
  // lane 0: e(site 1 before) + e(site 2 before); lane 2: the same after
  const double pair = __dadd_rn(acc, __shfl_down_sync(kFull, acc, 1));
  e_un = __shfl_sync(kFull, pair, 0);
  e_sw = __shfl_sync(kFull, pair, 2);
}

template <class Lat>
__device__ inline void exact_pair_energies(const Geom& g, const Lat& lat, const double* V,
                                           const uint32_t* ents, const int16_t* sstart,
                                           const SitePair& p, int lane, double& e_un,
                                           double& e_sw) {
  const int nsh = g.nsh, ns = g.ns;
  const int nc = 4 * nsh;
  double part[2] = {0.0, 0.0};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int c = lane + 32 * r;
    if (c < nc) {
      const int ev = c / nsh, sh = c - ev * nsh;
      const bool on2 = ev & 1, after = ev >= 2;
      const int cx = on2 ? p.bx : p.ax, cy = on2 ? p.by : p.ay, cz = on2 ? p.bz : p.az;
      const int own = on2 ? p.bi : p.ai, other = on2 ? p.ai : p.bi;
      const int s_own_before = on2 ? p.sb : p.sa;
      const int s_own_after = on2 ? p.sa : p.sb;
      const int cs = after ? s_own_after : s_own_before;
      double sum = 0.0;
      for (int k = sstart[sh]; k < sstart[sh + 1]; ++k) {
        int dx, dy, dz, shk;
        unpack_entry(ents[k], dx, dy, dz, shk);
        const int ni = neighbour_index(g, cx, cy, cz, dx, dy, dz);
        int s = lat(ni);
        if (after) {
          if (ni == other) s = s_own_before;        // the partner now holds our old species
          else if (ni == own) s = s_own_after;
        }
        sum = __dadd_rn(sum, V[(cs - 1) + ns * ((s - 1) + ns * sh)]);
      }
      part[r] = sum;
    }
  }
  combine_pair_energies(part, nsh, lane, e_un, e_sw);
}

// The same sums with the terms staged first: every (evaluation, neighbour)
// term V(species, neighbour species, shell) is looked up in parallel into
// vbuf (4 * z doubles of shared memory), then each (evaluation, shell) chain
// adds its terms in list order from 0.0, so the chain of dependent FP64 adds
// is the only latency left.  Same values, same order: identical results.
template <class Lat>
__device__ inline void exact_pair_energies_staged(const Geom& g, const Lat& lat, const double* V,
                                                  const uint32_t* ents, const int16_t* sstart,
                                                  const SitePair& p, int lane, double& e_un,
                                                  double& e_sw, double* vbuf) {
  const int z = g.z, nsh = g.nsh, ns = g.ns;
#pragma unroll 1
  for (int ev = 0; ev < 4; ++ev) {
    const bool on2 = ev & 1, after = ev >= 2;
    const int cx = on2 ? p.bx : p.ax, cy = on2 ? p.by : p.ay, cz = on2 ? p.bz : p.az;
    const int own = on2 ? p.bi : p.ai, other = on2 ? p.ai : p.bi;
    const int s_own_before = on2 ? p.sb : p.sa;
    const int s_own_after = on2 ? p.sa : p.sb;
    const int cs = after ? s_own_after : s_own_before;
    for (int k = lane; k < z; k += 32) {
      int dx, dy, dz, sh;
      unpack_entry(ents[k], dx, dy, dz, sh);
      const int ni = neighbour_index(g, cx, cy, cz, dx, dy, dz);
      int s = lat(ni);
      if (after) {
        if (ni == other) s = s_own_before;        // the partner now holds our old species
        else if (ni == own) s = s_own_after;
      }
      vbuf[ev * z + k] = V[(cs - 1) + ns * ((s - 1) + ns * sh)];
    }
  }
  __syncwarp();
  const int nc = 4 * nsh;
  double part[2] = {0.0, 0.0};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int c = lane + 32 * r;
    if (c < nc) {
      const int ev = c / nsh, sh = c - ev * nsh;
      const double* t = vbuf + ev * z + sstart[sh];
      const int len = sstart[sh + 1] - sstart[sh];
      double sum = 0.0;
      // four terms loaded ahead of their adds, so the loads of the next
      // group overlap the dependent adds of this one
      int k = 0;
      for (; k + 4 <= len; k += 4) {
        const double v0 = t[k], v1 = t[k + 1], v2 = t[k + 2], v3 = t[k + 3];
        sum = __dadd_rn(sum, v0);
        sum = __dadd_rn(sum, v1);
        sum = __dadd_rn(sum, v2);
        sum = __dadd_rn(sum, v3);
      }
      for (; k < len; ++k) sum = __dadd_rn(sum, t[k]);
      part[r] = sum;
    }
  }
  combine_pair_energies(part, nsh, lane, e_un, e_sw);
  __syncwarp();  // vbuf is reused by the next call
}

// Fixed-point swap delta for any pair, from canonical neighbour indices
// (lanes 0-15 site 1, 16-31 site 2).
__device__ __forceinline__ int compact_fixed_delta(const Geom& g, const int8_t* lat, const int32_t* F,
                                              const uint32_t* ents, const SitePair& p, int lane) {
  const bool h = lane >= 16;
  const int cx = h ? p.bx : p.ax, cy = h ? p.by : p.ay, cz = h ? p.bz : p.az;
  const int own = h ? p.bi : p.ai, other = h ? p.ai : p.bi;
  const int so = h ? p.sb : p.sa, sn = h ? p.sa : p.sb;
  const int nsp = g.ns + 1;
  const int rowN = sn * g.nsh * nsp, rowO = so * g.nsh * nsp;
  int acc = 0;
  for (int k = lane & 15; k < g.z; k += 16) {
    int dx, dy, dz, sh;
    unpack_entry(ents[k], dx, dy, dz, sh);
    const int ni = neighbour_index(g, cx, cy, cz, dx, dy, dz);
    const int sb = lat[ni];
    const int sa = ni == other ? so : (ni == own ? sn : sb);
    acc += F[rowN + sh * nsp + sa] - F[rowO + sh * nsp + sb];
  }
  return __reduce_add_sync(kFull, acc);
}

// FP32 filter of u < exp(-beta*dE) for a fixed-point dE > band.
// Returns 1 accept, 0 reject, -1 undecided.
__device__ __forceinline__ int fast_exp_decision(const ChainJob& J, int dE, uint32_t w) {
  float xf = -__fmul_rn(J.beta_q, __int2float_rn(dE));
  float D = fabsf(xf) * 2.0e-7f + J.beta_band * 1.0001f;
  float M = 1.1f * D + 7.0e-7f;
  if (!(M < 0.01f)) return -1;
  if (xf < -40.0f) return w != 0u ? 0 : -1;
  float thr = __fmul_rn(expf(xf), 4294967296.0f);
  float wf = __uint2float_rn(w);
  if (wf < __fmul_rn(thr, 1.0f - M)) return 1;
  if (wf > __fmul_rn(thr, 1.0f + M)) return 0;
  return -1;
}

// The base-2 filter below with the hardware 2^x (ex2.approx, whose error is
// far inside the 4e-6 relative allowed for it here) and the per-chain part of
// the margin taken once: c0 = 1.01 beta_band + 4.5e-6 when that is under
// 0.0099, else +inf (every test undecided).  Only x2 in [-57.5, 0] is
// decided with 2^x2; below, u = w 2^-32 >= 2^-32 is above 2^x2 for w > 0.
__device__ __forceinline__ float exp2_filter_c0(float beta_band) {
  const float c0 = beta_band * 1.01f + 4.5e-6f;
  return c0 < 0.0099f ? c0 : INFINITY;
}

__device__ __forceinline__ int fast_ex2_decision(float nbql2, float c0, int dE, uint32_t w) {
  const float x2 = __fmul_rn(nbql2, __int2float_rn(dE));
  if (!(x2 >= -57.5f && x2 <= 0.0f)) return (x2 < -57.5f && w != 0u && c0 < 1.0f) ? 0 : -1;
  const float M = __fmaf_rn(-x2, 1.5e-7f, c0);
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x2));
  const float thr = __fmul_rn(e, 4294967296.0f);
  const float wf = __uint2float_rn(w);
  if (wf < __fmul_rn(thr, 1.0f - M)) return 1;
  if (wf > __fmul_rn(thr, 1.0f + M)) return 0;
  return -1;
}

// The same filter in the base-2 domain: x2 = -beta*q*log2(e)*dE, 2^x2 with
// exp2f (<= 2 ulp).  The argument's float rounding (3 roundings, relative
// 1.8e-7 of |x2|, i.e. 1.25e-7 |x2| relative on 2^x2), the band term and the
// libm's own error are covered by M.
__device__ __forceinline__ int fast_exp2_decision(float beta_q_l2, float beta_band, int dE,
                                                  uint32_t w) {
  const float x2 = -__fmul_rn(beta_q_l2, __int2float_rn(dE));
  const float M = fabsf(x2) * 1.5e-7f + beta_band * 1.01f + 8.0e-7f;
  if (!(M < 0.01f)) return -1;
  if (x2 < -57.5f) return w != 0u ? 0 : -1;
  const float thr = __fmul_rn(exp2f(x2), 4294967296.0f);
  const float wf = __uint2float_rn(w);
  if (wf < __fmul_rn(thr, 1.0f - M)) return 1;
  if (wf > __fmul_rn(thr, 1.0f + M)) return 0;
  return -1;
}

}  // namespace brawl
