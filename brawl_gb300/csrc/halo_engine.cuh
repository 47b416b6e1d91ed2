// halo_engine.cuh -- the fast per-trial machinery for fcc and bcc chains
// whose lattice fits in shared memory with a periodic halo.
//
// Lattice.  The compact lattice (Z, Y', X') = (z, y >> ys, x >> xs) is
// staged with a halo of (hz, hy, hx) cells on each side holding the periodic
// images, so every neighbour of a site is base(site) + delta[j] with no
// wrapping: delta depends only on the entry and on the site's parity (the
// x >> 1 of the compact layout).  A swap writes the two sites and their
// images (at most 8 copies each).
//
// Stream.  mt19937ar words are consumed from a ring of two tempered blocks
// (tbuf); a block is generated (twist + temper) when the consumer gets
// within a trial of the end of the generated words, so a trial reads its
// words with plain shared loads.  The state written back is the reference's
// (mt[624], mti): when consumption is still in the older block, that block's
// untempered words are recovered by inverting the tempering.
#pragma once

#include "chain_engine.cuh"

namespace brawl {


// ---------------------------------------------------------------------------
// tempered ring
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mt_untemper(uint32_t y) {
  // inverse of mt_temper, step by step from the last
  y ^= y >> 18;
  y ^= (y << 15) & 0xefc60000u;
  // y ^= (y << 7) & 0x9d2c5680: recover 7 bits at a time
  uint32_t t = y;
  t = y ^ ((t << 7) & 0x9d2c5680u);
  t = y ^ ((t << 7) & 0x9d2c5680u);
  t = y ^ ((t << 7) & 0x9d2c5680u);
  t = y ^ ((t << 7) & 0x9d2c5680u);
  y = t;
  // y ^= y >> 11
  t = y ^ (y >> 11);
  y = y ^ (t >> 11);
  return y;
}

// Ring of two tempered blocks in tbuf[0, 1248), plus a mirror of the first
// kRingMirror words at tbuf[1248, 1248 + kRingMirror) so the words of a
// trial (or of a round of speculated trials, or of a batch of redraws)
// never wrap.  `idx` is the
// ring slot of the next word, `avail` the generated words not yet consumed
// (0..1248), `next_half` the half the next generated block goes to; mt holds
// the newest generated block, untempered.
constexpr int kRing = 2 * kMTN;

struct Ring {
  int idx;
  int avail;
  int next_half;
};

// Twists mt in place and tempers the new block into the ring half next_half.
static __device__ __noinline__ void ring_generate(uint32_t* mt, uint32_t* tbuf, int next_half,
                                           int lane) {
  mt_twist_warp(mt, lane);
  uint32_t* dst = tbuf + next_half * kMTN;
  for (int i = lane; i < kMTN; i += 32) dst[i] = mt_temper(mt[i]);
  if (next_half == 0)
    for (int i = lane; i < kRingMirror; i += 32) tbuf[kRing + i] = mt_temper(mt[i]);
  __syncwarp();
}

// The block in mt is current with mti = pos0 (0..624): temper it into half 0.
__device__ __forceinline__ void ring_init(const uint32_t* mt, uint32_t* tbuf, int pos0, int lane,
                                          Ring& R) {
  for (int i = lane; i < kMTN; i += 32) tbuf[i] = mt_temper(mt[i]);
  for (int i = lane; i < kRingMirror; i += 32) tbuf[kRing + i] = mt_temper(mt[i]);
  R.idx = pos0;
  R.avail = kMTN - pos0;
  R.next_half = 1;
  __syncwarp();
}

// Makes n <= kRingMirror words available from R.idx.  A block is only generated when
// fewer than n remain, so the half it overwrites has been consumed.
__device__ __forceinline__ void ring_ensure(uint32_t* mt, uint32_t* tbuf, Ring& R, int n,
                                            int lane) {
  if (R.avail < n) {
    ring_generate(mt, tbuf, R.next_half, lane);
    R.avail += kMTN;
    R.next_half ^= 1;
  }
}

__device__ __forceinline__ void ring_consume(Ring& R, int n) {
  R.idx += n;
  R.idx = R.idx >= kRing ? R.idx - kRing : R.idx;
  R.avail -= n;
}

// Writes (mt, mti) in the reference's form.  If the next word lies in the
// block before the newest one, that block is recovered by untempering.
__device__ inline void ring_writeback(const uint32_t* mt, const uint32_t* tbuf, const Ring& R,
                                      uint32_t* out, int lane) {
  if (R.avail <= kMTN) {
    for (int i = lane; i < kMTN; i += 32) out[i] = mt[i];
    if (lane == 0) out[kMTN] = (uint32_t)(kMTN - R.avail);
  } else {
    const int older = R.next_half;  // the half after the newest is the older one
    for (int i = lane; i < kMTN; i += 32) out[i] = mt_untemper(tbuf[older * kMTN + i]);
    if (lane == 0) out[kMTN] = (uint32_t)(kRing - R.avail);
  }
}

// ---------------------------------------------------------------------------
// Site tables.  The site an fcc/bcc proposal draws from the three words at
// ring positions (p, p+1, p+2) does not depend on the lattice, so it is
// decoded for every position when the words are generated:
//   ptab[p] = padded index | parity << 30   (parity: bcc z & 1, fcc x & 1)
//   ctab[p] = x | y << 10 | z << 20          (doubled-grid coordinates)
// (entries kRing + k mirror entries k, like the words' mirror).  A trial then
// reads its sites with shared loads instead of decoding six words.  Entry p
// is written when the block holding word p + 2 is generated, so the words a
// trial may read (ring_ensure's n >= 6) always have their entries.
// ---------------------------------------------------------------------------
constexpr int32_t kPadMask = (1 << 30) - 1;

struct SiteDraw {
  uint32_t z2, n1, n2, x2;  // 2 n3, n1, n2, 2 n1
  int32_t origin, SZ, SY;
  int32_t bcc;
};

__device__ __forceinline__ SiteDraw make_site_draw(const Geom& g, const HaloGeom& H) {
  SiteDraw S;
  S.z2 = 2u * (uint32_t)g.n3;
  S.n1 = (uint32_t)g.n1;
  S.n2 = (uint32_t)g.n2;
  S.x2 = 2u * (uint32_t)g.n1;
  S.origin = H.origin;
  S.SZ = H.SZ;
  S.SY = H.SY;
  S.bcc = g.lattice == kBcc;
  return S;
}

// The site draw_site_halo gives for words (w0, w1, w2): its ptab and ctab
// entries.
__device__ __forceinline__ void site_entries(const SiteDraw& S, uint32_t w0, uint32_t w1,
                                             uint32_t w2, int32_t& pe, int32_t& ce) {
  const int z = (int)umulhi32(w0, S.z2);
  int x, y, Yc, Xc, par;
  if (S.bcc) {
    const int p = z & 1;
    Xc = (int)umulhi32(w1, S.n1);
    Yc = (int)umulhi32(w2, S.n2);
    x = 2 * Xc + p;
    y = 2 * Yc + p;
    par = p;
  } else {
    x = (int)umulhi32(w1, S.x2);
    y = 2 * (int)umulhi32(w2, S.n2) + ((x + z) & 1);
    Yc = y;
    Xc = x >> 1;
    par = x & 1;
  }
  pe = (S.origin + z * S.SZ + Yc * S.SY + Xc) | (par << 30);
  ce = x | (y << 10) | (z << 20);
}

__device__ __forceinline__ void site_coords(int32_t ce, int& x, int& y, int& z) {
  x = ce & 1023;
  y = (ce >> 10) & 1023;
  z = ce >> 20;
}

// Entries for positions [lo, hi) (hi <= kRing; words up to hi + 1 exist,
// through the mirror), then the tables' mirrors when position 0 was among
// them.
__device__ __forceinline__ void site_table_fill(const SiteDraw& S, const uint32_t* tbuf,
                                                int32_t* ptab, int32_t* ctab, int lo, int hi,
                                                int lane) {
  for (int p = lo + lane; p < hi; p += 32) {
    int32_t pe, ce;
    site_entries(S, tbuf[p], tbuf[p + 1], tbuf[p + 2], pe, ce);
    ptab[p] = pe;
    ctab[p] = ce;
  }
  __syncwarp();
  if (lo == 0)
    for (int i = lane; i < kRingMirror; i += 32) {
      ptab[kRing + i] = ptab[i];
      ctab[kRing + i] = ctab[i];
    }
  __syncwarp();
}

// ring_init plus the entries of every position whose three words are in
// the initial block.
__device__ __forceinline__ void ring_init_sites(const uint32_t* mt, uint32_t* tbuf, int32_t* ptab,
                                                int32_t* ctab, const SiteDraw& S, int pos0,
                                                int lane, Ring& R) {
  ring_init(mt, tbuf, pos0, lane, R);
  site_table_fill(S, tbuf, ptab, ctab, 0, kMTN - 2, lane);
}

// A new block into half h with its entries: the two positions before the
// block (their last words are its first) and the block's first 622.  Out of
// line: it runs once per 624 words, and the trial loop stays small.
static __device__ __noinline__ void ring_generate_sites(uint32_t* mt, uint32_t* tbuf,
                                                        int32_t* ptab, int32_t* ctab,
                                                        const SiteDraw S, int h, int lane) {
  ring_generate(mt, tbuf, h, lane);
  if (h == 0) {
    site_table_fill(S, tbuf, ptab, ctab, kRing - 2, kRing, lane);
    site_table_fill(S, tbuf, ptab, ctab, 0, kMTN - 2, lane);
  } else {
    site_table_fill(S, tbuf, ptab, ctab, kMTN - 2, kRing - 2, lane);
  }
}

// ring_ensure, keeping the site tables current.
__device__ __forceinline__ void ring_ensure_sites(uint32_t* mt, uint32_t* tbuf, int32_t* ptab,
                                                  int32_t* ctab, const SiteDraw& S, Ring& R,
                                                  int n, int lane) {
  if (R.avail < n) {
    ring_generate_sites(mt, tbuf, ptab, ctab, S, R.next_half, lane);
    R.avail += kMTN;
    R.next_half ^= 1;
  }
}

// ---------------------------------------------------------------------------
// halo lattice
// ---------------------------------------------------------------------------
__device__ __forceinline__ int halo_index(const HaloGeom& H, int Z, int Yp, int Xp) {
  return H.origin + Z * H.SZ + Yp * H.SY + Xp;
}

// Fills the padded lattice from the compact one (every padded cell reads its
// canonical cell).
__device__ inline void halo_fill(const Geom& g, const HaloGeom& H, const int8_t* lat_c,
                                 int8_t* lat_p, int lane, int stride = 32) {
  const int PX = H.NX + 2 * H.hx, PY = H.NY + 2 * H.hy, PZ = H.NZ + 2 * H.hz;
  const int total = PX * PY * PZ;
  for (int t = lane; t < total; t += stride) {
    const int px = t % PX, py = (t / PX) % PY, pz = t / (PX * PY);
    int X = px - H.hx, Y = py - H.hy, Z = pz - H.hz;
    X = X < 0 ? X + H.NX : (X >= H.NX ? X - H.NX : X);
    Y = Y < 0 ? Y + H.NY : (Y >= H.NY ? Y - H.NY : Y);
    Z = Z < 0 ? Z + H.NZ : (Z >= H.NZ ? Z - H.NZ : Z);
    lat_p[pz * H.SZ + py * H.SY + px] = lat_c[Z * g.sz + Y * g.sy + X];
  }
}

// Copies the interior back to the compact lattice.
__device__ inline void halo_store(const Geom& g, const HaloGeom& H, const int8_t* lat_p,
                                  int8_t* lat_c, int lane, int stride = 32) {
  for (int t = lane; t < g.n_sites; t += stride) {
    const int Z = t / g.sz, r = t - Z * g.sz, Y = r / g.sy, X = r - Y * g.sy;
    lat_c[t] = lat_p[halo_index(H, Z, Y, X)];
  }
}

// The padded cell that lane `lane` writes when the pair is swapped, or -1:
// lanes 8k..8k+7 take site k's canonical cell and its images (one
// combination of image axes each; at most 8 copies).  Lanes take different
// combinations, so every choice is a select, not a branch.
__device__ __forceinline__ int halo_image_shift(int c, int h, int N) {
  // the image shift of coordinate c on an axis with halo h, 0 when none
  return c < h ? N : (c >= N - h ? -N : 0);
}

__device__ __forceinline__ int halo_image_index(const HaloGeom& H, int lane, int Za, int Ya,
                                                int Xa, int Zb, int Yb, int Xb) {
  const bool b = lane >= 8;
  const int combo = lane & 7;
  const int Z = b ? Zb : Za, Y = b ? Yb : Ya, X = b ? Xb : Xa;
  const int sx = halo_image_shift(X, H.hx, H.NX);
  const int sy = halo_image_shift(Y, H.hy, H.NY);
  const int sz = halo_image_shift(Z, H.hz, H.NZ);
  const bool ux = combo & 1, uy = combo & 2, uz = combo & 4;
  const bool ok = lane < 16 && (!ux || sx != 0) && (!uy || sy != 0) && (!uz || sz != 0);
  const int idx = halo_index(H, Z + (uz ? sz : 0), Y + (uy ? sy : 0), X + (ux ? sx : 0));
  return ok ? idx : -1;
}

// draw_site for fcc and bcc, also giving the site's compact (Y', X') =
// (y >> ys, x >> 1) without going through the doubled coordinates.
__device__ __forceinline__ void draw_site_halo(const Geom& g, bool bcc, uint32_t w0, uint32_t w1,
                                               uint32_t w2, int& x, int& y, int& z, int& Yc,
                                               int& Xc) {
  z = (int)umulhi32(w0, 2u * g.n3);
  if (bcc) {
    const int p = z & 1;
    Xc = (int)umulhi32(w1, (uint32_t)g.n1);
    Yc = (int)umulhi32(w2, (uint32_t)g.n2);
    x = 2 * Xc + p;
    y = 2 * Yc + p;
  } else {
    x = (int)umulhi32(w1, 2u * g.n1);
    y = 2 * (int)umulhi32(w2, (uint32_t)g.n2) + ((x + z) & 1);
    Yc = y;
    Xc = x >> 1;
  }
}

// Conservative test that site b may be within the interaction range of site
// a (minimum-image displacement within the largest offsets on every axis).
__device__ __forceinline__ bool pair_near(const Geom& g, const HaloGeom& H, int ax, int ay,
                                          int az, int bx, int by, int bz) {
  // z first: most pairs are already apart there
  int dz = bz - az;
  const int W3 = 2 * g.n3;
  dz = dz > g.n3 ? dz - W3 : (dz < -g.n3 ? dz + W3 : dz);
  if (abs(dz) > H.dmz) return false;
  int dx = bx - ax, dy = by - ay;
  const int W1 = 2 * g.n1, W2 = 2 * g.n2;
  dx = dx > g.n1 ? dx - W1 : (dx < -g.n1 ? dx + W1 : dx);
  dy = dy > g.n2 ? dy - W2 : (dy < -g.n2 ? dy + W2 : dy);
  return abs(dx) <= H.dmx && abs(dy) <= H.dmy;
}

// pair_near without early exits (every lane evaluates all three axes, so
// it compiles to selects and can be issued ahead of the species test).
__device__ __forceinline__ bool pair_near_flat(const Geom& g, const HaloGeom& H, int ax, int ay,
                                               int az, int bx, int by, int bz) {
  int dz = bz - az, dx = bx - ax, dy = by - ay;
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3;
  dz = dz > g.n3 ? dz - W3 : (dz < -g.n3 ? dz + W3 : dz);
  dx = dx > g.n1 ? dx - W1 : (dx < -g.n1 ? dx + W1 : dx);
  dy = dy > g.n2 ? dy - W2 : (dy < -g.n2 ? dy + W2 : dy);
  return (abs(dz) <= H.dmz) & (abs(dx) <= H.dmx) & (abs(dy) <= H.dmy);
}

// Per-lane entry plan of the halo tier: for entry j of this lane's site, the
// padded-index delta for the site's parity (0/1) and shell * (ns+1).
template <int NJ>
struct HaloPlan {
  int32_t d0[NJ], d1[NJ];
  int32_t shp[NJ];
  uint32_t valid;
};

template <int NJ>
__device__ __forceinline__ void make_halo_plan(const Geom& g, const HaloGeom& H,
                                               const uint32_t* ents, int lane, HaloPlan<NJ>& P) {
  const int sub = lane & 15;
  P.valid = 0;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int k = sub + 16 * j;
    int dx = 0, dy = 0, dz = 0, sh = 0;
    if (k < g.z) {
      unpack_entry(ents[k], dx, dy, dz, sh);
      P.valid |= 1u << j;
    }
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      // parity: bcc the shared parity of x, y, z; fcc the parity of x
      const int ddx = (par + dx) >> 1;                       // x is always halved
      const int ddy = g.lattice == kBcc ? ((par + dy) >> 1) : dy;
      const int dd = dz * H.SZ + ddy * H.SY + ddx;
      if (par == 0) P.d0[j] = dd;
      else P.d1[j] = dd;
    }
    P.shp[j] = sh * (g.ns + 1);
  }
}

// Fixed-point swap delta for a pair that is not near: neighbours never
// include the partner or the site itself.  FULL: every lane entry is a
// neighbour (z = 16 NJ), so none is masked.
template <int NJ, bool FULL = false>
__device__ __forceinline__ int halo_delta(const Geom& g, int lat_off, int D_off_abs,
                                          const HaloPlan<NJ>& P, int base_a, int base_b, int par_a,
                                          int par_b, int sa, int sb, int lane) {
  extern __shared__ int32_t s_i32[];
  extern __shared__ int8_t s_i8[];
  const bool h = lane >= 16;
  const int base = lat_off + (h ? base_b : base_a);
  const bool par = h ? par_b : par_a;
  const int so = h ? sb : sa, sn = h ? sa : sb;
  const int nsp = g.ns + 1;
  const int rowD = D_off_abs + (so * nsp + sn) * g.nsh * nsp;
  int acc = 0;
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int s = s_i8[base + (par ? P.d1[j] : P.d0[j])];
    const int t = s_i32[rowD + P.shp[j] + s];
    acc += (FULL || ((P.valid >> j) & 1u)) ? t : 0;
  }
  return __reduce_add_sync(kFull, acc);
}

}  // namespace brawl
