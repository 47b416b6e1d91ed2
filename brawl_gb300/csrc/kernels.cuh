// kernels.cuh -- launch-side declarations shared by the kernel translation
// units and the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "chain_engine.cuh"

namespace brawl {

// Shared-memory layout of one chain's CTA, identical on host and device.
// The int32 region I holds the six axis tables, then F, then (when small
// enough) D.
struct SmemLayout {
  uint32_t mt, V, ents, sstart, I, lat, total;
  uint32_t tab_len[3];        // 2n + 2*kHalo per axis
  int32_t F_off, D_off;       // element offsets in I
  int32_t use_D;
};

__host__ __device__ inline uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

constexpr uint32_t kMaxDBytes = 12 * 1024;

__host__ __device__ inline SmemLayout smem_layout(const Geom& g, bool lattice_in_smem) {
  SmemLayout L;
  const uint32_t nsp = (uint32_t)g.ns + 1;
  const uint32_t nF = nsp * (uint32_t)g.nsh * nsp;
  const uint32_t nD = nsp * nsp * (uint32_t)g.nsh * nsp;
  L.mt = 0;
  L.V = align_up(L.mt + kMTN * 4, 16);
  L.ents = L.V + (uint32_t)(g.ns * g.ns * g.nsh) * 8;
  L.sstart = L.ents + (uint32_t)g.z * 4;
  L.I = align_up(L.sstart + (uint32_t)(g.nsh + 1) * 2, 16);
  L.tab_len[0] = 2 * (uint32_t)g.n1 + 2 * kHalo;
  L.tab_len[1] = 2 * (uint32_t)g.n2 + 2 * kHalo;
  L.tab_len[2] = 2 * (uint32_t)g.n3 + 2 * kHalo;
  const uint32_t ntab = 2 * (L.tab_len[0] + L.tab_len[1] + L.tab_len[2]);
  L.use_D = nD * 4 <= kMaxDBytes ? 1 : 0;
  L.F_off = (int32_t)ntab;
  L.D_off = (int32_t)(ntab + nF);
  const uint32_t nI = ntab + nF + (L.use_D ? nD : 0);
  L.lat = align_up(L.I + nI * 4, 16);
  L.total = lattice_in_smem ? align_up(L.lat + (uint32_t)g.n_sites, 16) : L.lat;
  return L;
}

// Builds the wrapping and identity axis tables (see AxisTables).
__device__ inline void build_axis_tables(const Geom& g, int32_t* tabs, const uint32_t* tab_len,
                                         int lane, AxisTables& T) {
  // tabs: the start of the int32 region I
  int32_t* base = tabs;
  const int n[3] = {g.n1, g.n2, g.n3};
  const int W[3] = {g.W1, g.W2, g.W3};
  for (int a = 0; a < 3; ++a) {
    const int len = (int)tab_len[a];
    int32_t* wrap = base;
    int32_t* ident = base + len;
    for (int i = lane; i < len; i += 32) {
      const int t = i - kHalo;
      int w = t % W[a];
      w = w < 0 ? w + W[a] : w;
      int vw, vi;
      const int ti = t < 0 ? 0 : (t >= 2 * n[a] ? 2 * n[a] - 1 : t);
      if (a == 0) {
        vw = w >> g.xs;
        vi = ti >> g.xs;
      } else if (a == 1) {
        vw = (w >> g.ys) * g.sy;
        vi = (ti >> g.ys) * g.sy;
      } else {
        vw = w * g.sz;
        vi = ti * g.sz;
      }
      wrap[i] = vw;
      ident[i] = vi;
    }
    if (a == 0) {
      T.tx[0] = wrap;
      T.tx[1] = ident;
    } else if (a == 1) {
      T.ty[0] = wrap;
      T.ty[1] = ident;
    } else {
      T.tz[0] = wrap;
      T.tz[1] = ident;
    }
    base += 2 * len;
  }
}

// Shared-memory layout of a chain staged with a halo (halo_engine.cuh).
struct HaloLayout {
  uint32_t mt, tbuf, ptab, ctab, V, ents, sstart, I, lat, total;
  int32_t F_off, D_off;
};

constexpr int kTbufWords = 2 * kMTN + kRingMirror;  // the ring and its mirror

__host__ __device__ inline HaloLayout halo_layout(const Geom& g, const HaloGeom& H) {
  HaloLayout L;
  const uint32_t nsp = (uint32_t)g.ns + 1;
  const uint32_t nF = nsp * (uint32_t)g.nsh * nsp;
  const uint32_t nD = nsp * nsp * (uint32_t)g.nsh * nsp;
  L.mt = 0;
  L.tbuf = align_up(kMTN * 4, 16);
  L.ptab = align_up(L.tbuf + kTbufWords * 4, 16);  // the site tables, one int32 per word each
  L.ctab = L.ptab + kTbufWords * 4;
  L.V = align_up(L.ctab + kTbufWords * 4, 16);
  L.ents = L.V + (uint32_t)(g.ns * g.ns * g.nsh) * 8;
  L.sstart = L.ents + (uint32_t)g.z * 4;
  L.I = align_up(L.sstart + (uint32_t)(g.nsh + 1) * 2, 16);
  L.F_off = 0;
  L.D_off = (int32_t)nF;
  L.lat = align_up(L.I + (nF + nD) * 4, 16);
  L.total = align_up(L.lat + (uint32_t)H.padded, 16);
  return L;
}

int lane_entries_for(int max_z);

// Sampling reductions of the annealing loop on the device (sampling.cu).
void launch_energy_accumulate(const double* d_e, double* d_sums, double* d_traj, int n, cudaStream_t s);
void launch_acceptance_snapshot(const unsigned long long* d_counters, unsigned long long* d_acc0, int n,
                                cudaStream_t s);
void launch_asro_finish(const unsigned long long* d_counts, const unsigned long long* d_mask, int n_class,
                        int ns, int wc, double* d_rho_out, double* d_rho_sum, cudaStream_t s);
void launch_temperature_stats(int n, const double* d_sums, const unsigned long long* d_counters,
                              const unsigned long long* d_acc0, const double* d_n_atoms, double n_save,
                              double sim_temp, double temp, double n_mc_real, int with_energies,
                              double* d_out, cudaStream_t s);
void launch_asro_stats(int n, int m, const double* d_rho_sum, double n_save, double* d_out, cudaStream_t s);

// Load the code of every kernel variant a translation unit launches (module
// loading is lazy by default; a launch that first loads code waits for the
// kernels already running on the device).
void preload_metropolis_kernels();
void preload_halo_kernels();
void preload_ns_kernels();
void preload_wl_kernels();
void preload_lattice_kernels();

// Metropolis swap trials for chains staged with a halo (fcc/bcc that fit).
// Speculative rounds of nc (2-4) trials per chain, nc(nc+1)/2 warps per CTA
// (metropolis_spec.cu); spec_static_smem is the static shared memory the
// kernel adds to smem_bytes.
void launch_metropolis_spec(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int max_z, int nc,
                            cudaStream_t stream);
uint32_t spec_static_smem(int nc);
// The halo chains: speculative rounds of nc trials when nc >= 2 and the
// slots fit beside the dynamic shared memory, the one-trial kernel otherwise.
// min_z/max_z: the smallest and largest neighbour count of the chains.
void launch_halo_chains(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int min_z, int max_z,
                        int nc, int max_optin, cudaStream_t stream);
void launch_metropolis_halo(const ChainJob* d_jobs, int n_jobs, uint32_t smem_bytes, int min_z,
                            int max_z, cudaStream_t stream);

// Metropolis swap trials, one warp (CTA) per chain; max_z is the largest
// neighbour count in the batch (it selects the unrolling of the fast tier).
void launch_metropolis(const ChainJob* d_jobs, int n_jobs, bool lattice_in_smem, bool use_D,
                       uint32_t smem_bytes, int max_z, cudaStream_t stream);

// initial_setup (src/initialise.F90:434-617) on the device, one warp per
// chain.  Per chain: counts[ns] species quotas, lo_w/hi_w[ns] the interval
// bounds in units of 2^-32 (w >= lo_w and w <= hi_w <=> lo <= u <= hi).
// ---------------------------------------------------------------------------
// Site energies in the reference's order: each shell sum starts from 0.0
// and adds V_ex(species, neighbour, shell) in list order; the shell sums are
// added left to right (src/bw_hamiltonian.f90:898-1262, 1712-1910,
// 2059-2106).
// ---------------------------------------------------------------------------
__device__ inline double site_energy_ref(const Geom& g, const int8_t* lat, const double* V,
                                  const uint32_t* ents, const int16_t* sstart, int x, int y,
                                  int z) {
  const int cs = lat[compact_index(g, x, y, z)];
  double total = 0.0;
  for (int sh = 0; sh < g.nsh; ++sh) {
    double e = 0.0;
    for (int k = sstart[sh]; k < sstart[sh + 1]; ++k) {
      int dx, dy, dz, shk;
      unpack_entry(ents[k], dx, dy, dz, shk);
      const int s = lat[neighbour_index(g, x, y, z, dx, dy, dz)];
      e = __dadd_rn(e, V[(cs - 1) + g.ns * ((s - 1) + g.ns * sh)]);
    }
    total = sh == 0 ? e : __dadd_rn(total, e);
  }
  return total;
}

// total_energy's ordered sum (src/bw_hamiltonian.f90:67-79): energy =
// energy + e(site) over the sites in order, then 0.5 * energy, for one warp.
// The warp loads 32 site energies at a time (the next 32 already in flight)
// and every lane runs the same ordered chain of adds on them through
// shuffles, so the chain waits on the adds, not on the loads.  Every lane
// returns the result.
__device__ inline double ordered_half_sum_warp(const double* __restrict__ e, int n, int lane) {
  double energy = 0.0;
  double v = lane < n ? e[lane] : 0.0;
  for (int base = 0; base < n; base += 32) {
    const int nxt = base + 32 + lane;
    const double v_next = nxt < n ? e[nxt] : 0.0;
    const int m = min(32, n - base);
    for (int k = 0; k < m; ++k) energy = __dadd_rn(energy, __shfl_sync(kFull, v, k));
    v = v_next;
  }
  return __dmul_rn(0.5, energy);
}

struct InitJob {
  int8_t* lat;
  uint32_t* rng;
  int32_t n_sites, ns;
  int64_t counts[kMaxSpecies];
  int64_t lo_w[kMaxSpecies];
  int64_t hi_w[kMaxSpecies];
  unsigned long long* counters;
  int32_t* status;
};
void launch_initial_setup(const InitJob* d_jobs, int n_jobs, cudaStream_t stream);

// The site-by-site draw loop of initial_setup for one configuration
// (src/initialise.F90:434-617), on the warp's stream (mt in shared memory at
// position pos); check is shared scratch of kMaxSpecies counters.  Every
// word of the stream is one draw: species l + 1 when it falls in the
// interval of species l whose count is below its quota (the last such l,
// as the reference's loop over l leaves it), else no species and the site
// draws again.  Accepted words fill the sites in order.
//
// The warp decides 32 consecutive words at once.  While no word in the
// batch falls in two intervals and no quota can fill inside the batch
// (check + the batch's words of that species <= count), every word's fate
// is known from the counts at the batch's start: the accepted words take
// the next sites in order (a ballot and a prefix count).  A batch where a
// quota fills, or a word sits on two intervals, is decided word by word.
// Returns false when a quota can never be met (guards against a corrupted
// job; the host validates counts).
__device__ inline bool initial_setup_warp(const InitJob& J, int8_t* lat, uint32_t* mt, int& pos,
                                          int64_t* check, unsigned long long& draws, int lane) {
  if (lane < kMaxSpecies) check[lane] = 0;
  __syncwarp();
  const int ns = J.ns;
  const int n_sites = J.n_sites;
  const unsigned long long limit = draws + (unsigned long long)n_sites * 4096ull + 1000000ull;
  const unsigned lt_mask = (1u << lane) - 1u;
  int site = 0;
  while (site < n_sites) {
    // the next n <= 32 words, none past the end of the current block
    const int avail = kMTN - pos;
    const int n = avail > 0 ? min(32, avail) : 32;
    const uint32_t w = mt_peek(mt, pos, n, lane);
    const int64_t wl = (int64_t)w;
    int cand = 0, hits = 0;
    if (lane < n)
      for (int l = 0; l < ns; ++l)
        if (wl >= J.lo_w[l] && wl <= J.hi_w[l]) {
          cand = l + 1;
          ++hits;
        }
    bool fast = !__any_sync(kFull, hits > 1);
    // a candidate whose quota is already full is a plain rejection; one
    // whose quota fills inside the batch needs the word-by-word pass
    bool open = false;
    if (cand > 0) open = check[cand - 1] < J.counts[cand - 1];
    unsigned acc = __ballot_sync(kFull, open);
    int need_mine = 0;  // lane l < ns: accepted words of species l + 1 in the batch
    for (int l = 0; l < ns; ++l) {
      const int c = __popc(__ballot_sync(kFull, open && cand == l + 1));
      if (lane == l) need_mine = c;
    }
    if (lane < ns && check[lane] + need_mine > J.counts[lane]) fast = false;
    fast = __all_sync(kFull, fast);
    int consumed = n;
    if (fast) {
      const int r = n_sites - site;
      if (__popc(acc) >= r) {
        // the configuration ends inside the batch: its r-th accepted word
        // is the last one consumed (the words after it are not drawn)
        unsigned m = acc;
        for (int k = 1; k < r; ++k) m &= m - 1u;
        const int last = __ffs(m) - 1;
        consumed = last + 1;
        acc &= (last == 31) ? 0xffffffffu : ((1u << (last + 1)) - 1u);
      }
      const bool mine = (acc >> lane) & 1u;
      if (mine) lat[site + __popc(acc & lt_mask)] = (int8_t)cand;
      int add = 0;
      for (int l = 0; l < ns; ++l) {
        const int c = __popc(__ballot_sync(kFull, mine && cand == l + 1));
        if (lane == l) add = c;
      }
      __syncwarp();
      if (lane < ns) check[lane] += add;
      site += __popc(acc);
    } else {
      for (int k = 0; k < n; ++k) {
        const int64_t wk = (int64_t)__shfl_sync(kFull, w, k);
        // every species whose interval holds the word and whose quota is
        // open takes the site in turn and uses up one of its quota (a word
        // on the boundary of two intervals uses up both); the last one keeps it
        int s = 0;
        unsigned taken = 0u;
        for (int l = 0; l < ns; ++l)
          if (wk >= J.lo_w[l] && wk <= J.hi_w[l] && check[l] < J.counts[l]) {
            s = l + 1;
            taken |= 1u << l;
          }
        __syncwarp();
        if (s > 0) {
          if (lane < ns && ((taken >> lane) & 1u)) check[lane] += 1;
          if (lane == 0) lat[site] = (int8_t)s;
          ++site;
          if (site == n_sites) {
            consumed = k + 1;
            __syncwarp();
            break;
          }
        }
        __syncwarp();
      }
    }
    __syncwarp();
    pos += consumed;
    draws += (unsigned long long)consumed;
    if (draws > limit) return false;
  }
  __syncwarp();
  return true;
}

// total_energy (src/bw_hamiltonian.f90:58-81): per-site FP64 energies in the
// reference's order, then the sequential sum over sites in z, y, x order.
struct EnergyJob {
  Geom g;
  const int8_t* lat;
  const double* V;
  const uint32_t* entries;
  const int16_t* shell_start;
  double* site_energy;        // n_sites scratch
  double* out;                // total energy
  int64_t site_offset;        // prefix over chains (for the grid-stride map)
};
void launch_total_energy(const EnergyJob* d_jobs, int n_jobs, int64_t total_sites,
                         cudaStream_t stream);
// Every job's compact lattice (n_sites bytes) copied from src[c].lat to
// dst[c].lat: the snapshot an energy on another stream reads while the
// chains move on.
void launch_lattice_snapshot(const EnergyJob* d_src, const EnergyJob* d_dst, int n_jobs, int max_sites,
                             cudaStream_t stream);

// Site energy of one site (nbr_energy), one thread.
void launch_site_energy(const EnergyJob* d_job, int x, int y, int z, double* out,
                        cudaStream_t stream);

// Conversions between the reference's full doubled grid config(1,2n1,2n2,2n3)
// (x fastest) and the compact occupied-site array.
void launch_pack(const Geom& g, const int8_t* d_grid, int8_t* d_lat, int32_t* d_status,
                 cudaStream_t stream);
void launch_unpack(const Geom& g, const int8_t* d_lat, int8_t* d_grid, cudaStream_t stream);

// The same for every chain of a batch at once: grids concatenated in chain
// order starting at grid_offset[c].
struct GridJob {
  Geom g;
  int8_t* lat;
  int64_t grid_offset;
  int32_t* status;
};
void launch_pack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells,
                       const int8_t* d_grids, cudaStream_t stream);
void launch_unpack_batch(const GridJob* d_jobs, int n_jobs, int64_t total_cells, int8_t* d_grids,
                         cudaStream_t stream);
// counts[offsets[c] + (s - 1) * n_sites + i] += 1 for chain c's site i of species s
void launch_alro_add(const GridJob* d_jobs, int n_jobs, double* d_counts, const int64_t* d_offsets,
                     cudaStream_t stream);

}  // namespace brawl
