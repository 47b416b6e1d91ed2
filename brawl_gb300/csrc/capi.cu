// capi.cu -- the C ABI declared in include/brawl_gpu.h.
//
// A brawl_batch owns one device arena holding, per chain, the compact
// lattice, the mt19937ar block, V_ex, its fixed-point image and the neighbour
// entries, so a chain's whole state stays resident between calls.  A
// brawl_ctx is a batch of one chain.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/brawl_gpu.h"
#include "api_internal.h"
#include "asro.cuh"
#include "kernels.cuh"

using namespace brawl;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(x)                                                                   \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess) {                                                          \
      return fail(e_ == cudaErrorMemoryAllocation ? BRAWL_ENOMEM : BRAWL_ECUDA,       \
                  std::string(#x) + ": " + cudaGetErrorString(e_));                   \
    }                                                                                 \
  } while (0)

// Device memory of the objects is stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the object's own stream): creating and destroying an
// object never waits for kernels of other streams, so a serving loop keeps
// other jobs' work in flight while objects come and go.
// Objects' own streams (set-up, read-back, single calls) run at the
// device's highest priority: a serving loop keeps long rounds of batched
// kernels queued on low-priority streams, and the short work of admitting
// or finishing a job should not wait behind them.
inline cudaError_t object_stream(cudaStream_t* s) {
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, hi);
}

template <typename T>
cudaError_t dalloc(T** p, size_t bytes, cudaStream_t s) {
  return cudaMallocAsync(reinterpret_cast<void**>(p), bytes, s);
}
inline void dfree(const void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(const_cast<void*>(p), s);
}

#define TRY(x)                 \
  do {                         \
    int r_ = (x);              \
    if (r_ != BRAWL_OK) return r_; \
  } while (0)

// ---------------------------------------------------------------------------
// host-side model preparation
// ---------------------------------------------------------------------------
int make_geom(const brawl_setup& s, Geom& g) {
  if (s.lattice < BRAWL_SIMPLE_CUBIC || s.lattice > BRAWL_FCC)
    return fail(BRAWL_EINVAL, "Lattice type not yet implemented!");
  if (s.n_1 < 1 || s.n_2 < 1 || s.n_3 < 1 || s.n_1 > 1024 || s.n_2 > 1024 || s.n_3 > 1024)
    return fail(BRAWL_EINVAL, "n_1, n_2, n_3 must be in 1..1024");
  if (s.n_species < 1 || s.n_species > kMaxSpecies)
    return fail(BRAWL_EINVAL, "n_species must be in 1..15");
  if (s.interaction_range < 1 || s.interaction_range > max_shells(s.lattice))
    return fail(BRAWL_EINVAL, "Unsupported number of shells");
  const int64_t sites = (int64_t)n_atoms(s.lattice, s.n_1, s.n_2, s.n_3);
  if (sites > (int64_t)1 << 30) return fail(BRAWL_EINVAL, "lattice too large");
  std::memset(&g, 0, sizeof(g));
  g.lattice = s.lattice;
  g.n1 = s.n_1;
  g.n2 = s.n_2;
  g.n3 = s.n_3;
  g.nsh = s.interaction_range;
  g.ns = s.n_species;
  g.n_sites = (int32_t)sites;
  g.z = shell_starts(s.lattice)[g.nsh];
  if (s.lattice == kBcc) {
    g.sz = s.n_1 * s.n_2;
    g.sy = s.n_1;
    g.ys = 1;
    g.xs = 1;
  } else if (s.lattice == kFcc) {
    g.sz = 2 * s.n_2 * s.n_1;
    g.sy = s.n_1;
    g.ys = 0;
    g.xs = 1;
  } else {
    g.sz = 4 * s.n_1 * s.n_2;
    g.sy = 2 * s.n_1;
    g.ys = 0;
    g.xs = 0;
  }
  const int f = s.lattice == kSimpleCubic ? 1 : 2;  // sc wraps modulo n
  g.W1 = f * s.n_1;
  g.W2 = f * s.n_2;
  g.W3 = f * s.n_3;
  int dmax = 0;
  const int8_t(*offs)[3] = shell_offsets(s.lattice);
  for (int k = 0; k < g.z; ++k)
    for (int a = 0; a < 3; ++a) dmax = std::max(dmax, std::abs((int)offs[k][a]));
  g.fast_wrap = (s.lattice != kSimpleCubic) && std::min(g.W1, std::min(g.W2, g.W3)) >= dmax;
  g.nbr_k = s.lattice == kSimpleCubic ? 6 : s.lattice == kBcc ? 8 : 12;
  return BRAWL_OK;
}

// Halo staging of an fcc/bcc lattice (halo_engine.cuh): halo widths from the
// largest compact-index step of any entry at either parity; usable when the
// images of a site are unique (2h <= N per axis), the pair-distance test is
// exact (offsets within n per axis) and the difference table is staged.
void make_halo(const Geom& g, HaloGeom& H, bool& ok) {
  std::memset(&H, 0, sizeof(H));
  ok = false;
  if (g.lattice != kBcc && g.lattice != kFcc) return;
  const int8_t(*offs)[3] = shell_offsets(g.lattice);
  int hx = 0, hy = 0, hz = 0, dmx = 0, dmy = 0, dmz = 0;
  for (int k = 0; k < g.z; ++k) {
    const int dx = offs[k][0], dy = offs[k][1], dz = offs[k][2];
    dmx = std::max(dmx, std::abs(dx));
    dmy = std::max(dmy, std::abs(dy));
    dmz = std::max(dmz, std::abs(dz));
    for (int par = 0; par < 2; ++par) {
      const int ddx = (par + dx) >> 1;
      const int ddy = g.lattice == kBcc ? ((par + dy) >> 1) : dy;
      hx = std::max(hx, std::abs(ddx));
      hy = std::max(hy, std::abs(ddy));
      hz = std::max(hz, std::abs(dz));
    }
  }
  H.NX = g.n1;
  H.NY = g.lattice == kBcc ? g.n2 : 2 * g.n2;
  H.NZ = 2 * g.n3;
  H.hx = hx;
  H.hy = hy;
  H.hz = hz;
  H.SY = H.NX + 2 * hx;
  H.SZ = (H.NY + 2 * hy) * H.SY;
  const int64_t padded = (int64_t)(H.NZ + 2 * hz) * H.SZ;
  H.origin = hz * H.SZ + hy * H.SY + hx;
  H.dmx = dmx;
  H.dmy = dmy;
  H.dmz = dmz;
  if (padded > (int64_t)1 << 30) return;
  H.padded = (int32_t)padded;
  ok = 2 * hx <= H.NX && 2 * hy <= H.NY && 2 * hz <= H.NZ && dmx <= g.n1 && dmy <= g.n2 &&
       dmz <= g.n3 && smem_layout(g, false).use_D;
}

struct Model {
  Geom g;
  std::vector<double> V;
  std::vector<int32_t> F;
  std::vector<uint32_t> entries;
  std::vector<int16_t> sstart;
  int S = 0;
  int band = 0;
};

// Fixed-point image of V_ex for the fast tier.  S is the largest shift with
// 4 z max|V| 2^S <= 2^30, so a swap's 2z terms (each a difference of two
// entries) sum without overflow in int32.  band bounds, in quanta, the
// distance between the fixed-point sum and the reference's FP64 value of
// e_swapped - e_unswapped: one quantum per term for rounding V to the grid,
// plus the worst case of the reference's own recursive FP64 sums (every term
// passes through at most kmax + nsh - 1 roundings; |error| <= gamma_h *
// sum|terms| for each of the two pair energies), plus two quanta of slack.
int make_model(const brawl_setup& s, const double* V_ex, Model& m) {
  TRY(make_geom(s, m.g));
  if (!V_ex) return fail(BRAWL_EINVAL, "V_ex is NULL");
  const Geom& g = m.g;
  const int nv = g.ns * g.ns * g.nsh;
  m.V.assign(V_ex, V_ex + nv);
  double vmax = 0.0;
  for (double v : m.V) {
    if (!std::isfinite(v)) return fail(BRAWL_EINVAL, "V_ex contains a non-finite value");
    vmax = std::max(vmax, std::fabs(v));
  }
  const int nsp = g.ns + 1;
  m.F.assign((size_t)nsp * nsp * g.nsh, 0);
  if (vmax > 0.0) {
    m.S = (int)std::floor(std::log2(std::ldexp(1.0, 30) / (4.0 * g.z * vmax)));
    m.S = std::max(-200, std::min(m.S, 200));
    for (int a = 1; a <= g.ns; ++a)
      for (int b = 1; b <= g.ns; ++b)
        for (int sh = 0; sh < g.nsh; ++sh) {
          double v = m.V[(a - 1) + g.ns * ((b - 1) + g.ns * sh)];
          m.F[(a * g.nsh + sh) * nsp + b] = (int32_t)std::llrint(std::ldexp(v, m.S));
        }
    const int16_t* st = shell_starts(g.lattice);
    int kmax = 0;
    for (int sh = 0; sh < g.nsh; ++sh) kmax = std::max(kmax, (int)(st[sh + 1] - st[sh]));
    const int h = kmax + g.nsh - 1;
    const double fp = 4.0 * h * std::ldexp(1.0, -53) * g.z * vmax * std::ldexp(1.0, m.S) * 1.01;
    m.band = 2 * g.z + 2 + (int)std::ceil(fp);
  } else {
    m.S = 0;
    m.band = 0;
  }
  // D (see fixed_delta) follows F when it is small enough to stage
  if (smem_layout(g, false).use_D) {
    const size_t nF = m.F.size();
    m.F.resize(nF + (size_t)nsp * nsp * g.nsh * nsp, 0);
    for (int so = 1; so <= g.ns; ++so)
      for (int sn = 1; sn <= g.ns; ++sn)
        for (int sh = 0; sh < g.nsh; ++sh)
          for (int b = 1; b <= g.ns; ++b)
            m.F[nF + ((size_t)(so * nsp + sn) * g.nsh + sh) * nsp + b] =
                m.F[(sn * g.nsh + sh) * nsp + b] - m.F[(so * g.nsh + sh) * nsp + b];
  }
  const int16_t* st = shell_starts(g.lattice);
  const int8_t(*offs)[3] = shell_offsets(g.lattice);
  m.sstart.assign(st, st + g.nsh + 1);
  m.entries.resize(g.z);
  for (int sh = 0; sh < g.nsh; ++sh)
    for (int k = st[sh]; k < st[sh + 1]; ++k)
      m.entries[k] = (uint32_t)(uint8_t)offs[k][0] | ((uint32_t)(uint8_t)offs[k][1] << 8) |
                     ((uint32_t)(uint8_t)offs[k][2] << 16) | ((uint32_t)sh << 24);
  return BRAWL_OK;
}

void set_beta(ChainJob& j, const Model& m, double beta) {
  j.beta = beta;
  const double q = std::ldexp(1.0, -m.S);
  j.beta_q = (float)(beta * q);
  double bb = beta * (double)m.band * q;
  float bf = (float)bb;
  if ((double)bf < bb) bf = std::nextafter(bf, INFINITY);
  j.beta_band = bf;
  j.beta_q_l2 = (float)(beta * q * 1.4426950408889634);
}

// init_genrand (src/mt19937ar.c:63-78)
void mt_seed_host(uint32_t seed, uint32_t* state) {
  state[0] = seed;
  for (int i = 1; i < kMTN; ++i)
    state[i] = 1812433253u * (state[i - 1] ^ (state[i - 1] >> 30)) + (uint32_t)i;
  state[kMTN] = kMTN;
}

// Species quotas and interval bounds of initial_setup
// (src/initialise.F90:468-506, 534-535).
int make_init_job(const Model& m, double* conc, const int64_t* numbers, InitJob& ij) {
  const Geom& g = m.g;
  const int ns = g.ns;
  const int64_t n_atoms = g.n_sites;
  int64_t count[kMaxSpecies];
  int64_t sumnum = 0;
  if (numbers)
    for (int i = 0; i < ns; ++i) sumnum += numbers[i];
  if (numbers && sumnum == n_atoms) {
    for (int i = 0; i < ns; ++i) {
      count[i] = numbers[i];
      conc[i + 1] = (double)((float)count[i] / (float)n_atoms);
    }
  } else {
    int64_t total = 0;
    for (int i = 0; i < ns; ++i) {
      const double prod = (double)(float)n_atoms * conc[i + 1];
      if (!std::isfinite(prod)) return fail(BRAWL_EINVAL, "invalid species_concentrations");
      count[i] = (int64_t)std::llround(prod);
      total += count[i];
    }
    int64_t round_check = total - n_atoms;
    const int64_t inc = (-round_check >= 0) ? 1 : -1;
    int guard = 0;
    while (round_check != 0) {
      bool any = false;
      for (int j = 0; j < ns; ++j) {
        if (count[j] == 0 || round_check == 0) continue;
        count[j] += inc;
        round_check += inc;
        any = true;
      }
      if (!any || ++guard > 1000000) break;
    }
  }
  int64_t sum = 0;
  for (int i = 0; i < ns; ++i) {
    if (count[i] < 0) return fail(BRAWL_EINVAL, "negative species count");
    sum += count[i];
  }
  if (sum != n_atoms) return fail(BRAWL_EINVAL, "Species counts do not sum to the number of lattice sites");
  std::memset(&ij, 0, sizeof(ij));
  ij.n_sites = g.n_sites;
  ij.ns = ns;
  double lo = 0.0;
  for (int l = 1; l <= ns; ++l) {
    // sum(c(0:l-1)) and sum(c(0:l)), sequential as gfortran's SUM
    double a = 0.0;
    for (int i = 0; i <= l - 1; ++i) a = a + conc[i];
    double b = 0.0;
    for (int i = 0; i <= l; ++i) b = b + conc[i];
    lo = a;
    // w*2^-32 >= lo  <=>  w >= ceil(lo*2^32);  w*2^-32 <= b  <=>  w <= floor(b*2^32)
    double los = std::ceil(std::ldexp(lo, 32)), his = std::floor(std::ldexp(b, 32));
    los = std::max(-1.0, std::min(los, 8589934592.0));
    his = std::max(-1.0, std::min(his, 8589934592.0));
    ij.lo_w[l - 1] = (int64_t)los;
    ij.hi_w[l - 1] = (int64_t)his;
    ij.counts[l - 1] = count[l - 1];
    // a species whose quota is open must be reachable, or the loop never ends
    if (count[l - 1] > 0 && ij.lo_w[l - 1] > ij.hi_w[l - 1])
      return fail(BRAWL_EINVAL, "a species with atoms has an empty concentration interval");
    if (count[l - 1] > 0 && (ij.hi_w[l - 1] < 0 || ij.lo_w[l - 1] > 4294967295LL))
      return fail(BRAWL_EINVAL, "a species with atoms has an unreachable concentration interval");
  }
  return BRAWL_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
struct brawl_batch {
  std::vector<Model> models;
  std::vector<ChainJob> jobs;            // host images (pointers into the arena)
  std::vector<int> nbr_swap;
  unsigned char* arena = nullptr;        // every chain's mutable state and tables, one allocation
  size_t arena_bytes = 0;
  ChainJob* d_jobs = nullptr;
  EnergyJob* d_ejobs = nullptr;
  AsroJob* d_ajob = nullptr;
  unsigned long long* d_counters = nullptr;
  int32_t* d_status = nullptr;
  double* d_energy = nullptr;
  double* d_site_e = nullptr;            // lazily sized scratch
  size_t site_e_cap = 0;
  int8_t* d_grid = nullptr;              // staging for one full grid
  size_t grid_cap = 0;
  int8_t* d_grids = nullptr;             // staging for every chain's grid
  GridJob* d_gjobs = nullptr;
  int64_t total_cells = 0;
  void* d_scratch = nullptr;             // ASRO offsets and counts
  size_t scratch_cap = 0;
  cudaStream_t stream = nullptr;
  uint32_t smem_bytes = 0;
  bool smem_lat = true;
  bool use_D = true;
  int max_z = 0;
  // chains run by the halo kernel, and its shared-memory size / unrolling
  std::vector<int> halo;
  uint32_t halo_smem = 0;
  int halo_min_z = 0, halo_max_z = 0;
  std::vector<ChainJob> staged;          // jobs in launch order
  int n_halo_launch = 0;
  // classes of the shared-memory chains: chains of one (lattice, n1, n2, n3,
  // species, shells) share a class; each class is launched on its own
  // stream with its own shared memory, unrolling and trials per round
  std::vector<int> cls;                  // per chain: class, or -1 (not a halo chain)
  std::vector<uint32_t> class_smem;
  std::vector<int> class_z, class_depth;
  std::vector<int> class_first, class_count;  // in launch order (upload_jobs)
  std::vector<cudaStream_t> side;        // one per class beyond the first
  std::vector<cudaEvent_t> ev_side;
  cudaEvent_t ev_fork = nullptr;
  bool per_class = false;                // class depths chosen (brawl_batch_autotune_classes)
  std::vector<unsigned long long> last_counters;
  int device = 0;
  int max_optin = 0;
  int spec_nc = kDefaultSpeculation;  // trials per speculative round (1: none)
  double* d_alro = nullptr;              // ALRO counts: per chain ns x n_sites
  int64_t* d_alro_off = nullptr;
  std::vector<int64_t> alro_off;
  // sampling sums of the annealing loop (sampling.cu): one block holding
  // step_E and step_Esq (2n), the accepted counts at the loop's start (n),
  // n_atoms (n), the temperature's statistics (3n + 3), then the radial
  // densities' sums (n m) and statistics ((n + 1) m), m = wc ns^2
  unsigned char* d_samp = nullptr;
  int samp_wc = -1;                      // wc_range the block was laid out for
  double* d_sums = nullptr;
  unsigned long long* d_acc0 = nullptr;
  double* d_natoms = nullptr;
  double* d_tstats = nullptr;
  double* d_rho_sum = nullptr;
  double* d_rho_stats = nullptr;
  unsigned long long* d_mask = nullptr;  // ASRO class masks (64)
  // anneal blocks (brawl_batch_anneal_sweeps): 3n energy jobs (the live
  // lattices, then two snapshot buffers), the snapshots (2 x total sites),
  // the sampled energies (sweeps x n), and the stream the energies run on
  unsigned char* d_snap = nullptr;
  size_t snap_cap = 0;
  EnergyJob* d_snap_jobs = nullptr;
  int8_t* d_snap_lat = nullptr;
  double* d_traj = nullptr;
  size_t traj_rows = 0;
  cudaStream_t energy_stream = nullptr;
  cudaEvent_t ev_snap[2] = {nullptr, nullptr};
  cudaEvent_t ev_free[2] = {nullptr, nullptr};
};

struct brawl_ctx {
  brawl_batch* b;
};

namespace {

int check_status(brawl_batch* b) {
  std::vector<int32_t> st(b->jobs.size());
  CUDA_TRY(cudaMemcpyAsync(st.data(), b->d_status, st.size() * 4, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  for (size_t i = 0; i < st.size(); ++i)
    if (st[i] != 0) {
      int32_t zero = 0;
      cudaMemcpyAsync(b->d_status + i, &zero, 4, cudaMemcpyHostToDevice, b->stream);
      stream_wait(b->stream);
      return fail(BRAWL_ESTATE, "device check failed on chain " + std::to_string(i) + " (code " +
                                    std::to_string(st[i]) + ")");
    }
  return BRAWL_OK;
}

int ensure_grid(brawl_batch* b, size_t bytes) {
  if (bytes <= b->grid_cap) return BRAWL_OK;
  dfree(b->d_grid, b->stream);
  b->d_grid = nullptr;
  b->grid_cap = 0;
  CUDA_TRY(dalloc(&b->d_grid, bytes, b->stream));
  b->grid_cap = bytes;
  return BRAWL_OK;
}

// Jobs go to the device in launch order: halo chains first, then the rest,
// each group by decreasing trial count so the longest chains start first.
int upload_jobs(brawl_batch* b) {
  const int n = (int)b->jobs.size();
  const int nk = (int)b->class_smem.size();
  // classes by their longest chain, longest first; chains by trials
  std::vector<int64_t> class_most(nk, 0);
  for (int c = 0; c < n; ++c)
    if (b->cls[c] >= 0) class_most[b->cls[c]] = std::max(class_most[b->cls[c]], b->jobs[c].n_trials);
  std::vector<int> corder(nk), crank(nk);
  for (int k = 0; k < nk; ++k) corder[k] = k;
  std::stable_sort(corder.begin(), corder.end(), [&](int x, int y) { return class_most[x] > class_most[y]; });
  for (int r = 0; r < nk; ++r) crank[corder[r]] = r;
  std::vector<int> order(n);
  for (int c = 0; c < n; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    if (b->halo[x] != b->halo[y]) return b->halo[x] > b->halo[y];
    if (b->halo[x] && b->per_class && b->cls[x] != b->cls[y]) return crank[b->cls[x]] < crank[b->cls[y]];
    return b->jobs[x].n_trials > b->jobs[y].n_trials;
  });
  b->staged.resize(n);
  b->n_halo_launch = 0;
  b->class_first.assign(nk, 0);
  b->class_count.assign(nk, 0);
  for (int k = 0; k < n; ++k) {
    b->staged[k] = b->jobs[order[k]];
    b->n_halo_launch += b->halo[order[k]];
    const int cl = b->cls[order[k]];
    if (cl >= 0) {
      if (b->class_count[cl] == 0) b->class_first[cl] = k;
      b->class_count[cl] += 1;
    }
  }
  CUDA_TRY(cudaMemcpyAsync(b->d_jobs, b->staged.data(), n * sizeof(ChainJob),
                           cudaMemcpyHostToDevice, b->stream));
  return BRAWL_OK;
}

int read_counters(brawl_batch* b, std::vector<unsigned long long>& out) {
  out.resize(b->jobs.size() * kNumCounters);
  CUDA_TRY(cudaMemcpyAsync(out.data(), b->d_counters, out.size() * 8, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int set_chain_config(brawl_batch* b, int c, const int8_t* config) {
  const Geom& g = b->models[c].g;
  const size_t grid = (size_t)8 * g.n1 * g.n2 * g.n3;
  TRY(ensure_grid(b, grid));
  CUDA_TRY(cudaMemcpyAsync(b->d_grid, config, grid, cudaMemcpyHostToDevice, b->stream));
  launch_pack(g, b->d_grid, b->jobs[c].lat, b->d_status + c, b->stream);
  CUDA_TRY(cudaGetLastError());
  int r = check_status(b);
  if (r != BRAWL_OK) return fail(BRAWL_EINVAL, "config holds a species outside 1..n_species on an occupied site, or an atom on an empty site");
  return BRAWL_OK;
}

int run_metropolis_once(brawl_batch* b, const int64_t* n_trials, int64_t* accepted, bool serial,
                        cudaStream_t stream, bool wait);

// Side streams for the classes beyond the first (created once).
int ensure_side_streams(brawl_batch* b) {
  const size_t need = b->class_smem.empty() ? 0 : b->class_smem.size() - 1;
  if (!b->ev_fork) CUDA_TRY(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  while (b->side.size() < need) {
    cudaStream_t st;
    cudaEvent_t ev;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->side.push_back(st);
    b->ev_side.push_back(ev);
  }
  return BRAWL_OK;
}

// The shared-memory chains of every class (only = -1) or of class `only`,
// each class in its own launch with its own shared memory, unrolling and
// trials per round: the first on `stream`, the others on side streams
// forked from it and joined back.
int launch_classes(brawl_batch* b, cudaStream_t stream, int only) {
  TRY(ensure_side_streams(b));
  const int nk = (int)b->class_smem.size();
  std::vector<int> ks;
  for (int k = 0; k < nk; ++k)
    if (b->class_count[k] > 0 && (only < 0 || k == only)) ks.push_back(k);
  std::sort(ks.begin(), ks.end(), [&](int x, int y) { return b->class_first[x] < b->class_first[y]; });
  if (ks.size() > 1) CUDA_TRY(cudaEventRecord(b->ev_fork, stream));
  for (size_t i = 0; i < ks.size(); ++i) {
    const int k = ks[i];
    cudaStream_t st = i == 0 ? stream : b->side[i - 1];
    if (i > 0) CUDA_TRY(cudaStreamWaitEvent(st, b->ev_fork, 0));
    launch_halo_chains(b->d_jobs + b->class_first[k], b->class_count[k], b->class_smem[k], b->class_z[k],
                       b->class_z[k], b->class_depth[k], b->max_optin, st);
    CUDA_TRY(cudaGetLastError());
    if (i > 0) CUDA_TRY(cudaEventRecord(b->ev_side[i - 1], st));
  }
  for (size_t i = 1; i < ks.size(); ++i) CUDA_TRY(cudaStreamWaitEvent(stream, b->ev_side[i - 1], 0));
  return BRAWL_OK;
}

// Kernel launches run fewer than 2^31 trials per chain (their tallies are
// 32-bit); longer runs are split into consecutive launches, which continue
// every chain exactly where the previous one stopped.
constexpr int64_t kMaxLaunchTrials = ((int64_t)1 << 31) - 1;

int run_metropolis(brawl_batch* b, const int64_t* n_trials, int64_t* accepted, bool serial,
                   cudaStream_t stream, bool wait) {
  const int n = (int)b->jobs.size();
  int64_t most = 0;
  for (int c = 0; c < n; ++c) {
    if (n_trials[c] < 0) return fail(BRAWL_EINVAL, "n_trials < 0");
    most = std::max(most, n_trials[c]);
  }
  if (most <= kMaxLaunchTrials) return run_metropolis_once(b, n_trials, accepted, serial, stream, wait);
  std::vector<int64_t> left(n_trials, n_trials + n), part(n), acc(n, 0), acc_part(n);
  while (true) {
    bool any = false;
    for (int c = 0; c < n; ++c) {
      part[c] = std::min(left[c], kMaxLaunchTrials);
      left[c] -= part[c];
      any = any || part[c] > 0;
    }
    if (!any) break;
    TRY(run_metropolis_once(b, part.data(), acc_part.data(), serial, stream, true));
    for (int c = 0; c < n; ++c) acc[c] += acc_part[c];
  }
  if (accepted) std::copy(acc.begin(), acc.end(), accepted);
  return BRAWL_OK;
}

// Every chain's uploaded job (b->d_jobs) once on `stream`: the halo chains
// per class or in one launch, the others in one launch of the plain kernel.
int launch_sweep(brawl_batch* b, cudaStream_t stream) {
  const int n = (int)b->jobs.size();
  const int nh = b->n_halo_launch;
  if (nh > 0 && b->per_class)
    TRY(launch_classes(b, stream, -1));
  else if (nh > 0)
    launch_halo_chains(b->d_jobs, nh, b->halo_smem, b->halo_min_z, b->halo_max_z, b->spec_nc, b->max_optin,
                       stream);
  if (n - nh > 0)
    launch_metropolis(b->d_jobs + nh, n - nh, b->smem_lat, b->use_D, b->smem_bytes, b->max_z, stream);
  CUDA_TRY(cudaGetLastError());
  return BRAWL_OK;
}

int run_metropolis_once(brawl_batch* b, const int64_t* n_trials, int64_t* accepted, bool serial,
                        cudaStream_t stream, bool wait) {
  const int n = (int)b->jobs.size();
  for (int c = 0; c < n; ++c) {
    b->jobs[c].n_trials = n_trials[c];
    b->jobs[c].nbr_swap = b->nbr_swap[c];
  }
  TRY(upload_jobs(b));
  if (stream != b->stream) {
    // order the job upload before the launch on the caller's stream
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, b->stream));
    CUDA_TRY(cudaStreamWaitEvent(stream, ev, 0));
    cudaEventDestroy(ev);
  }
  if (!serial) {
    TRY(launch_sweep(b, stream));
  } else {
    const int nh = b->n_halo_launch;
    for (int k = 0; k < n; ++k) {
      if (k < nh)
        launch_halo_chains(b->d_jobs + k, 1, b->halo_smem, b->halo_min_z, b->halo_max_z, b->spec_nc, b->max_optin,
                           stream);
      else
        launch_metropolis(b->d_jobs + k, 1, b->smem_lat, b->use_D, b->smem_bytes, b->max_z,
                          stream);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(stream_wait(stream));
    }
  }
  if (!wait) return BRAWL_OK;
  CUDA_TRY(stream_wait(stream));
  std::vector<unsigned long long> cnt;
  TRY(read_counters(b, cnt));
  if (accepted)
    for (int c = 0; c < n; ++c)
      accepted[c] = (int64_t)(cnt[c * kNumCounters + kCntAccepted] -
                              b->last_counters[c * kNumCounters + kCntAccepted]);
  b->last_counters = cnt;
  return check_status(b);
}

}  // namespace

extern "C" {

const char* brawl_last_error(void) { return g_err.c_str(); }
int brawl_version(void) { return 10000; }

int brawl_batch_create(const brawl_chain_desc* chains, int n_chains, brawl_batch** out) {
  if (!out || !chains || n_chains < 1) return fail(BRAWL_EINVAL, "no chains");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fail(BRAWL_ECUDA, "no CUDA device");
  brawl_batch* b = new brawl_batch();
  auto cleanup = [&](int rc) {
    brawl_batch_destroy(b);
    return rc;
  };
  cudaGetDevice(&b->device);
  b->models.resize(n_chains);
  b->jobs.resize(n_chains);
  b->nbr_swap.resize(n_chains);
  for (int c = 0; c < n_chains; ++c) {
    int r = make_model(chains[c].setup, chains[c].V_ex, b->models[c]);
    if (r != BRAWL_OK) return cleanup(fail(r, "chain " + std::to_string(c) + ": " + g_err));
    b->nbr_swap[c] = chains[c].nbr_swap ? 1 : 0;
  }
  // shared memory: lattice staged when every chain fits
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  b->max_optin = max_optin;
  uint32_t need_smem = 0, need_gmem = 0;
  for (size_t c = 0; c < b->models.size(); ++c) {
    HaloGeom H;
    bool ok;
    make_halo(b->models[c].g, H, ok);
    if (ok && halo_layout(b->models[c].g, H).total <= (uint32_t)max_optin) continue;
    need_smem = std::max(need_smem, smem_layout(b->models[c].g, true).total);
    need_gmem = std::max(need_gmem, smem_layout(b->models[c].g, false).total);
  }
  b->halo.assign(n_chains, 0);
  b->cls.assign(n_chains, -1);
  for (int c = 0; c < n_chains; ++c) {
    const Model& m = b->models[c];
    HaloGeom H;
    bool ok;
    make_halo(m.g, H, ok);
    if (ok && halo_layout(m.g, H).total <= (uint32_t)max_optin) {
      b->halo[c] = 1;
      int k = 0;
      for (; k < c; ++k) {
        if (b->cls[k] < 0) continue;
        const Geom& o = b->models[k].g;
        if (o.lattice == m.g.lattice && o.n1 == m.g.n1 && o.n2 == m.g.n2 && o.n3 == m.g.n3 &&
            o.ns == m.g.ns && o.nsh == m.g.nsh)
          break;
      }
      if (k < c) {
        b->cls[c] = b->cls[k];
      } else {
        b->cls[c] = (int)b->class_smem.size();
        b->class_smem.push_back(halo_layout(m.g, H).total);
        b->class_z.push_back((int)m.g.z);
        b->class_depth.push_back(kDefaultSpeculation);
      }
      b->halo_smem = std::max(b->halo_smem, halo_layout(m.g, H).total);
      b->halo_min_z = b->halo_max_z == 0 ? (int)m.g.z : std::min(b->halo_min_z, (int)m.g.z);
      b->halo_max_z = std::max(b->halo_max_z, (int)m.g.z);
      continue;
    }
    b->max_z = std::max(b->max_z, (int)m.g.z);
    if (!smem_layout(m.g, false).use_D) b->use_D = false;
  }
  b->smem_lat = need_smem <= (uint32_t)max_optin;
  b->smem_bytes = b->smem_lat ? need_smem : need_gmem;
  if (b->smem_bytes > (uint32_t)max_optin)
    return cleanup(fail(BRAWL_EINVAL, "interaction tables exceed shared memory"));
  // arena layout
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  std::vector<size_t> off_lat(n_chains), off_rng(n_chains), off_V(n_chains), off_F(n_chains),
      off_e(n_chains), off_s(n_chains);
  size_t total = 0;
  for (int c = 0; c < n_chains; ++c) {
    const Model& m = b->models[c];
    off_lat[c] = total;
    total = al(total + m.g.n_sites);
    off_rng[c] = total;
    total = al(total + (kMTN + 1) * 4);
    off_V[c] = total;
    total = al(total + m.V.size() * 8);
    off_F[c] = total;
    total = al(total + m.F.size() * 4);
    off_e[c] = total;
    total = al(total + m.entries.size() * 4);
    off_s[c] = total;
    total = al(total + m.sstart.size() * 2);
  }
  const size_t off_jobs = total;
  total = al(total + n_chains * sizeof(ChainJob));
  const size_t off_ejobs = total;
  total = al(total + n_chains * sizeof(EnergyJob));
  const size_t off_ajob = total;
  total = al(total + sizeof(AsroJob));
  const size_t off_cnt = total;
  total = al(total + (size_t)n_chains * kNumCounters * 8);
  const size_t off_status = total;
  total = al(total + (size_t)n_chains * 4);
  const size_t off_energy = total;
  total = al(total + (size_t)n_chains * 8);
  if (object_stream(&b->stream) != cudaSuccess)
    return cleanup(fail(BRAWL_ECUDA, "stream create failed"));
  cudaError_t e = dalloc(&b->arena, total, b->stream);
  b->arena_bytes = total;
  if (e != cudaSuccess) {
    b->arena = nullptr;
    b->arena_bytes = 0;
    return cleanup(fail(BRAWL_ENOMEM, std::string("arena: ") + cudaGetErrorString(e)));
  }
  std::vector<unsigned char> h(total, 0);
  for (int c = 0; c < n_chains; ++c) {
    const Model& m = b->models[c];
    mt_seed_host(chains[c].seed, reinterpret_cast<uint32_t*>(&h[off_rng[c]]));
    std::memcpy(&h[off_V[c]], m.V.data(), m.V.size() * 8);
    std::memcpy(&h[off_F[c]], m.F.data(), m.F.size() * 4);
    std::memcpy(&h[off_e[c]], m.entries.data(), m.entries.size() * 4);
    std::memcpy(&h[off_s[c]], m.sstart.data(), m.sstart.size() * 2);
    ChainJob& j = b->jobs[c];
    std::memset(&j, 0, sizeof(j));
    j.g = m.g;
    {
      bool ok;
      make_halo(m.g, j.hg, ok);
      j.halo = b->halo[c];
    }
    j.nbr_swap = b->nbr_swap[c];
    j.band = m.band;
    set_beta(j, m, chains[c].beta);
    j.lat = reinterpret_cast<int8_t*>(b->arena + off_lat[c]);
    j.rng = reinterpret_cast<uint32_t*>(b->arena + off_rng[c]);
    j.V = reinterpret_cast<const double*>(b->arena + off_V[c]);
    j.F = reinterpret_cast<const int32_t*>(b->arena + off_F[c]);
    j.entries = reinterpret_cast<const uint32_t*>(b->arena + off_e[c]);
    j.shell_start = reinterpret_cast<const int16_t*>(b->arena + off_s[c]);
    j.counters = reinterpret_cast<unsigned long long*>(b->arena + off_cnt) + c * kNumCounters;
    j.status = reinterpret_cast<int32_t*>(b->arena + off_status) + c;
  }
  b->d_jobs = reinterpret_cast<ChainJob*>(b->arena + off_jobs);
  b->d_ejobs = reinterpret_cast<EnergyJob*>(b->arena + off_ejobs);
  b->d_ajob = reinterpret_cast<AsroJob*>(b->arena + off_ajob);
  b->d_counters = reinterpret_cast<unsigned long long*>(b->arena + off_cnt);
  b->d_status = reinterpret_cast<int32_t*>(b->arena + off_status);
  b->d_energy = reinterpret_cast<double*>(b->arena + off_energy);
  std::memcpy(&h[off_jobs], b->jobs.data(), n_chains * sizeof(ChainJob));
  e = cudaMemcpyAsync(b->arena, h.data(), total, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = stream_wait(b->stream);
  if (e != cudaSuccess) return cleanup(fail(BRAWL_ECUDA, cudaGetErrorString(e)));
  b->last_counters.assign((size_t)n_chains * kNumCounters, 0);
  // configurations: given ones are packed, the others drawn by initial_setup
  std::vector<InitJob> init;
  for (int c = 0; c < n_chains; ++c) {
    if (chains[c].config) {
      int r = set_chain_config(b, c, chains[c].config);
      if (r != BRAWL_OK) return cleanup(fail(r, "chain " + std::to_string(c) + ": " + g_err));
    } else {
      if (!chains[c].species_concentrations)
        return cleanup(fail(BRAWL_EINVAL, "chain " + std::to_string(c) +
                                              ": needs a config or species_concentrations"));
      std::vector<double> conc(chains[c].species_concentrations,
                               chains[c].species_concentrations + b->models[c].g.ns + 1);
      InitJob ij;
      int r = make_init_job(b->models[c], conc.data(), chains[c].species_numbers, ij);
      if (r != BRAWL_OK) return cleanup(fail(r, "chain " + std::to_string(c) + ": " + g_err));
      ij.lat = b->jobs[c].lat;
      ij.rng = b->jobs[c].rng;
      ij.counters = b->jobs[c].counters;
      ij.status = b->jobs[c].status;
      init.push_back(ij);
    }
  }
  if (!init.empty()) {
    InitJob* d_init = nullptr;
    e = dalloc(&d_init, init.size() * sizeof(InitJob), b->stream);
    if (e != cudaSuccess) return cleanup(fail(BRAWL_ENOMEM, cudaGetErrorString(e)));
    cudaMemcpyAsync(d_init, init.data(), init.size() * sizeof(InitJob), cudaMemcpyHostToDevice,
                    b->stream);
    launch_initial_setup(d_init, (int)init.size(), b->stream);
    dfree(d_init, b->stream);
    e = stream_wait(b->stream);
    if (e != cudaSuccess) return cleanup(fail(BRAWL_ECUDA, cudaGetErrorString(e)));
    int r = check_status(b);
    if (r != BRAWL_OK) return cleanup(r);
  }
  {
    std::vector<unsigned long long> cnt;
    int r = read_counters(b, cnt);
    if (r != BRAWL_OK) return cleanup(r);
    b->last_counters = cnt;
  }
  *out = b;
  return BRAWL_OK;
}

int brawl_batch_destroy(brawl_batch* b) {
  if (!b) return BRAWL_OK;
  if (b->stream) {
    for (const void* p : {(const void*)b->arena, (const void*)b->d_site_e, (const void*)b->d_grid,
                          (const void*)b->d_grids, (const void*)b->d_gjobs, (const void*)b->d_scratch,
                          (const void*)b->d_alro, (const void*)b->d_alro_off, (const void*)b->d_samp,
                          (const void*)b->d_snap, (const void*)b->d_traj})
      dfree(p, b->stream);
    stream_wait(b->stream);
    if (b->energy_stream) {
      stream_wait(b->energy_stream);
      cudaStreamDestroy(b->energy_stream);
    }
    for (cudaEvent_t ev : {b->ev_snap[0], b->ev_snap[1], b->ev_free[0], b->ev_free[1]})
      if (ev) cudaEventDestroy(ev);
    for (size_t k = 0; k < b->side.size(); ++k) {
      stream_wait(b->side[k]);
      cudaEventDestroy(b->ev_side[k]);
      cudaStreamDestroy(b->side[k]);
    }
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    cudaStreamDestroy(b->stream);
  }
  delete b;
  return BRAWL_OK;
}

int brawl_batch_size(brawl_batch* b, int* n) {
  if (!b || !n) return fail(BRAWL_EINVAL, "null argument");
  *n = (int)b->jobs.size();
  return BRAWL_OK;
}

int brawl_batch_set_speculation(brawl_batch* b, int trials_per_round) {
  if (!b || trials_per_round < 1 || trials_per_round > 4) return fail(BRAWL_EINVAL, "trials per round must be 1-4");
  b->spec_nc = trials_per_round;
  return BRAWL_OK;
}

// Trials per round chosen per class of shared-memory chains, by
// measurement of the whole batch: the classes in order of decreasing work
// (the class holding the longest chains first), each class's depth 1..
// max_depth tried while the others keep theirs, every try run three times
// from the same state (restored after each) and the median kept; a deeper
// round is taken only when it is at least 2% faster.  Every depth is
// bit-exact, so the results never depend on the choice.
int brawl_batch_autotune_classes(brawl_batch* b, const int64_t* n_trials, int max_depth, int* depths,
                                 double* ms, int* n_classes) {
  if (!b || !n_trials || max_depth < 1 || max_depth > 4) return fail(BRAWL_EINVAL, "bad argument");
  for (size_t c = 0; c < b->jobs.size(); ++c)
    if (n_trials[c] < 0) return fail(BRAWL_EINVAL, "n_trials < 0");
  const int nk = (int)b->class_smem.size();
  if (n_classes) *n_classes = nk;
  if (nk == 0) return BRAWL_OK;
  cudaStream_t s = b->stream;
  unsigned char* snap = nullptr;
  if (dalloc(&snap, b->arena_bytes, s) != cudaSuccess) return fail(BRAWL_ENOMEM, "autotune snapshot");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const std::vector<unsigned long long> last = b->last_counters;
  const std::vector<int> keep = b->class_depth;
  const bool keep_pc = b->per_class;
  int rc = BRAWL_OK;
  auto cuda = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == BRAWL_OK) rc = fail(BRAWL_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return rc == BRAWL_OK;
  };
  std::vector<double> work(nk, 0.0);
  for (size_t c = 0; c < b->jobs.size(); ++c)
    if (b->cls[c] >= 0) work[b->cls[c]] += (double)n_trials[c];
  std::vector<int> order(nk);
  for (int k = 0; k < nk; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
  b->per_class = true;
  b->class_depth.assign(nk, 1);
  auto timed = [&](float& out) {
    std::vector<float> t(3, 0.0f);
    for (int r = 0; r < 3 && rc == BRAWL_OK; ++r) {
      if (!cuda(cudaEventRecord(e0, s), "event")) return;
      const int q = run_metropolis(b, n_trials, nullptr, false, s, false);
      if (q != BRAWL_OK) {
        rc = q;
        return;
      }
      if (!cuda(cudaEventRecord(e1, s), "event") || !cuda(cudaEventSynchronize(e1), "timed run") ||
          !cuda(cudaEventElapsedTime(&t[r], e0, e1), "event"))
        return;
      if (!cuda(cudaMemcpyAsync(b->arena, snap, b->arena_bytes, cudaMemcpyDeviceToDevice, s), "restore")) return;
      b->last_counters = last;
    }
    std::sort(t.begin(), t.end());
    out = t[1];
  };
  if (cuda(cudaEventCreate(&e0), "event") && cuda(cudaEventCreate(&e1), "event") &&
      cuda(cudaMemcpyAsync(snap, b->arena, b->arena_bytes, cudaMemcpyDeviceToDevice, s), "snapshot")) {
    for (int k : order) {
      float best_t = 0.0f;
      int best_d = 1;
      for (int d = 1; d <= max_depth && rc == BRAWL_OK; ++d) {
        b->class_depth[k] = d;
        float t = 0.0f;
        timed(t);
        if (rc != BRAWL_OK) break;
        if (ms) ms[k * max_depth + d - 1] = (double)t;
        if (d == 1 || t < 0.98f * best_t) {
          best_t = t;
          best_d = d;
        }
      }
      b->class_depth[k] = best_d;
      if (rc != BRAWL_OK) break;
    }
    cuda(stream_wait(s), "restore");
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dfree(snap, s);
  if (rc != BRAWL_OK) {
    b->class_depth = keep;
    b->per_class = keep_pc;
  }
  if (depths)
    for (int k = 0; k < nk; ++k) depths[k] = b->class_depth[k];
  return rc;
}

// Trials per round of every class, set by the caller (1-4 each); every
// class then runs in its own launch.
int brawl_batch_set_class_depths(brawl_batch* b, const int* depths) {
  if (!b || !depths) return fail(BRAWL_EINVAL, "null argument");
  for (size_t k = 0; k < b->class_depth.size(); ++k)
    if (depths[k] < 1 || depths[k] > 4) return fail(BRAWL_EINVAL, "trials per round must be 1-4");
  for (size_t k = 0; k < b->class_depth.size(); ++k) b->class_depth[k] = depths[k];
  b->per_class = true;
  return BRAWL_OK;
}

// The class of every chain (-1: not a shared-memory chain).
int brawl_batch_chain_classes(brawl_batch* b, int* classes) {
  if (!b || !classes) return fail(BRAWL_EINVAL, "null argument");
  for (size_t c = 0; c < b->cls.size(); ++c) classes[c] = b->cls[c];
  return BRAWL_OK;
}

// The CTA shape of the shared-memory chains, picked by measurement: every
// depth of 1..max_depth trials per round (1: one warp per chain; d: the
// d(d+1)/2-warp speculative rounds) runs the same trials from the same
// state, timed with events on the batch's stream, and the arena (lattices,
// streams, counters, status) is put back after each, so the results the
// caller sees do not depend on the choice -- every depth is bit-exact.
int brawl_batch_autotune(brawl_batch* b, const int64_t* n_trials, int max_depth, double* ms, int* chosen) {
  if (!b || !n_trials || max_depth < 1 || max_depth > 4) return fail(BRAWL_EINVAL, "bad argument");
  for (size_t c = 0; c < b->jobs.size(); ++c)
    if (n_trials[c] < 0) return fail(BRAWL_EINVAL, "n_trials < 0");
  cudaStream_t s = b->stream;
  unsigned char* snap = nullptr;
  if (dalloc(&snap, b->arena_bytes, s) != cudaSuccess) return fail(BRAWL_ENOMEM, "autotune snapshot");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const std::vector<unsigned long long> last = b->last_counters;
  const int keep = b->spec_nc;
  int rc = BRAWL_OK, best = keep;
  float best_ms = 0.0f;
  auto cuda = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == BRAWL_OK) rc = fail(BRAWL_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return rc == BRAWL_OK;
  };
  if (cuda(cudaEventCreate(&e0), "event") && cuda(cudaEventCreate(&e1), "event") &&
      cuda(cudaMemcpyAsync(snap, b->arena, b->arena_bytes, cudaMemcpyDeviceToDevice, s), "snapshot")) {
    for (int d = 1; d <= max_depth && rc == BRAWL_OK; ++d) {
      b->spec_nc = d;
      if (!cuda(cudaEventRecord(e0, s), "event")) break;
      const int r = run_metropolis(b, n_trials, nullptr, false, s, false);
      if (r != BRAWL_OK) {
        rc = r;
        break;
      }
      float t = 0.0f;
      if (!cuda(cudaEventRecord(e1, s), "event") || !cuda(cudaEventSynchronize(e1), "timed run") ||
          !cuda(cudaEventElapsedTime(&t, e0, e1), "event"))
        break;
      if (!cuda(cudaMemcpyAsync(b->arena, snap, b->arena_bytes, cudaMemcpyDeviceToDevice, s), "restore")) break;
      b->last_counters = last;
      if (ms) ms[d - 1] = (double)t;
      if (d == 1 || t < best_ms) {
        best_ms = t;
        best = d;
      }
    }
    cuda(stream_wait(s), "restore");
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dfree(snap, s);
  b->spec_nc = rc == BRAWL_OK ? best : keep;
  if (chosen) *chosen = b->spec_nc;
  return rc;
}

int brawl_batch_set_beta(brawl_batch* b, const double* beta) {
  if (!b || !beta) return fail(BRAWL_EINVAL, "null argument");
  for (size_t c = 0; c < b->jobs.size(); ++c) set_beta(b->jobs[c], b->models[c], beta[c]);
  return BRAWL_OK;
}

int brawl_batch_metropolis_run(brawl_batch* b, const int64_t* n_trials, int64_t* accepted) {
  if (!b || !n_trials) return fail(BRAWL_EINVAL, "null argument");
  return run_metropolis(b, n_trials, accepted, false, b->stream, true);
}

int brawl_batch_metropolis_run_async(brawl_batch* b, const int64_t* n_trials, void* stream) {
  if (!b || !n_trials) return fail(BRAWL_EINVAL, "null argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
  return run_metropolis(b, n_trials, nullptr, false, s, false);
}

int brawl_batch_sync(brawl_batch* b) {
  if (!b) return fail(BRAWL_EINVAL, "null argument");
  CUDA_TRY(cudaDeviceSynchronize());
  std::vector<unsigned long long> cnt;
  TRY(read_counters(b, cnt));
  b->last_counters = cnt;
  return check_status(b);
}

int brawl_batch_metropolis_run_serial(brawl_batch* b, const int64_t* n_trials, int64_t* accepted) {
  if (!b || !n_trials) return fail(BRAWL_EINVAL, "null argument");
  return run_metropolis(b, n_trials, accepted, true, b->stream, true);
}

// Queues full_energy of every chain into b->d_energy on the batch stream.
static int queue_batch_energy(brawl_batch* b) {
  const int n = (int)b->jobs.size();
  int64_t total_sites = 0;
  for (int c = 0; c < n; ++c) total_sites += b->models[c].g.n_sites;
  if ((size_t)total_sites * 8 > b->site_e_cap) {
    dfree(b->d_site_e, b->stream);
    b->d_site_e = nullptr;
    b->site_e_cap = 0;
    CUDA_TRY(dalloc(&b->d_site_e, (size_t)total_sites * 8, b->stream));
    b->site_e_cap = (size_t)total_sites * 8;
  }
  std::vector<EnergyJob> ej(n);
  int64_t off = 0;
  for (int c = 0; c < n; ++c) {
    EnergyJob& j = ej[c];
    j.g = b->models[c].g;
    j.lat = b->jobs[c].lat;
    j.V = b->jobs[c].V;
    j.entries = b->jobs[c].entries;
    j.shell_start = b->jobs[c].shell_start;
    j.site_energy = b->d_site_e + off;
    j.out = b->d_energy + c;
    j.site_offset = off;
    off += j.g.n_sites;
  }
  CUDA_TRY(cudaMemcpyAsync(b->d_ejobs, ej.data(), n * sizeof(EnergyJob), cudaMemcpyHostToDevice,
                           b->stream));
  launch_total_energy(b->d_ejobs, n, total_sites, b->stream);
  CUDA_TRY(cudaGetLastError());
  return BRAWL_OK;
}

int brawl_batch_total_energy(brawl_batch* b, double* energies) {
  if (!b || !energies) return fail(BRAWL_EINVAL, "null argument");
  TRY(queue_batch_energy(b));
  const int n = (int)b->jobs.size();
  CUDA_TRY(cudaMemcpyAsync(energies, b->d_energy, n * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_get_config(brawl_batch* b, int c, int8_t* config) {
  if (!b || !config || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad argument");
  const Geom& g = b->models[c].g;
  const size_t grid = (size_t)8 * g.n1 * g.n2 * g.n3;
  TRY(ensure_grid(b, grid));
  launch_unpack(g, b->jobs[c].lat, b->d_grid, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(config, b->d_grid, grid, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_set_config(brawl_batch* b, int c, const int8_t* config) {
  if (!b || !config || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad argument");
  return set_chain_config(b, c, config);
}

static int ensure_grids(brawl_batch* b) {
  if (b->d_grids) return BRAWL_OK;
  const int n = (int)b->jobs.size();
  std::vector<GridJob> gj(n);
  int64_t off = 0;
  for (int c = 0; c < n; ++c) {
    gj[c].g = b->models[c].g;
    gj[c].lat = b->jobs[c].lat;
    gj[c].grid_offset = off;
    gj[c].status = b->jobs[c].status;
    off += (int64_t)8 * gj[c].g.n1 * gj[c].g.n2 * gj[c].g.n3;
  }
  CUDA_TRY(dalloc(&b->d_grids, (size_t)off, b->stream));
  CUDA_TRY(dalloc(&b->d_gjobs, n * sizeof(GridJob), b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->d_gjobs, gj.data(), n * sizeof(GridJob), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  b->total_cells = off;
  return BRAWL_OK;
}

int brawl_batch_get_configs(brawl_batch* b, int8_t* configs) {
  if (!b || !configs) return fail(BRAWL_EINVAL, "null argument");
  TRY(ensure_grids(b));
  launch_unpack_batch(b->d_gjobs, (int)b->jobs.size(), b->total_cells, b->d_grids, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(configs, b->d_grids, (size_t)b->total_cells, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_set_configs(brawl_batch* b, const int8_t* configs) {
  if (!b || !configs) return fail(BRAWL_EINVAL, "null argument");
  TRY(ensure_grids(b));
  CUDA_TRY(cudaMemcpyAsync(b->d_grids, configs, (size_t)b->total_cells, cudaMemcpyHostToDevice,
                           b->stream));
  launch_pack_batch(b->d_gjobs, (int)b->jobs.size(), b->total_cells, b->d_grids, b->stream);
  CUDA_TRY(cudaGetLastError());
  int r = check_status(b);
  if (r != BRAWL_OK) return fail(BRAWL_EINVAL, "a config holds a species outside 1..n_species on an occupied site, or an atom on an empty site");
  return BRAWL_OK;
}

// The device address of a page-locked, 16-byte aligned host buffer (the
// batch conversions read and write it 4 bytes at a time), or null.
static const void* host_alias(const void* p) {
  if (reinterpret_cast<uintptr_t>(p) & 15u) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int brawl_batch_metropolis_host(brawl_batch* b, const int8_t* configs_in, const int64_t* n_trials,
                                int8_t* configs_out, int64_t* accepted) {
  if (!b || !configs_in || !n_trials || !configs_out) return fail(BRAWL_EINVAL, "null argument");
  TRY(ensure_grids(b));
  const int n = (int)b->jobs.size();
  cudaStream_t s = b->stream;
  const int8_t* src = static_cast<const int8_t*>(host_alias(configs_in));
  if (!src) {
    CUDA_TRY(cudaMemcpyAsync(b->d_grids, configs_in, (size_t)b->total_cells, cudaMemcpyHostToDevice, s));
    src = b->d_grids;
  }
  // a chain whose grid holds a bad species is flagged here and runs no trial
  launch_pack_batch(b->d_gjobs, n, b->total_cells, src, s);
  CUDA_TRY(cudaGetLastError());
  TRY(run_metropolis(b, n_trials, nullptr, false, s, false));
  int8_t* dst = static_cast<int8_t*>(const_cast<void*>(host_alias(configs_out)));
  launch_unpack_batch(b->d_gjobs, n, b->total_cells, dst ? dst : b->d_grids, s);
  CUDA_TRY(cudaGetLastError());
  if (!dst)
    CUDA_TRY(cudaMemcpyAsync(configs_out, b->d_grids, (size_t)b->total_cells, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(stream_wait(s));
  std::vector<unsigned long long> cnt;
  TRY(read_counters(b, cnt));
  if (accepted)
    for (int c = 0; c < n; ++c)
      accepted[c] = (int64_t)(cnt[c * kNumCounters + kCntAccepted] -
                              b->last_counters[c * kNumCounters + kCntAccepted]);
  b->last_counters = cnt;
  return check_status(b);
}

static int ensure_alro(brawl_batch* b) {
  if (b->d_alro) return BRAWL_OK;
  TRY(ensure_grids(b));
  const int n = (int)b->jobs.size();
  b->alro_off.assign(n + 1, 0);
  for (int c = 0; c < n; ++c)
    b->alro_off[c + 1] = b->alro_off[c] + (int64_t)b->models[c].g.ns * b->models[c].g.n_sites;
  CUDA_TRY(dalloc(&b->d_alro, (size_t)b->alro_off[n] * 8, b->stream));
  CUDA_TRY(dalloc(&b->d_alro_off, (size_t)n * 8, b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->d_alro_off, b->alro_off.data(), (size_t)n * 8, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaMemsetAsync(b->d_alro, 0, (size_t)b->alro_off[n] * 8, b->stream));
  return BRAWL_OK;
}

int brawl_batch_alro_add(brawl_batch* b) {
  if (!b) return fail(BRAWL_EINVAL, "null argument");
  TRY(ensure_alro(b));
  launch_alro_add(b->d_gjobs, (int)b->jobs.size(), b->d_alro, b->d_alro_off, b->stream);
  CUDA_TRY(cudaGetLastError());
  return BRAWL_OK;
}

int brawl_batch_alro_reset(brawl_batch* b) {
  if (!b) return fail(BRAWL_EINVAL, "null argument");
  TRY(ensure_alro(b));
  CUDA_TRY(cudaMemsetAsync(b->d_alro, 0, (size_t)b->alro_off.back() * 8, b->stream));
  return BRAWL_OK;
}

int brawl_batch_alro_get(brawl_batch* b, int c, double* order) {
  if (!b || !order || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad argument");
  TRY(ensure_alro(b));
  const Geom& g = b->models[c].g;
  std::vector<double> cnt((size_t)g.ns * g.n_sites);
  CUDA_TRY(cudaMemcpyAsync(cnt.data(), b->d_alro + b->alro_off[c], cnt.size() * 8, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(stream_wait(b->stream));
  // order(species, basis, x, y, z), species fastest; empty cells stay 0
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3, ns = g.ns;
  std::fill(order, order + (size_t)ns * W1 * W2 * W3, 0.0);
  for (int z = 0; z < W3; ++z)
    for (int y = 0; y < W2; ++y)
      for (int x = 0; x < W1; ++x) {
        const bool occ = g.lattice == kBcc   ? (((x & 1) == (z & 1)) && ((y & 1) == (z & 1)))
                         : g.lattice == kFcc ? (((x + y + z) & 1) == 0)
                                             : true;
        if (!occ) continue;
        const int i = z * g.sz + (y >> g.ys) * g.sy + (x >> g.xs);
        double* cell = order + ((size_t)(z * W2 + y) * W1 + x) * ns;
        for (int s = 0; s < ns; ++s) cell[s] = cnt[(size_t)s * g.n_sites + i];
      }
  return BRAWL_OK;
}

int brawl_batch_rng_get(brawl_batch* b, int c, uint32_t state[625]) {
  if (!b || !state || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad argument");
  CUDA_TRY(cudaMemcpyAsync(state, b->jobs[c].rng, (kMTN + 1) * 4, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_counters(brawl_batch* b, int64_t* counters) {
  if (!b || !counters) return fail(BRAWL_EINVAL, "null argument");
  std::vector<unsigned long long> cnt;
  TRY(read_counters(b, cnt));
  for (size_t i = 0; i < cnt.size(); ++i) counters[i] = (int64_t)cnt[i];
  return BRAWL_OK;
}

// The ASRO pair counts of chain c queued on the batch's stream; *d_counts
// receives their device address (in the batch's scratch).
static int queue_asro_counts(brawl_batch* b, int c, int wc_range, const double* shells, AsroPlan& plan,
                             unsigned long long** d_counts) {
  const Geom& g = b->models[c].g;
  TRY(make_asro_plan(g, wc_range, shells, plan) == 0 ? BRAWL_OK
                                                     : fail(BRAWL_EINVAL, "bad ASRO plan"));
  const int nsp = g.ns + 1;
  const size_t n_counts = (size_t)nsp * nsp * plan.n_class + nsp;
  const size_t bytes = plan.offsets.size() * 4 + 256 + n_counts * 8;
  if (bytes > b->scratch_cap) {
    dfree(b->d_scratch, b->stream);
    b->d_scratch = nullptr;
    b->scratch_cap = 0;
    CUDA_TRY(dalloc(&b->d_scratch, bytes, b->stream));
    b->scratch_cap = bytes;
  }
  unsigned char* s = reinterpret_cast<unsigned char*>(b->d_scratch);
  uint32_t* d_offs = reinterpret_cast<uint32_t*>(s);
  unsigned long long* d_cnt =
      reinterpret_cast<unsigned long long*>(s + (plan.offsets.size() * 4 + 255) / 256 * 256);
  CUDA_TRY(cudaMemcpyAsync(d_offs, plan.offsets.data(), plan.offsets.size() * 4,
                           cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaMemsetAsync(d_cnt, 0, n_counts * 8, b->stream));
  AsroJob aj;
  aj.g = g;
  aj.lat = b->jobs[c].lat;
  aj.offsets = d_offs;
  aj.n_offsets = (int)plan.offsets.size();
  aj.n_class = plan.n_class;
  aj.counts = d_cnt;
  aj.species_counts = d_cnt + (size_t)nsp * nsp * plan.n_class;
  CUDA_TRY(cudaMemcpyAsync(b->d_ajob, &aj, sizeof(aj), cudaMemcpyHostToDevice, b->stream));
  launch_asro(b->d_ajob, g, plan.n_class, b->stream);
  CUDA_TRY(cudaGetLastError());
  *d_counts = d_cnt;
  return BRAWL_OK;
}

int brawl_batch_radial_densities(brawl_batch* b, int c, int wc_range, const double* shells,
                                 double* rho) {
  if (!b || !shells || !rho || c < 0 || c >= (int)b->jobs.size() || wc_range < 1 || wc_range > 64)
    return fail(BRAWL_EINVAL, "bad argument");
  const Geom& g = b->models[c].g;
  AsroPlan plan;
  unsigned long long* d_cnt = nullptr;
  TRY(queue_asro_counts(b, c, wc_range, shells, plan, &d_cnt));
  const int nsp = g.ns + 1;
  const size_t n_counts = (size_t)nsp * nsp * plan.n_class + nsp;
  std::vector<unsigned long long> cnt(n_counts);
  CUDA_TRY(cudaMemcpyAsync(cnt.data(), d_cnt, n_counts * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  finish_asro(g, wc_range, plan, cnt.data(), rho);
  return BRAWL_OK;
}

// ---------------------------------------------------------------------------
// Sampling reductions of the annealing loop (sampling.cu)
// ---------------------------------------------------------------------------
// The sampling block, laid out for wc_range (0: no radial densities); every
// chain must have the same species count when wc_range > 0.
static int ensure_sampling(brawl_batch* b, int wc_range) {
  const int n = (int)b->jobs.size();
  if (b->d_samp && b->samp_wc == wc_range) return BRAWL_OK;
  int ns = b->models[0].g.ns;
  if (wc_range > 0)
    for (int c = 1; c < n; ++c)
      if (b->models[c].g.ns != ns) return fail(BRAWL_EINVAL, "radial-density sums need equal species counts");
  const size_t m = wc_range > 0 ? (size_t)wc_range * ns * ns : 0;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_sums = 0, o_acc0 = al(o_sums + 2 * n * 8), o_nat = al(o_acc0 + n * 8),
               o_t = al(o_nat + n * 8), o_rs = al(o_t + (3 * n + 3) * 8), o_rst = al(o_rs + n * m * 8),
               o_mask = al(o_rst + (n + 1) * m * 8), total = al(o_mask + 64 * 8);
  dfree(b->d_samp, b->stream);
  b->d_samp = nullptr;
  CUDA_TRY(dalloc(&b->d_samp, total, b->stream));
  b->samp_wc = wc_range;
  b->d_sums = reinterpret_cast<double*>(b->d_samp + o_sums);
  b->d_acc0 = reinterpret_cast<unsigned long long*>(b->d_samp + o_acc0);
  b->d_natoms = reinterpret_cast<double*>(b->d_samp + o_nat);
  b->d_tstats = reinterpret_cast<double*>(b->d_samp + o_t);
  b->d_rho_sum = reinterpret_cast<double*>(b->d_samp + o_rs);
  b->d_rho_stats = reinterpret_cast<double*>(b->d_samp + o_rst);
  b->d_mask = reinterpret_cast<unsigned long long*>(b->d_samp + o_mask);
  std::vector<double> nat(n);
  for (int c = 0; c < n; ++c) nat[c] = (double)b->models[c].g.n_sites;
  CUDA_TRY(cudaMemcpyAsync(b->d_natoms, nat.data(), n * 8, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaMemsetAsync(b->d_samp, 0, o_nat, b->stream));
  if (m) CUDA_TRY(cudaMemsetAsync(b->d_rho_sum, 0, n * m * 8, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_sampling_reset(brawl_batch* b, int wc_range) {
  if (!b || wc_range < 0 || wc_range > 64) return fail(BRAWL_EINVAL, "bad argument");
  TRY(ensure_sampling(b, wc_range));
  const int n = (int)b->jobs.size();
  const size_t m = wc_range > 0 ? (size_t)wc_range * b->models[0].g.ns * b->models[0].g.ns : 0;
  CUDA_TRY(cudaMemsetAsync(b->d_sums, 0, 2 * n * 8, b->stream));
  if (m) CUDA_TRY(cudaMemsetAsync(b->d_rho_sum, 0, n * m * 8, b->stream));
  launch_acceptance_snapshot(b->d_counters, b->d_acc0, n, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_energy_sample(brawl_batch* b, double* energies) {
  if (!b) return fail(BRAWL_EINVAL, "null argument");
  if (!b->d_samp) return fail(BRAWL_EINVAL, "brawl_batch_sampling_reset first");
  const int n = (int)b->jobs.size();
  TRY(queue_batch_energy(b));
  launch_energy_accumulate(b->d_energy, b->d_sums, nullptr, n, b->stream);
  CUDA_TRY(cudaGetLastError());
  if (energies)
    CUDA_TRY(cudaMemcpyAsync(energies, b->d_energy, n * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

// The energy jobs of the live lattices and of the two snapshot buffers, the
// site-energy scratch, the snapshots and n_rows rows of sampled energies;
// returns the batch's total and largest site counts.
static int ensure_anneal_block(brawl_batch* b, int64_t n_rows, int64_t& total_sites, int& max_sites) {
  const int n = (int)b->jobs.size();
  total_sites = 0;
  max_sites = 0;
  for (int c = 0; c < n; ++c) {
    total_sites += b->models[c].g.n_sites;
    max_sites = std::max(max_sites, (int)b->models[c].g.n_sites);
  }
  if ((size_t)total_sites * 8 > b->site_e_cap) {
    dfree(b->d_site_e, b->stream);
    b->d_site_e = nullptr;
    b->site_e_cap = 0;
    CUDA_TRY(dalloc(&b->d_site_e, (size_t)total_sites * 8, b->stream));
    b->site_e_cap = (size_t)total_sites * 8;
  }
  const size_t jobs_bytes = ((size_t)3 * n * sizeof(EnergyJob) + 255) / 256 * 256;
  const size_t need = jobs_bytes + 2 * (size_t)total_sites;
  if (need > b->snap_cap) {
    dfree(b->d_snap, b->stream);
    b->d_snap = nullptr;
    b->snap_cap = 0;
    CUDA_TRY(dalloc(&b->d_snap, need, b->stream));
    b->snap_cap = need;
  }
  b->d_snap_jobs = reinterpret_cast<EnergyJob*>(b->d_snap);
  b->d_snap_lat = reinterpret_cast<int8_t*>(b->d_snap + jobs_bytes);
  if ((size_t)n_rows > b->traj_rows) {
    dfree(b->d_traj, b->stream);
    b->d_traj = nullptr;
    b->traj_rows = 0;
    CUDA_TRY(dalloc(&b->d_traj, (size_t)n_rows * n * 8, b->stream));
    b->traj_rows = (size_t)n_rows;
  }
  if (!b->energy_stream) {
    CUDA_TRY(object_stream(&b->energy_stream));
    for (cudaEvent_t* ev : {&b->ev_snap[0], &b->ev_snap[1], &b->ev_free[0], &b->ev_free[1]})
      CUDA_TRY(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  }
  std::vector<EnergyJob> ej((size_t)3 * n);
  int64_t off = 0;
  for (int c = 0; c < n; ++c) {
    EnergyJob j;
    j.g = b->models[c].g;
    j.lat = b->jobs[c].lat;
    j.V = b->jobs[c].V;
    j.entries = b->jobs[c].entries;
    j.shell_start = b->jobs[c].shell_start;
    j.site_energy = b->d_site_e + off;
    j.out = b->d_energy + c;
    j.site_offset = off;
    ej[c] = j;
    for (int k = 0; k < 2; ++k) {
      j.lat = b->d_snap_lat + (size_t)k * total_sites + off;
      ej[(size_t)(1 + k) * n + c] = j;
    }
    off += j.g.n_sites;
  }
  CUDA_TRY(cudaMemcpyAsync(b->d_snap_jobs, ej.data(), ej.size() * sizeof(EnergyJob), cudaMemcpyHostToDevice,
                           b->stream));
  return BRAWL_OK;
}

int brawl_batch_anneal_sweeps(brawl_batch* b, int64_t n_sweeps, int64_t sweep_trials, int accumulate,
                              double* energies, int64_t* accepted) {
  if (!b || n_sweeps < 0 || sweep_trials < 0 || sweep_trials > kMaxLaunchTrials)
    return fail(BRAWL_EINVAL, "bad argument");
  const int n = (int)b->jobs.size();
  if (n_sweeps > ((int64_t)1 << 28) / n) return fail(BRAWL_EINVAL, "too many sweeps for one block");
  if (accumulate && !b->d_samp) return fail(BRAWL_EINVAL, "brawl_batch_sampling_reset first");
  const bool sample = accumulate || energies;
  for (int c = 0; c < n; ++c) {
    b->jobs[c].n_trials = sweep_trials;
    b->jobs[c].nbr_swap = b->nbr_swap[c];
  }
  TRY(upload_jobs(b));
  int64_t total_sites = 0;
  int max_sites = 0;
  if (sample) TRY(ensure_anneal_block(b, std::max<int64_t>(n_sweeps, 1), total_sites, max_sites));
  cudaStream_t ms = b->stream, es = b->energy_stream;
  // sweep i's lattices go to snapshot buffer i % 2; its energies run on the
  // energy stream while sweep i + 1 runs, and the buffer is written again
  // (sweep i + 2) only after they have read it
  for (int64_t i = 0; i < n_sweeps; ++i) {
    TRY(launch_sweep(b, ms));
    if (!sample) continue;
    const int k = (int)(i & 1);
    if (i >= 2) CUDA_TRY(cudaStreamWaitEvent(ms, b->ev_free[k], 0));
    launch_lattice_snapshot(b->d_snap_jobs, b->d_snap_jobs + (size_t)(1 + k) * n, n, max_sites, ms);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(b->ev_snap[k], ms));
    CUDA_TRY(cudaStreamWaitEvent(es, b->ev_snap[k], 0));
    launch_total_energy(b->d_snap_jobs + (size_t)(1 + k) * n, n, total_sites, es);
    launch_energy_accumulate(b->d_energy, accumulate ? b->d_sums : nullptr,
                             energies ? b->d_traj + (size_t)i * n : nullptr, n, es);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(b->ev_free[k], es));
  }
  if (sample && n_sweeps > 0) {
    CUDA_TRY(cudaStreamWaitEvent(ms, b->ev_free[(n_sweeps - 1) & 1], 0));
    if (energies)
      CUDA_TRY(cudaMemcpyAsync(energies, b->d_traj, (size_t)n_sweeps * n * 8, cudaMemcpyDeviceToHost, ms));
  }
  CUDA_TRY(stream_wait(ms));
  std::vector<unsigned long long> cnt;
  TRY(read_counters(b, cnt));
  if (accepted)
    for (int c = 0; c < n; ++c)
      accepted[c] = (int64_t)(cnt[c * kNumCounters + kCntAccepted] -
                              b->last_counters[c * kNumCounters + kCntAccepted]);
  b->last_counters = cnt;
  return check_status(b);
}

int brawl_batch_asro_sample(brawl_batch* b, int c, const double* shells, double* rho) {
  if (!b || !shells || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad argument");
  if (!b->d_samp || b->samp_wc < 1)
    return fail(BRAWL_EINVAL, "brawl_batch_sampling_reset with wc_range >= 1 first");
  const Geom& g = b->models[c].g;
  const int wc = b->samp_wc;
  const size_t m = (size_t)wc * g.ns * g.ns;
  AsroPlan plan;
  unsigned long long* d_cnt = nullptr;
  TRY(queue_asro_counts(b, c, wc, shells, plan, &d_cnt));
  if (plan.n_class > 64) return fail(BRAWL_EINVAL, "too many ASRO offset classes");
  CUDA_TRY(cudaMemcpyAsync(b->d_mask, plan.class_mask.data(), plan.class_mask.size() * 8,
                           cudaMemcpyHostToDevice, b->stream));
  double* rho_out = b->d_rho_stats;  // staging for this sample
  launch_asro_finish(d_cnt, b->d_mask, plan.n_class, g.ns, wc, rho ? rho_out : nullptr,
                     b->d_rho_sum + (size_t)c * m, b->stream);
  CUDA_TRY(cudaGetLastError());
  if (rho) CUDA_TRY(cudaMemcpyAsync(rho, rho_out, m * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_temperature_stats(brawl_batch* b, int64_t n_save_energy, int64_t n_mc_steps, double temp,
                                  double sim_temp, int with_energies, double* per_chain, double* average) {
  if (!b || !per_chain || !average || n_mc_steps < 1 || (with_energies && n_save_energy < 1))
    return fail(BRAWL_EINVAL, "bad argument");
  if (!b->d_samp) return fail(BRAWL_EINVAL, "brawl_batch_sampling_reset first");
  const int n = (int)b->jobs.size();
  launch_temperature_stats(n, b->d_sums, b->d_counters, b->d_acc0, b->d_natoms, (double)n_save_energy,
                           sim_temp, temp, (double)(float)n_mc_steps, with_energies ? 1 : 0, b->d_tstats,
                           b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(per_chain, b->d_tstats, 3 * n * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaMemcpyAsync(average, b->d_tstats + 3 * n, 3 * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_batch_asro_stats(brawl_batch* b, int64_t n_save_asro, double* per_chain, double* average) {
  if (!b || !per_chain || !average || n_save_asro < 1) return fail(BRAWL_EINVAL, "bad argument");
  if (!b->d_samp || b->samp_wc < 1)
    return fail(BRAWL_EINVAL, "brawl_batch_sampling_reset with wc_range >= 1 first");
  const int n = (int)b->jobs.size();
  const int m = b->samp_wc * b->models[0].g.ns * b->models[0].g.ns;
  launch_asro_stats(n, m, b->d_rho_sum, (double)n_save_asro, b->d_rho_stats, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(per_chain, b->d_rho_stats, (size_t)n * m * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaMemcpyAsync(average, b->d_rho_stats + (size_t)n * m, (size_t)m * 8, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

// ---------------------------------------------------------------------------
// single chain
// ---------------------------------------------------------------------------
int brawl_ctx_create(const brawl_setup* setup, const double* V_ex, brawl_ctx** out) {
  if (!setup || !out) return fail(BRAWL_EINVAL, "null argument");
  *out = nullptr;
  Geom g;
  TRY(make_geom(*setup, g));
  // an empty lattice until set_config / initial_setup: all sites species 1
  std::vector<int8_t> grid((size_t)8 * setup->n_1 * setup->n_2 * setup->n_3, 0);
  {
    const int W1 = 2 * g.n1, W2 = 2 * g.n2;
    for (size_t t = 0; t < grid.size(); ++t) {
      int x = (int)(t % W1), y = (int)((t / W1) % W2), z = (int)(t / ((size_t)W1 * W2));
      bool occ = g.lattice == kBcc   ? (((x & 1) == (z & 1)) && ((y & 1) == (z & 1)))
                 : g.lattice == kFcc ? (((x + y + z) & 1) == 0)
                                     : true;
      grid[t] = occ ? 1 : 0;
    }
  }
  brawl_chain_desc d;
  std::memset(&d, 0, sizeof(d));
  d.setup = *setup;
  d.V_ex = V_ex;
  d.seed = 5489u;
  d.beta = 0.0;
  d.config = grid.data();
  brawl_batch* b = nullptr;
  TRY(brawl_batch_create(&d, 1, &b));
  *out = new brawl_ctx{b};
  return BRAWL_OK;
}

int brawl_ctx_destroy(brawl_ctx* ctx) {
  if (!ctx) return BRAWL_OK;
  brawl_batch_destroy(ctx->b);
  delete ctx;
  return BRAWL_OK;
}

int brawl_set_interactions(brawl_ctx* ctx, const double* V_ex) {
  if (!ctx || !V_ex) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = ctx->b;
  brawl_setup s = {b->models[0].g.lattice, b->models[0].g.n1, b->models[0].g.n2, b->models[0].g.n3,
                   b->models[0].g.ns, b->models[0].g.nsh};
  Model m;
  TRY(make_model(s, V_ex, m));
  ChainJob& j = b->jobs[0];
  CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(j.V), m.V.data(), m.V.size() * 8,
                           cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaMemcpyAsync(const_cast<int32_t*>(j.F), m.F.data(), m.F.size() * 4,
                           cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  const double beta = j.beta;
  b->models[0] = m;
  j.band = m.band;
  set_beta(j, m, beta);
  return BRAWL_OK;
}

int brawl_seed(brawl_ctx* ctx, uint32_t seed) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  uint32_t st[kMTN + 1];
  mt_seed_host(seed, st);
  return brawl_rng_set(ctx, st);
}

int brawl_f90_init_genrand(brawl_ctx* ctx, int seedtime, int my_rank, uint32_t job_id,
                           uint32_t* seed_out) {
  // src/mt19937ar.c:127-142
  uint32_t seed;
  if (seedtime) {
    seed = (uint32_t)time(nullptr);
    seed += 11u * (uint32_t)my_rank;
    seed += job_id;
    if (seed % 2 == 0) seed += 1;
  } else {
    seed = 110179u + 11u * (uint32_t)my_rank;
  }
  if (seed_out) *seed_out = seed;
  return brawl_seed(ctx, seed);
}

int brawl_rng_get(brawl_ctx* ctx, uint32_t state[625]) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_rng_get(ctx->b, 0, state);
}

int brawl_rng_set(brawl_ctx* ctx, const uint32_t state[625]) {
  if (!ctx || !state) return fail(BRAWL_EINVAL, "null argument");
  if (state[kMTN] > (uint32_t)kMTN) {
    // mti == N+1 means "never seeded": the reference then seeds with 5489
    if (state[kMTN] == (uint32_t)kMTN + 1) return brawl_seed(ctx, 5489u);
    return fail(BRAWL_EINVAL, "mti out of range");
  }
  brawl_batch* b = ctx->b;
  CUDA_TRY(cudaMemcpyAsync(b->jobs[0].rng, state, (kMTN + 1) * 4, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_genrand(brawl_ctx* ctx, int64_t n, double* out) {
  if (!ctx || (n > 0 && !out) || n < 0) return fail(BRAWL_EINVAL, "bad argument");
  // The stream is advanced on the host from the device state: the draws the
  // host needs (clone choices, exchange shuffles) are few.
  uint32_t st[kMTN + 1];
  TRY(brawl_rng_get(ctx, st));
  int pos = (int)st[kMTN];
  for (int64_t i = 0; i < n; ++i) {
    if (pos >= kMTN) {
      for (int k = 0; k < kMTN; ++k) {
        uint32_t y = (st[k] & 0x80000000u) | (st[(k + 1) % kMTN] & 0x7fffffffu);
        st[k] = st[(k + kMTM) % kMTN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      pos = 0;
    }
    uint32_t y = st[pos++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    out[i] = (double)y * (1.0 / 4294967296.0);
  }
  st[kMTN] = (uint32_t)pos;
  return brawl_rng_set(ctx, st);
}

int brawl_set_config(brawl_ctx* ctx, const int8_t* config) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_set_config(ctx->b, 0, config);
}

int brawl_get_config(brawl_ctx* ctx, int8_t* config) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_get_config(ctx->b, 0, config);
}

int brawl_initial_setup(brawl_ctx* ctx, double* conc, const int64_t* numbers) {
  if (!ctx || !conc) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = ctx->b;
  std::vector<double> c(conc, conc + b->models[0].g.ns + 1);
  InitJob ij;
  TRY(make_init_job(b->models[0], c.data(), numbers, ij));
  ij.lat = b->jobs[0].lat;
  ij.rng = b->jobs[0].rng;
  ij.counters = b->jobs[0].counters;
  ij.status = b->jobs[0].status;
  InitJob* d = nullptr;
  CUDA_TRY(dalloc(&d, sizeof(InitJob), b->stream));
  cudaMemcpyAsync(d, &ij, sizeof(ij), cudaMemcpyHostToDevice, b->stream);
  launch_initial_setup(d, 1, b->stream);
  dfree(d, b->stream);
  cudaError_t e = stream_wait(b->stream);
  if (e != cudaSuccess) return fail(BRAWL_ECUDA, cudaGetErrorString(e));
  TRY(check_status(b));
  std::copy(c.begin(), c.end(), conc);
  return BRAWL_OK;
}

int brawl_total_energy(brawl_ctx* ctx, double* energy) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_total_energy(ctx->b, energy);
}

static int site_from_idx(const Geom& g, const int idx[4], int& x, int& y, int& z) {
  if (idx[0] != 1) return fail(BRAWL_EINVAL, "basis index must be 1");
  x = idx[1] - 1;
  y = idx[2] - 1;
  z = idx[3] - 1;
  if (x < 0 || y < 0 || z < 0 || x >= 2 * g.n1 || y >= 2 * g.n2 || z >= 2 * g.n3)
    return fail(BRAWL_EINVAL, "site outside the lattice");
  bool occ = g.lattice == kBcc   ? (((x & 1) == (z & 1)) && ((y & 1) == (z & 1)))
             : g.lattice == kFcc ? (((x + y + z) & 1) == 0)
                                 : true;
  if (!occ) return fail(BRAWL_EINVAL, "site is not a lattice site");
  return BRAWL_OK;
}

int brawl_site_energy(brawl_ctx* ctx, const int idx[4], double* energy) {
  if (!ctx || !idx || !energy) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = ctx->b;
  int x, y, z;
  TRY(site_from_idx(b->models[0].g, idx, x, y, z));
  EnergyJob j;
  std::memset(&j, 0, sizeof(j));
  j.g = b->models[0].g;
  j.lat = b->jobs[0].lat;
  j.V = b->jobs[0].V;
  j.entries = b->jobs[0].entries;
  j.shell_start = b->jobs[0].shell_start;
  CUDA_TRY(cudaMemcpyAsync(b->d_ejobs, &j, sizeof(j), cudaMemcpyHostToDevice, b->stream));
  launch_site_energy(b->d_ejobs, x, y, z, b->d_energy, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(energy, b->d_energy, 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

int brawl_pair_energy(brawl_ctx* ctx, const int idx1[4], const int idx2[4], double* energy) {
  double e1, e2;
  TRY(brawl_site_energy(ctx, idx1, &e1));
  TRY(brawl_site_energy(ctx, idx2, &e2));
  *energy = e1 + e2;
  return BRAWL_OK;
}

int brawl_metropolis_run(brawl_ctx* ctx, double beta, int64_t n_trials, int nbr_swap,
                         int64_t* accepted) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = ctx->b;
  set_beta(b->jobs[0], b->models[0], beta);
  b->nbr_swap[0] = nbr_swap ? 1 : 0;
  return run_metropolis(b, &n_trials, accepted, false, b->stream, true);
}

int brawl_anneal_sweeps(brawl_ctx* ctx, double beta, int64_t n_sweeps, int64_t sweep_trials, int nbr_swap,
                        double* energies, int64_t* accepted) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = ctx->b;
  set_beta(b->jobs[0], b->models[0], beta);
  b->nbr_swap[0] = nbr_swap ? 1 : 0;
  return brawl_batch_anneal_sweeps(b, n_sweeps, sweep_trials, 0, energies, accepted);
}

int brawl_lattice_shells(brawl_ctx* ctx, int wc_range, double* shells) {
  if (!ctx || !shells || wc_range < 1) return fail(BRAWL_EINVAL, "bad argument");
  lattice_shells_host(ctx->b->models[0].g, wc_range, shells);
  return BRAWL_OK;
}

int brawl_batch_lattice_shells(brawl_batch* b, int c, int wc_range, double* shells) {
  if (!b || !shells || wc_range < 1 || c < 0 || c >= (int)b->jobs.size())
    return fail(BRAWL_EINVAL, "bad argument");
  lattice_shells_host(b->models[c].g, wc_range, shells);
  return BRAWL_OK;
}

int brawl_radial_densities(brawl_ctx* ctx, int wc_range, const double* shells, double* rho) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_radial_densities(ctx->b, 0, wc_range, shells, rho);
}

int brawl_counters(brawl_ctx* ctx, int64_t* counters) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_counters(ctx->b, counters);
}

int brawl_alro_add(brawl_ctx* ctx) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_alro_add(ctx->b);
}

int brawl_alro_reset(brawl_ctx* ctx) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_alro_reset(ctx->b);
}

int brawl_alro_get(brawl_ctx* ctx, double* order) {
  if (!ctx) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_alro_get(ctx->b, 0, order);
}

}  // extern "C"

namespace brawl {
int api_fail(int code, const std::string& msg) { return fail(code, msg); }
int api_make_geom(const brawl_setup& s, Geom& g) { return make_geom(s, g); }
}  // namespace brawl

// ---------------------------------------------------------------------------
// nested sampling
// ---------------------------------------------------------------------------
#include "ns_kernels.cuh"

struct brawl_ns {
  std::vector<Model> models;
  std::vector<NsRun> runs;               // host images
  std::vector<void*> allocs;
  NsRun* d_runs = nullptr;
  double* d_limits = nullptr;
  size_t limits_cap = 0;
  cudaStream_t stream = nullptr;
  uint32_t smem = 0;
  int max_z = 0;        // the kernel variant: entries per lane and D staged
  bool all_D = true;
};

extern "C" int brawl_ns_destroy(brawl_ns* ns) {
  if (!ns) return BRAWL_OK;
  if (ns->stream) {
    for (void* p : ns->allocs) dfree(p, ns->stream);
    dfree(ns->d_limits, ns->stream);
    stream_wait(ns->stream);
    cudaStreamDestroy(ns->stream);
  }
  delete ns;
  return BRAWL_OK;
}

extern "C" int brawl_ns_create(const brawl_ns_desc* descs, int n_runs, brawl_ns** out) {
  if (!descs || !out || n_runs < 1) return fail(BRAWL_EINVAL, "no runs");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(BRAWL_ECUDA, "no CUDA device");
  brawl_ns* ns = new brawl_ns();
  auto cleanup = [&](int rc) {
    brawl_ns_destroy(ns);
    return rc;
  };
  if (object_stream(&ns->stream) != cudaSuccess)
    return cleanup(fail(BRAWL_ECUDA, "stream create failed"));
  int max_optin = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  ns->models.resize(n_runs);
  ns->runs.resize(n_runs);
  int64_t total_sites = 0;
  int max_K = 0;
  for (int r = 0; r < n_runs; ++r) {
    const brawl_ns_desc& d = descs[r];
    Model& m = ns->models[r];
    int rc = make_model(d.setup, d.V_ex, m);
    if (rc != BRAWL_OK) return cleanup(fail(rc, "run " + std::to_string(r) + ": " + g_err));
    if (d.n_walkers < 1 || d.n_steps < 0 || !d.species_concentrations)
      return cleanup(fail(BRAWL_EINVAL, "run " + std::to_string(r) + ": bad n_walkers/n_steps/concentrations"));
    NsRun& R = ns->runs[r];
    std::memset(&R, 0, sizeof(R));
    R.lazy_cap = lazy_cap_for(m.g, ns_smem_bytes(m.g, 0), (uint32_t)max_optin);
    if (R.lazy_cap == 0)
      return cleanup(fail(BRAWL_EINVAL, "run " + std::to_string(r) + ": lattice too large for shared memory"));
    ns->smem = std::max(ns->smem, ns_smem_bytes(m.g, R.lazy_cap));
    ns->max_z = std::max(ns->max_z, (int)m.g.z);
    ns->all_D = ns->all_D && walker_layout(m.g, 0, R.lazy_cap).use_D;
    std::vector<double> conc(d.species_concentrations, d.species_concentrations + m.g.ns + 1);
    rc = make_init_job(m, conc.data(), d.species_numbers, R.init);
    if (rc != BRAWL_OK) return cleanup(fail(rc, "run " + std::to_string(r) + ": " + g_err));
    R.K = d.n_walkers;
    R.n_steps = d.n_steps;
    R.n_at = d.setup.n_1 * d.setup.n_2 * d.setup.n_3 * 1 * d.setup.n_species;
    R.half = (int)((float)d.n_walkers / 2.0f);
    R.S = m.S;
    total_sites += (int64_t)R.K * m.g.n_sites;
    max_K = std::max(max_K, R.K);
  }
  if (ns->smem > (uint32_t)max_optin)
    return cleanup(fail(BRAWL_EINVAL, "a run's lattice and tables exceed shared memory"));
  auto nsalloc = [&](size_t bytes, void** p) -> int {
    cudaError_t e = dalloc(p, bytes, ns->stream);
    if (e != cudaSuccess) return fail(BRAWL_ENOMEM, cudaGetErrorString(e));
    ns->allocs.push_back(*p);
    return BRAWL_OK;
  };
  for (int r = 0; r < n_runs; ++r) {
    const Model& m = ns->models[r];
    NsRun& R = ns->runs[r];
    ChainJob& j = R.job;
    j.g = m.g;
    j.band = m.band;
    void *pV, *pF, *pE, *pS, *pRng, *pCnt, *pSt, *pW, *pEn, *pRn;
    int rc = BRAWL_OK;
    rc |= nsalloc(m.V.size() * 8, &pV);
    rc |= nsalloc(m.F.size() * 4, &pF);
    rc |= nsalloc(m.entries.size() * 4, &pE);
    rc |= nsalloc(m.sstart.size() * 2, &pS);
    rc |= nsalloc((kMTN + 1) * 4, &pRng);
    rc |= nsalloc(kNumCounters * 8, &pCnt);
    rc |= nsalloc(4, &pSt);
    rc |= nsalloc((size_t)R.K * m.g.n_sites, &pW);
    rc |= nsalloc((size_t)R.K * 8, &pEn);
    rc |= nsalloc((size_t)R.K * 4, &pRn);
    if (rc != BRAWL_OK) return cleanup(BRAWL_ENOMEM);
    uint32_t st[kMTN + 1];
    mt_seed_host(descs[r].seed, st);
    cudaMemcpyAsync(pV, m.V.data(), m.V.size() * 8, cudaMemcpyHostToDevice, ns->stream);
    cudaMemcpyAsync(pF, m.F.data(), m.F.size() * 4, cudaMemcpyHostToDevice, ns->stream);
    cudaMemcpyAsync(pE, m.entries.data(), m.entries.size() * 4, cudaMemcpyHostToDevice, ns->stream);
    cudaMemcpyAsync(pS, m.sstart.data(), m.sstart.size() * 2, cudaMemcpyHostToDevice, ns->stream);
    cudaMemcpyAsync(pRng, st, sizeof(st), cudaMemcpyHostToDevice, ns->stream);
    cudaMemsetAsync(pCnt, 0, kNumCounters * 8, ns->stream);
    cudaMemsetAsync(pSt, 0, 4, ns->stream);
    CUDA_TRY(stream_wait(ns->stream));
    j.V = (const double*)pV;
    j.F = (const int32_t*)pF;
    j.entries = (const uint32_t*)pE;
    j.shell_start = (const int16_t*)pS;
    j.rng = (uint32_t*)pRng;
    j.counters = (unsigned long long*)pCnt;
    j.status = (int32_t*)pSt;
    R.init.n_sites = m.g.n_sites;
    R.init.ns = m.g.ns;
    R.init.counters = j.counters;
    R.init.status = j.status;
    R.walkers = (int8_t*)pW;
    R.energies = (double*)pEn;
    R.rnde = (uint32_t*)pRn;
  }
  void* pRuns;
  if (nsalloc(n_runs * sizeof(NsRun), &pRuns) != BRAWL_OK) return cleanup(BRAWL_ENOMEM);
  ns->d_runs = (NsRun*)pRuns;
  CUDA_TRY(cudaMemcpyAsync(ns->d_runs, ns->runs.data(), n_runs * sizeof(NsRun), cudaMemcpyHostToDevice, ns->stream));
  launch_ns_init(ns->d_runs, n_runs, ns->stream);
  // walker energies: total_energy of every walker, then the jitter
  void *pSite, *pEj;
  if (nsalloc((size_t)total_sites * 8, &pSite) != BRAWL_OK) return cleanup(BRAWL_ENOMEM);
  std::vector<EnergyJob> ej;
  int64_t off = 0;
  for (int r = 0; r < n_runs; ++r) {
    const NsRun& R = ns->runs[r];
    for (int w = 0; w < R.K; ++w) {
      EnergyJob e;
      std::memset(&e, 0, sizeof(e));
      e.g = R.job.g;
      e.lat = R.walkers + (size_t)w * R.job.g.n_sites;
      e.V = R.job.V;
      e.entries = R.job.entries;
      e.shell_start = R.job.shell_start;
      e.site_energy = (double*)pSite + off;
      e.out = R.energies + w;
      e.site_offset = off;
      off += R.job.g.n_sites;
      ej.push_back(e);
    }
  }
  if (nsalloc(ej.size() * sizeof(EnergyJob), &pEj) != BRAWL_OK) return cleanup(BRAWL_ENOMEM);
  CUDA_TRY(cudaMemcpyAsync(pEj, ej.data(), ej.size() * sizeof(EnergyJob), cudaMemcpyHostToDevice, ns->stream));
  launch_total_energy((EnergyJob*)pEj, (int)ej.size(), total_sites, ns->stream);
  launch_ns_jitter(ns->d_runs, n_runs, max_K, ns->stream);
  cudaError_t e = stream_wait(ns->stream);
  if (e != cudaSuccess) return cleanup(fail(BRAWL_ECUDA, cudaGetErrorString(e)));
  // the per-site scratch is only needed at set-up
  dfree(pSite, ns->stream);
  dfree(pEj, ns->stream);
  ns->allocs.erase(std::remove(ns->allocs.begin(), ns->allocs.end(), pSite), ns->allocs.end());
  ns->allocs.erase(std::remove(ns->allocs.begin(), ns->allocs.end(), pEj), ns->allocs.end());
  for (int r = 0; r < n_runs; ++r) {
    int32_t st = 0;
    cudaMemcpyAsync(&st, ns->runs[r].job.status, 4, cudaMemcpyDeviceToHost, ns->stream);
    stream_wait(ns->stream);
    if (st) return cleanup(fail(BRAWL_ESTATE, "walker initialisation failed on run " + std::to_string(r)));
  }
  *out = ns;
  return BRAWL_OK;
}

extern "C" int brawl_ns_iterate(brawl_ns* ns, int n_iter, double* limits) {
  if (!ns || n_iter < 0) return fail(BRAWL_EINVAL, "bad argument");
  if (n_iter == 0) return BRAWL_OK;
  const int n_runs = (int)ns->runs.size();
  const size_t need = (size_t)n_runs * n_iter * 8;
  if (need > ns->limits_cap) {
    dfree(ns->d_limits, ns->stream);
    ns->d_limits = nullptr;
    ns->limits_cap = 0;
    CUDA_TRY(dalloc(&ns->d_limits, need, ns->stream));
    ns->limits_cap = need;
  }
  // the device-side run state (iteration counters) is authoritative: read it back
  std::vector<NsRun> cur(n_runs);
  CUDA_TRY(cudaMemcpyAsync(cur.data(), ns->d_runs, n_runs * sizeof(NsRun), cudaMemcpyDeviceToHost, ns->stream));
  CUDA_TRY(stream_wait(ns->stream));
  for (int r = 0; r < n_runs; ++r) {
    cur[r].limits = ns->d_limits + (size_t)r * n_iter;
    cur[r].n_iter = n_iter;
  }
  CUDA_TRY(cudaMemcpyAsync(ns->d_runs, cur.data(), n_runs * sizeof(NsRun), cudaMemcpyHostToDevice, ns->stream));
  launch_ns_iterate(ns->d_runs, n_runs, ns->smem, ns->max_z, ns->all_D, ns->stream);
  CUDA_TRY(cudaGetLastError());
  if (limits)
    CUDA_TRY(cudaMemcpyAsync(limits, ns->d_limits, need, cudaMemcpyDeviceToHost, ns->stream));
  CUDA_TRY(stream_wait(ns->stream));
  for (int r = 0; r < n_runs; ++r) {
    int32_t st = 0;
    CUDA_TRY(cudaMemcpy(&st, ns->runs[r].job.status, 4, cudaMemcpyDeviceToHost));
    if (st) return fail(BRAWL_ESTATE, "nested sampling check failed on run " + std::to_string(r));
  }
  return BRAWL_OK;
}

extern "C" int brawl_ns_energies(brawl_ns* ns, int run, double* energies) {
  if (!ns || !energies || run < 0 || run >= (int)ns->runs.size()) return fail(BRAWL_EINVAL, "bad argument");
  CUDA_TRY(cudaMemcpy(energies, ns->runs[run].energies, ns->runs[run].K * 8, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

extern "C" int brawl_ns_walker_config(brawl_ns* ns, int run, int walker, int8_t* config) {
  if (!ns || !config || run < 0 || run >= (int)ns->runs.size()) return fail(BRAWL_EINVAL, "bad argument");
  const NsRun& R = ns->runs[run];
  if (walker < 0 || walker >= R.K) return fail(BRAWL_EINVAL, "bad walker");
  const Geom& g = R.job.g;
  const size_t grid = (size_t)8 * g.n1 * g.n2 * g.n3;
  int8_t* d_grid = nullptr;
  CUDA_TRY(dalloc(&d_grid, grid, ns->stream));
  launch_unpack(g, R.walkers + (size_t)walker * g.n_sites, d_grid, ns->stream);
  cudaError_t e = cudaMemcpyAsync(config, d_grid, grid, cudaMemcpyDeviceToHost, ns->stream);
  dfree(d_grid, ns->stream);
  if (e == cudaSuccess) e = stream_wait(ns->stream);
  if (e != cudaSuccess) return fail(BRAWL_ECUDA, cudaGetErrorString(e));
  return BRAWL_OK;
}

extern "C" int brawl_ns_counters(brawl_ns* ns, int run, int64_t* counters) {
  if (!ns || !counters || run < 0 || run >= (int)ns->runs.size()) return fail(BRAWL_EINVAL, "bad argument");
  CUDA_TRY(cudaMemcpy(counters, ns->runs[run].job.counters, kNumCounters * 8, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

// ---------------------------------------------------------------------------
// Wang-Landau walkers: a batch (lattices, streams, tables, energies) plus
// ln g and histogram buffers.
// ---------------------------------------------------------------------------
#include "wl_kernels.cuh"

struct brawl_wl {
  brawl_batch* b = nullptr;
  int bins = 0;
  double e1 = 0.0, range = 0.0;
  std::vector<double> edges;             // bin_edges (bins + 1)
  std::vector<WlWalker> w;
  std::vector<WlGroup> groups;
  WlWalker* d_w = nullptr;
  WlGroup* d_groups = nullptr;
  double* d_lng = nullptr;
  double* d_hist = nullptr;
  uint32_t smem = 0;
  int max_z = 0;        // the kernel variant: entries per lane and D staged
  bool all_D = true;
  // radial-density samples (brawl_wl_radial_enable)
  int rad_wc = 0, rad_n_off = 0, rad_n_class = 0;
  WlRadial* d_rad = nullptr;
  uint32_t* d_rad_offsets = nullptr;
  unsigned long long* d_rad_masks = nullptr;
  uint8_t* d_rad_done = nullptr;
  int32_t* d_rad_record = nullptr;
  double* d_rad_rho = nullptr;
  int32_t* d_rad_steps = nullptr;
  // exchange / flatness / combine scratch
  int per_window = 0;                    // walkers per window when all windows have as many
  int* d_ibin = nullptr;
  int2* d_ov = nullptr;
  int* d_partner = nullptr;
  int* d_exchanged = nullptr;
  int* d_nacc = nullptr;
  double* d_flat = nullptr;
  double* d_combined = nullptr;
  // configuration store (brawl_wl_store_enable): every walker's bins slots,
  // their open flags (walker-major) and merge_configs' picks
  int8_t* d_store = nullptr;
  uint8_t* d_store_open = nullptr;
  int* d_pick = nullptr;
};

namespace {
int batch_genrand(brawl_batch* b, int c, int64_t n, double* out) {
  uint32_t st[kMTN + 1];
  TRY(brawl_batch_rng_get(b, c, st));
  int pos = (int)st[kMTN];
  for (int64_t i = 0; i < n; ++i) {
    if (pos >= kMTN) {
      for (int k = 0; k < kMTN; ++k) {
        uint32_t y = (st[k] & 0x80000000u) | (st[(k + 1) % kMTN] & 0x7fffffffu);
        st[k] = st[(k + kMTM) % kMTN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      pos = 0;
    }
    uint32_t y = st[pos++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    out[i] = (double)y * (1.0 / 4294967296.0);
  }
  st[kMTN] = (uint32_t)pos;
  CUDA_TRY(cudaMemcpyAsync(b->jobs[c].rng, st, sizeof(st), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}
}  // namespace

extern "C" int brawl_wl_destroy(brawl_wl* wl) {
  if (!wl) return BRAWL_OK;
  if (wl->b) {
    // freed on the batch's stream, which the batch's destruction then drains
    for (const void* p : {(const void*)wl->d_w, (const void*)wl->d_groups, (const void*)wl->d_lng,
                          (const void*)wl->d_hist, (const void*)wl->d_ibin, (const void*)wl->d_ov,
                          (const void*)wl->d_partner, (const void*)wl->d_exchanged, (const void*)wl->d_nacc,
                          (const void*)wl->d_flat, (const void*)wl->d_combined, (const void*)wl->d_rad,
                          (const void*)wl->d_rad_offsets, (const void*)wl->d_rad_masks,
                          (const void*)wl->d_rad_done, (const void*)wl->d_rad_record,
                          (const void*)wl->d_rad_rho, (const void*)wl->d_rad_steps,
                          (const void*)wl->d_store, (const void*)wl->d_store_open, (const void*)wl->d_pick})
      dfree(p, wl->b->stream);
    brawl_batch_destroy(wl->b);
  }
  delete wl;
  return BRAWL_OK;
}

extern "C" int brawl_wl_create(const brawl_wl_desc* walkers, int n, int bins,
                               const double* bin_edges, brawl_wl** out) {
  if (!walkers || !out || n < 1 || bins < 1 || !bin_edges) return fail(BRAWL_EINVAL, "bad argument");
  *out = nullptr;
  for (int c = 0; c < n; ++c) {
    if (!walkers[c].config) return fail(BRAWL_EINVAL, "walker " + std::to_string(c) + ": config required");
    if (walkers[c].start_idx < 1 || walkers[c].end_idx > bins || walkers[c].start_idx > walkers[c].end_idx)
      return fail(BRAWL_EINVAL, "walker " + std::to_string(c) + ": window outside 1..bins");
    for (int k = 0; k < c; ++k)
      if (walkers[k].window == walkers[c].window && walkers[c - 1].window != walkers[c].window)
        return fail(BRAWL_EINVAL, "walkers of a window must be consecutive");
  }
  std::vector<brawl_chain_desc> d(n);
  for (int c = 0; c < n; ++c) {
    std::memset(&d[c], 0, sizeof(d[c]));
    d[c].setup = walkers[c].setup;
    d[c].V_ex = walkers[c].V_ex;
    d[c].seed = walkers[c].seed;
    d[c].config = walkers[c].config;
    d[c].nbr_swap = walkers[c].nbr_swap ? 1 : 0;
  }
  brawl_wl* wl = new brawl_wl();
  auto cleanup = [&](int rc) {
    brawl_wl_destroy(wl);
    return rc;
  };
  int rc = brawl_batch_create(d.data(), n, &wl->b);
  if (rc != BRAWL_OK) return cleanup(rc);
  wl->bins = bins;
  wl->e1 = bin_edges[0];
  wl->edges.assign(bin_edges, bin_edges + bins + 1);
  wl->range = bin_edges[bins] - bin_edges[0];
  size_t hist_total = 0;
  for (int c = 0; c < n; ++c) hist_total += walkers[c].end_idx - walkers[c].start_idx + 1;
  cudaStream_t ws = wl->b->stream;
  if (dalloc(&wl->d_lng, (size_t)n * bins * 8, ws) != cudaSuccess ||
      dalloc(&wl->d_hist, hist_total * 8, ws) != cudaSuccess ||
      dalloc(&wl->d_w, n * sizeof(WlWalker), ws) != cudaSuccess)
    return cleanup(fail(BRAWL_ENOMEM, "walker buffers"));
  cudaMemsetAsync(wl->d_lng, 0, (size_t)n * bins * 8, ws);
  cudaMemsetAsync(wl->d_hist, 0, hist_total * 8, ws);
  wl->w.resize(n);
  size_t hoff = 0;
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, wl->b->device);
  for (int c = 0; c < n; ++c) {
    WlWalker& W = wl->w[c];
    std::memset(&W, 0, sizeof(W));
    W.job = wl->b->jobs[c];
    W.S = wl->b->models[c].S;
    W.lng = wl->d_lng + (size_t)c * bins;
    W.hist = wl->d_hist + hoff;
    W.start = walkers[c].start_idx;
    W.end = walkers[c].end_idx;
    W.bins = bins;
    W.e1 = wl->e1;
    W.range = wl->range;
    hoff += W.end - W.start + 1;
    const uint32_t base = wl_smem_bytes(W.job.g, W.end - W.start + 1, 0);
    W.lazy_cap = lazy_cap_for(W.job.g, base, (uint32_t)max_optin);
    if (W.lazy_cap == 0) return cleanup(fail(BRAWL_EINVAL, "window or lattice too large for shared memory"));
    wl->smem = std::max(wl->smem, wl_smem_bytes(W.job.g, W.end - W.start + 1, W.lazy_cap));
    wl->max_z = std::max(wl->max_z, (int)W.job.g.z);
    wl->all_D = wl->all_D && walker_layout(W.job.g, W.end - W.start + 1, W.lazy_cap).use_D;
    if (c == 0 || walkers[c].window != walkers[c - 1].window) wl->groups.push_back({c, 0});
    wl->groups.back().count += 1;
  }
  if (wl->smem > (uint32_t)max_optin) return cleanup(fail(BRAWL_EINVAL, "window or lattice too large for shared memory"));
  if (dalloc(&wl->d_groups, wl->groups.size() * sizeof(WlGroup), ws) != cudaSuccess)
    return cleanup(fail(BRAWL_ENOMEM, "groups"));
  wl->per_window = wl->groups[0].count;
  for (const WlGroup& G : wl->groups)
    if (G.count != wl->per_window) wl->per_window = 0;
  if (dalloc(&wl->d_ibin, n * sizeof(int), ws) != cudaSuccess ||
      dalloc(&wl->d_ov, n * sizeof(int2), ws) != cudaSuccess ||
      dalloc(&wl->d_partner, n * sizeof(int), ws) != cudaSuccess ||
      dalloc(&wl->d_exchanged, n * sizeof(int), ws) != cudaSuccess ||
      dalloc(&wl->d_nacc, 2 * sizeof(int), ws) != cudaSuccess ||
      dalloc(&wl->d_flat, n * sizeof(double), ws) != cudaSuccess ||
      dalloc(&wl->d_combined, (size_t)bins * sizeof(double), ws) != cudaSuccess)
    return cleanup(fail(BRAWL_ENOMEM, "exchange buffers"));
  cudaMemcpyAsync(wl->d_groups, wl->groups.data(), wl->groups.size() * sizeof(WlGroup), cudaMemcpyHostToDevice, ws);
  if (stream_wait(ws) != cudaSuccess) return cleanup(fail(BRAWL_ECUDA, "walker set-up"));
  *out = wl;
  return BRAWL_OK;
}

extern "C" int brawl_wl_sweeps(brawl_wl* wl, int64_t n_trials, double wl_f, int hist_period,
                               int64_t* accepted) {
  if (!wl || n_trials < 0 || n_trials > 0x7fffffff) return fail(BRAWL_EINVAL, "n_trials must be 0 .. 2^31-1");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  TRY(queue_batch_energy(b));
  for (int c = 0; c < n; ++c) {
    WlWalker& W = wl->w[c];
    W.e0_src = b->d_energy + c;
    W.wl_f = wl_f;
    W.n_trials = n_trials;
    W.hist_period = hist_period;
  }
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), n * sizeof(WlWalker), cudaMemcpyHostToDevice, b->stream));
  launch_wl_sweeps(wl->d_w, n, wl->smem, wl->max_z, wl->all_D, b->stream);
  launch_wl_average(wl->d_groups, (int)wl->groups.size(), wl->d_w, wl->bins, 1, b->stream);
  CUDA_TRY(cudaGetLastError());
  std::vector<WlWalker> res(n);
  CUDA_TRY(cudaMemcpyAsync(res.data(), wl->d_w, n * sizeof(WlWalker), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  if (accepted)
    for (int c = 0; c < n; ++c) accepted[c] = res[c].accepted;
  int r = check_status(b);
  if (r != BRAWL_OK) return fail(BRAWL_ESTATE, "a walker's energy is outside its window");
  return BRAWL_OK;
}

extern "C" int brawl_wl_average(brawl_wl* wl) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), wl->w.size() * sizeof(WlWalker), cudaMemcpyHostToDevice, wl->b->stream));
  launch_wl_average(wl->d_groups, (int)wl->groups.size(), wl->d_w, wl->bins, 0, wl->b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(stream_wait(wl->b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_replica_exchange(brawl_wl* wl, int* partner, int* exchanged,
                                         int* n_accepted) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  if (wl->per_window <= 0)
    return fail(BRAWL_EINVAL, "replica exchange needs the same number of walkers in every window");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  const Geom& g0 = b->models[0].g;
  for (int c = 1; c < n; ++c) {
    const Geom& g = b->models[c].g;
    if (g.lattice != g0.lattice || g.n1 != g0.n1 || g.n2 != g0.n2 || g.n3 != g0.n3)
      return fail(BRAWL_EINVAL, "walkers have different lattices");
  }
  TRY(queue_batch_energy(b));
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), n * sizeof(WlWalker), cudaMemcpyHostToDevice, b->stream));
  launch_wl_exchange(wl->d_w, b->d_energy, wl->d_groups, (int)wl->groups.size(), wl->per_window,
                     wl->d_ibin, wl->d_ov, wl->d_partner, wl->d_exchanged, wl->d_nacc, b->stream);
  CUDA_TRY(cudaGetLastError());
  int nacc = 0;
  CUDA_TRY(cudaMemcpyAsync(&nacc, wl->d_nacc, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  if (partner)
    CUDA_TRY(cudaMemcpyAsync(partner, wl->d_partner, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  if (exchanged)
    CUDA_TRY(cudaMemcpyAsync(exchanged, wl->d_exchanged, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  if (n_accepted) *n_accepted = nacc;
  return BRAWL_OK;
}

extern "C" int brawl_wl_flatness(brawl_wl* wl, double* flatness) {
  if (!wl || !flatness) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), n * sizeof(WlWalker), cudaMemcpyHostToDevice, b->stream));
  launch_wl_flatness(wl->d_w, n, wl->d_flat, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(flatness, wl->d_flat, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_dos_combine(brawl_wl* wl, double* lng) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), n * sizeof(WlWalker), cudaMemcpyHostToDevice, b->stream));
  launch_wl_combine(wl->d_w, n, wl->d_groups, (int)wl->groups.size(), wl->bins, wl->d_combined,
                    wl->d_nacc + 1, b->stream);
  CUDA_TRY(cudaGetLastError());
  int status = 0;
  CUDA_TRY(cudaMemcpyAsync(&status, wl->d_nacc + 1, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  if (lng)
    CUDA_TRY(cudaMemcpyAsync(lng, wl->d_combined, (size_t)wl->bins * 8, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  if (status != 0) return fail(BRAWL_ESTATE, "a window has no overlap with the previous one");
  return BRAWL_OK;
}

extern "C" int brawl_wl_reset_hist(brawl_wl* wl) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  size_t total = 0;
  for (const WlWalker& W : wl->w) total += W.end - W.start + 1;
  CUDA_TRY(cudaMemsetAsync(wl->d_hist, 0, total * 8, wl->b->stream));
  CUDA_TRY(stream_wait(wl->b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_enter_windows(brawl_wl* wl, double energy_min, double energy_max,
                                      const double* conc, const int64_t* numbers, int initial,
                                      int64_t max_steps, int64_t* steps) {
  if (!wl || !conc || max_steps < 1) return fail(BRAWL_EINVAL, "bad argument");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  cudaStream_t s = b->stream;
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  std::vector<WlEnterJob> jobs(n);
  uint32_t smem = 0;
  int64_t scratch = 0;
  std::vector<int64_t> off(n);
  for (int c = 0; c < n; ++c) {
    off[c] = scratch;
    scratch += b->models[c].g.n_sites;
  }
  double* d_site_e = nullptr;
  WlEnterJob* d_jobs = nullptr;
  if (dalloc(&d_site_e, (size_t)scratch * 8, s) != cudaSuccess ||
      dalloc(&d_jobs, (size_t)n * sizeof(WlEnterJob), s) != cudaSuccess) {
    dfree(d_site_e, s);
    return fail(BRAWL_ENOMEM, "burn-in scratch");
  }
  auto cleanup = [&](int rc) {
    dfree(d_site_e, s);
    dfree(d_jobs, s);
    return rc;
  };
  for (int c = 0; c < n; ++c) {
    const Model& m = b->models[c];
    WlEnterJob& E = jobs[c];
    std::memset(&E, 0, sizeof(E));
    E.job = b->jobs[c];
    std::vector<double> cc(conc, conc + m.g.ns + 1);
    int rc = make_init_job(m, cc.data(), numbers, E.init);
    if (rc != BRAWL_OK) return cleanup(fail(rc, "walker " + std::to_string(c) + ": " + g_err));
    E.init.lat = E.job.lat;
    E.init.rng = E.job.rng;
    E.init.counters = E.job.counters;
    E.init.status = E.job.status;
    const WlWalker& W = wl->w[c];
    E.min_e = wl->edges[W.start - 1];
    E.max_e = wl->edges[W.end];
    // (2.0 * (0.0025 * ABS(energy_max - energy_min) * n_atoms / (Ry_to_eV * 1000))**2):
    // energy_min/max and 0.0025 are default (single precision) reals, so the
    // product up to n_atoms is single precision; the division by the double
    // Ry_to_eV * 1000 and the rest are double
    const float d4 = std::fabs((float)energy_max - (float)energy_min);
    const float x4 = (0.0025f * d4) * (float)m.g.n_sites;
    const double x = (double)x4 / (13.605693122 * 1000.0);
    E.sig2x2 = 2.0 * (x * x);
    E.max_steps = max_steps;
    E.site_e = d_site_e + off[c];
    E.initial = initial ? 1 : 0;
    smem = std::max(smem, wl_enter_smem_bytes(m.g));
  }
  if (smem > (uint32_t)max_optin) return cleanup(fail(BRAWL_EINVAL, "lattice too large for the burn-in kernel"));
  CUDA_TRY(cudaMemcpyAsync(d_jobs, jobs.data(), (size_t)n * sizeof(WlEnterJob), cudaMemcpyHostToDevice, s));
  launch_wl_enter(d_jobs, n, smem, s);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(jobs.data(), d_jobs, (size_t)n * sizeof(WlEnterJob), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(stream_wait(s));
  cleanup(BRAWL_OK);
  int rc = check_status(b);
  if (rc != BRAWL_OK) return rc;
  bool all = true;
  for (int c = 0; c < n; ++c) {
    if (steps) steps[c] = jobs[c].steps;
    all = all && jobs[c].steps > 0;
  }
  if (!all) return fail(BRAWL_ESTATE, "a walker did not enter its window within max_steps");
  return BRAWL_OK;
}

extern "C" int brawl_wl_radial_enable(brawl_wl* wl, int wc_range, const double* shells,
                                      int radial_samples, int num_walkers) {
  if (!wl || !shells || wc_range < 1 || wc_range > 64 || num_walkers < 1 || radial_samples < 0)
    return fail(BRAWL_EINVAL, "bad argument");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  const Geom& g0 = b->models[0].g;
  for (int c = 1; c < n; ++c) {
    const Geom& g = b->models[c].g;
    if (g.lattice != g0.lattice || g.n1 != g0.n1 || g.n2 != g0.n2 || g.n3 != g0.n3 || g.ns != g0.ns)
      return fail(BRAWL_EINVAL, "radial samples need walkers on one lattice");
  }
  if (wl->d_rad) return fail(BRAWL_EINVAL, "radial samples already enabled");
  AsroPlan plan;
  if (make_asro_plan(g0, wc_range, shells, plan) != 0) return fail(BRAWL_EINVAL, "bad ASRO shells");
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  const int n_off = (int)plan.offsets.size(), n_class = plan.n_class;
  uint32_t smem = 0;
  for (const WlWalker& W : wl->w)
    smem = std::max(smem, wl_smem_bytes(W.job.g, W.end - W.start + 1, W.lazy_cap, wl->bins, n_off, n_class));
  if (smem > (uint32_t)max_optin) return fail(BRAWL_EINVAL, "radial-sample scratch does not fit in shared memory");
  const size_t per = (size_t)g0.ns * g0.ns * wc_range;
  cudaStream_t s = b->stream;
  std::vector<unsigned long long> masks(plan.class_mask.begin(), plan.class_mask.end());
  if (masks.empty()) masks.push_back(0ull);
  if (dalloc(&wl->d_rad, sizeof(WlRadial), s) != cudaSuccess ||
      dalloc(&wl->d_rad_offsets, std::max<size_t>(n_off, 1) * 4, s) != cudaSuccess ||
      dalloc(&wl->d_rad_masks, masks.size() * 8, s) != cudaSuccess ||
      dalloc(&wl->d_rad_done, (size_t)wl->bins, s) != cudaSuccess ||
      dalloc(&wl->d_rad_record, (size_t)n * wl->bins * 4, s) != cudaSuccess ||
      dalloc(&wl->d_rad_rho, (size_t)n * wl->bins * per * 8, s) != cudaSuccess ||
      dalloc(&wl->d_rad_steps, (size_t)n * 4, s) != cudaSuccess)
    return fail(BRAWL_ENOMEM, "radial-sample arrays");
  WlRadial R;
  R.offsets = wl->d_rad_offsets;
  R.class_masks = wl->d_rad_masks;
  R.done = wl->d_rad_done;
  R.n_offsets = n_off;
  R.n_class = n_class;
  R.wc_range = wc_range;
  R.cap = std::max(radial_samples / num_walkers, 1);
  if (n_off > 0)
    CUDA_TRY(cudaMemcpyAsync(wl->d_rad_offsets, plan.offsets.data(), (size_t)n_off * 4, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(wl->d_rad_masks, masks.data(), masks.size() * 8, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(wl->d_rad, &R, sizeof(R), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemsetAsync(wl->d_rad_done, 0, (size_t)wl->bins, s));
  CUDA_TRY(cudaMemsetAsync(wl->d_rad_record, 0, (size_t)n * wl->bins * 4, s));
  CUDA_TRY(cudaMemsetAsync(wl->d_rad_rho, 0, (size_t)n * wl->bins * per * 8, s));
  CUDA_TRY(cudaMemsetAsync(wl->d_rad_steps, 0, (size_t)n * 4, s));
  CUDA_TRY(stream_wait(s));
  wl->rad_wc = wc_range;
  wl->rad_n_off = n_off;
  wl->rad_n_class = n_class;
  wl->smem = std::max(wl->smem, smem);
  for (int c = 0; c < n; ++c) {
    WlWalker& W = wl->w[c];
    W.radial = wl->d_rad;
    W.radial_record = wl->d_rad_record + (size_t)c * wl->bins;
    W.rho_of_E = wl->d_rad_rho + (size_t)c * wl->bins * per;
    W.radial_steps = wl->d_rad_steps + c;
    W.rad_n_offsets = n_off;
    W.rad_n_class = n_class;
  }
  return BRAWL_OK;
}

extern "C" int brawl_wl_radial_set_done(brawl_wl* wl, const uint8_t* done) {
  if (!wl || !done) return fail(BRAWL_EINVAL, "bad argument");
  if (!wl->d_rad) return fail(BRAWL_EINVAL, "radial samples not enabled");
  bool all = true;
  for (int k = 0; k < wl->bins; ++k) all = all && done[k] != 0;
  CUDA_TRY(cudaMemcpyAsync(wl->d_rad_done, done, (size_t)wl->bins, cudaMemcpyHostToDevice, wl->b->stream));
  CUDA_TRY(stream_wait(wl->b->stream));
  if (all)  // rho_saved: the walkers stop sampling
    for (WlWalker& W : wl->w) W.radial_record = nullptr;
  return BRAWL_OK;
}

extern "C" int brawl_wl_radial_get(brawl_wl* wl, int c, int32_t* record, double* rho_of_E, int32_t* steps) {
  if (!wl || c < 0 || c >= (int)wl->w.size() || !record) return fail(BRAWL_EINVAL, "bad argument");
  if (!wl->d_rad) return fail(BRAWL_EINVAL, "radial samples not enabled");
  const size_t per = (size_t)wl->b->models[0].g.ns * wl->b->models[0].g.ns * wl->rad_wc;
  CUDA_TRY(cudaMemcpy(record, wl->d_rad_record + (size_t)c * wl->bins, (size_t)wl->bins * 4, cudaMemcpyDeviceToHost));
  if (rho_of_E)
    CUDA_TRY(cudaMemcpy(rho_of_E, wl->d_rad_rho + (size_t)c * wl->bins * per, (size_t)wl->bins * per * 8,
                        cudaMemcpyDeviceToHost));
  if (steps) CUDA_TRY(cudaMemcpy(steps, wl->d_rad_steps + c, 4, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

namespace {
bool same_lattice(const Geom& a, const Geom& b) {
  return a.lattice == b.lattice && a.n1 == b.n1 && a.n2 == b.n2 && a.n3 == b.n3;
}
}  // namespace

extern "C" int brawl_wl_store_enable(brawl_wl* wl) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  if (wl->d_store) return fail(BRAWL_EINVAL, "configuration store already enabled");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  std::vector<size_t> off(n);
  size_t total = 0;
  for (int c = 0; c < n; ++c) {
    off[c] = total;
    total += (size_t)wl->bins * (size_t)b->models[c].g.n_sites;
  }
  cudaStream_t s = b->stream;
  if (dalloc(&wl->d_store, total, s) != cudaSuccess ||
      dalloc(&wl->d_store_open, (size_t)n * wl->bins, s) != cudaSuccess ||
      dalloc(&wl->d_pick, (size_t)wl->bins * sizeof(int), s) != cudaSuccess) {
    for (const void* p : {(const void*)wl->d_store, (const void*)wl->d_store_open, (const void*)wl->d_pick})
      dfree(p, s);
    wl->d_store = nullptr;
    wl->d_store_open = nullptr;
    wl->d_pick = nullptr;
    return fail(BRAWL_ENOMEM, "configuration store (bins x sites per walker)");
  }
  CUDA_TRY(cudaMemsetAsync(wl->d_store, 0, total, s));             // config_per_bin = 0
  CUDA_TRY(cudaMemsetAsync(wl->d_store_open, 1, (size_t)n * wl->bins, s));  // config_store = .True.
  CUDA_TRY(stream_wait(s));
  for (int c = 0; c < n; ++c) {
    wl->w[c].store = wl->d_store + off[c];
    wl->w[c].store_open = wl->d_store_open + (size_t)c * wl->bins;
  }
  return BRAWL_OK;
}

extern "C" int brawl_wl_store_flags(brawl_wl* wl, uint8_t* open) {
  if (!wl || !open) return fail(BRAWL_EINVAL, "null argument");
  if (!wl->d_store) return fail(BRAWL_EINVAL, "configuration store not enabled");
  CUDA_TRY(cudaMemcpy(open, wl->d_store_open, wl->w.size() * (size_t)wl->bins, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

extern "C" int brawl_wl_store_merge(brawl_wl* wl, const int* pick) {
  if (!wl || !pick) return fail(BRAWL_EINVAL, "null argument");
  if (!wl->d_store) return fail(BRAWL_EINVAL, "configuration store not enabled");
  brawl_batch* b = wl->b;
  const int n = (int)wl->w.size();
  for (int c = 1; c < n; ++c)
    if (!same_lattice(b->models[c].g, b->models[0].g)) return fail(BRAWL_EINVAL, "walkers have different lattices");
  std::vector<uint8_t> open((size_t)n * wl->bins);
  CUDA_TRY(cudaMemcpy(open.data(), wl->d_store_open, open.size(), cudaMemcpyDeviceToHost));
  for (int k = 0; k < wl->bins; ++k) {
    if (pick[k] < -1 || pick[k] >= n) return fail(BRAWL_EINVAL, "pick outside -1 .. n_walkers-1");
    if (pick[k] >= 0 && open[(size_t)pick[k] * wl->bins + k])
      return fail(BRAWL_EINVAL, "bin " + std::to_string(k + 1) + ": the picked walker holds no configuration");
  }
  cudaStream_t s = b->stream;
  CUDA_TRY(cudaMemcpyAsync(wl->d_pick, pick, (size_t)wl->bins * sizeof(int), cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(wl->d_w, wl->w.data(), n * sizeof(WlWalker), cudaMemcpyHostToDevice, s));
  launch_wl_store_merge(wl->d_w, n, wl->bins, wl->d_pick, s);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(stream_wait(s));
  return BRAWL_OK;
}

namespace {
int store_slot(brawl_wl* wl, int c, int bin, const int8_t** slot) {
  if (!wl || c < 0 || c >= (int)wl->w.size() || bin < 1 || bin > wl->bins) return fail(BRAWL_EINVAL, "bad argument");
  if (!wl->d_store) return fail(BRAWL_EINVAL, "configuration store not enabled");
  uint8_t open = 1;
  CUDA_TRY(cudaMemcpy(&open, wl->w[c].store_open + (bin - 1), 1, cudaMemcpyDeviceToHost));
  if (open) return fail(BRAWL_ESTATE, "walker " + std::to_string(c) + ": bin " + std::to_string(bin) +
                                          " holds no stored configuration");
  *slot = wl->w[c].store + (size_t)(bin - 1) * (size_t)wl->b->models[c].g.n_sites;
  return BRAWL_OK;
}
}  // namespace

extern "C" int brawl_wl_store_load(brawl_wl* wl, int c, int bin) {
  const int8_t* slot = nullptr;
  TRY(store_slot(wl, c, bin, &slot));
  brawl_batch* b = wl->b;
  CUDA_TRY(cudaMemcpyAsync(b->jobs[c].lat, slot, (size_t)b->models[c].g.n_sites, cudaMemcpyDeviceToDevice,
                           b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_store_get(brawl_wl* wl, int c, int bin, int8_t* config) {
  if (!config) return fail(BRAWL_EINVAL, "null argument");
  const int8_t* slot = nullptr;
  TRY(store_slot(wl, c, bin, &slot));
  brawl_batch* b = wl->b;
  const Geom& g = b->models[c].g;
  const size_t grid = (size_t)8 * g.n1 * g.n2 * g.n3;
  TRY(ensure_grid(b, grid));
  launch_unpack(g, slot, b->d_grid, b->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(config, b->d_grid, grid, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_set_windows(brawl_wl* wl, const int* start_idx, const int* end_idx) {
  if (!wl || !start_idx || !end_idx) return fail(BRAWL_EINVAL, "null argument");
  const int nwin = (int)wl->groups.size();
  for (int k = 0; k < nwin; ++k)
    if (start_idx[k] < 1 || end_idx[k] > wl->bins || start_idx[k] > end_idx[k])
      return fail(BRAWL_EINVAL, "window " + std::to_string(k + 1) + " outside 1..bins");
  brawl_batch* b = wl->b;
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  const int rad_bins = wl->d_rad ? wl->bins : 0;
  // the layout of every walker first: nothing changes if one does not fit
  std::vector<int> cap(wl->w.size());
  uint32_t smem = 0;
  bool all_D = true;
  size_t hist_total = 0;
  for (int k = 0; k < nwin; ++k) {
    const WlGroup& G = wl->groups[k];
    const int nb = end_idx[k] - start_idx[k] + 1;
    for (int c = G.first; c < G.first + G.count; ++c) {
      const Geom& g = wl->w[c].job.g;
      const uint32_t base = wl_smem_bytes(g, nb, 0, rad_bins, wl->rad_n_off, wl->rad_n_class);
      cap[c] = lazy_cap_for(g, base, (uint32_t)max_optin);
      if (cap[c] == 0) return fail(BRAWL_EINVAL, "window " + std::to_string(k + 1) + " too large for shared memory");
      smem = std::max(smem, wl_smem_bytes(g, nb, cap[c], rad_bins, wl->rad_n_off, wl->rad_n_class));
      all_D = all_D && walker_layout(g, nb, cap[c]).use_D;
      hist_total += (size_t)nb;
    }
  }
  if (smem > (uint32_t)max_optin) return fail(BRAWL_EINVAL, "windows too large for shared memory");
  // mpi_arrays (src/wang-landau.F90:1351-1379): the histograms start from 0
  cudaStream_t s = b->stream;
  double* d_hist = nullptr;
  if (dalloc(&d_hist, hist_total * 8, s) != cudaSuccess) return fail(BRAWL_ENOMEM, "window histograms");
  CUDA_TRY(cudaMemsetAsync(d_hist, 0, hist_total * 8, s));
  dfree(wl->d_hist, s);
  wl->d_hist = d_hist;
  size_t hoff = 0;
  for (int k = 0; k < nwin; ++k) {
    const WlGroup& G = wl->groups[k];
    for (int c = G.first; c < G.first + G.count; ++c) {
      WlWalker& W = wl->w[c];
      W.start = start_idx[k];
      W.end = end_idx[k];
      W.hist = d_hist + hoff;
      W.lazy_cap = cap[c];
      hoff += (size_t)(W.end - W.start + 1);
    }
  }
  wl->smem = smem;
  wl->all_D = all_D;
  CUDA_TRY(stream_wait(s));
  return BRAWL_OK;
}

extern "C" int brawl_wl_get_lng(brawl_wl* wl, int c, double* lng) {
  if (!wl || !lng || c < 0 || c >= (int)wl->w.size()) return fail(BRAWL_EINVAL, "bad argument");
  CUDA_TRY(cudaMemcpy(lng, wl->w[c].lng, (size_t)wl->bins * 8, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

extern "C" int brawl_wl_set_lng(brawl_wl* wl, int c, const double* lng) {
  if (!wl || !lng || c < 0 || c >= (int)wl->w.size()) return fail(BRAWL_EINVAL, "bad argument");
  CUDA_TRY(cudaMemcpy(wl->w[c].lng, lng, (size_t)wl->bins * 8, cudaMemcpyHostToDevice));
  return BRAWL_OK;
}

extern "C" int brawl_wl_get_hist(brawl_wl* wl, int c, double* hist) {
  if (!wl || !hist || c < 0 || c >= (int)wl->w.size()) return fail(BRAWL_EINVAL, "bad argument");
  const WlWalker& W = wl->w[c];
  CUDA_TRY(cudaMemcpy(hist, W.hist, (size_t)(W.end - W.start + 1) * 8, cudaMemcpyDeviceToHost));
  return BRAWL_OK;
}

extern "C" int brawl_wl_set_hist(brawl_wl* wl, int c, const double* hist) {
  if (!wl || !hist || c < 0 || c >= (int)wl->w.size()) return fail(BRAWL_EINVAL, "bad argument");
  const WlWalker& W = wl->w[c];
  CUDA_TRY(cudaMemcpy(W.hist, hist, (size_t)(W.end - W.start + 1) * 8, cudaMemcpyHostToDevice));
  return BRAWL_OK;
}

extern "C" int brawl_wl_energies(brawl_wl* wl, double* energies) {
  if (!wl || !energies) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_total_energy(wl->b, energies);
}

extern "C" int brawl_wl_get_config(brawl_wl* wl, int c, int8_t* config) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_get_config(wl->b, c, config);
}

extern "C" int brawl_wl_set_config(brawl_wl* wl, int c, const int8_t* config) {
  if (!wl) return fail(BRAWL_EINVAL, "null argument");
  return brawl_batch_set_config(wl->b, c, config);
}

extern "C" int brawl_wl_swap_configs(brawl_wl* wl, int a, int c) {
  if (!wl || a < 0 || c < 0 || a >= (int)wl->w.size() || c >= (int)wl->w.size())
    return fail(BRAWL_EINVAL, "bad argument");
  if (a == c) return BRAWL_OK;
  brawl_batch* b = wl->b;
  const Geom& ga = b->models[a].g;
  const Geom& gc = b->models[c].g;
  if (ga.lattice != gc.lattice || ga.n1 != gc.n1 || ga.n2 != gc.n2 || ga.n3 != gc.n3)
    return fail(BRAWL_EINVAL, "walkers have different lattices");
  TRY(ensure_grid(b, (size_t)ga.n_sites));
  CUDA_TRY(cudaMemcpyAsync(b->d_grid, b->jobs[a].lat, ga.n_sites, cudaMemcpyDeviceToDevice, b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->jobs[a].lat, b->jobs[c].lat, ga.n_sites, cudaMemcpyDeviceToDevice, b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->jobs[c].lat, b->d_grid, ga.n_sites, cudaMemcpyDeviceToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

extern "C" int brawl_wl_genrand(brawl_wl* wl, int c, int64_t n, double* out) {
  if (!wl || c < 0 || c >= (int)wl->w.size() || n < 0 || (n > 0 && !out)) return fail(BRAWL_EINVAL, "bad argument");
  return batch_genrand(wl->b, c, n, out);
}

extern "C" int brawl_wl_counters(brawl_wl* wl, int c, int64_t* counters) {
  if (!wl || !counters || c < 0 || c >= (int)wl->w.size()) return fail(BRAWL_EINVAL, "bad argument");
  std::vector<int64_t> all(wl->w.size() * kNumCounters);
  TRY(brawl_batch_counters(wl->b, all.data()));
  std::copy(all.begin() + (size_t)c * kNumCounters, all.begin() + (size_t)(c + 1) * kNumCounters, counters);
  return BRAWL_OK;
}

// ---------------------------------------------------------------------------
// accessors for the serving loop (server.cu), which batches chains, walkers
// and runs of many objects into shared launches
// ---------------------------------------------------------------------------
namespace brawl {

int api_batch_chain(brawl_batch* b, int c, ChainSlot& out) {
  if (!b || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad chain");
  const Model& m = b->models[c];
  out.job = b->jobs[c];
  out.halo = b->halo[c];
  HaloGeom H;
  bool ok;
  make_halo(m.g, H, ok);
  out.halo_smem = out.halo ? halo_layout(m.g, H).total : 0;
  out.smem_lat_bytes = smem_layout(m.g, true).total;
  out.smem_glob_bytes = smem_layout(m.g, false).total;
  out.use_D = smem_layout(m.g, false).use_D;
  out.energy.g = m.g;
  out.energy.lat = b->jobs[c].lat;
  out.energy.V = b->jobs[c].V;
  out.energy.entries = b->jobs[c].entries;
  out.energy.shell_start = b->jobs[c].shell_start;
  out.energy.site_energy = nullptr;
  out.energy.out = nullptr;
  out.energy.site_offset = 0;
  return BRAWL_OK;
}

void api_batch_beta(brawl_batch* b, int c, ChainJob& j, double beta) { set_beta(j, b->models[c], beta); }

int api_batch_set_rng(brawl_batch* b, int c, const uint32_t state[625]) {
  if (!b || c < 0 || c >= (int)b->jobs.size()) return fail(BRAWL_EINVAL, "bad chain");
  CUDA_TRY(cudaMemcpyAsync(b->jobs[c].rng, state, (kMTN + 1) * 4, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(stream_wait(b->stream));
  return BRAWL_OK;
}

cudaStream_t api_batch_stream(brawl_batch* b) { return b->stream; }
brawl_batch* api_wl_batch(brawl_wl* wl) { return wl->b; }
std::vector<WlWalker>& api_wl_walkers(brawl_wl* wl) { return wl->w; }
uint32_t api_wl_smem(brawl_wl* wl) { return wl->smem; }
void api_wl_variant(brawl_wl* wl, int* max_z, bool* all_D) {
  *max_z = wl->max_z;
  *all_D = wl->all_D;
}

NsRun* api_ns_device_run(brawl_ns* ns, int r) { return ns->d_runs + r; }
uint32_t api_ns_smem(brawl_ns* ns) { return ns->smem; }
void api_ns_variant(brawl_ns* ns, int* max_z, bool* all_D) {
  *max_z = ns->max_z;
  *all_D = ns->all_D;
}
int api_last_error_set(int code, const std::string& msg) { return fail(code, msg); }
namespace {
struct WaitEvent {
  cudaEvent_t e = nullptr;
  ~WaitEvent() {
    if (e) cudaEventDestroy(e);
  }
};
thread_local bool tl_blocking = false;
thread_local WaitEvent tl_wait;
}  // namespace

void set_blocking_waits(bool on) { tl_blocking = on; }

cudaError_t stream_wait(cudaStream_t s) {
  if (!tl_blocking) return cudaStreamSynchronize(s);
  if (!tl_wait.e) {
    const cudaError_t e = cudaEventCreateWithFlags(&tl_wait.e, cudaEventBlockingSync | cudaEventDisableTiming);
    if (e != cudaSuccess) {
      tl_wait.e = nullptr;
      return cudaStreamSynchronize(s);
    }
  }
  const cudaError_t e = cudaEventRecord(tl_wait.e, s);
  if (e != cudaSuccess) return e;
  return cudaEventSynchronize(tl_wait.e);
}

std::string api_last_error() { return g_err; }

}  // namespace brawl
