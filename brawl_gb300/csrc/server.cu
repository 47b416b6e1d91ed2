// server.cu -- the serving loop: continuous batching of anneal, Wang-Landau
// and nested-sampling jobs over the device kernels.
//
// brawl_serve_submit queues a job.  Workers admit queued jobs in arrival
// order while the device-memory budget and the slot count allow and build
// their device objects (lattice, stream, tables, ln g, histograms, walkers),
// which stay on the device until the job ends.  Each job kind has a pipeline
// of its own (stream, pinned staging, event) driven by the scheduler thread:
// a round gives every resident job of that kind its next quantum of work --
// Metropolis trials up to the end of its temperature, Wang-Landau trials up
// to the end of its sweeps() call, nested-sampling iterations -- in one
// launch per kernel (the anneal chains in the halo and table Metropolis
// kernels, the walkers in the sweep kernel, the runs in the iterate kernel).
// The three pipelines overlap on the device; when a round completes it is
// settled and the next one launched at once with the jobs that became ready
// meanwhile.  Every chain's CTA records its device time, and a job's next
// quantum is sized so that its work takes about round_ms: jobs of very
// different cost then finish their quanta together and no round waits long
// for one slow job.  The scheduler thread never waits for the device; ended
// jobs are handed to the workers, which read their results back and free
// them.  A chain's trials continue its own stream and lattice, and a split
// sweeps() call carries its running energy and trial count, so splitting work
// into quanta and running it beside other jobs leaves every result unchanged.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "api_internal.h"

using namespace brawl;

namespace {

// k_b_in_Ry (src/constants.f90:41-46)
constexpr double kBoltzmannRy = 8.167333262e-5 / 13.605693122990;

#define SV_TRY(x)                  \
  do {                             \
    int r_ = (x);                  \
    if (r_ != BRAWL_OK) return r_; \
  } while (0)

#define SV_CUDA(x)                                                           \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess)                                                   \
      return api_fail(e_ == cudaErrorMemoryAllocation ? BRAWL_ENOMEM : BRAWL_ECUDA, \
                      std::string(#x) + ": " + cudaGetErrorString(e_));      \
  } while (0)

enum { kAnneal = 0, kWl = 1, kNs = 2, kKinds = 3 };
// threads building admitted jobs' device objects and reading back ended
// ones (a nested-sampling run's walker initialisation is one warp's
// sequential work, so several run at once)
constexpr int kWorkers = 8;
// initial capacity of the pinned buffers: growing one (a pinned allocation)
// waits for the whole device, so it should be rare
constexpr size_t kPinnedEntries = 4096;
constexpr size_t kPinnedStage = (size_t)8 << 20;
// first quanta, before a job's device time per unit of work is known
constexpr int64_t kFirstTrials = 4096;
constexpr int64_t kFirstWlTrials = 2048;

struct Job {
  uint64_t id = 0;
  brawl_job_desc d;
  std::vector<double> V, conc;
  std::vector<int64_t> numbers;
  bool has_numbers = false;
  brawl_job_result res;
  std::string err;
  std::vector<double> values;
  std::vector<int8_t> config;
  size_t footprint = 0;
  bool done = false;
  int n_sites = 0;
  // resident state
  brawl_batch* b = nullptr;
  brawl_wl* wl = nullptr;
  brawl_ns* ns = nullptr;
  int64_t quantum = 0;   // work given in the pipeline's current round
  double unit_ns = 0.0;  // device ns per unit of work (trial, NS iteration)
  // anneal
  ChainSlot slot;
  int stage = 0;
  int64_t stage_trials = 0, stage_left = 0;
  unsigned long long acc0 = 0;
  int e_idx = -1;        // this round's stage-end energy slot
  // Wang-Landau
  int calls = 0;
  int64_t call_pos = 0;  // trials of the current sweeps() call done
  double f = 0.0;
  int hist_period = 0;
  bool reset_hist = false;
  std::vector<double> bin_edges;
  double* d_estate = nullptr;  // running e_unswapped of each walker
  std::vector<EnergyJob> wl_energy;
  // nested sampling
  int iter_done = 0;
  NsRun* d_run = nullptr;
  const int32_t* ns_status = nullptr;
  const unsigned long long* ns_counters = nullptr;
};

using JobP = std::shared_ptr<Job>;

// grow-only device buffer, stream-ordered on the pipeline's stream
template <typename T>
int grow(T*& p, size_t& cap, size_t n, cudaStream_t s) {
  if (n <= cap) return BRAWL_OK;
  const size_t want = std::max(n, cap * 2);
  if (p) cudaFreeAsync(p, s);
  p = nullptr;
  cap = 0;
  SV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), want * sizeof(T), s));
  cap = want;
  return BRAWL_OK;
}

// grow-only pinned host buffer
template <typename T>
int grow_host(T*& p, size_t& cap, size_t n) {
  if (n <= cap) return BRAWL_OK;
  const size_t want = std::max(n, cap * 2);
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  SV_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), want * sizeof(T)));
  cap = want;
  return BRAWL_OK;
}

// status word and accepted counter of every chain / walker / run
__global__ void gather_kernel(const int32_t* const* __restrict__ st,
                              const unsigned long long* const* __restrict__ acc, int n,
                              int32_t* __restrict__ st_out, unsigned long long* __restrict__ acc_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  st_out[i] = *st[i];
  acc_out[i] = acc[i] ? *acc[i] : 0ull;
}

// nested-sampling runs into (and out of) the round's contiguous array
__global__ void ns_stage_kernel(NsRun* __restrict__ dst, NsRun* const* __restrict__ src, int n,
                                double* __restrict__ limits, const int* __restrict__ n_iter,
                                const int* __restrict__ lim_off, unsigned long long* __restrict__ t_ns) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  NsRun r = *src[i];
  r.limits = limits + lim_off[i];
  r.n_iter = n_iter[i];
  r.job.t_ns = t_ns + i;
  dst[i] = r;
}

__global__ void ns_unstage_kernel(const NsRun* __restrict__ from, NsRun* const* __restrict__ to, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  NsRun r = from[i];
  r.job.t_ns = nullptr;
  *to[i] = r;
}

// One job kind's pipeline.
// A round's chains, walkers or runs are launched in up to 1 + kSide groups
// of similar shared-memory size, the first on the pipeline's stream and the
// others on side streams forked from it and joined back: one launch sized
// for the largest lattice would give every small one the same shared
// memory and leave most of each SM's slots empty.
constexpr int kSide = 3;

struct Pipe {
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  cudaStream_t side[kSide] = {};
  cudaEvent_t ev_fork = nullptr, ev_side[kSide] = {};
  bool inflight = false;
  std::vector<JobP> jobs;      // resident
  std::vector<JobP> launched;  // in the in-flight round, in staged order
  // pinned staging of this round's host-to-device copies
  unsigned char* h_stage = nullptr;
  size_t h_stage_cap = 0, stage_used = 0;
  // energies
  EnergyJob* d_ej = nullptr;
  size_t ej_cap = 0;
  double* d_site = nullptr;
  size_t site_cap = 0;
  double* d_eout = nullptr;
  size_t eout_cap = 0;
  double* h_eout = nullptr;
  size_t h_eout_cap = 0;
  // status / accepted / device time per entry
  const void** d_ptrs = nullptr;
  size_t ptrs_cap = 0;
  int32_t* d_st = nullptr;
  size_t st_cap = 0;
  unsigned long long* d_acc = nullptr;
  size_t acc_cap = 0;
  unsigned long long* d_tns = nullptr;
  size_t tns_cap = 0;
  int32_t* h_st = nullptr;
  size_t h_st_cap = 0;
  unsigned long long* h_acc = nullptr;
  size_t h_acc_cap = 0;
  unsigned long long* h_tns = nullptr;
  size_t h_tns_cap = 0;
  // anneal
  ChainJob* d_chain = nullptr;
  size_t chain_cap = 0;
  // Wang-Landau
  WlWalker* d_wl = nullptr;
  size_t wl_cap = 0;
  WlGroup* d_groups = nullptr;
  size_t groups_cap = 0;
  double* d_flat = nullptr;
  size_t flat_cap = 0;
  WlWalker* h_wl = nullptr;
  size_t h_wl_cap = 0;
  double* h_flat = nullptr;
  size_t h_flat_cap = 0;
  std::vector<char> call_ends;  // per launched WL job: its sweeps() call completes this round
  // nested sampling
  NsRun* d_ns = nullptr;
  size_t ns_cap = 0;
  NsRun** d_ns_src = nullptr;
  size_t ns_src_cap = 0;
  int* d_ns_int = nullptr;
  size_t ns_int_cap = 0;
  double* d_limits = nullptr;
  size_t limits_cap = 0;
  double* h_limits = nullptr;
  size_t h_limits_cap = 0;
  std::vector<int> lim_off;
  // telemetry (seconds of host clock)
  double t_launched = 0.0;
  double busy_s = 0.0, launch_s = 0.0, settle_s = 0.0;
  int64_t n_rounds = 0, work = 0;

  void release() {
    for (const void* p : {(const void*)d_ej, (const void*)d_site, (const void*)d_eout, (const void*)d_ptrs,
                          (const void*)d_st, (const void*)d_acc, (const void*)d_tns, (const void*)d_chain,
                          (const void*)d_wl, (const void*)d_groups, (const void*)d_flat, (const void*)d_ns,
                          (const void*)d_ns_src, (const void*)d_ns_int, (const void*)d_limits})
      if (p && s) cudaFreeAsync(const_cast<void*>(p), s);
    if (s) cudaStreamSynchronize(s);
    for (void* p : {(void*)h_stage, (void*)h_eout, (void*)h_st, (void*)h_acc, (void*)h_tns, (void*)h_wl,
                    (void*)h_flat, (void*)h_limits})
      if (p) cudaFreeHost(p);
    for (int g = 0; g < kSide; ++g) {
      if (side[g]) cudaStreamSynchronize(side[g]);
      if (ev_side[g]) cudaEventDestroy(ev_side[g]);
      if (side[g]) cudaStreamDestroy(side[g]);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev) cudaEventDestroy(ev);
    if (s) cudaStreamDestroy(s);
  }
};

// Copies bytes into the round's pinned staging area (16-byte aligned) and
// queues the host-to-device copy from there.
int stage_copy(Pipe& P, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return BRAWL_OK;
  const size_t at = (P.stage_used + 15) & ~(size_t)15;
  if (at + bytes <= P.h_stage_cap) {
    std::memcpy(P.h_stage + at, src, bytes);
    P.stage_used = at + bytes;
    SV_CUDA(cudaMemcpyAsync(dst, P.h_stage + at, bytes, cudaMemcpyHostToDevice, P.s));
  } else {
    SV_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, P.s));
    SV_CUDA(cudaStreamSynchronize(P.s));  // pageable source: keep it alive until copied
  }
  return BRAWL_OK;
}

bool make_side_streams(Pipe& P, int prio) {
  for (int g = 0; g < kSide; ++g)
    if (cudaStreamCreateWithPriority(&P.side[g], cudaStreamNonBlocking, prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&P.ev_side[g], cudaEventDisableTiming) != cudaSuccess)
      return false;
  return true;
}

// Groups of a round's items in staged order, which is by decreasing shared
// memory: a new group starts where an item needs less than two thirds of
// its group's first (largest), so it would fit 1.5 times as many CTAs per
// SM; the last group takes the rest.
struct Group {
  int first, count;
};

std::vector<Group> smem_groups(const std::vector<uint32_t>& smem) {
  std::vector<Group> gs;
  for (int i = 0; i < (int)smem.size(); ++i) {
    if (gs.empty() || ((int)gs.size() <= kSide && 3ull * smem[i] < 2ull * smem[gs.back().first]))
      gs.push_back({i, 0});
    gs.back().count += 1;
  }
  return gs;
}

// Launches group g with launch(first, count, stream): group 0 on the
// pipeline's stream, the others on side streams that wait for the work
// queued so far and that the pipeline's stream waits for afterwards.
template <class F>
int launch_groups(Pipe& P, const std::vector<Group>& gs, F launch) {
  if (gs.empty()) return BRAWL_OK;
  if (gs.size() > 1) SV_CUDA(cudaEventRecord(P.ev_fork, P.s));
  for (size_t g = 0; g < gs.size(); ++g) {
    cudaStream_t st = g == 0 ? P.s : P.side[g - 1];
    if (g > 0) SV_CUDA(cudaStreamWaitEvent(st, P.ev_fork, 0));
    launch(gs[g].first, gs[g].count, st);
    SV_CUDA(cudaGetLastError());
    if (g > 0) SV_CUDA(cudaEventRecord(P.ev_side[g - 1], st));
  }
  for (size_t g = 1; g < gs.size(); ++g) SV_CUDA(cudaStreamWaitEvent(P.s, P.ev_side[g - 1], 0));
  return BRAWL_OK;
}

}  // namespace

struct brawl_server {
  brawl_server_opts o;
  int device = 0;
  int max_optin = 0;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  // cv_work: workers wait for admissible or ended jobs; cv_sched: the
  // scheduler waits for ready jobs; cv_done: callers wait for results
  std::condition_variable cv_work, cv_sched, cv_done;
  std::deque<JobP> queue;   // submitted, not admitted
  std::deque<JobP> ready;   // set up, not yet in a pipeline
  std::deque<std::pair<JobP, int>> ending;  // left their pipeline, results not read yet
  std::map<uint64_t, JobP> jobs;
  uint64_t next_id = 1;
  bool stop = false;
  size_t used = 0;
  int admitted = 0;         // jobs in set-up, ready, resident or ending
  int admitted_kind[4] = {0, 0, 0, 0};  // the same by job kind (BRAWL_JOB_*)
  int64_t rounds = 0, ended = 0;
  std::thread th;
  std::vector<std::thread> workers;
  Pipe pipe[kKinds];  // scheduler thread only

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

double beta_of(double T) { return 1.0 / (T * kBoltzmannRy); }

int kind_index(int kind) { return kind == BRAWL_JOB_ANNEAL ? kAnneal : (kind == BRAWL_JOB_WL ? kWl : kNs); }

size_t footprint_of(const brawl_job_desc& d, int n_sites) {
  const size_t chain = (size_t)n_sites * 9 + 16384;
  switch (d.kind) {
    case BRAWL_JOB_ANNEAL:
      return chain;
    case BRAWL_JOB_WL:
      return (size_t)d.wl_walkers * (chain + (size_t)d.wl_bins * 16 + 64);
    default:
      return (size_t)d.ns_walkers * ((size_t)n_sites * 9 + 16) + chain + (size_t)d.ns_iter * 8;
  }
}

// The round's length: round_ms, or longer when some job's smallest quantum
// (one unit) takes longer -- the others then fill the same time.
double round_ns(const brawl_server* S, const std::vector<JobP>& jobs) {
  double t = S->o.round_ms * 1.0e6;
  for (const auto& j : jobs) t = std::max(t, j->unit_ns);
  return t;
}

// The job's next quantum: t_round of device time at its measured cost per
// unit (first: first_q), at least one unit, within cap and what is left.
int64_t next_quantum(double t_round, const Job& j, int64_t left, int64_t first_q, int64_t cap) {
  int64_t q = first_q;
  if (j.unit_ns > 0.0) {
    const double t = t_round / j.unit_ns;
    q = t > 4.0e18 ? (int64_t)4e18 : (int64_t)t;
  }
  q = std::max<int64_t>(q, 1);
  q = std::min<int64_t>(q, (int64_t)1 << 30);  // a launch's per-chain tallies are 32-bit
  if (cap > 0) q = std::min(q, cap);
  return std::min(q, left);
}

void learn_cost(Job& j, unsigned long long t_ns) {
  if (j.quantum <= 0 || t_ns == 0) return;
  const double u = (double)t_ns / (double)j.quantum;
  j.unit_ns = j.unit_ns > 0.0 ? 0.5 * (j.unit_ns + u) : u;
}

void finish(brawl_server* S, const JobP& j, int status) {
  if (j->d_estate && j->wl) cudaFreeAsync(j->d_estate, api_batch_stream(api_wl_batch(j->wl)));
  j->d_estate = nullptr;
  if (j->b) brawl_batch_destroy(j->b);
  if (j->wl) brawl_wl_destroy(j->wl);
  if (j->ns) brawl_ns_destroy(j->ns);
  j->b = nullptr;
  j->wl = nullptr;
  j->ns = nullptr;
  std::lock_guard<std::mutex> lk(S->mu);
  S->used -= j->footprint;
  S->admitted -= 1;
  S->admitted_kind[kind_index(j->d.kind)] -= 1;
  j->res.status = status;
  j->res.t_finish = S->now();
  j->res.n_values = (int)j->values.size();
  j->done = true;
  S->ended += 1;
  S->cv_done.notify_all();
  S->cv_work.notify_all();
}

int grid_config(const Geom& g, std::vector<int8_t>& cfg) {
  cfg.assign((size_t)8 * g.n1 * g.n2 * g.n3, 0);
  return BRAWL_OK;
}

// A job that left its pipeline: its results read back (by a worker).
int collect(Job& j) {
  switch (j.d.kind) {
    case BRAWL_JOB_ANNEAL:
      grid_config(j.slot.job.g, j.config);
      return brawl_batch_get_config(j.b, 0, j.config.data());
    case BRAWL_JOB_WL: {
      SV_TRY(brawl_wl_get_lng(j.wl, 0, j.values.data()));
      std::copy(j.bin_edges.begin(), j.bin_edges.end(), j.values.begin() + j.d.wl_bins);
      grid_config(j.wl_energy[0].g, j.config);
      return brawl_wl_get_config(j.wl, 0, j.config.data());
    }
    default: {
      int64_t cnt[BRAWL_NUM_COUNTERS];
      SV_TRY(brawl_ns_counters(j.ns, 0, cnt));
      j.res.trials = cnt[0];
      Geom g;
      SV_TRY(api_make_geom(j.d.setup, g));
      grid_config(g, j.config);
      return brawl_ns_walker_config(j.ns, 0, 0, j.config.data());
    }
  }
}

// Queues the energies of a list of chains on the pipe's stream; out[k] ends
// up in P.d_eout[k].
int queue_energies(Pipe& P, std::vector<EnergyJob>& ej) {
  const int n = (int)ej.size();
  if (n == 0) return BRAWL_OK;
  int64_t total = 0;
  for (auto& e : ej) total += e.g.n_sites;
  SV_TRY(grow(P.d_site, P.site_cap, (size_t)total, P.s));
  SV_TRY(grow(P.d_eout, P.eout_cap, (size_t)n, P.s));
  SV_TRY(grow(P.d_ej, P.ej_cap, (size_t)n, P.s));
  SV_TRY(grow_host(P.h_eout, P.h_eout_cap, (size_t)n));
  int64_t off = 0;
  for (int k = 0; k < n; ++k) {
    ej[k].site_energy = P.d_site + off;
    ej[k].site_offset = off;
    ej[k].out = P.d_eout + k;
    off += ej[k].g.n_sites;
  }
  SV_TRY(stage_copy(P, P.d_ej, ej.data(), n * sizeof(EnergyJob)));
  launch_total_energy(P.d_ej, n, total, P.s);
  SV_CUDA(cudaGetLastError());
  return BRAWL_OK;
}

// Queues, after the round's kernels, the gather of status words (and
// accepted counters) and the copy of the device times into pinned buffers.
int queue_gather(Pipe& P, const std::vector<const int32_t*>& st, const std::vector<const unsigned long long*>& acc,
                 size_t n_tns) {
  const int n = (int)st.size();
  if (n == 0) return BRAWL_OK;
  SV_TRY(grow(P.d_ptrs, P.ptrs_cap, (size_t)2 * n, P.s));
  SV_TRY(grow(P.d_st, P.st_cap, (size_t)n, P.s));
  SV_TRY(grow(P.d_acc, P.acc_cap, (size_t)n, P.s));
  SV_TRY(grow_host(P.h_st, P.h_st_cap, (size_t)n));
  SV_TRY(grow_host(P.h_acc, P.h_acc_cap, (size_t)n));
  SV_TRY(grow_host(P.h_tns, P.h_tns_cap, n_tns));
  std::vector<const void*> ptrs(2 * n, nullptr);
  for (int i = 0; i < n; ++i) {
    ptrs[i] = st[i];
    ptrs[n + i] = acc.empty() ? nullptr : acc[i];
  }
  SV_TRY(stage_copy(P, P.d_ptrs, ptrs.data(), 2 * n * sizeof(void*)));
  BRAWL_CARVEOUT(gather_kernel);
  gather_kernel<<<(n + 127) / 128, 128, 0, P.s>>>(reinterpret_cast<const int32_t* const*>(P.d_ptrs),
                                                  reinterpret_cast<const unsigned long long* const*>(P.d_ptrs + n),
                                                  n, P.d_st, P.d_acc);
  SV_CUDA(cudaGetLastError());
  SV_CUDA(cudaMemcpyAsync(P.h_st, P.d_st, n * 4, cudaMemcpyDeviceToHost, P.s));
  SV_CUDA(cudaMemcpyAsync(P.h_acc, P.d_acc, n * 8, cudaMemcpyDeviceToHost, P.s));
  if (n_tns) SV_CUDA(cudaMemcpyAsync(P.h_tns, P.d_tns, n_tns * 8, cudaMemcpyDeviceToHost, P.s));
  return BRAWL_OK;
}

// ---------------------------------------------------------------------------
// admission: build the job's device objects
// ---------------------------------------------------------------------------
int setup_anneal(Job& j) {
  brawl_chain_desc cd;
  std::memset(&cd, 0, sizeof(cd));
  cd.setup = j.d.setup;
  cd.V_ex = j.V.data();
  cd.seed = j.d.seed;
  cd.beta = beta_of(j.d.T_start);
  cd.species_concentrations = j.conc.data();
  cd.species_numbers = j.has_numbers ? j.numbers.data() : nullptr;
  SV_TRY(brawl_batch_create(&cd, 1, &j.b));
  SV_TRY(api_batch_chain(j.b, 0, j.slot));
  j.n_sites = j.slot.job.g.n_sites;
  j.stage = 0;
  j.stage_trials = j.d.sweeps_per_T * (int64_t)j.n_sites;
  j.stage_left = j.stage_trials;
  int64_t cnt[BRAWL_NUM_COUNTERS];
  SV_TRY(brawl_batch_counters(j.b, cnt));
  j.acc0 = (unsigned long long)cnt[kCntAccepted];
  j.values.assign(2 * (size_t)j.d.T_steps, 0.0);
  return BRAWL_OK;
}

int setup_wl(Job& j) {
  const int nw = j.d.wl_walkers;
  std::vector<brawl_chain_desc> cd(nw);
  for (int k = 0; k < nw; ++k) {
    std::memset(&cd[k], 0, sizeof(cd[k]));
    cd[k].setup = j.d.setup;
    cd[k].V_ex = j.V.data();
    cd[k].seed = j.d.seed + 11u * (uint32_t)k;
    cd[k].beta = 0.0;
    cd[k].species_concentrations = j.conc.data();
    cd[k].species_numbers = j.has_numbers ? j.numbers.data() : nullptr;
  }
  // initial_setup of every walker, then the walkers take over the configs
  // and the streams where initial_setup left them
  brawl_batch* tmp = nullptr;
  SV_TRY(brawl_batch_create(cd.data(), nw, &tmp));
  std::vector<std::vector<int8_t>> cfg(nw);
  std::vector<std::vector<uint32_t>> rng(nw, std::vector<uint32_t>(kMTN + 1));
  std::vector<double> e(nw);
  int rc = brawl_batch_total_energy(tmp, e.data());
  ChainSlot s0;
  if (rc == BRAWL_OK) rc = api_batch_chain(tmp, 0, s0);
  for (int k = 0; k < nw && rc == BRAWL_OK; ++k) {
    grid_config(s0.job.g, cfg[k]);
    rc = brawl_batch_get_config(tmp, k, cfg[k].data());
    if (rc == BRAWL_OK) rc = brawl_batch_rng_get(tmp, k, rng[k].data());
  }
  brawl_batch_destroy(tmp);
  SV_TRY(rc);
  j.n_sites = s0.job.g.n_sites;
  const int bins = j.d.wl_bins;
  // the window: centred on the walkers' mean initial energy, wide enough
  // for every walker
  double c = 0.0;
  for (int k = 0; k < nw; ++k) c = c + e[k];
  c = c / (double)nw;
  double hw = j.d.wl_half_width;
  for (int k = 0; k < nw; ++k) hw = std::max(hw, 1.25 * std::fabs(e[k] - c));
  j.bin_edges.resize(bins + 1);
  for (int i = 0; i <= bins; ++i) j.bin_edges[i] = (c - hw) + (double)i * ((2.0 * hw) / (double)bins);
  std::vector<brawl_wl_desc> wd(nw);
  for (int k = 0; k < nw; ++k) {
    std::memset(&wd[k], 0, sizeof(wd[k]));
    wd[k].setup = j.d.setup;
    wd[k].V_ex = j.V.data();
    wd[k].seed = cd[k].seed;
    wd[k].config = cfg[k].data();
    wd[k].start_idx = 1;
    wd[k].end_idx = bins;
    wd[k].window = 0;
  }
  SV_TRY(brawl_wl_create(wd.data(), nw, bins, j.bin_edges.data(), &j.wl));
  brawl_batch* wb = api_wl_batch(j.wl);
  for (int k = 0; k < nw; ++k) SV_TRY(api_batch_set_rng(wb, k, rng[k].data()));
  SV_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&j.d_estate), nw * sizeof(double), api_batch_stream(wb)));
  SV_CUDA(stream_wait(api_batch_stream(wb)));
  j.wl_energy.resize(nw);
  for (int k = 0; k < nw; ++k) {
    ChainSlot cs;
    SV_TRY(api_batch_chain(wb, k, cs));
    j.wl_energy[k] = cs.energy;
  }
  j.f = j.d.wl_f;
  j.calls = 0;
  j.call_pos = 0;
  j.hist_period = (int)(0.02 * (double)(float)j.n_sites);
  j.values.assign((size_t)bins + bins + 1, 0.0);
  return BRAWL_OK;
}

int setup_ns(Job& j) {
  brawl_ns_desc nd;
  std::memset(&nd, 0, sizeof(nd));
  nd.setup = j.d.setup;
  nd.V_ex = j.V.data();
  nd.seed = j.d.seed;
  nd.n_walkers = j.d.ns_walkers;
  nd.n_steps = j.d.ns_steps;
  nd.species_concentrations = j.conc.data();
  nd.species_numbers = j.has_numbers ? j.numbers.data() : nullptr;
  SV_TRY(brawl_ns_create(&nd, 1, &j.ns));
  j.d_run = api_ns_device_run(j.ns, 0);
  NsRun h;
  SV_CUDA(cudaMemcpy(&h, j.d_run, sizeof(NsRun), cudaMemcpyDeviceToHost));
  j.ns_status = h.job.status;
  j.ns_counters = h.job.counters;
  j.iter_done = 0;
  j.values.assign((size_t)j.d.ns_iter, 0.0);
  Geom g;
  SV_TRY(api_make_geom(j.d.setup, g));
  j.n_sites = g.n_sites;
  return BRAWL_OK;
}

int setup_job(Job& j) {
  switch (j.d.kind) {
    case BRAWL_JOB_ANNEAL:
      return setup_anneal(j);
    case BRAWL_JOB_WL:
      return setup_wl(j);
    default:
      return setup_ns(j);
  }
}

// ---------------------------------------------------------------------------
// launches (one round of a pipeline, asynchronous) and settling
// ---------------------------------------------------------------------------
int launch_anneal(brawl_server* S, Pipe& P) {
  std::vector<ChainJob> staged;
  std::vector<EnergyJob> ej;
  P.launched.clear();
  uint32_t lat_smem = 0, glob_smem = 0;
  int table_z = 0;
  bool use_D = true;
  SV_TRY(grow(P.d_tns, P.tns_cap, std::max<size_t>(P.jobs.size(), 1), P.s));
  const double t_round = round_ns(S, P.jobs);
  std::stable_sort(P.jobs.begin(), P.jobs.end(), [](const JobP& a, const JobP& b) {
    return a->slot.halo_smem > b->slot.halo_smem;
  });
  for (int pass = 0; pass < 2; ++pass)
    for (auto& j : P.jobs) {
      if (j->slot.halo != (pass == 0 ? 1 : 0)) continue;
      j->quantum = next_quantum(t_round, *j, j->stage_left, kFirstTrials, S->o.max_trials);
      ChainJob c = j->slot.job;
      c.n_trials = j->quantum;
      c.t_ns = P.d_tns + staged.size();
      staged.push_back(c);
      P.launched.push_back(j);
      j->e_idx = -1;
      if (j->quantum == j->stage_left) {
        j->e_idx = (int)ej.size();
        ej.push_back(j->slot.energy);
      }
      if (pass == 1) {
        lat_smem = std::max(lat_smem, j->slot.smem_lat_bytes);
        glob_smem = std::max(glob_smem, j->slot.smem_glob_bytes);
        table_z = std::max(table_z, (int)c.g.z);
        use_D = use_D && j->slot.use_D;
      }
    }
  int nh = 0;
  for (auto& j : P.launched) nh += j->slot.halo;
  const int n = (int)staged.size();
  SV_TRY(grow(P.d_chain, P.chain_cap, (size_t)n, P.s));
  SV_TRY(stage_copy(P, P.d_chain, staged.data(), n * sizeof(ChainJob)));
  if (nh > 0) {
    std::vector<uint32_t> sm(nh);
    for (int k = 0; k < nh; ++k) sm[k] = P.launched[k]->slot.halo_smem;
    SV_TRY(launch_groups(P, smem_groups(sm), [&](int first, int count, cudaStream_t st) {
      int zmin = 0, zmax = 0;
      for (int k = first; k < first + count; ++k) {
        const int z = staged[k].g.z;
        zmin = zmax == 0 ? z : std::min(zmin, z);
        zmax = std::max(zmax, z);
      }
      launch_halo_chains(P.d_chain + first, count, sm[first], zmin, zmax, kDefaultSpeculation,
                         S->max_optin, st);
    }));
  }
  if (n - nh > 0) {
    const bool smem_lat = lat_smem <= (uint32_t)S->max_optin;
    launch_metropolis(P.d_chain + nh, n - nh, smem_lat, use_D, smem_lat ? lat_smem : glob_smem, table_z, P.s);
  }
  SV_CUDA(cudaGetLastError());
  // the energy at the end of every temperature that ends in this round
  SV_TRY(queue_energies(P, ej));
  if (!ej.empty()) SV_CUDA(cudaMemcpyAsync(P.h_eout, P.d_eout, ej.size() * 8, cudaMemcpyDeviceToHost, P.s));
  std::vector<const int32_t*> st;
  std::vector<const unsigned long long*> acc;
  for (auto& j : P.launched) {
    st.push_back(j->slot.job.status);
    acc.push_back(j->slot.job.counters + kCntAccepted);
  }
  return queue_gather(P, st, acc, (size_t)n);
}

int launch_wl(brawl_server* S, Pipe& P) {
  std::vector<WlWalker> staged;
  std::vector<WlGroup> groups;
  std::vector<EnergyJob> ej;
  std::vector<int> ej_walker;
  std::vector<uint32_t> w_smem;
  std::vector<int> w_z;
  std::vector<char> w_D;
  int max_bins = 0;
  std::stable_sort(P.jobs.begin(), P.jobs.end(),
                   [](const JobP& a, const JobP& b) { return api_wl_smem(a->wl) > api_wl_smem(b->wl); });
  P.launched = P.jobs;
  P.call_ends.assign(P.launched.size(), 0);
  size_t n_all = 0;
  for (auto& j : P.launched) n_all += j->d.wl_walkers;
  SV_TRY(grow(P.d_tns, P.tns_cap, std::max<size_t>(n_all, 1), P.s));
  const double t_round = round_ns(S, P.launched);
  for (size_t q = 0; q < P.launched.size(); ++q) {
    Job& j = *P.launched[q];
    std::vector<WlWalker>& w = api_wl_walkers(j.wl);
    if (j.reset_hist) {
      for (const WlWalker& W : w)
        SV_CUDA(cudaMemsetAsync(W.hist, 0, (size_t)(W.end - W.start + 1) * 8, P.s));
      j.reset_hist = false;
    }
    j.quantum = next_quantum(t_round, j, j.d.wl_trials - j.call_pos, kFirstWlTrials, S->o.max_trials);
    const bool starts = j.call_pos == 0;
    const bool ends = j.call_pos + j.quantum == j.d.wl_trials;
    P.call_ends[q] = ends;
    if (ends) groups.push_back({(int32_t)staged.size(), (int32_t)w.size()});
    for (size_t k = 0; k < w.size(); ++k) {
      WlWalker W = w[k];
      W.wl_f = j.f;
      W.n_trials = j.quantum;
      W.hist_period = j.hist_period;
      W.i0 = j.call_pos;
      W.e_state = j.d_estate + k;
      W.e0_src = nullptr;
      W.job.t_ns = P.d_tns + staged.size();
      if (starts) {
        ej.push_back(j.wl_energy[k]);
        ej_walker.push_back((int)staged.size());
      }
      staged.push_back(W);
    }
    int jz = 0;
    bool jd = true;
    api_wl_variant(j.wl, &jz, &jd);
    w_smem.insert(w_smem.end(), w.size(), api_wl_smem(j.wl));
    w_z.insert(w_z.end(), w.size(), jz);
    w_D.insert(w_D.end(), w.size(), jd ? 1 : 0);
    max_bins = std::max(max_bins, j.d.wl_bins);
  }
  const int n = (int)staged.size();
  // e_unswapped at the start of a call: full_energy of the walker
  SV_TRY(queue_energies(P, ej));
  for (size_t k = 0; k < ej_walker.size(); ++k) staged[ej_walker[k]].e0_src = P.d_eout + k;
  SV_TRY(grow(P.d_wl, P.wl_cap, (size_t)n, P.s));
  SV_TRY(grow(P.d_groups, P.groups_cap, std::max<size_t>(groups.size(), 1), P.s));
  SV_TRY(grow(P.d_flat, P.flat_cap, (size_t)n, P.s));
  SV_TRY(grow_host(P.h_wl, P.h_wl_cap, (size_t)n));
  SV_TRY(grow_host(P.h_flat, P.h_flat_cap, (size_t)n));
  SV_TRY(stage_copy(P, P.d_wl, staged.data(), n * sizeof(WlWalker)));
  if (!groups.empty()) SV_TRY(stage_copy(P, P.d_groups, groups.data(), groups.size() * sizeof(WlGroup)));
  SV_TRY(launch_groups(P, smem_groups(w_smem), [&](int first, int count, cudaStream_t st) {
    int max_z = 0;
    bool all_D = true;
    for (int k = first; k < first + count; ++k) {
      max_z = std::max(max_z, w_z[k]);
      all_D = all_D && w_D[k];
    }
    launch_wl_sweeps(P.d_wl + first, count, w_smem[first], max_z, all_D, st);
  }));
  if (!groups.empty()) launch_wl_average(P.d_groups, (int)groups.size(), P.d_wl, max_bins, 1, P.s);
  launch_wl_flatness(P.d_wl, n, P.d_flat, P.s);
  SV_CUDA(cudaGetLastError());
  SV_CUDA(cudaMemcpyAsync(P.h_wl, P.d_wl, n * sizeof(WlWalker), cudaMemcpyDeviceToHost, P.s));
  SV_CUDA(cudaMemcpyAsync(P.h_flat, P.d_flat, n * 8, cudaMemcpyDeviceToHost, P.s));
  std::vector<const int32_t*> st;
  for (const WlWalker& W : staged) st.push_back(W.job.status);
  return queue_gather(P, st, {}, (size_t)n);
}

int launch_ns(brawl_server* S, Pipe& P) {
  std::stable_sort(P.jobs.begin(), P.jobs.end(),
                   [](const JobP& a, const JobP& b) { return api_ns_smem(a->ns) > api_ns_smem(b->ns); });
  P.launched = P.jobs;
  const int n = (int)P.launched.size();
  std::vector<NsRun*> src(n);
  std::vector<int> ints(2 * n);
  std::vector<uint32_t> r_smem(n);
  std::vector<int> r_z(n);
  std::vector<char> r_D(n);
  int total = 0;
  const double t_round = round_ns(S, P.launched);
  for (int k = 0; k < n; ++k) {
    Job& j = *P.launched[k];
    j.quantum = next_quantum(t_round, j, j.d.ns_iter - j.iter_done, 1, S->o.max_iterations);
    src[k] = j.d_run;
    ints[k] = (int)j.quantum;
    ints[n + k] = total;
    total += (int)j.quantum;
    r_smem[k] = api_ns_smem(j.ns);
    int jz = 0;
    bool jd = true;
    api_ns_variant(j.ns, &jz, &jd);
    r_z[k] = jz;
    r_D[k] = jd ? 1 : 0;
  }
  P.lim_off.assign(ints.begin() + n, ints.end());
  SV_TRY(grow(P.d_ns, P.ns_cap, (size_t)n, P.s));
  SV_TRY(grow(P.d_ns_src, P.ns_src_cap, (size_t)n, P.s));
  SV_TRY(grow(P.d_ns_int, P.ns_int_cap, (size_t)2 * n, P.s));
  SV_TRY(grow(P.d_limits, P.limits_cap, (size_t)std::max(total, 1), P.s));
  SV_TRY(grow(P.d_tns, P.tns_cap, (size_t)n, P.s));
  SV_TRY(grow_host(P.h_limits, P.h_limits_cap, (size_t)std::max(total, 1)));
  SV_TRY(stage_copy(P, P.d_ns_src, src.data(), n * sizeof(NsRun*)));
  SV_TRY(stage_copy(P, P.d_ns_int, ints.data(), 2 * n * sizeof(int)));
  BRAWL_CARVEOUT(ns_stage_kernel);
  ns_stage_kernel<<<(n + 63) / 64, 64, 0, P.s>>>(P.d_ns, P.d_ns_src, n, P.d_limits, P.d_ns_int, P.d_ns_int + n,
                                                  P.d_tns);
  SV_TRY(launch_groups(P, smem_groups(r_smem), [&](int first, int count, cudaStream_t st) {
    int max_z = 0;
    bool all_D = true;
    for (int k = first; k < first + count; ++k) {
      max_z = std::max(max_z, r_z[k]);
      all_D = all_D && r_D[k];
    }
    launch_ns_iterate(P.d_ns + first, count, r_smem[first], max_z, all_D, st);
  }));
  BRAWL_CARVEOUT(ns_unstage_kernel);
  ns_unstage_kernel<<<(n + 63) / 64, 64, 0, P.s>>>(P.d_ns, P.d_ns_src, n);
  SV_CUDA(cudaGetLastError());
  if (total > 0) SV_CUDA(cudaMemcpyAsync(P.h_limits, P.d_limits, total * 8, cudaMemcpyDeviceToHost, P.s));
  std::vector<const int32_t*> st;
  std::vector<const unsigned long long*> acc;
  for (auto& j : P.launched) {
    st.push_back(j->ns_status);
    acc.push_back(j->ns_counters + kCntAccepted);
  }
  return queue_gather(P, st, acc, (size_t)n);
}

int launch_round(brawl_server* S, int kind) {
  Pipe& P = S->pipe[kind];
  const double t0 = S->now();
  P.stage_used = 0;
  int rc = kind == kAnneal ? launch_anneal(S, P) : (kind == kWl ? launch_wl(S, P) : launch_ns(S, P));
  SV_TRY(rc);
  SV_CUDA(cudaEventRecord(P.ev, P.s));
  P.inflight = true;
  P.t_launched = S->now();
  int64_t work = 0;
  // trials; Wang-Landau: of every walker; nested sampling: walk steps at
  // n_steps per iteration (adaptive extra steps not counted)
  for (auto& j : P.launched)
    work += j->quantum * (kind == kWl ? j->d.wl_walkers : (kind == kNs ? j->d.ns_steps : 1));
  std::lock_guard<std::mutex> lk(S->mu);  // telemetry is read by brawl_serve_profile
  P.launch_s += P.t_launched - t0;
  P.work += work;
  return BRAWL_OK;
}

using Ended = std::vector<std::pair<JobP, int>>;

int settle_anneal(Pipe& P, Ended& ended) {
  for (size_t k = 0; k < P.launched.size(); ++k) {
    const JobP& jp = P.launched[k];
    Job& j = *jp;
    if (P.h_st[k] != 0) {
      j.err = "device check failed (code " + std::to_string(P.h_st[k]) + ")";
      ended.push_back({jp, BRAWL_ESTATE});
      continue;
    }
    learn_cost(j, P.h_tns[k]);
    j.stage_left -= j.quantum;
    j.res.trials += j.quantum;
    if (j.e_idx < 0) continue;
    const unsigned long long a = P.h_acc[k] - j.acc0;
    const double E = P.h_eout[j.e_idx];
    j.values[j.stage] = E;
    j.values[j.d.T_steps + j.stage] = j.stage_trials > 0 ? (double)a / (double)j.stage_trials : 0.0;
    j.res.accepted += (int64_t)a;
    j.res.energy = E;
    j.acc0 = P.h_acc[k];
    j.stage += 1;
    if (j.stage == j.d.T_steps) {
      ended.push_back({jp, BRAWL_OK});
      continue;
    }
    api_batch_beta(j.b, 0, j.slot.job, beta_of(j.d.T_start + (double)j.stage * j.d.delta_T));
    j.stage_left = j.stage_trials;
  }
  return BRAWL_OK;
}

int settle_wl(Pipe& P, Ended& ended) {
  int k0 = 0;
  for (size_t q = 0; q < P.launched.size(); ++q) {
    const JobP& jp = P.launched[q];
    Job& j = *jp;
    const int nw = j.d.wl_walkers;
    bool bad = false, all_flat = true;
    unsigned long long t = 0;
    for (int k = k0; k < k0 + nw; ++k) {
      bad = bad || P.h_st[k] != 0;
      all_flat = all_flat && P.h_flat[k] > j.d.wl_flatness;
      j.res.accepted += P.h_wl[k].accepted;
      t = std::max(t, P.h_tns[k]);
    }
    j.res.trials += (int64_t)nw * j.quantum;
    j.res.energy = P.h_wl[k0].e_out;
    k0 += nw;
    if (bad) {
      j.err = "a walker's energy is outside its window";
      ended.push_back({jp, BRAWL_ESTATE});
      continue;
    }
    learn_cost(j, t);
    j.call_pos += j.quantum;
    if (!P.call_ends[q]) continue;
    j.call_pos = 0;
    j.calls += 1;
    if (all_flat) {
      j.f *= 0.5;
      j.res.wl_halvings += 1;
      j.reset_hist = true;
    }
    j.res.wl_f = j.f;
    if (j.calls >= j.d.wl_calls || j.f < j.d.wl_tolerance) ended.push_back({jp, BRAWL_OK});
  }
  return BRAWL_OK;
}

int settle_ns(Pipe& P, Ended& ended) {
  for (size_t k = 0; k < P.launched.size(); ++k) {
    const JobP& jp = P.launched[k];
    Job& j = *jp;
    std::copy(P.h_limits + P.lim_off[k], P.h_limits + P.lim_off[k] + j.quantum, j.values.begin() + j.iter_done);
    j.iter_done += (int)j.quantum;
    j.res.accepted = (int64_t)P.h_acc[k];
    if (j.iter_done > 0) j.res.energy = j.values[j.iter_done - 1];
    if (P.h_st[k] != 0) {
      j.err = "nested sampling check failed";
      ended.push_back({jp, BRAWL_ESTATE});
      continue;
    }
    learn_cost(j, P.h_tns[k]);
    if (j.iter_done >= j.d.ns_iter) ended.push_back({jp, BRAWL_OK});
  }
  return BRAWL_OK;
}

// Ended jobs leave their pipeline; a worker reads their results and frees them.
void end_jobs(brawl_server* S, Pipe& P, Ended& ended) {
  if (ended.empty()) return;
  for (auto& e : ended) P.jobs.erase(std::remove(P.jobs.begin(), P.jobs.end(), e.first), P.jobs.end());
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& e : ended) S->ending.push_back(e);
  }
  S->cv_work.notify_all();
}

// A pipeline failed as a whole (a launch or a copy): its jobs end with the error.
void fail_pipe(brawl_server* S, Pipe& P, int rc) {
  const std::string msg = api_last_error();
  cudaStreamSynchronize(P.s);
  Ended ended;
  for (auto& j : P.jobs) {
    j->err = msg;
    ended.push_back({j, rc});
  }
  P.launched.clear();
  P.inflight = false;
  end_jobs(S, P, ended);
}

// Workers: read back and free ended jobs first, then admit queued jobs in
// arrival order while the slot count and the device-memory budget allow (a
// job larger than the budget is admitted alone) and build their device
// objects on the objects' own streams, so the pipelines keep running.
// Wang-Landau and nested-sampling jobs have their own resident caps: a
// walker or run on a large lattice holds a whole SM (its shared memory) for
// a long round, and past a few dozen of them the anneal chains lose more
// SMs than the walks add work (on a mixed stream at 250 jobs/s, 45 s:
// 7.3e8 trials/s with 32 of each kind resident, 6.8e8 with 64, 2.5e8 with
// 128), while anneal chains keep gaining up to thousands.  A queued job of
// a kind at its cap waits; the first later job of another kind is admitted
// instead.
int kind_cap(const brawl_server* S, int kind) {
  if (kind == BRAWL_JOB_WL) return S->o.max_active_wl;
  if (kind == BRAWL_JOB_NS) return S->o.max_active_ns;
  return S->o.max_active;
}

// The queue index of the next job to admit, or -1.
long admissible_index(brawl_server* S) {
  if (S->queue.empty() || S->admitted >= S->o.max_active) return -1;
  for (size_t q = 0; q < S->queue.size(); ++q) {
    const JobP& j = S->queue[q];
    const int k = j->d.kind;
    if (S->admitted_kind[kind_index(k)] >= kind_cap(S, k)) continue;
    if (S->admitted == 0 || S->used + j->footprint <= S->o.hbm_budget) return (long)q;
    return -1;  // the budget: wait for memory, in arrival order
  }
  return -1;
}

bool admissible(brawl_server* S) { return admissible_index(S) >= 0; }

void end_one(brawl_server* S, const JobP& j, int status) {
  if (status == BRAWL_OK) {
    status = collect(*j);
    if (status != BRAWL_OK) j->err = api_last_error();
  }
  finish(S, j, status);
}

void worker(brawl_server* S) {
  cudaSetDevice(S->device);
  set_blocking_waits(true);
  for (;;) {
    JobP j;
    int end_status = 0;
    bool ending = false;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || !S->ending.empty() || admissible(S); });
      if (!S->ending.empty()) {
        j = S->ending.front().first;
        end_status = S->ending.front().second;
        S->ending.pop_front();
        ending = true;
      } else if (S->stop) {
        return;
      } else {
        const long q = admissible_index(S);
        j = S->queue[(size_t)q];
        S->queue.erase(S->queue.begin() + q);
        S->used += j->footprint;
        S->admitted += 1;
        S->admitted_kind[kind_index(j->d.kind)] += 1;
        j->res.t_admit = S->now();
      }
    }
    if (ending) {
      end_one(S, j, end_status);
      continue;
    }
    const int rc = setup_job(*j);
    if (rc != BRAWL_OK) {
      j->err = api_last_error();
      finish(S, j, rc);
      continue;
    }
    bool cancel = false;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      j->res.t_ready = S->now();
      cancel = S->stop;
      if (!cancel) S->ready.push_back(j);
    }
    if (cancel) {
      finish(S, j, BRAWL_ECANCELLED);
      continue;
    }
    S->cv_sched.notify_one();
  }
}

void scheduler(brawl_server* S) {
  cudaSetDevice(S->device);
  for (;;) {
    bool progressed = false;
    std::vector<JobP> joined;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      bool idle = true;
      for (int k = 0; k < kKinds; ++k) idle = idle && !S->pipe[k].inflight && S->pipe[k].jobs.empty();
      if (idle) S->cv_sched.wait(lk, [&] { return S->stop || !S->ready.empty(); });
      if (S->stop) break;
      joined.assign(S->ready.begin(), S->ready.end());
      S->ready.clear();
    }
    for (auto& j : joined) {
      S->pipe[kind_index(j->d.kind)].jobs.push_back(j);
      progressed = true;
    }
    for (int k = 0; k < kKinds; ++k) {
      Pipe& P = S->pipe[k];
      if (P.inflight) {
        const cudaError_t q = cudaEventQuery(P.ev);
        if (q == cudaErrorNotReady) continue;
        P.inflight = false;
        progressed = true;
        const double t_done = S->now();
        Ended ended;
        int rc = q == cudaSuccess ? BRAWL_OK : api_fail(BRAWL_ECUDA, cudaGetErrorString(q));
        if (rc == BRAWL_OK)
          rc = k == kAnneal ? settle_anneal(P, ended) : (k == kWl ? settle_wl(P, ended) : settle_ns(P, ended));
        if (rc != BRAWL_OK) {
          fail_pipe(S, P, rc);
          continue;
        }
        end_jobs(S, P, ended);
        std::lock_guard<std::mutex> lk(S->mu);
        P.busy_s += t_done - P.t_launched;
        P.n_rounds += 1;
        P.settle_s += S->now() - t_done;
        S->rounds += 1;
      }
      if (!P.inflight && !P.jobs.empty()) {
        int rc = launch_round(S, k);
        if (rc != BRAWL_OK) fail_pipe(S, P, rc);
        progressed = true;
      }
    }
    if (!progressed) {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_sched.wait_for(lk, std::chrono::microseconds(50), [&] { return S->stop || !S->ready.empty(); });
    }
  }
  // stopping: resident jobs end cancelled (read back and freed by the caller)
  for (int k = 0; k < kKinds; ++k) {
    Pipe& P = S->pipe[k];
    if (P.s) cudaStreamSynchronize(P.s);
    P.inflight = false;
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& j : P.jobs) S->ending.push_back({j, BRAWL_ECANCELLED});
    P.jobs.clear();
  }
}

int validate(const brawl_job_desc& d, Geom& g) {
  SV_TRY(api_make_geom(d.setup, g));
  if (!d.V_ex || !d.species_concentrations) return api_fail(BRAWL_EINVAL, "job needs V_ex and concentrations");
  switch (d.kind) {
    case BRAWL_JOB_ANNEAL:
      if (d.T_steps < 1 || d.sweeps_per_T < 0) return api_fail(BRAWL_EINVAL, "anneal needs T_steps >= 1, sweeps >= 0");
      for (int k = 0; k < d.T_steps; ++k)
        if (!(d.T_start + k * d.delta_T > 0.0)) return api_fail(BRAWL_EINVAL, "temperatures must be positive");
      return BRAWL_OK;
    case BRAWL_JOB_WL:
      if (d.wl_walkers < 1 || d.wl_bins < 1 || d.wl_calls < 1 || d.wl_trials < 0 || !(d.wl_half_width > 0.0))
        return api_fail(BRAWL_EINVAL, "bad Wang-Landau job");
      return BRAWL_OK;
    case BRAWL_JOB_NS:
      if (d.ns_walkers < 1 || d.ns_steps < 0 || d.ns_iter < 0) return api_fail(BRAWL_EINVAL, "bad nested-sampling job");
      return BRAWL_OK;
    default:
      return api_fail(BRAWL_EINVAL, "unknown job kind");
  }
}

}  // namespace

extern "C" {

int brawl_serve_create(const brawl_server_opts* opts, brawl_server** out) {
  if (!out) return api_fail(BRAWL_EINVAL, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return api_fail(BRAWL_ECUDA, "no CUDA device");
  brawl_server* S = new brawl_server();
  std::memset(&S->o, 0, sizeof(S->o));
  if (opts) S->o = *opts;
  cudaGetDevice(&S->device);
  // The worker threads wait on their objects' streams; spinning waits (the
  // runtime's default with few threads) would take the cores the scheduler
  // thread needs, so host waits in this process block instead.
  cudaSetDeviceFlags(cudaDeviceScheduleBlockingSync);
  cudaGetLastError();
  if (S->o.hbm_budget == 0) {
    // 60% of the device memory free now
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    S->o.hbm_budget = free_b / 10 * 6;
  }
  if (S->o.max_active <= 0) S->o.max_active = 4096;
  if (S->o.max_active_wl <= 0) S->o.max_active_wl = 64;
  if (S->o.max_active_ns <= 0) S->o.max_active_ns = 64;
  if (!(S->o.round_ms > 0.0)) S->o.round_ms = 20.0;
  if (S->o.max_trials < 0) S->o.max_trials = 0;
  if (S->o.max_iterations < 0) S->o.max_iterations = 0;
  cudaDeviceGetAttribute(&S->max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, S->device);
  // every kernel a round may launch is loaded now: a round that first used
  // a variant would otherwise wait for every round in flight
  preload_metropolis_kernels();
  preload_halo_kernels();
  preload_ns_kernels();
  preload_wl_kernels();
  preload_lattice_kernels();
  {
    cudaFuncAttributes a;
    cudaFuncGetAttributes(&a, gather_kernel);
    cudaFuncGetAttributes(&a, ns_stage_kernel);
    cudaFuncGetAttributes(&a, ns_unstage_kernel);
  }
  cudaGetLastError();
  {
    // keep freed stream-ordered memory in this process's pool for reuse
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
      uint64_t keep = S->o.hbm_budget;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      // no reuse that makes one stream wait for another: a job's set-up
      // would otherwise wait for a whole round of another pipeline
      int no = 0;
      cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
  }
  for (int k = 0; k < kKinds; ++k) {
    Pipe& P = S->pipe[k];
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    // rounds run at the lowest priority: set-up and read-back of jobs go first
    if (cudaStreamCreateWithPriority(&P.s, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&P.ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&P.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        !make_side_streams(P, prio_lo) ||
        grow_host(P.h_stage, P.h_stage_cap, kPinnedStage) != BRAWL_OK ||
        grow_host(P.h_eout, P.h_eout_cap, kPinnedEntries) != BRAWL_OK ||
        grow_host(P.h_st, P.h_st_cap, kPinnedEntries) != BRAWL_OK ||
        grow_host(P.h_acc, P.h_acc_cap, kPinnedEntries) != BRAWL_OK ||
        grow_host(P.h_tns, P.h_tns_cap, kPinnedEntries) != BRAWL_OK ||
        (k == kWl && (grow_host(P.h_wl, P.h_wl_cap, kPinnedEntries) != BRAWL_OK ||
                      grow_host(P.h_flat, P.h_flat_cap, kPinnedEntries) != BRAWL_OK)) ||
        (k == kNs && grow_host(P.h_limits, P.h_limits_cap, 16 * kPinnedEntries) != BRAWL_OK)) {
      for (int q = 0; q <= k; ++q) S->pipe[q].release();
      delete S;
      return api_fail(BRAWL_ECUDA, "server streams / pinned buffers");
    }
  }
  S->t0 = std::chrono::steady_clock::now();
  S->th = std::thread(scheduler, S);
  for (int k = 0; k < kWorkers; ++k) S->workers.emplace_back(worker, S);
  *out = S;
  return BRAWL_OK;
}

int brawl_serve_destroy(brawl_server* S) {
  if (!S) return BRAWL_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    for (auto& j : S->queue) {
      j->res.status = BRAWL_ECANCELLED;
      j->res.t_finish = S->now();
      j->done = true;
    }
    S->queue.clear();
  }
  S->cv_sched.notify_all();
  if (S->th.joinable()) S->th.join();
  S->cv_work.notify_all();
  for (auto& t : S->workers)
    if (t.joinable()) t.join();
  // what the workers left: ended jobs to read back, set-up jobs never run
  std::deque<std::pair<JobP, int>> ending;
  std::deque<JobP> ready;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    ending.swap(S->ending);
    ready.swap(S->ready);
  }
  for (auto& e : ending) end_one(S, e.first, e.second);
  for (auto& j : ready) finish(S, j, BRAWL_ECANCELLED);
  S->cv_done.notify_all();
  for (int k = 0; k < kKinds; ++k) S->pipe[k].release();
  delete S;
  return BRAWL_OK;
}

int brawl_serve_submit(brawl_server* S, const brawl_job_desc* d, uint64_t* id) {
  if (!S || !d || !id) return api_fail(BRAWL_EINVAL, "null argument");
  Geom g;
  SV_TRY(validate(*d, g));
  JobP j = std::make_shared<Job>();
  j->d = *d;
  j->V.assign(d->V_ex, d->V_ex + (size_t)g.ns * g.ns * g.nsh);
  j->conc.assign(d->species_concentrations, d->species_concentrations + g.ns + 1);
  if (d->species_numbers) {
    j->numbers.assign(d->species_numbers, d->species_numbers + g.ns);
    j->has_numbers = true;
  }
  j->d.V_ex = nullptr;
  j->d.species_concentrations = nullptr;
  j->d.species_numbers = nullptr;
  std::memset(&j->res, 0, sizeof(j->res));
  j->res.kind = d->kind;
  j->footprint = footprint_of(*d, g.n_sites);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return api_fail(BRAWL_ECANCELLED, "server is stopping");
    j->id = S->next_id++;
    j->res.t_submit = S->now();
    S->jobs[j->id] = j;
    S->queue.push_back(j);
    *id = j->id;
  }
  S->cv_work.notify_one();
  return BRAWL_OK;
}

int brawl_serve_poll(brawl_server* S, uint64_t id, brawl_job_result* res) {
  return brawl_serve_wait(S, id, 0.0, res);
}

int brawl_serve_wait(brawl_server* S, uint64_t id, double timeout_s, brawl_job_result* res) {
  if (!S) return api_fail(BRAWL_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return api_fail(BRAWL_EINVAL, "unknown job");
  JobP j = it->second;
  if (!j->done) {
    if (timeout_s == 0.0) return api_fail(BRAWL_EAGAIN, "job has not finished");
    auto pred = [&] { return j->done; };
    if (timeout_s < 0.0) {
      S->cv_done.wait(lk, pred);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
      return api_fail(BRAWL_ETIMEDOUT, "job has not finished in time");
    }
  }
  if (res) *res = j->res;
  if (j->res.status != BRAWL_OK && !j->err.empty()) api_fail(j->res.status, j->err);
  return BRAWL_OK;
}

int brawl_serve_values(brawl_server* S, uint64_t id, double* values) {
  if (!S || !values) return api_fail(BRAWL_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return api_fail(BRAWL_EINVAL, "unknown job");
  if (!it->second->done) return api_fail(BRAWL_EAGAIN, "job has not finished");
  std::copy(it->second->values.begin(), it->second->values.end(), values);
  return BRAWL_OK;
}

int brawl_serve_config(brawl_server* S, uint64_t id, int8_t* config) {
  if (!S || !config) return api_fail(BRAWL_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return api_fail(BRAWL_EINVAL, "unknown job");
  if (!it->second->done) return api_fail(BRAWL_EAGAIN, "job has not finished");
  if (it->second->config.empty()) return api_fail(BRAWL_ESTATE, "job ended without a configuration");
  std::copy(it->second->config.begin(), it->second->config.end(), config);
  return BRAWL_OK;
}

int brawl_serve_release(brawl_server* S, uint64_t id) {
  if (!S) return api_fail(BRAWL_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return api_fail(BRAWL_EINVAL, "unknown job");
  if (!it->second->done) return api_fail(BRAWL_EAGAIN, "job has not finished");
  S->jobs.erase(it);
  return BRAWL_OK;
}

int brawl_serve_profile(brawl_server* S, double out[15]) {
  if (!S || !out) return api_fail(BRAWL_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  for (int k = 0; k < kKinds; ++k) {
    const Pipe& P = S->pipe[k];
    out[5 * k + 0] = (double)P.n_rounds;
    out[5 * k + 1] = P.busy_s;
    out[5 * k + 2] = P.launch_s;
    out[5 * k + 3] = P.settle_s;
    out[5 * k + 4] = (double)P.work;
  }
  return BRAWL_OK;
}

int brawl_serve_stats(brawl_server* S, int64_t stats[4]) {
  if (!S || !stats) return api_fail(BRAWL_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  int64_t resident = 0;
  for (auto& kv : S->jobs)
    if (!kv.second->done) ++resident;
  stats[0] = S->rounds;
  stats[1] = resident - (int64_t)S->queue.size();
  stats[2] = (int64_t)S->queue.size();
  stats[3] = S->ended;
  return BRAWL_OK;
}

}  // extern "C"
