// wang_landau.cu -- Wang-Landau walker updates on the device
// (src/wang-landau.F90:515-632): sweeps() for every walker of a batch, then
// the in-window average of ln g and of the histogram that the reference
// does with MPI_Allreduce over the walkers of a window followed by a
// division by their number.
//
// One warp per walker.  Each trial's bins depend on the walker's running
// FP64 energy, so a trial whose two species differ takes the reference-order
// FP64 pair energies (e_swapped = e_unswapped - pair_unswapped +
// pair_swapped); the acceptance test log(genrand()) < lng(i) - lng(j) is
// decided in FP32 first (exact_fp.cuh).  The window's ln g and histogram
// slices are staged in shared memory.
#include "halo_engine.cuh"
#include "kernels.cuh"
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

__global__ void __launch_bounds__(32) wl_sweep_kernel(WlWalker* __restrict__ walkers) {
  extern __shared__ __align__(16) unsigned char smem[];
  WlWalker& W = walkers[blockIdx.x];
  const ChainJob& J = W.job;
  const Geom g = J.g;
  const int lane = threadIdx.x;
  const int nV = g.ns * g.ns * g.nsh;
  const int nb = W.end - W.start + 1;
  // layout: mt | tbuf | V | lng slice | hist slice | ents | sstart | lattice
  uint32_t* mt = reinterpret_cast<uint32_t*>(smem);
  uint32_t* tbuf = mt + kMTN;
  double* V = reinterpret_cast<double*>(smem + align_up((kMTN + kTbufWords) * 4, 16));
  double* lng = V + nV;
  double* hist = lng + nb;
  uint32_t* ents = reinterpret_cast<uint32_t*>(hist + nb);
  int16_t* sstart = reinterpret_cast<int16_t*>(ents + g.z);
  int8_t* lat = reinterpret_cast<int8_t*>(
      smem + align_up((uint32_t)((reinterpret_cast<unsigned char*>(sstart + g.nsh + 1)) - smem), 16));
  for (int i = lane; i < kMTN; i += 32) mt[i] = J.rng[i];
  for (int i = lane; i < nV; i += 32) V[i] = J.V[i];
  for (int i = lane; i < nb; i += 32) {
    lng[i] = W.lng[W.start - 1 + i];
    hist[i] = W.hist[i];
  }
  for (int i = lane; i < g.z; i += 32) ents[i] = J.entries[i];
  for (int i = lane; i <= g.nsh; i += 32) sstart[i] = J.shell_start[i];
  for (int i = lane; i < g.n_sites; i += 32) lat[i] = J.lat[i];
  __syncwarp();
  Ring ring;
  ring_init(mt, tbuf, (int)J.rng[kMTN], lane, ring);

  const double e1 = W.e1, range = W.range, f = W.wl_f;
  const int bins = W.bins, start = W.start, end = W.end;
  const int period = W.hist_period;
  double e_un = W.e0;
  int ibin = wl_bin_index(e_un, e1, range, bins);
  int status = (ibin < start || ibin > end) ? kStatusWalkerOutsideWindow : kStatusOk;
  unsigned long long c_eval = 0, c_draws = 0, c_exp = 0;
  long long accepted = 0;
  DecideStats st = {0u, 0u};

  for (long long i = 1; i <= W.n_trials && status == kStatusOk; ++i) {
    ring_ensure(mt, tbuf, ring, 7, lane);
    const int wb = ring.idx;
    SitePair p;
    draw_site(g, tbuf[wb], tbuf[wb + 1], tbuf[wb + 2], p.ax, p.ay, p.az);
    draw_site(g, tbuf[wb + 3], tbuf[wb + 4], tbuf[wb + 5], p.bx, p.by, p.bz);
    p.ai = compact_index(g, p.ax, p.ay, p.az);
    p.bi = compact_index(g, p.bx, p.by, p.bz);
    p.sa = lat[p.ai];
    p.sb = lat[p.bi];
    double e_sw = e_un;
    int jbin = ibin;
    const bool differ = p.sa != p.sb;
    if (differ) {
      ++c_eval;
      double p_un, p_sw;
      exact_pair_energies(g, CompactLat{lat}, V, ents, sstart, p, lane, p_un, p_sw);
      e_sw = __dadd_rn(__dsub_rn(e_un, p_un), p_sw);
      jbin = wl_bin_index(e_sw, e1, range, bins);
    }
    int consumed = 6;
    if (jbin >= start && jbin <= end) {
      consumed = 7;
      ++c_exp;
      const uint32_t wu = tbuf[wb + 6];
      const double d = __dsub_rn(lng[ibin - start], lng[jbin - start]);
      if (log_u_lt(wu, d, st)) {
        ++accepted;
        e_un = e_sw;
        if (differ && lane == 0) {
          lat[p.ai] = (int8_t)p.sb;
          lat[p.bi] = (int8_t)p.sa;
        }
        ibin = jbin;
      } else {
        jbin = ibin;
      }
    } else {
      jbin = ibin;
    }
    if (period > 0 && (i % period) == 0 && lane == 0)
      hist[jbin - start] = __dadd_rn(hist[jbin - start], 1.0);
    if (lane == 0) lng[jbin - start] = __dadd_rn(lng[jbin - start], f);
    __syncwarp();
    c_draws += consumed;
    ring_consume(ring, consumed);
  }

  __syncwarp();
  for (int i = lane; i < nb; i += 32) {
    W.lng[W.start - 1 + i] = lng[i];
    W.hist[i] = hist[i];
  }
  for (int i = lane; i < g.n_sites; i += 32) J.lat[i] = lat[i];
  ring_writeback(mt, tbuf, ring, J.rng, lane);
  if (lane == 0) {
    W.e_out = e_un;
    W.accepted = accepted;
    unsigned long long* c = J.counters;
    c[kCntTrials] += (unsigned long long)W.n_trials;
    c[kCntEvaluated] += c_eval;
    c[kCntDraws] += c_draws;
    c[kCntAccepted] += (unsigned long long)accepted;
    c[kCntExpTests] += c_exp;
    c[kCntExactPath] += c_eval;
    c[kCntExpFp64] += st.fp64;
    c[kCntExpCr] += st.cr;
    if (status != kStatusOk) *J.status = status;
  }
}

// The window average: for every bin, the walkers' values summed in walker
// order and divided by their count (MPI_Allreduce SUM then /num_walkers,
// src/wang-landau.F90:628-631).  groups[k] lists the walkers of window k.
__global__ void wl_average_kernel(const WlGroup* __restrict__ groups, WlWalker* walkers,
                                  int bins) {
  const WlGroup G = groups[blockIdx.y];
  if (G.count <= 1) return;
  const double inv = (double)(float)G.count;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < bins; b += gridDim.x * blockDim.x) {
    double s = walkers[G.first].lng[b];
    for (int k = 1; k < G.count; ++k) s = __dadd_rn(s, walkers[G.first + k].lng[b]);
    const double a = __ddiv_rn(s, inv);
    for (int k = 0; k < G.count; ++k) walkers[G.first + k].lng[b] = a;
  }
  const int nb = walkers[G.first].end - walkers[G.first].start + 1;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    double s = walkers[G.first].hist[b];
    for (int k = 1; k < G.count; ++k) s = __dadd_rn(s, walkers[G.first + k].hist[b]);
    const double a = __ddiv_rn(s, inv);
    for (int k = 0; k < G.count; ++k) walkers[G.first + k].hist[b] = a;
  }
}

uint32_t wl_smem_bytes(const Geom& g, int nb) {
  uint32_t b = align_up((kMTN + kTbufWords) * 4, 16);
  b += (uint32_t)(g.ns * g.ns * g.nsh) * 8 + 2u * (uint32_t)nb * 8 + (uint32_t)g.z * 4 +
       (uint32_t)(g.nsh + 1) * 2;
  b = align_up(b, 16) + (uint32_t)g.n_sites;
  return align_up(b, 16);
}

void launch_wl_sweeps(WlWalker* d_walkers, int n, uint32_t smem, cudaStream_t stream) {
  cudaFuncSetAttribute(wl_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  wl_sweep_kernel<<<n, 32, smem, stream>>>(d_walkers);
}

void launch_wl_average(const WlGroup* d_groups, int n_groups, WlWalker* d_walkers, int bins,
                       cudaStream_t stream) {
  if (n_groups <= 0) return;
  dim3 grid((bins + 255) / 256, n_groups);
  wl_average_kernel<<<grid, 256, 0, stream>>>(d_groups, d_walkers, bins);
}

}  // namespace brawl
