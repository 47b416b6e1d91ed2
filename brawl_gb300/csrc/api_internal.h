// api_internal.h -- helpers the C-ABI translation units share (not exported
// through include/brawl_gpu.h).
#pragma once

#include <string>

#include <vector>

#include "../../include/brawl_gpu.h"
#include "chain_engine.cuh"
#include "kernels.cuh"
#include "lazy_exact.cuh"
#include "ns_kernels.cuh"
#include "wl_kernels.cuh"

namespace brawl {

// Records msg as the calling thread's last error and returns code.
int api_fail(int code, const std::string& msg);
// Validates a brawl_setup and derives the lattice geometry.
int api_make_geom(const brawl_setup& s, Geom& g);

// One chain of a batch as the serving loop launches it: its job image, the
// kernel it runs in and that kernel's shared memory for it, and an energy
// job (site_energy / out / site_offset left for the caller).
struct ChainSlot {
  ChainJob job;
  int halo;
  uint32_t halo_smem;
  uint32_t smem_lat_bytes, smem_glob_bytes;
  bool use_D;
  EnergyJob energy;
};
int api_batch_chain(brawl_batch* b, int c, ChainSlot& out);
// beta and its fixed-point images for chain c written into j.
void api_batch_beta(brawl_batch* b, int c, ChainJob& j, double beta);
int api_batch_set_rng(brawl_batch* b, int c, const uint32_t state[625]);
cudaStream_t api_batch_stream(brawl_batch* b);
brawl_batch* api_wl_batch(brawl_wl* wl);
std::vector<WlWalker>& api_wl_walkers(brawl_wl* wl);
uint32_t api_wl_smem(brawl_wl* wl);
// the sweep kernel's variant for the walkers: largest z, every D staged
void api_wl_variant(brawl_wl* wl, int* max_z, bool* all_D);
NsRun* api_ns_device_run(brawl_ns* ns, int r);
uint32_t api_ns_smem(brawl_ns* ns);
void api_ns_variant(brawl_ns* ns, int* max_z, bool* all_D);
std::string api_last_error();

// Waits for a stream.  In a thread that set_blocking_waits(true) the wait
// sleeps on a blocking-sync event instead of spinning: the serving loop's
// worker threads, many more than the host cores' share left for the
// scheduler, wait this way whatever flags the CUDA context was created
// with.  Elsewhere it is cudaStreamSynchronize.
cudaError_t stream_wait(cudaStream_t s);
void set_blocking_waits(bool on);

}  // namespace brawl
