// asro.cu -- ASRO pair counts on the device and the host-side plan.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>

#include "asro.cuh"

namespace brawl {

namespace {

// nint(): round half away from zero
inline double nint_d(double v) { return (double)std::llround(v); }

}  // namespace

int make_asro_plan(const Geom& g, int wc_range, const double* shells, AsroPlan& plan) {
  if (wc_range < 1 || wc_range > 64) return -1;
  plan.offsets.clear();
  plan.class_mask.clear();
  const int W[3] = {2 * g.n1, 2 * g.n2, 2 * g.n3};
  const int m[3] = {std::min(g.n1, 5), std::min(g.n2, 5), std::min(g.n3, 5)};
  std::map<uint64_t, int> classes;
  for (int dz = -m[2]; dz <= m[2]; ++dz)
    for (int dy = -m[1]; dy <= m[1]; ++dy)
      for (int dx = -m[0]; dx <= m[0]; ++dx) {
        const int d[3] = {dx, dy, dz};
        if (g.lattice == kBcc && !((((dx - dz) & 1) == 0) && (((dy - dz) & 1) == 0))) continue;
        if (g.lattice == kFcc && ((dx + dy + dz) & 1)) continue;
        // minimum image exactly as the reference forms it, for site 0:
        // d = real(i - j); d = d - float(2n) * nint(d / float(2n))
        double comp[3];
        for (int a = 0; a < 3; ++a) {
          int j = ((0 + d[a]) % W[a] + W[a]) % W[a];
          double v = (double)(float)(0 - j);
          const float wf = (float)W[a];
          v = v - (double)(wf * (float)nint_d(v / (double)wf));
          comp[a] = v;
        }
        const double dist = std::sqrt(comp[0] * comp[0] + comp[1] * comp[1] + comp[2] * comp[2]);
        uint64_t mask = 0;
        for (int l = 0; l < wc_range; ++l)
          if (std::fabs(dist - shells[l]) < 1e-3) mask |= 1ull << l;
        if (!mask) continue;
        auto it = classes.find(mask);
        int cls;
        if (it == classes.end()) {
          cls = (int)plan.class_mask.size();
          classes[mask] = cls;
          plan.class_mask.push_back(mask);
        } else {
          cls = it->second;
        }
        if (cls > 255) return -1;
        plan.offsets.push_back((uint32_t)(uint8_t)dx | ((uint32_t)(uint8_t)dy << 8) |
                               ((uint32_t)(uint8_t)dz << 16) | ((uint32_t)cls << 24));
      }
  plan.n_class = std::max(1, (int)plan.class_mask.size());
  return 0;
}

// One grid-stride pass over the chain's sites; each block keeps a shared
// histogram of (species_i, species_j, class) and merges it at the end.
__global__ void asro_kernel(const AsroJob* __restrict__ jp) {
  extern __shared__ unsigned int hist[];
  const AsroJob J = *jp;
  const Geom& g = J.g;
  const int nsp = g.ns + 1;
  const int nh = nsp * nsp * J.n_class;
  unsigned int* pcs = hist + nh;
  for (int i = threadIdx.x; i < nh + nsp; i += blockDim.x) hist[i] = 0u;
  __syncthreads();
  const int W1 = 2 * g.n1, W2 = 2 * g.n2, W3 = 2 * g.n3;
  for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < g.n_sites;
       site += gridDim.x * blockDim.x) {
    int x, y, z;
    decode_site(g, site, x, y, z);
    const int si = J.lat[site];
    atomicAdd(&pcs[si], 1u);
    const int row = si * nsp;
    for (int o = 0; o < J.n_offsets; ++o) {
      int dx, dy, dz, cls;
      unpack_entry(J.offsets[o], dx, dy, dz, cls);
      const int nx = wrap_general(x, dx, W1), ny = wrap_general(y, dy, W2),
                nz = wrap_general(z, dz, W3);
      const int sj = J.lat[compact_index(g, nx, ny, nz)];
      atomicAdd(&hist[(row + sj) * J.n_class + cls], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nh; i += blockDim.x)
    if (hist[i]) atomicAdd(&J.counts[i], (unsigned long long)hist[i]);
  for (int i = threadIdx.x; i < nsp; i += blockDim.x)
    if (pcs[i]) atomicAdd(&J.species_counts[i], (unsigned long long)pcs[i]);
}

void launch_asro(const AsroJob* d_job, const Geom& g, int n_class, cudaStream_t stream) {
  int blocks = (g.n_sites + 255) / 256;
  blocks = std::max(1, std::min(blocks, 152 * 4));
  const int nsp = g.ns + 1;
  const size_t smem = (size_t)(nsp * nsp * n_class + nsp) * 4;
  cudaFuncSetAttribute(asro_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  BRAWL_CARVEOUT(asro_kernel);
  asro_kernel<<<blocks, 256, smem, stream>>>(d_job);
}

void finish_asro(const Geom& g, int wc_range, const AsroPlan& plan,
                 const unsigned long long* counts, double* rho) {
  const int ns = g.ns, nsp = ns + 1;
  const unsigned long long* pc = counts + (size_t)nsp * nsp * plan.n_class;
  for (int l = 0; l < wc_range; ++l)
    for (int j = 1; j <= ns; ++j)
      for (int i = 1; i <= ns; ++i) {
        unsigned long long c = 0;
        for (int k = 0; k < (int)plan.class_mask.size(); ++k)
          if ((plan.class_mask[k] >> l) & 1ull) c += counts[(i * nsp + j) * plan.n_class + k];
        // the reference accumulates +1.0 per pair in FP64 (exact) and
        // divides by the integer particle count
        rho[(i - 1) + ns * ((j - 1) + ns * l)] = (double)c / (double)(long long)pc[i];
      }
}

void lattice_shells_host(const Geom& g, int wc_range, double* shells) {
  // Distinct single-precision distances of occupied sites from the origin
  // (sqrt(real((k-1)**2) + real((j-1)**2) + real((i-1)**2))), with the zeros
  // of the unfilled slots; a value is kept when the next larger distinct
  // value is at least 1e-3 away, as the de-duplication loop does.
  std::set<double> vals;
  vals.insert(0.0);
  for (int z = 0; z < 2 * g.n3; ++z)
    for (int y = 0; y < 2 * g.n2; ++y)
      for (int x = 0; x < 2 * g.n1; ++x) {
        bool occ = g.lattice == kBcc   ? (((x & 1) == (z & 1)) && ((y & 1) == (z & 1)))
                   : g.lattice == kFcc ? (((x + y + z) & 1) == 0)
                                       : true;
        if (!occ) continue;
        float d2 = (float)(z * z) + (float)(y * y) + (float)(x * x);
        vals.insert((double)std::sqrt(d2));
      }
  std::vector<double> v(vals.begin(), vals.end());
  for (int l = 0; l < wc_range; ++l) shells[l] = 0.0;
  int out = 0;
  for (size_t i = 0; i + 1 < v.size() && out < wc_range; ++i) {
    if (std::fabs(v[i] - v[i + 1]) < 1e-3) continue;
    shells[out++] = v[i];
  }
}

}  // namespace brawl
