// Device side of the CMFD accelerator: the flux reduction onto the coarse
// mesh and the prolongation of the coarse solution back onto the FSRs.  The
// partial currents are tallied by the sweep itself (sweep_kernel.cuh, mode
// 2); the coarse solve runs on the host (cmfd_solve.cpp).
#include <algorithm>

#include "moc_internal.cuh"

namespace moc {

namespace {

constexpr int kPairThreads = 256;

// One warp per (coarse cell, material) pair: S[p][g] = sum over the pair's
// FSRs of phi[r][g] * V[r] in FP64, lanes over groups, FSRs from the CSR
// list of the pair (the per-FSR terms of Cmfd::collapseXS,
// src/Cmfd.cpp:770-900, before the cross sections weight them).
__global__ void __launch_bounds__(kPairThreads)
cmfd_pair_sums_kernel(const float* __restrict__ phi,
                      const float* __restrict__ vol,
                      const int32_t* __restrict__ pair_off,
                      const int32_t* __restrict__ pair_fsr, int P, int G,
                      int ld, double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P;
       p += warps) {
    const int b = pair_off[p], e = pair_off[p + 1];
    for (int g0 = 0; g0 < G; g0 += 32) {
      const int g = g0 + lane;
      double s = 0.0;
      if (g < G)
        for (int i = b; i < e; i++) {
          const int r = pair_fsr[i];
          s += (double) phi[(int64_t) r * ld + g] * (double) vol[r];
        }
      if (g < G) out[(int64_t) p * G + g] = s;
    }
  }
}

// phi[r][g] *= ratio[cell(r)][coarse group(g)] (Cmfd::updateMOCFlux,
// src/Cmfd.cpp:1509-1560); the first thread also installs the coarse
// eigenvalue as the solver's keff (Solver::computeEigenvalue takes
// Cmfd::computeKeff's result, src/Solver.cpp:1600-1604).
__global__ void cmfd_prolong_kernel(float* __restrict__ phi,
                                    const int32_t* __restrict__ fsr_cell,
                                    const int32_t* __restrict__ group_of,
                                    const double* __restrict__ ratio,
                                    int64_t R, int G, int ld, int E,
                                    DevScalars* sc, double keff) {
  const int64_t n = R * ld;
  const int64_t i0 = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i0 == 0) sc->keff = keff;
  for (int64_t i = i0; i < n; i += (int64_t) gridDim.x * blockDim.x) {
    const int64_t r = i / ld;
    const int g = (int) (i - r * ld);
    if (g >= G) continue;
    phi[i] *= (float) ratio[(int64_t) fsr_cell[r] * E + group_of[g]];
  }
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

}  // namespace

void launch_cmfd_pair_sums(const float* phi, const float* vol,
                           const int32_t* pair_off, const int32_t* pair_fsr,
                           int P, int G, int ld, double* out,
                           cudaStream_t s) {
  if (P <= 0) return;
  const int64_t warps_needed = P;
  const int per_block = kPairThreads / 32;
  int blocks = (int) std::min<int64_t>((warps_needed + per_block - 1) / per_block,
                                       (int64_t) 8 * sm_count());
  cmfd_pair_sums_kernel<<<blocks, kPairThreads, 0, s>>>(phi, vol, pair_off,
                                                        pair_fsr, P, G, ld, out);
}

void launch_cmfd_prolong(float* phi, const int32_t* fsr_cell,
                         const int32_t* group_of, const double* ratio,
                         int64_t R, int G, int ld, int E, DevScalars* sc,
                         double keff, cudaStream_t s) {
  const int64_t n = R * ld;
  int blocks = (int) std::min<int64_t>((n + 255) / 256, (int64_t) 8 * sm_count());
  if (blocks < 1) blocks = 1;
  cmfd_prolong_kernel<<<blocks, 256, 0, s>>>(phi, fsr_cell, group_of, ratio, R,
                                             G, ld, E, sc, keff);
}

}  // namespace moc
