// Source, add-source, keff / normalisation and residual kernels for sm_103a.
//
// These replace the reference GPU solver's per-FSR kernels and its Thrust
// reductions (src/accel/cuda/GPUSolver.cu:234-760, 1513-1800) and restate
// the CPUSolver semantics (src/CPUSolver.cpp:1860-2660):
//   - reduced source Q/(4 pi) with the negative-source clamp of the first
//     30 iterations, stored divided by sigma_t for the sweep;
//   - phi = phi / (sigma_t V) + 4 pi Q / sigma_t with the negative-flux clamp;
//   - keff *= (sum of nu-fission rates) / R and normalisation factor
//     R / (total fission source), both in FP64;
//   - FISSION_SOURCE, SCALAR_FLUX and TOTAL_SOURCE residuals in FP64.
// All reductions are block reductions in double followed by one double
// atomic per block; the last block (ticket counter) finishes the scalar
// update on the device, so the host never reads intermediate sums.
#include "moc_internal.cuh"

namespace moc {

namespace {

constexpr float kFluxEpsilon = 1.0e-25f;           // src/constants.h:15
constexpr double kFourPi = 12.566370614359172;     // src/constants.h:27
constexpr double kOneOverFourPi = 0.07957747154594767;
constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum_all(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_all_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums v over the block, adds it to *accum and returns true in thread 0 of
// the last block to do so (after which *accum holds the grid total).
__device__ bool block_accumulate(double v, double* accum,
                                 unsigned int* ticket) {
  __shared__ double part[kThreads / 32];
  __shared__ int last;
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int) (blockDim.x >> 5); i++) s += part[i];
    atomicAdd(accum, s);
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  return last && threadIdx.x == 0;
}

__device__ __forceinline__ bool skip(const SolverArgs& a) {
  return a.check_done && *(volatile int*) &a.sc->done;
}

// ---------------------------------------------------------------- sources
// One warp per FSR: the FSR's flux row is staged in shared memory, the
// nu-fission rate is a warp reduction and each lane produces the sources of
// groups lane, lane+32, ... as dot products with rows of the
// (destination-major) scattering matrix.
__global__ void __launch_bounds__(kThreads)
compute_sources_kernel(const SolverArgs a, int iteration, int zero_phi) {
  if (skip(a)) return;
  extern __shared__ float sm[];
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* row = sm + warp * G;
  const double inv_k = 1.0 / a.sc->keff;
  // iteration < 0: the device iteration counter of the running solve
  if (iteration < 0) iteration = a.sc->iteration;
  unsigned long long negatives = 0;
  for (int64_t r = (int64_t) blockIdx.x * wpb + warp; r < a.num_fsrs;
       r += (int64_t) gridDim.x * wpb) {
    const int m = a.fsr_mat[r];
    float* phi = a.phi + r * a.ld;
    for (int g = lane; g < G; g += 32) row[g] = phi[g];
    // fused: the sweep that follows starts from zero tallies; each lane
    // clears exactly the entries it staged
    if (zero_phi)
      for (int g = lane; g < G; g += 32) phi[g] = 0.0f;
    __syncwarp();
    float fr = 0.0f;
    if (a.fissile[m]) {
      const float* nf = a.nu_sigma_f + (int64_t) m * G;
      for (int g = lane; g < G; g += 32) fr = fmaf(nf[g], row[g], fr);
      fr = warp_sum_all(fr);
    }
    const float* ss = a.sigma_s + (int64_t) m * G * G;
    const float* chi = a.chi + (int64_t) m * G;
    const float* st = a.sigma_t + (int64_t) m * G;
    for (int gd = lane; gd < G; gd += 32) {
      const float* srow = ss + (int64_t) gd * G;
      float s = 0.0f;
      for (int g = 0; g < G; g++) s = fmaf(__ldg(srow + g), row[g], s);
      float q = (float) ((double) chi[gd] * (double) fr * inv_k);
      q += s;
      if (a.fixed) q += a.fixed[r * a.ld + gd];
      q *= (float) kOneOverFourPi;
      if (q < 0.0f) {
        negatives++;
        if (iteration < 30) q = kFluxEpsilon;
      }
      a.qt[r * a.ld + gd] = q / st[gd];
    }
    __syncwarp();
  }
  if (negatives) atomicAdd(&a.sc->neg_sources, negatives);
}

// ------------------------------------------------------------- add source
__global__ void __launch_bounds__(kThreads)
add_source_kernel(const SolverArgs a, int update) {
  if (skip(a)) return;
  const int G = a.num_groups;
  const int64_t n = a.num_fsrs * G;
  double rate = 0.0;
  unsigned long long negatives = 0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int64_t r = i / G;
    const int g = (int) (i - r * G);
    const int m = a.fsr_mat[r];
    const float vol0 = a.fsr_vol[r];
    const float vol = (vol0 < 1.0e-12f) ? 1.0e30f : vol0;
    const float st = a.sigma_t[(int64_t) m * G + g];
    const int64_t j = r * a.ld + g;
    float v = a.phi[j];
    v /= (st * vol);
    v += (float) kFourPi * a.qt[j];
    if (v < 0.0f) {
      v = kFluxEpsilon;
      negatives++;
    }
    a.phi[j] = v;
    if (update)
      rate += (double) (a.nu_sigma_f[(int64_t) m * G + g] * v) * (double) vol0;
  }
  if (negatives) atomicAdd(&a.sc->neg_fluxes, negatives);
  if (!update) return;
  DevScalars* sc = a.sc;
  if (block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate)) {
    const double total = *(volatile double*) &sc->accum_rate;
    const double R = (double) a.num_fsrs;
    // CPUSolver::computeKeff then normalizeFluxes (src/CPUSolver.cpp:2327,
    // 1910): both use the same volume-integrated nu-fission total.
    sc->keff = sc->keff * (total / R);
    sc->factor = R / total;
    sc->scale[sc->cur] *= (float) sc->factor;
    sc->accum_rate = 0.0;
    sc->ticket_rate = 0;
    __threadfence();
  }
}

// --------------------------------------------------------------- residual
// One warp per FSR.  Optionally scales phi by sc->factor (the normalisation
// of the eigenvalue loop), accumulates the residual of res_type against
// phi_old, optionally stores phi into phi_old, and the last block finishes
// the iteration: convergence test and counters
// (Solver::computeEigenvalue / computeSource / computeFlux loop bodies,
// src/Solver.cpp:1390-1450, 1500-1530, 1614-1685).
__global__ void __launch_bounds__(kThreads)
residual_kernel(const SolverArgs a, int res_type, int normalise, int store,
                int finish) {
  if (skip(a)) return;
  DevScalars* sc = a.sc;
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const double factor = normalise ? sc->factor : 1.0;
  const double inv_k = 1.0 / sc->keff;
  double part = 0.0;
  for (int64_t r = (int64_t) blockIdx.x * wpb + warp; r < a.num_fsrs;
       r += (int64_t) gridDim.x * wpb) {
    const int m = a.fsr_mat[r];
    const bool fis = a.fissile[m] != 0;
    const float* nf = a.nu_sigma_f + (int64_t) m * G;
    const float* so = a.scat_out + (int64_t) m * G;
    double nw = 0.0, od = 0.0, sq = 0.0, snw = 0.0, sod = 0.0;
    for (int g = lane; g < G; g += 32) {
      const int64_t j = r * a.ld + g;
      float v = a.phi[j];
      if (normalise) {
        v = (float) ((double) v * factor);
        a.phi[j] = v;
      }
      const float o = a.phi_old[j];
      if (res_type == 0) {
        if (o > 0.0f) {
          const double d = ((double) v - (double) o) / (double) o;
          sq += d * d;
        }
      } else {
        if (fis) {
          nw += (double) v * nf[g];
          od += (double) o * nf[g];
        }
        if (res_type == 2) {
          snw += (double) so[g] * v;
          sod += (double) so[g] * o;
        }
      }
      if (store) a.phi_old[j] = v;
    }
    if (res_type == 0) {
      sq = warp_sum_all_d(sq);
      if (lane == 0) part += sq;
    } else {
      nw = warp_sum_all_d(nw);
      od = warp_sum_all_d(od);
      if (res_type == 2) {
        snw = warp_sum_all_d(snw);
        sod = warp_sum_all_d(sod);
        nw = nw * inv_k + snw;
        od = od * inv_k + sod;
        if (lane == 0 && od > 0.0) part += ((nw - od) / od) * ((nw - od) / od);
      } else if (lane == 0 && fis && od > 0.0) {
        part += ((nw - od) / od) * ((nw - od) / od);
      }
    }
  }
  if (block_accumulate(part, &sc->accum_res, &sc->ticket_res)) {
    double total = *(volatile double*) &sc->accum_res;
    if (total < 0.0) total = 0.0;
    double norm = (res_type == 1) ? (double) sc->num_fissionable
                                  : (double) a.num_fsrs;
    if (norm <= 0.0) norm = 1.0;
    const double residual = sqrt(total / norm);
    sc->residual = residual;
    sc->accum_res = 0.0;
    sc->ticket_res = 0;
    if (finish) {
      const int i = sc->iteration;
      if (sc->mode == kModeEigen) {
        const int dk = (int) (1e5 * (sc->keff - sc->k_prev));
        sc->dk = dk;
        sc->k_prev = sc->keff;
        sc->iteration = i + 1;
        if (residual < sc->threshold && abs(dk) < 1) {
          sc->converged = 1;
          sc->done = 1;
        }
      } else {
        sc->iteration = i + 1;
        if (i > 1 && residual < sc->threshold) {
          sc->converged = 1;
          sc->done = 1;
        }
      }
      if (sc->iteration >= sc->max_iters) sc->done = 1;
    }
    __threadfence();
  }
}

// ---------------------------------------------- fission-rate reductions
// what = 0: keff *= total / R (CPUSolver::computeKeff, src/CPUSolver.cpp:
// 2258-2333); what = 1: factor = R / total and the next sweep's angular
// fluxes are scaled (CPUSolver::normalizeFluxes, src/CPUSolver.cpp:
// 1860-1933).
__global__ void __launch_bounds__(kThreads)
fission_rate_kernel(const SolverArgs a, int what) {
  const int G = a.num_groups;
  const int64_t n = a.num_fsrs * G;
  double rate = 0.0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int64_t r = i / G;
    const int g = (int) (i - r * G);
    const int m = a.fsr_mat[r];
    rate += (double) (a.nu_sigma_f[(int64_t) m * G + g] *
                      a.phi[r * a.ld + g]) *
            (double) a.fsr_vol[r];
  }
  DevScalars* sc = a.sc;
  if (block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate)) {
    const double total = *(volatile double*) &sc->accum_rate;
    const double R = (double) a.num_fsrs;
    if (what == 0) {
      sc->keff = sc->keff * (total / R);
    } else {
      sc->factor = R / total;
      sc->scale[sc->cur] *= (float) sc->factor;
    }
    sc->accum_rate = 0.0;
    sc->ticket_rate = 0;
    __threadfence();
  }
}

__global__ void scale_phi_kernel(const SolverArgs a) {
  const double f = a.sc->factor;
  const int64_t n = a.num_fsrs * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    a.phi[i] = (float) ((double) a.phi[i] * f);
}

__global__ void zero_phi_kernel(const SolverArgs a) {
  if (skip(a)) return;
  const int64_t n = a.num_fsrs * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    a.phi[i] = 0.0f;
}

__global__ void fill_kernel(float* p, int64_t n, float v) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void fill_chi_kernel(float* phi, const float* chi, int64_t R,
                                int G, int ld) {
  const int64_t n = R * ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int g = (int) (i % ld);
    phi[i] = (g < G) ? chi[g] : 0.0f;
  }
}

// Per-FSR volume-integrated (nu-)fission rate, one warp per FSR
// (GPUSolver::computeFSRFissionRates, src/accel/cuda/GPUSolver.cu:1970).
__global__ void fsr_rates_kernel(const SolverArgs a, double* out, int nu) {
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  for (int64_t r = (int64_t) blockIdx.x * wpb + warp; r < a.num_fsrs;
       r += (int64_t) gridDim.x * wpb) {
    const int m = a.fsr_mat[r];
    const float* xs = (nu ? a.nu_sigma_f : a.sigma_f) + (int64_t) m * G;
    double s = 0.0;
    for (int g = lane; g < G; g += 32)
      s += (double) xs[g] * a.phi[r * a.ld + g];
    s = warp_sum_all_d(s);
    if (lane == 0) out[r] = s * (double) a.fsr_vol[r];
  }
}

int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int) b;
}

}  // namespace

void launch_compute_sources(const SolverArgs& a, int iteration, int fused,
                            cudaStream_t s) {
  const int wpb = kThreads / 32;
  size_t smem = sizeof(float) * (size_t) a.num_groups * wpb;
  int blocks = grid_for(a.num_fsrs, wpb);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(compute_sources_kernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int) smem);
  compute_sources_kernel<<<blocks, kThreads, smem, s>>>(a, iteration, fused);
}

void launch_add_source(const SolverArgs& a, int update, cudaStream_t s) {
  add_source_kernel<<<grid_for(a.num_fsrs * a.num_groups, kThreads), kThreads,
                      0, s>>>(a, update);
}

void launch_residual(const SolverArgs& a, int res_type, int normalise,
                     int store, int finish, cudaStream_t s) {
  residual_kernel<<<grid_for(a.num_fsrs, kThreads / 32), kThreads, 0, s>>>(
      a, res_type, normalise, store, finish);
}

void launch_fission_rate(const SolverArgs& a, int what, cudaStream_t s) {
  fission_rate_kernel<<<grid_for(a.num_fsrs * a.num_groups, kThreads),
                        kThreads, 0, s>>>(a, what);
}

void launch_scale_phi(const SolverArgs& a, cudaStream_t s) {
  scale_phi_kernel<<<grid_for(a.num_fsrs * a.num_groups, kThreads), kThreads,
                     0, s>>>(a);
}

void launch_zero_phi(const SolverArgs& a, cudaStream_t s) {
  zero_phi_kernel<<<grid_for(a.num_fsrs * a.num_groups, kThreads), kThreads,
                    0, s>>>(a);
}

void launch_fill(float* p, int64_t n, float v, cudaStream_t s) {
  fill_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(p, n, v);
}

void launch_fill_chi(float* phi, const float* chi, int64_t R, int G, int ld,
                     cudaStream_t s) {
  fill_chi_kernel<<<grid_for(R * ld, kThreads), kThreads, 0, s>>>(phi, chi, R,
                                                                 G, ld);
}

void launch_fsr_rates(const SolverArgs& a, double* out, int nu,
                      cudaStream_t s) {
  fsr_rates_kernel<<<grid_for(a.num_fsrs, kThreads / 32), kThreads, 0, s>>>(
      a, out, nu);
}

}  // namespace moc
