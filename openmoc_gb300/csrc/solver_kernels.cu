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
// Every kernel maps one warp to one FSR row (lanes over groups, no integer
// division), runs on a grid of a few blocks per SM, and reduces in FP64:
// warp shuffles, one shared-memory pass per block, one double atomic per
// block; the last block (ticket counter) finishes the scalar update on the
// device, so the host never reads intermediate sums.
#include <algorithm>

#include "moc_internal.cuh"

namespace moc {

namespace {

constexpr float kFluxEpsilon = 1.0e-25f;           // src/constants.h:15
constexpr double kFourPi = 12.566370614359172;     // src/constants.h:27
constexpr double kOneOverFourPi = 0.07957747154594767;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRowThreads = 1024;   // row kernels: 32 warps per block

__device__ __forceinline__ double warp_sum_all_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum_all(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums v (one value per warp, taken from lane 0) over the block, adds it to
// *accum and returns true in thread 0 of the last block to do so (after
// which *accum holds the grid total).
__device__ bool block_accumulate(double v, double* accum,
                                 unsigned int* ticket) {
  __shared__ double part[32];
  __shared__ int last;
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

// block_accumulate for two sums sharing one ticket
__device__ bool block_accumulate2(double v, double w, double* accum_v,
                                  double* accum_w, unsigned int* ticket) {
  __shared__ double part[2][32];
  __shared__ int last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    part[0][warp] = v;
    part[1][warp] = w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, t = 0.0;
    for (int i = 0; i < (int) (blockDim.x >> 5); i++) {
      s += part[0][i];
      t += part[1][i];
    }
    atomicAdd(accum_v, s);
    atomicAdd(accum_w, t);
    __threadfence();
    unsigned int k = atomicAdd(ticket, 1u);
    last = (k == gridDim.x - 1);
  }
  __syncthreads();
  return last && threadIdx.x == 0;
}

// keff from the neutron balance, fission / (absorption + leakage)
// (CPUSolver::computeKeff, src/CPUSolver.cpp:2258-2330), by the last block
// of a reduction that accumulated the absorption rate; the leakage is the
// last sweep's tally
__device__ void finish_balance_keff(DevScalars* sc, double fission) {
  const double absorption = *(volatile double*) &sc->accum_abs;
  const double leakage = *(volatile double*) &sc->leakage;
  sc->keff = fission / (absorption + leakage);
  sc->accum_abs = 0.0;
}

__device__ __forceinline__ bool skip(const SolverArgs& a) {
  return a.check_done && *(volatile int*) &a.sc->done;
}

__device__ __forceinline__ int64_t first_row() {
  return ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

__device__ __forceinline__ int64_t row_step() {
  return ((int64_t) gridDim.x * blockDim.x) >> 5;
}

// ---------------------------------------------------------------- sources
// Instances (a.inst set): for each of the lane's destination groups, the
// fission rate of its own instance (the groups [k G_i, (k+1) G_i)) times
// that instance's 1 / keff.  A segmented inclusive scan of nu_sigma_f * phi
// over each instance's groups by shuffles, the instance's total read at its
// last group; only the instance's own terms enter its sum.
template <int S>
__device__ __forceinline__ void instance_fission(const SolverArgs& a,
                                                 const float* nf,
                                                 const float (&ph)[S],
                                                 bool fissile,
                                                 const float* s_ik,
                                                 float (&out)[S]) {
  const int G = a.num_groups, ig = a.inst_groups;
  const int lane = threadIdx.x & 31;
  float scan[S];
  float carry = 0.0f;
#pragma unroll
  for (int j = 0; j < S; j++) {
    const int g = lane + 32 * j;
    float v = (fissile && g < G) ? nf[g] * ph[j] : 0.0f;
    const int start = (g / ig) * ig;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o && g - o >= start) v += t;
    }
    // the instance that runs across the chunk boundary carries on
    if (start < 32 * j) v += carry;
    scan[j] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
#pragma unroll
  for (int j = 0; j < S; j++) {
    const int g = lane + 32 * j;
    const int k = min(g, G - 1) / ig;
    const int last = min((k + 1) * ig, G) - 1;
    float tot = 0.0f;
#pragma unroll
    for (int jj = 0; jj < S; jj++) {
      const float t = __shfl_sync(0xffffffffu, scan[jj], last & 31);
      if (jj == (last >> 5)) tot = t;
    }
    out[j] = tot * s_ik[k];
  }
}

// One warp per FSR: the flux row sits in registers (lane l holds groups
// l, l+32, ...) and is broadcast group by group with shuffles; the
// transposed scattering matrices of all materials ([m][orig][dest]) are
// staged in shared memory, so each step reads one contiguous row of
// destinations.  The fission term is rank one: chi[dest] * (nu_sigma_f .
// phi) / k.  S = ceil(G / 32) destination groups per lane.
// Two FSR rows per warp pass give two independent accumulation chains.
// Row r0 + i is computed when bit i of `on` is set, with its own
// 1 / keff and iteration count (those of its solve in a pool).
template <int S>
__device__ __forceinline__ void source_rows(const SolverArgs& a,
                                            const float* ssT, int64_t r0,
                                            int on_mask, int zero_phi,
                                            int it0, int it1, float ik0,
                                            float ik1,
                                            unsigned long long& negatives,
                                            const float* s_ik = nullptr) {
  const int G = a.num_groups;
  const int GG = G * G;
  const int lane = threadIdx.x & 31;
  float ph[2][S], acc[2][S], fr[2], fi[2][S];
  const float* mT[2];
  int mat[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const int64_t r = r0 + i;
    const bool on = (on_mask >> i) & 1;
    mat[i] = on ? a.fsr_mat[r] : 0;
    float* phi = a.phi + r * a.ld;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      ph[i][j] = (on && g < G) ? phi[g] : 0.0f;
      acc[i][j] = 0.0f;
    }
    // fused: the sweep that follows starts from zero tallies
    if (on && zero_phi) {
#pragma unroll
      for (int j = 0; j < S; j++)
        if (lane + 32 * j < G) phi[lane + 32 * j] = 0.0f;
    }
    fr[i] = 0.0f;
    if (on && a.fissile[mat[i]]) {
      const float* nf = a.nu_sigma_f + (int64_t) mat[i] * G;
#pragma unroll
      for (int j = 0; j < S; j++)
        if (lane + 32 * j < G) fr[i] = fmaf(nf[lane + 32 * j], ph[i][j], fr[i]);
    }
    fr[i] = warp_sum_all(fr[i]);
    if (s_ik) {
      const float* nf = a.nu_sigma_f + (int64_t) mat[i] * G;
      instance_fission<S>(a, nf, ph[i], on && a.fissile[mat[i]], s_ik, fi[i]);
    }
    mT[i] = ssT + (int64_t) mat[i] * GG + lane;
  }
#pragma unroll
  for (int js = 0; js < S; js++) {
    const int gbase = 32 * js;
    const int gcount = min(32, G - gbase);
#pragma unroll 4
    for (int l = 0; l < gcount; l++) {
      const float p0 = __shfl_sync(0xffffffffu, ph[0][js], l);
      const float p1 = __shfl_sync(0xffffffffu, ph[1][js], l);
      const float* c0 = mT[0] + (int64_t) (gbase + l) * G;
      const float* c1 = mT[1] + (int64_t) (gbase + l) * G;
#pragma unroll
      for (int j = 0; j < S; j++)
        if (lane + 32 * j < G) {
          acc[0][j] = fmaf(c0[32 * j], p0, acc[0][j]);
          acc[1][j] = fmaf(c1[32 * j], p1, acc[1][j]);
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 2; i++) {
    if (!((on_mask >> i) & 1)) continue;
    const int64_t r = r0 + i;
    const float* chi = a.chi + (int64_t) mat[i] * G;
    const float* st = a.sigma_t + (int64_t) mat[i] * G;
    const float fk = fr[i] * (i == 0 ? ik0 : ik1);
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int gd = lane + 32 * j;
      if (gd >= G) continue;
      float q = chi[gd] * (s_ik ? fi[i][j] : fk);
      q += acc[i][j];
      if (a.fixed) q += a.fixed[r * a.ld + gd];
      q *= (float) kOneOverFourPi;
      if (q < 0.0f) {
        negatives++;
        if ((i == 0 ? it0 : it1) < 30 && !a.negative_ok) q = kFluxEpsilon;
      }
      a.qt[r * a.ld + gd] = q / st[gd];
    }
  }
}

template <int S>
__global__ void __launch_bounds__(kThreads)
compute_sources_kernel(const SolverArgs a, int iteration, int zero_phi,
                       int staged) {
  if (skip(a)) return;
  extern __shared__ float4 s_ss4[];
  const int G = a.num_groups;
  if (staged) {
    // all materials' transposed matrices, 16 bytes per load, all in flight
    const int n4 = (a.num_materials * G * G + 3) / 4;
    const float4* src = reinterpret_cast<const float4*>(a.sigma_s_T);
#pragma unroll 8
    for (int i = threadIdx.x; i < n4; i += blockDim.x) s_ss4[i] = src[i];
    __syncthreads();
  }
  const float* ssT =
      staged ? reinterpret_cast<const float*>(s_ss4) : a.sigma_s_T;
  const float inv_k1 = a.row_slot ? 0.0f : (float) (1.0 / a.sc->keff);
  // instances: each instance's 1 / keff
  __shared__ float s_ik[kMaxInstances];
  const bool inst = a.inst && !a.row_slot;
  if (inst) {
    if (threadIdx.x < kMaxInstances)
      s_ik[threadIdx.x] = threadIdx.x < a.num_instances
                              ? (float) (1.0 / a.inst->keff[threadIdx.x])
                              : 0.0f;
    __syncthreads();
  }
  // iteration < 0: the device iteration counter of the running solve
  if (iteration < 0 && !a.row_slot) iteration = a.sc->iteration;
  unsigned long long negatives = 0;
  const int64_t warp = first_row(), warps = row_step();
  for (int64_t r = 2 * warp; r < a.num_fsrs; r += 2 * warps) {
    int on = (r + 1 < a.num_fsrs) ? 3 : 1;
    int it0 = iteration, it1 = iteration;
    float ik0 = inv_k1, ik1 = inv_k1;
    if (a.row_slot) {
      // pool rows: each row's own solve; unused rows and finished solves
      // are left untouched
      const int s0 = a.row_slot[r];
      const int s1 = (on & 2) ? a.row_slot[r + 1] : -1;
      const DevScalars* p0 = (s0 >= 0) ? a.slots + s0 : nullptr;
      const DevScalars* p1 = (s1 >= 0) ? a.slots + s1 : nullptr;
      if (!p0 || p0->done) on &= ~1;
      if (!p1 || p1->done) on &= ~2;
      // a computeFlux solve keeps the sources of its first iteration (the
      // fixed source; Solver::computeFlux computes them once): its rows only
      // get their tallies zeroed
      int keep = 0;
      if ((on & 1) && p0->mode == kModeFlux && p0->iteration > 0) keep |= 1;
      if ((on & 2) && p1->mode == kModeFlux && p1->iteration > 0) keep |= 2;
      if (keep && zero_phi) {
        const int lane = threadIdx.x & 31;
        for (int i = 0; i < 2; i++)
          if ((keep >> i) & 1)
            for (int g = lane; g < G; g += 32) a.phi[(r + i) * a.ld + g] = 0.0f;
      }
      on &= ~keep;
      if (!on) continue;
      // the FP64 reciprocals in one lane (the rows are the whole warp's);
      // the flat source reads the iteration only for the clamp of negative
      // sources in the first 30 iterations, which a solve that allows
      // negative fluxes never applies
      const bool lane0 = (threadIdx.x & 31) == 0;
      if (on & 1) {
        it0 = p0->negative_ok ? 30 : p0->iteration;
        if (lane0) ik0 = (float) (1.0 / p0->keff);
      }
      if (on & 2) {
        it1 = p1->negative_ok ? 30 : p1->iteration;
        if (lane0) ik1 = (float) (1.0 / p1->keff);
      }
      ik0 = __shfl_sync(0xffffffffu, ik0, 0);
      ik1 = __shfl_sync(0xffffffffu, ik1, 0);
    }
    source_rows<S>(a, ssT, r, on, zero_phi, it0, it1, ik0, ik1, negatives,
                   inst ? s_ik : nullptr);
  }
  if (negatives) atomicAdd(&a.sc->neg_sources, negatives);
}

// ------------------------------------------------------------- add source
// update = 1: eigenvalue loop -- the nu-fission total also updates keff,
// the normalisation factor and the next sweep's angular-flux scale
// (CPUSolver::computeKeff then normalizeFluxes, src/CPUSolver.cpp:2327,
// 1910: both use the same volume-integrated nu-fission total).
// Row kernels keep a whole FSR row in registers (S = ceil(G/32) values per
// lane): every load of the row is issued before the first store, so a row
// costs one memory round trip.
template <int S>
__global__ void __launch_bounds__(kRowThreads)
add_source_kernel(const SolverArgs a, int update) {
  if (skip(a)) return;
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  double rate = 0.0, arate = 0.0;
  unsigned long long negatives = 0;
  const bool balance = update && a.keff_balance;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const float vol0 = a.fsr_vol[r];
    const float vol = (vol0 < 1.0e-12f) ? 1.0e30f : vol0;
    const float* __restrict__ st = a.sigma_t + (int64_t) m * G;
    const float* __restrict__ so = a.scat_out + (int64_t) m * G;
    const float* __restrict__ nf = a.nu_sigma_f + (int64_t) m * G;
    float* __restrict__ phi = a.phi + r * a.ld;
    const float* __restrict__ qt = a.qt + r * a.ld;
    float v[S], q[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      v[j] = (g < G) ? phi[g] : 0.0f;
      q[j] = (g < G) ? qt[g] : 0.0f;
    }
    float rr = 0.0f, ra = 0.0f;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      if (g >= G) continue;
      const float stg = st[g];
      float x = v[j] / (stg * vol);
      x += (float) kFourPi * q[j];
      if (x < 0.0f && !a.negative_ok) {
        x = kFluxEpsilon;
        negatives++;
      }
      phi[g] = x;
      rr = fmaf(nf[g], x, rr);
      if (balance) ra = fmaf(stg - so[g], x, ra);
    }
    if (update) rate += (double) rr * (double) vol0;
    if (balance) arate += (double) ra * (double) vol0;
  }
  if (negatives) atomicAdd(&a.sc->neg_fluxes, negatives);
  if (!update) return;
  rate = warp_sum_all_d(rate);
  DevScalars* sc = a.sc;
  bool last;
  if (balance)
    last = block_accumulate2(rate, warp_sum_all_d(arate), &sc->accum_rate,
                             &sc->accum_abs, &sc->ticket_rate);
  else
    last = block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate);
  if (last) {
    const double total = *(volatile double*) &sc->accum_rate;
    const double R = (double) a.num_fsrs;
    if (balance) {
      finish_balance_keff(sc, total);
      sc->leakage = 0.0;   // the next sweep tallies afresh
    } else {
      sc->keff = sc->keff * (total / R);
    }
    if (update == 2) {
      // the normalisation factor comes from the stabilized flux
      sc->accum_rate = 0.0;
      sc->ticket_rate = 0;
      __threadfence();
      return;
    }
    sc->factor = R / total;
    sc->scale[sc->cur] *= (float) sc->factor;
    sc->accum_rate = 0.0;
    sc->ticket_rate = 0;
    __threadfence();
  }
}

// --------------------------------------------------------------- residual
// One warp per FSR.  Optionally scales phi by sc->factor (the normalisation
// of the eigenvalue loop), accumulates the residual of type RT against
// phi_old, optionally stores phi into phi_old, and the last block finishes
// the iteration: convergence test and counters
// (Solver::computeEigenvalue / computeSource / computeFlux loop bodies,
// src/Solver.cpp:1390-1450, 1500-1530, 1614-1685).
template <int RT, int S>
__global__ void __launch_bounds__(kRowThreads)
residual_kernel(const SolverArgs a, int normalise, int store, int finish) {
  if (skip(a)) return;
  DevScalars* sc = a.sc;
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  const float factor = normalise ? (float) sc->factor : 1.0f;
  const float inv_k = (float) (1.0 / sc->keff);
  double part = 0.0;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const bool fis = a.fissile[m] != 0;
    if (RT == 1 && !fis && !normalise && !store) continue;
    const float* __restrict__ nf = a.nu_sigma_f + (int64_t) m * G;
    float* __restrict__ phi = a.phi + r * a.ld;
    float* __restrict__ old = a.phi_old + r * a.ld;
    float vv[S], oo[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      vv[j] = (g < G) ? phi[g] : 0.0f;
      oo[j] = (g < G) ? old[g] : 0.0f;
    }
    // RT 0: sum of squared relative changes; otherwise x accumulates the
    // source change from the exact differences v - o and y the old source,
    // so the relative change keeps its accuracy near convergence
    float x = 0.0f, y = 0.0f;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      if (g >= G) continue;
      float v = vv[j];
      if (normalise) {
        // instances: each group takes its own instance's factor
        v *= a.inst ? (float) a.inst->factor[g / a.inst_groups] : factor;
        phi[g] = v;
      }
      const float o = oo[j];
      if (RT == 0) {
        if (o > 0.0f) {
          const float d = (v - o) / o;
          x = fmaf(d, d, x);
        }
      } else if (RT == 1) {
        if (fis) {
          x = fmaf(v - o, nf[g], x);
          y = fmaf(o, nf[g], y);
        }
      } else {
        const float w = (fis ? nf[g] * inv_k : 0.0f) +
                        a.scat_out[(int64_t) m * G + g];
        x = fmaf(v - o, w, x);
        y = fmaf(o, w, y);
      }
      if (store) old[g] = v;
    }
    x = warp_sum_all(x);
    if (RT != 0) y = warp_sum_all(y);
    // block_accumulate takes lane 0's part: the FP64 quotient (1/64 of the
    // FP32 issue rate) runs in that lane alone
    if (lane == 0) {
      if (RT == 0) {
        part += (double) x;
      } else if ((RT == 2 || fis) && y > 0.0f) {
        const double t = (double) x / (double) y;
        part += t * t;
      }
    }
  }
  if (block_accumulate(part, &sc->accum_res, &sc->ticket_res)) {
    double total = *(volatile double*) &sc->accum_res;
    if (total < 0.0) total = 0.0;
    double norm = (RT == 1) ? (double) sc->num_fissionable
                            : (double) a.num_fsrs;
    if (norm <= 0.0) norm = 1.0;
    const double residual = sqrt(total / norm);
    sc->residual = residual;
    sc->accum_res = 0.0;
    sc->ticket_res = 0;
    if (finish) {
      const int i = sc->iteration;
      if (sc->mode == kModeEigen) {
        // instances: the largest change of the instances' keff
        const int dk =
            a.inst ? a.inst->dk : (int) (1e5 * (sc->keff - sc->k_prev));
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
__global__ void __launch_bounds__(kRowThreads)
fission_rate_kernel(const SolverArgs a, int what) {
  if (skip(a)) return;
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  const bool balance = what == 0 && a.keff_balance;
  double rate = 0.0, arate = 0.0;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const float* nf = a.nu_sigma_f + (int64_t) m * G;
    const float* st = a.sigma_t + (int64_t) m * G;
    const float* so = a.scat_out + (int64_t) m * G;
    const float* phi = a.phi + r * a.ld;
    double s = 0.0, t = 0.0;
    for (int g = lane; g < G; g += 32) {
      s += (double) (nf[g] * phi[g]);
      if (balance) t += (double) ((st[g] - so[g]) * phi[g]);
    }
    rate += s * (double) a.fsr_vol[r];
    arate += t * (double) a.fsr_vol[r];
  }
  rate = warp_sum_all_d(rate);
  DevScalars* sc = a.sc;
  bool last;
  if (balance)
    last = block_accumulate2(rate, warp_sum_all_d(arate), &sc->accum_rate,
                             &sc->accum_abs, &sc->ticket_rate);
  else
    last = block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate);
  if (last) {
    const double total = *(volatile double*) &sc->accum_rate;
    const double R = (double) a.num_fsrs;
    if (balance) {
      finish_balance_keff(sc, total);
    } else if (what == 0) {
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

// -------------------------------------------------- transport stabilization
// CPUSolver::computeStabilizingFlux + stabilizeFlux (src/CPUSolver.cpp:
// 2665-2810) in one pass: the stabilizing flux is c1 times the flux at the
// start of the iteration (`base`), added to the new flux, the sum scaled by
// c2; per material and group (DIAGONAL: c1 = -f sigma_s,gg / sigma_t,g,
// c2 = 1 / (1 + c1) where sigma_s,gg < 0, else 0 and 1; YAMAMOTO: the
// group's largest |sigma_s,gg / sigma_t,g| over the FSRs' materials times f,
// c2 = 1 / (1 + c1); GLOBAL: c1 = 1 / f - 1, c2 = f).  In the eigenvalue
// loop (in_loop) it applies from the second iteration on and then computes
// the normalisation factor of the stabilized flux (normalizeFluxes follows
// stabilizeFlux, src/Solver.cpp:1632-1640).  With base_mom set, the flux
// moments of the linear source take the same coefficients against their
// own start-of-iteration values (CPULSSolver::computeStabilizingFlux /
// stabilizeFlux, src/CPULSSolver.cpp:886-1049; base_momz: the z moment).
__global__ void __launch_bounds__(kRowThreads)
stabilize_kernel(const SolverArgs a, const float* base, int in_loop,
                 const float* base_mom, const float* base_momz) {
  if (skip(a)) return;
  DevScalars* sc = a.sc;
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  const bool apply = !in_loop || sc->iteration > 0;
  double rate = 0.0;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const float2* cf = a.stab + (int64_t) m * a.ld;
    const float* nf = a.nu_sigma_f + (int64_t) m * G;
    float* phi = a.phi + r * a.ld;
    const float* b = base + r * a.ld;
    double s = 0.0;
    for (int g = lane; g < G; g += 32) {
      float x = phi[g];
      if (apply) {
        const float2 c = cf[g];
        x = (x + c.x * b[g]) * c.y;
        phi[g] = x;
      }
      s += (double) (nf[g] * x);
    }
    if (base_mom && apply) {
      float2* mom = reinterpret_cast<float2*>(a.mom + r * 2 * a.ld);
      const float2* bm = reinterpret_cast<const float2*>(base_mom + r * 2 * a.ld);
      for (int g = lane; g < G; g += 32) {
        const float2 c = cf[g];
        const float2 b = bm[g];
        float2 v = mom[g];
        v.x = (v.x + c.x * b.x) * c.y;
        v.y = (v.y + c.x * b.y) * c.y;
        mom[g] = v;
        if (base_momz) {
          float* z = a.momz + r * a.ld + g;
          *z = (*z + c.x * base_momz[r * a.ld + g]) * c.y;
        }
      }
    }
    rate += s * (double) a.fsr_vol[r];
  }
  if (!in_loop) return;
  rate = warp_sum_all_d(rate);
  if (block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate)) {
    const double total = *(volatile double*) &sc->accum_rate;
    sc->factor = (double) a.num_fsrs / total;
    sc->scale[sc->cur] *= (float) sc->factor;
    sc->accum_rate = 0.0;
    sc->ticket_rate = 0;
    __threadfence();
  }
}

// ------------------------------------------------------------- instances
// Each instance's fission-rate total sum_r V_r sum over its groups of
// nu_sigma_f phi: per row and instance a warp sum, lane k keeping instance
// k's running total; per block through shared memory, one FP64 atomic per
// instance and block.  The last block finishes: what = 0, the eigenvalue
// update of every instance (keff *= total / R, factor = R / total, the
// pending angular-flux scale, the largest keff change in 1e-5 units, the
// first instance's keff as the solve's); what = 1, the factors alone (the
// starting flux is then scaled by instance_scale_phi_kernel).
__global__ void __launch_bounds__(kRowThreads)
instance_rates_kernel(const SolverArgs a, int what) {
  if (skip(a)) return;
  InstState* in = a.inst;
  const int G = a.num_groups, ig = a.inst_groups, K = a.num_instances;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double mine = 0.0;   // lane k: instance k
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    if (!a.fissile[m]) continue;
    const float* nf = a.nu_sigma_f + (int64_t) m * G;
    const float* phi = a.phi + r * a.ld;
    const double vol = (double) a.fsr_vol[r];
    for (int k = 0; k < K; k++) {
      double p = 0.0;
      for (int g = k * ig + lane; g < (k + 1) * ig; g += 32)
        p += (double) (nf[g] * phi[g]);
      p = warp_sum_all_d(p);
      if (lane == k) mine += p * vol;
    }
  }
  __shared__ double part[kRowThreads / 32][kMaxInstances];
  __shared__ int last;
  if (lane < kMaxInstances) part[warp][lane] = lane < K ? mine : 0.0;
  __syncthreads();
  if (threadIdx.x < K) {
    double t = 0.0;
    for (int w = 0; w < kRowThreads / 32; w++) t += part[w][threadIdx.x];
    atomicAdd(&in->accum[threadIdx.x], t);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&in->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ int s_dk[kMaxInstances];
  const double R = (double) a.num_fsrs;
  if (threadIdx.x < K) {
    const int k = threadIdx.x;
    const double total = *(volatile double*) &in->accum[k];
    in->accum[k] = 0.0;
    in->factor[k] = R / total;
    if (what == 0) {
      in->keff[k] = in->keff[k] * (total / R);
      in->scale[a.sc->cur][k] *= (float) in->factor[k];
      s_dk[k] = abs((int) (1e5 * (in->keff[k] - in->k_prev[k])));
      in->k_prev[k] = in->keff[k];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (what == 0) {
      int dk = 0;
      for (int k = 0; k < K; k++) dk = max(dk, s_dk[k]);
      in->dk = dk;
      a.sc->keff = in->keff[0];
    }
    in->ticket = 0;
    __threadfence();
  }
}

__global__ void instance_scale_phi_kernel(const SolverArgs a) {
  const int64_t n = a.num_fsrs * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int g = (int) (i % a.ld);
    if (g < a.num_groups)
      a.phi[i] = (float) ((double) a.phi[i] * a.inst->factor[g / a.inst_groups]);
  }
}

// --------------------------------------------- fission / scatter sources
// CPUSolver::computeFSRFissionSources / computeFSRScatterSources
// (src/CPUSolver.cpp:2030-2110): one part of the reduced source alone,
// sum over g' of M[g][g'] phi[g'] / (4 pi), M the fission matrix
// chi[g] nu_sigma_f[g'] (which = 0) or the scattering matrix (which = 1);
// no 1 / keff, fixed source or clamping.  Stored divided by sigma_t like
// every reduced source on the device.
__global__ void __launch_bounds__(kRowThreads)
partial_sources_kernel(const SolverArgs a, int which) {
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const float* phi = a.phi + r * a.ld;
    const float* st = a.sigma_t + (int64_t) m * G;
    float* qt = a.qt + r * a.ld;
    double fis = 0.0;
    if (which == 0 && a.fissile[m]) {
      const float* nf = a.nu_sigma_f + (int64_t) m * G;
      for (int g = lane; g < G; g += 32) fis += (double) (nf[g] * phi[g]);
      fis = warp_sum_all_d(fis);
    }
    for (int gd = lane; gd < G; gd += 32) {
      double q = 0.0;
      if (which == 0) {
        q = (double) a.chi[(int64_t) m * G + gd] * fis;
      } else {
        const float* row = a.sigma_s + ((int64_t) m * G + gd) * G;
        for (int g = 0; g < G; g++) q += (double) (row[g] * phi[g]);
      }
      qt[gd] = (float) (q * kOneOverFourPi) / st[gd];
    }
  }
}

__global__ void scale_phi_kernel(const SolverArgs a) {
  const double f = a.sc->factor;
  const int64_t n = a.num_fsrs * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    a.phi[i] = (float) ((double) a.phi[i] * f);
}

// zeroes the flux tallies (and the moment tallies of a linear source)
__global__ void zero_phi_kernel(const SolverArgs a) {
  if (skip(a)) return;
  const int64_t n = a.num_fsrs * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    a.phi[i] = 0.0f;
    if (a.mom) {
      a.mom[2 * i] = 0.0f;
      a.mom[2 * i + 1] = 0.0f;
    }
    if (a.momz) a.momz[i] = 0.0f;
  }
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
  const int lane = threadIdx.x & 31;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const int m = a.fsr_mat[r];
    const float* xs = (nu ? a.nu_sigma_f : a.sigma_f) + (int64_t) m * G;
    double s = 0.0;
    for (int g = lane; g < G; g += 32)
      s += (double) xs[g] * a.phi[r * a.ld + g];
    s = warp_sum_all_d(s);
    if (lane == 0) out[r] = s * (double) a.fsr_vol[r];
  }
}

// Batched pools: the state of the solve owning row r; null for unused rows and finished solves.
__device__ __forceinline__ DevScalars* live_slot(const SolverArgs& a,
                                                 int64_t r) {
  const int sl = a.row_slot[r];
  if (sl < 0) return nullptr;
  DevScalars* ss = a.slots + sl;
  return ss->done ? nullptr : ss;
}

// ----------------------------------------------------------- linear source
// CPULSSolver::computeFSRSources (src/CPULSSolver.cpp:386-527): one warp per
// FSR computes the flat source of CPUSolver and, from the same pass over the
// transposed scattering matrices, the scatter + fission sources of the x
// and y flux moments; the moments go through the FSR's inverse expansion
// matrix, times 1/(8 pi), and are zeroed where the flat source is not
// above 1e-24 during the first 30 iterations (unless negative fluxes are
// allowed).  Stores Q/sigma_t and (q_x, q_y)/sigma_t for the sweep; fused:
// zeroes the flux and moment tallies.  In a pool (a.row_slot set) each row
// takes keff, the iteration count and the negative-flux rule of its solve;
// a computeFlux solve keeps the sources of its first iteration and only has
// its tallies zeroed.
// D3: explicit 3D tracks -- the z moments too and the 3x3 inverse
// (src/CPULSSolver.cpp:466-487).
template <int S, bool D3>
__global__ void __launch_bounds__(kThreads)
ls_sources_kernel(const SolverArgs a, int iteration, int zero, int staged) {
  if (skip(a)) return;
  extern __shared__ float4 s_ss4[];
  const int G = a.num_groups;
  if (staged) {
    const int n4 = (a.num_materials * G * G + 3) / 4;
    const float4* src = reinterpret_cast<const float4*>(a.sigma_s_T);
#pragma unroll 8
    for (int i = threadIdx.x; i < n4; i += blockDim.x) s_ss4[i] = src[i];
    __syncthreads();
  }
  const float* ssT =
      staged ? reinterpret_cast<const float*>(s_ss4) : a.sigma_s_T;
  const bool pool = a.row_slot != nullptr;
  const float inv_k1 = pool ? 0.0f : (float) (1.0 / a.sc->keff);
  if (iteration < 0 && !pool) iteration = a.sc->iteration;
  const int GG = G * G;
  const int lane = threadIdx.x & 31;
  const int ld = a.ld;
  unsigned long long negatives = 0;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    float* phi = a.phi + r * ld;
    float2* mom = reinterpret_cast<float2*>(a.mom + r * 2 * ld);
    float inv_k = inv_k1;
    int it = iteration;
    bool neg_ok = a.negative_ok;
    if (pool) {
      const DevScalars* ss = live_slot(a, r);
      if (!ss) continue;
      if (ss->mode == kModeFlux && ss->iteration > 0) {
        if (zero)
          for (int g = lane; g < G; g += 32) {
            phi[g] = 0.0f;
            mom[g] = make_float2(0.f, 0.f);
            if constexpr (D3) a.momz[r * ld + g] = 0.0f;
          }
        continue;
      }
      it = ss->iteration;
      neg_ok = ss->negative_ok != 0;
      // the FP64 reciprocal in one lane (the row is the whole warp's)
      if (lane == 0) inv_k = (float) (1.0 / ss->keff);
      inv_k = __shfl_sync(0xffffffffu, inv_k, 0);
    }
    const int m = a.fsr_mat[r];
    float* momz = D3 ? a.momz + r * ld : nullptr;
    float ph[S], mx[S], my[S], mz[S], s0[S], s1[S], s2[S], s3[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      const float2 mm = (g < G) ? mom[g] : make_float2(0.f, 0.f);
      ph[j] = (g < G) ? phi[g] : 0.0f;
      mx[j] = mm.x;
      my[j] = mm.y;
      mz[j] = (D3 && g < G) ? momz[g] : 0.0f;
      s0[j] = s1[j] = s2[j] = s3[j] = 0.0f;
    }
    if (zero) {
#pragma unroll
      for (int j = 0; j < S; j++) {
        const int g = lane + 32 * j;
        if (g < G) {
          phi[g] = 0.0f;
          mom[g] = make_float2(0.f, 0.f);
          if constexpr (D3) momz[g] = 0.0f;
        }
      }
    }
    float f0 = 0.0f, f1 = 0.0f, f2v = 0.0f, f3 = 0.0f;
    if (a.fissile[m]) {
      const float* nf = a.nu_sigma_f + (int64_t) m * G;
#pragma unroll
      for (int j = 0; j < S; j++) {
        const int g = lane + 32 * j;
        if (g < G) {
          f0 = fmaf(nf[g], ph[j], f0);
          f1 = fmaf(nf[g], mx[j], f1);
          f2v = fmaf(nf[g], my[j], f2v);
          if constexpr (D3) f3 = fmaf(nf[g], mz[j], f3);
        }
      }
    }
    f0 = warp_sum_all(f0) * inv_k;
    f1 = warp_sum_all(f1) * inv_k;
    f2v = warp_sum_all(f2v) * inv_k;
    if constexpr (D3) f3 = warp_sum_all(f3) * inv_k;
    const float* mT = ssT + (int64_t) m * GG + lane;
#pragma unroll
    for (int js = 0; js < S; js++) {
      const int gbase = 32 * js;
      const int gcount = min(32, G - gbase);
#pragma unroll 2
      for (int l = 0; l < gcount; l++) {
        const float p0 = __shfl_sync(0xffffffffu, ph[js], l);
        const float p1 = __shfl_sync(0xffffffffu, mx[js], l);
        const float p2 = __shfl_sync(0xffffffffu, my[js], l);
        const float p3 = D3 ? __shfl_sync(0xffffffffu, mz[js], l) : 0.0f;
        const float* c = mT + (int64_t) (gbase + l) * G;
#pragma unroll
        for (int j = 0; j < S; j++)
          if (lane + 32 * j < G) {
            const float cf = c[32 * j];
            s0[j] = fmaf(cf, p0, s0[j]);
            s1[j] = fmaf(cf, p1, s1[j]);
            s2[j] = fmaf(cf, p2, s2[j]);
            if constexpr (D3) s3[j] = fmaf(cf, p3, s3[j]);
          }
      }
    }
    const float* chi = a.chi + (int64_t) m * G;
    const float* st = a.sigma_t + (int64_t) m * G;
    constexpr int NC = D3 ? 6 : 3;
    const float il0 = a.ls_ilem[NC * r], il1 = a.ls_ilem[NC * r + 1],
                il2 = a.ls_ilem[NC * r + 2];
    float il3 = 0.0f, il4 = 0.0f, il5 = 0.0f;
    if constexpr (D3) {
      il3 = a.ls_ilem[6 * r + 3];
      il4 = a.ls_ilem[6 * r + 4];
      il5 = a.ls_ilem[6 * r + 5];
    }
    float2* qxy = reinterpret_cast<float2*>(a.qxy + r * 2 * ld);
    const float2* fxy =
        a.fixed_xy ? reinterpret_cast<const float2*>(a.fixed_xy + r * 2 * ld)
                   : nullptr;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int gd = lane + 32 * j;
      if (gd >= G) continue;
      float q = chi[gd] * f0;
      q += s0[j];
      if (a.fixed) q += a.fixed[r * ld + gd];
      q *= (float) kOneOverFourPi;
      if (q < 0.0f) {
        negatives++;
        if (it < 30 && !neg_ok) q = kFluxEpsilon;
      }
      float sx = fmaf(chi[gd], f1, s1[j]);
      float sy = fmaf(chi[gd], f2v, s2[j]);
      float sz = D3 ? fmaf(chi[gd], f3, s3[j]) : 0.0f;
      if (fxy) {
        const float2 fx = fxy[gd];
        sx += fx.x;
        sy += fx.y;
      }
      if (D3 && a.fixed_z) sz += a.fixed_z[r * ld + gd];
      float rx = 0.0f, ry = 0.0f, rz = 0.0f;
      if (neg_ok || q > 10.0f * kFluxEpsilon || it > 29) {
        if constexpr (D3) {
          rx = (float) (kOneOverFourPi / 2) *
               fmaf(il0, sx, fmaf(il2, sy, il3 * sz));
          ry = (float) (kOneOverFourPi / 2) *
               fmaf(il2, sx, fmaf(il1, sy, il4 * sz));
          rz = (float) (kOneOverFourPi / 2) *
               fmaf(il3, sx, fmaf(il4, sy, il5 * sz));
        } else {
          rx = (float) (kOneOverFourPi / 2) * fmaf(il0, sx, il2 * sy);
          ry = (float) (kOneOverFourPi / 2) * fmaf(il2, sx, il1 * sy);
        }
      }
      const float ist = 1.0f / st[gd];
      a.qt[r * ld + gd] = q * ist;
      qxy[gd] = make_float2(rx * ist, ry * ist);
      if constexpr (D3) a.qz[r * ld + gd] = rz * ist;
    }
  }
  if (negatives) atomicAdd(&a.sc->neg_sources, negatives);
}

// CPULSSolver::addSourceToScalarFlux (2D, src/CPULSSolver.cpp:787-882):
//   phi = phi / (sigma_t V) + 4 pi Q / sigma_t,
//   m_x = m_x / (sigma_t V) + 8 pi (q_x c_xx + q_y c_xy) / sigma_t,
//   m_y = m_y / (sigma_t V) + 8 pi (q_x c_xy + q_y c_yy) / sigma_t,
// a negative flux (unless allowed) becomes max(old flux, 1e-25) with zero
// moments.  update = 1 also finishes the keff / normalisation update as
// add_source_kernel does.  In a pool (a.row_slot set; update = 0) each row
// follows its solve's negative-flux rule and leaves its FP64 nu-fission
// term in row_val, as batch_add_source_kernel does.
// D3: explicit 3D tracks -- six source constants per group and the z
// moment (src/CPULSSolver.cpp:824-846).
template <int S, bool D3>
__global__ void __launch_bounds__(kRowThreads)
ls_add_source_kernel(const SolverArgs a, int update) {
  if (skip(a)) return;
  const int G = a.num_groups;
  const int ld = a.ld;
  const int lane = threadIdx.x & 31;
  double rate = 0.0;
  unsigned long long negatives = 0;
  const bool pool = a.row_slot != nullptr;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    DevScalars* ss = nullptr;
    bool neg_ok = a.negative_ok;
    if (pool) {
      ss = live_slot(a, r);
      if (!ss) continue;
      neg_ok = ss->negative_ok != 0;
    }
    const int m = a.fsr_mat[r];
    const float vol0 = a.fsr_vol[r];
    const float vol = (vol0 < 1.0e-12f) ? 1.0e30f : vol0;
    const float* __restrict__ st = a.sigma_t + (int64_t) m * G;
    const float* __restrict__ so = a.scat_out + (int64_t) m * G;
    const float* __restrict__ nf = a.nu_sigma_f + (int64_t) m * G;
    float* __restrict__ phi = a.phi + r * ld;
    const float* __restrict__ qt = a.qt + r * ld;
    const float* __restrict__ old = a.phi_old + r * ld;
    float2* __restrict__ mom = reinterpret_cast<float2*>(a.mom + r * 2 * ld);
    const float2* __restrict__ qm =
        reinterpret_cast<const float2*>(a.qxy + r * 2 * ld);
    constexpr int NC = D3 ? 6 : 3;
    const float* __restrict__ cst = a.ls_const + r * NC * ld;
    float v[S], q[S], o[S], c0[S], c1[S], c2[S], c3[S], c4[S], c5[S];
    float mzv[S], qzv[S];
    float2 mm[S], qq[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      const bool on = g < G;
      v[j] = on ? phi[g] : 0.0f;
      q[j] = on ? qt[g] : 0.0f;
      o[j] = on ? old[g] : 0.0f;
      mm[j] = on ? mom[g] : make_float2(0.f, 0.f);
      qq[j] = on ? qm[g] : make_float2(0.f, 0.f);
      c0[j] = on ? cst[g] : 0.0f;
      c1[j] = on ? cst[ld + g] : 0.0f;
      c2[j] = on ? cst[2 * ld + g] : 0.0f;
      c3[j] = (D3 && on) ? cst[3 * ld + g] : 0.0f;
      c4[j] = (D3 && on) ? cst[4 * ld + g] : 0.0f;
      c5[j] = (D3 && on) ? cst[5 * ld + g] : 0.0f;
      mzv[j] = (D3 && on) ? a.momz[r * ld + g] : 0.0f;
      qzv[j] = (D3 && on) ? a.qz[r * ld + g] : 0.0f;
    }
    float rr = 0.0f;
    int row_neg = 0;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      if (g >= G) continue;
      const float inv = 1.0f / (st[g] * vol);
      float x = fmaf(v[j], inv, (float) kFourPi * q[j]);
      float mx = fmaf(mm[j].x, inv, (float) (2 * kFourPi) *
                                        fmaf(qq[j].x, c0[j], qq[j].y * c2[j]));
      float my = fmaf(mm[j].y, inv, (float) (2 * kFourPi) *
                                        fmaf(qq[j].x, c2[j], qq[j].y * c1[j]));
      float mz = 0.0f;
      if constexpr (D3) {
        // the z terms of the x and y moments, and the z moment
        mx = fmaf((float) (2 * kFourPi) * qzv[j], c3[j], mx);
        my = fmaf((float) (2 * kFourPi) * qzv[j], c4[j], my);
        mz = fmaf(mzv[j], inv,
                  (float) (2 * kFourPi) *
                      fmaf(qq[j].x, c3[j], fmaf(qq[j].y, c4[j], qzv[j] * c5[j])));
      }
      if (x < 0.0f && !neg_ok) {
        x = fmaxf(o[j], kFluxEpsilon);
        mx = 0.0f;
        my = 0.0f;
        mz = 0.0f;
        row_neg++;
      }
      phi[g] = x;
      mom[g] = make_float2(mx, my);
      if constexpr (D3) a.momz[r * ld + g] = mz;
      rr = fmaf(nf[g], x, rr);
    }
    if (pool) {
      const double row_rate = warp_sum_all_d((double) rr * (double) vol0);
      row_neg = __reduce_add_sync(0xffffffffu, row_neg);
      if (lane == 0) {
        a.row_val[r] = row_rate;
        if (row_neg) atomicAdd(&ss->neg_fluxes, (unsigned long long) row_neg);
      }
      continue;
    }
    negatives += row_neg;
    if (update) rate += (double) rr * (double) vol0;
  }
  if (negatives) atomicAdd(&a.sc->neg_fluxes, negatives);
  if (!update) return;
  rate = warp_sum_all_d(rate);
  DevScalars* sc = a.sc;
  if (block_accumulate(rate, &sc->accum_rate, &sc->ticket_rate)) {
    const double total = *(volatile double*) &sc->accum_rate;
    const double R = (double) a.num_fsrs;
    sc->keff = sc->keff * (total / R);
    if (update != 2) {   // 2: the stabilized flux sets the normalisation
      sc->factor = R / total;
      sc->scale[sc->cur] *= (float) sc->factor;
    }
    sc->accum_rate = 0.0;
    sc->ticket_rate = 0;
    __threadfence();
  }
}

// The moments' share of CPULSSolver::normalizeFluxes (src/CPULSSolver.cpp:
// 362-378): moments *= factor.
__global__ void ls_scale_moments_kernel(const SolverArgs a) {
  if (skip(a)) return;
  const float f = (float) a.sc->factor;
  const int64_t n = a.num_fsrs * 2 * a.ld;
  float4* m4 = reinterpret_cast<float4*>(a.mom);
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n / 4;
       i += (int64_t) gridDim.x * blockDim.x) {
    float4 v = m4[i];
    v.x *= f;
    v.y *= f;
    v.z *= f;
    v.w *= f;
    m4[i] = v;
  }
  if (a.momz) {
    float2* z2 = reinterpret_cast<float2*>(a.momz);
    for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
         i < n / 4; i += (int64_t) gridDim.x * blockDim.x) {
      float2 v = z2[i];
      v.x *= f;
      v.y *= f;
      z2[i] = v;
    }
  }
}

// ------------------------------------------------------- batched pools
// A pool holds many independent solves of one group count in shared
// arrays: each solve owns a contiguous range of FSR rows, tracks, segments,
// materials and angle rows.  The row kernels below are the add-source and
// residual kernels above with every scalar taken from the row's solve, and
// the grid-wide reductions split in two: each row leaves its FP64 term in
// row_val, and one block per solve sums its rows in a fixed order and
// updates the solve's state.

template <int S>
__global__ void __launch_bounds__(kRowThreads)
batch_add_source_kernel(const SolverArgs a) {
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    DevScalars* ss = live_slot(a, r);
    if (!ss) continue;
    const int m = a.fsr_mat[r];
    const float vol0 = a.fsr_vol[r];
    const float vol = (vol0 < 1.0e-12f) ? 1.0e30f : vol0;
    const float* __restrict__ st = a.sigma_t + (int64_t) m * G;
    const float* __restrict__ nf = a.nu_sigma_f + (int64_t) m * G;
    float* __restrict__ phi = a.phi + r * a.ld;
    const float* __restrict__ qt = a.qt + r * a.ld;
    float v[S], q[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      v[j] = (g < G) ? phi[g] : 0.0f;
      q[j] = (g < G) ? qt[g] : 0.0f;
    }
    float rr = 0.0f;
    int negatives = 0;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      if (g >= G) continue;
      float x = v[j] / (st[g] * vol);
      x += (float) kFourPi * q[j];
      if (x < 0.0f && !ss->negative_ok) {
        x = kFluxEpsilon;
        negatives++;
      }
      phi[g] = x;
      rr = fmaf(nf[g], x, rr);
    }
    const double rate = warp_sum_all_d((double) rr * (double) vol0);
    negatives = __reduce_add_sync(0xffffffffu, negatives);
    if (lane == 0) {
      a.row_val[r] = rate;
      if (negatives) atomicAdd(&ss->neg_fluxes, (unsigned long long) negatives);
    }
  }
}

// Sum of row_val over the rows of solve blockIdx.x, in a fixed order;
// valid in thread 0.
__device__ double slot_row_sum(const SolverArgs& a, const DevScalars* ss) {
  __shared__ double part[32];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < ss->nrows; i += blockDim.x)
    s += a.row_val[ss->row0 + i];
  s = warp_sum_all_d(s);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = s;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int) (blockDim.x >> 5); i++) t += part[i];
  return t;
}

// keff *= total / R, factor = R / total and the next sweep's angular-flux
// scale, per eigenvalue solve (CPUSolver::computeKeff then normalizeFluxes,
// src/CPUSolver.cpp:2327, 1910).
__global__ void batch_rate_finish_kernel(const SolverArgs a) {
  DevScalars* ss = a.slots + blockIdx.x;
  if (ss->done || ss->mode != kModeEigen) return;
  const double total = slot_row_sum(a, ss);
  if (threadIdx.x == 0) {
    const double R = (double) ss->nrows;
    ss->keff = ss->keff * (total / R);
    ss->factor = R / total;
    ss->scale[a.sc->cur] *= (float) ss->factor;
  }
}

// Residual terms per row: eigenvalue solves are normalised first (with a
// linear source, the flux moments too: CPULSSolver::normalizeFluxes,
// src/CPULSSolver.cpp:362-378); phi is stored into phi_old.  The residual
// type is the solve's own.
template <int S>
__global__ void __launch_bounds__(kRowThreads)
batch_residual_kernel(const SolverArgs a) {
  const int G = a.num_groups;
  const int lane = threadIdx.x & 31;
  for (int64_t r = first_row(); r < a.num_fsrs; r += row_step()) {
    const DevScalars* ss = live_slot(a, r);
    if (!ss) continue;
    const int RT = ss->res_type;
    const bool normalise = ss->mode == kModeEigen;
    const float factor = normalise ? (float) ss->factor : 1.0f;
    // the FP64 reciprocal in one lane (RT is the same for the whole warp)
    float inv_k = 0.0f;
    if (RT == 2) {
      if (lane == 0) inv_k = (float) (1.0 / ss->keff);
      inv_k = __shfl_sync(0xffffffffu, inv_k, 0);
    }
    if (a.mom && normalise) {
      float4* m4 = reinterpret_cast<float4*>(a.mom + r * 2 * a.ld);
      for (int i = lane; i < (a.ld >> 1); i += 32) {
        float4 v = m4[i];
        v.x *= factor;
        v.y *= factor;
        v.z *= factor;
        v.w *= factor;
        m4[i] = v;
      }
    }
    const int m = a.fsr_mat[r];
    const bool fis = a.fissile[m] != 0;
    const float* __restrict__ nf = a.nu_sigma_f + (int64_t) m * G;
    float* __restrict__ phi = a.phi + r * a.ld;
    float* __restrict__ old = a.phi_old + r * a.ld;
    float vv[S], oo[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      vv[j] = (g < G) ? phi[g] : 0.0f;
      oo[j] = (g < G) ? old[g] : 0.0f;
    }
    float x = 0.0f, y = 0.0f;
#pragma unroll
    for (int j = 0; j < S; j++) {
      const int g = lane + 32 * j;
      if (g >= G) continue;
      float v = vv[j];
      if (normalise) {
        v *= factor;
        phi[g] = v;
      }
      const float o = oo[j];
      if (RT == 0) {
        if (o > 0.0f) {
          const float d = (v - o) / o;
          x = fmaf(d, d, x);
        }
      } else if (RT == 1) {
        if (fis) {
          x = fmaf(v - o, nf[g], x);
          y = fmaf(o, nf[g], y);
        }
      } else {
        const float w = (fis ? nf[g] * inv_k : 0.0f) +
                        a.scat_out[(int64_t) m * G + g];
        x = fmaf(v - o, w, x);
        y = fmaf(o, w, y);
      }
      old[g] = v;
    }
    x = warp_sum_all(x);
    y = warp_sum_all(y);
    if (lane == 0) {
      double part = 0.0;
      if (RT == 0) {
        part = (double) x;
      } else if ((RT == 2 || fis) && y > 0.0f) {
        const double t = (double) x / (double) y;
        part = t * t;
      }
      a.row_val[r] = part;
    }
  }
}

// Residual, convergence test and counters per solve (the ends of
// Solver::computeEigenvalue / computeSource loop bodies,
// src/Solver.cpp:1500-1530, 1614-1685).
__global__ void batch_residual_finish_kernel(const SolverArgs a) {
  DevScalars* ss = a.slots + blockIdx.x;
  if (ss->done) return;
  double total = slot_row_sum(a, ss);
  if (threadIdx.x != 0) return;
  if (total < 0.0) total = 0.0;
  double norm = (ss->res_type == 1) ? (double) ss->num_fissionable
                                    : (double) ss->nrows;
  if (norm <= 0.0) norm = 1.0;
  const double residual = sqrt(total / norm);
  ss->residual = residual;
  const int i = ss->iteration;
  if (ss->mode == kModeEigen) {
    const int dk = (int) (1e5 * (ss->keff - ss->k_prev));
    ss->dk = dk;
    ss->k_prev = ss->keff;
    ss->iteration = i + 1;
    if (residual < ss->threshold && abs(dk) < 1) {
      ss->converged = 1;
      ss->done = 1;
    }
  } else {
    ss->iteration = i + 1;
    if (i > 1 && residual < ss->threshold) {
      ss->converged = 1;
      ss->done = 1;
    }
  }
  if (ss->iteration >= ss->max_iters) ss->done = 1;
}

__global__ void batch_init_rows_kernel(const SolverArgs a, int64_t r0,
                                       int64_t n, float value) {
  const int64_t base = r0 * a.ld, count = n * a.ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
       i < count; i += (int64_t) gridDim.x * blockDim.x) {
    a.phi[base + i] = value;
    a.phi_old[base + i] = value;
    a.qt[base + i] = 0.0f;
    if (a.mom) {
      // the flux moments of a flat flux, and no source moments yet
      reinterpret_cast<float2*>(a.mom)[base + i] = make_float2(0.f, 0.f);
      reinterpret_cast<float2*>(a.qxy)[base + i] = make_float2(0.f, 0.f);
    }
  }
}

__global__ void batch_rebase_kernel(int2* segs, int64_t S,
                                    const int32_t* fsr_mat, int32_t r0,
                                    int64_t* seg_off, int32_t* next,
                                    int32_t* track_ang, int32_t* track_slot,
                                    int64_t T, int64_t s0, int32_t t0,
                                    int32_t a0, int32_t slot) {
  const int64_t n = (S > 2 * T + 2) ? S : 2 * T + 2;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    if (i < S) {
      const int f = segs[i].y + r0;
      segs[i].y = f | (fsr_mat[f] << 24);
    }
    if (i <= T) {
      seg_off[i] += s0;
      track_slot[i] = slot;
    }
    if (i < T) track_ang[i] += a0;
    if (i < 2 * T) next[i] += t0;
  }
}

int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int) b;
}

// Row kernels: one warp per FSR, about one block per SM; few blocks keep
// the grid-wide finish (one double atomic, a fence and a ticket per block)
// short.
int row_grid(int64_t rows) {
  int64_t b = (rows + 2 * 32 - 1) / (2 * 32);
  if (b > 152) b = 152;
  if (b < 1) b = 1;
  return (int) b;
}

template <int S>
void launch_sources_s(const SolverArgs& a, int iteration, int fused,
                      cudaStream_t s) {
  // staged as whole float4 words: round up to 16 bytes
  const size_t need =
      (sizeof(float) * (size_t) a.num_materials * a.num_groups * a.num_groups +
       15) & ~(size_t) 15;
  const int staged = need <= 160 * 1024;
  const size_t smem = staged ? need : 0;
  auto kern = compute_sources_kernel<S>;
  // staging costs one matrix copy per block: keep the grid near one wave
  int64_t blocks = (a.num_fsrs + kWarps - 1) / kWarps;
  if (blocks > 152 * 2) blocks = 152 * 2;
  kern<<<(unsigned) blocks, kThreads, smem, s>>>(a, iteration, fused, staged);
}

}  // namespace

void launch_compute_sources(const SolverArgs& a, int iteration, int fused,
                            cudaStream_t s) {
  if (a.tc_tiles > 0 && !a.row_slot) {
    launch_sources_tc(a, iteration, fused, s);
    return;
  }
  switch ((a.num_groups + 31) / 32) {
    case 1: launch_sources_s<1>(a, iteration, fused, s); break;
    case 2: launch_sources_s<2>(a, iteration, fused, s); break;
    case 3: launch_sources_s<3>(a, iteration, fused, s); break;
    case 4: launch_sources_s<4>(a, iteration, fused, s); break;
    case 5: launch_sources_s<5>(a, iteration, fused, s); break;
    case 6: launch_sources_s<6>(a, iteration, fused, s); break;
    case 7: launch_sources_s<7>(a, iteration, fused, s); break;
    default: launch_sources_s<12>(a, iteration, fused, s); break;
  }
}

namespace {

template <int S>
void launch_add_source_s(const SolverArgs& a, int update, cudaStream_t s) {
  add_source_kernel<S><<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a, update);
}

template <int S>
void launch_residual_s(const SolverArgs& a, int res_type, int normalise,
                       int store, int finish, cudaStream_t s) {
  const int b = row_grid(a.num_fsrs);
  if (res_type == 0)
    residual_kernel<0, S><<<b, kRowThreads, 0, s>>>(a, normalise, store,
                                                     finish);
  else if (res_type == 1)
    residual_kernel<1, S><<<b, kRowThreads, 0, s>>>(a, normalise, store,
                                                     finish);
  else
    residual_kernel<2, S><<<b, kRowThreads, 0, s>>>(a, normalise, store,
                                                     finish);
}

}  // namespace

void launch_add_source(const SolverArgs& a, int update, cudaStream_t s) {
  switch ((a.num_groups + 31) / 32) {
    case 1: launch_add_source_s<1>(a, update, s); break;
    case 2: launch_add_source_s<2>(a, update, s); break;
    case 3: launch_add_source_s<3>(a, update, s); break;
    case 4: launch_add_source_s<4>(a, update, s); break;
    case 5: launch_add_source_s<5>(a, update, s); break;
    case 6: launch_add_source_s<6>(a, update, s); break;
    case 7: launch_add_source_s<7>(a, update, s); break;
    default: launch_add_source_s<12>(a, update, s); break;
  }
}

void launch_residual(const SolverArgs& a, int res_type, int normalise,
                     int store, int finish, cudaStream_t s) {
  switch ((a.num_groups + 31) / 32) {
    case 1: launch_residual_s<1>(a, res_type, normalise, store, finish, s); break;
    case 2: launch_residual_s<2>(a, res_type, normalise, store, finish, s); break;
    case 3: launch_residual_s<3>(a, res_type, normalise, store, finish, s); break;
    case 4: launch_residual_s<4>(a, res_type, normalise, store, finish, s); break;
    case 5: launch_residual_s<5>(a, res_type, normalise, store, finish, s); break;
    case 6: launch_residual_s<6>(a, res_type, normalise, store, finish, s); break;
    case 7: launch_residual_s<7>(a, res_type, normalise, store, finish, s); break;
    default: launch_residual_s<12>(a, res_type, normalise, store, finish, s); break;
  }
}

void launch_fission_rate(const SolverArgs& a, int what, cudaStream_t s) {
  fission_rate_kernel<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a, what);
}

void launch_stabilize(const SolverArgs& a, const float* base, int in_loop,
                      cudaStream_t s, const float* base_mom,
                      const float* base_momz) {
  stabilize_kernel<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(
      a, base, in_loop, base_mom, base_momz);
}

void launch_instance_rates(const SolverArgs& a, int what, cudaStream_t s) {
  instance_rates_kernel<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a, what);
  if (what == 1)
    instance_scale_phi_kernel<<<grid_for(a.num_fsrs * a.ld, kThreads), kThreads,
                                0, s>>>(a);
}

void launch_partial_sources(const SolverArgs& a, int which, cudaStream_t s) {
  partial_sources_kernel<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a,
                                                                     which);
}

void launch_scale_phi(const SolverArgs& a, cudaStream_t s) {
  scale_phi_kernel<<<grid_for(a.num_fsrs * a.num_groups, kThreads), kThreads,
                     0, s>>>(a);
}

void launch_zero_phi(const SolverArgs& a, cudaStream_t s) {
  zero_phi_kernel<<<grid_for(a.num_fsrs * a.ld, kThreads), kThreads, 0, s>>>(
      a);
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
  fsr_rates_kernel<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a, out, nu);
}

// ---- batched pools -------------------------------------------------------
void launch_batch_sources(const SolverArgs& a, cudaStream_t s) {
  launch_compute_sources(a, 0, 1, s);
}

void launch_batch_add_source(const SolverArgs& a, cudaStream_t s) {
  const int b = row_grid(a.num_fsrs);
  switch ((a.num_groups + 31) / 32) {
    case 1: batch_add_source_kernel<1><<<b, kRowThreads, 0, s>>>(a); break;
    case 2: batch_add_source_kernel<2><<<b, kRowThreads, 0, s>>>(a); break;
    case 3: batch_add_source_kernel<3><<<b, kRowThreads, 0, s>>>(a); break;
    case 4: batch_add_source_kernel<4><<<b, kRowThreads, 0, s>>>(a); break;
    case 5: batch_add_source_kernel<5><<<b, kRowThreads, 0, s>>>(a); break;
    case 6: batch_add_source_kernel<6><<<b, kRowThreads, 0, s>>>(a); break;
    case 7: batch_add_source_kernel<7><<<b, kRowThreads, 0, s>>>(a); break;
    default: batch_add_source_kernel<12><<<b, kRowThreads, 0, s>>>(a); break;
  }
}

void launch_batch_rate_finish(const SolverArgs& a, cudaStream_t s) {
  batch_rate_finish_kernel<<<a.num_slots, kThreads, 0, s>>>(a);
}

void launch_batch_residual(const SolverArgs& a, cudaStream_t s) {
  const int b = row_grid(a.num_fsrs);
  switch ((a.num_groups + 31) / 32) {
    case 1: batch_residual_kernel<1><<<b, kRowThreads, 0, s>>>(a); break;
    case 2: batch_residual_kernel<2><<<b, kRowThreads, 0, s>>>(a); break;
    case 3: batch_residual_kernel<3><<<b, kRowThreads, 0, s>>>(a); break;
    case 4: batch_residual_kernel<4><<<b, kRowThreads, 0, s>>>(a); break;
    case 5: batch_residual_kernel<5><<<b, kRowThreads, 0, s>>>(a); break;
    case 6: batch_residual_kernel<6><<<b, kRowThreads, 0, s>>>(a); break;
    case 7: batch_residual_kernel<7><<<b, kRowThreads, 0, s>>>(a); break;
    default: batch_residual_kernel<12><<<b, kRowThreads, 0, s>>>(a); break;
  }
}

void launch_batch_residual_finish(const SolverArgs& a, cudaStream_t s) {
  batch_residual_finish_kernel<<<a.num_slots, kThreads, 0, s>>>(a);
}

void launch_batch_init_rows(const SolverArgs& a, int64_t r0, int64_t n,
                            float value, cudaStream_t s) {
  batch_init_rows_kernel<<<grid_for(n * a.ld, kThreads), kThreads, 0, s>>>(
      a, r0, n, value);
}

void launch_batch_rebase(int2* segs, int64_t S, const int32_t* fsr_mat,
                         int32_t r0, int64_t* seg_off, int32_t* next,
                         int32_t* track_ang, int32_t* track_slot, int64_t T,
                         int64_t s0, int32_t t0, int32_t a0, int32_t slot,
                         cudaStream_t s) {
  const int64_t n = std::max<int64_t>(S, 2 * T + 2);
  batch_rebase_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(
      segs, S, fsr_mat, r0, seg_off, next, track_ang, track_slot, T, s0, t0,
      a0, slot);
}

// ---- linear source ---------------------------------------------------------
namespace {

template <int S>
void launch_ls_sources_s(const SolverArgs& a, int iteration, int fused,
                         cudaStream_t s) {
  const size_t need =
      (sizeof(float) * (size_t) a.num_materials * a.num_groups * a.num_groups +
       15) & ~(size_t) 15;
  const int staged = need <= 160 * 1024;
  const size_t smem = staged ? need : 0;
  auto kern = a.momz ? ls_sources_kernel<S, true> : ls_sources_kernel<S, false>;
  int64_t blocks = (a.num_fsrs + kWarps - 1) / kWarps;
  if (blocks > 152 * 2) blocks = 152 * 2;
  kern<<<(unsigned) blocks, kThreads, smem, s>>>(a, iteration, fused, staged);
}

template <int S>
void launch_ls_add_source_s(const SolverArgs& a, int update, cudaStream_t s) {
  auto kern = a.momz ? ls_add_source_kernel<S, true> : ls_add_source_kernel<S, false>;
  kern<<<row_grid(a.num_fsrs), kRowThreads, 0, s>>>(a,
                                                                       update);
}

}  // namespace

void launch_ls_sources(const SolverArgs& a, int iteration, int fused,
                       cudaStream_t s) {
  switch ((a.num_groups + 31) / 32) {
    case 1: launch_ls_sources_s<1>(a, iteration, fused, s); break;
    case 2: launch_ls_sources_s<2>(a, iteration, fused, s); break;
    case 3: launch_ls_sources_s<3>(a, iteration, fused, s); break;
    case 4: launch_ls_sources_s<4>(a, iteration, fused, s); break;
    default: launch_ls_sources_s<8>(a, iteration, fused, s); break;
  }
}

void launch_ls_add_source(const SolverArgs& a, int update, cudaStream_t s) {
  switch ((a.num_groups + 31) / 32) {
    case 1: launch_ls_add_source_s<1>(a, update, s); break;
    case 2: launch_ls_add_source_s<2>(a, update, s); break;
    case 3: launch_ls_add_source_s<3>(a, update, s); break;
    case 4: launch_ls_add_source_s<4>(a, update, s); break;
    default: launch_ls_add_source_s<8>(a, update, s); break;
  }
}

void launch_ls_scale_moments(const SolverArgs& a, cudaStream_t s) {
  ls_scale_moments_kernel<<<grid_for(a.num_fsrs * a.ld / 2, kThreads),
                            kThreads, 0, s>>>(a);
}

void configure_sources(int optin) {
  raise_smem_limit(compute_sources_kernel<1>, optin);
  raise_smem_limit(compute_sources_kernel<2>, optin);
  raise_smem_limit(compute_sources_kernel<3>, optin);
  raise_smem_limit(compute_sources_kernel<4>, optin);
  raise_smem_limit(compute_sources_kernel<5>, optin);
  raise_smem_limit(compute_sources_kernel<6>, optin);
  raise_smem_limit(compute_sources_kernel<7>, optin);
  raise_smem_limit(compute_sources_kernel<12>, optin);
  raise_smem_limit(ls_sources_kernel<1, false>, optin);
  raise_smem_limit(ls_sources_kernel<1, true>, optin);
  raise_smem_limit(ls_sources_kernel<2, false>, optin);
  raise_smem_limit(ls_sources_kernel<2, true>, optin);
  raise_smem_limit(ls_sources_kernel<3, false>, optin);
  raise_smem_limit(ls_sources_kernel<3, true>, optin);
  raise_smem_limit(ls_sources_kernel<4, false>, optin);
  raise_smem_limit(ls_sources_kernel<4, true>, optin);
  raise_smem_limit(ls_sources_kernel<8, false>, optin);
  raise_smem_limit(ls_sources_kernel<8, true>, optin);
}

}  // namespace moc
