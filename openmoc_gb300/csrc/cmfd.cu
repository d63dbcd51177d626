// Device side of the CMFD accelerator: the flux reduction onto the coarse
// mesh, the coarse solve, and the prolongation of the coarse solution back
// onto the FSRs.  The partial currents are tallied by the sweep itself
// (sweep_kernel.cuh, mode 2).  cmfd_solve.cpp holds the same coarse solve on
// the host in FP64.
//
// The coarse solve runs in one block: the coarse problem (a few thousand
// unknowns) is far too small to fill the GPU, and the power iteration's
// hundreds of red-black SOR sweeps are latency-bound, so they run between
// __syncthreads barriers of a single block, with the operands in L1, instead
// of as hundreds of dependent launches or host round trips.  Arithmetic is
// FP32, as in the reference's single-precision build (CMFD_PRECISION float,
// LINALG_TOL 1e-7); block-wide sums are compensated FP32 within a thread,
// FP32 within a warp and FP64 across warps, and the scalar work after them
// runs in one thread, since FP64 issues at a small fraction of the FP32 rate.
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>

#include "moc_internal.cuh"

namespace moc {

namespace {

constexpr int kPairThreads = 256;
constexpr int kSolveThreads = 512;
// the solve kernel's block: up to 4 coarse groups a thread holds little, so
// twice the warps
constexpr int solve_threads(int ec) {
  return (ec > 0 && ec <= 4) ? 1024 : kSolveThreads;
}
// shared memory for the coarse system (vectors, A and couplings)
constexpr int kSolveSmemMax = 216 * 1024;
constexpr float kZeroSigmaT = 1e-6f;          // src/constants.h:34
constexpr double kFluxEps = 1e-25;            // src/constants.h:15
constexpr double kLinalgTol = 1e-7;           // LINALG_TOL, FP32 build
constexpr int kMinIters = 25;                 // src/constants.h:74-81
constexpr int kMaxPowerIters = 25000;
constexpr int kMaxLinearIters = 10000;
// Divergence of a linear solve is a thousandfold rise of the fission-source
// change over its minimum (src/linalg.cpp:345-356); in FP32 a minimum below
// the single-precision resolution is rounding noise, not a trend, so the
// minimum must also exceed this floor (the reference's floor, 1e-10, is
// meant for its double build).
constexpr double kNoiseFloor = 1e-7;
// Near convergence an FP32 iterate stops changing except for rounding: the
// measured change then hovers at the single-precision resolution and may
// never drop below the tolerance.  A change below kStallMax that has not
// halved over kStallWindow checks counts as converged.
constexpr double kStallMax = 1e-6;
constexpr int kStallWindow = 8;
// Bound on the SOR sweeps of one coarse solve (about 0.1 s): past it the
// solve counts as failed and the MOC iteration goes on without prolongation.
constexpr int kMaxSweeps = 200000;

// One warp per (coarse cell, material) pair: S[p][g] = sum over the pair's
// FSRs of phi[r][g] * V[r] in FP64, lanes over groups, FSRs from the CSR
// list of the pair (the per-FSR terms of Cmfd::collapseXS,
// src/Cmfd.cpp:770-900, before the cross sections weight them).
__global__ void __launch_bounds__(kPairThreads)
cmfd_pair_sums_kernel(const float* __restrict__ phi,
                      const float* __restrict__ vol,
                      const int32_t* __restrict__ pair_off,
                      const int32_t* __restrict__ pair_fsr, int P, int G,
                      int ld, double* __restrict__ out, const DevScalars* sc) {
  if (*(volatile const int*) &sc->done) return;
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
// src/Cmfd.cpp:1509-1560).
__global__ void cmfd_prolong_kernel(float* __restrict__ phi,
                                    float2* __restrict__ mom,
                                    const int32_t* __restrict__ fsr_cell,
                                    const int32_t* __restrict__ group_of,
                                    const float* __restrict__ ratio,
                                    CmfdStencil st, int64_t R, int G, int ld,
                                    int E, int unbounded,
                                    const DevScalars* sc) {
  if (*(volatile const int*) &sc->done) return;
  const bool bound = sc->iteration > unbounded;
  const int64_t n = R * ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int64_t r = i / ld;
    const int g = (int) (i - r * ld);
    if (g >= G) continue;
    const int e = group_of[g];
    float q;
    if (st.off) {              // Cmfd::getUpdateRatio with k-nearest stencils
      q = 0.0f;
      for (int j = st.off[r]; j < st.off[r + 1]; j++)
        q += st.coef[j] * ratio[(int64_t) st.cell[j] * E + e];
    } else {
      q = ratio[(int64_t) fsr_cell[r] * E + e];
    }
    if (bound) q = fminf(20.0f, fmaxf(0.05f, q));
    phi[i] *= q;
    if (mom) {                 // linear source: the moments of the group too
      float2 m = mom[i];
      mom[i] = make_float2(m.x * q, m.y * q);
    }
  }
}

// ------------------------------------------------------------ coarse solve
// Neumaier's compensated summation (A. Neumaier, ZAMM 54, 1974) in FP32: a
// thread's partial sum over its share of a vector, accurate to a few units
// in the last place however many values the thread adds.
struct FSum {
  float s = 0.0f, c = 0.0f;
  __device__ void add(float v) {
    const float t = s + v;
    c += fabsf(s) >= fabsf(v) ? (s - t) + v : (v - t) + s;
    s = t;
  }
  __device__ float value() const { return s + c; }
};

// Sum over the block of one FP32 value per thread: FP32 within each warp,
// FP64 across the warps.  Thread 0 alone passes the total to `finish` and
// every thread gets finish's result, so the FP64 arithmetic after a
// reduction (a root, a quotient, a convergence test) runs once, not in each
// of the block's threads: an SM issues FP64 at 1/64 of its FP32 rate, and
// those per-thread copies were most of the coarse solve's time.  red holds
// 33 doubles.
// The warp partials red[0..31] of the previous call were read by warp 0
// before that call's last barrier, and its result red[32] is read by every
// thread before it reaches this call's barrier, so writing the partials
// needs no barrier of its own.  Warp 0 adds the partials as a shuffle tree.
template <class F>
__device__ double block_sum(float v, double* red, F finish) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = (double) v;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double t = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[32] = finish(t);
  }
  __syncthreads();
  return red[32];
}

// The coarse system lives in colour order: j is a cell's position in the
// list of red cells ((ix + iy) even) followed by black ones, so that the
// threads of a half sweep take consecutive j.  Arrays are group-major:
// vector element (e, j) at e * C + j, A(e, g) of cell j at (e * E + g) * C +
// j, the coupling of face f at (f * E + e) * C + j, so a warp's loads are
// contiguous.  The collapse works per cell, in cell order.
struct Work {
  // cell order [C][E] ([C][E][E] for sig_s, [C][4][E] for J)
  float *sig_t, *nu_f, *chi, *dif, *dlx, *dly, *phi_c, *sig_s, *J;
  // colour order
  float *A, *nb, *M;                                  // [E][E][C], [4][E][C]
  float *x, *b;          // iterate, right side of the SOR sweeps [E][C]
  float *src_a, *src_b, *ls_a, *ls_b;                 // [E][C]
  float *sa, *sb;        // per row (1 - w) d / w and w / d of the SOR update
  float *phi_t, *rhs, *dd_a, *dd_b, *ddv;             // [E][C]
  const int32_t* nbr;    // [4][C] neighbours in colour order
  // on-chip copies for the SOR sweeps (null: not placed): the neighbour
  // table in 16 bits, and A's off-diagonal part [e][g != e][C] (its
  // diagonal lives in sa / sb)
  const int16_t* nbr16;
  const float* aoff;
};

constexpr int kColourVecs = 13;   // every colour-order vector

__device__ Work carve(float* w, int C, int E) {
  const int64_t CE = (int64_t) C * E, CEE = CE * E, C4E = 4 * CE;
  Work k;
  float** cell_order[] = {&k.sig_t, &k.nu_f, &k.chi, &k.dif, &k.dlx, &k.dly,
                          &k.phi_c};
  for (float** p : cell_order) { *p = w; w += CE; }
  k.sig_s = w; w += CEE;
  k.J = w; w += C4E;
  k.A = w; w += CEE;
  k.nb = w; w += C4E;
  k.M = w; w += CEE;
  float** vecs[] = {&k.x, &k.b, &k.src_a, &k.src_b, &k.ls_a, &k.ls_b, &k.sa,
                    &k.sb, &k.phi_t, &k.rhs, &k.dd_a, &k.dd_b, &k.ddv};
  for (float** p : vecs) { *p = w; w += CE; }
  k.nbr = nullptr;
  k.nbr16 = nullptr;
  k.aoff = nullptr;
  return k;
}

// Shared memory holds what every SOR sweep reads, in this order of
// priority, each array while the budget lasts: x, b, sa, sb (C E floats
// each), the couplings (4 C E), the neighbour table (4 C 16-bit ids; up to
// 32767 cells), A's off-diagonal part (C E (E - 1)).
constexpr int kSmemItems = 7;

__host__ __device__ inline int64_t smem_item_bytes(int i, int C, int E) {
  const int64_t CE = (int64_t) C * E;
  switch (i) {
    case 4: return 16 * CE;
    case 5: return C <= 32767 ? 8 * (int64_t) C : 0;
    // only the instances for up to 8 coarse groups read the copy
    case 6: return E <= 8 ? 4 * CE * (E - 1) : 0;
    default: return 4 * CE;
  }
}

// Items placed (bit i) and their bytes for a budget.
inline int smem_plan(int C, int E, int64_t budget, int64_t* bytes) {
  int mask = 0;
  int64_t used = 0;
  for (int i = 0; i < kSmemItems; i++) {
    const int64_t n = smem_item_bytes(i, C, E);
    if (n > 0 && used + n <= budget) {
      mask |= 1 << i;
      used += n;
    }
  }
  *bytes = used;
  return mask;
}

// Points the placed arrays at shared memory and fills the neighbour table
// and A's off-diagonal part (from A in global memory, written by the build
// kernel); the caller syncs before they are read.
__device__ void place_in_smem(Work& k, char* s, int mask, const CmfdArgs& a) {
  const int C = a.C, E = a.E;
  float** vecs[] = {&k.x, &k.b, &k.sa, &k.sb, &k.nb};
  for (int i = 0; i < kSmemItems; i++) {
    if (!(mask & (1 << i))) continue;
    if (i < 5) {
      *vecs[i] = reinterpret_cast<float*>(s);
    } else if (i == 5) {
      int16_t* t = reinterpret_cast<int16_t*>(s);
      for (int q = threadIdx.x; q < 4 * C; q += blockDim.x)
        t[q] = (int16_t) a.nbr_j[q];
      k.nbr16 = t;
    } else {
      float* t = reinterpret_cast<float*>(s);
      const int n = C * E * (E - 1);
      for (int q = threadIdx.x; q < n; q += blockDim.x) {
        // q = (e * (E - 1) + gi) * C + j, gi-th of the groups g != e
        const int j = q % C, eg = q / C, e = eg / (E - 1), gi = eg % (E - 1);
        const int g = gi < e ? gi : gi + 1;
        t[q] = k.A[((int64_t) e * E + g) * C + j];
      }
      k.aoff = t;
    }
    s += smem_item_bytes(i, C, E);
  }
}

__device__ __forceinline__ int neighbour(const CmfdArgs& a, int c, int f) {
  const int ix = c % a.nx, iy = c / a.nx;
  switch (f) {
    case 0: return ix > 0 ? c - 1 : -1;
    case 1: return iy > 0 ? c - a.nx : -1;
    case 2: return ix + 1 < a.nx ? c + 1 : -1;
    default: return iy + 1 < a.ny ? c + a.nx : -1;
  }
}

// Larsen's effective diffusion coefficient factor
// (Cmfd::computeLarsensEDCFactor, src/Cmfd.cpp:1625-1650).
__device__ float larsen(const CmfdArgs& a, float d, float delta) {
  double rho = 0.0;
  for (int i = 0; i < a.n_edc; i++) {
    const float mu = a.edc_mu[i];
    const float e = expf(-delta / (3.0f * d * mu));
    const float alpha = (1.0f + e) / (1.0f - e) - 2.0f * (3.0f * d * mu) / delta;
    rho += 2.0 * mu * a.edc_w[i] * alpha;
  }
  return (float) (1.0 + delta * rho / (2.0 * d));
}

// out = M x over all (e, j) (no barrier); EC as in sor_half
template <int EC>
__device__ void mat_fission(const CmfdArgs& a, const Work& k, const float* x,
                            float* out) {
  const int E = EC > 0 ? EC : a.E;
  const int C = a.C, CE = a.C * E;
  for (int r = threadIdx.x; r < CE; r += blockDim.x) {
    const int e = r / C, j = r - e * C;
    const float* m = k.M + (int64_t) e * E * C + j;
    float s = 0.0f;
    if constexpr (EC > 0) {
#pragma unroll
      for (int g = 0; g < EC; g++) s += m[g * C] * x[g * C + j];
    } else {
      for (int g = 0; g < E; g++) s += m[(int64_t) g * C] * x[g * C + j];
    }
    out[r] = s;
  }
}

// finish(sum of v[0, n)) for every thread (block_sum)
template <class F>
__device__ double block_total(const float* v, int n, double* red, F finish) {
  FSum t;
  for (int r = threadIdx.x; r < n; r += blockDim.x) t.add(v[r]);
  return block_sum(t.value(), red, finish);
}

__device__ double block_total(const float* v, int n, double* red) {
  return block_total(v, n, red, [](double s) { return s; });
}

// computeRMSE(integrated) (src/linalg.cpp:595-680): the root mean square
// over the cells of the relative change of a cell's source summed over its
// groups, handed to judge (thread 0); every thread gets judge's result.  A
// cell's change is summed from its group differences, which FP32 subtracts
// exactly while old and new are within a factor of two, so the quotient
// keeps FP32 precision without the reference's double sums.
template <class F>
__device__ double rmse(const CmfdArgs& a, const float* x, const float* y,
                       double* red, F judge) {
  FSum part;
  for (int j = threadIdx.x; j < a.C; j += blockDim.x) {
    float d = 0.0f, t = 0.0f;
    for (int e = 0; e < a.E; e++) {
      const float yo = y[e * a.C + j];
      d += x[e * a.C + j] - yo;
      t += yo;
    }
    if (fabsf(t) > (float) kFluxEps) {
      const float r = d / t;
      part.add(r * r);
    }
  }
  const double inv_c = 1.0 / (double) max(a.C, 1);
  return block_sum(part.value(), red, [&](double tot) {
    // the root in FP32: the verdicts need a few digits, not FP64's 16
    return judge((double) sqrtf((float) (tot * inv_c)));
  });
}

// Cmfd::collapseXS (src/Cmfd.cpp:720-1000) for cell c, coarse group e, and
// the coarse currents and Larsen-corrected diffusion coefficients.
__device__ void collapse_one(const CmfdArgs& a, const Work& k, int c, int e) {
  const int E = a.E, G = a.G;
  const int ce = c * E + e;
  const int p0 = a.cell_pair[c], p1 = a.cell_pair[c + 1];
  double prod_tot = 0.0, chi_t = 0.0;
  for (int p = p0; p < p1; p++) {
    const int m = a.pair_mat[p];
    const double* s = a.S + (int64_t) p * G;
    double prod = 0.0;
    for (int h = 0; h < G; h++) prod += (double) a.nf[m * G + h] * s[h];
    chi_t += (double) a.chi_m[m * E + e] * prod;
    prod_tot += prod;
  }
  // the cell's coarse scattering row, accumulated in registers for up to
  // kRowRegs coarse groups (else in place)
  constexpr int kRowRegs = 8;
  float* ss_row = k.sig_s + (int64_t) ce * E;
  float acc[kRowRegs];
  const bool in_regs = E <= kRowRegs;
#pragma unroll
  for (int g = 0; g < kRowRegs; g++) acc[g] = 0.0f;
  if (!in_regs)
    for (int g = 0; g < E; g++) ss_row[g] = 0.0f;
  double total = 0.0, nuf = 0.0, rxn = 0.0, dsum = 0.0;
  for (int h = a.gstart[e]; h < a.gstart[e + 1]; h++) {
    double r = 0.0, t = 0.0;
    for (int p = p0; p < p1; p++) {
      const int m = a.pair_mat[p];
      const double s = a.S[(int64_t) p * G + h];
      r += s;
      t += (double) a.st[m * G + h] * s;
      nuf += (double) a.nf[m * G + h] * s;
      const float* sr = a.ss_m + ((int64_t) m * G + h) * E;
      if (in_regs) {
#pragma unroll
        for (int g = 0; g < kRowRegs; g++)
          if (g < E) acc[g] += (float) ((double) sr[g] * s);
      } else {
        for (int g = 0; g < E; g++) ss_row[g] += (float) ((double) sr[g] * s);
      }
    }
    total += t;
    rxn += r;
    if (fabs(t) > fabs(r) * (double) FLT_EPSILON) dsum += r / (3.0 * (t / r));
  }
  if (in_regs)
#pragma unroll
    for (int g = 0; g < kRowRegs; g++)
      if (g < E) ss_row[g] = acc[g];
  if (rxn <= 0.0) {
    rxn = kZeroSigmaT;
    dsum = kZeroSigmaT;
    total = kZeroSigmaT;
    if (nuf != 0.0) nuf = kZeroSigmaT;
    for (int g = 0; g < E; g++) ss_row[g] = 0.0f;
  }
  k.sig_t[ce] = (float) (total / rxn);
  k.nu_f[ce] = (float) (nuf / rxn);
  k.dif[ce] = (float) (dsum / rxn);
  k.chi[ce] = fabs(prod_tot) > 0.0 ? (float) (chi_t / prod_tot) : 0.0f;
  k.phi_c[ce] = (float) (rxn / (double) a.cell_vol[c]);
  for (int g = 0; g < E; g++) ss_row[g] = (float) ((double) ss_row[g] / rxn);
  for (int f = 0; f < 4; f++) {
    const float* src = a.cur + ((int64_t) c * 4 + f) * a.ld;
    double j = 0.0;
    for (int h = a.gstart[e]; h < a.gstart[e + 1]; h++) j += src[h];
    k.J[((int64_t) c * 4 + f) * E + e] = (float) j;
  }
  const float d = k.dif[ce];
  k.dlx[ce] = a.n_edc ? d * larsen(a, d, a.wx[c % a.nx]) : d;
  k.dly[ce] = a.n_edc ? d * larsen(a, d, a.wy[c / a.nx]) : d;
}

// Cmfd::getSurfaceDiffusionCoefficient and Cmfd::constructMatrices
// (src/Cmfd.cpp:1048-1170, 1353-1500): row (c, e) of A and M, written in
// colour order.
__device__ void build_row(const CmfdArgs& a, const Work& k, int c, int e,
                          int it, bool valid) {
  const int E = a.E, C = a.C;
  const int ce = c * E + e;
  const int j = a.cell_pos[c];
  const int ix = c % a.nx, iy = c / a.nx;
  const float V = a.cell_vol[c];
  float* arow = k.A + (int64_t) e * E * C + j;        // A(e, g) at g * C
  for (int g = 0; g < E; g++) {
    const float v = -k.sig_s[((int64_t) c * E + g) * E + e] * V;
    arow[(int64_t) g * C] = fabsf(v) > FLT_EPSILON ? v : 0.0f;
  }
  float diag = arow[(int64_t) e * C] + k.sig_t[ce] * V;
  const float flux = k.phi_c[ce];
  for (int f = 0; f < 4; f++) {
    const bool xf = (f == 0 || f == 2);
    const float width = xf ? a.wy[iy] : a.wx[ix];
    const float delta = xf ? a.wx[ix] : a.wy[iy];
    const float d = xf ? k.dlx[ce] : k.dly[ce];
    const int n = neighbour(a, c, f);
    const float j_out = k.J[((int64_t) c * 4 + f) * E + e];
    float dh = 0.0f, dt = 0.0f;
    if (n < 0) {
      if (a.bc[f] == 0) {
        const float cur_out = j_out / width;
        dh = 2.0f * d / delta / (1.0f + 4.0f * d / delta);
        dt = (dh * flux - cur_out) / flux;
      }
    } else {
      const int ne = n * E + e;
      const float delta_n = xf ? a.wx[n % a.nx] : a.wy[n / a.nx];
      const float dn = xf ? k.dlx[ne] : k.dly[ne];
      const float flux_n = k.phi_c[ne];
      const float j_in = k.J[((int64_t) n * 4 + (f ^ 2)) * E + e];
      dh = 2.0f * d * dn / (delta_n * d + delta * dn);
      const float current = (j_out - j_in) / width;
      dt = -(dh * (flux_n - flux) + current) / (flux_n + flux);
      if (a.flux_limiting && it > 0 && fabsf(dt / dh) > 1.0f) {
        dh = current > 0.0f ? fabsf(current / (2.0f * flux))
                            : fabsf(current / (2.0f * flux_n));
        dt = -(dh * (flux_n - flux) + current) / (flux_n + flux);
        dh = fmaxf(dh, fabsf(dt));
      }
    }
    float* old = a.dcorr_old + ((int64_t) c * 4 + f) * E + e;
    if (valid) dt = a.relax * dt + (1.0f - a.relax) * *old;
    if (it == 0) dt = 0.0f;
    *old = dt;
    diag += (dh - dt) * width;
    k.nb[((int64_t) f * E + e) * C + j] = n >= 0 ? -(dh + dt) * width : 0.0f;
  }
  arow[(int64_t) e * C] = diag;
  float* mrow = k.M + (int64_t) e * E * C + j;
  for (int g = 0; g < E; g++) {
    const float v = k.chi[ce] * k.nu_f[c * E + g] * V;
    mrow[(int64_t) g * C] = fabsf(v) > FLT_EPSILON ? v : 0.0f;
  }
  k.x[e * C + j] = flux;           // the collapsed flux starts the solve
  k.phi_t[e * C + j] = flux;
}

// One red-black half sweep of SOR over the cells of `color` (colour order:
// red j < n_color0, black after), groups in order within a cell.  EC > 0:
// the coarse group count fixed at compile time (loops unrolled, the cell's
// iterate in registers); EC = 0: any count.
template <int EC>
__device__ void sor_half(const CmfdArgs& a, const Work& k, const float* b,
                         int color) {
  const int C = a.C;
  const float w = a.sor;
  const int j0 = color ? a.n_color0 : 0;
  const int j1 = color ? a.C : a.n_color0;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    int nbj[4];
    if (k.nbr16) {
#pragma unroll
      for (int f = 0; f < 4; f++) nbj[f] = k.nbr16[f * C + j];
    } else {
#pragma unroll
      for (int f = 0; f < 4; f++) nbj[f] = k.nbr[f * C + j];
    }
    if constexpr (EC > 0) {
      // a missing neighbour points at the cell itself with a zero coupling
#pragma unroll
      for (int f = 0; f < 4; f++) nbj[f] = nbj[f] < 0 ? j : nbj[f];
      // everything that does not depend on this cell's update first (the
      // neighbours are of the other colour), the stores last, so that no
      // load waits behind a store
      float xo[EC], t[EC], sa[EC], sb[EC];
#pragma unroll
      for (int e = 0; e < EC; e++) {
        const int r = e * C + j;
        xo[e] = k.x[r];
        sa[e] = k.sa[r];
        sb[e] = k.sb[r];
        float u = b[r];
#pragma unroll
        for (int f = 0; f < 4; f++)
          u -= k.nb[(f * EC + e) * C + j] * k.x[e * C + nbj[f]];
        t[e] = u;
      }
#pragma unroll
      for (int e = 0; e < EC; e++) {
        float s0 = 0.0f, s1 = 0.0f;      // two partial sums over the groups
        if (k.aoff) {
          const float* arow = k.aoff + e * (EC - 1) * C + j;
#pragma unroll
          for (int g = 0; g < EC; g++)
            if (g != e) {
              const float v = arow[(g < e ? g : g - 1) * C] * xo[g];
              if (g & 1) s1 -= v;
              else s0 -= v;
            }
        } else {
          const float* arow = k.A + e * EC * C + j;
#pragma unroll
          for (int g = 0; g < EC; g++)
            if (g != e) {
              if (g & 1) s1 -= arow[g * C] * xo[g];
              else s0 -= arow[g * C] * xo[g];
            }
        }
        xo[e] = (sa[e] * xo[e] + (t[e] + (s0 + s1))) * sb[e];
      }
#pragma unroll
      for (int e = 0; e < EC; e++) k.x[e * C + j] = xo[e];
    } else {
      const int E = a.E;
      for (int e = 0; e < E; e++) {
        const float* arow = k.A + (int64_t) e * E * C + j;
        const float d = arow[(int64_t) e * C];
        float v = (1.0f - w) * k.x[e * C + j] * (d / w);
        for (int g = 0; g < E; g++)
          if (g != e) v -= arow[(int64_t) g * C] * k.x[g * C + j];
        for (int f = 0; f < 4; f++)
          if (nbj[f] >= 0)
            v -= k.nb[((int64_t) f * E + e) * C + j] * k.x[e * C + nbj[f]];
        v += b[e * C + j];
        k.x[e * C + j] = v * (w / d);
      }
    }
  }
}

// The SOR update's diagonal factors for the current A (no barrier).
template <int EC>
__device__ void sor_prep(const CmfdArgs& a, const Work& k) {
  const int E = EC > 0 ? EC : a.E, C = a.C, CE = a.C * E;
  const float w = a.sor;
  for (int r = threadIdx.x; r < CE; r += blockDim.x) {
    const int e = r / C, j = r - e * C;
    const float d = k.A[((int64_t) e * E + e) * C + j];
    k.sa[r] = (1.0f - w) * (d / w);
    k.sb[r] = w / d;
  }
}

// linearSolve (src/linalg.cpp:179-385): red-black SOR on A x = b until the
// fission source settles; false when it diverges or does not converge.
// Uniform across the block (every branch depends on block-wide values).
template <int EC>
__device__ bool linear_solve(const CmfdArgs& a, const Work& k, const float* b,
                             double tol, double* red, int& sweeps) {
  tol = fmax(kLinalgTol, tol);
  float* ls_old = k.ls_a;
  float* ls_new = k.ls_b;
  sor_prep<EC>(a, k);
  mat_fission<EC>(a, k, k.x, ls_old);
  __syncthreads();
  // the convergence state lives in thread 0, which judges each residual
  double linit = 0.0, inv_linit = INFINITY, min_res = 1e6, stall_res = INFINITY;
  int li = 0, stall_li = 0;
  while (li < kMaxLinearIters) {
    sor_half<EC>(a, k, b, 0);
    __syncthreads();
    sor_half<EC>(a, k, b, 1);
    __syncthreads();
    sweeps++;
    // the new fission source is read at the first sweep and from the 25th
    // on (residuals and the copy to the old source)
    if (li == 0 || li + 1 >= kMinIters) {
      mat_fission<EC>(a, k, k.x, ls_new);
      __syncthreads();
    }
    if (li == 0)
      rmse(a, ls_new, ls_old, red, [&](double r) {
        inv_linit = r > 0.0 ? 1.0 / r : INFINITY;
        return linit = r;
      });
    li++;
    if (li > kMinIters) {
      // 1 converged, -1 diverged, 0 not yet
      const double verdict = rmse(a, ls_new, ls_old, red, [&](double r) {
        min_res = fmin(min_res, r);
        if ((r > 1e3 * min_res && min_res > kNoiseFloor) || !isfinite(r)) return -1.0;
        const double q = linit > 0.0 ? r * inv_linit : INFINITY;
        if (q < 0.1 || r < tol) return 1.0;
        if (li - stall_li >= kStallWindow) {
          if (r < kStallMax && r > 0.5 * stall_res) return 1.0;
          stall_res = r;
          stall_li = li;
        }
        return 0.0;
      });
      if (verdict < 0.0) return false;
      if (verdict > 0.0) return true;
    }
    if (li > kMinIters - 1 && li < kMaxLinearIters) {
      float* t = ls_old;
      ls_old = ls_new;
      ls_new = t;
    }
    if (sweeps >= kMaxSweeps) return false;
    __syncthreads();   // ls_new is rewritten by the next sweep
  }
  return false;
}

// ddLinearSolve (src/linalg.cpp:717-900): A made diagonally dominant by
// adding dd = max(0, sum |off-diagonal| - diagonal) to each diagonal, the
// difference moved to the right side (b + dd x) and linearSolve repeated
// until the fission source settles; A is restored on success.
template <int EC>
__device__ bool dd_linear_solve(const CmfdArgs& a, const Work& k,
                                const float* b, double tol, double* red,
                                int& sweeps) {
  const int E = a.E, C = a.C, CE = a.C * a.E;
  for (int r = threadIdx.x; r < CE; r += blockDim.x) {   // r = e * C + j
    const int e = r / C, j = r - e * C;
    float* arow = k.A + (int64_t) e * E * C + j;
    double sum = 0.0;
    for (int g = 0; g < E; g++)
      if (g != e) sum += fabsf(arow[(int64_t) g * C]);
    for (int f = 0; f < 4; f++) sum += fabsf(k.nb[((int64_t) f * E + e) * C + j]);
    const float diag = arow[(int64_t) e * C];
    const float dd = sum > (double) diag ? (float) (sum - diag) : 0.0f;
    k.ddv[r] = dd;
    arow[(int64_t) e * C] = diag + dd;
  }
  __syncthreads();
  // b (on chip) takes the right sides b0 + dd x; b0 waits in k.rhs
  float* bw = const_cast<float*>(b);
  for (int r = threadIdx.x; r < CE; r += blockDim.x) k.rhs[r] = b[r];
  float* old_src = k.dd_a;
  float* new_src = k.dd_b;
  mat_fission<EC>(a, k, k.x, new_src);
  __syncthreads();
  double initial = 0.0, inv_initial = 0.0, min_res = 1e6, stall_res = INFINITY;
  int stall_it = 0;
  for (int it = 0; it < kMaxLinearIters; it++) {
    float* t = old_src;
    old_src = new_src;
    new_src = t;
    for (int r = threadIdx.x; r < CE; r += blockDim.x)
      bw[r] = k.rhs[r] + k.ddv[r] * k.x[r];
    __syncthreads();
    linear_solve<EC>(a, k, bw, tol, red, sweeps);   // a failure is only noted
    mat_fission<EC>(a, k, k.x, new_src);
    __syncthreads();
    // thread 0 judges: 1 settled, -1 diverged, 0 not yet
    const double verdict = rmse(a, new_src, old_src, red, [&](double res) {
      if (it == 0) {
        initial = res < 1e-14 ? 1e-10 : res;
        inv_initial = 1.0 / initial;
      }
      min_res = fmin(min_res, res);
      if ((res > 1e3 * min_res && min_res > kNoiseFloor) || !isfinite(res)) return -1.0;
      if (res * inv_initial < 0.1 || res < tol) return 1.0;
      if (it - stall_it >= kStallWindow) {
        if (res < kStallMax && res > 0.5 * stall_res) return 1.0;
        stall_res = res;
        stall_it = it;
      }
      return 0.0;
    });
    if (verdict < 0.0) return false;
    if (verdict > 0.0) break;
    if (sweeps >= kMaxSweeps) return false;
  }
  for (int r = threadIdx.x; r < CE; r += blockDim.x) {
    const int e = r / C, j = r - e * C;
    k.A[((int64_t) e * E + e) * C + j] -= k.ddv[r];
    bw[r] = k.rhs[r];
  }
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------------------
// The cell-parallel coarse solve.  One thread holds one coarse cell for the
// whole solve, with the cell's row of the system in registers: A's
// off-diagonal part within the cell, the diagonal and the SOR factors, the
// four couplings to its neighbours, its iterate and its right side.  A half
// sweep then reads from shared memory only the neighbours' iterates, and the
// fission products, totals and residuals are per-thread work plus one
// reduction.  Meshes larger than a block (cmfd_cells_threads) split over a
// thread-block cluster by runs of cells: a block keeps, after its own cells'
// slots, copies of the other blocks' cells that border its own, which their
// owners write into its shared memory (distributed shared memory) after
// each of their updates; the hardware cluster barrier after a half sweep
// orders those writes before the reads of the next.  Each block's threads
// hold red cells first, then black ones, so a half sweep leaves whole warps
// idle rather than half of every warp.
//
// Every branch of the solve follows a value all blocks compute identically:
// a block total is written into every block's shared memory, and each
// block's thread 0 adds the totals in block order and judges them, so the
// blocks run the same sweeps and meet at the same cluster barriers.

// Shared-memory stride of a cell's iterate: its E floats in one or two
// 16-byte loads, padded so that eight consecutive cells fall on distinct
// banks.
__host__ __device__ constexpr int cells_xs_stride(int E) {
  return E <= 2 ? E : E <= 4 ? 4 : 12;
}
// Each thread's own rows in shared memory, contiguous so that they move in
// 16-byte (8-byte for E = 2) vectors: the cell's fission matrix M [E][EP],
// kCellVecs vectors of EP floats (the linear solve's old and new fission
// sources, and A's diagonal, read where the SOR factors are formed), and
// from 7 coarse groups on the couplings to the four neighbours [4][EP]
// (which then leave the registers).  EP pads E to the vector width; the
// thread stride is padded to an odd number of vectors so that consecutive
// threads fall on distinct banks.
constexpr int kCellVecs = 3;
constexpr int kDiagVec = 2;
__host__ __device__ constexpr bool cells_nbc_shared(int E) { return E >= 7; }
__host__ __device__ constexpr int cells_ep(int E) {
  return E <= 2 ? E : 4 * ((E + 3) / 4);
}
__host__ __device__ constexpr int cells_row_words(int E) {
  return (E + kCellVecs + (cells_nbc_shared(E) ? 4 : 0)) * cells_ep(E);
}
__host__ __device__ constexpr int cells_row_stride(int E) {
  return E == 1 ? cells_row_words(E)
         : E == 2 ? ((cells_row_words(E) / 2) % 2 == 0 ? cells_row_words(E) + 2
                                                        : cells_row_words(E))
         : ((cells_row_words(E) / 4) % 2 == 0 ? cells_row_words(E) + 4
                                               : cells_row_words(E));
}

// A cell's EC iterates at p (a slot, cells_xs_stride(EC) floats, 8- or
// 16-byte aligned): in one or two vector accesses.
template <int EC>
__device__ __forceinline__ void load_cell(const float* p, float (&v)[EC]) {
  if constexpr (EC == 1) {
    v[0] = p[0];
  } else if constexpr (EC == 2) {
    const float2 q = *reinterpret_cast<const float2*>(p);
    v[0] = q.x;
    v[1] = q.y;
  } else {
#pragma unroll
    for (int k = 0; k < (EC + 3) / 4; k++) {
      const float4 q = reinterpret_cast<const float4*>(p)[k];
      const float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (4 * k + i < EC) v[4 * k + i] = qq[i];
    }
  }
}
template <int EC>
__device__ __forceinline__ void store_cell(float* p, const float (&v)[EC]) {
  if constexpr (EC == 1) {
    p[0] = v[0];
  } else if constexpr (EC == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int k = 0; k < (EC + 3) / 4; k++) {
      float qq[4];
#pragma unroll
      for (int i = 0; i < 4; i++) qq[i] = (4 * k + i < EC) ? v[4 * k + i] : 0.0f;
      reinterpret_cast<float4*>(p)[k] = make_float4(qq[0], qq[1], qq[2], qq[3]);
    }
  }
}

// The convergence state of the nested solves, kept by thread 0 alone (in
// shared memory, so that it holds no registers in the other threads).
// The judgements are threshold tests on residuals formed from FP32 sums,
// so they run in FP32 (an SM issues FP64 at a small fraction of that rate,
// and thread 0's chain of them held every block).
struct CellsJudge {
  float linit, inv_linit, min_res, stall_res, tol;      // linear solve
  float dd_initial, dd_inv_initial, dd_min_res, dd_stall_res;
  float initial, inv_initial, e_stall_res, inv_c;       // power iteration
  int stall_li, stall_it, stall_p;
};

// a + b = s + e exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

template <int EC>
__global__ void __launch_bounds__(cmfd_cells_threads(EC), 1)
cmfd_cells_kernel(const CmfdArgs a) {
  namespace cg = cooperative_groups;
  DevScalars* sc = a.sc;
  if (*(volatile int*) &sc->done) return;    // the same for every block
  constexpr int XS = cells_xs_stride(EC);
  constexpr int EO = EC > 1 ? EC - 1 : 1;
  const int NB = a.map_nb, T = blockDim.x, t = threadIdx.x;
  const int rank = NB > 1 ? (int) cg::this_cluster().block_rank() : 0;
  const int NT = NB * T, gid = rank * T + t;
  const int C = a.C;
  extern __shared__ float4 s_dyn[];
  constexpr int EP = cells_ep(EC), RS = cells_row_stride(EC);
  float* xs = reinterpret_cast<float*>(s_dyn);       // [slots][XS]
  // this thread's rows: M [EC][EP], then the vectors
  float* row = xs + a.map_slots * XS + t * RS;
  float* mm = row;
  __shared__ double red[33];
  __shared__ float2 red2[32];
  __shared__ double part[2][kCmfdMaxClusterBlocks];   // block totals
  __shared__ CellsJudge J;
  int buf = 0;
  auto vrow = [&](int v) { return row + EC * EP + v * EP; };
  auto barrier = [&]() {
    if (NB > 1) cg::this_cluster().sync();
    else __syncthreads();
  };

  // every block of the cluster runs before any writes into another's
  // shared memory
  if (NB > 1) cg::this_cluster().sync();
  const Work g = carve(a.work, C, EC);   // as the build kernel wrote it
  const int j = a.map_j[gid];
  const bool has = j >= 0;
  const int colour = has ? (j >= a.n_color0 ? 1 : 0) : -1;
  // the barrier after a half sweep of colour h: the threads that updated a
  // cell (and wrote its iterate here and into other blocks) release their
  // writes, the others arrive without ordering; all acquire
  auto sweep_barrier = [&](int h) {
    if (NB > 1) {
      if (colour == h)
        asm volatile("barrier.cluster.arrive.release;" ::: "memory");
      else
        asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory");
      asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
    } else {
      __syncthreads();
    }
  };
  int nsl[4], push[2];
#pragma unroll
  for (int f = 0; f < 4; f++) nsl[f] = a.map_nslot[f * NT + gid];
#pragma unroll
  for (int q = 0; q < 2; q++) push[q] = a.map_push[q * NT + gid];
  constexpr bool kNbcShared = cells_nbc_shared(EC);
  float* nbs = row + (EC + kCellVecs) * EP;   // [4][EP] when kNbcShared
  float x[EC], b[EC], sa[EC], sb[EC], nbc[kNbcShared ? 1 : 4][EC], aoff[EC][EO];
#pragma unroll
  for (int e = 0; e < EC; e++) {
    x[e] = has ? g.x[e * C + j] : 0.0f;
    b[e] = 0.0f;
    vrow(kDiagVec)[e] = has ? g.A[(e * EC + e) * C + j] : 1.0f;
#pragma unroll
    for (int q = 0; q < EO; q++) {
      const int gg = q < e ? q : q + 1;
      aoff[e][q] = (has && EC > 1) ? g.A[(e * EC + gg) * C + j] : 0.0f;
    }
#pragma unroll
    for (int f = 0; f < 4; f++) {
      const float v = has ? g.nb[(f * EC + e) * C + j] : 0.0f;
      if constexpr (kNbcShared) nbs[f * EP + e] = v;
      else nbc[f][e] = v;
    }
    float mr[EC];
#pragma unroll
    for (int gg = 0; gg < EC; gg++) mr[gg] = has ? g.M[(e * EC + gg) * C + j] : 0.0f;
    store_cell<EC>(mm + e * EP, mr);
  }
  const float w = a.sor;

  // this cell's iterate into its slot and into the copies other blocks hold
  auto publish = [&]() {
    if (!has) return;
    store_cell<EC>(xs + t * XS, x);
#pragma unroll
    for (int q = 0; q < 2; q++) {
      if (push[q] < 0) continue;
      store_cell<EC>(cg::this_cluster().map_shared_rank(xs, push[q] >> 24) +
                         (push[q] & 0xFFFFFF) * XS,
                     x);
    }
  };
  // One red-black half sweep for this cell: row e of the SOR update,
  //   x_e <- ((1 - w) d_e / w x_e + b_e - sum_f c_fe y_fe - sum_g A_eg x_g) w / d_e,
  // groups in order (x_g new for g < e).  Each row's sum over the old
  // iterates (g > e) is formed first; each new x_e then enters the later
  // rows at once, so that a row waits on one multiply-add of the previous.
  auto half = [&](int h) {
    if (colour != h) return;
    float y[4][EC];   // the neighbours' iterates
#pragma unroll
    for (int f = 0; f < 4; f++) load_cell<EC>(xs + nsl[f] * XS, y[f]);
    float r[EC];
#pragma unroll
    for (int e = 0; e < EC; e++) r[e] = b[e];
#pragma unroll
    for (int f = 0; f < 4; f++) {
      if constexpr (kNbcShared) {
        float cf[EC];
        load_cell<EC>(nbs + f * EP, cf);
#pragma unroll
        for (int e = 0; e < EC; e++) r[e] -= cf[e] * y[f][e];
      } else {
#pragma unroll
        for (int e = 0; e < EC; e++) r[e] -= nbc[f][e] * y[f][e];
      }
    }
#pragma unroll
    for (int e = 0; e < EC; e++) {
      float v = r[e];
#pragma unroll
      for (int gg = e + 1; gg < EC; gg++) v -= aoff[e][gg - 1] * x[gg];
      r[e] = v;
    }
#pragma unroll
    for (int e = 0; e < EC; e++) {
      x[e] = (sa[e] * x[e] + r[e]) * sb[e];
#pragma unroll
      for (int ee = e + 1; ee < EC; ee++) r[ee] -= aoff[ee][e] * x[e];
    }
    publish();
  };
  auto sor_factors = [&]() {
#pragma unroll
    for (int e = 0; e < EC; e++) {
      const float d = vrow(kDiagVec)[e];
      sa[e] = (1.0f - w) * (d / w);
      sb[e] = w / d;
    }
  };
  // out = M v for this cell
  auto fission = [&](const float (&v)[EC], float (&out)[EC]) {
#pragma unroll
    for (int e = 0; e < EC; e++) {
      float mr[EC];
      load_cell<EC>(mm + e * EP, mr);
      float s = 0.0f;
#pragma unroll
      for (int gg = 0; gg < EC; gg++) s += mr[gg] * v[gg];
      out[e] = s;
    }
  };
  auto fission_to = [&](int vi) {
    float o[EC];
    fission(x, o);
    store_cell<EC>(vrow(vi), o);
  };
  // finish(the sum over all cells of every thread's v) for every thread:
  // within a warp and across warps FP32 trees of exact pair sums carrying
  // the rounding errors, across blocks FP64 (blocks in order)
  auto total = [&](float v, auto&& finish) -> double {
    float c = 0.0f;
    for (int o = 16; o > 0; o >>= 1) {
      const float vo = __shfl_xor_sync(0xffffffffu, v, o);
      const float co = __shfl_xor_sync(0xffffffffu, c, o);
      float e;
      two_sum(v, vo, v, e);
      c += co + e;
    }
    const int wi = t >> 5, lane = t & 31;
    if (lane == 0) red2[wi] = make_float2(v, c);
    __syncthreads();
    double s = 0.0;
    if (wi == 0) {
      const float2 q = lane < (T >> 5) ? red2[lane] : make_float2(0.0f, 0.0f);
      v = q.x;
      c = q.y;
      for (int o = 16; o > 0; o >>= 1) {
        const float vo = __shfl_xor_sync(0xffffffffu, v, o);
        const float co = __shfl_xor_sync(0xffffffffu, c, o);
        float e;
        two_sum(v, vo, v, e);
        c += co + e;
      }
      s = (double) v + (double) c;
    }
    if (NB > 1) {
      if (t == 0)
        for (int r = 0; r < NB; r++)
          cg::this_cluster().map_shared_rank(&part[0][0], r)[buf * kCmfdMaxClusterBlocks + rank] = s;
      cg::this_cluster().sync();
      if (t == 0) {
        s = 0.0;
        for (int r = 0; r < NB; r++) s += part[buf][r];
      }
      buf ^= 1;
    }
    if (t == 0) red[32] = finish(s);
    __syncthreads();
    return red[32];
  };
  auto cell_sum = [&](const float (&v)[EC]) {
    FSum s;
#pragma unroll
    for (int e = 0; e < EC; e++) s.add(v[e]);
    return has ? s.value() : 0.0f;
  };
  if (t == 0) J.inv_c = 1.0f / (float) max(C, 1);
  // computeRMSE of this cell's change from y to xv, judged by thread 0
  auto rmse = [&](const float (&xv)[EC], const float (&y)[EC], auto&& judge) {
    float r2 = 0.0f;
    if (has) {
      float d = 0.0f, tt = 0.0f;
#pragma unroll
      for (int e = 0; e < EC; e++) {
        d += xv[e] - y[e];
        tt += y[e];
      }
      if (fabsf(tt) > (float) kFluxEps) {
        const float r = d / tt;
        r2 = r * r;
      }
    }
    return total(r2, [&](double tot) {
      return judge(sqrtf((float) tot * J.inv_c));
    });
  };
  auto load = [&](int vi, float (&o)[EC]) { load_cell<EC>(vrow(vi), o); };

  int sweeps = 0, power = 0;
  // linearSolve (src/linalg.cpp:179-385), as linear_solve
  auto linear = [&](double tol) -> bool {
    if (t == 0) {
      J.tol = (float) fmax(kLinalgTol, tol);
      J.linit = 0.0f;
      J.inv_linit = INFINITY;
      J.min_res = 1e6f;
      J.stall_res = INFINITY;
      J.stall_li = 0;
    }
    int ls_old = 0, ls_new = 1;
    sor_factors();
    fission_to(ls_old);
    int li = 0;
    while (li < kMaxLinearIters) {
      half(0);
      sweep_barrier(0);
      half(1);
      sweep_barrier(1);
      sweeps++;
      float fo[EC], fn[EC];
      if (li == 0 || li + 1 >= kMinIters) fission_to(ls_new);
      if (li == 0) {
        load(ls_new, fn);
        load(ls_old, fo);
        rmse(fn, fo, [&](float r) {
          J.inv_linit = r > 0.0f ? 1.0f / r : INFINITY;
          J.linit = r;
          return 0.0;
        });
      }
      li++;
      if (li > kMinIters) {
        load(ls_new, fn);
        load(ls_old, fo);
        const double verdict = rmse(fn, fo, [&](float r) {
          J.min_res = fminf(J.min_res, r);
          if ((r > 1e3f * J.min_res && J.min_res > (float) kNoiseFloor) || !isfinite(r))
            return -1.0;
          const float q = J.linit > 0.0f ? r * J.inv_linit : INFINITY;
          if (q < 0.1f || r < J.tol) return 1.0;
          if (li - J.stall_li >= kStallWindow) {
            if (r < (float) kStallMax && r > 0.5f * J.stall_res) return 1.0;
            J.stall_res = r;
            J.stall_li = li;
          }
          return 0.0;
        });
        if (verdict < 0.0) return false;
        if (verdict > 0.0) return true;
      }
      if (li > kMinIters - 1 && li < kMaxLinearIters) {
        const int tmp = ls_old;
        ls_old = ls_new;
        ls_new = tmp;
      }
      if (sweeps >= kMaxSweeps) return false;
    }
    return false;
  };
  // ddLinearSolve (src/linalg.cpp:717-900), as dd_linear_solve; the
  // increments in vector 5, the plain right side in vector 4
  auto dd_linear = [&](double tol) -> bool {
    // the increments, the plain right side and the old / new sources in the
    // solve's global scratch (colour order), rarely touched
    auto gv = [&](float* v, int e) -> float& { return v[e * C + j]; };
    auto fission_g = [&](float* v) {
      float o[EC];
      fission(x, o);
      if (has)
#pragma unroll
        for (int e = 0; e < EC; e++) gv(v, e) = o[e];
    };
    auto load_g = [&](float* v, float (&o)[EC]) {
#pragma unroll
      for (int e = 0; e < EC; e++) o[e] = has ? gv(v, e) : 0.0f;
    };
#pragma unroll
    for (int e = 0; e < EC; e++) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < EO; q++)
        if (EC > 1) s += fabsf(aoff[e][q]);
#pragma unroll
      for (int f = 0; f < 4; f++) {
        if constexpr (kNbcShared) s += fabsf(nbs[f * EP + e]);
        else s += fabsf(nbc[f][e]);
      }
      const float d = vrow(kDiagVec)[e];
      const float dd = s > (double) d ? (float) (s - d) : 0.0f;
      vrow(kDiagVec)[e] = d + dd;
      if (has) {
        gv(g.ddv, e) = dd;
        gv(g.rhs, e) = b[e];
      }
    }
    float* old_src = g.dd_a;
    float* new_src = g.dd_b;
    fission_g(new_src);
    if (t == 0) {
      J.dd_initial = 0.0f;
      J.dd_inv_initial = 0.0f;
      J.dd_min_res = 1e6f;
      J.dd_stall_res = INFINITY;
      J.stall_it = 0;
    }
    for (int it = 0; it < kMaxLinearIters; it++) {
      float* tmp = old_src;
      old_src = new_src;
      new_src = tmp;
#pragma unroll
      for (int e = 0; e < EC; e++)
        b[e] = has ? gv(g.rhs, e) + gv(g.ddv, e) * x[e] : 0.0f;
      linear(tol);   // a failure is only noted
      fission_g(new_src);
      float fn[EC], fo[EC];
      load_g(new_src, fn);
      load_g(old_src, fo);
      const double verdict = rmse(fn, fo, [&](float res) {
        if (it == 0) {
          J.dd_initial = res < 1e-14f ? 1e-10f : res;
          J.dd_inv_initial = 1.0f / J.dd_initial;
        }
        J.dd_min_res = fminf(J.dd_min_res, res);
        if ((res > 1e3f * J.dd_min_res && J.dd_min_res > (float) kNoiseFloor) ||
            !isfinite(res))
          return -1.0;
        if (res * J.dd_inv_initial < 0.1f || res < (float) tol) return 1.0;
        if (it - J.stall_it >= kStallWindow) {
          if (res < (float) kStallMax && res > 0.5f * J.dd_stall_res) return 1.0;
          J.dd_stall_res = res;
          J.stall_it = it;
        }
        return 0.0;
      });
      if (verdict < 0.0) return false;
      if (verdict > 0.0) break;
      if (sweeps >= kMaxSweeps) return false;
    }
#pragma unroll
    for (int e = 0; e < EC; e++) {
      const float dd = has ? gv(g.ddv, e) : 0.0f;
      vrow(kDiagVec)[e] = vrow(kDiagVec)[e] - dd;
      b[e] = has ? gv(g.rhs, e) : 0.0f;
    }
    return true;
  };

  CmfdDevState* cm = a.cm;
  const int it = sc->iteration;
  double src_thr = 0.1 * sc->threshold;
  if (it > 0) src_thr = 0.01 * (sc->residual > 0.0 ? sc->residual : 1e-6);
  double keff = cm->keff;
  const double rows = (double) C * EC;
  const double tol = fmax(kLinalgTol, src_thr);
  const double lin_tol = fmax(kLinalgTol, tol * 1e-1);
  // ---- eigenvalueSolve (src/linalg.cpp:25-176), as cmfd_solve_kernel
  fission(x, b);
  const double s0 = total(cell_sum(b), [](double s) { return s; });
  bool failed = !(s0 > 0.0) || !isfinite(s0);
  if (!failed) {
#pragma unroll
    for (int e = 0; e < EC; e++) {
      b[e] = (float) (b[e] * (rows / s0));
      x[e] = (float) (x[e] * (rows * keff / s0));
    }
    if (t == 0) {
      J.initial = 0.0f;
      J.inv_initial = 0.0f;
      J.e_stall_res = INFINITY;
      J.stall_p = 0;
    }
    publish();
    barrier();
    bool dd_mode = false;
    for (power = 0; power < kMaxPowerIters; power++) {
      bool ok = false;
      if (!dd_mode) ok = linear(lin_tol);
      if (!ok) {
        dd_mode = true;
        ok = dd_linear(lin_tol);
      }
      if (!ok) {
        failed = true;
        break;
      }
      float sn[EC];
      fission(x, sn);
      keff = total(cell_sum(sn), [&](double s) { return s / rows; });
      const float kf = (float) keff;
#pragma unroll
      for (int e = 0; e < EC; e++) sn[e] /= kf;
      const double stop = rmse(sn, b, [&](float res) {
        if (power == 0) {
          J.initial = res < 1e-14f ? 1e-10f : res;
          J.inv_initial = 1.0f / J.initial;
        }
        if ((res * J.inv_initial < 0.03f || res < (float) kLinalgTol) && power > kMinIters)
          return 1.0;
        if (power > kMinIters && power - J.stall_p >= kStallWindow) {
          if (res < (float) kStallMax && res > 0.5f * J.e_stall_res) return 1.0;
          J.e_stall_res = res;
          J.stall_p = power;
        }
        return 0.0;
      });
#pragma unroll
      for (int e = 0; e < EC; e++) b[e] = sn[e];
      if (stop > 0.0) {
        power++;
        break;
      }
    }
    if (!(fabs(keff + 1.0) > FLT_EPSILON) || !isfinite(keff)) failed = true;
  }

  if (failed) {
    if (has)
#pragma unroll
      for (int e = 0; e < EC; e++) a.ratio[a.color_cells[j] * EC + e] = 1.0f;
    if (gid == 0) {
      cm->failed = 1;
      cm->power_iters = power;
      cm->linear_iters = sweeps;
      cm->max_ratio = 1.0f;
      cm->valid = 1;
      sc->keff = cm->keff;
    }
    if (NB > 1) cg::this_cluster().sync();   // no block leaves while others may write to it
    return;
  }
  // ---- Cmfd::rescaleFlux and the ratios of Cmfd::updateMOCFlux
  float pt[EC], fa[EC], fb[EC];
#pragma unroll
  for (int e = 0; e < EC; e++) pt[e] = has ? g.phi_t[e * C + j] : 0.0f;
  fission(x, fa);
  fission(pt, fb);
  const auto inverse = [](double s) { return 1.0 / s; };
  const double sn = total(cell_sum(fa), inverse);
  const double so = total(cell_sum(fb), inverse);
  float far = 1.0f;
  if (has) {
#pragma unroll
    for (int e = 0; e < EC; e++) {
      const int out = a.color_cells[j] * EC + e;
      const float xn = (float) (x[e] * sn);
      const float xo = (float) (pt[e] * so);
      const float q = fabs((double) xo) > kFluxEps ? xn / xo : 0.0f;
      a.ratio[out] = q;
      a.flux_new[out] = xn;
      a.flux_old[out] = xo;
      if (q > 0.0f && fabsf(logf(q)) > fabsf(logf(far))) far = q;
    }
  }
  // the ratio farthest from 1 (log distance): warps, then blocks in order
  for (int o = 16; o > 0; o >>= 1) {
    const float y = __shfl_xor_sync(0xffffffffu, far, o);
    if (fabsf(logf(y)) > fabsf(logf(far))) far = y;
  }
  if ((t & 31) == 0) red[t >> 5] = (double) far;
  __syncthreads();
  if (t == 0) {
    float best = 1.0f;
    for (int i = 0; i < (T >> 5); i++) {
      const float y = (float) red[i];
      if (fabsf(logf(y)) > fabsf(logf(best))) best = y;
    }
    if (NB > 1)
      cg::this_cluster().map_shared_rank(&part[0][0], 0)[buf * kCmfdMaxClusterBlocks + rank] = best;
    else
      part[buf][0] = best;
  }
  if (NB > 1) cg::this_cluster().sync();
  if (gid == 0) {
    float best = 1.0f;
    for (int r = 0; r < NB; r++) {
      const float y = (float) part[buf][r];
      if (fabsf(logf(y)) > fabsf(logf(best))) best = y;
    }
    cm->max_ratio = best;
    cm->failed = 0;
    cm->power_iters = power;
    cm->linear_iters = sweeps;
    cm->valid = 1;
    cm->keff = keff;
    sc->keff = keff;
  }
}

// Cmfd::collapseXS over the whole GPU, one thread per (cell, coarse group).
__global__ void __launch_bounds__(256)
cmfd_collapse_kernel(const CmfdArgs a) {
  if (*(volatile const int*) &a.sc->done) return;
  const Work k = carve(a.work, a.C, a.E);
  const int CE = a.C * a.E;
  for (int ce = blockIdx.x * blockDim.x + threadIdx.x; ce < CE;
       ce += gridDim.x * blockDim.x)
    collapse_one(a, k, ce / a.E, ce % a.E);
}

// The surface coefficients and matrices, one thread per row; reads the
// neighbours' collapse, so it follows the collapse kernel.
__global__ void __launch_bounds__(256)
cmfd_build_kernel(const CmfdArgs a) {
  if (*(volatile const int*) &a.sc->done) return;
  const Work k = carve(a.work, a.C, a.E);
  const int it = a.sc->iteration;
  const bool valid = a.cm->valid != 0;
  const int CE = a.C * a.E;
  for (int ce = blockIdx.x * blockDim.x + threadIdx.x; ce < CE;
       ce += gridDim.x * blockDim.x)
    build_row(a, k, ce / a.E, ce % a.E, it, valid);
}

template <int EC>
__global__ void __launch_bounds__(solve_threads(EC), 1)
cmfd_solve_kernel(const CmfdArgs a, int smem_mask) {
  DevScalars* sc = a.sc;
  if (*(volatile int*) &sc->done) return;
  __shared__ double red[33];
  extern __shared__ float4 s_dyn[];
  const int C = a.C, E = a.E;
  const int CE = C * E;
  const Work g = carve(a.work, C, E);   // as the build kernels wrote it
  Work k = g;
  k.nbr = a.nbr_j;
  place_in_smem(k, reinterpret_cast<char*>(s_dyn), smem_mask, a);
  // the placed couplings and the starting iterate onto the chip
  if (k.x != g.x)
    for (int r = threadIdx.x; r < CE; r += blockDim.x) k.x[r] = g.x[r];
  if (k.nb != g.nb)
    for (int r = threadIdx.x; r < 4 * CE; r += blockDim.x) k.nb[r] = g.nb[r];
  __syncthreads();
  CmfdDevState* cm = a.cm;
  const int it = sc->iteration;                 // MOC iteration
  // the coarse tolerance follows the transport residual
  // (Solver::computeEigenvalue, src/Solver.cpp:1671-1675)
  double src_thr = 0.1 * sc->threshold;         // Solver::initializeCmfd
  if (it > 0) src_thr = 0.01 * (sc->residual > 0.0 ? sc->residual : 1e-6);
  double keff = cm->keff;

  // ---- eigenvalueSolve (src/linalg.cpp:25-176)
  const double rows = (double) CE;
  const double tol = fmax(kLinalgTol, src_thr);
  const double lin_tol = fmax(kLinalgTol, tol * 1e-1);
  float* src_old = k.b;          // the SOR's right side, on chip if placed
  float* src_new = k.src_a;
  mat_fission<EC>(a, k, k.x, src_old);
  const double s0 = block_total(src_old, CE, red);
  bool failed = !(s0 > 0.0) || !isfinite(s0);
  int sweeps = 0, power = 0;
  if (!failed) {
    for (int r = threadIdx.x; r < CE; r += blockDim.x) {
      src_old[r] = (float) (src_old[r] * (rows / s0));
      k.x[r] = (float) (k.x[r] * (rows * keff / s0));
    }
    __syncthreads();
    double initial = 0.0, inv_initial = 0.0, stall_res = INFINITY;
    int stall_p = 0;
    bool dd_mode = false;
    for (power = 0; power < kMaxPowerIters; power++) {
      // eigenvalueSolve's linear solves: plain, or diagonally dominated
      // from the first failure on
      bool ok = false;
      if (!dd_mode) ok = linear_solve<EC>(a, k, src_old, lin_tol, red, sweeps);
      if (!ok) {
        dd_mode = true;
        ok = dd_linear_solve<EC>(a, k, src_old, lin_tol, red, sweeps);
      }
      if (!ok) {
        failed = true;
        break;
      }
      mat_fission<EC>(a, k, k.x, src_new);
      __syncthreads();
      keff = block_total(src_new, CE, red, [&](double s) { return s / rows; });
      const float kf = (float) keff;
      for (int r = threadIdx.x; r < CE; r += blockDim.x) src_new[r] /= kf;
      __syncthreads();
      // thread 0 judges: 1 converged, 0 not yet
      const double stop = rmse(a, src_new, src_old, red, [&](double res) {
        if (power == 0) {
          initial = res < 1e-14 ? 1e-10 : res;
          inv_initial = 1.0 / initial;
        }
        if ((res * inv_initial < 0.03 || res < kLinalgTol) && power > kMinIters)
          return 1.0;
        if (power > kMinIters && power - stall_p >= kStallWindow) {
          if (res < kStallMax && res > 0.5 * stall_res) return 1.0;
          stall_res = res;
          stall_p = power;
        }
        return 0.0;
      });
      for (int r = threadIdx.x; r < CE; r += blockDim.x) src_old[r] = src_new[r];
      __syncthreads();
      if (stop > 0.0) {
        power++;
        break;
      }
    }
    if (!(fabs(keff + 1.0) > FLT_EPSILON) || !isfinite(keff)) failed = true;
  }
  __syncthreads();

  // ---- Cmfd::rescaleFlux and the ratios of Cmfd::updateMOCFlux
  // (src/Cmfd.cpp:1304-1350, 1509-1560, 3222-3300)
  if (failed) {
    for (int r = threadIdx.x; r < CE; r += blockDim.x) a.ratio[r] = 1.0f;
    if (threadIdx.x == 0) {
      cm->failed = 1;
      cm->power_iters = power;
      cm->linear_iters = sweeps;
      cm->max_ratio = 1.0f;
      cm->valid = 1;
      sc->keff = cm->keff;          // the previous coarse eigenvalue stands
    }
    return;
  }
  mat_fission<EC>(a, k, k.x, k.src_a);
  mat_fission<EC>(a, k, k.phi_t, k.src_b);
  __syncthreads();
  // the reciprocals of the two source totals, formed once by thread 0
  const auto inverse = [](double s) { return 1.0 / s; };
  const double sn = block_total(k.src_a, CE, red, inverse);
  const double so = block_total(k.src_b, CE, red, inverse);
  float far = 1.0f;
  for (int r = threadIdx.x; r < CE; r += blockDim.x) {   // r = e * C + j
    const int e = r / C, j = r - e * C;
    const int out = a.color_cells[j] * E + e;            // cell order
    const float xn = (float) (k.x[r] * sn);
    const float xo = (float) (k.phi_t[r] * so);
    // bounded by the prolongation, after any k-nearest weighting
    const float q = fabs((double) xo) > kFluxEps ? xn / xo : 0.0f;
    a.ratio[out] = q;
    a.flux_new[out] = xn;
    a.flux_old[out] = xo;
    if (q > 0.0f && fabsf(logf(q)) > fabsf(logf(far))) far = q;
  }
  // the ratio farthest from 1 (log distance) over the block
  for (int o = 16; o > 0; o >>= 1) {
    const float y = __shfl_xor_sync(0xffffffffu, far, o);
    if (fabsf(logf(y)) > fabsf(logf(far))) far = y;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double) far;
  __syncthreads();
  if (threadIdx.x == 0) {
    float best = 1.0f;
    for (int i = 0; i < (int) (blockDim.x >> 5); i++) {
      const float y = (float) red[i];
      if (fabsf(logf(y)) > fabsf(logf(best))) best = y;
    }
    cm->max_ratio = best;
    cm->failed = 0;
    cm->power_iters = power;
    cm->linear_iters = sweeps;
    cm->valid = 1;
    cm->keff = keff;
    sc->keff = keff;
  }
}

template <int EC>
void solve_instance(const CmfdArgs& a, int threads, int smem, int level,
                    cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(cmfd_solve_kernel<EC>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kSolveSmemMax);
    configured = true;
  }
  cmfd_solve_kernel<EC><<<1, threads, smem, s>>>(a, level);
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

int64_t cmfd_work_floats(int C, int E) {
  const int64_t CE = (int64_t) C * E;
  return 7 * CE + 3 * CE * E + 8 * CE + kColourVecs * CE;
}

void launch_cmfd_pair_sums(const float* phi, const float* vol,
                           const int32_t* pair_off, const int32_t* pair_fsr,
                           int P, int G, int ld, double* out, DevScalars* sc,
                           cudaStream_t s) {
  if (P <= 0) return;
  const int per_block = kPairThreads / 32;
  const int blocks = (int) std::min<int64_t>((P + per_block - 1) / per_block,
                                             (int64_t) 8 * sm_count());
  cmfd_pair_sums_kernel<<<blocks, kPairThreads, 0, s>>>(phi, vol, pair_off,
                                                        pair_fsr, P, G, ld, out,
                                                        sc);
}

int64_t cmfd_cells_smem(int E, int threads, int slots) {
  return 4 * ((int64_t) slots * cells_xs_stride(E) +
              (int64_t) threads * cells_row_stride(E));
}

namespace {

template <int EC>
bool cells_instance(const CmfdArgs& a, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(cmfd_cells_kernel<EC>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kSolveSmemMax);
    configured = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned) a.map_nb);
  cfg.blockDim = dim3((unsigned) a.map_threads);
  cfg.dynamicSmemBytes = (size_t) cmfd_cells_smem(EC, a.map_threads, a.map_slots);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned) a.map_nb;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, cmfd_cells_kernel<EC>, a) == cudaSuccess)
    return true;
  cudaGetLastError();   // a launch-configuration error is not sticky
  return false;
}

bool launch_cells(const CmfdArgs& a, cudaStream_t s) {
  switch (a.E) {
    case 1: return cells_instance<1>(a, s);
    case 2: return cells_instance<2>(a, s);
    case 3: return cells_instance<3>(a, s);
    case 4: return cells_instance<4>(a, s);
    case 5: return cells_instance<5>(a, s);
    case 6: return cells_instance<6>(a, s);
    case 7: return cells_instance<7>(a, s);
    case 8: return cells_instance<8>(a, s);
    default: return false;
  }
}

}  // namespace

bool launch_cmfd_solve(const CmfdArgs& a, cudaStream_t s) {
  // collapse and matrices over the GPU, then the solve: cell-parallel when
  // the cells are mapped onto a cluster, else on one block (one thread per
  // cell of a colour, at least four warps)
  const int CE = a.C * a.E;
  const int nb = (int) std::min<int64_t>((CE + 255) / 256, (int64_t) 4 * sm_count());
  cmfd_collapse_kernel<<<std::max(nb, 1), 256, 0, s>>>(a);
  cmfd_build_kernel<<<std::max(nb, 1), 256, 0, s>>>(a);
  if (a.map_nb > 0 && a.solve_kind == 0 && launch_cells(a, s)) return true;
  int threads = (std::max(a.n_color0, a.C - a.n_color0) + 31) / 32 * 32;
  threads = std::max(128, std::min(solve_threads(a.E <= 8 ? a.E : 0), threads));
  int64_t bytes = 0;
  const int level = smem_plan(a.C, a.E, kSolveSmemMax, &bytes);   // item mask
  const int smem = (int) bytes;
  switch (a.E) {
    case 1: solve_instance<1>(a, threads, smem, level, s); break;
    case 2: solve_instance<2>(a, threads, smem, level, s); break;
    case 3: solve_instance<3>(a, threads, smem, level, s); break;
    case 4: solve_instance<4>(a, threads, smem, level, s); break;
    case 5: solve_instance<5>(a, threads, smem, level, s); break;
    case 6: solve_instance<6>(a, threads, smem, level, s); break;
    case 7: solve_instance<7>(a, threads, smem, level, s); break;
    case 8: solve_instance<8>(a, threads, smem, level, s); break;
    default: solve_instance<0>(a, threads, smem, level, s); break;
  }
  return !(a.map_nb > 0 && a.solve_kind == 0);
}

void launch_cmfd_prolong(float* phi, float* mom, const int32_t* fsr_cell,
                         const int32_t* group_of, const float* ratio,
                         const CmfdStencil& st, int64_t R, int G, int ld,
                         int E, int unbounded, DevScalars* sc,
                         cudaStream_t s) {
  const int64_t n = R * ld;
  int blocks = (int) std::min<int64_t>((n + 255) / 256, (int64_t) 8 * sm_count());
  if (blocks < 1) blocks = 1;
  cmfd_prolong_kernel<<<blocks, 256, 0, s>>>(
      phi, reinterpret_cast<float2*>(mom), fsr_cell, group_of, ratio, st, R, G,
      ld, E, unbounded, sc);
}

}  // namespace moc
