// FSR sources as a per-material batched contraction on the sm_103a tensor
// cores (tcgen05), in 3xTF32 split precision.
//
// Restates CPUSolver::computeFSRSources (src/CPUSolver.cpp:1939-2025) and the
// reference GPU's computeFSRSourcesOnDevice (src/accel/cuda/GPUSolver.cu:
// 300-345): Q[r, d] = (sum_o S_m[d, o] phi[r, o] + chi_m[d] (nu_sigma_f_m .
// phi[r]) / k + fixed[r, d]) / (4 pi), stored divided by sigma_t.  The
// scattering part is, for the FSRs of one material m, the product of their
// flux rows (R_m x G) with S_m^T (G x G): one GEMM per material.
//
// One CTA computes a tile of kTcRows = 128 FSRs of one material:
//   - the material's operand B (S_m split into TF32 high and low parts,
//     pre-laid-out on the host in the MMA's K-major core-matrix order) is
//     brought into shared memory by one bulk asynchronous copy (TMA engine,
//     cp.async.bulk) completing on an mbarrier;
//   - the 128 flux rows are gathered by FSR id (one warp per row, lanes over
//     groups), split into TF32 high and low parts and written in the same
//     layout; the fission rate of each row is summed on the way and, in the
//     eigenvalue loop, the row is zeroed for the sweep's tallies;
//   - one thread issues, per K step of 8 groups, the three products
//     A_hi B_hi + A_hi B_lo + A_lo B_hi (tcgen05.mma kind::tf32, M = 128,
//     N = G rounded up to 16) into an FP32 accumulator in tensor memory, and
//     commits them to a second mbarrier;
//   - each warp reads its 32 accumulator lanes (one FSR per thread) with
//     tcgen05.ld and finishes the source: fission term, fixed source,
//     1 / 4 pi, the negative-source clamp, division by sigma_t.
// Dropping A_lo B_lo leaves a relative error of about 2^-22 per product, so
// the contraction carries FP32 accuracy.  Every mbarrier wait is bounded; a
// wait that runs out records DevScalars::tc_error, waits (bounded) for the
// work still in flight and frees the tensor memory before returning.
#include <cstring>
#include <vector>

#include "moc_internal.cuh"

namespace moc {

namespace {

constexpr int kTcThreads = 128;
static_assert(kTcThreads == kTcRows, "one thread per tile row");
constexpr int kTcColumns = 128;         // tensor-memory columns allocated
constexpr float kTcFluxEpsilon = 1.0e-25f;
constexpr double kTcOneOverFourPi = 0.07957747154594767;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Shared-memory matrix descriptor of a K-major operand without swizzling:
// 8-row x 16-byte core matrices; lbo = byte step between core matrices along
// K, sbo = byte step between 8-row groups; bits 46-47 hold the descriptor
// version 1.
__device__ __forceinline__ uint64_t kmajor_desc(uint32_t addr, uint32_t lbo,
                                                uint32_t sbo) {
  return (uint64_t) ((addr & 0x3FFFFu) >> 4) |
         ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator,
// A and B TF32, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t tf32_idesc(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t) (n >> 3) << 17) |
         ((uint32_t) (128 >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          unsigned limit) {
  for (unsigned i = 0; i < limit; i++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a,
                                         uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
        "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) in a K-major operand of kc = K/4 chunks:
// core matrix (row / 8, k / 4) at ((row / 8) * kc + k / 4) * 128, rows of a
// core matrix 16 bytes apart.
__host__ __device__ __forceinline__ int core_offset(int row, int k, int kc) {
  return ((row >> 3) * kc + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

template <int N>
__global__ void __launch_bounds__(kTcThreads, 1)
sources_tc_kernel(const SolverArgs a, int iteration, int zero_phi) {
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ float s_fr[kTcRows];
  __shared__ int s_row[kTcRows];
  __shared__ int s_ok;

  const int K = a.tc_k, kc = K >> 2;
  const int a_bytes = kTcRows * K * 4;   // one of the high / low parts
  const int b_bytes = N * K * 4;
  uint8_t* sa_hi = smem;
  uint8_t* sa_lo = smem + a_bytes;
  uint8_t* sb = smem + 2 * a_bytes;      // B high then B low
  const int G = a.num_groups;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x;
  const int m = a.tc_tile_mat[tile];
  const uint32_t bar_b = smem_addr(&bars[0]), bar_mma = smem_addr(&bars[1]);

  // the tile's FSR ids, one per thread (kTcThreads == kTcRows)
  s_row[threadIdx.x] = a.tc_rows[(size_t) tile * kTcRows + threadIdx.x];
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_b));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_mma));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    s_ok = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the material's B operand: one bulk copy of 2 * b_bytes
    const float* src = a.tc_b + (size_t) m * 2 * N * K;
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_b),
        "r"(2 * b_bytes)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_addr(sb)),
        "l"(src), "r"(2 * b_bytes), "r"(bar_b)
        : "memory");
  }
  if (warp == 0) {
    __syncwarp();   // the .sync.aligned forms need the whole warp converged
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
            "r"(smem_addr(&tmem_slot)),
        "r"(kTcColumns)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
  }

  // operand A: the tile's flux rows, TF32 high and low parts.  A warp takes
  // rows warp, warp + 4, ...; kRowBatch rows at a time with every load of
  // the batch issued before the first is used (K <= 96: three per lane);
  // the row ids were read into shared memory before the barrier above.
  const float* nf = a.nu_sigma_f + (size_t) m * G;
  float nfl[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int k = lane + 32 * j;
    nfl[j] = (k < G) ? nf[k] : 0.0f;
  }
  constexpr int kRowBatch = 16;
  for (int i0 = warp; i0 < kTcRows; i0 += 4 * kRowBatch) {
    float v[kRowBatch][3];
    int rows[kRowBatch];
#pragma unroll
    for (int u = 0; u < kRowBatch; u++) {
      const int i = i0 + 4 * u;
      rows[u] = s_row[i];
      const float* phi = a.phi + (size_t) (rows[u] >= 0 ? rows[u] : 0) * a.ld;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int k = lane + 32 * j;
        v[u][j] = (rows[u] >= 0 && k < G) ? phi[k] : 0.0f;
      }
    }
#pragma unroll
    for (int u = 0; u < kRowBatch; u++) {
      const int i = i0 + 4 * u;
      float fr = 0.0f;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int k = lane + 32 * j;
        if (k >= K) continue;
        fr = fmaf(nfl[j], v[u][j], fr);
        const float hi = tf32_round(v[u][j]);
        const float lo = tf32_round(v[u][j] - hi);
        const int off = core_offset(i, k, kc);
        *reinterpret_cast<float*>(sa_hi + off) = hi;
        *reinterpret_cast<float*>(sa_lo + off) = lo;
      }
      // fused: the sweep that follows starts from zero tallies
      if (rows[u] >= 0 && zero_phi) {
        float* phi = a.phi + (size_t) rows[u] * a.ld;
#pragma unroll
        for (int j = 0; j < 3; j++)
          if (lane + 32 * j < G) phi[lane + 32 * j] = 0.0f;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) fr += __shfl_xor_sync(0xffffffffu, fr, o);
      if (lane == 0) s_fr[i] = fr;
    }
  }
  // the generic-proxy stores above become visible to the tensor core
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // one thread issues the products and waits for them; the others learn
  // the outcome at the barrier
  if (threadIdx.x == 0) {
    if (mbar_wait(bar_b, 0, a.tc_wait_limit)) {
      const uint32_t idesc = tf32_idesc(N);
      const uint32_t a_hi = smem_addr(sa_hi), a_lo = smem_addr(sa_lo);
      const uint32_t b_hi = smem_addr(sb), b_lo = b_hi + b_bytes;
      const uint32_t sbo = (uint32_t) kc * 128;
      for (int s = 0; s < K / 8; s++) {
        const uint32_t step = (uint32_t) s * 256;   // two core matrices
        const uint64_t dah = kmajor_desc(a_hi + step, 128, sbo);
        const uint64_t dal = kmajor_desc(a_lo + step, 128, sbo);
        const uint64_t dbh = kmajor_desc(b_hi + step, 128, sbo);
        const uint64_t dbl = kmajor_desc(b_lo + step, 128, sbo);
        mma_tf32(tmem, dah, dbh, idesc, s > 0 ? 1u : 0u);
        mma_tf32(tmem, dah, dbl, idesc, 1u);
        mma_tf32(tmem, dal, dbh, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster."
          "b64 [%0];" ::"r"(bar_mma)
          : "memory");
      if (!mbar_wait(bar_mma, 0, a.tc_wait_limit)) {
        // record it, and give the products a second wait, bounded by the
        // full default limit, before the tensor memory is freed
        sc->tc_error = 1;
        s_ok = 0;
        mbar_wait(bar_mma, 0, kTcDefaultWaitLimit);
      }
    } else {
      // the bulk copy did not complete in time: record it, and give it a
      // second wait, bounded by the full default limit, before the shared
      // memory goes away
      sc->tc_error = 1;
      s_ok = 0;
      mbar_wait(bar_b, 0, kTcDefaultWaitLimit);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue, in two passes: thread t copies accumulator lane t (tile row
  // t) into shared memory over the A operands, which the finished products
  // no longer need (row stride N + 1 keeps the writes conflict-free); then
  // each warp finishes whole rows with lanes over groups, so the source rows
  // leave as coalesced stores.
  float* s_acc = reinterpret_cast<float*>(smem);
  if (s_ok) {
    const uint32_t lane_base = tmem + ((uint32_t) (warp * 32) << 16);
#pragma unroll
    for (int c = 0; c < N / 16; c++) {
      float acc[16];
      __syncwarp();   // the loads are warp-collective
      tmem_load16(lane_base + c * 16, acc);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; j++)
        s_acc[threadIdx.x * (N + 1) + 16 * c + j] = acc[j];
    }
  }
  __syncthreads();
  if (s_ok) {
    const float inv_k = (float) (1.0 / sc->keff);
    if (iteration < 0) iteration = sc->iteration;
    float chil[3], stl[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int d = lane + 32 * j;
      chil[j] = (d < G) ? a.chi[(size_t) m * G + d] : 0.0f;
      stl[j] = (d < G) ? a.sigma_t[(size_t) m * G + d] : 1.0f;
    }
    unsigned negatives = 0;
    for (int i = warp; i < kTcRows; i += kTcThreads / 32) {
      const int r = s_row[i];
      if (r < 0) continue;
      const float fk = s_fr[i] * inv_k;
      const float* fixed = a.fixed ? a.fixed + (size_t) r * a.ld : nullptr;
      float* qt = a.qt + (size_t) r * a.ld;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const int d = lane + 32 * j;
        if (d >= G) continue;
        float q = chil[j] * fk;
        q += s_acc[i * (N + 1) + d];
        if (fixed) q += fixed[d];
        q *= (float) kTcOneOverFourPi;
        if (q < 0.0f) {
          negatives++;
          if (iteration < 30) q = kTcFluxEpsilon;
        }
        qt[d] = q / stl[j];
      }
    }
    if (negatives) atomicAdd(&sc->neg_sources, (unsigned long long) negatives);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile(
        "tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
        "r"(kTcColumns)
        : "memory");
  }
}

// host-side round to TF32 (nearest, ties away from zero): the 13 low
// mantissa bits dropped
float tf32_round_host(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u = (u + 0x1000u) & ~0x1FFFu;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

}  // namespace

bool tc_sources_supported(int num_groups) {
  return num_groups >= 64 && num_groups <= 96;
}

int tc_pad_n(int G) { return (G + 15) / 16 * 16; }
int tc_pad_k(int G) { return (G + 7) / 8 * 8; }

void tc_pack_scattering(const float* sigma_s, int M, int G,
                        std::vector<float>& out) {
  const int N = tc_pad_n(G), K = tc_pad_k(G), kc = K / 4;
  out.assign((size_t) M * 2 * N * K, 0.0f);
  for (int m = 0; m < M; m++) {
    float* hi = out.data() + (size_t) m * 2 * N * K;
    float* lo = hi + (size_t) N * K;
    for (int d = 0; d < G; d++)
      for (int o = 0; o < G; o++) {
        const float v = sigma_s[((size_t) m * G + d) * G + o];
        const float h = tf32_round_host(v);
        const int off = core_offset(d, o, kc) / 4;
        hi[off] = h;
        lo[off] = tf32_round_host(v - h);
      }
  }
}

void launch_sources_tc(const SolverArgs& a, int iteration, int zero_phi,
                       cudaStream_t s) {
  const int K = a.tc_k;
  const size_t smem = (size_t) 2 * kTcRows * K * 4 + (size_t) 2 * a.tc_n * K * 4;
  switch (a.tc_n) {
    case 64:
      cudaFuncSetAttribute(sources_tc_kernel<64>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
      sources_tc_kernel<64><<<a.tc_tiles, kTcThreads, smem, s>>>(a, iteration, zero_phi);
      break;
    case 80:
      cudaFuncSetAttribute(sources_tc_kernel<80>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
      sources_tc_kernel<80><<<a.tc_tiles, kTcThreads, smem, s>>>(a, iteration, zero_phi);
      break;
    default:
      cudaFuncSetAttribute(sources_tc_kernel<96>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
      sources_tc_kernel<96><<<a.tc_tiles, kTcThreads, smem, s>>>(a, iteration, zero_phi);
      break;
  }
}

}  // namespace moc
