// Transport sweep kernels for sm_103a.
//
// Replaces the reference's transportSweepOnDevice / tallyScalarFlux /
// transferBoundaryFlux (src/accel/cuda/GPUSolver.cu:480-660) and restates
// the flat-source attenuation of CPUSolver::tallyScalarFlux
// (src/CPUSolver.cpp:2402-2498) and TransportSweep::onTrack
// (src/TrackTraversingAlgorithms.cpp:890-1052).
//
// Work decomposition: a "stream" is one direction of one track.  A warp
// carries 32/lps streams; the lps lanes of a stream split the energy groups
// (lane sub handles groups sub, sub+lps, ...), and each lane keeps the
// angular flux of its groups for all polar angles in registers along the
// whole track.  The forward and backward streams of a track sit next to each
// other, so they share segment cache lines.  Streams are ordered by
// decreasing segment count (sc order[]) so that warps of one block do
// similar amounts of work and the longest tracks start first.
//
// Per segment and group the lane sums the polar contributions in registers
// and issues one fire-and-forget float reduction to the FSR tally; the lps
// lanes of a stream write lps consecutive floats of one FSR row, so a warp
// instruction touches 32/lps rows.
//
// Attenuation: delta = (psi - Q/sigma_t) * g(x), g(x) = 1 - exp(-x),
// x = sigma_t * l / sin(theta), which is algebraically the reference's
// (tau*psi - l*Q) * F1(x)/sin(theta) (src/CPUSolver.cpp:2463-2484).
#include "moc_internal.cuh"

namespace moc {

// g(x) = 1 - exp(-x) from a shared-memory table of g at x_i = i*h, h = 1/16,
// expanded around the node: g(x_i + d) = g_i + (1 - g_i) * (1 - exp(-d)),
// 1 - exp(-d) by its Taylor series to d^4 (next term d^5/120 < 8e-9).
// The caller passes u = x / h.  Relative accuracy is kept for small x
// because the i = 0 node has g_0 = 0 exactly.
struct AttenTable {
  static constexpr float c1 = kExpTableH;
  static constexpr float c2 = -kExpTableH * kExpTableH / 2.0f;
  static constexpr float c3 = kExpTableH * kExpTableH * kExpTableH / 6.0f;
  static constexpr float c4 =
      -kExpTableH * kExpTableH * kExpTableH * kExpTableH / 24.0f;
  __device__ __forceinline__ static float eval(float u, const float* tab) {
    u = fminf(u, (float) (kExpTableSize - 1));
    // u + 2^23 rounded down carries floor(u) in its low mantissa bits
    const float t = __fadd_rd(u, 8388608.0f);
    const int i = __float_as_int(t) - 0x4B000000;
    const float du = u - (t - 8388608.0f);
    const float q = du * fmaf(du, fmaf(du, fmaf(du, c4, c3), c2), c1);
    const float gi = tab[i];
    return fmaf(1.0f - gi, q, gi);
  }
};

// g(x) = 1 - exp(-x) from the hardware base-2 exponential, with the
// series x - x^2/2 + x^3/6 - x^4/24 + x^5/120 below x = 1/4 where the
// subtraction would lose relative accuracy.
struct AttenIntrinsic {
  __device__ __forceinline__ static float ex2(float v) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
  }
  __device__ __forceinline__ static float eval(float x) {
    const float e = ex2(x * -1.4426950408889634f);
    const float big = 1.0f - e;
    const float small =
        x * fmaf(x, fmaf(x, fmaf(x, fmaf(x, 1.0f / 120.0f, -1.0f / 24.0f),
                                 1.0f / 6.0f), -0.5f), 1.0f);
    return x < 0.25f ? small : big;
  }
};

template <int PH, int SLOTS, int EXPK>
__global__ void __launch_bounds__(kSweepThreads, kSweepMinBlocks)
sweep_kernel(const SweepArgs a) {
  extern __shared__ float smem[];
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;

  const int G = a.num_groups;
  const int MG = a.num_materials * G;
  float* s_st = smem;
  float* s_tab = smem + MG;
  for (int i = threadIdx.x; i < MG; i += blockDim.x) s_st[i] = a.sigma_t[i];
  if (EXPK == kExpTable)
    for (int i = threadIdx.x; i < kExpTableSize; i += blockDim.x)
      s_tab[i] = a.exp_table[i];
  __syncthreads();

  const int cur = sc->cur;
  const float* psi_in = a.psi[cur];
  float* psi_out = a.psi[cur ^ 1];
  const float scale = sc->scale[cur];

  const int lane = threadIdx.x & 31;
  const int lps = a.lps;
  const int sub = lane & (lps - 1);
  const int64_t gwarp =
      ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t stream = gwarp * (32 / lps) + lane / lps;

  if (stream < 2 * a.num_tracks) {
    const int t = a.order[stream >> 1];
    const int dir = (int) (stream & 1);
    const int64_t b = a.seg_off[t];
    const int n = (int) (a.seg_off[t + 1] - b);
    const int ang = a.track_ang[t];
    const int F = G * PH;

    float w[PH], xs[PH];
#pragma unroll
    for (int p = 0; p < PH; p++) {
      w[p] = a.weights[ang * PH + p];
      const float is = a.inv_sin[ang * PH + p];
      xs[p] = (EXPK == kExpTable) ? is * kExpTableInvH : is;
    }

    float psi[SLOTS][PH];
    const float* pin = psi_in + ((int64_t) t * 2 + dir) * F;
#pragma unroll
    for (int j = 0; j < SLOTS; j++) {
      const int g = sub + j * lps;
#pragma unroll
      for (int p = 0; p < PH; p++)
        psi[j][p] = (g < G) ? pin[p * G + g] * scale : 0.0f;
    }

    // Segment stream, software-pipelined.  The lps lanes of a stream load
    // lps consecutive segments with one coalesced access (a "chunk", one
    // segment per lane) a whole chunk ahead of use; segment k reaches every
    // lane of the stream by a shuffle from lane k % lps.  The sources of
    // segment k+1 are gathered while segment k is integrated.
    const int2* seg = a.segs + b;
    const unsigned gmask =
        (lps == 32) ? 0xffffffffu
                    : (((1u << lps) - 1u) << (lane & ~(lps - 1)));
    auto fetch = [&](int kk) -> int2 {
      return (kk < n) ? __ldg(seg + (dir ? n - 1 - kk : kk))
                      : make_int2(0, 0);
    };
    auto unpack = [&](int2 sg, float& len, int& fsr, int& mat) {
      len = __int_as_float(sg.x);
      if (a.mat_packed) {
        fsr = sg.y & 0xFFFFFF;
        mat = (int) ((unsigned) sg.y >> 24);
      } else {
        fsr = sg.y;
        mat = __ldg(a.fsr_mat + fsr);
      }
    };
    int2 chunk = fetch(sub);
    int2 chunk_next = fetch(lps + sub);
    int2 sg;
    sg.x = __shfl_sync(gmask, chunk.x, 0, lps);
    sg.y = __shfl_sync(gmask, chunk.y, 0, lps);
    float len;
    int fsr, mat;
    unpack(sg, len, fsr, mat);
    float q[SLOTS];
#pragma unroll
    for (int j = 0; j < SLOTS; j++) {
      const int g = sub + j * lps;
      q[j] = (g < G && n > 0) ? __ldg(a.qt + (int64_t) fsr * G + g) : 0.0f;
    }
    for (int k = 0; k < n; k++) {
      // next segment: rotate chunks at chunk boundaries
      const int kn = k + 1;
      const int src = kn & (lps - 1);
      if (src == 0) {
        chunk = chunk_next;
        chunk_next = fetch(kn + lps + sub);
      }
      int2 sgn;
      sgn.x = __shfl_sync(gmask, chunk.x, src, lps);
      sgn.y = __shfl_sync(gmask, chunk.y, src, lps);
      float len_n;
      int fsr_n, mat_n;
      unpack(sgn, len_n, fsr_n, mat_n);
      float qn[SLOTS];
#pragma unroll
      for (int j = 0; j < SLOTS; j++) {
        const int g = sub + j * lps;
        qn[j] = (g < G && kn < n) ? __ldg(a.qt + (int64_t) fsr_n * G + g)
                                  : 0.0f;
      }

      const float* st = s_st + mat * G;
      float* ph = a.phi + (int64_t) fsr * G;
#pragma unroll
      for (int j = 0; j < SLOTS; j++) {
        const int g = sub + j * lps;
        if (g < G) {
          const float tau = st[g] * len;
          const float qv = q[j];
          float tally = 0.0f;
#pragma unroll
          for (int p = 0; p < PH; p++) {
            const float gx = (EXPK == kExpTable)
                                 ? AttenTable::eval(tau * xs[p], s_tab)
                                 : AttenIntrinsic::eval(tau * xs[p]);
            const float d = (psi[j][p] - qv) * gx;
            psi[j][p] -= d;
            tally = fmaf(w[p], d, tally);
          }
          atomicAdd(ph + g, tally);
        }
      }
      len = len_n;
      fsr = fsr_n;
      mat = mat_n;
#pragma unroll
      for (int j = 0; j < SLOTS; j++) q[j] = qn[j];
    }

    // boundary-flux transfer to the connecting track, fused into the sweep
    // (CPUSolver::transferBoundaryFlux, src/CPUSolver.cpp:2560-2600)
    const int f = a.flags[t];
    if (f & (dir ? 8 : 4)) {
      const int nt = a.next[2 * t + dir];
      const int nd = (f & (dir ? 2 : 1)) ? 0 : 1;
      float* po = psi_out + ((int64_t) nt * 2 + nd) * F;
#pragma unroll
      for (int j = 0; j < SLOTS; j++) {
        const int g = sub + j * lps;
        if (g < G) {
#pragma unroll
          for (int p = 0; p < PH; p++) po[p * G + g] = psi[j][p];
        }
      }
    }
  }

  // The last block to finish flips the buffer index: every block has read
  // sc->cur by then.  The buffer just written starts with scale 1.
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int ticket = atomicAdd(&sc->ticket_sweep, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    sc->ticket_sweep = 0;
    sc->scale[cur ^ 1] = 1.0f;
    sc->cur = cur ^ 1;
    __threadfence();
  }
}

template <int PH, int SLOTS, int EXPK>
static void launch_one(const SweepArgs& a, cudaStream_t stream) {
  const int spw = 32 / a.lps;
  const int64_t warps = (2 * a.num_tracks + spw - 1) / spw;
  const int wpb = kSweepThreads / 32;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  size_t smem = sizeof(float) * ((size_t) a.num_materials * a.num_groups +
                                 (EXPK == kExpTable ? kExpTableSize : 0));
  auto kern = sweep_kernel<PH, SLOTS, EXPK>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int) smem);
  kern<<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a);
}

template <int PH, int EXPK>
static bool dispatch_slots(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (slots) {
    case 1: launch_one<PH, 1, EXPK>(a, s); return true;
    case 2: launch_one<PH, 2, EXPK>(a, s); return true;
    case 3: launch_one<PH, 3, EXPK>(a, s); return true;
    case 4: launch_one<PH, 4, EXPK>(a, s); return true;
    case 5: launch_one<PH, 5, EXPK>(a, s); return true;
    case 6: launch_one<PH, 6, EXPK>(a, s); return true;
    case 7: launch_one<PH, 7, EXPK>(a, s); return true;
    case 8: launch_one<PH, 8, EXPK>(a, s); return true;
    case 9: launch_one<PH, 9, EXPK>(a, s); return true;
    default: return false;
  }
}

template <int EXPK>
static bool dispatch_ph(const SweepArgs& a, int ph, int slots,
                        cudaStream_t s) {
  switch (ph) {
    case 1: return dispatch_slots<1, EXPK>(a, slots, s);
    case 2: return dispatch_slots<2, EXPK>(a, slots, s);
    case 3: return dispatch_slots<3, EXPK>(a, slots, s);
    default: return false;
  }
}

__global__ void pack_materials_kernel(int2* segs, int64_t n,
                                      const int32_t* fsr_mat) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int fsr = segs[i].y & 0xFFFFFF;
    segs[i].y = fsr | (fsr_mat[fsr] << 24);
  }
}

void launch_pack_materials(int2* segs, int64_t num_segments,
                           const int32_t* fsr_mat, cudaStream_t stream) {
  if (num_segments == 0) return;
  int64_t blocks = (num_segments + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  pack_materials_kernel<<<(unsigned) blocks, 256, 0, stream>>>(
      segs, num_segments, fsr_mat);
}

int sweep_max_slots(int polar_half) {
  return (polar_half >= 1 && polar_half <= 3) ? kMaxSlots : 0;
}

bool launch_sweep(const SweepArgs& a, int polar_half, int slots, int exp_kind,
                  cudaStream_t stream) {
  if (exp_kind == kExpIntrinsic)
    return dispatch_ph<kExpIntrinsic>(a, polar_half, slots, stream);
  return dispatch_ph<kExpTable>(a, polar_half, slots, stream);
}

}  // namespace moc
