// The transport sweep kernel template for sm_103a, included by the
// sweep_p<Ph>_e<exp>.cu translation units (one per polar count and
// exponential evaluator, compiled in parallel).
//
// Replaces the reference's transportSweepOnDevice / tallyScalarFlux /
// transferBoundaryFlux (src/accel/cuda/GPUSolver.cu:480-660) and restates
// the flat-source attenuation of CPUSolver::tallyScalarFlux
// (src/CPUSolver.cpp:2402-2498) and TransportSweep::onTrack
// (src/TrackTraversingAlgorithms.cpp:890-1052).
//
// Work decomposition: a "stream" is one direction of one track.  A warp
// carries 32/LPS streams; the LPS lanes of a stream split the energy groups
// (lane `sub` handles groups sub, sub+LPS, ..., SLOTS of them), and each
// lane keeps the angular flux of its groups for all polar angles in
// registers along the whole track.  The forward and backward streams of a
// track are adjacent (they share segment cache lines).  Streams are ordered
// by decreasing segment count so that the longest tracks start first.
//
// Per segment and group the lane sums the polar contributions in registers
// and issues one fire-and-forget float reduction into the FSR tally; the
// LPS lanes of a stream write LPS consecutive floats of one FSR row.
//
// Attenuation: delta = (psi - Q/sigma_t) * g(x), g(x) = 1 - exp(-x),
// x = sigma_t * l / sin(theta): algebraically the reference's
// (tau*psi - l*Q) * F1(x)/sin(theta) (src/CPUSolver.cpp:2463-2484).
#pragma once

#include "moc_internal.cuh"

namespace moc {

// g(x) = 1 - exp(-x) from a shared-memory table of (g_i, 1 - g_i) at
// x_i = i*h, h = 1/16, expanded around the node:
//   g(x_i + d) = g_i + (1 - g_i) * (1 - exp(-d)),
// with 1 - exp(-d) by its Taylor series to d^4 (next term d^5/120 < 8e-9).
// The caller passes u = x / h.  Relative accuracy holds for small x because
// the i = 0 node has g_0 = 0 exactly.
struct AttenTable {
  static constexpr float c1 = kExpTableH;
  static constexpr float c2 = -kExpTableH * kExpTableH / 2.0f;
  static constexpr float c3 = kExpTableH * kExpTableH * kExpTableH / 6.0f;
  static constexpr float c4 =
      -kExpTableH * kExpTableH * kExpTableH * kExpTableH / 24.0f;
  __device__ __forceinline__ static float eval(float u, const float2* tab) {
    u = fminf(u, (float) (kExpTableSize - 1));
    // u + 2^23 rounded down carries floor(u) in its low mantissa bits
    const float t = __fadd_rd(u, 8388608.0f);
    const int i = __float_as_int(t) - 0x4B000000;
    const float du = u - (t - 8388608.0f);
    const float q = du * fmaf(du, fmaf(du, fmaf(du, c4, c3), c2), c1);
    const float2 ge = tab[i];
    return fmaf(ge.y, q, ge.x);
  }
};

// g(x) = 1 - exp(-x) from the hardware base-2 exponential, with the series
// x - x^2/2 + x^3/6 - x^4/24 + x^5/120 below x = 1/4 where 1 - exp(-x)
// would lose relative accuracy to cancellation.
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

// Registers available per thread: the busy instances keep 6 blocks of 128
// threads resident per SM, the small ones 8.
template <int PH, int SLOTS>
struct SweepOccupancy {
  static constexpr int min_blocks = (PH * SLOTS > 12) ? 6 : 8;
};

template <int PH, int LPS, int SLOTS, int EXPK>
__global__ void __launch_bounds__(kSweepThreads,
                                  (SweepOccupancy<PH, SLOTS>::min_blocks))
sweep_kernel(const SweepArgs a) {
  extern __shared__ float smem[];
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;

  const int G = a.num_groups;
  const int MG = a.num_materials * G;
  float2* s_tab = reinterpret_cast<float2*>(smem);
  float* s_st = smem + ((EXPK == kExpTable) ? 2 * kExpTableSize : 0);
  for (int i = threadIdx.x; i < MG; i += blockDim.x) s_st[i] = a.sigma_t[i];
  if (EXPK == kExpTable)
    for (int i = threadIdx.x; i < kExpTableSize; i += blockDim.x) {
      const float gi = a.exp_table[i];
      s_tab[i] = make_float2(gi, a.exp_table[kExpTableSize + i]);
    }
  __syncthreads();

  const int cur = sc->cur;
  const float* psi_in = a.psi[cur];
  float* psi_out = a.psi[cur ^ 1];
  const float scale = sc->scale[cur];

  const int lane = threadIdx.x & 31;
  const int sub = lane & (LPS - 1);
  const int64_t gwarp =
      ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t stream = gwarp * (32 / LPS) + lane / LPS;

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
    const float* pin = psi_in + ((int64_t) t * 2 + dir) * F + sub;
#pragma unroll
    for (int j = 0; j < SLOTS; j++) {
      const bool on = sub + j * LPS < G;
#pragma unroll
      for (int p = 0; p < PH; p++)
        psi[j][p] = on ? pin[p * G + j * LPS] * scale : 0.0f;
    }

    // Segment stream, software-pipelined.  The LPS lanes of a stream load
    // LPS consecutive segments with one coalesced access (a "chunk", one
    // segment per lane) a whole chunk ahead of use; segment k reaches every
    // lane of the stream by a shuffle from lane k % LPS.  The sources of
    // segment k+1 are gathered while segment k is integrated.
    const int2* seg = a.segs + b;
    const unsigned gmask =
        (LPS == 32) ? 0xffffffffu
                    : (((1u << LPS) - 1u) << (lane & ~(LPS - 1)));
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
    int2 chunk_next = fetch(LPS + sub);
    int2 sg;
    sg.x = __shfl_sync(gmask, chunk.x, 0, LPS);
    sg.y = __shfl_sync(gmask, chunk.y, 0, LPS);
    float len;
    int fsr, mat;
    unpack(sg, len, fsr, mat);
    const float* qbase = a.qt + sub;
    float q[SLOTS];
#pragma unroll
    for (int j = 0; j < SLOTS; j++)
      q[j] = (sub + j * LPS < G && n > 0)
                 ? __ldg(qbase + (int64_t) fsr * G + j * LPS)
                 : 0.0f;
    for (int k = 0; k < n; k++) {
      // next segment: rotate chunks at chunk boundaries
      const int kn = k + 1;
      const int src = kn & (LPS - 1);
      if (src == 0) {
        chunk = chunk_next;
        chunk_next = fetch(kn + LPS + sub);
      }
      int2 sgn;
      sgn.x = __shfl_sync(gmask, chunk.x, src, LPS);
      sgn.y = __shfl_sync(gmask, chunk.y, src, LPS);
      float len_n;
      int fsr_n, mat_n;
      unpack(sgn, len_n, fsr_n, mat_n);
      float qn[SLOTS];
      const float* qrow = qbase + (int64_t) fsr_n * G;
#pragma unroll
      for (int j = 0; j < SLOTS; j++)
        qn[j] = (sub + j * LPS < G && kn < n) ? __ldg(qrow + j * LPS) : 0.0f;

      const float* st = s_st + mat * G + sub;
      float* ph = a.phi + (int64_t) fsr * G + sub;
#pragma unroll
      for (int j = 0; j < SLOTS; j++) {
        if (sub + j * LPS < G) {
          const float tau = st[j * LPS] * len;
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
          atomicAdd(ph + j * LPS, tally);
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
      float* po = psi_out + ((int64_t) nt * 2 + nd) * F + sub;
#pragma unroll
      for (int j = 0; j < SLOTS; j++) {
        if (sub + j * LPS < G) {
#pragma unroll
          for (int p = 0; p < PH; p++) po[p * G + j * LPS] = psi[j][p];
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

template <int PH, int LPS, int SLOTS, int EXPK>
void launch_sweep_instance(const SweepArgs& a, cudaStream_t stream) {
  const int spw = 32 / LPS;
  const int64_t warps = (2 * a.num_tracks + spw - 1) / spw;
  const int wpb = kSweepThreads / 32;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  const size_t smem =
      sizeof(float) * ((size_t) a.num_materials * a.num_groups +
                       (EXPK == kExpTable ? 2 * kExpTableSize : 0));
  auto kern = sweep_kernel<PH, LPS, SLOTS, EXPK>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int) smem);
  kern<<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a);
}

template <int PH, int LPS, int EXPK>
bool dispatch_sweep_slots(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (slots) {
    case 1: launch_sweep_instance<PH, LPS, 1, EXPK>(a, s); return true;
    case 2: launch_sweep_instance<PH, LPS, 2, EXPK>(a, s); return true;
    case 3: launch_sweep_instance<PH, LPS, 3, EXPK>(a, s); return true;
    case 4: launch_sweep_instance<PH, LPS, 4, EXPK>(a, s); return true;
    case 5: launch_sweep_instance<PH, LPS, 5, EXPK>(a, s); return true;
    case 6: launch_sweep_instance<PH, LPS, 6, EXPK>(a, s); return true;
    case 7: launch_sweep_instance<PH, LPS, 7, EXPK>(a, s); return true;
    case 8: launch_sweep_instance<PH, LPS, 8, EXPK>(a, s); return true;
    case 9: launch_sweep_instance<PH, LPS, 9, EXPK>(a, s); return true;
    default: return false;
  }
}

template <int PH, int EXPK>
bool dispatch_sweep_lps(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (a.lps) {
    case 2: return dispatch_sweep_slots<PH, 2, EXPK>(a, slots, s);
    case 4: return dispatch_sweep_slots<PH, 4, EXPK>(a, slots, s);
    case 8: return dispatch_sweep_slots<PH, 8, EXPK>(a, slots, s);
    case 16: return dispatch_sweep_slots<PH, 16, EXPK>(a, slots, s);
    case 32: return dispatch_sweep_slots<PH, 32, EXPK>(a, slots, s);
    default: return false;
  }
}

}  // namespace moc
