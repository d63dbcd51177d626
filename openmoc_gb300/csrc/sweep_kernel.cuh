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
// in pairs (lane `sub` handles group pairs sub, sub+LPS, ..., PS of them)
// and keep the angular flux of those groups for every polar angle in
// registers along the whole track.  Each pair is integrated with the packed
// two-wide FP32 instructions of sm_100+ (FFMA2 / FADD2 / FMUL2), so one
// instruction advances two groups; sources are read 8 bytes at a time and
// tallies leave as one two-wide vector reduction (red.global.add.v2.f32)
// per pair and segment.  Flux rows are padded to an even group count (ld).
// The forward and backward streams of a track are adjacent (they share
// segment cache lines), and streams are ordered by decreasing segment count
// so that the longest tracks start first.
//
// Attenuation: delta = (psi - Q/sigma_t) * g(x), g(x) = 1 - exp(-x),
// x = sigma_t * l / sin(theta): algebraically the reference's
// (tau*psi - l*Q) * F1(x)/sin(theta) (src/CPUSolver.cpp:2463-2484).
#pragma once

#include "moc_internal.cuh"

namespace moc {

__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }

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
  // two groups; u2 = x / h
  __device__ __forceinline__ static float2 eval2(float2 u2, const float2* tab) {
    return make_float2(eval(u2.x, tab), eval(u2.y, tab));
  }
};

// g(x) = 1 - exp(-x) from the hardware base-2 exponential e ~ exp(-x)
// (relative error about 2^-22) and the Taylor polynomial
// T5(x) = x - x^2/2 + x^3/6 - x^4/24 + x^5/120.  T5 never falls below g
// (its remainder is -exp(-z) x^6/720 for some z in (0, x)), and it is
// accurate to 1e-9 relative below x = 0.1, where 1 - e loses relative
// accuracy to cancellation.  So
//   g = min(T5(x), 1 - (1 - kRel) e)
// takes T5 for small x and the exponential for larger x (where T5 rises
// away from g): one min instead of a compare and a select.  The factor
// 1 - kRel lifts the exponential branch above g by kRel*e, more than the
// hardware error, so both branches overestimate and the min is the closer
// one; the bias vanishes with e for optically thick segments.  The relative
// error is below ~2e-6 for every x (largest near the crossover x ~ 0.26).
// Both branches take the exponent u = -x log2(e) that ex2 needs: with
// x = -u ln 2, T5 is the polynomial u (b1 + u (b2 + ... + u b5)),
// b_i = -(ln 2)^i / i!, so x itself is never formed.
struct AttenIntrinsic {
  static constexpr float kRel = 5.0e-7f;
  static constexpr float b1 = -0.6931471805599453f;
  static constexpr float b2 = -0.2402265069591007f;
  static constexpr float b3 = -0.05550410866482158f;
  static constexpr float b4 = -0.009618129107628477f;
  static constexpr float b5 = -0.0013333558146428443f;
  __device__ __forceinline__ static float ex2(float v) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
  }
  // u2 = -x * log2(e) for two groups
  __device__ __forceinline__ static float2 eval2(float2 u2) {
    const float2 e = make_float2(ex2(u2.x), ex2(u2.y));
    const float2 big = __ffma2_rn(e, f2(kRel - 1.0f), f2(1.0f));
    float2 s = __ffma2_rn(u2, f2(b5), f2(b4));
    s = __ffma2_rn(u2, s, f2(b3));
    s = __ffma2_rn(u2, s, f2(b2));
    s = __ffma2_rn(u2, s, f2(b1));
    s = __fmul2_rn(u2, s);
    return make_float2(fminf(s.x, big.x), fminf(s.y, big.y));
  }
};

// Source look-ahead.  The busy instances (more than 6 pair-polar values per
// lane) stage the sources of the segments ahead in a shared-memory ring by
// asynchronous copies, which hold no registers: up to three segments ahead,
// bounded by the chunk window (a segment word is reachable from chunk or
// chunk_next up to LPS segments ahead).  The light instances, whose loop is
// short, keep the next segment's sources in registers (staging costs them
// more instructions than it hides: 51x51 / 7 groups 2.12 -> 3.12 ms).
template <int PH, int LPS, int PS>
struct SweepRing {
  static constexpr bool staged = PH * PS > 6;
  static constexpr int ahead = !staged ? 0 : (LPS < 3 ? LPS : 3);
};

__device__ __forceinline__ void cp_async8(void* smem_dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   (uint32_t) __cvta_generic_to_shared(smem_dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Registers available per thread: the busy instances keep 5 blocks of 128
// threads resident per SM (4 at 18 pair-polar values per lane), the small
// ones 8; one-polar (3D) instances with 3 or more pairs, whose shared-memory
// tallies need a few registers more, 6.  Measured on 17 x 17 / 70 groups
// (8 lanes x 5 pairs, ex2, loop unrolled by 4): 5 blocks 485 us per sweep,
// 6 blocks 513 us, 4 blocks 510 us.
#ifndef MOC_SWEEP_BIG_MIN_BLOCKS
#define MOC_SWEEP_BIG_MIN_BLOCKS 5
#endif
// Blocks per SM of the one-polar (3D) instances with one group pair per
// lane: their sweeps wait on loads, so resident warps (loads in flight) set
// their speed.  3D 17x17 assembly, 7 groups, 4 lanes x 1 pair: 8 blocks
// (56 registers, 9 resident) 1.692 ms per sweep, 10 blocks 1.723 ms,
// 12 blocks (40 registers) 1.516 ms; 14 and 16 leave 32 registers and
// spill 76 bytes.  The two-pair instances spill 60 bytes at 12 and keep 8.
#ifndef MOC_SWEEP_3D_MIN_BLOCKS
#define MOC_SWEEP_3D_MIN_BLOCKS 12
#endif
// ... and of the one-polar two-pair instances (adjacent pairs; the 3D
// assembly's autotuned 2 lanes x 2 pairs: 8 blocks, 62 registers, 1.394 ms
// per sweep; 10 blocks, 48 registers and 12 bytes spilled, 1.370 ms; 12
// blocks spill 64 bytes)
#ifndef MOC_SWEEP_3D_PAIRS2_MIN_BLOCKS
#define MOC_SWEEP_3D_PAIRS2_MIN_BLOCKS 10
#endif
// The busy instances of the CMFD mode, which also tally partial currents,
// take 4 blocks (their registers would spill at 5).
template <int PH, int PS, int MODE = 0>
struct SweepOccupancy {
  static constexpr int min_blocks =
      (PH * PS >= 18)              ? 4
      : (PH * PS > 6 && MODE == 2) ? 4
      : (PH * PS > 6)              ? MOC_SWEEP_BIG_MIN_BLOCKS
      : (PH == 1 && PS > 2)        ? 6
      : (PH == 1 && PS == 1)       ? MOC_SWEEP_3D_MIN_BLOCKS
      : (PH == 1 && PS == 2)       ? MOC_SWEEP_3D_PAIRS2_MIN_BLOCKS
                                   : 8;
};

// CMFD partial currents (mode 2 of the sweeps): faces 0 x-, 1 y-, 2 x+,
// 3 y+ of cell iy * nx + ix; a crossing adds sum_p w_p psi_p of the lane's
// group pairs (Cmfd::tallyCurrent, src/Cmfd.h:572-660).
// ADJ: the lane's pairs are adjacent (2 sub + s2), as in the sweep's light
// two-pair instances, instead of interleaved (sub + s2 LPS).
template <int PH, int LPS, int PS, bool ADJ = false>
__device__ __forceinline__ void cmfd_add_current(
    const SweepArgs& a, int cell, int face, float frac, int sub, int npairs,
    int ld, const float2 (&w2)[PH], const float2 (&psi)[PS][PH]) {
  float2* cp = reinterpret_cast<float2*>(
                   a.cm_cur + ((int64_t) cell * 4 + face) * ld) +
               (ADJ ? PS * sub : sub);
#pragma unroll
  for (int s2 = 0; s2 < PS; s2++) {
    if ((ADJ ? PS * sub + s2 : sub + s2 * LPS) < npairs) {
      float2 j = f2(0.0f);
#pragma unroll
      for (int p = 0; p < PH; p++) j = __ffma2_rn(w2[p], psi[s2][p], j);
      atomicAdd(cp + (ADJ ? s2 : s2 * LPS), __fmul2_rn(j, f2(frac)));
    }
  }
}

// The current out of segment f0's coarse cell when the next segment f1
// lies in another (a corner crossing half by each neighbouring cell,
// Cmfd::splitEdgeCurrents, src/Cmfd.cpp:2249-2345), or, at the end of the
// track (f1 < 0), through the boundary face of the track end.
template <int PH, int LPS, int PS, bool ADJ = false>
__device__ __forceinline__ void cmfd_tally_crossing(
    const SweepArgs& a, int t, int dir, int f0, int f1, bool at_end, int sub,
    int npairs, int ld, const float2 (&w2)[PH], const float2 (&psi)[PS][PH]) {
  const int c0 = __ldg(a.cm_cell + f0);
  if (f1 >= 0) {
    const int c1 = __ldg(a.cm_cell + f1);
    if (c1 == c0) return;
    const int dx = c1 % a.cm_nx - c0 % a.cm_nx;
    const int dy = c1 / a.cm_nx - c0 / a.cm_nx;
    const int fx = dx > 0 ? 2 : 0, fy = dy > 0 ? 3 : 1;
    if (dx != 0 && dy != 0) {
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0, fx, 0.5f, sub, npairs, ld, w2, psi);
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0 + dx, fy, 0.5f, sub, npairs, ld, w2,
                                    psi);
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0, fy, 0.5f, sub, npairs, ld, w2, psi);
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0 + dy * a.cm_nx, fx, 0.5f, sub,
                                    npairs, ld, w2, psi);
    } else {
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0, dx != 0 ? fx : fy, 1.0f, sub, npairs,
                                    ld, w2, psi);
    }
  } else if (at_end) {
    const int face = a.cm_end[2 * t + dir];
    if (face >= 0)
      cmfd_add_current<PH, LPS, PS, ADJ>(a, c0, face, 1.0f, sub, npairs, ld, w2,
                                    psi);
  }
}

// MODE 1: the tracks of many solves (a batched pool); each track takes its
// pending angular-flux scale and done flag from its own solve's state.
// MODE 2: one problem, also tallying the partial currents out of the
// coarse-mesh cells for CMFD (a.cm_cell set).
template <int PH, int LPS, int PS, int EXPK, int MODE>
__global__ void __launch_bounds__(kSweepThreads,
                                  (SweepOccupancy<PH, PS, MODE>::min_blocks))
sweep_kernel(const SweepArgs a) {
  constexpr bool POOL = MODE == 1;
  constexpr bool CMFD = MODE == 2;
  extern __shared__ float smem[];
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;

  const int G = a.num_groups;
  const int ld = a.ld;                       // even row stride >= G
  float2* s_tab = reinterpret_cast<float2*>(smem);
  float* s_st = smem + ((EXPK == kExpTable) ? 2 * kExpTableSize : 0);
  float* s_hot = s_st + a.num_materials * ld;   // [hot_count][ld]
  // [slot][pair][thread] ring of staged sources (8-byte aligned: every
  // region before it is an even number of floats)
  float2* s_ring = reinterpret_cast<float2*>(s_hot + a.hot_count * ld);
  // sigma_t rows padded to ld; the padding group gets sigma_t = 1
  for (int i = threadIdx.x; i < a.num_materials * ld; i += blockDim.x) {
    const int m = i / ld, g = i - m * ld;
    s_st[i] = (g < G) ? a.sigma_t[m * G + g] : 1.0f;
  }
  for (int i = threadIdx.x; i < a.hot_count * ld; i += blockDim.x) s_hot[i] = 0.0f;
  if (EXPK == kExpTable)
    for (int i = threadIdx.x; i < kExpTableSize; i += blockDim.x)
      s_tab[i] = make_float2(a.exp_table[i], a.exp_table[kExpTableSize + i]);
  __syncthreads();

  const int cur = sc->cur;
  const float* psi_in = a.psi[cur];
  float* psi_out = a.psi[cur ^ 1];

  const int lane = threadIdx.x & 31;
  const int sub = lane & (LPS - 1);
  const int64_t gwarp =
      ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t stream = gwarp * (32 / LPS) + lane / LPS;
  const int npairs = ld >> 1;
  // Pair s of this lane holds groups.  The host gives an instance at least
  // (PS - 1) * LPS group pairs (every shape it runs has PS = ceil(npairs /
  // LPS), and moc_set_sweep_shape and the server check it), so only a
  // lane's last pair can lie past the groups: in the busy (staged)
  // instances the others need no test and no branch.  The light instances
  // test every pair (holding the predicate costs them a spill).
  const bool last_live = sub + (PS - 1) * LPS < npairs;
  // Lane sub of a stream owns the group pairs pidx(s), s < PS: interleaved
  // with the stream's other lanes (sub + s LPS), or in the light two-pair
  // instances adjacent (2 sub + s), so that when the rows are padded to a
  // multiple of four floats one 16-byte gather and one 16-byte reduction
  // serve both pairs (the light instances' per-segment accesses, one line
  // per stream each, bound them by L1TEX throughput).
  constexpr bool kAdj = PS == 2 && !SweepRing<PH, LPS, PS>::staged;
  auto pidx = [&](int s) { return kAdj ? PS * sub + s : sub + s * LPS; };
  const bool vec4 = kAdj && (ld & 3) == 0;
  auto live_pair = [&](int s) {
    if constexpr (SweepRing<PH, LPS, PS>::staged)
      return s < PS - 1 || last_live;
    else
      return pidx(s) < npairs;
  };

  // the track and its pending scale; in a pool the solve of the track may
  // be finished (the LPS lanes of a stream share the track, so they agree
  // on skipping it)
  // The one-polar (3D) instances read their track from its record in
  // visiting order (coalesced; their tracks are short, so the scattered
  // per-track reads were a tenth of their DRAM traffic); the 2D ones, whose
  // long tracks amortise them, read per track.
  constexpr bool kRec = PH == 1;
  int t = 0;
  float scale = 1.0f;
  bool live = stream < 2 * a.num_tracks;
  int64_t b = 0;
  int n = 0, ang = 0;
  if (POOL) {
    if (live) {
      t = a.order[stream >> 1];
      const DevScalars* ts = a.slots + a.track_slot[t];
      live = ts->done == 0;
      scale = ts->scale[cur];
    }
  } else {
    scale = sc->scale[cur];
    if (live && kRec && a.rec) {
      // the track's record, in visiting order: one coalesced 32-byte read
      const int4* rp = reinterpret_cast<const int4*>(a.rec + (stream >> 1));
      const int4 r0 = __ldg(rp);
      b = (int64_t) (((uint64_t) (uint32_t) r0.y << 32) | (uint32_t) r0.x);
      t = r0.z;
      n = r0.w;
      ang = __ldg(&a.rec[stream >> 1].ang);
    } else if (live) {
      t = a.order[stream >> 1];
    }
  }
  if (live) {
    const int dir = (int) (stream & 1);
    if (POOL || !kRec || !a.rec) {
      b = a.seg_off[t];
      n = (int) (a.seg_off[t + 1] - b);
      ang = a.track_ang[t];
    }
    const int F = G * PH;

    // the exponent scale of each polar angle: x / h for the table, -x log2 e
    // for the hardware exponential
    float2 w2[PH], xs2[PH], xl2[PH];
#pragma unroll
    for (int p = 0; p < PH; p++) {
      w2[p] = f2(a.weights[ang * PH + p]);
      const float is = a.inv_sin[ang * PH + p];
      if (EXPK == kExpTable)
        xs2[p] = f2(is * kExpTableInvH);
      else
        xl2[p] = f2(is * -1.4426950408889634f);
    }

    // angular flux of this lane's groups: pair s holds groups
    // 2*(sub + s*LPS) and 2*(sub + s*LPS) + 1
    float2 psi[PS][PH];
    const float* pin = psi_in + ((int64_t) t * 2 + dir) * F;
#pragma unroll
    for (int s = 0; s < PS; s++) {
      const int g0 = 2 * pidx(s);
      // with instances each group takes its own instance's pending scale
      float sx = scale, sy = scale;
      if (!POOL && a.inst && g0 < G) {
        sx = a.inst->scale[cur][g0 / a.inst_groups];
        if (g0 + 1 < G) sy = a.inst->scale[cur][(g0 + 1) / a.inst_groups];
      }
#pragma unroll
      for (int p = 0; p < PH; p++) {
        psi[s][p].x = (g0 < G) ? pin[p * G + g0] * sx : 0.0f;
        psi[s][p].y = (g0 + 1 < G) ? pin[p * G + g0 + 1] * sy : 0.0f;
      }
    }

    // Segment stream, software-pipelined.  The LPS lanes of a stream load
    // LPS consecutive segments with one coalesced access (a "chunk", one
    // segment per lane) a whole chunk ahead of use; segment k reaches every
    // lane of the stream by a shuffle from lane k % LPS.  The sources of
    // segment k + kAhead are copied into shared memory while segment k is
    // integrated.
    constexpr bool kStaged = SweepRing<PH, LPS, PS>::staged;
    constexpr int kAhead = SweepRing<PH, LPS, PS>::ahead;
    constexpr int kRing = kAhead + 1;
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
    // `chunk` holds the LPS-aligned run of segments containing the current
    // segment k, chunk_next the run after it; segment j (k <= j < k + LPS)
    // comes from lane j % LPS of the one that holds it
    int kc = 0;   // the current segment
    auto word = [&](int j) -> int2 {
      const int2 w = ((j ^ kc) < LPS) ? chunk : chunk_next;
      int2 r;
      r.x = __shfl_sync(gmask, w.x, j & (LPS - 1), LPS);
      r.y = __shfl_sync(gmask, w.y, j & (LPS - 1), LPS);
      return r;
    };
    // The sources of segment j travel by asynchronous copies (8 bytes per
    // group pair) into ring slot j % kRing of this thread, kAhead segments
    // before use, so the look-ahead holds no registers; one copy group per
    // segment (empty past the end of the track).
    const float2* qbase = reinterpret_cast<const float2*>(a.qt) + sub;
    auto slot = [&](int j, int s) -> float2* {
      return s_ring + ((j % kRing) * PS + s) * kSweepThreads + threadIdx.x;
    };
    auto stage = [&](int j) {
      if (j < n) {
        float l;
        int f, m;
        unpack(word(j), l, f, m);
        const float2* src = qbase + (int64_t) f * npairs;
#pragma unroll
        for (int s = 0; s < PS; s++)
          if (live_pair(s)) cp_async8(slot(j, s), src + s * LPS);
      }
      cp_async_commit();
    };
    // the register path: segment k + 1's word from `chunk` and its sources
    // in registers, loaded while segment k is integrated
    auto word_cur = [&](int j) -> int2 {
      int2 r;
      r.x = __shfl_sync(gmask, chunk.x, j & (LPS - 1), LPS);
      r.y = __shfl_sync(gmask, chunk.y, j & (LPS - 1), LPS);
      return r;
    };
    auto gather = [&](float2* qq, int f, bool valid) {
      if constexpr (kAdj) {
        const float2* qrow = reinterpret_cast<const float2*>(a.qt) +
                             (int64_t) f * npairs + PS * sub;
        if (vec4) {
          // npairs even: a lane's second pair is live with its first
          const float4 v = (valid && live_pair(0))
                               ? __ldg(reinterpret_cast<const float4*>(qrow))
                               : make_float4(0.f, 0.f, 0.f, 0.f);
          qq[0] = make_float2(v.x, v.y);
          qq[1] = make_float2(v.z, v.w);
        } else {
#pragma unroll
          for (int s = 0; s < PS; s++)
            qq[s] = (live_pair(s) && valid) ? __ldg(qrow + s) : f2(0.0f);
        }
      } else {
        const float2* qrow = qbase + (int64_t) f * npairs;
#pragma unroll
        for (int s = 0; s < PS; s++)
          qq[s] = (live_pair(s) && valid) ? __ldg(qrow + s * LPS) : f2(0.0f);
      }
    };
    float len = 0.0f;
    int fsr = 0, mat = 0;
    float2 q[PS];
    auto tally_current = [&](int f0, int f1, bool at_end) {
      cmfd_tally_crossing<PH, LPS, PS, kAdj>(a, t, dir, f0, f1, at_end, sub,
                                             npairs, ld, w2, psi);
    };
    if constexpr (kStaged) {
#pragma unroll
      for (int j = 0; j < kAhead; j++) stage(j);
    } else {
      unpack(word_cur(0), len, fsr, mat);
      gather(q, fsr, n > 0);
    }
    // the staged loop unrolled by the ring's depth (4): the ring slots of
    // the four copies are compile-time offsets
#pragma unroll(kStaged ? 4 : 1)
    for (int k = 0; k < n; k++) {
      float len_n = 0.0f;
      int fsr_n = 0, mat_n = 0;
      float2 qn[PS];
      if constexpr (kStaged) {
        kc = k;
        stage(k + kAhead);
        // segment k always lies in `chunk` here (it rotates below, once
        // segment k + 1 leaves it)
        unpack(word_cur(k), len, fsr, mat);
        if (((k + 1) & (LPS - 1)) == 0) {
          chunk = chunk_next;
          chunk_next = fetch(k + 1 + LPS + sub);
        }
        cp_async_wait<kAhead>();   // segment k's sources have landed
      } else {
        // segment k + 1 opens a chunk: rotate
        if (((k + 1) & (LPS - 1)) == 0) {
          chunk = chunk_next;
          chunk_next = fetch(k + 1 + LPS + sub);
        }
        unpack(word_cur(k + 1), len_n, fsr_n, mat_n);
        gather(qn, fsr_n, k + 1 < n);
      }

      const float2* st =
          reinterpret_cast<const float2*>(s_st + mat * ld) + pidx(0);
      float2* ph =
          reinterpret_cast<float2*>(a.phi + (int64_t) fsr * ld) + pidx(0);
      // a region crossed by most tracks tallies into this block's copy
      // (3D problems only, PH == 1: one moderator region above the fuel)
      const int hot = (PH == 1) ? fsr - a.hot_base : -1;
      const float2 len2 = f2(len);
      float2 tl0 = f2(0.0f);   // the first adjacent pair's tally, sent with the second
#pragma unroll
      for (int s = 0; s < PS; s++) {
        if (live_pair(s)) {
          const float2 qs = kStaged ? *slot(k, s) : q[s];
          const float2 tau = __fmul2_rn(st[pidx(s) - pidx(0)], len2);
          float2 tally = f2(0.0f);
#pragma unroll
          for (int p = 0; p < PH; p++) {
            float2 gx;
            if (EXPK == kExpTable)
              gx = AttenTable::eval2(__fmul2_rn(tau, xs2[p]), s_tab);
            else
              gx = AttenIntrinsic::eval2(__fmul2_rn(tau, xl2[p]));
            // d = (psi - q) * g;  psi -= d;  tally += w * d
            const float2 d =
                __fmul2_rn(__ffma2_rn(qs, f2(-1.0f), psi[s][p]), gx);
            psi[s][p] = __ffma2_rn(d, f2(-1.0f), psi[s][p]);
            tally = __ffma2_rn(w2[p], d, tally);
          }
          if (PH == 1 && hot >= 0) {
            float* hp = s_hot + hot * ld + 2 * pidx(s);
            atomicAdd(hp, tally.x);
            atomicAdd(hp + 1, tally.y);
          } else if constexpr (kAdj) {
            if (!vec4)
              atomicAdd(ph + s, tally);
            else if (s == 0)
              tl0 = tally;
            else
              atomicAdd(reinterpret_cast<float4*>(ph),
                        make_float4(tl0.x, tl0.y, tally.x, tally.y));
          } else {
            atomicAdd(ph + s * LPS, tally);
          }
        }
      }

      if constexpr (CMFD) {
        // partial current out of the coarse cell when the next segment lies
        // in another one (through an intermediate cell at a corner), or out
        // through the boundary at the end of a track that is not continued
        int fsr_next = -1;
        if (k + 1 < n) {
          if constexpr (kStaged) {
            // segment k + 1 lies in `chunk` once the rotation above is done
            float l2;
            int m2;
            unpack(word_cur(k + 1), l2, fsr_next, m2);
          } else {
            fsr_next = fsr_n;
          }
        }
        tally_current(fsr, fsr_next, k + 1 == n);
      }
      if constexpr (!kStaged) {
        len = len_n;
        fsr = fsr_n;
        mat = mat_n;
#pragma unroll
        for (int s = 0; s < PS; s++) q[s] = qn[s];
      }
    }

    // boundary-flux transfer to the connecting track, fused into the sweep
    // (CPUSolver::transferBoundaryFlux, src/CPUSolver.cpp:2560-2600); at a
    // vacuum end, when keff comes from the neutron balance, the leakage:
    // the outgoing angular flux of every polar value and group weighted by
    // the quadrature weight of the track's polar index, which is 0 for 2D
    // tracks (src/CPUSolver.cpp:2593-2600, src/TrackTraversingAlgorithms.cpp
    // :895-905), summed over the stream's lanes, one FP64 atomic per stream
    // the record's flags and connecting tracks (read again here rather
    // than held in registers through the segment loop)
    int4 r1 = make_int4(0, 0, 0, 0);
    if (!POOL && kRec && a.rec) {
      // the stream index again from the thread's coordinates (cheaper than
      // keeping it live through the loop)
      const int64_t gw = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      const int64_t st2 = gw * (32 / LPS) + (threadIdx.x & 31) / LPS;
      r1 = __ldg(reinterpret_cast<const int4*>(a.rec + (st2 >> 1)) + 1);
    }
    const int f = (!POOL && kRec && a.rec) ? r1.y : a.flags[t];
    if (!(f & (dir ? 8 : 4)) && a.leakage) {
      float2 acc = f2(0.0f);
#pragma unroll
      for (int s = 0; s < PS; s++) {
        const int g0 = 2 * pidx(s);
#pragma unroll
        for (int p = 0; p < PH; p++) {
          if (g0 < G) acc.x += psi[s][p].x;
          if (g0 + 1 < G) acc.y += psi[s][p].y;
        }
      }
      float v = (acc.x + acc.y) * w2[0].x;
#pragma unroll
      for (int o = LPS / 2; o > 0; o >>= 1)
        v += __shfl_xor_sync(gmask, v, o, LPS);
      if (sub == 0) atomicAdd(a.leakage, (double) v);
    }
    if (f & (dir ? 8 : 4)) {
      const int nt =
          (!POOL && kRec && a.rec) ? (dir ? r1.w : r1.z) : a.next[2 * t + dir];
      const int nd = (f & (dir ? 2 : 1)) ? 0 : 1;
      float* po = psi_out + ((int64_t) nt * 2 + nd) * F;
#pragma unroll
      for (int s = 0; s < PS; s++) {
        const int g0 = 2 * pidx(s);
#pragma unroll
        for (int p = 0; p < PH; p++) {
          if (g0 < G) po[p * G + g0] = psi[s][p].x;
          if (g0 + 1 < G) po[p * G + g0 + 1] = psi[s][p].y;
        }
      }
    }
  }

  // The last block to finish flips the buffer index: every block has read
  // sc->cur by then.  The buffer just written starts with scale 1.
  __shared__ int last;
  __syncthreads();
  // this block's totals of the shared-memory tallies
  for (int i = threadIdx.x; i < a.hot_count * ld; i += blockDim.x) {
    const float v = s_hot[i];
    if (v != 0.0f) atomicAdd(a.phi + (int64_t) a.hot_base * ld + i, v);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int ticket = atomicAdd(&sc->ticket_sweep, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    if (POOL)
      for (int i = threadIdx.x; i < a.num_slots; i += blockDim.x)
        a.slots[i].scale[cur ^ 1] = 1.0f;
    if (!POOL && a.inst)
      for (int i = threadIdx.x; i < kMaxInstances; i += blockDim.x)
        a.inst->scale[cur ^ 1][i] = 1.0f;
    if (threadIdx.x == 0) {
      sc->ticket_sweep = 0;
      sc->scale[cur ^ 1] = 1.0f;
      sc->cur = cur ^ 1;
      __threadfence();
    }
  }
}

template <int PH, int LPS, int PS, int EXPK, int MODE>
void launch_sweep_instance(const SweepArgs& a, cudaStream_t stream) {
  const int spw = 32 / LPS;
  const int64_t warps = (2 * a.num_tracks + spw - 1) / spw;
  const int wpb = kSweepThreads / 32;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  const size_t smem =
      sizeof(float) * ((size_t) (a.num_materials + a.hot_count) * a.ld +
                       (EXPK == kExpTable ? 2 * kExpTableSize : 0)) +
      (SweepRing<PH, LPS, PS>::staged
           ? sizeof(float2) * (SweepRing<PH, LPS, PS>::ahead + 1) * PS *
                 kSweepThreads
           : 0);
  auto kern = sweep_kernel<PH, LPS, PS, EXPK, MODE>;
  kern<<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a);
}

// The shared-memory limit of every instance dispatch_sweep_lps can launch.
template <int PH, int LPS, int EXPK>
void configure_sweep_lps(int optin) {
  raise_smem_limit(sweep_kernel<PH, LPS, 1, EXPK, 0>, optin);
  raise_smem_limit(sweep_kernel<PH, LPS, 2, EXPK, 0>, optin);
  raise_smem_limit(sweep_kernel<PH, LPS, 3, EXPK, 0>, optin);
  raise_smem_limit(sweep_kernel<PH, LPS, 4, EXPK, 0>, optin);
  raise_smem_limit(sweep_kernel<PH, LPS, 5, EXPK, 0>, optin);
  raise_smem_limit(sweep_kernel<PH, LPS, 6, EXPK, 0>, optin);
  if constexpr (EXPK == kExpIntrinsic) {
    raise_smem_limit(sweep_kernel<PH, LPS, 1, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 2, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 3, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 4, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 5, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 6, EXPK, 1>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 1, EXPK, 2>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 2, EXPK, 2>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 3, EXPK, 2>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 4, EXPK, 2>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 5, EXPK, 2>, optin);
    raise_smem_limit(sweep_kernel<PH, LPS, 6, EXPK, 2>, optin);
  }
}

template <int PH, int EXPK>
void configure_sweep(int optin) {
  configure_sweep_lps<PH, 1, EXPK>(optin);
  configure_sweep_lps<PH, 2, EXPK>(optin);
  configure_sweep_lps<PH, 4, EXPK>(optin);
  configure_sweep_lps<PH, 8, EXPK>(optin);
  configure_sweep_lps<PH, 16, EXPK>(optin);
  configure_sweep_lps<PH, 32, EXPK>(optin);
}

// slots = pairs of groups per lane
template <int PH, int LPS, int EXPK, int MODE>
bool launch_sweep_pairs(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (slots) {
    case 1: launch_sweep_instance<PH, LPS, 1, EXPK, MODE>(a, s); return true;
    case 2: launch_sweep_instance<PH, LPS, 2, EXPK, MODE>(a, s); return true;
    case 3: launch_sweep_instance<PH, LPS, 3, EXPK, MODE>(a, s); return true;
    case 4: launch_sweep_instance<PH, LPS, 4, EXPK, MODE>(a, s); return true;
    case 5: launch_sweep_instance<PH, LPS, 5, EXPK, MODE>(a, s); return true;
    case 6: launch_sweep_instance<PH, LPS, 6, EXPK, MODE>(a, s); return true;
    default: return false;
  }
}

// Pools (a.track_slot set) have instances for the hardware-ex2 evaluator
// only.
template <int PH, int LPS, int EXPK>
bool dispatch_sweep_slots(const SweepArgs& a, int slots, cudaStream_t s) {
  if (a.track_slot) {
    if constexpr (EXPK == kExpIntrinsic)
      return launch_sweep_pairs<PH, LPS, EXPK, 1>(a, slots, s);
    else
      return false;
  }
  if (a.cm_cell) {
    if constexpr (EXPK == kExpIntrinsic)
      return launch_sweep_pairs<PH, LPS, EXPK, 2>(a, slots, s);
    else
      return false;
  }
  return launch_sweep_pairs<PH, LPS, EXPK, 0>(a, slots, s);
}

template <int PH, int EXPK>
bool dispatch_sweep_lps(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (a.lps) {
    case 1: return dispatch_sweep_slots<PH, 1, EXPK>(a, slots, s);
    case 2: return dispatch_sweep_slots<PH, 2, EXPK>(a, slots, s);
    case 4: return dispatch_sweep_slots<PH, 4, EXPK>(a, slots, s);
    case 8: return dispatch_sweep_slots<PH, 8, EXPK>(a, slots, s);
    case 16: return dispatch_sweep_slots<PH, 16, EXPK>(a, slots, s);
    case 32: return dispatch_sweep_slots<PH, 32, EXPK>(a, slots, s);
    default: return false;
  }
}

}  // namespace moc
