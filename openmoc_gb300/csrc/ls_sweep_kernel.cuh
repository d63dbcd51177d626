// The linear-source transport sweep kernel for sm_103a, included by the
// ls_sweep_p<Ph>.cu translation units (one per polar count).
//
// Restates CPULSSolver::tallyLSScalarFlux (2D branch,
// src/CPULSSolver.cpp:653-741) and accumulateLinearFluxContribution
// (:749-781) inside TransportSweep::onTrack (src/TrackTraversingAlgorithms.
// cpp:890-1052), with the work decomposition of the flat-source sweep
// (sweep_kernel.cuh): a "stream" is one direction of one track, its LPS
// lanes split the energy groups in pairs (PS pairs per lane) and keep the
// angular flux of every polar angle in registers; pairs are integrated with
// the packed two-wide FP32 instructions.
//
// Per segment the lanes read one 16-byte word {length, FSR | material << 24,
// x, y} ((x, y) = forward start relative to the FSR centroid), and per group
// pair the flat source Q/sigma_t (8 bytes) and the x / y source moments
// divided by sigma_t (16 bytes).  Tallies leave as one two-wide reduction
// for the scalar flux and one four-wide reduction (x and y of two groups)
// for the moments per pair and segment.
//
// With x = sigma_t l / sin(theta), G(x) = (x - 1 + exp(-x)) / x^2,
// u = 1 - x G = (1 - exp(-x)) / x, A = x u = 1 - exp(-x):
//   source along the segment   s_f = (Q + q_x c_x + q_y c_y) / sigma_t,
//                              c = 2 p + l d (twice the segment midpoint),
//   linear part                s_l = l (d . q) / sigma_t,
//   delta = (psi - s_f) A - s_l x (2 G - u),
//   psi -= delta, phi += w delta,
//   moments += w l x (u - G) psi_in d + w delta p,
// which is the reference's (tau psi - l s) F1 - l^2 s_lin F2 and
// exp_H = (F1 - G/sin) w tau l psi with F1 = u / sin, F2 = (2G - u) / sin
// (ExpEvaluator::retrieveExponentialComponents, src/ExpEvaluator.h:
// 343-380), rearranged so that every term is per unit sigma_t.
#pragma once

#include "sweep_kernel.cuh"

namespace moc {

// G(x) = (x - 1 + exp(-x)) / x^2 for x >= 0 by a rational P5(x) / Q6(x)
// fitted for least maximum relative error (iteratively reweighted least
// squares; openmoc_gb300/csrc/fit_ls_exponential.py derives the
// coefficients), with P(0)/Q(0) = 1/2 and the leading coefficients equal so
// that G ~ 1/x for large x.  Relative error 1.6e-7 in exact arithmetic,
// below 6e-7 evaluated in FP32 (every x from 1e-7 to 5000).  neg_eval2
// returns -G (the numerator's coefficients negated), which lets the sweep
// form every term with plain fused multiply-adds.
struct LsExpG {
  static constexpr float p0 = 5.0000000000e-01f;
  static constexpr float p1 = 1.7653049922e-01f;
  static constexpr float p2 = 4.0405449407e-02f;
  static constexpr float p3 = 6.1757359007e-03f;
  static constexpr float p4 = 6.4268462614e-04f;
  static constexpr float p5 = 6.0568726961e-05f;
  static constexpr float q1 = 6.8639100170e-01f;
  static constexpr float q2 = 2.2629653913e-01f;
  static constexpr float q3 = 4.7201237695e-02f;
  static constexpr float q4 = 6.8802606036e-03f;
  static constexpr float q5 = 7.0324702263e-04f;
  static constexpr float q6 = 6.0568726961e-05f;
  __device__ __forceinline__ static float rcp(float v) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
  }
  __device__ __forceinline__ static float2 neg_eval2(float2 x) {
    float2 n = __ffma2_rn(x, f2(-p5), f2(-p4));
    n = __ffma2_rn(x, n, f2(-p3));
    n = __ffma2_rn(x, n, f2(-p2));
    n = __ffma2_rn(x, n, f2(-p1));
    n = __ffma2_rn(x, n, f2(-p0));
    float2 d = __ffma2_rn(x, f2(q6), f2(q5));
    d = __ffma2_rn(x, d, f2(q4));
    d = __ffma2_rn(x, d, f2(q3));
    d = __ffma2_rn(x, d, f2(q2));
    d = __ffma2_rn(x, d, f2(q1));
    d = __ffma2_rn(x, d, f2(1.0f));
    return __fmul2_rn(n, make_float2(rcp(d.x), rcp(d.y)));
  }
};

// Blocks of 128 threads kept resident per SM: the register file bounds the
// busy instances (PH * PS pair-polar values per lane); the 3D instances
// carry the z source moments and tallies of every pair as well, and their
// light ones wait on loads (MOC_LS3D_MIN_BLOCKS: 3D 17x17 assembly, 7
// groups, 4 lanes x 1 pair, 6 blocks (72 registers) 4.277 ms per sweep,
// 8 blocks (62) 4.205 ms; 10 spills).
#ifndef MOC_LS3D_MIN_BLOCKS
#define MOC_LS3D_MIN_BLOCKS 8
#endif
template <int PH, int PS, bool D3>
struct LsOccupancy {
  static constexpr int min_blocks =
      D3 ? ((PS >= 4) ? 3 : (PS >= 3) ? 4 : (PS == 2) ? 6 : MOC_LS3D_MIN_BLOCKS)
         : ((PH * PS >= 12) ? 4 : (PH * PS >= 6) ? 5 : 6);
};

// CM: also the CMFD partial currents (a.cm_cell set), as the flat sweep's
// mode 2.  In a pool (a.track_slot set) each track takes the pending
// angular-flux scale of its solve and is skipped once its solve is done, as
// in the flat sweep's mode 1.  D3 (PH = 1): explicit 3D tracks, the 3D
// branch of tallyLSScalarFlux (src/CPULSSolver.cpp:555-646) -- true
// lengths (inv_sin = 1), the 3D direction of the angle row, the z start of
// each segment and the z source moment and tally.
template <int PH, int LPS, int PS, bool CM, bool D3 = false>
__global__ void __launch_bounds__(kSweepThreads,
                                  (LsOccupancy<PH, PS, D3>::min_blocks))
ls_sweep_kernel(const SweepArgs a) {
  extern __shared__ float smem[];
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;

  const int G = a.num_groups;
  const int ld = a.ld;
  float* s_st = smem;   // sigma_t rows padded to ld (padding group: 1)
  for (int i = threadIdx.x; i < a.num_materials * ld; i += blockDim.x) {
    const int m = i / ld, g = i - m * ld;
    s_st[i] = (g < G) ? a.sigma_t[m * G + g] : 1.0f;
  }
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
  // lane sub owns the group pairs pidx(s): interleaved (sub + s LPS), or in
  // the two-pair instances adjacent (2 sub + s), so that with rows padded to
  // a multiple of four floats the flat and z sources and their tallies of
  // both pairs travel in 16-byte accesses (as in the flat sweep)
  constexpr bool kAdj = PS == 2;
  auto pidx = [&](int s) { return kAdj ? PS * sub + s : sub + s * LPS; };
  const bool vec4 = kAdj && (ld & 3) == 0;

  // the LPS lanes of a stream share its track, so they agree on skipping it
  bool live = stream < 2 * a.num_tracks;
  int t = 0;
  float scale = sc->scale[cur];
  if (live) {
    t = a.order[stream >> 1];
    if (a.track_slot) {
      const DevScalars* ts = a.slots + a.track_slot[t];
      live = ts->done == 0;
      scale = ts->scale[cur];
    }
  }
  if (live) {
    const int dir = (int) (stream & 1);
    const int64_t b = a.seg_off[t];
    const int n = (int) (a.seg_off[t + 1] - b);
    const int ang = a.track_ang[t];
    const int F = G * PH;
    // forward direction, and the direction of travel of this stream
    float2 fd;
    float fdz = 0.0f;
    if constexpr (D3) {
      const float4 d3 = a.ang_dir3[ang];
      fd = make_float2(d3.x, d3.y);
      fdz = d3.z;
    } else {
      fd = a.ang_dir[ang];
    }
    const float dx = dir ? -fd.x : fd.x;
    const float dy = dir ? -fd.y : fd.y;
    const float dz = dir ? -fdz : fdz;

    float2 w2[PH], xs2[PH], xw2[PH];
#pragma unroll
    for (int p = 0; p < PH; p++) {
      const float w = a.weights[ang * PH + p];
      const float is = a.inv_sin[ang * PH + p];
      w2[p] = f2(w);
      xs2[p] = f2(is);
      xw2[p] = f2(is * w);
    }

    float2 psi[PS][PH];
    const float* pin = psi_in + ((int64_t) t * 2 + dir) * F;
#pragma unroll
    for (int s = 0; s < PS; s++) {
      const int g0 = 2 * pidx(s);
#pragma unroll
      for (int p = 0; p < PH; p++) {
        psi[s][p].x = (g0 < G) ? pin[p * G + g0] * scale : 0.0f;
        psi[s][p].y = (g0 + 1 < G) ? pin[p * G + g0 + 1] * scale : 0.0f;
      }
    }

    // Segment words, LPS per coalesced load (one per lane), a chunk ahead;
    // word k reaches every lane of the stream by shuffles from lane k % LPS.
    const int4* seg = a.segs_ls + b;
    const unsigned gmask =
        (LPS == 32) ? 0xffffffffu
                    : (((1u << LPS) - 1u) << (lane & ~(LPS - 1)));
    auto fetch = [&](int kk) -> int4 {
      return (kk < n) ? __ldg(seg + (dir ? n - 1 - kk : kk))
                      : make_int4(0, 0, 0, 0);
    };
    auto word = [&](const int4& c, int j) -> int4 {
      int4 r;
      r.x = __shfl_sync(gmask, c.x, j & (LPS - 1), LPS);
      r.y = __shfl_sync(gmask, c.y, j & (LPS - 1), LPS);
      r.z = __shfl_sync(gmask, c.z, j & (LPS - 1), LPS);
      r.w = __shfl_sync(gmask, c.w, j & (LPS - 1), LPS);
      return r;
    };
    int4 chunk = fetch(sub);
    int4 chunk_next = fetch(LPS + sub);
    int4 wcur = word(chunk, 0);
    // 3D: the z starts, fetched and broadcast like the words
    const float* segz = D3 ? a.seg_z + b : nullptr;
    auto fetchz = [&](int kk) -> float {
      return (D3 && kk < n) ? __ldg(segz + (dir ? n - 1 - kk : kk)) : 0.0f;
    };
    float zchunk = fetchz(sub);
    float zchunk_next = fetchz(LPS + sub);
    float zcur = D3 ? __shfl_sync(gmask, zchunk, 0, LPS) : 0.0f;

    const float2* qf_base = reinterpret_cast<const float2*>(a.qt) + pidx(0);
    const float4* qm_base = reinterpret_cast<const float4*>(a.qxy) + pidx(0);
    const float2* qz_base =
        D3 ? reinterpret_cast<const float2*>(a.qz) + pidx(0) : nullptr;
    for (int k = 0; k < n; k++) {
      // the next segment's word: segment k + 1 opens a chunk every LPS
      if (((k + 1) & (LPS - 1)) == 0) {
        chunk = chunk_next;
        chunk_next = fetch(k + 1 + LPS + sub);
        if constexpr (D3) {
          zchunk = zchunk_next;
          zchunk_next = fetchz(k + 1 + LPS + sub);
        }
      }
      const int4 wnext = word(chunk, k + 1);
      float znext = 0.0f;
      if constexpr (D3)
        znext = __shfl_sync(gmask, zchunk, (k + 1) & (LPS - 1), LPS);

      const float len = __int_as_float(wcur.x);
      const int fsr = wcur.y & 0xFFFFFF;
      const int mat = (int) ((unsigned) wcur.y >> 24);
      const float px = __int_as_float(wcur.z);
      const float py = __int_as_float(wcur.w);
      // start of the segment in the direction of travel; twice its midpoint
      const float sx = dir ? fmaf(fd.x, len, px) : px;
      const float sy = dir ? fmaf(fd.y, len, py) : py;
      const float c2x = fmaf(2.0f, px, len * fd.x);
      const float c2y = fmaf(2.0f, py, len * fd.y);
      const float pz = zcur;
      const float sz = dir ? fmaf(fdz, len, pz) : pz;
      const float c2z = fmaf(2.0f, pz, len * fdz);

      float2 qf[PS], qzz[PS];
      float4 qm[PS];
#pragma unroll
      for (int s = 0; s < PS; s++) {
        const int ds = pidx(s) - pidx(0);
        const bool on = pidx(s) < npairs;
        qm[s] = on ? __ldg(qm_base + (int64_t) fsr * npairs + ds)
                   : make_float4(0.f, 0.f, 0.f, 0.f);
        if (!vec4) {
          qf[s] = on ? __ldg(qf_base + (int64_t) fsr * npairs + ds) : f2(0.0f);
          qzz[s] = (D3 && on) ? __ldg(qz_base + (int64_t) fsr * npairs + ds)
                              : f2(0.0f);
        }
      }
      if (vec4) {
        // npairs even: a lane's second pair is live with its first
        const bool on = pidx(0) < npairs;
        const float4 f4 =
            on ? __ldg(reinterpret_cast<const float4*>(qf_base +
                                                       (int64_t) fsr * npairs))
               : make_float4(0.f, 0.f, 0.f, 0.f);
        qf[0] = make_float2(f4.x, f4.y);
        qf[1 % PS] = make_float2(f4.z, f4.w);
        float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (D3 && on)
          z4 = __ldg(reinterpret_cast<const float4*>(qz_base +
                                                     (int64_t) fsr * npairs));
        qzz[0] = make_float2(z4.x, z4.y);
        qzz[1 % PS] = make_float2(z4.z, z4.w);
      }

      const float2* st =
          reinterpret_cast<const float2*>(s_st + mat * ld) + pidx(0);
      float2* ph =
          reinterpret_cast<float2*>(a.phi + (int64_t) fsr * ld) + pidx(0);
      float4* pm =
          reinterpret_cast<float4*>(a.mom + (int64_t) fsr * 2 * ld) + pidx(0);
      float2* pmz =
          D3 ? reinterpret_cast<float2*>(a.momz + (int64_t) fsr * ld) + pidx(0)
             : nullptr;
      const float2 len2 = f2(len);
      // the first adjacent pair's flux and z tallies, sent with the second's
      float2 ph0 = f2(0.0f), pz0 = f2(0.0f);
#pragma unroll
      for (int s = 0; s < PS; s++) {
        const int ds = pidx(s) - pidx(0);
        if (pidx(s) < npairs) {
          const float2 tau = __fmul2_rn(st[ds], len2);
          const float2 qx = make_float2(qm[s].x, qm[s].z);
          const float2 qy = make_float2(qm[s].y, qm[s].w);
          float2 sf = __ffma2_rn(qy, f2(c2y), __ffma2_rn(qx, f2(c2x), qf[s]));
          float2 sdq = __ffma2_rn(qy, f2(dy), __fmul2_rn(qx, f2(dx)));
          if constexpr (D3) {
            sf = __ffma2_rn(qzz[s], f2(c2z), sf);
            sdq = __ffma2_rn(qzz[s], f2(dz), sdq);
          }
          const float2 sl = __fmul2_rn(sdq, len2);
          // gn = -G, u = 1 - x G, m = u - 2 G = -(2G - u):
          //   delta = (psi - s_f) x u + (s_l x) m
          //   moment term w l x (u - G) psi = l tau (w / sin) (u + gn) psi
          float2 dacc = f2(0.0f), hacc = f2(0.0f);
#pragma unroll
          for (int p = 0; p < PH; p++) {
            const float2 x = __fmul2_rn(tau, xs2[p]);
            const float2 gn = LsExpG::neg_eval2(x);
            const float2 u = __ffma2_rn(x, gn, f2(1.0f));
            const float2 att = __fmul2_rn(x, u);
            const float2 m = __ffma2_rn(f2(2.0f), gn, u);
            const float2 e = __ffma2_rn(sf, f2(-1.0f), psi[s][p]);
            const float2 d =
                __ffma2_rn(e, att, __fmul2_rn(__fmul2_rn(sl, x), m));
            hacc = __ffma2_rn(__fmul2_rn(__fadd2_rn(u, gn), psi[s][p]), xw2[p],
                              hacc);
            psi[s][p] = __ffma2_rn(d, f2(-1.0f), psi[s][p]);
            dacc = __ffma2_rn(w2[p], d, dacc);
          }
          const float2 hl = __fmul2_rn(__fmul2_rn(hacc, tau), len2);
          const float2 mx = __ffma2_rn(dacc, f2(sx), __fmul2_rn(hl, f2(dx)));
          const float2 my = __ffma2_rn(dacc, f2(sy), __fmul2_rn(hl, f2(dy)));
          atomicAdd(pm + ds, make_float4(mx.x, my.x, mx.y, my.y));
          float2 mz = f2(0.0f);
          if constexpr (D3)
            mz = __ffma2_rn(dacc, f2(sz), __fmul2_rn(hl, f2(dz)));
          if (!vec4) {
            atomicAdd(ph + ds, dacc);
            if constexpr (D3) atomicAdd(pmz + ds, mz);
          } else if (s == 0) {
            ph0 = dacc;
            pz0 = mz;
          } else {
            atomicAdd(reinterpret_cast<float4*>(ph),
                      make_float4(ph0.x, ph0.y, dacc.x, dacc.y));
            if constexpr (D3)
              atomicAdd(reinterpret_cast<float4*>(pmz),
                        make_float4(pz0.x, pz0.y, mz.x, mz.y));
          }
        }
      }
      if constexpr (CM) {
        const int fsr_next = (k + 1 < n) ? (wnext.y & 0xFFFFFF) : -1;
        cmfd_tally_crossing<PH, LPS, PS, kAdj>(a, t, dir, fsr, fsr_next,
                                               k + 1 == n, sub, npairs, ld, w2,
                                               psi);
      }
      wcur = wnext;
      if constexpr (D3) zcur = znext;
    }

    // boundary-flux transfer to the connecting track
    // (CPUSolver::transferBoundaryFlux, src/CPUSolver.cpp:2560-2600)
    const int f = a.flags[t];
    if (f & (dir ? 8 : 4)) {
      const int nt = a.next[2 * t + dir];
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

  // the last block to finish flips the angular-flux buffer
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int ticket = atomicAdd(&sc->ticket_sweep, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    if (a.track_slot)
      for (int i = threadIdx.x; i < a.num_slots; i += blockDim.x)
        a.slots[i].scale[cur ^ 1] = 1.0f;
    if (threadIdx.x == 0) {
      sc->ticket_sweep = 0;
      sc->scale[cur ^ 1] = 1.0f;
      sc->cur = cur ^ 1;
      __threadfence();
    }
  }
}

template <int PH, int LPS, int PS>
void launch_ls_instance(const SweepArgs& a, cudaStream_t stream) {
  const int spw = 32 / LPS;
  const int64_t warps = (2 * a.num_tracks + spw - 1) / spw;
  const int wpb = kSweepThreads / 32;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  const size_t smem = sizeof(float) * (size_t) a.num_materials * a.ld;
  if constexpr (PH == 1) {
    if (a.momz) {
      ls_sweep_kernel<1, LPS, PS, false, true>
          <<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a);
      return;
    }
  }
  auto kern = a.cm_cell ? ls_sweep_kernel<PH, LPS, PS, true>
                        : ls_sweep_kernel<PH, LPS, PS, false>;
  kern<<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a);
}

// The shared-memory limit of every instance dispatch_ls_lps can launch.
template <int PH, int LPS>
void configure_ls_lps(int optin) {
  if constexpr (PH == 1) {
    raise_smem_limit(ls_sweep_kernel<1, LPS, 1, false, true>, optin);
    raise_smem_limit(ls_sweep_kernel<1, LPS, 2, false, true>, optin);
    raise_smem_limit(ls_sweep_kernel<1, LPS, 3, false, true>, optin);
    raise_smem_limit(ls_sweep_kernel<1, LPS, 4, false, true>, optin);
    raise_smem_limit(ls_sweep_kernel<1, LPS, 5, false, true>, optin);
  }
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 1, true>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 2, true>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 3, true>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 4, true>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 5, true>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 1, false>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 2, false>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 3, false>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 4, false>, optin);
  raise_smem_limit(ls_sweep_kernel<PH, LPS, 5, false>, optin);
}

template <int PH>
void configure_ls(int optin) {
  configure_ls_lps<PH, 1>(optin);
  configure_ls_lps<PH, 2>(optin);
  configure_ls_lps<PH, 4>(optin);
  configure_ls_lps<PH, 8>(optin);
  configure_ls_lps<PH, 16>(optin);
  configure_ls_lps<PH, 32>(optin);
}

template <int PH, int LPS>
bool launch_ls_pairs(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (slots) {
    case 1: launch_ls_instance<PH, LPS, 1>(a, s); return true;
    case 2: launch_ls_instance<PH, LPS, 2>(a, s); return true;
    case 3: launch_ls_instance<PH, LPS, 3>(a, s); return true;
    case 4: launch_ls_instance<PH, LPS, 4>(a, s); return true;
    case 5: launch_ls_instance<PH, LPS, 5>(a, s); return true;
    default: return false;
  }
}

template <int PH>
bool dispatch_ls_lps(const SweepArgs& a, int slots, cudaStream_t s) {
  switch (a.lps) {
    case 1: return launch_ls_pairs<PH, 1>(a, slots, s);
    case 2: return launch_ls_pairs<PH, 2>(a, slots, s);
    case 4: return launch_ls_pairs<PH, 4>(a, slots, s);
    case 8: return launch_ls_pairs<PH, 8>(a, slots, s);
    case 16: return launch_ls_pairs<PH, 16>(a, slots, s);
    case 32: return launch_ls_pairs<PH, 32>(a, slots, s);
    default: return false;
  }
}

}  // namespace moc
