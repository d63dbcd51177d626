// On-the-fly axial segmentation of extruded 3D tracks inside the sweep
// (OpenMOC's OTF_TRACKS idea, src/TraverseSegments.cpp:151-265 and
// :304-925, for the extruded-lattice laydown of moc_lattice_extrude):
// instead of reading a stored stream of explicit 3D segments, every 3D
// track keeps a 32-byte descriptor -- the radial track it runs over, the
// range [0, A] of its traversal along that radial track (after the start
// a0), its height above the cut plane at the start (w0), and the direction
// of traversal -- and the sweep cuts the radial segments under it at the
// cut plane as it goes:
//
//   radial segment [s, s + l] (traversal coordinate relative to a0), clipped
//   to [0, A]; heights w = w0 + u cot(theta) at both ends; one piece of 3D
//   length (u_e - u_s) / sin(theta) in the radial FSR (w <= 0 throughout) or
//   in the region above the cut (w >= 0), else two pieces split at
//   u_c = u_s - w_s / cot(theta).
//
// The explicit generator (moc_lattice_extrude) makes the same pieces and
// additionally merges consecutive pieces of one region (above the cut, the
// radial segments of one 3D track all fall into the one region): the
// on-the-fly sweep integrates them one by one, which is the same
// attenuation up to rounding.  The 3D storage drops from 8 bytes per 3D
// segment to 32 bytes per 3D track plus the radial segments (read from L2).
//
// Decomposition as in the explicit sweep (sweep_kernel.cuh): one stream per
// track direction, LPS lanes over group pairs (PS per lane), one polar
// value; lane k of a stream cuts radial segment k of a chunk of LPS and the
// pieces reach the other lanes by shuffles; sources and tallies of the
// region above the cut (crossed by most tracks) are tallied in shared memory.
#include "sweep_kernel.cuh"

namespace moc {

namespace {

struct Piece2 {
  int n;          // pieces from this radial segment (0, 1 or 2)
  float l0, l1;   // 3D lengths in stream order
  int w0, w1;     // fsr | material << 24
};

// Blocks per SM: 6 (up to 85 registers); MOC_OTF_MIN_BLOCKS for the
// one-pair instances, whose sweeps wait on loads: 3D 17x17 assembly,
// 7 groups, 4 lanes x 1 pair, 6 blocks (69 registers) 3.767 ms per sweep,
// 8 blocks (61 registers) 3.257 ms; 10 spills 52 bytes.
#ifndef MOC_OTF_MIN_BLOCKS
#define MOC_OTF_MIN_BLOCKS 8
#endif
template <int LPS, int PS>
__global__ void __launch_bounds__(kSweepThreads,
                                  (PS == 1 ? MOC_OTF_MIN_BLOCKS : 6))
otf_sweep_kernel(const SweepArgs a, const OtfArgs o) {
  extern __shared__ float smem[];
  DevScalars* sc = a.sc;
  if (a.check_done && *(volatile int*) &sc->done) return;
  const int G = a.num_groups;
  const int ld = a.ld;
  float* s_st = smem;                          // [M][ld]
  float* s_hot = s_st + a.num_materials * ld;  // [ld] region above the cut
  for (int i = threadIdx.x; i < a.num_materials * ld; i += blockDim.x) {
    const int m = i / ld, g = i - m * ld;
    s_st[i] = (g < G) ? a.sigma_t[m * G + g] : 1.0f;
  }
  for (int i = threadIdx.x; i < ld; i += blockDim.x) s_hot[i] = 0.0f;
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
  const int npairs = ld >> 1;

  if (stream < 2 * a.num_tracks) {
    const int t = a.order[stream >> 1];
    const int dir = (int) (stream & 1);
    const int4 td = o.trk[t];       // radial track, first segment, count, reversed
    const float4 tf = o.trk_f[t];   // a0, span A, w0
    const int ang = a.track_ang[t];
    const float4 af = o.ang[ang];   // cot, 1 / cot, 1 / sin
    const int t2 = td.x, first = td.y, nrad = td.z, rev = td.w;
    const int64_t rb = o.rad_off[t2];
    const float L2 = o.rad_total[t2];
    const float2 w2 = f2(a.weights[ang]);
    const float2 xl2 = f2(-1.4426950408889634f);

    float2 psi[PS];
    const float* pin = psi_in + ((int64_t) t * 2 + dir) * G;
#pragma unroll
    for (int s = 0; s < PS; s++) {
      const int g0 = 2 * (sub + s * LPS);
      psi[s].x = (g0 < G) ? pin[g0] * scale : 0.0f;
      psi[s].y = (g0 + 1 < G) ? pin[g0 + 1] * scale : 0.0f;
    }
    const unsigned gmask =
        (LPS == 32) ? 0xffffffffu
                    : (((1u << LPS) - 1u) << (lane & ~(LPS - 1)));

    // pieces of the radial segment at stream position k (in stream order)
    auto cut = [&](int k) -> Piece2 {
      Piece2 p{0, 0.f, 0.f, 0, 0};
      if (k >= nrad) return p;
      const int kt = dir ? nrad - 1 - k : k;          // traversal position
      const int idx = rev ? first - kt : first + kt;  // natural index
      const int2 w = __ldg(o.rad_segs + rb + idx);
      const float l = __int_as_float(w.x);
      const float c0 = __ldg(o.rad_start + rb + idx);
      const float s = rev ? (L2 - c0 - l) - tf.x : c0 - tf.x;
      const float us = fmaxf(s, 0.0f), ue = fminf(s + l, tf.y);
      if (!(ue > us)) return p;
      const float ws = fmaf(us, af.x, tf.z), we = fmaf(ue, af.x, tf.z);
      const int below = w.y, above = o.above;
      if (fmaxf(ws, we) <= 0.0f || fminf(ws, we) >= 0.0f) {
        p.n = 1;
        p.l0 = (ue - us) * af.z;
        p.w0 = (fmaxf(ws, we) <= 0.0f) ? below : above;
      } else {
        const float uc = fmaf(-ws, af.y, us);
        const float la = (uc - us) * af.z, lb = (ue - uc) * af.z;
        const int ra = (ws < 0.0f) ? below : above;
        const int rbw = (ws < 0.0f) ? above : below;
        p.n = 2;
        // stream order: traversal order forward, reversed backward
        p.l0 = dir ? lb : la;
        p.l1 = dir ? la : lb;
        p.w0 = dir ? rbw : ra;
        p.w1 = dir ? ra : rbw;
      }
      return p;
    };

    // one piece with its sources already loaded
    auto integrate = [&](float len, int word, const float2* qv) {
      const int fsr = word & 0xFFFFFF;
      const int mat = (int) ((unsigned) word >> 24);
      const float2* st = reinterpret_cast<const float2*>(s_st + mat * ld) + sub;
      const bool hot = fsr == o.above_fsr;
      const float2 len2 = f2(len);
#pragma unroll
      for (int s = 0; s < PS; s++) {
        if (sub + s * LPS < npairs) {
          const float2 tau = __fmul2_rn(st[s * LPS], len2);
          const float2 gx =
              AttenIntrinsic::eval2(__fmul2_rn(tau, xl2));
          const float2 d =
              __fmul2_rn(__ffma2_rn(qv[s], f2(-1.0f), psi[s]), gx);
          psi[s] = __ffma2_rn(d, f2(-1.0f), psi[s]);
          const float2 tally = __fmul2_rn(w2, d);
          if (hot) {
            float* hp = s_hot + 2 * (sub + s * LPS);
            atomicAdd(hp, tally.x);
            atomicAdd(hp + 1, tally.y);
          } else {
            atomicAdd(reinterpret_cast<float2*>(a.phi + (int64_t) fsr * ld) +
                          sub + s * LPS,
                      tally);
          }
        }
      }
    };
    auto load_q = [&](int word, float2* qv) {
      const float2* qrow = reinterpret_cast<const float2*>(
                               a.qt + (int64_t) (word & 0xFFFFFF) * ld) + sub;
#pragma unroll
      for (int s = 0; s < PS; s++)
        qv[s] = (sub + s * LPS < npairs) ? __ldg(qrow + s * LPS) : f2(0.0f);
    };

    // Pieces of a chunk of LPS radial segments reach every lane of the
    // stream by shuffles; where the registers allow (LPS x PS <= 4) the
    // sources of all of a chunk's pieces are loaded before the first is
    // integrated, else those of each radial segment's pieces.
    constexpr bool kBatched = LPS * PS <= 4;
    constexpr int kBatch = kBatched ? 2 * LPS : 1;
    Piece2 mine = cut(sub);
    for (int cb = 0; cb < nrad; cb += LPS) {
      const Piece2 nxt = cut(cb + LPS + sub);   // the next chunk, ahead
      const int m = min(LPS, nrad - cb);
      if constexpr (kBatched) {
        float pl[kBatch];
        int pw[kBatch];
        float2 pq[kBatch][PS];
        int np = 0;
#pragma unroll
        for (int j = 0; j < LPS; j++) {
          if (j < m) {
            const int n = __shfl_sync(gmask, mine.n, j, LPS);
            const float l0 = __shfl_sync(gmask, mine.l0, j, LPS);
            const int w0 = __shfl_sync(gmask, mine.w0, j, LPS);
            const float l1 = __shfl_sync(gmask, mine.l1, j, LPS);
            const int w1 = __shfl_sync(gmask, mine.w1, j, LPS);
            pl[2 * j] = l0;
            pw[2 * j] = (n > 0) ? w0 : -1;
            pl[2 * j + 1] = l1;
            pw[2 * j + 1] = (n > 1) ? w1 : -1;
          } else {
            pw[2 * j] = pw[2 * j + 1] = -1;
            pl[2 * j] = pl[2 * j + 1] = 0.0f;
          }
        }
#pragma unroll
        for (int i = 0; i < kBatch; i++)
          if (pw[i] >= 0) load_q(pw[i], pq[i]);
#pragma unroll
        for (int i = 0; i < kBatch; i++)
          if (pw[i] >= 0) integrate(pl[i], pw[i], pq[i]);
        (void) np;
      } else {
        for (int j = 0; j < m; j++) {
          const int n = __shfl_sync(gmask, mine.n, j, LPS);
          const float l0 = __shfl_sync(gmask, mine.l0, j, LPS);
          const int w0 = __shfl_sync(gmask, mine.w0, j, LPS);
          const float l1 = __shfl_sync(gmask, mine.l1, j, LPS);
          const int w1 = __shfl_sync(gmask, mine.w1, j, LPS);
          float2 q0[PS], q1[PS];
          if (n > 0) load_q(w0, q0);
          if (n > 1) load_q(w1, q1);
          if (n > 0) integrate(l0, w0, q0);
          if (n > 1) integrate(l1, w1, q1);
        }
      }
      mine = nxt;
    }

    // boundary-flux transfer (CPUSolver::transferBoundaryFlux)
    const int f = a.flags[t];
    if (f & (dir ? 8 : 4)) {
      const int nt = a.next[2 * t + dir];
      const int nd = (f & (dir ? 2 : 1)) ? 0 : 1;
      float* po = psi_out + ((int64_t) nt * 2 + nd) * G;
#pragma unroll
      for (int s = 0; s < PS; s++) {
        const int g0 = 2 * (sub + s * LPS);
        if (g0 < G) po[g0] = psi[s].x;
        if (g0 + 1 < G) po[g0 + 1] = psi[s].y;
      }
    }
  }

  __shared__ int last;
  __syncthreads();
  for (int i = threadIdx.x; i < G; i += blockDim.x) {
    const float v = s_hot[i];
    if (v != 0.0f) atomicAdd(a.phi + (int64_t) o.above_fsr * ld + i, v);
  }
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

template <int LPS, int PS>
void launch_otf_instance(const SweepArgs& a, const OtfArgs& o,
                         cudaStream_t stream) {
  const int spw = 32 / LPS;
  const int64_t warps = (2 * a.num_tracks + spw - 1) / spw;
  const int wpb = kSweepThreads / 32;
  const int64_t blocks = (warps + wpb - 1) / wpb;
  const size_t smem = sizeof(float) * (size_t) (a.num_materials + 1) * a.ld;
  auto kern = otf_sweep_kernel<LPS, PS>;
  kern<<<(unsigned) blocks, kSweepThreads, smem, stream>>>(a, o);
}

template <int LPS>
void configure_otf_lps(int optin) {
  raise_smem_limit(otf_sweep_kernel<LPS, 1>, optin);
  raise_smem_limit(otf_sweep_kernel<LPS, 2>, optin);
  raise_smem_limit(otf_sweep_kernel<LPS, 3>, optin);
  raise_smem_limit(otf_sweep_kernel<LPS, 4>, optin);
}

template <int LPS>
bool launch_otf_pairs(const SweepArgs& a, const OtfArgs& o, int slots,
                      cudaStream_t s) {
  switch (slots) {
    case 1: launch_otf_instance<LPS, 1>(a, o, s); return true;
    case 2: launch_otf_instance<LPS, 2>(a, o, s); return true;
    case 3: launch_otf_instance<LPS, 3>(a, o, s); return true;
    case 4: launch_otf_instance<LPS, 4>(a, o, s); return true;
    default: return false;
  }
}

}  // namespace

void configure_otf_sweeps(int optin) {
  configure_otf_lps<1>(optin);
  configure_otf_lps<2>(optin);
  configure_otf_lps<4>(optin);
  configure_otf_lps<8>(optin);
  configure_otf_lps<16>(optin);
  configure_otf_lps<32>(optin);
}

bool launch_otf_sweep(const SweepArgs& a, const OtfArgs& o, int slots,
                      cudaStream_t s) {
  switch (a.lps) {
    case 1: return launch_otf_pairs<1>(a, o, slots, s);
    case 2: return launch_otf_pairs<2>(a, o, slots, s);
    case 4: return launch_otf_pairs<4>(a, o, slots, s);
    case 8: return launch_otf_pairs<8>(a, o, slots, s);
    case 16: return launch_otf_pairs<16>(a, o, slots, s);
    case 32: return launch_otf_pairs<32>(a, o, slots, s);
    default: return false;
  }
}

}  // namespace moc
