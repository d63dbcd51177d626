// Linear-source set-up for sm_103a: the packed 16-byte segment words and the
// per-FSR linear expansion constants, and the dispatch of the linear-source
// sweep instances (ls_sweep_p<Ph>.cu).
//
// The constants restate LinearExpansionGenerator (2D,
// src/TrackTraversingAlgorithms.cpp:470-830): for every segment of length l
// in FSR r, with (x, y) its start relative to the FSR centroid, direction
// (cos phi, sin phi), midpoint (xc, yc) and azimuthal weight w_a,
//   lem[r]      += w_a l / V_r (xc^2 + (cos l)^2 / 12, yc^2 + (sin l)^2 / 12,
//                               xc yc + sin cos l^2 / 12)
//   const[r][g] += w_a l / V_r (xc^2, yc^2, xc yc)
//                + (cos^2, sin^2, sin cos) sum_p l G2(l sigma_t / sin_p)
//                  w_a l^2 / (2 V_r) 2 w_p sin_p,
// summed in FP64 by one warp per FSR over its own segments (bucketed by FSR
// first; lanes over groups, no atomics), then the 2x2 inverse per FSR, or
// zeros where the determinant is below 1e-10 (the reference falls back to a
// flat source there).
#include <vector>

#include "moc_internal.cuh"

namespace moc {

bool launch_ls_sweep_p1(const SweepArgs&, int, cudaStream_t);
bool launch_ls_sweep_p2(const SweepArgs&, int, cudaStream_t);
bool launch_ls_sweep_p3(const SweepArgs&, int, cudaStream_t);

bool launch_ls_sweep(const SweepArgs& a, int polar_half, int slots,
                     cudaStream_t stream) {
  switch (polar_half) {
    case 1: return launch_ls_sweep_p1(a, slots, stream);
    case 2: return launch_ls_sweep_p2(a, slots, stream);
    case 3: return launch_ls_sweep_p3(a, slots, stream);
    default: return false;
  }
}

namespace {

constexpr double kMinDet = 1e-10;   // src/constants.h:70

// G2(x) = 2/3 - (1 + 2/x)(1/x + 1/2 - (1 + 1/x)(1 - exp(-x))/x), the
// quantity of the reference's expG2_fractional (src/exponentials.h:
// 283-323), in FP32 by a rational x P5(x) / Q6(x) fitted here
// (csrc/fit_ls_exponential.py): P(0) = -1/12, the slope of G2 at 0, and
// p5 = q6 / 6 (G2 -> 1/6).  Evaluated in FP32: absolute error 3.3e-7,
// relative 2.9e-6 where |G2| > 1e-3 and 4.3e-7 below x = 0.01 (the
// reference's rational is quoted at 1e-6).
__device__ __forceinline__ float ls_exp_g2(float x) {
  constexpr float kP[6] = {-8.3333333333e-02f, 2.3162673964e-03f,
                           1.5046986351e-03f, 5.4518176798e-04f,
                           4.1676890852e-05f, 9.9593943274e-06f};
  constexpr float kQ[7] = {1.0000000000e+00f, 6.7217634287e-01f,
                           2.1929234424e-01f, 4.4564577781e-02f,
                           6.5545427501e-03f, 6.0865601323e-04f,
                           5.9756365965e-05f};
  float n = kP[5], d = kQ[6];
#pragma unroll
  for (int k = 4; k >= 0; k--) n = fmaf(n, x, kP[k]);
#pragma unroll
  for (int k = 5; k >= 0; k--) d = fmaf(d, x, kQ[k]);
  return x * n / d;
}

__global__ void ls_pack_kernel(const int2* segs, const float* x,
                               const float* y, int4* out, int64_t S) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int2 s = segs[i];
    out[i] = make_int4(s.x, s.y, __float_as_int(x[i]), __float_as_int(y[i]));
  }
}

// The track of every segment (one warp per track).
__global__ void ls_seg_track_kernel(const int64_t* seg_off, int64_t T,
                                    int32_t* seg_track) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t) gridDim.x * blockDim.x) >> 5;
  for (int64_t t = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       t < T; t += warps)
    for (int64_t k = seg_off[t] + lane; k < seg_off[t + 1]; k += 32)
      seg_track[k] = (int32_t) t;
}

// Segments per FSR.
__global__ void ls_count_kernel(const int4* segs, int64_t S, int64_t* count) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x)
    atomicAdd(reinterpret_cast<unsigned long long*>(count + (segs[i].y & 0xFFFFFF)),
              1ull);
}

// Segment ids bucketed by FSR (start[r] .. start[r + 1]); fill counts up.
__global__ void ls_bucket_kernel(const int4* segs, int64_t S,
                                 const int64_t* start, int64_t* fill,
                                 int32_t* list) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int r = segs[i].y & 0xFFFFFF;
    const unsigned long long pos =
        atomicAdd(reinterpret_cast<unsigned long long*>(fill + r), 1ull);
    list[start[r] + (int64_t) pos] = (int32_t) i;
  }
}

// The expansion moments and source constants, summed over each FSR's
// segments in FP64.  The segments are bucketed by FSR; warp w takes list
// entries [w * chunk, (w + 1) * chunk) -- equal shares of segments,
// whatever the FSRs' sizes (one region crossed by most tracks, as the
// moderator above a 3D assembly, would leave one warp walking millions of
// segments) -- with lanes over groups (S_ groups per lane, G <= 32 S_).  A
// warp sums its run of an FSR in registers and adds it to the FP64 totals
// lem[R][NC] and acc[R][NC][ld] with FP64 atomics where the FSR changes.
// NC = 3 in 2D (xx, yy, xy; the polar loop of the 2D branch), 6 on 3D
// tracks (xx, yy, xy, xz, yz, zz; the row's 3D direction and weight
// w_a d_a w_p d_p, G2 at the segment's own optical length).
template <int S_, bool D3>
__global__ void ls_moments_kernel(const int4* segs, const float* seg_z,
                                  const int32_t* list, int64_t S, int chunk,
                                  const int32_t* seg_track,
                                  const int32_t* track_ang,
                                  const double* ang_dir, const double* ang_wgt,
                                  const double* pol_sin, const double* pol_wgt,
                                  const double* pol_cos, int Ph,
                                  const float* sigma_t, const float* fsr_vol,
                                  const int32_t* fsr_mat, int G, int ld,
                                  double* lem, double* acc) {
  constexpr int NC = D3 ? 6 : 3;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t e0 = warp * chunk;
  if (e0 >= S) return;
  const int64_t e1 = (e0 + chunk < S) ? e0 + chunk : S;
  double l[NC], c[NC][S_];
  float st[S_];
  int cur = -1;
  double vol = 1.0;
  auto flush = [&]() {
    if (lane == 0)
      for (int i = 0; i < NC; i++) atomicAdd(lem + (int64_t) cur * NC + i, l[i]);
#pragma unroll
    for (int j = 0; j < S_; j++) {
      const int g = lane + 32 * j;
      if (g < G)
#pragma unroll
        for (int i = 0; i < NC; i++)
          atomicAdd(acc + ((int64_t) cur * NC + i) * ld + g, c[i][j]);
    }
  };
  for (int64_t e = e0; e < e1; e++) {
    const int k = list[e];
    const int4 w = segs[k];
    const int r = w.y & 0xFFFFFF;
    if (r != cur) {
      if (cur >= 0) flush();
      cur = r;
      vol = (double) fsr_vol[r];
      const int m = fsr_mat[r];
#pragma unroll
      for (int i = 0; i < NC; i++) {
        l[i] = 0.0;
#pragma unroll
        for (int j = 0; j < S_; j++) c[i][j] = 0.0;
      }
#pragma unroll
      for (int j = 0; j < S_; j++) {
        const int g = lane + 32 * j;
        st[j] = (g < G) ? sigma_t[(int64_t) m * G + g] : 0.0f;
      }
    }
    const int a = track_ang[seg_track[k]];
    const double cph = ang_dir[2 * a], sph = ang_dir[2 * a + 1];
    const float lenf = __int_as_float(w.x);
    const double len = (double) lenf;
    const double l12 = len * len / 12.0;
    if constexpr (D3) {
      const double sth = pol_sin[a], cth = pol_cos[a];
      const double wgt = ang_wgt[a] * pol_wgt[a];
      const double xc = (double) __int_as_float(w.z) + len * 0.5 * cph * sth;
      const double yc = (double) __int_as_float(w.w) + len * 0.5 * sph * sth;
      const double zc = (double) seg_z[k] + len * 0.5 * cth;
      const double vi = wgt * len / vol;
      const double half = vi * len / 2.0;
      l[0] += vi * (xc * xc + cph * cph * sth * sth * l12);
      l[1] += vi * (yc * yc + sph * sph * sth * sth * l12);
      l[2] += vi * (xc * yc + sph * cph * sth * sth * l12);
      l[3] += vi * (xc * zc + cph * cth * sth * l12);
      l[4] += vi * (yc * zc + sph * cth * sth * l12);
      l[5] += vi * (zc * zc + cth * cth * l12);
#pragma unroll
      for (int j = 0; j < S_; j++) {
        const double g2 = (double) ls_exp_g2(lenf * st[j]) * len * half;
        c[0][j] += vi * xc * xc + cph * cph * g2 * sth * sth;
        c[1][j] += vi * yc * yc + sph * sph * g2 * sth * sth;
        c[2][j] += vi * xc * yc + sph * cph * g2 * sth * sth;
        c[3][j] += vi * xc * zc + cph * cth * g2 * sth;
        c[4][j] += vi * yc * zc + sph * cth * g2 * sth;
        c[5][j] += vi * zc * zc + cth * cth * g2;
      }
    } else {
      const double xc = (double) __int_as_float(w.z) + 0.5 * len * cph;
      const double yc = (double) __int_as_float(w.w) + 0.5 * len * sph;
      const double vi = ang_wgt[a] * len / vol;
      l[0] += vi * (xc * xc + cph * cph * l12);
      l[1] += vi * (yc * yc + sph * sph * l12);
      l[2] += vi * (xc * yc + sph * cph * l12);
      // per group: sum_p l G2(l sigma_t / sin_p) (vi l / 2) 2 w_p sin_p
      const double k2f = len * vi * len / 2.0;
#pragma unroll
      for (int j = 0; j < S_; j++) {
        const float tau = lenf * st[j];
        float k2 = 0.0f;
        for (int p = 0; p < Ph; p++) {
          const float sn = (float) pol_sin[a * Ph + p];
          k2 = fmaf(ls_exp_g2(tau / sn), (float) (2.0 * pol_wgt[a * Ph + p]) * sn,
                    k2);
        }
        const double kk = k2f * (double) k2;
        c[0][j] += vi * xc * xc + cph * cph * kk;
        c[1][j] += vi * yc * yc + sph * sph * kk;
        c[2][j] += vi * xc * yc + sph * cph * kk;
      }
    }
  }
  if (cur >= 0) flush();
}

// The inverse expansion matrix of every FSR from its FP64 moments (2x2, or
// 3x3 on 3D tracks; zeros -- a flat source -- where the determinant is
// below 1e-10, or in 3D the volume below 1e-6), and the source constants
// rounded to FP32 (zero in the padding groups).
template <bool D3>
__global__ void ls_finish_kernel(const double* lem, const double* acc,
                                 const float* fsr_vol, int64_t R, int G,
                                 int ld, float* ilem, float* cst,
                                 unsigned int* num_flat) {
  constexpr int NC = D3 ? 6 : 3;
  const int64_t n = R * NC * ld;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int g = (int) (i % ld);
    cst[i] = (g < G) ? (float) acc[i] : 0.0f;
  }
  for (int64_t r = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; r < R;
       r += (int64_t) gridDim.x * blockDim.x) {
    const double* m = lem + r * NC;
    float* il = ilem + r * NC;
    if constexpr (D3) {
      const double det = m[0] * m[1] * m[5] + m[2] * m[4] * m[3] +
                         m[3] * m[2] * m[4] - m[0] * m[4] * m[4] -
                         m[3] * m[1] * m[3] - m[2] * m[2] * m[5];
      if (fabs(det) < kMinDet || (double) fsr_vol[r] < 1e-6) {
        for (int i = 0; i < 6; i++) il[i] = 0.0f;
        atomicAdd(num_flat, 1u);
      } else {
        il[0] = (float) ((m[1] * m[5] - m[4] * m[4]) / det);
        il[1] = (float) ((m[0] * m[5] - m[3] * m[3]) / det);
        il[2] = (float) ((m[3] * m[4] - m[2] * m[5]) / det);
        il[3] = (float) ((m[2] * m[4] - m[3] * m[1]) / det);
        il[4] = (float) ((m[3] * m[2] - m[0] * m[4]) / det);
        il[5] = (float) ((m[0] * m[1] - m[2] * m[2]) / det);
      }
    } else {
      const double det = m[0] * m[1] - m[2] * m[2];
      if (fabs(det) < kMinDet) {
        il[0] = il[1] = il[2] = 0.0f;
        atomicAdd(num_flat, 1u);
      } else {
        il[0] = (float) (m[1] / det);
        il[1] = (float) (m[0] / det);
        il[2] = (float) (-m[2] / det);
      }
    }
  }
}

__global__ void ls_refresh_kernel(const int2* segs, int4* out, int64_t S) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x)
    out[i].y = segs[i].y;
}

int64_t grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return b;
}

}  // namespace

void launch_ls_pack_segments(const int2* segs, const float* x, const float* y,
                             int4* out, int64_t S, cudaStream_t s) {
  if (S == 0) return;
  ls_pack_kernel<<<(unsigned) grid_for(S, 256), 256, 0, s>>>(segs, x, y, out,
                                                             S);
}

void launch_ls_refresh_ids(const int2* segs, int4* out, int64_t S,
                           cudaStream_t s) {
  if (S == 0) return;
  ls_refresh_kernel<<<(unsigned) grid_for(S, 256), 256, 0, s>>>(segs, out, S);
}

void launch_ls_seg_track(const int64_t* seg_off, int64_t T, int32_t* seg_track,
                         cudaStream_t s) {
  if (T == 0) return;
  ls_seg_track_kernel<<<(unsigned) grid_for(32 * T, 256), 256, 0, s>>>(
      seg_off, T, seg_track);
}

int64_t ls_constants_scratch(int64_t R, int ld, bool d3) {
  const int64_t nc = d3 ? 6 : 3;
  return R * nc * (1 + (int64_t) ld);
}

void launch_ls_constants_bucketed(const int4* segs_ls, const int32_t* list,
                                  int64_t S, const int32_t* seg_track,
                                  const int32_t* track_ang,
                                  const double* ang_dir, const double* ang_wgt,
                                  const double* pol_sin, const double* pol_wgt,
                                  int Ph, const float* sigma_t,
                                  const float* fsr_vol, const int32_t* fsr_mat,
                                  int64_t R, int G, int ld, float* ilem,
                                  float* cst, unsigned int* num_flat,
                                  double* scratch, cudaStream_t s,
                                  const float* seg_z, const double* pol_cos) {
  const bool d3 = seg_z != nullptr;
  const int64_t nc = d3 ? 6 : 3;
  double* lem = scratch;
  double* acc = scratch + R * nc;
  cudaMemsetAsync(scratch, 0, sizeof(double) * ls_constants_scratch(R, ld, d3),
                  s);
  // about 48 warps per SM, at least 32 segments each
  int64_t chunk = (S + 152 * 48 - 1) / (152 * 48);
  if (chunk < 32) chunk = 32;
  const int64_t warps = (S + chunk - 1) / chunk;
  if (warps > 0) {
    const unsigned blocks = (unsigned) ((warps * 32 + 255) / 256);
#define MOC_LS_MOM(SS, D)                                                     \
  ls_moments_kernel<SS, D><<<blocks, 256, 0, s>>>(                            \
      segs_ls, seg_z, list, S, (int) chunk, seg_track, track_ang, ang_dir,    \
      ang_wgt, pol_sin, pol_wgt, pol_cos, Ph, sigma_t, fsr_vol, fsr_mat, G,   \
      ld, lem, acc)
#define MOC_LS_MOM_S(D)                   \
    switch ((ld + 31) / 32) {             \
      case 1: MOC_LS_MOM(1, D); break;    \
      case 2: MOC_LS_MOM(2, D); break;    \
      case 3: MOC_LS_MOM(3, D); break;    \
      case 4: MOC_LS_MOM(4, D); break;    \
      default: MOC_LS_MOM(8, D); break;   \
    }
    if (d3) {
      MOC_LS_MOM_S(true)
    } else {
      MOC_LS_MOM_S(false)
    }
#undef MOC_LS_MOM_S
#undef MOC_LS_MOM
  }
  const unsigned fb = (unsigned) grid_for(R * nc * ld, 256);
  if (d3)
    ls_finish_kernel<true><<<fb, 256, 0, s>>>(lem, acc, fsr_vol, R, G, ld,
                                             ilem, cst, num_flat);
  else
    ls_finish_kernel<false><<<fb, 256, 0, s>>>(lem, acc, fsr_vol, R, G, ld,
                                              ilem, cst, num_flat);
}

int launch_ls_constants(const int4* segs_ls, const int64_t* seg_off,
                        const int32_t* track_ang, int64_t T, int64_t S,
                        const double* ang_dir, const double* ang_wgt,
                        const double* pol_sin, const double* pol_wgt, int Ph,
                        const float* sigma_t, const float* fsr_vol,
                        const int32_t* fsr_mat, int64_t R, int G, int ld,
                        float* ilem, float* cst, unsigned int* num_flat,
                        cudaStream_t s, const float* seg_z,
                        const double* pol_cos) {
  // segment buckets by FSR: counts, exclusive scan on the host, scatter
  int64_t* count = nullptr;
  int64_t* startp = nullptr;
  int32_t* list = nullptr;
  int32_t* seg_track = nullptr;
  double* scratch = nullptr;
  cudaError_t e = cudaMalloc(&count, sizeof(int64_t) * (R + 1));
  if (e == cudaSuccess) e = cudaMalloc(&startp, sizeof(int64_t) * (R + 1));
  if (e == cudaSuccess) e = cudaMalloc(&list, sizeof(int32_t) * (S > 0 ? S : 1));
  if (e == cudaSuccess)
    e = cudaMalloc(&seg_track, sizeof(int32_t) * (S > 0 ? S : 1));
  if (e == cudaSuccess)
    e = cudaMalloc(&scratch,
                   sizeof(double) * ls_constants_scratch(R, ld, seg_z != nullptr));
  std::vector<int64_t> h((size_t) R + 1, 0);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(count, 0, sizeof(int64_t) * (R + 1), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(num_flat, 0, sizeof(unsigned), s);
  if (e == cudaSuccess && S > 0) {
    ls_count_kernel<<<(unsigned) grid_for(S, 256), 256, 0, s>>>(segs_ls, S,
                                                               count);
    ls_seg_track_kernel<<<(unsigned) grid_for(32 * T, 256), 256, 0, s>>>(
        seg_off, T, seg_track);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), count, sizeof(int64_t) * R,
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) {
    int64_t run = 0;
    for (int64_t r = 0; r < R; r++) {
      const int64_t c = h[r];
      h[r] = run;
      run += c;
    }
    h[R] = run;
    e = cudaMemcpyAsync(startp, h.data(), sizeof(int64_t) * (R + 1),
                        cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess)
    e = cudaMemsetAsync(count, 0, sizeof(int64_t) * (R + 1), s);
  if (e == cudaSuccess && S > 0) {
    ls_bucket_kernel<<<(unsigned) grid_for(S, 256), 256, 0, s>>>(
        segs_ls, S, startp, count, list);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    launch_ls_constants_bucketed(segs_ls, list, S, seg_track, track_ang,
                                 ang_dir, ang_wgt, pol_sin, pol_wgt, Ph,
                                 sigma_t, fsr_vol, fsr_mat, R, G, ld, ilem, cst,
                                 num_flat, scratch, s, seg_z, pol_cos);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(count);
  cudaFree(startp);
  cudaFree(list);
  cudaFree(seg_track);
  cudaFree(scratch);
  return e == cudaSuccess ? 0 : (int) e;
}

}  // namespace moc
