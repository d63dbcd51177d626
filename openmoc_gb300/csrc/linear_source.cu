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
// summed in FP64 (one warp per track, lanes over groups, FP64 atomics), then
// the 2x2 inverse per FSR, or zeros where the determinant is below 1e-10
// (the reference falls back to a flat source there).
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

// Series coefficients of G2 below: c_m = (m+1)/(m+2)! - 2(m+2)/(m+3)!,
// m = 1..23, filled once by the host.
__constant__ double c_g2_series[23];

// G2(x) = 2/3 - (1 + 2/x)(1/x + 1/2 - (1 + 1/x)(1 - exp(-x))/x), the
// quantity of the reference's expG2_fractional (src/exponentials.h:
// 283-323); below x = 1 from its series sum_{m>=1} c_m (-x)^m by Horner
// (the closed form cancels there), above from the closed form in FP64.
__device__ double ls_exp_g2(double x) {
  if (x < 1.0) {
    double s = c_g2_series[22];
    for (int m = 21; m >= 0; m--) s = fma(s, -x, c_g2_series[m]);
    return -x * s;
  }
  const double f1 = -expm1(-x) / x;
  return 2.0 / 3.0 - (1.0 + 2.0 / x) * (1.0 / x + 0.5 - (1.0 + 1.0 / x) * f1);
}

__global__ void ls_pack_kernel(const int2* segs, const float* x,
                               const float* y, int4* out, int64_t S) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int2 s = segs[i];
    out[i] = make_int4(s.x, s.y, __float_as_int(x[i]), __float_as_int(y[i]));
  }
}

// One warp per track; lane l takes groups l, l + 32, ...
__global__ void ls_moments_kernel(const int4* segs, const int64_t* seg_off,
                                  const int32_t* track_ang, int64_t T,
                                  const double* ang_dir, const double* ang_wgt,
                                  const double* pol_sin, const double* pol_wgt,
                                  int Ph, const float* sigma_t,
                                  const float* fsr_vol, int G, double* lem,
                                  double* acc) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t) gridDim.x * blockDim.x) >> 5;
  for (int64_t t = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       t < T; t += warps) {
    const int a = track_ang[t];
    const double cph = ang_dir[2 * a], sph = ang_dir[2 * a + 1];
    const double wgt = ang_wgt[a];
    for (int64_t k = seg_off[t]; k < seg_off[t + 1]; k++) {
      const int4 w = segs[k];
      const double len = (double) __int_as_float(w.x);
      const int fsr = w.y & 0xFFFFFF;
      const int mat = (int) ((unsigned) w.y >> 24);
      const double xc = (double) __int_as_float(w.z) + 0.5 * len * cph;
      const double yc = (double) __int_as_float(w.w) + 0.5 * len * sph;
      const double vol = (double) fsr_vol[fsr];
      const double vi = wgt * len / vol;
      const double src_constant = vi * len / 2.0;
      if (lane == 0) {
        const double l2 = len * len / 12.0;
        atomicAdd(lem + 3 * (int64_t) fsr + 0, vi * (xc * xc + cph * cph * l2));
        atomicAdd(lem + 3 * (int64_t) fsr + 1, vi * (yc * yc + sph * sph * l2));
        atomicAdd(lem + 3 * (int64_t) fsr + 2, vi * (xc * yc + sph * cph * l2));
      }
      const float* st = sigma_t + (int64_t) mat * G;
      double* out = acc + (int64_t) fsr * 3 * G;
      for (int g = lane; g < G; g += 32) {
        const double tau = len * (double) st[g];
        double k2 = 0.0;
        for (int p = 0; p < Ph; p++) {
          const double sn = pol_sin[a * Ph + p];
          k2 += ls_exp_g2(tau / sn) * 2.0 * pol_wgt[a * Ph + p] * sn;
        }
        k2 *= len * src_constant;
        atomicAdd(out + g, vi * xc * xc + cph * cph * k2);
        atomicAdd(out + G + g, vi * yc * yc + sph * sph * k2);
        atomicAdd(out + 2 * G + g, vi * xc * yc + sph * cph * k2);
      }
    }
  }
}

__global__ void ls_invert_kernel(const double* lem, const double* acc,
                                 int64_t R, int G, int ld, float* ilem,
                                 float* cst, unsigned int* num_flat) {
  for (int64_t r = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; r < R;
       r += (int64_t) gridDim.x * blockDim.x) {
    const double a = lem[3 * r], b = lem[3 * r + 1], c = lem[3 * r + 2];
    const double det = a * b - c * c;
    if (fabs(det) < kMinDet) {
      ilem[3 * r] = ilem[3 * r + 1] = ilem[3 * r + 2] = 0.0f;
      atomicAdd(num_flat, 1u);
    } else {
      ilem[3 * r] = (float) (b / det);
      ilem[3 * r + 1] = (float) (a / det);
      ilem[3 * r + 2] = (float) (-c / det);
    }
    for (int i = 0; i < 3; i++)
      for (int g = 0; g < ld; g++)
        cst[(r * 3 + i) * ld + g] =
            (g < G) ? (float) acc[(r * 3 + i) * G + g] : 0.0f;
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

// c_m for m = 1..23 (index m - 1)
static void upload_g2_series(cudaStream_t s) {
  double c[23];
  double f = 2.0;   // (m+2)!
  for (int m = 1; m <= 23; m++) {
    f *= (double) (m + 2);
    c[m - 1] = (double) (m + 1) / f - 2.0 * (double) (m + 2) / (f * (m + 3));
  }
  cudaMemcpyToSymbolAsync(c_g2_series, c, sizeof(c), 0,
                          cudaMemcpyHostToDevice, s);
}

void launch_ls_constants(const int4* segs_ls, const int64_t* seg_off,
                         const int32_t* track_ang, int64_t T,
                         const double* ang_dir, const double* ang_wgt,
                         const double* pol_sin, const double* pol_wgt,
                         int Ph, const float* sigma_t, const float* fsr_vol,
                         int64_t R, int G, int ld, double* lem, double* acc,
                         float* ilem, float* cst, unsigned int* num_flat,
                         cudaStream_t s) {
  cudaMemsetAsync(lem, 0, sizeof(double) * 3 * R, s);
  cudaMemsetAsync(acc, 0, sizeof(double) * 3 * R * G, s);
  cudaMemsetAsync(num_flat, 0, sizeof(unsigned int), s);
  upload_g2_series(s);
  ls_moments_kernel<<<(unsigned) grid_for(32 * T, 256), 256, 0, s>>>(
      segs_ls, seg_off, track_ang, T, ang_dir, ang_wgt, pol_sin, pol_wgt, Ph,
      sigma_t, fsr_vol, G, lem, acc);
  ls_invert_kernel<<<(unsigned) grid_for(R, 128), 128, 0, s>>>(
      lem, acc, R, G, ld, ilem, cst, num_flat);
}

}  // namespace moc
