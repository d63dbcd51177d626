// Dispatch of the transport sweep instances (sweep_kernel.cuh, instantiated
// in sweep_p<Ph>_e<exp>.cu) and the segment material packing kernel.
#include "moc_internal.cuh"

namespace moc {

bool launch_sweep_p1_e0(const SweepArgs&, int, cudaStream_t);
bool launch_sweep_p1_e1(const SweepArgs&, int, cudaStream_t);
bool launch_sweep_p2_e0(const SweepArgs&, int, cudaStream_t);
bool launch_sweep_p2_e1(const SweepArgs&, int, cudaStream_t);
bool launch_sweep_p3_e0(const SweepArgs&, int, cudaStream_t);
bool launch_sweep_p3_e1(const SweepArgs&, int, cudaStream_t);
void configure_sweep_p1_e0(int);
void configure_sweep_p1_e1(int);
void configure_sweep_p2_e0(int);
void configure_sweep_p2_e1(int);
void configure_sweep_p3_e0(int);
void configure_sweep_p3_e1(int);
void configure_ls_p1(int);
void configure_ls_p2(int);
void configure_ls_p3(int);

void configure_sweeps(int optin) {
  configure_sweep_p1_e0(optin);
  configure_sweep_p1_e1(optin);
  configure_sweep_p2_e0(optin);
  configure_sweep_p2_e1(optin);
  configure_sweep_p3_e0(optin);
  configure_sweep_p3_e1(optin);
}

void configure_ls_sweeps(int optin) {
  configure_ls_p1(optin);
  configure_ls_p2(optin);
  configure_ls_p3(optin);
}

__global__ void pack_materials_kernel(int2* segs, int64_t n,
                                      const int32_t* fsr_mat) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int fsr = segs[i].y & 0xFFFFFF;
    segs[i].y = fsr | (fsr_mat[fsr] << 24);
  }
}

// Packs (length, FSR id) pairs into segment words, checking each (FSR id in
// [0, R), length finite and non-negative): the first bad index goes to
// *bad.  Counts the segments of the last kMaxHotFsrs FSR ids (block
// counters in shared memory, one global add per block and counter).
__global__ void pack_segments_kernel(const float* len, const int32_t* fsr,
                                     int2* out, int64_t S, int64_t R,
                                     unsigned long long* bad,
                                     unsigned long long* tail) {
  __shared__ unsigned int cnt[kMaxHotFsrs];
  if (threadIdx.x < kMaxHotFsrs) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t tail0 = R - kMaxHotFsrs;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x) {
    const float l = len[i];
    const int32_t f = fsr[i];
    if (!(f >= 0 && f < R && isfinite(l) && l >= 0.0f))
      atomicMin(bad, (unsigned long long) i);
    out[i] = make_int2(__float_as_int(l), f);
    if (f >= tail0 && f < R) atomicAdd(&cnt[f - tail0], 1u);
  }
  __syncthreads();
  if (threadIdx.x < kMaxHotFsrs && cnt[threadIdx.x])
    atomicAdd(&tail[threadIdx.x], (unsigned long long) cnt[threadIdx.x]);
}

void launch_pack_segments(const float* len, const int32_t* fsr, int2* out,
                          int64_t S, int64_t R, unsigned long long* bad,
                          unsigned long long* tail, cudaStream_t stream) {
  if (S == 0) return;
  int64_t blocks = (S + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  pack_segments_kernel<<<(unsigned) blocks, 256, 0, stream>>>(len, fsr, out, S,
                                                              R, bad, tail);
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

bool sweep_lps_supported(int lps) {
  return lps == 1 || lps == 2 || lps == 4 || lps == 8 || lps == 16 ||
         lps == 32;
}

bool launch_sweep(const SweepArgs& a, int polar_half, int slots, int exp_kind,
                  cudaStream_t stream) {
  const bool tab = exp_kind != kExpIntrinsic;
  switch (polar_half) {
    case 1:
      return tab ? launch_sweep_p1_e0(a, slots, stream)
                 : launch_sweep_p1_e1(a, slots, stream);
    case 2:
      return tab ? launch_sweep_p2_e0(a, slots, stream)
                 : launch_sweep_p2_e1(a, slots, stream);
    case 3:
      return tab ? launch_sweep_p3_e0(a, slots, stream)
                 : launch_sweep_p3_e1(a, slots, stream);
    default:
      return false;
  }
}

}  // namespace moc
