// Total volume-integrated nu-fission source without any device allocation.
//
// moc_fission_source_total_noalloc computes the quantity that keff and the
// flux normalisation are built from, sum over FSRs r and groups g of
// V_r * nuSigma_f[m(r), g] * phi[r, g], for callers that hand in device
// arrays but cannot allocate device memory themselves: code whose device
// memory is owned by a pool or caching allocator of another framework (the
// free memory the driver reports may be zero while the pool holds it all),
// and code on a latency-critical path, where cudaMalloc's implicit
// synchronisation of the device is not acceptable.
//
// Its per-FSR scratch lives in g_noalloc_rates, a file-scope __device__
// array of MOC_NOALLOC_MAX_FSRS doubles (4 MiB) that every GPU loading the
// library holds until the process exits.  Host code cannot use the symbol's
// name as a device address: the first call in each CUDA context (on each
// device, and again after a cudaDeviceReset or under another driver-API
// context), with that device current, looks its address up once with
// cudaGetSymbolAddress.  The address belongs to the context, so the cache is
// keyed by the current context (cuCtxGetCurrent, reached through the
// runtime's driver entry point so the library needs no libcuda link).
//
// The sum is deterministic (a per-FSR pass, then one block summing the FSR
// values in a fixed order), like OpenMOC's pairwise sum over its per-FSR
// scratch (src/CPUSolver.cpp:1860-1908), unlike the atomic reductions of
// the solver's own kernels.
#include <cuda.h>

#include <mutex>

#include "../../include/openmoc_gb300.h"
#include "moc_internal.cuh"

namespace {

constexpr int64_t kMaxFsrs = MOC_NOALLOC_MAX_FSRS;
constexpr int kMaxDevices = 64;
constexpr int kSumThreads = 1024;

// Every call reuses this array and leaves its values behind; each call
// writes every element it reads before reading it.
__device__ __align__(256) double g_noalloc_rates[kMaxFsrs];

std::mutex g_symbol_mu;
struct SymbolCache {
  CUcontext ctx;
  double* addr;
};
SymbolCache g_symbol[kMaxDevices] = {};
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn g_ctx_get_current = nullptr;

// One warp per FSR: rates[r] = V_r * sum_g nuSigma_f * phi (FP64 sum).
// An FSR whose material id lies outside [0, M) reads nothing and gets a
// NaN rate, which makes the total NaN.
__global__ void noalloc_fsr_rates_kernel(const float* phi, int64_t ld,
                                         const float* nu_sigma_f, int M,
                                         const int32_t* fsr_mat,
                                         const float* fsr_vol, int64_t R,
                                         int G, double* rates) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t) gridDim.x * blockDim.x) >> 5;
  for (int64_t r = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       r < R; r += warps) {
    const int32_t m = fsr_mat[r];
    if (m < 0 || m >= M) {
      if (lane == 0) rates[r] = __longlong_as_double(0x7ff8000000000000LL);
      continue;
    }
    const float* nf = nu_sigma_f + (int64_t) m * G;
    const float* row = phi + r * ld;
    double s = 0.0;
    for (int g = lane; g < G; g += 32) s += (double) nf[g] * (double) row[g];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) rates[r] = s * (double) fsr_vol[r];
  }
}

// One block: each thread sums a strided subset in order, then a tree.
__global__ void noalloc_sum_kernel(const double* rates, int64_t R,
                                   double* total) {
  __shared__ double part[kSumThreads];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < R; i += blockDim.x) s += rates[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int) threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = part[0];
}

bool is_device_pointer(const void* p, int dev) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (attr.type == cudaMemoryTypeDevice ||
          attr.type == cudaMemoryTypeManaged) &&
         attr.device == dev;
}

// The scratch array's address in the current context of device `dev`.
int scratch_address(int dev, double** out) {
  std::lock_guard<std::mutex> lk(g_symbol_mu);
  if (!g_ctx_get_current) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion(
        "cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return moc::set_error(MOC_ERR_CUDA, "cuCtxGetCurrent is unavailable");
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
    return moc::set_error(MOC_ERR_CUDA, "no current CUDA context");
  SymbolCache& c = g_symbol[dev];
  if (c.ctx != ctx || !c.addr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_rates);
    if (e != cudaSuccess)
      return moc::set_error(MOC_ERR_CUDA, cudaGetErrorString(e));
    c.ctx = ctx;
    c.addr = static_cast<double*>(p);
  }
  *out = c.addr;
  return MOC_OK;
}

}  // namespace

extern "C" int moc_fission_source_total_noalloc(
    const float* phi, int64_t ld, const float* nu_sigma_f,
    int32_t num_materials, const int32_t* fsr_mat, const float* fsr_vol,
    int64_t num_fsrs, int32_t num_groups, void* stream, double* total) {
  if (!phi || !nu_sigma_f || !fsr_mat || !fsr_vol || !total)
    return moc::set_error(MOC_ERR_ARG, "null argument");
  if (num_materials < 1)
    return moc::set_error(MOC_ERR_ARG, "num_materials must be >= 1");
  if (num_fsrs < 1 || num_fsrs > kMaxFsrs)
    return moc::set_error(
        MOC_ERR_ARG,
        "num_fsrs must be in [1, 524288]: the no-allocation entry point's "
        "scratch holds MOC_NOALLOC_MAX_FSRS per-FSR values");
  if (num_groups < 1 || ld < num_groups)
    return moc::set_error(MOC_ERR_ARG,
                          "num_groups must be >= 1 and ld >= num_groups");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return moc::set_error(MOC_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return moc::set_error(MOC_ERR_UNSUPPORTED, "device ordinal out of range");
  if (!is_device_pointer(phi, dev) || !is_device_pointer(nu_sigma_f, dev) ||
      !is_device_pointer(fsr_mat, dev) || !is_device_pointer(fsr_vol, dev) ||
      !is_device_pointer(total, dev))
    return moc::set_error(MOC_ERR_ARG,
                          "every array must be device memory of the "
                          "current device");
  double* scratch = nullptr;
  const int rc = scratch_address(dev, &scratch);
  if (rc != MOC_OK) return rc;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return moc::set_error(MOC_ERR_CUDA, cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // 8 FSRs (warps) per block, at most 8 resident blocks per SM of this GPU
  int64_t blocks = (num_fsrs + 7) / 8;
  if (blocks > (int64_t) sms * 8) blocks = (int64_t) sms * 8;
  noalloc_fsr_rates_kernel<<<(unsigned) blocks, 256, 0, s>>>(
      phi, ld, nu_sigma_f, num_materials, fsr_mat, fsr_vol, num_fsrs,
      num_groups, scratch);
  noalloc_sum_kernel<<<1, kSumThreads, 0, s>>>(scratch, num_fsrs, total);
  e = cudaGetLastError();
  if (e != cudaSuccess) return moc::set_error(MOC_ERR_CUDA, cudaGetErrorString(e));
  return MOC_OK;
}
