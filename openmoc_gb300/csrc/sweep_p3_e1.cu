// Sweep kernel instances for 3 polar value(s) per track direction with
// the hardware ex2 exponential (see sweep_kernel.cuh).
#include "sweep_kernel.cuh"

namespace moc {

bool launch_sweep_p3_e1(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_sweep_lps<3, 1>(a, slots, s);
}

void configure_sweep_p3_e1(int optin) { configure_sweep<3, 1>(optin); }

// g(x) = 1 - exp(-x) for an array of x with the sweep's own evaluators
// (ExpEvaluator::computeExponential, src/ExpEvaluator.h:170-183).
__global__ void attenuation_kernel(int kind, const float* x, float* g,
                                   int64_t n, const float* exp_table) {
  __shared__ float2 tab[kExpTableSize];
  for (int i = threadIdx.x; i < kExpTableSize; i += blockDim.x)
    tab[i] = make_float2(exp_table[i], exp_table[kExpTableSize + i]);
  __syncthreads();
  for (int64_t i = 2 * ((int64_t) blockIdx.x * blockDim.x + threadIdx.x);
       i < n; i += 2 * (int64_t) gridDim.x * blockDim.x) {
    const float2 x2 = make_float2(x[i], (i + 1 < n) ? x[i + 1] : 0.0f);
    float2 r;
    if (kind == kExpTable)
      r = AttenTable::eval2(__fmul2_rn(x2, f2(kExpTableInvH)), tab);
    else
      r = AttenIntrinsic::eval2(__fmul2_rn(x2, f2(-1.4426950408889634f)));
    g[i] = r.x;
    if (i + 1 < n) g[i + 1] = r.y;
  }
}

void launch_attenuation(int kind, const float* x, float* g, int64_t n,
                        const float* exp_table, cudaStream_t s) {
  int64_t blocks = (n / 2 + 255) / 256 + 1;
  if (blocks > 1024) blocks = 1024;
  attenuation_kernel<<<(unsigned) blocks, 256, 0, s>>>(kind, x, g, n,
                                                       exp_table);
}

}  // namespace moc
