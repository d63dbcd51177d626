// Sweep kernel instances for 2 polar value(s) per track direction with
// the hardware ex2 exponential (see sweep_kernel.cuh).
#include "sweep_kernel.cuh"

namespace moc {

bool launch_sweep_p2_e1(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_sweep_lps<2, 1>(a, slots, s);
}

void configure_sweep_p2_e1(int optin) { configure_sweep<2, 1>(optin); }

}  // namespace moc
