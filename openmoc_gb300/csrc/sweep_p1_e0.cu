// Sweep kernel instances for 1 polar value(s) per track direction with
// the shared-memory table exponential (see sweep_kernel.cuh).
#include "sweep_kernel.cuh"

namespace moc {

bool launch_sweep_p1_e0(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_sweep_lps<1, 0>(a, slots, s);
}

void configure_sweep_p1_e0(int optin) { configure_sweep<1, 0>(optin); }

}  // namespace moc
