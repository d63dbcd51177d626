// Linear-source sweep instances for 1 polar value(s) per track direction
// (see ls_sweep_kernel.cuh).
#include "ls_sweep_kernel.cuh"

namespace moc {

bool launch_ls_sweep_p1(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_ls_lps<1>(a, slots, s);
}

void configure_ls_p1(int optin) { configure_ls<1>(optin); }

}  // namespace moc
