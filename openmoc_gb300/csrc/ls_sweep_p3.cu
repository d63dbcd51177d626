// Linear-source sweep instances for 3 polar value(s) per track direction
// (see ls_sweep_kernel.cuh).
#include "ls_sweep_kernel.cuh"

namespace moc {

bool launch_ls_sweep_p3(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_ls_lps<3>(a, slots, s);
}

void configure_ls_p3(int optin) { configure_ls<3>(optin); }

}  // namespace moc
