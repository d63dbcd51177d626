// Linear-source sweep instances for 2 polar value(s) per track direction
// (see ls_sweep_kernel.cuh).
#include "ls_sweep_kernel.cuh"

namespace moc {

bool launch_ls_sweep_p2(const SweepArgs& a, int slots, cudaStream_t s) {
  return dispatch_ls_lps<2>(a, slots, s);
}

void configure_ls_p2(int optin) { configure_ls<2>(optin); }

}  // namespace moc
