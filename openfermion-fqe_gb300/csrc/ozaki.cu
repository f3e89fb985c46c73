// Tensor-core (tcgen05) contraction with Ozaki splitting — placeholder until
// the kernel lands; the FP64 path is the reference-exact drop-in.
#include "ham.cuh"

namespace fqegpu {
struct OzakiPlan {};
void ozaki_destroy(fqegpu_ham h) {
  delete h->oz;
  h->oz = nullptr;
}
int apply_ozaki(fqegpu_ham, const double2*, double2*, double2, double2, cudaStream_t) {
  set_error("tensor-core contraction not built yet");
  return FQEGPU_ERR_UNSUPPORTED;
}
}  // namespace fqegpu
