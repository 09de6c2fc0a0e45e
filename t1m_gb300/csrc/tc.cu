// Tensor-core (tcgen05) kernels — placeholder until the kernels land.
#include <string>
#include "internal.h"
#include "t1m_capi.h"
namespace t1m {
namespace gb300 {
bool tc_supported(int, int, const HostPlan&) { return false; }
cudaError_t launch_tc(int, int, const GemmArgs&, const HostPlan&, cudaStream_t, int* kernels,
                      std::string* err) {
  *kernels = 0;
  *err = "tensor-core methods are not built";
  return cudaErrorNotSupported;
}
}  // namespace gb300
}  // namespace t1m
