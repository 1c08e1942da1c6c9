// Traversal kernels for layout 3 (see trace_impl.cuh).
#include "trace_impl.cuh"

namespace hrt
{
cudaError_t trace_l3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  return trace_layout<3, 0>(a, kind, counting, c, numSMs, s);
}
}  // namespace hrt
