// Traversal kernels for layout 0 with the watertight triangle test (see trace_impl.cuh).
#include "trace_impl.cuh"

namespace hrt
{
cudaError_t trace_w0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  return trace_layout<0, 1>(a, kind, counting, c, numSMs, s);
}
}  // namespace hrt
