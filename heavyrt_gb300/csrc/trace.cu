// Traversal dispatch: validates the batch and calls the layout's kernels
// (trace_impl.cuh; one translation unit per layout, trace_l0..3.cu).
#include "hrt_kernels.cuh"

namespace hrt
{
cudaError_t trace_l0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l1(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l2(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);

cudaError_t trace(const TraceArgs& a, int kind, int counting, int layout, const TraceConfig& c, int numSMs,
                  cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  if (a.n > 0x7FFFFFFFull) return cudaErrorInvalidValue;  // the pool's counter may overshoot n by a few warps
  switch (layout)
  {
    case 0: return trace_l0(a, kind, counting, c, numSMs, s);
    case 1: return trace_l1(a, kind, counting, c, numSMs, s);
    case 2: return trace_l2(a, kind, counting, c, numSMs, s);
    case 3: return trace_l3(a, kind, counting, c, numSMs, s);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace hrt
