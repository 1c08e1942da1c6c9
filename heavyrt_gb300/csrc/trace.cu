// Traversal dispatch: validates the batch and calls the layout's kernels
// (trace_impl.cuh; one translation unit per layout and triangle test,
// trace_l0..3.cu for Moller-Trumbore, trace_w0..3.cu for the watertight test).
#include "hrt_kernels.cuh"

namespace hrt
{
cudaError_t trace_l0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l1(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l2(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w1(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w2(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);

cudaError_t trace(const TraceArgs& a, int kind, int counting, int layout, const TraceConfig& c, int numSMs,
                  cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  if (a.n > 0x7FFFFFFFull) return cudaErrorInvalidValue;  // the pool's counter may overshoot n by a few warps
  if (a.triTest == 1)
    switch (layout)
    {
      case 0: return trace_w0(a, kind, counting, c, numSMs, s);
      case 1: return trace_w1(a, kind, counting, c, numSMs, s);
      case 2: return trace_w2(a, kind, counting, c, numSMs, s);
      case 3: return trace_w3(a, kind, counting, c, numSMs, s);
      default: return cudaErrorInvalidValue;
    }
  if (a.triTest != 0) return cudaErrorInvalidValue;
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
