// Instantiation of the W = 64 launch path.
#include "path_impl.cuh"

namespace pty {
template int run_path<64>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*,
                          double*, float2*, float2*, float*, float*, void*, cudaStream_t);
template int run_forward<64>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*,
                             double*, void*, cudaStream_t);
template int run_backward<64>(const pty_problem_t*, const Plan&, double*, float2*, float2*, float*, void*,
                              cudaStream_t);
template int run_ms_forward<64>(const MsPlan&, const float2*, const float2*, const float2*, float, float2*,
                                float2*, void*, cudaStream_t);
template int run_ms_grads<64>(const MsPlan&, const float2*, const float2*, const float2*, const float2*, float,
                              const float*, int, float2*, float2*, void*, cudaStream_t);
template int run_scatteradd<64>(const MsPlan&, float2*, const float2*, void*, cudaStream_t);
template int run_fft2<64>(const float2*, float2*, int, int, int, float2*, cudaStream_t, int);
}  // namespace pty
