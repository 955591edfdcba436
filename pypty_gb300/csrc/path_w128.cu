// Instantiation of the W = 128 launch path.
#include "path_impl.cuh"

namespace pty {
template int run_path<128>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*,
                          double*, float2*, float2*, float*, float*, void*, cudaStream_t);
template int run_forward<128>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*,
                             double*, void*, cudaStream_t);
template int run_backward<128>(const pty_problem_t*, const Plan&, double*, float2*, float2*, float*, void*,
                              cudaStream_t);
template int run_ms_forward<128>(const MsPlan&, const float2*, const float2*, const float2*, float, float2*,
                                float2*, void*, cudaStream_t);
template int run_ms_grads<128>(const MsPlan&, const float2*, const float2*, const float2*, const float2*, float,
                              const float*, int, float2*, float2*, void*, cudaStream_t);
template int run_scatteradd<128>(const MsPlan&, float2*, const float2*, void*, cudaStream_t);
template int run_fft2<128>(const float2*, float2*, int, int, int, float2*, cudaStream_t, int);
}  // namespace pty
