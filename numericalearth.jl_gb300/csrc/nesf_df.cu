// nesf_df.cu -- the check of the double-float arithmetic (nesf_df.cuh) that the adaptive
// solver's replays run in: each operation on device arrays of FP64 arguments, rounded to
// double-float, the result widened back to FP64. Built with the solve files' fast-math
// flags, so that the check covers the arithmetic as the solves compile it.
#include "nesf_device.cuh"

namespace nesf {

__global__ void __launch_bounds__(256) df_check_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                                       double* __restrict__ out, int64_t n, int op) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const df a(x[i]), b(y ? y[i] : 0.0);
    df r;
    switch (op) {
    case NESF_DF_ADD: r = a + b; break;
    case NESF_DF_SUB: r = a - b; break;
    case NESF_DF_MUL: r = a * b; break;
    case NESF_DF_DIV: r = a / b; break;
    case NESF_DF_SQRT: r = M<df>::sqrt(a); break;
    case NESF_DF_CBRT: r = M<df>::cbrt(a); break;
    case NESF_DF_EXP: r = M<df>::exp(a); break;
    case NESF_DF_LOG: r = M<df>::log(a); break;
    case NESF_DF_POW: r = M<df>::pow(a, b); break;
    default: r = M<df>::atan(a); break;
    }
    out[i] = (double)r;
}

cudaError_t launch_df_check(const double* x, const double* y, double* out, int64_t n, int op, cudaStream_t s) {
    df_check_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, y, out, n, op);
    return cudaGetLastError();
}

}  // namespace nesf
