// nesf_integrals.cu -- compensated FP64 area integrals of surface fields, the
// global sums behind the reference's conservation checks
// (test/test_conservation.jl:100-101: int dA(a) = sum(a) * A_z, int dA(a, b) =
// sum(a .* b) * A_z).
//
// Each integral is carried as an unevaluated pair (hi, lo) with hi + lo the sum:
// every cell term is added with an error-free two-sum (Knuth), pairs are combined
// in a fixed order -- threads by a warp-shuffle tree, warps in index order, blocks
// in index order by one finishing block -- so the result does not depend on
// scheduling. The products are rounded once in FP64 (explicit _rn intrinsics: no
// contraction into the sums). The pass reads each field once and is HBM-bound
// with FP32 fields; with FP64 fields the FP64 adds (about 8 per term) bound it.
#include "nesf_kernels.cuh"

namespace nesf {

struct DD {
    double hi, lo;
};

// s + e = a + b exactly (Knuth's two-sum, no ordering assumption).
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ __forceinline__ void dd_add(DD& d, double x) {
    double s, e;
    two_sum(d.hi, x, s, e);
    d.hi = s;
    d.lo = __dadd_rn(d.lo, e);
}

__device__ __forceinline__ DD dd_combine(DD a, DD b) {
    double s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __dadd_rn(e, __dadd_rn(a.lo, b.lo));
    DD r;
    r.hi = __dadd_rn(s, e);                  // renormalise: |e| << |s| unless s cancels
    r.lo = __dsub_rn(e, __dsub_rn(r.hi, s));
    return r;
}

template <class S> struct IntegralArgs {
    Layout2 L;
    int n;
    const S* field[NESF_MAX_INTEGRALS];
    const S* factor[NESF_MAX_INTEGRALS];
    const uint8_t* inactive;
    const double* area;
    const double* row_area;
};

constexpr int kIntegralThreads = 256;

// Pass 1: per-block partial sums of every integral.
template <class S>
__global__ void __launch_bounds__(kIntegralThreads) integral_partials_kernel(IntegralArgs<S> a, DD* partials) {
    DD acc[NESF_MAX_INTEGRALS];
#pragma unroll
    for (int k = 0; k < NESF_MAX_INTEGRALS; k++) acc[k] = DD{0.0, 0.0};
    const int64_t cells = (int64_t)a.L.nx * a.L.ny;
    const bool weighted = a.area != nullptr || a.row_area != nullptr;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < cells; r += (int64_t)gridDim.x * blockDim.x) {
        int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
        int64_t c = a.L.at(i, j);
        if (a.inactive && a.inactive[c] != 0) continue;
        double w = a.area ? a.area[c] : (a.row_area ? a.row_area[j - 1] : 1.0);
#pragma unroll
        for (int k = 0; k < NESF_MAX_INTEGRALS; k++) {
            if (k >= a.n) break;
            double x = (double)a.field[k][c];
            if (a.factor[k]) x = __dmul_rn(x, (double)a.factor[k][c]);
            if (weighted) x = __dmul_rn(x, w);
            dd_add(acc[k], x);
        }
    }
    __shared__ DD warp_sum[kIntegralThreads / 32][NESF_MAX_INTEGRALS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NESF_MAX_INTEGRALS; k++) {
        if (k >= a.n) break;
        DD v = acc[k];
        for (int off = 16; off > 0; off >>= 1) {
            DD o;
            o.hi = __shfl_down_sync(0xffffffffu, v.hi, off);
            o.lo = __shfl_down_sync(0xffffffffu, v.lo, off);
            v = dd_combine(v, o);
        }
        if (lane == 0) warp_sum[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < a.n) {
        DD v = warp_sum[0][threadIdx.x];
        for (int w = 1; w < kIntegralThreads / 32; w++) v = dd_combine(v, warp_sum[w][threadIdx.x]);
        partials[(int64_t)blockIdx.x * NESF_MAX_INTEGRALS + threadIdx.x] = v;
    }
}

// Pass 2: one thread per integral sums the block partials in block order; without
// cell areas the sum is multiplied by the uniform area (the product kept exact:
// hi * A = p + e with an FMA).
__global__ void integral_finish_kernel(const DD* partials, int blocks, int n, bool uniform, double area,
                                       double* result) {
    int k = threadIdx.x;
    if (k >= n) return;
    DD v = partials[k];
    for (int b = 1; b < blocks; b++) v = dd_combine(v, partials[(int64_t)b * NESF_MAX_INTEGRALS + k]);
    if (uniform) {
        double p = __dmul_rn(v.hi, area);
        double e = __fma_rn(v.hi, area, -p);
        e = __fma_rn(v.lo, area, e);
        v.hi = __dadd_rn(p, e);
        v.lo = __dsub_rn(e, __dsub_rn(v.hi, p));
    }
    result[2 * k] = v.hi;
    result[2 * k + 1] = v.lo;
}

template <class S>
static cudaError_t launch_integrals_t(const nesf_integral_fields& f, void* partials, int max_blocks, double* result,
                                      cudaStream_t s) {
    IntegralArgs<S> a;
    a.L = Layout2{f.grid.nx, f.grid.ny, f.grid.hx, f.grid.hy, f.grid.stride_j};
    a.n = f.n;
    for (int k = 0; k < NESF_MAX_INTEGRALS; k++) {
        a.field[k] = k < f.n ? (const S*)f.field[k] : nullptr;
        a.factor[k] = k < f.n ? (const S*)f.factor[k] : nullptr;
    }
    a.inactive = f.inactive;
    a.area = f.area;
    a.row_area = f.row_area;
    int64_t cells = (int64_t)f.grid.nx * f.grid.ny;
    int blocks = (int)((cells + kIntegralThreads - 1) / kIntegralThreads);
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    integral_partials_kernel<S><<<blocks, kIntegralThreads, 0, s>>>(a, (DD*)partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bool uniform = f.area == nullptr && f.row_area == nullptr;
    integral_finish_kernel<<<1, 32, 0, s>>>((const DD*)partials, blocks, f.n, uniform, f.uniform_area, result);
    return cudaGetLastError();
}

// Partials buffer: max_blocks x NESF_MAX_INTEGRALS pairs.
cudaError_t launch_integrals(const nesf_integral_fields& f, void* partials, int max_blocks, double* result,
                             cudaStream_t s) {
    return f.dtype == NESF_F64 ? launch_integrals_t<double>(f, partials, max_blocks, result, s)
                               : launch_integrals_t<float>(f, partials, max_blocks, result, s);
}

}  // namespace nesf
