// nesf_mlp.cu -- the learned warm start: a 6 -> 64 -> 64 -> 3 GELU network whose
// inference and training run on the tcgen05 tensor cores (BF16 operands, FP32
// accumulation in TMEM).
//
// This file holds the GEMM self-check of the tcgen05 building blocks (nesf_tc.cuh)
// in the three operand arrangements the network uses, checked against the host.
#include <cstddef>
#include <cstdio>

#include "nesf_kernels.cuh"
#include "nesf_tc.cuh"

namespace nesf {

// Kernel-side error word: set when a bounded wait gives up.
struct TcStatus {
    unsigned int error;
};

constexpr int kSelfTestSmem = 200 * 1024;   // generous: every descriptor read stays inside

// Copy a row-major R x C BF16 matrix from global memory into the blocked layout.
__device__ __forceinline__ void to_blocked(const __nv_bfloat16* __restrict__ g, unsigned char* s, int R, int C) {
    for (int e = threadIdx.x; e < R * C; e += blockDim.x) {
        int r = e / C, c = e % C;
        *(__nv_bfloat16*)(s + tc::blocked_offset(r, c, R)) = g[e];
    }
}

// D = A x B^T (case 0), A x B (case 1), A^T x B (case 2); see nesf_mlp_selftest.
// Case 3 checks the failure path of the bounded wait: no MMA is issued and nothing
// arrives on the mbarrier, so the wait gives up after kTimeoutCheckPolls polls, the
// status word records the error and the kernel frees its TMEM (nothing is in
// flight) and returns.
constexpr int kTimeoutCheckPolls = 64;

__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const __nv_bfloat16* __restrict__ A,
                                                             const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                             int which, TcStatus* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    unsigned char* sa = smem;
    unsigned char* sb = smem + 64 * 1024;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int N, ksteps, a_mn, b_mn;
    uint32_t a_lbo, a_sbo, a_step, b_lbo, b_sbo, b_step;
    int RA, RB;
    bool a_kcol, b_kcol;
    if (which == 0) {          // A [128 x 64], B [64 (N) x 64 (K)]: both K-major
        RA = 128; RB = 64; to_blocked(A, sa, 128, 64); to_blocked(B, sb, 64, 64);
        N = 64; ksteps = 4; a_kcol = true; b_kcol = true;
    } else if (which == 1) {   // A [128 x 64] K-major, B [64 (K) x 64 (N)]: N contiguous
        RA = 128; RB = 64; to_blocked(A, sa, 128, 64); to_blocked(B, sb, 64, 64);
        N = 64; ksteps = 4; a_kcol = true; b_kcol = false;
    } else if (which == 3) {   // the wait-timeout check: no operands
        RA = 128; RB = 64;
        N = 64; ksteps = 4; a_kcol = true; b_kcol = true;
    } else {                   // A [128 (K) x 128 (M)], B [128 (K) x 16 (N)]: both MN-major
        RA = 128; RB = 128; to_blocked(A, sa, 128, 128); to_blocked(B, sb, 128, 16);
        N = 16; ksteps = 8; a_kcol = false; b_kcol = false;
    }
    a_mn = a_kcol ? 0 : 1;
    b_mn = b_kcol ? 0 : 1;
    a_lbo = tc::blocked_lbo(RA, a_kcol); a_sbo = tc::blocked_sbo(RA, a_kcol); a_step = tc::blocked_kstep(RA, a_kcol);
    b_lbo = tc::blocked_lbo(RB, b_kcol); b_sbo = tc::blocked_sbo(RB, b_kcol); b_step = tc::blocked_kstep(RB, b_kcol);
    tc::fence_smem_to_async();
    if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
    if (warp == 0) tc::tmem_alloc(&tslot, 64);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tslot;
    const bool issue = which != 3;
    if (threadIdx.x == 0 && issue) {
        uint32_t id = tc::idesc_bf16(128, N, a_mn, b_mn);
        tc::mma_chain(tbase, tc::smem_addr(sa), a_lbo, a_sbo, a_step, tc::smem_addr(sb), b_lbo, b_sbo, b_step, id,
                      ksteps, false);
        tc::mma_commit(&bar);
    }
    const int limit = issue ? tc::kSpinLimit : kTimeoutCheckPolls;
    bool ok = __all_sync(0xffffffffu, tc::mbar_wait(&bar, 0, limit));   // warp-uniform: tcgen05.ld is .aligned
    if (!ok) {
        if (lane == 0) atomicExch(&status->error, 1u);
        tc::mbar_wait(&bar, 0, limit);   // give the MMA a second bounded chance to drain before TMEM is freed
    }
    tc::fence_after_sync();
    if (ok) {
        const int r = 32 * warp + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tbase, warp, c0), v);
#pragma unroll
            for (int i = 0; i < 16; i++) D[r * N + c0 + i] = v[i];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 64);
}

cudaError_t launch_tc_selftest(const void* A, const void* B, float* D, int which, unsigned int* status,
                               cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSelfTestSmem);
    if (e != cudaSuccess) return e;
    tc_selftest_kernel<<<1, 128, kSelfTestSmem, s>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, which,
                                                      (TcStatus*)status);
    return cudaGetLastError();
}

}  // namespace nesf

// =====================================================================
// The network: initialisation, normalisation, the tcgen05 tile pass (inference
// or forward + backward), Adam.
// =====================================================================
#include "nesf_mlp.cuh"

namespace nesf {
namespace mlp {

// Counter-based uniform in [-1, 1) (splitmix64 of seed and index).
__device__ __forceinline__ float hash_uniform(uint64_t seed, uint64_t i) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((z >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
}

__device__ __forceinline__ void refresh_bf16(Blob* b, int i) {
    if (i < kB1) b->w1h[i - kW1] = __float2bfloat16_rn(b->p[i]);
    else if (i >= kW2 && i < kB2) b->w2h[i - kW2] = __float2bfloat16_rn(b->p[i]);
    else if (i >= kW3 && i < kB3) b->w3h[i - kW3] = __float2bfloat16_rn(b->p[i]);
}

// Xavier-uniform weights (zero in the padding), zero biases, moments and
// gradient, identity normalisation.
__global__ void init_kernel(Blob* b, uint64_t seed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        float w = 0.0f;
        if (i < kB1) {
            int in = (i - kW1) % kInPad;
            w = in < kIn ? hash_uniform(seed, i) * sqrtf(6.0f / (kIn + kHid)) : 0.0f;
        } else if (i >= kW2 && i < kB2) {
            w = hash_uniform(seed, i) * sqrtf(6.0f / (kHid + kHid));
        } else if (i >= kW3 && i < kB3) {
            int out = (i - kW3) / kHid;
            w = out < kOut ? hash_uniform(seed, i) * sqrtf(6.0f / (kHid + kOut)) : 0.0f;
        }
        b->p[i] = w;
        b->g[i] = b->m[i] = b->v[i] = 0.0f;
        refresh_bf16(b, i);
    }
    if (blockIdx.x == 0 && threadIdx.x < 8) {
        b->in_mu[threadIdx.x] = 0.0f;
        b->in_sig[threadIdx.x] = 1.0f;
        if (threadIdx.x < 4) {
            b->out_mu[threadIdx.x] = 0.0f;
            b->out_sig[threadIdx.x] = 1.0f;
            b->loss[threadIdx.x] = 0.0f;
        }
        if (threadIdx.x == 0) { b->steps = 0; b->error = 0; }
    }
}

// Normalisation: sums and sums of squares of the 6 features and of the 3 targets
// (where their mask bit is set), in FP64.
__global__ void norm_sums_kernel(Blob* b, const float* __restrict__ x, const float* __restrict__ t, int64_t n) {
    __shared__ double acc[32];
    if (threadIdx.x < 32) acc[threadIdx.x] = 0.0;
    __syncthreads();
    double s[9] = {0}, q[9] = {0}, c[3] = {0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < kIn; k++) { double v = x[i * 8 + k]; s[k] += v; q[k] += v * v; }
        int mask = (int)t[i * 4 + 3];
#pragma unroll
        for (int k = 0; k < kOut; k++)
            if (mask >> k & 1) { double v = t[i * 4 + k]; s[6 + k] += v; q[6 + k] += v * v; c[k] += 1.0; }
    }
#pragma unroll
    for (int k = 0; k < 9; k++) { atomicAdd(&acc[k], s[k]); atomicAdd(&acc[9 + k], q[k]); }
#pragma unroll
    for (int k = 0; k < 3; k++) atomicAdd(&acc[18 + k], c[k]);
    __syncthreads();
    if (threadIdx.x < 21) atomicAdd(&b->stats[threadIdx.x], acc[threadIdx.x]);
}

__global__ void norm_finish_kernel(Blob* b, int64_t n) {
    int k = threadIdx.x;
    if (k >= 9) return;
    double cnt = k < kIn ? (double)n : b->stats[18 + (k - kIn)];
    double mu = cnt > 0 ? b->stats[k] / cnt : 0.0;
    double var = cnt > 1 ? b->stats[9 + k] / cnt - mu * mu : 1.0;
    float sig = var > 1e-20 ? (float)sqrt(var) : 1.0f;
    if (k < kIn) { b->in_mu[k] = (float)mu; b->in_sig[k] = sig; }
    else { b->out_mu[k - kIn] = (float)mu; b->out_sig[k - kIn] = sig; }
}

// ------------------------------------------------------------- tile pass
// Where the pass reads and writes: plain arrays (slot = i), or the work list of
// a solve (slot = i for the unstable part, per_member - 1 - (i - nu) for the
// stable part), n then read from the list's counters.
struct PassIO {
    const float* x;          // features, 8 per slot
    const float* t;          // targets (c_u, c_theta, c_q, mask), 4 per slot; null for inference
    float* y;                // outputs (c_u, c_theta, c_q, 1), 4 per slot; null for training
    int64_t n;
    const unsigned int* count;
    int64_t per_member;
    int state;               // outputs as (c_u dU, c_theta dtheta_0, c_q dq_0, 1): a solver's starting state
};

constexpr int kPassSmem = 132 * 1024;     // training: the backward operands too
constexpr int kInferSmem = 48 * 1024;     // inference: weights, X, H1, H2 (up to 4 CTAs per SM)
// shared-memory offsets of the operand tiles (blocked layout)
constexpr int oW1 = 0, oW2 = 2048, oW3 = 10240, oX = 12288, oH1 = 16384, oH2 = 32768, oDY = 65536, oDZ2 = 69632,
              oDZ1 = 102400;
// TMEM columns: layer scratch, then the weight-gradient accumulators
constexpr int tD = 0, tW2 = 64, tW1 = 128, tW3 = 144, kTmemCols = 256, kInferTmemCols = 64;

__device__ __forceinline__ void store_row16(unsigned char* buf, int R, int r, int c0, const float (&v)[16]) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        __align__(16) __nv_bfloat16 q[8];
#pragma unroll
        for (int i = 0; i < 8; i++) q[i] = __float2bfloat16_rn(v[8 * h + i]);
        *(uint4*)(buf + tc::blocked_offset(r, c0 + 8 * h, R)) = *(const uint4*)q;
    }
}

__device__ __forceinline__ int64_t pass_slot(const PassIO& io, int64_t i, unsigned nu) {
    if (!io.count) return i;
    return i < nu ? i : io.per_member - 1 - (i - nu);
}

// Sum of v over the 32 lanes of a warp.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <bool TRAIN>
__global__ void __launch_bounds__(128, TRAIN ? 1 : 4) pass_kernel(Blob* __restrict__ B, PassIO io) {
    constexpr int kSmem = TRAIN ? kPassSmem : kInferSmem;
    constexpr uint32_t kCols = TRAIN ? kTmemCols : kInferTmemCols;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    __shared__ __align__(16) float sb1[kHid];   // read as float2 pairs by the inference
    __shared__ __align__(16) float sb2[kHid];
    __shared__ float sb3[kOutPad];
    __shared__ float gb1[kHid], gb2[kHid], gb3[kOutPad];
    __shared__ float in_mu[8], in_sig[8], out_mu[4], out_sig[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
    const int r = tid;   // the row (sample) of the tile this thread owns

    unsigned nu = 0;
    int64_t n = io.n;
    if (io.count) { nu = io.count[0]; n = (int64_t)nu + io.count[1]; }
    const int64_t tiles = (n + 127) / 128;

    // zero the operand tiles (the MN-major weight-gradient operands read 128 columns)
    for (int i = tid; i < kSmem / 16; i += 128) ((uint4*)sm)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    // weights (BF16, row-major [out][in]) into the blocked layout; biases and normalisation
    for (int e = tid; e < kHid * kInPad; e += 128)
        *(__nv_bfloat16*)(sm + oW1 + tc::blocked_offset(e / kInPad, e % kInPad, kHid)) = B->w1h[e];
    for (int e = tid; e < kHid * kHid; e += 128)
        *(__nv_bfloat16*)(sm + oW2 + tc::blocked_offset(e / kHid, e % kHid, kHid)) = B->w2h[e];
    for (int e = tid; e < kOutPad * kHid; e += 128)
        *(__nv_bfloat16*)(sm + oW3 + tc::blocked_offset(e / kHid, e % kHid, kOutPad)) = B->w3h[e];
    if (tid < kHid) { sb1[tid] = B->p[kB1 + tid]; sb2[tid] = B->p[kB2 + tid]; gb1[tid] = 0.0f; gb2[tid] = 0.0f; }
    if (tid < kOutPad) { sb3[tid] = B->p[kB3 + tid]; gb3[tid] = 0.0f; }
    if (tid < 8) { in_mu[tid] = B->in_mu[tid]; in_sig[tid] = B->in_sig[tid]; }
    if (tid < 4) { out_mu[tid] = B->out_mu[tid]; out_sig[tid] = B->out_sig[tid]; }
    if (tid == 0) tc::mbar_init(&bar, 1);
    if (warp == 0) tc::tmem_alloc(&tslot, kCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tslot;
    const uint32_t aW1 = tc::smem_addr(sm + oW1), aW2 = tc::smem_addr(sm + oW2), aW3 = tc::smem_addr(sm + oW3);
    const uint32_t aX = tc::smem_addr(sm + oX), aH1 = tc::smem_addr(sm + oH1), aH2 = tc::smem_addr(sm + oH2);
    const uint32_t aDY = tc::smem_addr(sm + oDY), aDZ2 = tc::smem_addr(sm + oDZ2), aDZ1 = tc::smem_addr(sm + oDZ1);
    const uint32_t K = 2048, KS = 2 * 2048;   // 128-row tiles, K = columns: LBO and K step
    uint32_t phase = 0;
    bool ok = true, first = true;
    float lsum = 0.0f, lcnt = 0.0f;

    // one tensor-core stage: publish the shared-memory operands, issue, wait
    auto stage = [&](auto issue) {
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue();
            tc::mma_commit(&bar);
        }
        bool done = tc::mbar_wait(&bar, phase);
        phase ^= 1u;
        ok = __syncthreads_and(done) != 0;
        tc::fence_after_sync();
    };

    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t i = tile * 128 + r;
        const bool valid = i < n;
        const int64_t slot = valid ? pass_slot(io, i, nu) : 0;
        // ---- features (normalised, BF16) into X
        {
            float v[16];
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = 0.0f;
            if (valid) {
                const float4* xs = reinterpret_cast<const float4*>(io.x + slot * 8);   // 32-byte rows
                const float4 a = xs[0], b = xs[1];
                const float f[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
                for (int k = 0; k < kIn; k++) v[k] = (f[k] - in_mu[k]) / in_sig[k];
            }
            store_row16(sm + oX, 128, r, 0, v);
        }
        float Z1[kHid], Z2[kHid];
        // ---- layer 1: D = X W1^T
        stage([&] { tc::mma_chain(tm + tD, aX, K, 128, KS, aW1, 1024, 128, 2048, tc::idesc_bf16(128, 64, 0, 0), 1, false); });
        if (!ok) break;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tm + tD, warp, c0), v);
            if constexpr (TRAIN) {
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    Z1[c0 + k] = v[k] + sb1[c0 + k];
                    v[k] = gelu(Z1[c0 + k]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 16; k += 2)
                    gelu_bias_approx2(v[k], v[k + 1], *reinterpret_cast<const float2*>(&sb1[c0 + k]));
            }
            store_row16(sm + oH1, 128, r, c0, v);
        }
        // ---- layer 2: D = H1 W2^T
        stage([&] { tc::mma_chain(tm + tD, aH1, K, 128, KS, aW2, 1024, 128, 2048, tc::idesc_bf16(128, 64, 0, 0), 4, false); });
        if (!ok) break;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tm + tD, warp, c0), v);
            if constexpr (TRAIN) {
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    Z2[c0 + k] = v[k] + sb2[c0 + k];
                    v[k] = gelu(Z2[c0 + k]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 16; k += 2)
                    gelu_bias_approx2(v[k], v[k + 1], *reinterpret_cast<const float2*>(&sb2[c0 + k]));
            }
            store_row16(sm + oH2, 128, r, c0, v);
        }
        // ---- layer 3: D = H2 W3^T (16 columns, 3 used)
        stage([&] { tc::mma_chain(tm + tD, aH2, K, 128, KS, aW3, 256, 128, 512, tc::idesc_bf16(128, 16, 0, 0), 4, false); });
        if (!ok) break;
        float y[16];
        tc::tmem_ld16(tc::tmem_at(tm + tD, warp, 0), y);
#pragma unroll
        for (int k = 0; k < 16; k++) y[k] += sb3[k];
        if (!TRAIN) {
            if (valid) {
                float4 o;
                o.x = y[0] * out_sig[0] + out_mu[0];
                o.y = y[1] * out_sig[1] + out_mu[1];
                o.z = y[2] * out_sig[2] + out_mu[2];
                o.w = 1.0f;
                if (io.state) {
                    const float* f = io.x + slot * 8;
                    o.x *= f[6];              // dU
                    o.y *= f[2];              // dtheta_0
                    o.z *= 1e-3f * f[3];      // dq_0 (features hold it in g/kg)
                }
                *(float4*)(io.y + slot * 4) = o;
            }
            continue;
        }
        // ---- loss of the normalised outputs and its gradient dY (mean over the n samples)
        float dy[16];
#pragma unroll
        for (int k = 0; k < 16; k++) dy[k] = 0.0f;
        if (valid) {
            int mask = (int)io.t[slot * 4 + 3];
#pragma unroll
            for (int k = 0; k < kOut; k++) {
                if (!(mask >> k & 1)) continue;
                float tk = (io.t[slot * 4 + k] - out_mu[k]) / out_sig[k];
                float e = y[k] - tk;
                lsum += e * e;
                dy[k] = 2.0f * e / (float)n;
            }
            lcnt += 1.0f;
        }
        store_row16(sm + oDY, 128, r, 0, dy);
#pragma unroll
        for (int k = 0; k < kOut; k++) {
            float s = warp_sum(dy[k]);
            if (lane == 0) atomicAdd(&gb3[k], s);
        }
        // ---- dH2 = dY W3 (W3 MN-major: rows are K)
        stage([&] { tc::mma_chain(tm + tD, aDY, K, 128, KS, aW3, 128, 256, 256, tc::idesc_bf16(128, 64, 0, 1), 1, false); });
        if (!ok) break;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tm + tD, warp, c0), v);
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] *= gelu_grad(Z2[c0 + k]);
            store_row16(sm + oDZ2, 128, r, c0, v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                float s = warp_sum(v[k]);
                if (lane == 0) atomicAdd(&gb2[c0 + k], s);
            }
        }
        // ---- dH1 = dZ2 W2; dW2 += dZ2^T H1; dW3^T += H2^T dY
        const bool acc = !first;
        stage([&] {
            tc::mma_chain(tm + tD, aDZ2, K, 128, KS, aW2, 128, 1024, 256, tc::idesc_bf16(128, 64, 0, 1), 4, false);
            tc::mma_chain(tm + tW2, aDZ2, 128, 2048, 256, aH1, 128, 2048, 256, tc::idesc_bf16(128, 64, 1, 1), 8, acc);
            tc::mma_chain(tm + tW3, aH2, 128, 2048, 256, aDY, 128, 2048, 256, tc::idesc_bf16(128, 16, 1, 1), 8, acc);
        });
        if (!ok) break;
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tm + tD, warp, c0), v);
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] *= gelu_grad(Z1[c0 + k]);
            store_row16(sm + oDZ1, 128, r, c0, v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                float s = warp_sum(v[k]);
                if (lane == 0) atomicAdd(&gb1[c0 + k], s);
            }
        }
        // ---- dW1 += dZ1^T X
        stage([&] { tc::mma_chain(tm + tW1, aDZ1, 128, 2048, 256, aX, 128, 2048, 256, tc::idesc_bf16(128, 16, 1, 1), 8, acc); });
        if (!ok) break;
        first = false;
    }
    if (!ok) {
        if (tid == 0) atomicExch(&B->error, 1);
        tc::mbar_wait(&bar, phase ^ 1u);   // a bounded second chance for the MMA in flight before TMEM is freed
    }
    if (TRAIN && ok && !first) {
        // weight gradients: rows 0..63 of the accumulators (warps 0 and 1)
        if (warp < 2) {
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(tc::tmem_at(tm + tW2, warp, c0), v);
#pragma unroll
                for (int k = 0; k < 16; k++) atomicAdd(&B->g[kW2 + r * kHid + c0 + k], v[k]);
            }
            float v[16];
            tc::tmem_ld16(tc::tmem_at(tm + tW1, warp, 0), v);
#pragma unroll
            for (int k = 0; k < kIn; k++) atomicAdd(&B->g[kW1 + r * kInPad + k], v[k]);
            tc::tmem_ld16(tc::tmem_at(tm + tW3, warp, 0), v);
#pragma unroll
            for (int k = 0; k < kOut; k++) atomicAdd(&B->g[kW3 + k * kHid + r], v[k]);
        }
    }
    if (TRAIN) {
        __syncthreads();
        if (tid < kHid) { atomicAdd(&B->g[kB1 + tid], gb1[tid]); atomicAdd(&B->g[kB2 + tid], gb2[tid]); }
        if (tid < kOut) atomicAdd(&B->g[kB3 + tid], gb3[tid]);
        float ls = warp_sum(lsum), lc = warp_sum(lcnt);
        if (lane == 0) { atomicAdd(&B->loss[0], ls); atomicAdd(&B->loss[1], lc); }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, kCols);
}

// Adam on the FP32 parameters from the accumulated gradient; refreshes the BF16
// copies and clears the gradient.
__global__ void adam_kernel(Blob* b, float lr, float beta1, float beta2, float eps) {
    const int step = b->steps + 1;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        float g = b->g[i];
        float m = beta1 * b->m[i] + (1.0f - beta1) * g;
        float v = beta2 * b->v[i] + (1.0f - beta2) * g * g;
        b->m[i] = m;
        b->v[i] = v;
        b->p[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
        b->g[i] = 0.0f;
        refresh_bf16(b, i);
    }
}

__global__ void adam_count_kernel(Blob* b) { b->steps += 1; }

}  // namespace mlp

// ---------------------------------------------------------------- launchers
cudaError_t mlp_init(void* blob, uint64_t seed, cudaStream_t s) {
    mlp::init_kernel<<<32, 256, 0, s>>>((mlp::Blob*)blob, seed);
    return cudaGetLastError();
}

cudaError_t mlp_fit_normalization(void* blob, const float* x, const float* t, int64_t n, cudaStream_t s) {
    mlp::Blob* b = (mlp::Blob*)blob;
    cudaError_t e = cudaMemsetAsync(b->stats, 0, sizeof b->stats, s);
    if (e != cudaSuccess) return e;
    mlp::norm_sums_kernel<<<256, 256, 0, s>>>(b, x, t, n);
    mlp::norm_finish_kernel<<<1, 32, 0, s>>>(b, n);
    return cudaGetLastError();
}

// One pass of the tile kernel: inference (y != null) or forward + backward that
// adds the gradient of the mean loss to the blob's gradient (t != null).
cudaError_t mlp_pass(void* blob, const float* x, const float* t, float* y, int64_t n, const unsigned int* count,
                     int64_t per_member, int grid, bool state, cudaStream_t s) {
    mlp::PassIO io{x, t, y, n, count, per_member, state ? 1 : 0};
    const bool train = t != nullptr;
    cudaError_t e = train ? cudaFuncSetAttribute(mlp::pass_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 mlp::kPassSmem)
                          : cudaFuncSetAttribute(mlp::pass_kernel<false>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::kInferSmem);
    if (e != cudaSuccess) return e;
    if (train) mlp::pass_kernel<true><<<grid, 128, mlp::kPassSmem, s>>>((mlp::Blob*)blob, io);
    else mlp::pass_kernel<false><<<grid, 128, mlp::kInferSmem, s>>>((mlp::Blob*)blob, io);
    return cudaGetLastError();
}

cudaError_t mlp_adam(void* blob, float lr, float beta1, float beta2, float eps, cudaStream_t s) {
    mlp::adam_kernel<<<(mlp::kParams + 255) / 256, 256, 0, s>>>((mlp::Blob*)blob, lr, beta1, beta2, eps);
    mlp::adam_count_kernel<<<1, 1, 0, s>>>((mlp::Blob*)blob);
    return cudaGetLastError();
}

size_t mlp_blob_bytes() { return sizeof(mlp::Blob); }
size_t mlp_loss_offset() { return offsetof(mlp::Blob, loss); }

}  // namespace nesf
