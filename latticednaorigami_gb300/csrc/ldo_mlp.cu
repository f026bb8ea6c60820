// Kernels of the learned-proposal network (ldo_mlp.h).
//
// Matrix products run on the 5th-generation tensor cores (ldo_umma.cuh:
// tcgen05.mma, operands staged in shared memory, fp32 accumulators in tensor
// memory) as C = A * B^T with both operands K-major; the weight copies are
// kept in both orientations and the backward pass transposes activations and
// gradients for the weight-gradient products.  Every other step (bias, GELU
// and its derivative, the 256 -> 1 output layer, the loss, column sums, Adam)
// is an elementwise or reduction kernel in fp32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_mlp.h"
#include "ldo_umma.cuh"

namespace {

constexpr int H = LDO_LEARN_H;
constexpr int DIN = LDO_LEARN_DIN;
// bf16 weight copies: W1 [DIN][H], W2 [H][H], W3 [H][H], w4 [H], and the
// transposes W1t [H][DIN], W2t, W3t (K-major operands of the forward products)
constexpr int BF_W1 = 0;
constexpr int BF_W2 = BF_W1 + DIN * H;
constexpr int BF_W3 = BF_W2 + H * H;
constexpr int BF_W4 = BF_W3 + H * H;
constexpr int BF_W1T = BF_W4 + H;
constexpr int BF_W2T = BF_W1T + DIN * H;
constexpr int BF_W3T = BF_W2T + H * H;
constexpr int BF_N = BF_W3T + H * H;

__device__ __forceinline__ uint16_t f2bf(float f) {
    __nv_bfloat16 b = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t*>(&b);
}
__device__ __forceinline__ float bf2f(uint16_t u) {
    return __uint_as_float(((unsigned)u) << 16);
}

// ---------------------------------------------------------- products ---
// C[M][N] = A[M][K] * Bt[N][K]^T on the tensor cores
cudaError_t tn(const uint16_t* A, const uint16_t* Bt, float* C, int M, int N, int K, int* err, cudaStream_t s) {
    return ldo_umma::gemm_tn(A, Bt, C, M, N, K, err, s);
}
// Weight gradients (K = batch rows, M x N = a few 128 x 128 tiles): split K
// so that ~128 CTAs share the batch; C (the gradient) starts at zero.
cudaError_t tn_wgrad(const uint16_t* A, const uint16_t* Bt, float* C, int M, int N, int K, int* err,
                     cudaStream_t s) {
    int tiles = ((M + 127) / 128) * ((N + 127) / 128);
    int splits = (K + 511) / 512;
    int cap = 512 / tiles;
    if (splits > cap) splits = cap;
    return ldo_umma::gemm_tn(A, Bt, C, M, N, K, err, s, splits);
}

// dst[C][R] = src[R][C] (bf16), 32 x 32 tiles through shared memory
__global__ void transpose_kernel(const uint16_t* __restrict__ src, uint16_t* __restrict__ dst, int R, int C) {
    __shared__ uint16_t t[32][33];
    int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int r = r0 + i, c = c0 + threadIdx.x;
        if (r < R && c < C) t[i][threadIdx.x] = src[(size_t)r * C + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int c = c0 + i, r = r0 + threadIdx.x;
        if (r < R && c < C) dst[(size_t)c * R + r] = t[threadIdx.x][i];
    }
}

cudaError_t transpose(const uint16_t* src, uint16_t* dst, int R, int C, cudaStream_t s) {
    dim3 grid((C + 31) / 32, (R + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, s>>>(src, dst, R, C);
    return cudaGetLastError();
}

// ------------------------------------------------------ elementwise ---
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void build_x_kernel(const int32_t* idx, int n, uint16_t* x) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float v[DIN];
    ldo_learn_input(idx[r], v);
    for (int i = 0; i < DIN; ++i) x[(size_t)r * DIN + i] = f2bf(v[i]);
}

// z = z + b (in place); h = bf16(gelu(z))
__global__ void bias_gelu_kernel(float* z, const float* b, uint16_t* h, long long total) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    float v = z[e] + b[e % H];
    z[e] = v;
    h[e] = f2bf(gelu(v));
}

// out[r] = sum_j bf16(h3[r][j]) * bf16(w4[j]) + b4 : one warp per row
__global__ void out_layer_kernel(const uint16_t* h3, const uint16_t* w4, const float* b4, float* out, int n) {
    int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (r >= n) return;
    float s = 0.f;
    for (int j = lane; j < H; j += 32) s += bf2f(h3[(size_t)r * H + j]) * bf2f(w4[j]);
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[r] = s + b4[0];
}

// loss += (cnt_t*softplus(z) - cnt_b*z) / norm;  dout = (cnt_t*sigmoid(z) - cnt_b) / norm
__global__ void loss_kernel(const float* out, const float* cnt_b, const float* cnt_t, int n, double norm,
                            float* dout, double* loss) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0;
    if (r < n) {
        float z = out[r];
        float sp = z > 0.f ? z + log1pf(expf(-z)) : log1pf(expf(z));
        float sg = 1.f / (1.f + expf(-z));
        l = ((double)cnt_t[r] * sp - (double)cnt_b[r] * z) / norm;
        dout[r] = (float)(((double)cnt_t[r] * sg - (double)cnt_b[r]) / norm);
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0) atomicAdd(loss, l);
}

// Output layer backward: dw4[j] += sum_r dout[r]*h3[r][j]; db4 += sum_r dout[r];
// dz3[r][j] = dout[r] * w4[j] * gelu'(z3[r][j]) (fp32 and bf16).
__global__ void out_back_kernel(const float* dout, const uint16_t* h3, const uint16_t* w4, const float* z3, int n,
                                float* gw4, float* gb4, float* dz3, uint16_t* g3) {
    // block: 256 threads = one column each, loops over a slice of rows
    int j = threadIdx.x;
    int rows_per = (n + gridDim.x - 1) / gridDim.x;
    int r0 = blockIdx.x * rows_per, r1 = min(n, r0 + rows_per);
    float w = bf2f(w4[j]);
    float sw = 0.f, sb = 0.f;
    for (int r = r0; r < r1; ++r) {
        float d = dout[r];
        size_t e = (size_t)r * H + j;
        sw += d * bf2f(h3[e]);
        if (j == 0) sb += d;
        float v = d * w * gelu_grad(z3[e]);
        dz3[e] = v;
        g3[e] = f2bf(v);
    }
    atomicAdd(&gw4[j], sw);
    if (j == 0) atomicAdd(gb4, sb);
}

// dz = dh * gelu'(z) (in place on dh), bf16 copy
__global__ void gelu_back_kernel(float* dh, const float* z, uint16_t* g, long long total) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    float v = dh[e] * gelu_grad(z[e]);
    dh[e] = v;
    g[e] = f2bf(v);
}

// gb[j] += sum_r dz[r][j]
__global__ void colsum_kernel(const float* dz, int n, float* gb) {
    int j = threadIdx.x;
    int rows_per = (n + gridDim.x - 1) / gridDim.x;
    int r0 = blockIdx.x * rows_per, r1 = min(n, r0 + rows_per);
    float s = 0.f;
    for (int r = r0; r < r1; ++r) s += dz[(size_t)r * H + j];
    atomicAdd(&gb[j], s);
}

__global__ void to_bf16_kernel(const float* p, uint16_t* wbf) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < DIN * H) {
        uint16_t v = f2bf(p[LDO_LEARN_OFF_W1 + e]);
        wbf[BF_W1 + e] = v;
        wbf[BF_W1T + (e % H) * DIN + e / H] = v;
    }
    if (e < H * H) {
        uint16_t v2 = f2bf(p[LDO_LEARN_OFF_W2 + e]);
        uint16_t v3 = f2bf(p[LDO_LEARN_OFF_W3 + e]);
        wbf[BF_W2 + e] = v2;
        wbf[BF_W3 + e] = v3;
        wbf[BF_W2T + (e % H) * H + e / H] = v2;
        wbf[BF_W3T + (e % H) * H + e / H] = v3;
    }
    if (e < H) wbf[BF_W4 + e] = f2bf(p[LDO_LEARN_OFF_W4 + e]);
}

__global__ void adam_kernel(float* p, const float* gr, float* m, float* v, int n, float lr, float b1t, float b2t) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float g = gr[e];
    float mm = b1 * m[e] + (1.f - b1) * g;
    float vv = b2 * v[e] + (1.f - b2) * g * g;
    m[e] = mm;
    v[e] = vv;
    float mh = mm / (1.f - b1t), vh = vv / (1.f - b2t);
    p[e] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void table_kernel(const float* out, int n, double* table) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float z = fminf(fmaxf(out[r], -LDO_LEARN_LOGIT_CLAMP), LDO_LEARN_LOGIT_CLAMP);
    table[r] = (double)expf(z);
}

__global__ void iota_kernel(int32_t* idx, int base, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) idx[r] = base + r;
}

int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

} // namespace

#define MLP_CU(x)                                  \
    do {                                           \
        cudaError_t e_ = (x);                      \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)

template <typename T>
static cudaError_t dalloc(T** p, size_t n) {
    return cudaMalloc((void**)p, n * sizeof(T));
}

cudaError_t ldo_mlp_alloc(LdoMlp& m, int cap) {
    m.cap = cap;
    MLP_CU(dalloc(&m.params, LDO_LEARN_NPARAM));
    MLP_CU(dalloc(&m.grad, LDO_LEARN_NPARAM));
    MLP_CU(dalloc(&m.adam_m, LDO_LEARN_NPARAM));
    MLP_CU(dalloc(&m.adam_v, LDO_LEARN_NPARAM));
    MLP_CU(dalloc(&m.wbf, BF_N));
    MLP_CU(dalloc(&m.idx, cap));
    MLP_CU(dalloc(&m.cnt_b, cap));
    MLP_CU(dalloc(&m.cnt_t, cap));
    MLP_CU(dalloc(&m.x, (size_t)cap * DIN));
    for (int i = 0; i < 3; ++i) {
        MLP_CU(dalloc(&m.z[i], (size_t)cap * H));
        MLP_CU(dalloc(&m.h[i], (size_t)cap * H));
    }
    MLP_CU(dalloc(&m.dz, (size_t)cap * H));
    MLP_CU(dalloc(&m.gbf, (size_t)cap * H));
    MLP_CU(dalloc(&m.ht, (size_t)cap * H));
    MLP_CU(dalloc(&m.gt, (size_t)cap * H));
    MLP_CU(dalloc(&m.err, 1));
    MLP_CU(cudaMemset(m.err, 0, sizeof(int)));
    MLP_CU(dalloc(&m.out, cap));
    MLP_CU(dalloc(&m.dout, cap));
    MLP_CU(dalloc(&m.loss, 1));
    MLP_CU(cudaMemset(m.adam_m, 0, LDO_LEARN_NPARAM * sizeof(float)));
    MLP_CU(cudaMemset(m.adam_v, 0, LDO_LEARN_NPARAM * sizeof(float)));
    m.adam_t = 0;
    return cudaSuccess;
}

void ldo_mlp_free(LdoMlp& m) {
    void* ps[] = {m.params, m.grad, m.adam_m, m.adam_v, m.wbf, m.idx, m.cnt_b, m.cnt_t, m.x, m.z[0], m.z[1], m.z[2],
                  m.h[0], m.h[1], m.h[2], m.dz, m.gbf, m.ht, m.gt, m.err, m.out, m.dout, m.loss};
    for (void* p : ps)
        if (p) cudaFree(p);
    m = LdoMlp {};
}

cudaError_t ldo_mlp_sync_weights(LdoMlp& m, cudaStream_t s) {
    to_bf16_kernel<<<blocks_for(H * H, 256), 256, 0, s>>>(m.params, m.wbf);
    return cudaGetLastError();
}

cudaError_t ldo_mlp_forward(LdoMlp& m, int n, cudaStream_t s) {
    long long tot = (long long)n * H;
    build_x_kernel<<<blocks_for(n, 128), 128, 0, s>>>(m.idx, n, m.x);
    MLP_CU(cudaGetLastError());
    // layer 1: [n][64] x [64][256]
    MLP_CU(tn(m.x, m.wbf + BF_W1T, m.z[0], n, H, DIN, m.err, s));
    bias_gelu_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.z[0], m.params + LDO_LEARN_OFF_B1, m.h[0], tot);
    MLP_CU(tn(m.h[0], m.wbf + BF_W2T, m.z[1], n, H, H, m.err, s));
    bias_gelu_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.z[1], m.params + LDO_LEARN_OFF_B2, m.h[1], tot);
    MLP_CU(tn(m.h[1], m.wbf + BF_W3T, m.z[2], n, H, H, m.err, s));
    bias_gelu_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.z[2], m.params + LDO_LEARN_OFF_B3, m.h[2], tot);
    out_layer_kernel<<<blocks_for((long long)n * 32, 256), 256, 0, s>>>(m.h[2], m.wbf + BF_W4,
                                                                       m.params + LDO_LEARN_OFF_B4, m.out, n);
    return cudaGetLastError();
}

cudaError_t ldo_mlp_loss_grad(LdoMlp& m, int n, double norm, cudaStream_t s) {
    MLP_CU(ldo_mlp_forward(m, n, s));
    long long tot = (long long)n * H;
    MLP_CU(cudaMemsetAsync(m.loss, 0, sizeof(double), s));
    MLP_CU(cudaMemsetAsync(m.grad, 0, LDO_LEARN_NPARAM * sizeof(float), s));
    loss_kernel<<<blocks_for(n, 256), 256, 0, s>>>(m.out, m.cnt_b, m.cnt_t, n, norm, m.dout, m.loss);
    int rb = 1024;
    out_back_kernel<<<rb, H, 0, s>>>(m.dout, m.h[2], m.wbf + BF_W4, m.z[2], n, m.grad + LDO_LEARN_OFF_W4,
                                     m.grad + LDO_LEARN_OFF_B4, m.dz, m.gbf);
    MLP_CU(cudaGetLastError());
    // layer 3: dW3 = h2^T g3 ; db3 = colsum ; dh2 = g3 W3^T
    colsum_kernel<<<rb, H, 0, s>>>(m.dz, n, m.grad + LDO_LEARN_OFF_B3);
    MLP_CU(transpose(m.h[1], m.ht, n, H, s));
    MLP_CU(transpose(m.gbf, m.gt, n, H, s));
    MLP_CU(tn_wgrad(m.ht, m.gt, m.grad + LDO_LEARN_OFF_W3, H, H, n, m.err, s));
    MLP_CU(tn(m.gbf, m.wbf + BF_W3, m.dz, n, H, H, m.err, s));
    gelu_back_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.dz, m.z[1], m.gbf, tot);
    // layer 2
    colsum_kernel<<<rb, H, 0, s>>>(m.dz, n, m.grad + LDO_LEARN_OFF_B2);
    MLP_CU(transpose(m.h[0], m.ht, n, H, s));
    MLP_CU(transpose(m.gbf, m.gt, n, H, s));
    MLP_CU(tn_wgrad(m.ht, m.gt, m.grad + LDO_LEARN_OFF_W2, H, H, n, m.err, s));
    MLP_CU(tn(m.gbf, m.wbf + BF_W2, m.dz, n, H, H, m.err, s));
    gelu_back_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.dz, m.z[0], m.gbf, tot);
    // layer 1
    colsum_kernel<<<rb, H, 0, s>>>(m.dz, n, m.grad + LDO_LEARN_OFF_B1);
    MLP_CU(transpose(m.x, m.ht, n, DIN, s));
    MLP_CU(transpose(m.gbf, m.gt, n, H, s));
    MLP_CU(tn_wgrad(m.ht, m.gt, m.grad + LDO_LEARN_OFF_W1, DIN, H, n, m.err, s));
    return cudaGetLastError();
}

cudaError_t ldo_mlp_adam(LdoMlp& m, float lr, cudaStream_t s) {
    m.adam_t += 1;
    float b1t = (float)pow(0.9, (double)m.adam_t), b2t = (float)pow(0.999, (double)m.adam_t);
    adam_kernel<<<blocks_for(LDO_LEARN_NPARAM, 256), 256, 0, s>>>(m.params, m.grad, m.adam_m, m.adam_v,
                                                                  LDO_LEARN_NPARAM, lr, b1t, b2t);
    MLP_CU(cudaGetLastError());
    return ldo_mlp_sync_weights(m, s);
}

cudaError_t ldo_mlp_table(LdoMlp& m, double* table, cudaStream_t s) {
    for (int base = 0; base < LDO_LEARN_TABLE; base += m.cap) {
        int n = LDO_LEARN_TABLE - base < m.cap ? LDO_LEARN_TABLE - base : m.cap;
        iota_kernel<<<blocks_for(n, 256), 256, 0, s>>>(m.idx, base, n);
        MLP_CU(cudaGetLastError());
        MLP_CU(ldo_mlp_forward(m, n, s));
        table_kernel<<<blocks_for(n, 256), 256, 0, s>>>(m.out, n, table + base);
        MLP_CU(cudaGetLastError());
    }
    return cudaSuccess;
}

cudaError_t ldo_mlp_check(LdoMlp& m, cudaStream_t s, bool* timed_out) {
    int e = 0;
    MLP_CU(cudaMemcpyAsync(&e, m.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    MLP_CU(cudaStreamSynchronize(s));
    *timed_out = e != 0;
    if (e) MLP_CU(cudaMemsetAsync(m.err, 0, sizeof(int), s));
    return cudaSuccess;
}
