// Kernels of the learned-proposal network (ldo_mlp.h).
//
// Matrix products run on the tensor cores as bf16 x bf16 -> fp32 warp MMAs
// (m16n8k16) over 64x64 output tiles staged through shared memory; every
// other step (bias, GELU and its derivative, the 256 -> 1 output layer, the
// loss, column sums, Adam) is an elementwise or reduction kernel in fp32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_mlp.h"

namespace {

constexpr int H = LDO_LEARN_H;
constexpr int DIN = LDO_LEARN_DIN;
// bf16 weight copies: W1 [DIN][H], W2 [H][H], W3 [H][H], w4 [H]
constexpr int BF_W1 = 0;
constexpr int BF_W2 = BF_W1 + DIN * H;
constexpr int BF_W3 = BF_W2 + H * H;
constexpr int BF_W4 = BF_W3 + H * H;
constexpr int BF_N = BF_W4 + H;

__device__ __forceinline__ uint16_t f2bf(float f) {
    __nv_bfloat16 b = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t*>(&b);
}
__device__ __forceinline__ float bf2f(uint16_t u) {
    return __uint_as_float(((unsigned)u) << 16);
}

// ---------------------------------------------------------------- GEMM ---
// C[M][N] (fp32, row-major) = op(A) * op(B), bf16 operands.
// TA = 0: A is [M][K] row-major; TA = 1: A is stored [K][M] row-major.
// TB = 0: B is [K][N] row-major; TB = 1: B is stored [N][K] row-major.
constexpr int GT_M = 64, GT_N = 64, GT_K = 32, GT_PAD = 8;

template <int TA, int TB>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                        float* __restrict__ C, int M, int N, int K) {
    __shared__ __align__(16) uint16_t As[GT_M][GT_K + GT_PAD];   // [m][k]
    __shared__ __align__(16) uint16_t Bs[GT_N][GT_K + GT_PAD];   // [n][k]
    int tid = threadIdx.x;
    int warp = tid >> 5, lane = tid & 31;
    int g = lane >> 2, c = lane & 3;
    int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
    #pragma unroll
    for (int i = 0; i < 2; ++i)
        #pragma unroll
        for (int j = 0; j < 4; ++j)
            #pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k0 = 0; k0 < K; k0 += GT_K) {
        // stage the A and B tiles (consecutive threads read consecutive addresses)
        for (int e = tid; e < GT_M * GT_K; e += 128) {
            int m, k;
            if (TA == 0) { m = e / GT_K; k = e % GT_K; }
            else { k = e / GT_M; m = e % GT_M; }
            int gm = m0 + m, gk = k0 + k;
            uint16_t v = 0;
            if (gm < M && gk < K) v = TA == 0 ? A[(size_t)gm * K + gk] : A[(size_t)gk * M + gm];
            As[m][k] = v;
        }
        for (int e = tid; e < GT_N * GT_K; e += 128) {
            int n, k;
            if (TB == 0) { k = e / GT_N; n = e % GT_N; }
            else { n = e / GT_K; k = e % GT_K; }
            int gn = n0 + n, gk = k0 + k;
            uint16_t v = 0;
            if (gn < N && gk < K) v = TB == 0 ? B[(size_t)gk * N + gn] : B[(size_t)gn * K + gk];
            Bs[n][k] = v;
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < GT_K; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
            #pragma unroll
            for (int i = 0; i < 2; ++i) {
                int r = wm + i * 16 + g;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * c]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * c]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 8 + 2 * c]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 8 + 2 * c]);
            }
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                int n = wn + j * 8 + g;
                bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[n][kk + 2 * c]);
                bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[n][kk + 8 + 2 * c]);
            }
            #pragma unroll
            for (int i = 0; i < 2; ++i)
                #pragma unroll
                for (int j = 0; j < 4; ++j)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
                        : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]),
                          "r"(bfr[j][1]));
        }
        __syncthreads();
    }
    #pragma unroll
    for (int i = 0; i < 2; ++i)
        #pragma unroll
        for (int j = 0; j < 4; ++j) {
            int r = m0 + wm + i * 16 + g;
            int col = n0 + wn + j * 8 + 2 * c;
            if (r < M) {
                if (col < N) C[(size_t)r * N + col] = acc[i][j][0];
                if (col + 1 < N) C[(size_t)r * N + col + 1] = acc[i][j][1];
            }
            if (r + 8 < M) {
                if (col < N) C[(size_t)(r + 8) * N + col] = acc[i][j][2];
                if (col + 1 < N) C[(size_t)(r + 8) * N + col + 1] = acc[i][j][3];
            }
        }
}

template <int TA, int TB>
cudaError_t gemm(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K, cudaStream_t s) {
    dim3 grid((N + GT_N - 1) / GT_N, (M + GT_M - 1) / GT_M);
    gemm_bf16_kernel<TA, TB><<<grid, 128, 0, s>>>(A, B, C, M, N, K);
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

__global__ void add_kernel(float* dst, const float* src, int n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) dst[e] += src[e];
}

__global__ void to_bf16_kernel(const float* p, uint16_t* wbf) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < DIN * H) wbf[BF_W1 + e] = f2bf(p[LDO_LEARN_OFF_W1 + e]);
    if (e < H * H) {
        wbf[BF_W2 + e] = f2bf(p[LDO_LEARN_OFF_W2 + e]);
        wbf[BF_W3 + e] = f2bf(p[LDO_LEARN_OFF_W3 + e]);
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
                  m.h[0], m.h[1], m.h[2], m.dz, m.gbf, m.out, m.dout, m.loss};
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
    MLP_CU((gemm<0, 0>(m.x, m.wbf + BF_W1, m.z[0], n, H, DIN, s)));
    bias_gelu_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.z[0], m.params + LDO_LEARN_OFF_B1, m.h[0], tot);
    MLP_CU((gemm<0, 0>(m.h[0], m.wbf + BF_W2, m.z[1], n, H, H, s)));
    bias_gelu_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.z[1], m.params + LDO_LEARN_OFF_B2, m.h[1], tot);
    MLP_CU((gemm<0, 0>(m.h[1], m.wbf + BF_W3, m.z[2], n, H, H, s)));
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
    MLP_CU((gemm<1, 0>(m.h[1], m.gbf, m.grad + LDO_LEARN_OFF_W3, H, H, n, s)));
    MLP_CU((gemm<0, 1>(m.gbf, m.wbf + BF_W3, m.dz, n, H, H, s)));
    gelu_back_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.dz, m.z[1], m.gbf, tot);
    // layer 2
    colsum_kernel<<<rb, H, 0, s>>>(m.dz, n, m.grad + LDO_LEARN_OFF_B2);
    MLP_CU((gemm<1, 0>(m.h[0], m.gbf, m.grad + LDO_LEARN_OFF_W2, H, H, n, s)));
    MLP_CU((gemm<0, 1>(m.gbf, m.wbf + BF_W2, m.dz, n, H, H, s)));
    gelu_back_kernel<<<blocks_for(tot, 256), 256, 0, s>>>(m.dz, m.z[0], m.gbf, tot);
    // layer 1
    colsum_kernel<<<rb, H, 0, s>>>(m.dz, n, m.grad + LDO_LEARN_OFF_B1);
    MLP_CU((gemm<1, 0>(m.x, m.gbf, m.grad + LDO_LEARN_OFF_W1, DIN, H, n, s)));
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
