// Network of the learned insertion proposal: 64 -> 256 -> 256 -> 256 -> 1,
// GELU, bf16 weights and activations as tensor-core operands (tcgen05),
// fp32 accumulation and fp32 master weights (Adam).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_learn.h"

// Device workspace for batches of up to `cap` inputs.
struct LdoMlp {
    int cap {0};
    float* params {nullptr};     // [NPARAM] fp32 master weights
    float* grad {nullptr};       // [NPARAM]
    float* adam_m {nullptr};
    float* adam_v {nullptr};
    uint16_t* wbf {nullptr};     // bf16 weight copies, both orientations (ldo_mlp.cu)
    int32_t* idx {nullptr};      // [cap] table entries of the batch
    float* cnt_b {nullptr};      // [cap] bound counts
    float* cnt_t {nullptr};      // [cap] total counts
    uint16_t* x {nullptr};       // [cap][64] bf16
    float* z[3] {};              // [cap][256] pre-activations
    uint16_t* h[3] {};           // [cap][256] bf16 activations
    float* dz {nullptr};         // [cap][256] fp32 gradient scratch
    uint16_t* gbf {nullptr};     // [cap][256] bf16 gradient
    uint16_t* ht {nullptr};      // [256][cap] transposed activation (weight-gradient operand)
    uint16_t* gt {nullptr};      // [256][cap] transposed gradient
    int* err {nullptr};          // set if a tensor-core wait ran out (ldo_umma.cuh)
    float* out {nullptr};        // [cap] logits
    float* dout {nullptr};       // [cap]
    double* loss {nullptr};      // [1]
    long long adam_t {0};
};

cudaError_t ldo_mlp_alloc(LdoMlp& m, int cap);
void ldo_mlp_free(LdoMlp& m);
// Refresh the bf16 weight copies from the fp32 parameters.
cudaError_t ldo_mlp_sync_weights(LdoMlp& m, cudaStream_t s);
// Forward pass over m.idx[0..n) (logits in m.out).
cudaError_t ldo_mlp_forward(LdoMlp& m, int n, cudaStream_t s);
// Loss (sum over the batch of cnt_t*softplus(z) - cnt_b*z, divided by
// `norm`) into m.loss and its gradient into m.grad.
cudaError_t ldo_mlp_loss_grad(LdoMlp& m, int n, double norm, cudaStream_t s);
// One Adam step on m.params with m.grad.
cudaError_t ldo_mlp_adam(LdoMlp& m, float lr, cudaStream_t s);
// Weights exp(clamp(logit)) of every table entry (LDO_LEARN_TABLE doubles),
// evaluated in batches of m.cap.
cudaError_t ldo_mlp_table(LdoMlp& m, double* table, cudaStream_t s);
// Synchronises s and reports whether a tensor-core wait ran out since the
// last check (then the products are incomplete).
cudaError_t ldo_mlp_check(LdoMlp& m, cudaStream_t s, bool* timed_out);
