// Exact staple-only enumeration kernel (csrc/ldo_enum.cuh).  It lives in its
// own translation unit: compiled beside the MC kernel, its calls into the
// replica's methods changed the compiler's inlining there and grew the MC
// kernel's code by a tenth (that kernel is bound by instruction fetch).
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_bind.cuh"
#include "ldo_enum.cuh"

namespace {

template <class C>
__host__ __device__ constexpr int enum_smem_bytes() { return (int)((sizeof(ldo::Rep<C>) + 15) / 16 * 16); }

// One block per part of an enumeration unit (a unit is split into 6^split
// parts by the branch taken at each of its first `split` choice levels);
// its first lane runs the recursion on the replica state in shared memory
// (the other lanes only copy it in).
template <class C>
__global__ void __launch_bounds__(32) ldo_enum_kernel(LdoEnumLaunch E) {
    extern __shared__ __align__(16) unsigned char smem[];
    int parts = 1;
    for (int k = 0; k < E.split; ++k) parts *= 6;
    int b = blockIdx.x;
    int u = b / parts;
    int lane = threadIdx.x;
    if (u >= E.n_units) return;
    warp_copy16(smem, E.state, (int)sizeof(LdoState<C>), lane);
    __syncwarp();
    if (lane != 0) return;
    ldo::Rep<C>* R = reinterpret_cast<ldo::Rep<C>*>(smem);
    bind_rep<C>(*R, E.L, 0);
    auto* W = reinterpret_cast<ldo::EnumWork<C>*>(E.work + (size_t)b * E.work_stride);
    const LdoEnumUnit& U = E.units[u];
    for (int d = 0; d < C::DCAP; ++d) {
        W->gp_of[d] = -1;
        W->inv_gp[d] = -1;
        W->zero_ore[d] = 0;
    }
    W->sp = 0;
    W->npgp = 0;
    W->E = 0;
    W->E_lo = 0;
    W->mult = 1;
    W->prefix = 1;
    W->part = 0;
    W->nconf = 0;
    W->sumE = 0;
    W->part_c = 0;
    W->sumE_c = 0;
    // E.hist holds 2 x n1 x n2 doubles per part: the part's weights, then
    // the compensations of their sums, folded into the weights at the end
    W->row = E.hist + (size_t)b * 2 * E.n1 * E.n2;
    for (int k = 0; k < 2 * E.n1 * E.n2; ++k) W->row[k] = 0;
    W->op1 = E.op1;
    W->op2 = E.op2;
    W->n1 = E.n1;
    W->n2 = E.n2;
    W->overcount = E.overcount;
    W->bad = 0;
    W->full = E.full;
    W->depth = 0;
    W->npre = E.split;
    for (int k = 0, r = b % parts; k < E.split; ++k, r /= 6) W->pre[k] = (int8_t)(r % 6);
    // m_identities_to_num_unassigned: 1 for each scaffold identity
    // (ConformationalEnumerator's constructor, :203), then +1 per staple
    // domain (add_staple, :260)
    for (int k = 0; k < 2 * LDO_ENUM_MAX_IDENT + 1; ++k) W->cnt[k] = 0;
    for (int d = 0; d < R->ns; ++d) W->cnt[R->did[d] + LDO_ENUM_MAX_IDENT] = 1;
    // ConformationalEnumerator::add_staple (src/enumerate.cpp:260)
    int cs[LDO_ENUM_MAX_STAPLES];
    for (int k = 0; k < U.n_chains; ++k) {
        W->prefix *= R->c_staple_M;
        cs[k] = R->add_chain(U.ident[k]);
        if (R->mean_field) W->E += R->log6;   // (at most eight terms: no drift to speak of)
        W->E += R->t_init_e;
        int len = R->sys->type_len[U.ident[k]];
        if (!R->bad())
            for (int q = 0; q < len; ++q) W->cnt[R->did[R->slot_of(cs[k], q)] + LDO_ENUM_MAX_IDENT] += 1;
        double six = 1;
        for (int q = 0; q < 2 * len - 1; ++q) six *= 6.0;
        W->prefix /= six;
    }
    if (!R->bad()) {
        for (int g = 0; g < U.n_gp; ++g) {
            int oc = U.gp_old_chain[g];
            int old = oc < 0 ? U.gp_old_dom[g] : R->slot_of(cs[oc], U.gp_old_dom[g]);
            W->gp_of[old] = (int16_t)R->slot_of(cs[U.gp_new_chain[g]], U.gp_new_dom[g]);
        }
        ldo::Enumerator<C> en {*R, *W};
        if (E.full) en.run_full();
        else en.run();
    }
    // the compensated sums, folded
    for (int k = 0; k < E.n1 * E.n2; ++k) W->row[k] += W->row[E.n1 * E.n2 + k];
    double* st = E.stats + 4 * (size_t)b;
    st[0] = W->part + W->part_c;
    st[1] = W->nconf;
    st[2] = W->sumE + W->sumE_c;
    st[3] = R->bad() ? (double)R->hdr.status : (W->bad ? -1.0 : 0.0);
}

} // namespace

template <class C>
static cudaError_t launch_enum_class(const LdoEnumLaunch& E, cudaStream_t stream) {
    size_t smem = (size_t)enum_smem_bytes<C>();
    cudaError_t err = cudaFuncSetAttribute(ldo_enum_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    long long parts = 1;
    for (int k = 0; k < E.split; ++k) parts *= 6;
    long long blocks = (long long)E.n_units * parts;
    if (E.split < 0 || E.split > LDO_ENUM_MAX_SPLIT || blocks > 0x7fffffffll) return cudaErrorInvalidValue;
    if (blocks > 0) ldo_enum_kernel<C><<<(unsigned)blocks, 32, smem, stream>>>(E);
    return cudaGetLastError();
}

cudaError_t ldo_launch_enum(const LdoEnumLaunch& E, cudaStream_t stream) {
    switch (E.L.lay.cls) {
    case LDO_CLASS_S: return launch_enum_class<LdoCapS>(E, stream);
    case LDO_CLASS_M: return launch_enum_class<LdoCapM>(E, stream);
    default: return launch_enum_class<LdoCapL>(E, stream);
    }
}

size_t ldo_enum_work_bytes(int cls) {
    size_t b;
    switch (cls) {
    case LDO_CLASS_S: b = sizeof(ldo::EnumWork<LdoCapS>); break;
    case LDO_CLASS_M: b = sizeof(ldo::EnumWork<LdoCapM>); break;
    default: b = sizeof(ldo::EnumWork<LdoCapL>); break;
    }
    return (b + 255) / 256 * 256;
}

