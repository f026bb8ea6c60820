// Device helpers shared by the kernels of the engine's translation units:
// the warp's vector copy of a replica state and the binding of a replica's
// working object to its system, tables and controls.
#pragma once
#include "ldo_engine.cuh"
#include "ldo_kernels.h"

namespace {

__device__ __forceinline__ void warp_copy16(void* dst, const void* src, int bytes, int lane) {
    uint4* d = reinterpret_cast<uint4*>(dst);
    const uint4* s = reinterpret_cast<const uint4*>(src);
    int n = bytes >> 4;
    for (int k = lane; k < n; k += 32) d[k] = s[k];
}

template <class C>
__device__ void bind_rep(ldo::Rep<C>& r, const LdoLaunch& L, int rep) {
    r.ctl = L.ctl + rep;
    r.sys = L.sys + r.ctl->sys;
    r.bank = L.bank;
    r.grid = L.grid;
    r.learn_w = L.learn_w;
    r.ct = L.ct_ws ? reinterpret_cast<LdoCtWork<C>*>(L.ct_ws + (size_t)rep * L.ct_stride) : nullptr;
    r.bind_tables(L.tabs + r.ctl->tab);
    r.imax = r.sys->imax;
    r.dim = r.sys->dim;
    r.c_staple_M = r.ctl->staple_M;
    r.c_bias_mult = r.ctl->bias_mult;
    r.ns = r.sys->ns;
    r.lmax = r.sys->lmax;
    r.nmv = r.sys->n_moves;
    r.cyclic = r.sys->cyclic;
    r.tqt = r.sys->tqt;
    r.mean_field = r.sys->mean_field;
    r.log6 = log(6.0);
    r.log3 = log(3.0);
    r.rng.init(r.ctl->seed, r.ctl->rep, 0u, r.hdr.draws);
}

} // namespace
