// CUDA kernels of the engine.
//
// ldo_mc_kernel: one warp per replica.  The warp copies the replica's state
// (LdoLayout bytes) from the global arena into its slice of dynamic shared
// memory with 16-byte vector loads, one lane runs the move loop on it, and the
// warp writes it back.  Modes: initialise a replica from its loaded
// configuration (OrigamiSystem constructor: set_all_domains + order
// parameters + biases), recompute its energy after a table change
// (OrigamiSystem::update_temp), and run n_steps move attempts
// (GCMCSimulation::simulate), optionally recording order-parameter samples,
// a per-step trace and the PT dependent quantities.
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_engine.cuh"
#include "ldo_kernels.h"
#include "ldo_bind.cuh"

namespace {

template <class C>
__host__ __device__ constexpr int rep_bytes() { return (int)((sizeof(ldo::Rep<C>) + 15) / 16 * 16); }
template <class C>
__host__ __device__ constexpr int warp_bytes() { return rep_bytes<C>(); }

// Bytes of the replica state that snapshots hold (everything before the move
// statistics), and the distance between a replica's snapshots.
template <class C>
__host__ __device__ constexpr int snap_bytes() { return (int)offsetof(LdoState<C>, mstat); }
template <class C>
__host__ __device__ constexpr size_t snap_stride() { return (sizeof(LdoState<C>) + 255) / 256 * 256; }
static_assert(ldo::N_SNAPSHOTS == LDO_N_SNAPSHOTS, "snapshot count shared with the host");

// The warp's part of a step: the copies a move phase asked for (cmd), with
// the bookkeeping fields of the header kept across a restore.
template <class C>
__device__ __forceinline__ void snapshot_ops(int cmd, ldo::Rep<C>* R, unsigned char* base, unsigned char* snap,
                                             int lane) {
    static_assert(snap_bytes<C>() % 16 == 0, "snapshot region must be whole 16-byte vectors");
    int sn = (cmd & 15) - 1;
    int rs = ((cmd >> 4) & 15) - 1;
    LdoHdr& h = R->hdr;
    long long steps_done = 0;
    int sample_count = 0, status = 0, tab = 0;
    if (lane == 0 && rs >= 0) {
        steps_done = h.steps_done;
        sample_count = h.sample_count;
        status = h.status;
        tab = h.tab;
    }
    __syncwarp();
    if (sn >= 0 && !(cmd & ldo::CMD_REST_FIRST)) warp_copy16(snap + (size_t)sn * snap_stride<C>(), base, snap_bytes<C>(), lane);
    if (rs >= 0) warp_copy16(base, snap + (size_t)rs * snap_stride<C>(), snap_bytes<C>(), lane);
    if (sn >= 0 && (cmd & ldo::CMD_REST_FIRST)) warp_copy16(snap + (size_t)sn * snap_stride<C>(), base, snap_bytes<C>(), lane);
    __syncwarp();
    if (lane == 0 && rs >= 0) {
        h.steps_done = steps_done;
        h.sample_count = sample_count;
        h.status = status;
        h.tab = tab;
    }
}

// Shared memory per warp: Rep (replica state followed by the working fields).
// Lane 0 runs the moves; the whole warp loads and stores the state and
// copies the move snapshots (global memory, L.snap).
template <class C, bool CT>
__global__ void __launch_bounds__(128, 7) ldo_mc_kernel(LdoLaunch L) {
    extern __shared__ __align__(16) unsigned char smem[];
    int warp = threadIdx.x >> 5;
    int lane = threadIdx.x & 31;
    int slot = blockIdx.x * L.warps_per_block + warp;
    if (slot >= L.n_rep) return;
    int rep = L.rep_map ? L.rep_map[slot] : slot;
    if (L.only_rep >= 0 && rep != L.only_rep) return;
    unsigned char* base = smem + (size_t)warp * warp_bytes<C>();
    ldo::Rep<C>* R = reinterpret_cast<ldo::Rep<C>*>(base);
    unsigned char* gbase = L.arena + (size_t)rep * sizeof(LdoState<C>);
    warp_copy16(base, gbase, (int)sizeof(LdoState<C>), lane);
    __syncwarp();
    LdoHdr& h = R->hdr;
    long long nsteps = 0, sint = 0;
    double* tr = nullptr;
    bool live = false;
    if (lane == 0) {
        bind_rep<C>(*R, L, rep);
        live = h.status == 0;
        if (live) {
            if (L.mode == LDO_MODE_INIT) {
                R->set_all_current();
                R->init_biases();
                h.tab = R->ctl->tab;
            }
            else if (L.mode == LDO_MODE_RECOMPUTE) {
                R->recompute_energy();
                h.tab = R->ctl->tab;
            }
            else if (L.mode == LDO_MODE_OBSERVE) {
                // Reading observables changes nothing: the energy and the
                // dependent quantities use the tables the energy was last
                // computed with, even if the controls have moved since.
                R->bind_tables(L.tabs + h.tab);
            }
            else if (L.mode == LDO_MODE_COLLECT) {
                // training data of the learned insertion proposal: for every
                // bound or unbound domain, its network input and whether it
                // is bound
                R->bind_tables(L.tabs + h.tab);
                R->learn_collect(L.learn_cnt_b, L.learn_cnt_t);
            }
            else {
                if (L.force_recompute || h.tab != R->ctl->tab) {
                    R->recompute_energy();
                    h.tab = R->ctl->tab;
                }
                tr = (rep < L.n_trace) ? L.trace + (size_t)rep * L.trace_max * 8 : nullptr;
                long long unit = L.sweep_units ? (long long)R->ns : 1ll;
                nsteps = L.n_steps * unit;
                sint = (long long)L.sample_interval * unit;
            }
        }
    }
    nsteps = __shfl_sync(0xffffffffu, nsteps, 0);
    if (nsteps > 0) {
        unsigned char* snap = L.snap + (size_t)rep * ldo::N_SNAPSHOTS * snap_stride<C>();
        __syncwarp();
        warp_copy16(snap, base, snap_bytes<C>(), lane);   // snapshot 0: state at the start of the move
        for (long long k = 0; k < nsteps; ++k) {
            int cmd = 0;
            if (lane == 0) cmd = R->bad() ? ldo::CMD_STOP : R->template step_begin<CT>(h.steps_done + 1);
            cmd = __shfl_sync(0xffffffffu, cmd, 0);
            if (cmd & ldo::CMD_STOP) break;
            // a step has at most four phases (CB: three, then the post-move work)
            #pragma unroll 1
            for (int guard = 0; guard < 8; ++guard) {
                if (cmd & 0xff) snapshot_ops<C>(cmd, R, base, snap, lane);
                if (!(cmd & ldo::CMD_MORE)) break;
                if (lane == 0) cmd = R->template step_resume<CT>();
                cmd = __shfl_sync(0xffffffffu, cmd, 0);
            }
            if (lane == 0) {
                if (cmd & ldo::CMD_MORE) R->fail(LDO_RS_INVARIANT);
                long long s = h.steps_done + 1;
                h.steps_done = s;
                if (tr && k < L.trace_max) {
                    double* t = tr + 8 * k;
                    t[0] = (double)s;
                    t[1] = h.energy;
                    t[2] = h.num_staples;
                    t[3] = h.num_fully;
                    t[4] = h.num_bound;
                    t[5] = h.num_stacked;
                    t[6] = h.move_bias * R->c_bias_mult;
                    t[7] = (double)R->rng.draws;
                }
                if (L.us_hist) {
                    int oq = R->sys->bias_op[L.us_bias];
                    if (R->op[2 * oq + 1]) {
                        int x = R->op[2 * oq];
                        if (x >= 0 && x < L.us_len) L.us_hist[(size_t)L.us_window[rep] * L.us_len + x] += 1;
                    }
                }
                if (sint > 0 && s % sint == 0) {
                    int c = h.sample_count;
                    if (c < L.sample_cap) {
                        int16_t* o = L.samples + ((size_t)rep * L.sample_cap + c) * 2;
                        o[0] = (int16_t)h.num_fully;
                        o[1] = (int16_t)h.num_staples;
                    }
                    h.sample_count = c + 1;
                }
            }
        }
    }
    if (lane == 0 && live) {
        if (L.want_dep && !R->bad()) R->dependent_quantities();
        h.draws = R->rng.draws;
    }
    __syncwarp();
    warp_copy16(gbase, base, (int)sizeof(LdoState<C>), lane);
}

__global__ void ldo_status_kernel(const unsigned char* arena, int bytes, int o_hdr, int n_rep, int* out) {
    int rep = blockIdx.x * blockDim.x + threadIdx.x;
    if (rep >= n_rep) return;
    const LdoHdr* h = reinterpret_cast<const LdoHdr*>(arena + (size_t)rep * bytes + o_hdr);
    if (h->status != 0) atomicMax(out, h->status);
}

// One thread per ladder: the exchange attempts of one swap round between
// neighbouring control slots (OneDPTGCMCSimulation::attempt_exchange,
// src/ptmc_simulation.cpp:360-412, or the four-set T x stacking schedule of
// TwoDPTGCMCSimulation::attempt_exchange, :495-560), acceptance from
// calc_acceptance_p (:275-313) over staple types 1..S, and the master's
// control broadcast (master_send, :212).
__global__ void ldo_pt_swap_kernel(LdoPT P) {
    int lad = blockIdx.x * blockDim.x + threadIdx.x;
    if (lad >= P.n_ladders) return;
    int* perm = P.perm + (size_t)lad * P.n_rungs;
    if (P.hist_perm && P.hist_cap > 0) {
        long long k = P.hist_n[lad];
        size_t row = (size_t)(k % P.hist_cap) * P.n_ladders + lad;
        for (int q = 0; q < P.n_rungs; ++q) P.hist_perm[row * P.n_rungs + q] = perm[q];
        const LdoHdr* h0 = reinterpret_cast<const LdoHdr*>(P.arena + (size_t)perm[0] * P.lay.bytes + P.lay.o_hdr);
        P.hist_step[row] = h0->steps_done;
        P.hist_n[lad] = k + 1;
    }
    ldo::Rng rng;
    rng.init(P.seed, (uint32_t)lad, 1u, P.draws[lad]);
    int set = P.swap_i;
    for (int q = P.set_start[set]; q < P.set_start[set + 1]; ++q) {
        int i = P.pair_a[q], i2 = P.pair_b[q], ctr = P.pair_ctr[q];
        atomicAdd((unsigned long long*)&P.att[ctr], 1ull);
        double temp1 = P.slot_temp[i], temp2 = P.slot_temp[i2];
        double sm1 = P.slot_stack[i], sm2 = P.slot_stack[i2];
        int r1 = perm[i], r2 = perm[i2];
        const LdoHdr* h1 = reinterpret_cast<const LdoHdr*>(P.arena + (size_t)r1 * P.lay.bytes + P.lay.o_hdr);
        const LdoHdr* h2 = reinterpret_cast<const LdoHdr*>(P.arena + (size_t)r2 * P.lay.bytes + P.lay.o_hdr);
        const int16_t* n1 = reinterpret_cast<const int16_t*>(P.arena + (size_t)r1 * P.lay.bytes + P.lay.o_type_count);
        const int16_t* n2 = reinterpret_cast<const int16_t*>(P.arena + (size_t)r2 * P.lay.bytes + P.lay.o_type_count);
        double bias1 = h1->move_bias * P.ctl[r1].bias_mult;
        double bias2 = h2->move_bias * P.ctl[r2].bias_mult;
        double dbu_dn = 0;
        for (int t = 1; t < P.n_types; ++t) {
            double u1 = P.red_u[t - 1] * P.rep_q[4 * r1 + 0] * P.rep_q[4 * r1 + 1];
            double u2 = P.red_u[t - 1] * P.rep_q[4 * r2 + 0] * P.rep_q[4 * r2 + 1];
            double N1 = n1[t], N2 = n2[t];
            dbu_dn += (u2 / temp2 - u1 / temp1) * (N2 - N1);
        }
        double DB = 1 / temp2 - 1 / temp1;
        double DH = h2->H * temp2 - h1->H * temp1;
        double Dst = h2->stacking * temp2 - h1->stacking * temp1;
        double DBM = sm2 / temp2 - sm1 / temp1;
        double DBias = bias2 * temp2 - bias1 * temp1;
        double p = fmin(1.0, exp(DB * (DH + DBias) + DBM * Dst - dbu_dn));
        bool accept = (p == 1) ? true : (p > rng.uniform_real());
        if (accept) {
            atomicAdd((unsigned long long*)&P.acc[ctr], 1ull);
            perm[i] = r2;
            perm[i2] = r1;
        }
    }
    P.draws[lad] = rng.draws;
    // master_send: each replica takes the exchanged controls of its slot.
    // Temperature is exchanged by every variant, so the replica at slot k uses
    // the table set of slot k.
    for (int k = 0; k < P.n_rungs; ++k) {
        int r = perm[k];
        double* q = P.rep_q + 4 * r;
        if (P.exchange_q & 1) q[0] = P.slot_temp[k];
        if (P.exchange_q & 2) q[1] = P.slot_u[k];
        if (P.exchange_q & 4) q[2] = P.slot_bias[k];
        if (P.exchange_q & 8) q[3] = P.slot_stack[k];
        P.ctl[r].tab = P.tab_slot[k];
        P.ctl[r].staple_u_mult = q[1];
    }
}

} // namespace

cudaError_t ldo_launch_pt_swap(const LdoPT& P, cudaStream_t stream) {
    int threads = 128;
    int blocks = (P.n_ladders + threads - 1) / threads;
    ldo_pt_swap_kernel<<<blocks, threads, 0, stream>>>(P);
    return cudaGetLastError();
}

template <class C, bool CT>
static cudaError_t launch_mc_variant(const LdoLaunch& L, cudaStream_t stream) {
    int wpb = L.warps_per_block;
    size_t smem = (size_t)wpb * warp_bytes<C>() + (size_t)L.smem_pad;
    cudaError_t err =
        cudaFuncSetAttribute(ldo_mc_kernel<C, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int blocks = (L.n_rep + wpb - 1) / wpb;
    ldo_mc_kernel<C, CT><<<blocks, wpb * 32, smem, stream>>>(L);
    return cudaGetLastError();
}

// The scaffold regrowth movetypes live in their own kernel variant (the
// one with working memory): compiled into the staple-move kernel, their code
// made it 13 % slower (its time is instruction fetch).
template <class C>
static cudaError_t launch_mc_class(const LdoLaunch& L, cudaStream_t stream) {
    return L.ct_ws ? launch_mc_variant<C, true>(L, stream) : launch_mc_variant<C, false>(L, stream);
}

cudaError_t ldo_launch_mc(const LdoLaunch& L, cudaStream_t stream) {
    switch (L.lay.cls) {
    case LDO_CLASS_S: return launch_mc_class<LdoCapS>(L, stream);
    case LDO_CLASS_M: return launch_mc_class<LdoCapM>(L, stream);
    default: return launch_mc_class<LdoCapL>(L, stream);
    }
}

template <class C, bool CT>
static cudaError_t occupancy_variant(int wpb, size_t smem, int* blocks) {
    cudaError_t err =
        cudaFuncSetAttribute(ldo_mc_kernel<C, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, ldo_mc_kernel<C, CT>, wpb * 32, smem);
}

cudaError_t ldo_mc_occupancy(int cls, int ct, int wpb, size_t smem, int* blocks) {
    switch (cls) {
    case LDO_CLASS_S:
        return ct ? occupancy_variant<LdoCapS, true>(wpb, smem, blocks) : occupancy_variant<LdoCapS, false>(wpb, smem, blocks);
    case LDO_CLASS_M:
        return ct ? occupancy_variant<LdoCapM, true>(wpb, smem, blocks) : occupancy_variant<LdoCapM, false>(wpb, smem, blocks);
    default:
        return ct ? occupancy_variant<LdoCapL, true>(wpb, smem, blocks) : occupancy_variant<LdoCapL, false>(wpb, smem, blocks);
    }
}

int ldo_warp_smem_bytes(int cls) {
    switch (cls) {
    case LDO_CLASS_S: return warp_bytes<LdoCapS>();
    case LDO_CLASS_M: return warp_bytes<LdoCapM>();
    default: return warp_bytes<LdoCapL>();
    }
}

__global__ void ldo_exp_kernel(const double* x, double* y, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = ldo::dexp(x[i]);
}

cudaError_t ldo_launch_exp(const double* x, double* y, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    ldo_exp_kernel<<<(n + 255) / 256, 256, 0, stream>>>(x, y, n);
    return cudaGetLastError();
}

size_t ldo_ct_work_bytes(int cls) {
    size_t b;
    switch (cls) {
    case LDO_CLASS_S: b = sizeof(LdoCtWork<LdoCapS>); break;
    case LDO_CLASS_M: b = sizeof(LdoCtWork<LdoCapM>); break;
    default: b = sizeof(LdoCtWork<LdoCapL>); break;
    }
    return (b + 255) / 256 * 256;
}

cudaError_t ldo_launch_status(const unsigned char* arena, int bytes, int o_hdr, int n_rep, int* d_out,
                              cudaStream_t stream) {
    int threads = 256;
    int blocks = (n_rep + threads - 1) / threads;
    ldo_status_kernel<<<blocks, threads, 0, stream>>>(arena, bytes, o_hdr, n_rep, d_out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free status read-out.
//
// Some callers may not allocate device memory when they ask for the replicas'
// status: a host program that hands all device memory to its own pool
// allocator (a cudaMalloc outside the pool breaks its budget and its
// accounting), and a step loop that must not stall the device (cudaMalloc and
// cudaFree can synchronise the whole device and wait on other streams' work).
// This variant of ldo_status_kernel therefore keeps its scratch in a fixed
// device array that every GPU loading the library holds until the process
// exits: [0] largest status code, [1] number of replicas with a nonzero
// status (both must start at zero and are cleared by every call), then one
// status word per replica (overwritten by every call).  256 KiB + 8 bytes.
static __device__ __align__(256) int g_status_scratch[2 + LDO_NOALLOC_MAX_REPLICAS];

namespace {

__global__ void ldo_status_gather_kernel(const unsigned char* arena, int bytes, int o_hdr, int n_rep,
                                         int* scratch) {
    int rep = blockIdx.x * blockDim.x + threadIdx.x;
    if (rep >= n_rep) return;
    const LdoHdr* h = reinterpret_cast<const LdoHdr*>(arena + (size_t)rep * bytes + o_hdr);
    int s = h->status;
    scratch[2 + rep] = s;
    if (s != 0) {
        atomicMax(&scratch[0], s);
        atomicAdd(&scratch[1], 1);
    }
}

// Device address of g_status_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress with the device current.  It is looked up on every
// call, not cached: after a device reset the module, and with it the array,
// can be loaded at another address.  The lookup allocates nothing.
cudaError_t scratch_on_current_device(int** out) {
    void* p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_status_scratch);
    if (err != cudaSuccess) return err;
    *out = static_cast<int*>(p);
    return cudaSuccess;
}

} // namespace

cudaError_t ldo_status_noalloc(const unsigned char* arena, int bytes, int o_hdr, int n_rep, cudaStream_t stream,
                               int* status_of_replica, int* worst, int* n_bad) {
    if (n_rep < 0 || n_rep > LDO_NOALLOC_MAX_REPLICAS) return cudaErrorInvalidValue;
    int* scratch = nullptr;
    cudaError_t err = scratch_on_current_device(&scratch);
    if (err != cudaSuccess) return err;
    err = cudaMemsetAsync(scratch, 0, 2 * sizeof(int), stream);
    if (err != cudaSuccess) return err;
    if (n_rep > 0) {
        int threads = 256;
        int blocks = (n_rep + threads - 1) / threads;
        ldo_status_gather_kernel<<<blocks, threads, 0, stream>>>(arena, bytes, o_hdr, n_rep, scratch);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    int cells[2] = {0, 0};
    err = cudaMemcpyAsync(cells, scratch, sizeof(cells), cudaMemcpyDeviceToHost, stream);
    if (err != cudaSuccess) return err;
    if (status_of_replica && n_rep > 0) {
        err = cudaMemcpyAsync(status_of_replica, scratch + 2, (size_t)n_rep * sizeof(int), cudaMemcpyDeviceToHost,
                              stream);
        if (err != cudaSuccess) return err;
    }
    err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return err;
    *worst = cells[0];
    *n_bad = cells[1];
    return cudaSuccess;
}
