// Launch interface between the host library and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ldo_types.h"

enum { LDO_MODE_RUN = 0, LDO_MODE_INIT = 1, LDO_MODE_RECOMPUTE = 2, LDO_MODE_OBSERVE = 3, LDO_MODE_COLLECT = 4 };

struct LdoLaunch {
    const LdoSys* sys;
    const LdoTab* tabs;
    const double* bank;
    const LdoRepCtl* ctl;
    const double* grid;
    unsigned char* arena;
    // Move snapshots, LDO_N_SNAPSHOTS per replica, each ldo_snapshot_stride
    // bytes apart (run mode).
    unsigned char* snap;
    LdoLayout lay;
    int n_rep;
    int only_rep;                // >= 0: only this replica runs (configuration import)
    int warps_per_block;
    int smem_pad;                // extra dynamic shared memory per block (occupancy tuning)
    int mode;
    int want_dep;
    int force_recompute;
    int sweep_units;             // n_steps and sample_interval count sweeps of n_scaffold steps
    long long n_steps;
    int sample_interval, sample_cap;
    int16_t* samples;
    int n_trace, trace_max;
    double* trace;
    // Umbrella-sampling visit histogram (USGCMCSimulation::update_internal,
    // src/us_simulation.cpp:262): after every step the grid order parameter of
    // bias function us_bias is counted in us_hist[window * us_len + value].
    int* us_hist;
    const int* us_window;        // [n_rep] window held by each replica
    int us_bias, us_len;
    // Learned insertion proposal: weight exp(logit) of every network input
    // (LDO_LEARN_TABLE entries), read by LearnedStapleExchange.
    const double* learn_w;
    double* learn_cnt_b;         // collect mode: bound / total counts per network input
    double* learn_cnt_t;
    // Scaffold regrowth working memory, ct_stride bytes per replica (null
    // when no system regrows its scaffold).
    unsigned char* ct_ws;
    size_t ct_stride;
    // Warp w of the grid runs replica rep_map[w] (null: replica w).  The
    // autotuner's replica order: which replicas share a block and an SM.
    const int* rep_map;
};

cudaError_t ldo_launch_mc(const LdoLaunch& L, cudaStream_t stream);
// Resident blocks per SM of the MC kernel of class cls (ct: the scaffold-
// move variant) with wpb warps per block and smem bytes of dynamic shared
// memory per block, from the CUDA occupancy calculator.
cudaError_t ldo_mc_occupancy(int cls, int ct, int wpb, size_t smem, int* blocks);
enum { LDO_N_SNAPSHOTS = 3 };
// Bytes between a replica's move snapshots for a state of lay.bytes bytes.
inline size_t ldo_snapshot_stride(int state_bytes) { return ((size_t)state_bytes + 255) / 256 * 256; }
// Shared memory one replica's warp needs in capacity class cls.
int ldo_warp_smem_bytes(int cls);
// Bytes of one replica's scaffold regrowth working memory in class cls.
size_t ldo_ct_work_bytes(int cls);
// y[i] = the engine's exponential (ldo_math::exp) of x[i], on the device.
cudaError_t ldo_launch_exp(const double* x, double* y, int n, cudaStream_t stream);
cudaError_t ldo_launch_status(const unsigned char* arena, int bytes, int o_hdr, int n_rep, int* d_out,
                              cudaStream_t stream);

// Parallel-tempering exchange state (PTGCMCSimulation, src/ptmc_simulation.cpp).
struct LdoPT {
    int n_ladders, n_rungs;
    int exchange_q;              // bit set: 1 T, 2 staple u, 4 bias mult, 8 stacking mult
    int n_types;                 // staple types + 1
    const double* slot_temp;     // [n_rungs] control quantities by slot
    const double* slot_u;
    const double* slot_bias;
    const double* slot_stack;
    const double* red_u;         // [n_types-1] reduced staple chemical potentials
    int* perm;                   // [n_ladders * n_rungs] slot -> replica
    double* rep_q;               // [n_rep * 4] per-replica temp, u mult, bias mult, stack mult
    const int* tab_slot;         // [n_rungs] table set used at each slot
    LdoRepCtl* ctl;
    const unsigned char* arena;
    LdoLayout lay;
    unsigned long long* draws;   // [n_ladders] swap stream counters
    long long* att;              // [n_counters] attempts / accepts per pair counter
    long long* acc;
    uint32_t seed;
    int swap_i;                  // pair set of this round (swap counter mod n_sets)
    // Pair schedule: set s holds the slot pairs (pair_a[q], pair_b[q]) for
    // q in [set_start[s], set_start[s+1]), in the reference's loop order,
    // each with its attempt/accept counter pair_ctr[q].
    int n_sets;
    const int* set_start;
    const int* pair_a;
    const int* pair_b;
    const int* pair_ctr;
    // Swap history for the .swp file (PTGCMCSimulation::write_swap_entry,
    // src/ptmc_simulation.cpp:315): before its exchange attempts each ladder
    // stores its permutation (slot -> replica) and step count in row
    // hist_n[ladder] % hist_cap and counts the row (null: not recorded).
    int* hist_perm;              // [hist_cap][n_ladders][n_rungs]
    long long* hist_step;        // [hist_cap][n_ladders]
    long long* hist_n;           // [n_ladders]
    long long hist_cap;
};
cudaError_t ldo_launch_pt_swap(const LdoPT& P, cudaStream_t stream);

// Allocation-free status read-out.  The reduction cells and the per-replica
// copy live in a fixed device array inside the library instead of engine
// buffers, so the call allocates no memory.  At most LDO_NOALLOC_MAX_REPLICAS
// replicas.  Every call looks up the array's device address with the device
// current (not cached: a device reset can move it).  Every call uses the same array: calls
// whose work overlaps on the GPU race.  Copies the results to host memory and
// synchronises `stream` before returning.
enum { LDO_NOALLOC_MAX_REPLICAS = 65536 };
cudaError_t ldo_status_noalloc(const unsigned char* arena, int bytes, int o_hdr, int n_rep, cudaStream_t stream,
                               int* status_of_replica, int* worst, int* n_bad);

// Exact staple-only enumeration (csrc/ldo_enum.cuh).  One work unit: the
// staples added (identities in the reference's add order) and the
// growth-point map (old domain -> new staple domain) as the reference's
// m_growthpoints holds it when its conformational enumeration starts.  A
// domain reference is (chain, domain index) with chain -1 for the scaffold
// and k for the k-th added staple.
#define LDO_ENUM_MAX_STAPLES 8
// domain identities |d_ident| <= LDO_ENUM_MAX_IDENT keep an unassigned count
#define LDO_ENUM_MAX_IDENT 64
// choice levels a unit can be split at (6 branches each)
#define LDO_ENUM_MAX_SPLIT 4
struct LdoEnumUnit {
    int n_chains;
    int ident[LDO_ENUM_MAX_STAPLES];
    int n_gp;
    int gp_old_chain[LDO_ENUM_MAX_STAPLES];
    int gp_old_dom[LDO_ENUM_MAX_STAPLES];
    int gp_new_chain[LDO_ENUM_MAX_STAPLES];
    int gp_new_dom[LDO_ENUM_MAX_STAPLES];
};
struct LdoEnumLaunch {
    LdoLaunch L;                  // system, tables and controls of replica 0
    const unsigned char* state;   // the replica's state with the scaffold placed and no staples
    const LdoEnumUnit* units;
    int n_units;
    int full;                     // 1: the scaffold is enumerated too (ConformationalEnumerator::enumerate)
    int split;                    // each unit runs as 6^split parts, one per branch of its first choice levels
    unsigned char* work;          // per part: recursion state (ldo_enum_work_bytes)
    size_t work_stride;
    double* hist;                 // per part: n1 x n2 weights over (op1, op2)
    double* stats;                // per part: partition sum, configurations, sum of E w, status
    int op1, op2, n1, n2;
    int overcount;                // 0 MaxTwoDomain, 1 MisbindingOnly
};
cudaError_t ldo_launch_enum(const LdoEnumLaunch& E, cudaStream_t stream);
size_t ldo_enum_work_bytes(int cls);
