// Plain-data descriptors shared by the host library and the CUDA kernels.
//
// LdoSys      one origami system: chain types and identities, movetypes,
//             order parameters and bias functions (what the reference keeps in
//             OrigamiSystem, GCMCSimulation, SystemOrderParams, SystemBiases).
// LdoTab      one set of energy tables for one (temperature, stacking
//             multiplier), built on the host the way OrigamiPotential::
//             calc_energies does (src/origami_potential.cpp:1057).
// LdoRepCtl   per-replica controls (system, table set, window restraints).
// LdoLayout   byte offsets of one replica's state; the same bytes live in the
//             global arena between launches and in shared memory during one.
// LdoHdr      scalar part of a replica's state.
#pragma once
#include <stdint.h>

#define LDO_MAX_TYPES 96
#define LDO_MAX_IDENTS 1024
#define LDO_MAX_MOVES 8
#define LDO_MAX_OPS 16
#define LDO_MAX_BIASES 4
#define LDO_MAX_PARTS 4
#define LDO_MAX_LEN 4
#define LDO_MAX_KMAX 63
#define LDO_MAX_SCAF 320

enum LdoMove {
    LDO_MV_ORIENT = 0,
    LDO_MV_MET_EXCHANGE = 1,
    LDO_MV_MET_REGROWTH = 2,
    LDO_MV_CB_REGROWTH = 3,
    LDO_MV_LEARNED_EXCHANGE = 4,  // engine extension: exchange with the learned insertion proposal
    // conserved-topology scaffold regrowth
    LDO_MV_CTRG = 5,              // CTRGScaffoldRegrowth
    LDO_MV_CTRG_JUMP = 6,         // CTRGJumpScaffoldRegrowth
    LDO_MV_CTCB = 7,              // CTCBScaffoldRegrowth
    LDO_MV_CTCB_JUMP = 8,         // CTCBJumpScaffoldRegrowth
    LDO_MV_LEARNED_REGROWTH = 9,  // engine extension: Met regrowth with learned directions
    // scaffold transforms with linker regrowth (src/transform_movetypes.cpp)
    LDO_MV_CTCB_LINKER = 10,      // CTCBLinkerRegrowth
    LDO_MV_CTCB_CLINKER = 11,     // CTCBClusteredLinkerRegrowth
    LDO_MV_CTRG_LINKER = 12       // CTRGLinkerRegrowth
};
enum LdoMoveOpt {
    LDO_MO_MAX_REGROWTH = 0,
    LDO_MO_MAX_SEG_REGROWTH,
    LDO_MO_MAX_RECOILS,
    LDO_MO_MAX_C_ATTEMPTS,
    LDO_MO_MAX_DISP,          // linker movetypes: translation range per axis
    LDO_MO_MAX_TURNS,         // linker movetypes: quarter turns of the rotation
    LDO_MO_MAX_LINKER,        // linker movetypes: max_linker_length
    LDO_MO_NUM_TRANSFORMS,    // linker movetypes: trial transformations per configuration
    LDO_N_MOVE_OPTS
};
// trial transformations of a linker move kept for the Rosenbluth choice
#define LDO_CT_MAX_TRANSFORMS 32

enum LdoOp {
    LDO_OP_NUMSTAPLES = 0,
    LDO_OP_NUMSTAPLESTYPE,
    LDO_OP_STAPLETYPEFULLYBOUND,
    LDO_OP_NUMBOUND,
    LDO_OP_NUMMISBOUND,
    LDO_OP_NUMSTACKED,
    LDO_OP_ZERO,   // NumLinearHelices / NumStackedJuncts: never updated by the reference
    LDO_OP_SUM,
    LDO_OP_DIST,       // DistOrderParam: L1 distance of two scaffold domains (op_parts[q][0..1])
    LDO_OP_ADJACENT    // AdjacentSiteOrderParam: 1 if that distance is 1
};

enum LdoBias { LDO_B_LINEARSTEPWELL = 0, LDO_B_SQUAREWELL, LDO_B_GRID, LDO_B_HARMONIC };

// Replica status words (ldo_status values).
enum LdoRepStatus {
    LDO_RS_OK = 0,
    LDO_RS_INVARIANT = 4,
    LDO_RS_ITERCAP = 5,
    LDO_RS_CAPACITY = 6
};

struct LdoSys {
    int n_types;          // 1 + number of staple types
    int ns;               // scaffold domains
    int lmax;             // longest staple
    int kmax;             // staple chain slots
    int dcap;             // domain slots = ns + kmax * lmax
    int cyclic, tqt, mis_disallowed, mean_field;
    int max_total_staples, max_type_staples;
    int imax, dim;
    int type_len[LDO_MAX_TYPES];
    int type_off[LDO_MAX_TYPES];
    int16_t idents[LDO_MAX_IDENTS];
    int n_moves;
    int move_kind[LDO_MAX_MOVES];
    double move_cum[LDO_MAX_MOVES];
    int move_opt[LDO_MAX_MOVES][LDO_N_MOVE_OPTS];   // scaffold regrowth options (LdoMoveOpt)
    int has_ct;                       // some movetype regrows the scaffold
    int adaptive_exchange, allow_nonsensical;
    double exchange_mults[LDO_MAX_TYPES];
    int n_ops;
    int op_kind[LDO_MAX_OPS];
    int op_arg[LDO_MAX_OPS];
    int op_nparts[LDO_MAX_OPS];
    int op_parts[LDO_MAX_OPS][LDO_MAX_PARTS];
    int n_biases;
    int bias_kind[LDO_MAX_BIASES];
    int bias_nops[LDO_MAX_BIASES];
    int bias_op[LDO_MAX_BIASES];
    int bias_min[LDO_MAX_BIASES], bias_max[LDO_MAX_BIASES];
    double bias_well[LDO_MAX_BIASES], bias_minb[LDO_MAX_BIASES], bias_slope[LDO_MAX_BIASES];
    double bias_outside[LDO_MAX_BIASES], bias_k[LDO_MAX_BIASES], bias_centre[LDO_MAX_BIASES];
    int bias_grid_len[LDO_MAX_BIASES];
    double bias_mult;
    int centering_freq, centering_domain, constraint_check_freq;
    int fully_op;         // index of a NumBoundDomainPairs op, or -1 (sampling)
    // Learned insertion proposal: for each scaffold domain the staple type
    // (0: none) and domain index complementary to it, and the network's type
    // slot for that type.
    uint8_t comp_type[LDO_MAX_SCAF];
    uint8_t comp_dom[LDO_MAX_SCAF];
    uint8_t learn_tslot[LDO_MAX_SCAF];
};

struct LdoTab {
    int dense;            // 1: (2imax+1)^2 tables; 0: compact by |identity|
    int stack_dense;      // 1: sequence-specific stacking table at off_stack
    long long off_e, off_h, off_s, off_stack;
    double stack_const;
    double init_e, init_h, init_s;
    double temp;
};

struct LdoRepCtl {
    int sys;
    int tab;
    double staple_M;      // reduced fugacity (OrigamiSystem::m_reduced_fugacity)
    double staple_u_mult;
    double bias_mult;
    int win_min[LDO_MAX_BIASES];
    int win_max[LDO_MAX_BIASES];
    double centre[LDO_MAX_BIASES];
    int grid_off[LDO_MAX_BIASES];   // offset of this replica's grid values, -1 if none
    uint32_t seed;
    uint32_t rep;
};

struct LdoHdr {
    double energy;
    double move_bias;
    double H, S, stacking;
    double z_cache;       // learned insertion: Z of the scaffold states it was computed for
    unsigned long long draws;
    long long steps_done;
    int num_domains, num_staples, num_bound, num_fully, num_self, num_unassigned, num_stacked;
    int current_c_i;
    int n_chains;
    int status;
    int violated;
    int tab;              // table set the energy was last computed with
    int sample_count;
    int z_valid;          // z_cache holds for the current scaffold states and table
    int pad[2];
};

struct LdoLayout {
    int bytes;
    int o_hdr;
    int o_pp;                                  // int64[dcap] packed positions
    int o_bound, o_dident, o_nxt, o_prv;       // int16[dcap]
    int o_ore, o_state, o_slot_cs, o_slot_d;   // uint8[dcap]
    int o_chain_c;                             // int32[kmax+1]
    int o_chain_type, o_chain_order, o_clen;   // uint8[kmax+1]
    int o_type_count;                          // int16[ntypes]
    int o_hash;                                // uint64[hcap]
    int o_bias;                                // double[nb]
    int o_op;                                  // int32[2*nop]: value, defined
    int o_mstat;                               // int64[2*nmv]
    int dcap, kmax, hcap, ntypes, nb, nop, nmv;
    int cls;                                   // LDO_CLASS_*
};

// Capacity classes.  The replica state is a struct whose array sizes are
// compile-time constants, so that every field is one load at a constant
// offset (the kernel is instruction-fetch bound; address arithmetic through
// runtime offsets and pointers tripled its code size).
template <int DCAP_, int KMAX_, int HCAP_>
struct LdoCap {
    static constexpr int DCAP = DCAP_;    // domain slots
    static constexpr int KMAX = KMAX_;    // staple chain slots
    static constexpr int HCAP = HCAP_;    // occupancy hash entries (power of two)
    static constexpr int NT = LDO_MAX_TYPES;
    static constexpr int NB = LDO_MAX_BIASES;
    static constexpr int NOP = LDO_MAX_OPS;
    static constexpr int NMV = LDO_MAX_MOVES;
};
using LdoCapS = LdoCap<80, 32, 256>;
using LdoCapM = LdoCap<160, 56, 512>;
using LdoCapL = LdoCap<320, 63, 1024>;
enum { LDO_CLASS_S = 0, LDO_CLASS_M = 1, LDO_CLASS_L = 2 };

// Persistent state of one replica: the same bytes in the global arena between
// launches and in shared memory during a launch.  Everything before `mstat`
// is the configuration that move snapshots save and restore; the move
// statistics come last so that a restore leaves them alone.
template <class C>
struct __attribute__((aligned(16))) LdoState {
    LdoHdr hdr;
    unsigned long long hash[C::HCAP];
    double bias[C::NB];
    int32_t chain_c[C::KMAX + 1];
    int32_t op[2 * C::NOP];
    long long pp[C::DCAP];    // packed position x + y*2^16 + z*2^32
    int16_t bnd[C::DCAP], did[C::DCAP], nxt[C::DCAP], prv[C::DCAP];
    int16_t type_count[C::NT];
    uint8_t ore[C::DCAP], st[C::DCAP], scs[C::DCAP], sd[C::DCAP];
    uint8_t chain_type[C::KMAX + 1], chain_order[C::KMAX + 1], clen[C::KMAX + 1];
    alignas(16) long long mstat[2 * C::NMV];
};
