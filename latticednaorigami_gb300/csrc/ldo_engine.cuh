// Device-side Monte Carlo engine: one replica's lattice state lives in shared
// memory for the whole launch and one thread of the replica's warp applies
// moves to it.  The member functions restate, in this layout, the reference's
//   OrigamiSystem state transitions    (src/origami_system.cpp:343-871)
//   JunctionBindingPotential (FourBody) (src/origami_potential.cpp:51-934)
//   staple movetypes                   (src/movetypes.cpp, src/met_movetypes.cpp,
//                                       src/cb_movetypes.cpp, src/orientation_movetype.cpp)
//   the step body of GCMCSimulation::simulate (src/simulation.cpp:575-619).
// Terms are visited and summed in the reference's order so that energies and
// every random draw agree with it exactly.
//
// Layout in shared memory (one region per replica, see LdoLayout):
//   per domain slot   pos x/y/z (int16), orientation index (uint8, unit vector
//                     k of {+x,-x,+y,-y,+z,-z}), occupancy state, bound partner
//                     slot, identity, owning chain slot, index in chain
//   per chain slot    unique chain index, chain type; chain order list
//   occupancy hash    open addressing, linear probing, backward-shift delete;
//                     entry = packed position | site state | unbound slot
// Slot s < ns is scaffold domain s; staple chain slot k >= 1 owns slots
// ns + (k-1)*lmax + d.
#pragma once
#include <stdint.h>
#include "ldo_ct.h"
#include "ldo_learn.h"
#include "ldo_math.h"
#include "ldo_types.h"

#ifndef LDO_DEV
#define LDO_DEV __device__ __forceinline__
#endif

namespace ldo {

enum { UNASSIGNED = 0, UNBOUND = 1, BOUND = 2, MISBOUND = 3 };

// A lattice vector packed into one 64-bit integer: x + y*2^16 + z*2^32 with
// |x|, |y|, |z| < 2^15.  Sums, differences, negation and equality of packed
// values are those of the vectors, so every vector test of the reference is
// one integer operation here; the occupancy hash key is the packed value too.
typedef long long V3;
#define LDO_HD __host__ __device__ __forceinline__
LDO_HD constexpr V3 mk(int x, int y, int z) { return (long long)x + (long long)y * 65536ll + (long long)z * 4294967296ll; }
LDO_HD constexpr V3 add(V3 a, V3 b) { return a + b; }
LDO_HD constexpr V3 sub(V3 a, V3 b) { return a - b; }
LDO_HD constexpr V3 neg(V3 a) { return -a; }
LDO_HD constexpr bool eq(V3 a, V3 b) { return a == b; }
LDO_HD constexpr int vx(V3 p) { return (int)(short)(unsigned short)(p & 0xffff); }
LDO_HD constexpr int vy(V3 p) { return (int)(short)(unsigned short)(((p - vx(p)) >> 16) & 0xffff); }
LDO_HD constexpr int vz(V3 p) { return (int)((((p - vx(p)) >> 16) - vy(p)) >> 16); }

// Unit vector k in the order of include/.../utility.hpp:156-162.
LDO_HD constexpr V3 unit_c(int k) {
    return k == 0 ? mk(1, 0, 0) : k == 1 ? mk(-1, 0, 0) : k == 2 ? mk(0, 1, 0) : k == 3 ? mk(0, -1, 0)
                                                          : k == 4 ? mk(0, 0, 1) : mk(0, 0, -1);
}
// Index of a unit vector, -1 for any other vector.
LDO_HD constexpr int unit_index(V3 v) {
    return v == 1 ? 0 : v == -1 ? 1 : v == 65536ll ? 2 : v == -65536ll ? 3 : v == 4294967296ll ? 4
         : v == -4294967296ll ? 5 : -1;
}

// Rotations used by the twist constraints, tabulated over unit vectors:
//   half[o][axis]      VectorThree::rotate_half(axis)   (src/utility.cpp:68)
//   quarter[o][k]      VectorThree::rotate(unit k, -1)  (src/utility.cpp:102)
// For any vector that is not a unit vector both rotations leave the
// orientation unchanged (none of the reference's axis tests matches).
struct RotTab {
    unsigned char half[6][3];
    unsigned char quarter[6][6];
};
constexpr int rot_comp(int o, int c) { return c == 0 ? vx(unit_c(o)) : c == 1 ? vy(unit_c(o)) : vz(unit_c(o)); }
constexpr RotTab make_rot() {
    RotTab t {};
    for (int o = 0; o < 6; ++o) {
        for (int a = 0; a < 3; ++a) {
            int x = rot_comp(o, 0), y = rot_comp(o, 1), z = rot_comp(o, 2);
            if (a == 0) { y = -y; z = -z; }
            else if (a == 1) { x = -x; z = -z; }
            else { x = -x; y = -y; }
            t.half[o][a] = (unsigned char)unit_index(mk(x, y, z));
        }
        for (int k = 0; k < 6; ++k) {
            int x = rot_comp(o, 0), y = rot_comp(o, 1), z = rot_comp(o, 2);
            int dir = (k & 1) ? 1 : -1;   // turns = -1: dir -1, flipped for a negative axis
            int s = 0;
            if ((k >> 1) == 0) { s = y; y = z; z = s; y *= -dir; z *= dir; }
            else if ((k >> 1) == 1) { s = x; x = z; z = s; x *= -dir; z *= dir; }
            else { s = x; x = y; y = s; x *= -dir; y *= dir; }
            t.quarter[o][k] = (unsigned char)unit_index(mk(x, y, z));
        }
    }
    return t;
}
__constant__ const RotTab kRot = make_rot();
__constant__ const long long kUnitP[6] = {unit_c(0), unit_c(1), unit_c(2), unit_c(3), unit_c(4), unit_c(5)};
__device__ __forceinline__ V3 unit(int k) { return kUnitP[k]; }

// ------------------------------------------------------------- Philox ---
// Philox4x32-10 (Salmon et al., SC'11).  Stream contract: key (seed, replica),
// counter (draw >> 1, 0, stream, 0); draw n is the 64-bit word pair
// (2*(n&1), 2*(n&1)+1) of its block.
LDO_DEV void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                      uint32_t* out) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        unsigned long long p0 = (unsigned long long)0xD2511F53u * c0;
        unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Rng {
    uint32_t k0, k1, stream;
    unsigned long long draws;
    unsigned long long cblock;
    uint32_t w[4];

    __device__ void init(uint32_t seed, uint32_t rep, uint32_t s, unsigned long long d) {
        k0 = seed;
        k1 = rep;
        stream = s;
        draws = d;
        cblock = ~0ull;
    }
    __device__ __noinline__ unsigned long long next64() {
        unsigned long long b = draws >> 1;
        if (b != cblock) {
            philox10((uint32_t)b, (uint32_t)(b >> 32), stream, 0u, k0, k1, w);
            cblock = b;
        }
        int j = (int)(draws & 1ull) * 2;
        ++draws;
        return ((unsigned long long)w[j] << 32) | w[j + 1];
    }
    __device__ __noinline__ double uniform_real() { return (double)(next64() >> 11) * 0x1.0p-53; }
    __device__ __noinline__ int uniform_int(int lo, int hi) {
        unsigned long long range = (unsigned long long)((long long)hi - (long long)lo) + 1ull;
        return lo + (int)__umul64hi(next64(), range);
    }
};

// ------------------------------------------------------------ hashing ---
#define LDO_KEYMASK ((1ull << 48) - 1ull)
#define LDO_VALID (1ull << 63)

LDO_DEV unsigned long long pkey(V3 p) { return (unsigned long long)(p + mk(32768, 32768, 32768)); }
LDO_DEV int ent_occ(unsigned long long e) { return (int)((e >> 48) & 3ull); }
LDO_DEV int ent_slot(unsigned long long e) { return (int)((e >> 50) & 0xfffull); }
LDO_DEV unsigned long long mkent(unsigned long long key, int occ, int slot) {
    return key | ((unsigned long long)occ << 48) | ((unsigned long long)slot << 50) | LDO_VALID;
}

// Caps for the reference's data-dependent loops (rejection sampling of a
// growth point, src/movetypes.cpp:378-380).
#define LDO_GROWTHPOINT_CAP 1000000

struct Delta {
    double e;
    int stacked;
};

// The engine's own exponential (ldo_math.h: the same bits as host code
// computing it), one out-of-line copy to keep the hot code small (instruction
// fetch, not arithmetic, limits this kernel).
static __device__ __noinline__ double dexp(double x) { return ldo_math::exp(x); }

struct Scratch {
    // MCMovetype reversal lists (include/.../movetypes.hpp:156-163)
    int n_mod, n_asg, added_cs;
    int mod[LDO_MAX_LEN];
    V3 mod_pos[LDO_MAX_LEN];
    int mod_ore[LDO_MAX_LEN];
    int asg[LDO_MAX_LEN];
    // CB old configuration (include/.../movetypes.hpp:241-242)
    int n_old;
    int old_slot[LDO_MAX_LEN];
    V3 old_pos[LDO_MAX_LEN];
    int old_ore[LDO_MAX_LEN];
    // bound domains of the selected staple (new, old)
    int n_bd;
    int bd_new[LDO_MAX_LEN], bd_old[LDO_MAX_LEN];
    int cb_g;               // growth point index of the CB move's new configuration
};

// Commands from a replica's move phases to its warp, which copies the state
// to / from snapshots in global memory between phases (CMD_SNAP(k): state ->
// snapshot k; CMD_REST(k): snapshot k -> state; the snapshot is taken first
// unless CMD_REST_FIRST; CMD_MORE: call step_resume afterwards).
#define CMD_SNAP(k) ((k) + 1)
#define CMD_REST(k) (((k) + 1) << 4)
enum : int { CMD_MORE = 1 << 8, CMD_REST_FIRST = 1 << 9, CMD_STOP = 1 << 10 };
enum : int { PH_POST = 1, PH_CB2 = 2, PH_CB3 = 3, PH_RG2 = 4, PH_RG3 = 5, PH_RG4 = 6, PH_RG5 = 7, PH_CT2 = 8,
             PH_CT3 = 9, PH_LK2 = 10, PH_LK3 = 11, PH_LKR2 = 12 };
constexpr int N_SNAPSHOTS = 3;

// Scratch of the FourBody evaluation.
struct FBState {
    Delta pd;               // BindingPotential::m_delta_config
    int viol;               // BindingPotential::m_constraints_violated
    int fa[3], fb[3], sa[3], sb[3];   // single-junction candidate pairs
};

// One Rep per warp lives in shared memory next to the replica's state; its
// member data must never sit in a thread's local memory, where a single
// active lane would touch one 128-byte line per 4-byte access.
template <class C>
struct Rep : public LdoState<C> {
    using S_ = LdoState<C>;
    using S_::hdr;
    using S_::hash;
    using S_::bias;
    using S_::mstat;
    using S_::chain_c;
    using S_::op;
    using S_::pp;
    using S_::nxt;
    using S_::prv;
    using S_::bnd;
    using S_::did;
    using S_::type_count;
    using S_::ore;
    using S_::st;
    using S_::scs;
    using S_::sd;
    using S_::chain_type;
    using S_::chain_order;
    using S_::clen;
    static constexpr int hmask = C::HCAP - 1;
    static constexpr int hshift = 64 - (C::HCAP == 256 ? 8 : C::HCAP == 512 ? 9 : C::HCAP == 1024 ? 10 : C::HCAP == 2048 ? 11 : 12);

    const LdoSys* sys;
    const LdoTab* tab;
    const double* bank;
    const LdoRepCtl* ctl;
    const double* grid;
    const double* learn_w;   // learned insertion proposal weights (LDO_LEARN_TABLE)
    int learn_tb;            // temperature bin of the current tables
    // scalars of the current table set and controls, cached in the object
    int t_dense, t_stack_dense, imax, dim;
    long long t_off_e, t_off_h, t_off_s, t_off_stack;
    double t_stack_const, t_init_e, t_init_h, t_init_s;
    double c_staple_M, c_bias_mult;
    int ns, lmax, nmv;
    int cyclic, tqt, mean_field;
    Rng rng;
    FBState fb_;
    __device__ __forceinline__ FBState& fbst() { return fb_; }
    __device__ __forceinline__ const FBState& fbst() const { return fb_; }
    // CB trial-position arrays and the connector search stack (lane 0 only)
    V3 cb_pos[6];
    int cb_ore[6];
    double cb_bf[6];
    double cb_de[6];        // probed candidates: energy change and stacked-pair change
    int cb_stk[6];
    uint8_t dfs_stack[LDO_MAX_KMAX + 1];
    Scratch m;
    bool rejected;
    double modifier, delta_e;
    double w_bias, w_new_bias, new_modifier;
    bool regrow_old;
    int insertion_sites;
    bool staple_bound;
    double log6, log3;
    // step state machine (step_begin / step_resume)
    bool dirty;             // the move may have changed the state
    bool recalc;            // update_move_params + calc_move after the restore
    int phase;              // PH_* of the interrupted move
    int cur_mv;
    long long cur_s;
    int cb_cs;
    LdoCtWork<C>* ct;        // scaffold regrowth working memory (global), or null

    // Accessors used by the FourBody traversal.
    __device__ __forceinline__ int gst(int i) const { return st[i]; }
    __device__ __forceinline__ int gbnd(int i) const { return bnd[i]; }
    __device__ __forceinline__ int gore(int i) const { return ore[i]; }
    __device__ __forceinline__ V3 gorev(int i) const { return unit(gore(i)); }
    __device__ __forceinline__ V3 gpos(int i) const { return pos(i); }

    // ---------------------------------------------------------- errors ---
    __device__ void fail(int code) {
        if (hdr.status == 0) hdr.status = code;
    }
    __device__ bool bad() const { return hdr.status != 0; }

    // -------------------------------------------------------- accessors ---
    __device__ V3 pos(int i) const { return pp[i]; }
    __device__ void set_pos(int i, V3 p) {
        int x = vx(p), y = vy(p), z = vz(p);
        if (x < -32000 || x > 32000 || y < -32000 || y > 32000 || z < -32000 || z > 32000) {
            fail(LDO_RS_CAPACITY);
            return;
        }
        pp[i] = p;
    }
    __device__ V3 orev(int i) const { return unit(ore[i]); }
    __device__ int chain_len(int cs) const { return clen[cs]; }
    __device__ int slot_of(int cs, int d) const { return cs == 0 ? d : ns + (cs - 1) * lmax + d; }
    __device__ int cidx(int i) const { return chain_c[scs[i]]; }
    // Chain neighbours (stored links; the scaffold's wrap when it is cyclic).
    __device__ int fwd(int i) const { return nxt[i]; }
    __device__ int bwd(int i) const { return prv[i]; }
    __device__ int next(int i, int incr) const {   // Domain::operator+ (src/domain.cpp:9)
        #pragma unroll 1
        while (i >= 0 && incr > 0) { i = fwd(i); --incr; }
        #pragma unroll 1
        while (i >= 0 && incr < 0) { i = bwd(i); ++incr; }
        return i;
    }
    // A scaffold domain's state changed: the cached Z of the learned
    // insertion no longer holds (snapshot restores bring back both).
    __device__ __forceinline__ void z_touch(int i) {
        if (i < ns) hdr.z_valid = 0;
    }
    __device__ void bind_tables(const LdoTab* t) {
        tab = t;
        learn_tb = ldo_learn_tbin(t->temp);
        hdr.z_valid = 0;
        t_dense = t->dense;
        t_stack_dense = t->stack_dense;
        t_off_e = t->off_e;
        t_off_h = t->off_h;
        t_off_s = t->off_s;
        t_off_stack = t->off_stack;
        t_stack_const = t->stack_const;
        t_init_e = t->init_e;
        t_init_h = t->init_h;
        t_init_s = t->init_s;
    }
    __device__ double tval(long long off, int a, int b) const {
        if (t_dense) return __ldg(bank + off + (long long)(a + imax) * dim + (b + imax));
        return (a == -b) ? __ldg(bank + off + (a < 0 ? -a : a)) : __ldg(bank + off + imax + 1);
    }
    __device__ double hyb(int i, int j) const { return tval(t_off_e, did[i], did[j]); }
    __device__ double hyb_h(int i, int j) const { return tval(t_off_h, did[i], did[j]); }
    __device__ double hyb_s(int i, int j) const { return tval(t_off_s, did[i], did[j]); }
    __device__ double stack(int i, int j) const {
        if (t_stack_dense) return __ldg(bank + t_off_stack + (long long)(did[i] + imax) * dim + (did[j] + imax));
        return t_stack_const;
    }

    // ------------------------------------------------------------ hash ---
    __device__ int home(unsigned long long key) const {
        return (int)((key * 0x9E3779B97F4A7C15ull) >> hshift) & hmask;
    }
    // Index of the entry for key, or -1 (then *empty_at is the first free slot).
    __device__ __noinline__ int hfind(unsigned long long key, int* empty_at) const {
        int k = home(key);
        #pragma unroll 1
        for (int n = 0; n <= hmask; ++n) {
            unsigned long long e = hash[k];
            if (!(e & LDO_VALID)) {
                if (empty_at) *empty_at = k;
                return -1;
            }
            if ((e & LDO_KEYMASK) == key) return k;
            k = (k + 1) & hmask;
        }
        if (empty_at) *empty_at = -1;
        return -1;
    }
    __device__ __noinline__ void herase(int i) {
        int j = i;
        #pragma unroll 1
        for (int n = 0; n <= hmask; ++n) {
            j = (j + 1) & hmask;
            unsigned long long e = hash[j];
            if (!(e & LDO_VALID)) break;
            int k = home(e & LDO_KEYMASK);
            bool move = (i <= j) ? (k <= i || k > j) : (k <= i && k > j);
            if (move) {
                hash[i] = e;
                i = j;
            }
        }
        hash[i] = 0ull;
    }
    __device__ __noinline__ void hset(V3 p, int occ, int slot) {
        unsigned long long key = pkey(p);
        int emp;
        int k = hfind(key, &emp);
        if (k < 0) k = emp;
        if (k < 0) {
            fail(LDO_RS_CAPACITY);
            return;
        }
        hash[k] = mkent(key, occ, slot);
    }
    __device__ int occupancy(V3 p) const {
        int k = hfind(pkey(p), nullptr);
        return k < 0 ? UNASSIGNED : ent_occ(hash[k]);
    }
    __device__ int unbound_at(V3 p) const {
        int k = hfind(pkey(p), nullptr);
        return k < 0 ? -1 : ent_slot(hash[k]);
    }

    // ----------------------------------------------------- chain add/del ---
    // OrigamiSystem::add_chain(c_i_ident, c_i) (src/origami_system.cpp:402)
    __device__ __noinline__ int add_chain_with_index(int type, int c_i) {
        int cs = -1;
        int kmax = sys->kmax;
        #pragma unroll 1
        for (int k = 1; k <= kmax && k <= C::KMAX; ++k)
            if (chain_type[k] == 0xff) { cs = k; break; }
        if (cs < 0) {
            fail(LDO_RS_CAPACITY);
            return -1;
        }
        chain_c[cs] = c_i;
        chain_type[cs] = (uint8_t)type;
        clen[cs] = (uint8_t)sys->type_len[type];
        chain_order[hdr.n_chains++] = (uint8_t)cs;
        type_count[type]++;
        int len = sys->type_len[type];
        int off = sys->type_off[type];
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int s = slot_of(cs, d);
            st[s] = UNASSIGNED;
            bnd[s] = -1;
            did[s] = sys->idents[off + d];
            nxt[s] = (int16_t)(d + 1 < len ? s + 1 : -1);
            prv[s] = (int16_t)(d > 0 ? s - 1 : -1);
        }
        hdr.num_domains += len;
        hdr.num_unassigned += len;
        hdr.num_staples++;
        return cs;
    }
    // OrigamiSystem::add_chain(c_i_ident) (src/origami_system.cpp:387)
    __device__ __noinline__ int add_chain(int type) {
        hdr.current_c_i += 1;
        if (mean_field) hdr.energy += log6;
        hdr.energy += t_init_e;
        return add_chain_with_index(type, hdr.current_c_i);
    }
    // OrigamiSystem::delete_chain (src/origami_system.cpp:445)
    __device__ __noinline__ void delete_chain(int cs) {
        int n = hdr.n_chains;
        int k = 0;
        #pragma unroll 1
        while (k < n && chain_order[k] != cs) ++k;
        #pragma unroll 1
        for (int q = k; q + 1 < n; ++q) chain_order[q] = chain_order[q + 1];
        hdr.n_chains = n - 1;
        int type = chain_type[cs];
        type_count[type]--;
        int len = sys->type_len[type];
        hdr.num_domains -= len;
        hdr.num_staples--;
        hdr.num_unassigned -= len;
        chain_type[cs] = 0xff;
        if (mean_field) hdr.energy -= log6;
        hdr.energy -= t_init_e;
    }

    // ------------------------------------------------- state transitions ---
    // OrigamiSystem::update_occupancies (src/origami_system.cpp:770)
    __device__ __noinline__ void update_occupancies(int i, V3 p) {
        unsigned long long key = pkey(p);
        int emp;
        int k = hfind(key, &emp);
        int occ = k < 0 ? UNASSIGNED : ent_occ(hash[k]);
        if (occ == UNBOUND) {
            int j = ent_slot(hash[k]);
            hdr.num_bound += 1;
            int ns_;
            if (did[i] == -did[j]) {
                ns_ = BOUND;
                hdr.num_fully += 1;
            }
            else {
                if (cidx(i) == cidx(j)) hdr.num_self += 1;
                ns_ = MISBOUND;
            }
            st[i] = (uint8_t)ns_;
            st[j] = (uint8_t)ns_;
            z_touch(i);
            z_touch(j);
            hash[k] = mkent(key, ns_, 0);
            bnd[j] = (int16_t)i;
            bnd[i] = (int16_t)j;
        }
        else if (occ == UNASSIGNED) {
            st[i] = UNBOUND;
            z_touch(i);
            if (emp < 0) {
                fail(LDO_RS_CAPACITY);
                return;
            }
            hash[emp] = mkent(key, UNBOUND, i);
        }
        else {
            fail(LDO_RS_INVARIANT);   // "Trying to bind to an already bound domain"
        }
    }

    // unassign_bound_domain (src/origami_system.cpp:741)
    __device__ __noinline__ double unassign_bound(int i) {
        int j = bnd[i];
        double de = -hyb(i, j);
        bnd[i] = -1;
        bnd[j] = -1;
        st[i] = UNASSIGNED;
        hset(pos(i), UNBOUND, j);
        st[j] = UNBOUND;
        z_touch(i);
        z_touch(j);
        return de;
    }

    // internal_unassign_domain (src/origami_system.cpp:695)
    __device__ __noinline__ Delta internal_unassign(int i) {
        int occ = st[i];
        int j = bnd[i];
        Delta dc;
        dc.e = 0;
        dc.stacked = 0;
        if ((occ == BOUND || occ == MISBOUND) && j < 0) {
            fail(LDO_RS_INVARIANT);
            return dc;
        }
        switch (occ) {
        case BOUND:
            hdr.num_fully -= 1;
            hdr.num_bound -= 1;
            dc = check_stacking(i, j);
            dc.e *= -1;
            dc.stacked *= -1;
            dc.e += unassign_bound(i);
            break;
        case MISBOUND:
            hdr.num_bound -= 1;
            if (cidx(j) == cidx(i)) hdr.num_self -= 1;
            dc.e += unassign_bound(i);
            break;
        case UNBOUND: {
            int k = hfind(pkey(pos(i)), nullptr);
            if (k >= 0) herase(k);
            st[i] = UNASSIGNED;
            z_touch(i);
            break;
        }
        default:
            hdr.num_unassigned--;
            break;
        }
        if (mean_field && occ == BOUND) {
            if (hdr.num_fully == 0) dc.e -= 2 * log6;
            else if (hdr.num_fully == 1) dc.e -= log3;
        }
        return dc;
    }

    // internal_check_domain_constraints (src/origami_system.cpp:828)
    __device__ __noinline__ Delta internal_check(int i, V3 p, int o) {
        int occ = occupancy(p);
        Delta dc;
        dc.e = 0;
        dc.stacked = 0;
        switch (occ) {
        case BOUND:
        case MISBOUND:
            hdr.violated = 1;
            hdr.num_unassigned++;
            break;
        case UNBOUND:
            set_pos(i, p);
            ore[i] = (uint8_t)o;
            update_occupancies(i, p);
            if (bad()) return dc;
            dc = bind_domain(i);
            hdr.violated = fbst().viol ? 1 : 0;
            break;
        default:
            set_pos(i, p);
            ore[i] = (uint8_t)o;
            update_occupancies(i, p);
            break;
        }
        if (mean_field && !hdr.violated && st[i] == BOUND) {
            if (hdr.num_fully == 1) dc.e += 2 * log6;
            else if (hdr.num_fully == 2) dc.e += log3;
        }
        return dc;
    }

    // set_domain_config (src/origami_system.cpp:517)
    __device__ __noinline__ double set_domain_config(int i, V3 p, int o) {
        if (st[i] != UNASSIGNED) {
            fail(LDO_RS_INVARIANT);   // "Trying to set an already assigned domain"
            return 0;
        }
        Delta dc = internal_check(i, p, o);
        if (hdr.violated) {
            internal_unassign(i);
        }
        else {
            hdr.energy += dc.e;
            hdr.num_stacked += dc.stacked;
            hdr.num_unassigned--;
        }
        return dc.e;
    }

    // set_checked_domain_config (src/origami_system.cpp:478)
    __device__ __noinline__ double set_checked(int i, V3 p, int o) {
        set_pos(i, p);
        ore[i] = (uint8_t)o;
        update_occupancies(i, p);
        double de = 0;
        if (bad()) return 0;
        if (st[i] == MISBOUND) {
            de += hyb(i, bnd[i]);
        }
        else if (st[i] == BOUND) {
            de += hyb(i, bnd[i]);
            Delta dc = check_stacking(i, bnd[i]);
            de += dc.e;
            hdr.num_stacked += dc.stacked;
        }
        if (mean_field && st[i] == BOUND) {
            if (hdr.num_fully == 1) de += 2 * log6;
            else if (hdr.num_fully == 2) de += log3;
        }
        hdr.energy += de;
        hdr.num_unassigned--;
        return de;
    }

    // unassign_domain (src/origami_system.cpp:375)
    __device__ __noinline__ double unassign_domain(int i) {
        Delta dc = internal_unassign(i);
        hdr.energy += dc.e;
        hdr.num_stacked += dc.stacked;
        hdr.num_unassigned++;
        return dc.e;
    }

    // check_domain_constraints (src/origami_system.cpp:343)
    __device__ __noinline__ double check_domain_constraints(int i, V3 p, int o) {
        Delta dc = internal_check(i, p, o);
        internal_unassign(i);
        return dc.e;
    }

    // check_domain_constraints for a CB trial position (src/origami_system.cpp:343):
    // the same state change and energy; the undo skips the stacking traversal
    // whose result the reference discards (internal_unassign_domain :704).
    __device__ __noinline__ Delta probe_domain(int i, V3 p, int o) {
        Delta dc = internal_check(i, p, o);
        int occ = st[i];
        int j = bnd[i];
        if (occ == BOUND || occ == MISBOUND) {
            if (j < 0) {
                fail(LDO_RS_INVARIANT);
                return dc;
            }
            hdr.num_bound -= 1;
            if (occ == BOUND) hdr.num_fully -= 1;
            else if (cidx(j) == cidx(i)) hdr.num_self -= 1;
            bnd[i] = -1;
            bnd[j] = -1;
            st[i] = UNASSIGNED;
            hset(pos(i), UNBOUND, j);
            st[j] = UNBOUND;
            z_touch(i);
            z_touch(j);
        }
        else if (occ == UNBOUND) {
            int k = hfind(pkey(pos(i)), nullptr);
            if (k >= 0) herase(k);
            st[i] = UNASSIGNED;
            z_touch(i);
        }
        else {
            hdr.num_unassigned--;
        }
        return dc;
    }

    // set_checked_domain_config for a CB trial position that probe_domain has
    // evaluated in the same state: the energy change and stacked-pair change
    // are the probe's (hybridisation + stacking, the same two FP64 operands in
    // either order, plus the same mean-field term), so the stacking traversal
    // is not repeated.
    __device__ __noinline__ double set_checked_probed(int i, V3 p, int o, double de, int stacked) {
        set_pos(i, p);
        ore[i] = (uint8_t)o;
        update_occupancies(i, p);
        if (bad()) return 0;
        if (st[i] == BOUND) hdr.num_stacked += stacked;
        hdr.energy += de;
        hdr.num_unassigned--;
        return de;
    }

    // set_domain_orientation (src/origami_system.cpp:543)
    __device__ void set_domain_orientation(int i, int o) {
        if (st[i] == BOUND) hdr.violated = 1;
        else ore[i] = (uint8_t)o;
    }

    // center (src/origami_system.cpp:553)
    __device__ __noinline__ void center(int cd) {
        V3 ref = pos(cd);
        #pragma unroll 1
        for (int k = 0; k <= hmask; ++k) hash[k] = 0ull;
        #pragma unroll 1
        for (int c = 0; c < hdr.n_chains; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int s = slot_of(cs, d);
                V3 np = sub(pos(s), ref);
                set_pos(s, np);
                int o = st[s];
                if (o == UNBOUND) hset(np, UNBOUND, s);
                else if (o == BOUND || o == MISBOUND) hset(np, o, 0);
            }
        }
    }

    // set_all_domains (src/origami_system.cpp:573)
    __device__ __noinline__ void set_all_current() {
        #pragma unroll 1
        for (int c = 0; c < hdr.n_chains && !bad(); ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int s = slot_of(cs, d);
                set_domain_config(s, pos(s), ore[s]);
                if (hdr.violated) {
                    fail(LDO_RS_INVARIANT);   // "Constaints in violation after move complete"
                    return;
                }
            }
        }
    }

    // check_all_constraints (src/origami_system.cpp:267)
    __device__ __noinline__ void check_all_constraints() {
        if (hdr.num_unassigned != 0) {
            fail(LDO_RS_INVARIANT);
            return;
        }
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int s = slot_of(cs, d);
                if (st[s] == UNASSIGNED) {
                    fail(LDO_RS_INVARIANT);
                    return;
                }
                unassign_domain(s);
            }
        }
        unsigned long long nst = (unsigned long long)(nc - 1);
        if (mean_field) hdr.energy -= nst * log6;
        hdr.energy -= nst * t_init_e;
        if (hdr.num_stacked != 0) {
            set_all_current();
            fail(LDO_RS_INVARIANT);
            return;
        }
        double eps = 0.000001;
        if (hdr.energy < -eps || hdr.energy > eps) {
            set_all_current();
            fail(LDO_RS_INVARIANT);
            return;
        }
        hdr.energy = 0;
        set_all_current();
        if (mean_field) hdr.energy += nst * log6;
        hdr.energy += nst * t_init_e;
    }

    // update_energy (src/origami_system.cpp:808)
    __device__ __noinline__ void recompute_energy() {
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) unassign_domain(slot_of(cs, d));
        }
        hdr.energy = 0;
        unsigned long long nst = (unsigned long long)(nc - 1);
        if (mean_field) hdr.energy += nst * log6;
        hdr.energy += nst * t_init_e;
        set_all_current();
    }

    // update_enthalpy_and_entropy (src/origami_system.cpp:204)
    __device__ __noinline__ void dependent_quantities() {
        double H = 0, S = 0;
        // "accounted" = partner of an earlier domain in chain order; a pair is
        // counted at its first domain.
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int s = slot_of(cs, d);
                int o = st[s];
                if (o == BOUND || o == MISBOUND) {
                    int b = bnd[s];
                    if (!visited_before(s, b, c, d)) {
                        H += hyb_h(s, b);
                        S += hyb_s(s, b);
                    }
                }
            }
        }
        unsigned long long nst = (unsigned long long)(nc - 1);
        if (mean_field) {
            S -= nst * log6;
            if (hdr.num_fully >= 1) S -= 2 * log6;
            if (hdr.num_fully >= 2) S -= log3;
        }
        H += nst * t_init_h;
        S += nst * t_init_s;
        hdr.H = H;
        hdr.S = S;
        hdr.stacking = hdr.energy - (H - S);
    }
    // True if partner b comes before domain s (chain position c, index d) in
    // chain order, i.e. s was inserted into the reference's accounted set.
    __device__ __noinline__ bool visited_before(int s, int b, int c, int d) const {
        int cb = scs[b];
        #pragma unroll 1
        for (int q = 0; q < c; ++q)
            if (chain_order[q] == cb) return true;
        if (cb == chain_order[c]) return sd[b] < d;
        return false;
    }

    // ================================================ FourBody potential ===
    __device__ bool exists_bound(int i) const { return i >= 0 && gst(i) == BOUND; }

    __device__ __forceinline__ bool twist_ok(int i1, V3 ndr, int i2) const {   // src/domain.cpp:33,69
        int a = unit_index(ndr);
        int o1 = gore(i1);
        int r = a < 0 ? o1 : (tqt ? kRot.quarter[o1][a] : kRot.half[o1][a >> 1]);
        return r == gore(i2);
    }
    __device__ __noinline__ bool kink_ok(int i1, V3 ndr, int i2) const {   // src/domain.cpp:42,80
        V3 o1 = gorev(i1), o2 = gorev(i2);
        if (eq(ndr, neg(o1))) return false;
        if (eq(ndr, o1)) {
            if (tqt) return !(eq(o1, o2) || eq(o1, neg(o2)));
            return !eq(o2, neg(o1));
        }
        if (eq(ndr, o2) || eq(ndr, neg(o2))) return false;
        return true;
    }
    __device__ __noinline__ bool junction_ok(int j1, int j2, int k1, int k2) const {   // src/domain.cpp:59,99
        if (!tqt) return true;
        V3 ndr_k = sub(gpos(k2), gpos(k1));
        if (eq(ndr_k, gorev(k1))) {
            V3 ndr1 = sub(gpos(j2), gpos(j1));
            if (sd[j1] > sd[j2]) ndr1 = neg(ndr1);
            if (!twist_ok(k1, ndr1, k2)) return false;
        }
        return true;
    }
    __device__ __noinline__ bool doubly_contig(int a, int b) const {   // src/origami_potential.cpp:51
        if (scs[a] != scs[b] || sd[b] != sd[a] + 1) return false;
        int ba = gbnd(a), bb = gbnd(b);
        if (scs[ba] != scs[bb]) return false;
        int dd = sd[bb] - sd[ba];
        return dd == 1 || dd == -1;
    }
    __device__ __noinline__ bool pair_stacked(int a, int b) const {   // :70
        if (sd[a] > sd[b]) { int t = a; a = b; b = t; }
        V3 ndr = sub(gpos(b), gpos(a));
        V3 oa = gorev(a);
        if (!eq(ndr, oa) && !eq(ndr, neg(oa))) return twist_ok(a, ndr, b);
        return false;
    }
    __device__ __noinline__ int junction_penalty(int j1, int j2, int j3, int j4, int k1, int k2) const {   // :85
        V3 ndr_k = sub(gpos(k2), gpos(k1));
        if (!eq(ndr_k, gorev(k1))) return 0;
        V3 n1 = sub(gpos(j2), gpos(j1));
        if (sd[j1] > sd[j2]) n1 = neg(n1);
        V3 n3 = sub(gpos(j4), gpos(j3));
        if (sd[j3] > sd[j4]) n3 = neg(n3);
        if (eq(n1, n3)) return 2;
        if (eq(n1, neg(n3))) return 0;
        return 1;
    }
    __device__ __noinline__ void triplet_single(int h1, int h2, int h3) {   // :158
        V3 n1 = sub(gpos(h2), gpos(h1));
        if (eq(n1, gorev(h1))) return;
        V3 n2 = sub(gpos(h3), gpos(h2));
        if (!eq(n1, n2)) {
            fbst().pd.e -= stack(h2, h3);
            fbst().pd.stacked -= 1;
        }
    }
    __device__ __noinline__ void triplet_double(int h1, int h2, int h3) {   // :181
        V3 n1 = sub(gpos(h2), gpos(h1));
        V3 n2 = sub(gpos(h3), gpos(h2));
        if (!eq(n1, n2)) {
            fbst().pd.e -= stack(h1, h2) / 2;
            fbst().pd.e -= stack(h2, h3) / 2;
            fbst().pd.stacked -= 1;
        }
    }
    __device__ __noinline__ void triply_contig_helix(int h1, int h2, int h3) {   // :200
        V3 n1 = sub(gpos(h2), gpos(h1));
        V3 n2 = sub(gpos(h3), gpos(h2));
        if (!eq(n1, n2)) fbst().viol = true;
    }

    __device__ __noinline__ void stacking_and_steric(int i, int j) {   // :212
        constraints_around(i, 0);
        if (fbst().viol) return;
        constraints_around(j, 1);
        if (fbst().viol) return;
        central_triplets(i, j);
    }

    __device__ __noinline__ void constraints_around(int cd, int jj) {   // :231
        #pragma unroll 1
        for (int k = -1; k <= 0; ++k) {
            int c1 = next(cd, k);
            int c2 = next(cd, k + 1);
            if (!(exists_bound(c1) && exists_bound(c2))) continue;
            int b1 = gbnd(c1), b2 = gbnd(c2);
            if (scs[b1] == scs[b2]) {
                if (sd[b1] == sd[b2] - 1) doubly_contig_helix_pair(c1, c2, k, jj);
                else if (sd[b1] == sd[b2] + 1) doubly_contig_junction_pair(c1, c2, jj);
                else regular_pair(c1, c2, k);
            }
            else {
                regular_pair(c1, c2, k);
            }
            if (fbst().viol) return;
        }
        int prev = next(cd, -1);
        int forw = next(cd, 1);
        if (exists_bound(prev) && exists_bound(forw)) {
            if (pair_stacked(cd, forw)) {
                if (pair_stacked(prev, cd)) {
                    if (doubly_contig(prev, cd) && doubly_contig(cd, forw)) {
                        triply_contig_helix(prev, cd, forw);
                        if (fbst().viol) return;
                    }
                    triplet_double(prev, cd, forw);
                }
                else {
                    triplet_single(prev, cd, forw);
                }
            }
        }
    }

    __device__ __noinline__ void regular_pair(int c1, int c2, int k) {   // :288
        V3 ndr = sub(gpos(c2), gpos(c1));
        if (!kink_ok(c1, ndr, c2)) {
            fbst().viol = true;
            return;
        }
        if (pair_stacked(c1, c2)) {
            fbst().pd.e += stack(c1, c2);
            fbst().pd.stacked += 1;
            if (k == -1) backward_single_junction(c1, c2);
            else forward_single_junction(c1, c2);
        }
        else {
            central_single_junction(c1, c2);
        }
        if (k == -1) backward_triplets(c1, c2);
        else forward_triplets(c1, c2);
    }

    __device__ __noinline__ void doubly_contig_helix_pair(int c1, int c2, int k, int jj) {   // :322
        if (jj == 1) return;
        V3 ndr = sub(gpos(c2), gpos(c1));
        V3 o1 = gorev(c1);
        if (eq(ndr, o1) || eq(ndr, neg(o1))) {
            fbst().viol = true;
            return;
        }
        if (twist_ok(c1, ndr, c2)) {
            fbst().pd.e += stack(c1, c2);
            fbst().pd.stacked += 1;
        }
        else {
            fbst().viol = true;
            return;
        }
        if (k == -1) {
            backward_triplets(c1, c2);
            backward_single_junction(c1, c2);
        }
        else {
            forward_triplets(c1, c2);
            forward_single_junction(c1, c2);
        }
    }

    __device__ __noinline__ void doubly_contig_junction_pair(int c1, int c2, int jj) {   // :359
        int k1 = c1, k2 = c2;
        V3 ndr = sub(gpos(k2), gpos(k1));
        if (!eq(gorev(k1), ndr)) {
            fbst().viol = true;
            return;
        }
        if (jj == 1) return;
        #pragma unroll 1
        for (int a = 0; a < 2; ++a) {
            int j1 = a == 0 ? next(c1, -1) : next(gbnd(c1), 1);
            int j2 = a == 0 ? c1 : gbnd(c1);
            int j3 = k2, j4 = next(k2, 1);
            if (exists_bound(j4) && exists_bound(j1)) junction(j1, j2, j3, j4, k1, k2);
            j3 = gbnd(k2);
            j4 = next(j3, -1);
            if (exists_bound(j4) && exists_bound(j1)) junction(j1, j2, j3, j4, k1, k2);
        }
    }

    __device__ __noinline__ void junction(int j1, int j2, int j3, int j4, int k1, int k2) {   // :419
        if (sd[k1] > sd[k2]) {
            int t = k1; k1 = k2; k2 = t;
            t = j1; j1 = j4; j4 = t;
            t = j2; j2 = j3; j3 = t;
        }
        if (!(pair_stacked(j1, j2) && pair_stacked(j3, j4))) return;
        if (!junction_ok(j1, j2, k1, k2)) {
            fbst().viol = true;
            return;
        }
        int pen = junction_penalty(j1, j2, j3, j4, k1, k2);
        if (pen == 1) {
            fbst().pd.e -= stack(j1, j2) / 2;
            fbst().pd.e -= stack(j3, j4) / 2;
            fbst().pd.stacked -= 1;
        }
        else if (pen == 2) {
            fbst().pd.e -= stack(j1, j2);
            fbst().pd.e -= stack(j3, j4);
            fbst().pd.stacked -= 2;
        }
    }

    __device__ __noinline__ void backward_triplets(int c1, int c2) {   // :464
        int h2 = c1, h3 = c2;
        if (!pair_stacked(h2, h3)) return;
        int h1 = next(c1, -1);
        bool h23_dc = doubly_contig(h2, h3);
        if (exists_bound(h1)) {
            bool h12_dc = doubly_contig(h1, h2);
            if (pair_stacked(h1, h2)) {
                if (h12_dc && h23_dc) {
                    triply_contig_helix(h1, h2, h3);
                    if (fbst().viol) return;
                }
                triplet_double(h1, h2, h3);
            }
            else {
                triplet_single(h1, h2, h3);
            }
        }
        int h2_prev = h1;
        int b1 = gbnd(c1);
        h1 = next(b1, 1);
        if (exists_bound(h1) && gbnd(h1) != h2_prev && gbnd(h1) != h3) {
            if (pair_stacked(b1, h1)) triplet_double(h1, h2, h3);
        }
        h1 = next(b1, -1);
        if (exists_bound(h1) && gbnd(h1) != h2_prev && gbnd(h1) != h3) {
            if (pair_stacked(h1, b1)) triplet_double(h1, h2, h3);
            else triplet_single(h1, b1, h3);
        }
    }

    __device__ __noinline__ void forward_triplets(int c1, int c2) {   // :521
        int h2 = c2, h1 = c1;
        bool first = pair_stacked(h1, h2);
        int h3 = next(c2, 1);
        bool h12_dc = doubly_contig(h1, h2);
        if (exists_bound(h3)) {
            bool second = pair_stacked(h2, h3);
            if (first && second) {
                bool h23_dc = doubly_contig(h2, h3);
                if (h12_dc && h23_dc) {
                    triply_contig_helix(h1, h2, h3);
                    if (fbst().viol) return;
                }
                triplet_double(h1, h2, h3);
            }
            else if (second) {
                triplet_single(h1, h2, h3);
            }
        }
        int h2_next = h3;
        int b2 = gbnd(c2);
        h3 = next(b2, 1);
        if (exists_bound(h3) && gbnd(h3) != h2_next && gbnd(h3) != h1) {
            if (pair_stacked(b2, h3)) {
                if (first) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
        }
        h3 = next(b2, -1);
        if (exists_bound(h3) && gbnd(h3) != h2_next && gbnd(h3) != h1) {
            if (pair_stacked(h3, b2)) {
                if (first) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
            else if (first) {
                triplet_single(h3, b2, h1);
            }
        }
    }

    __device__ __noinline__ void central_triplets(int i, int j) {   // :587
        int h1 = next(i, -1);
        int h2 = i;
        int h3 = next(j, 1);
        int h2_next = next(i, 1);
        if (exists_bound(h1) && exists_bound(h3) && gbnd(h3) != h2_next && !doubly_contig(h1, h2)) {
            if (pair_stacked(j, h3)) {
                if (pair_stacked(h1, h2)) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
        }
        h3 = next(j, -1);
        if (exists_bound(h1) && exists_bound(h3) && gbnd(h3) != h1 && !doubly_contig(h1, h2)) {
            if (pair_stacked(h1, h2)) {
                if (pair_stacked(h3, j)) triplet_double(h1, h2, h3);
                else triplet_single(h3, j, h1);
            }
            else if (pair_stacked(h3, j)) {
                triplet_single(h1, h2, h3);
            }
        }
        h2 = i;
        h3 = next(i, 1);
        h1 = next(j, 1);
        int h2_prev = next(i, -1);
        if (exists_bound(h1) && exists_bound(h3) && gbnd(h1) != h3 && !doubly_contig(h2, h3)) {
            if (pair_stacked(j, h1) && pair_stacked(h2, h3)) triplet_double(h1, h2, h3);
        }
        h1 = next(j, -1);
        if (exists_bound(h1) && exists_bound(h3) && gbnd(h1) != h2_prev && !doubly_contig(h2, h3)) {
            if (pair_stacked(h2, h3)) {
                if (pair_stacked(h1, j)) triplet_double(h1, h2, h3);
                else triplet_single(h1, j, h3);
            }
        }
    }

    // The three single-junction searches (:654, :750, :846) share one shape:
    // up to three kink pairs, then up to three second junction pairs each.
    __device__ __noinline__ void backward_single_junction(int c1, int c2) {   // :654
        int j3 = c1, j4 = c2;
        FBState& F = fbst();
        int* fa = F.fa;
        int* fb = F.fb;
        int nf = 0;
        int j3_bac = bwd(j3);
        fa[nf] = j3; fb[nf] = j3_bac; nf++;
        int j3_b = gbnd(j3);
        int j3_b_for = fwd(j3_b), j3_b_bac = bwd(j3_b);
        if (j3_b_for == gbnd(j4)) {
            fa[nf] = j3_b; fb[nf] = j3_b_bac; nf++;
        }
        else if (exists_bound(j3_bac) && exists_bound(j3_b_bac) && gbnd(j3_bac) == j3_b_bac) {
            fa[nf] = j3_b; fb[nf] = j3_b_for; nf++;
        }
        else if (exists_bound(j3_bac) && exists_bound(j3_b_for) && gbnd(j3_bac) == j3_b_for) {
            fa[nf] = j3_b; fb[nf] = j3_b_bac; nf++;
        }
        else {
            fa[nf] = j3_b; fb[nf] = j3_b_for; nf++;
            fa[nf] = j3_b; fb[nf] = j3_b_bac; nf++;
        }
        #pragma unroll 1
        for (int a = 0; a < nf; ++a) {
            int k2 = fa[a], k1 = fb[a];
            if (!exists_bound(k1)) continue;
            if (pair_stacked(k1, k2)) continue;
            int* sa = F.sa;
            int* sb = F.sb;
            int ns_ = 0;
            int dir = sd[k1] - sd[k2];
            int k1_next = next(k1, dir);
            sa[ns_] = k1; sb[ns_] = k1_next; ns_++;
            int k1_b = gbnd(k1);
            int k1_b_for = fwd(k1_b), k1_b_bac = bwd(k1_b);
            if (exists_bound(k1_next)) {
                int kn_b = gbnd(k1_next);
                if (k1_b_for != kn_b) { sa[ns_] = k1_b; sb[ns_] = k1_b_for; ns_++; }
                if (k1_b_bac != kn_b) { sa[ns_] = k1_b; sb[ns_] = k1_b_bac; ns_++; }
            }
            else {
                sa[ns_] = k1_b; sb[ns_] = k1_b_for; ns_++;
                sa[ns_] = k1_b; sb[ns_] = k1_b_bac; ns_++;
            }
            #pragma unroll 1
            for (int b = 0; b < ns_; ++b) {
                int j2 = sa[b], j1 = sb[b];
                if (!exists_bound(j1)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    __device__ __noinline__ void forward_single_junction(int c1, int c2) {   // :750
        int j1 = c1, j2 = c2;
        FBState& F = fbst();
        int* fa = F.fa;
        int* fb = F.fb;
        int nf = 0;
        int j2_for = fwd(j2);
        fa[nf] = j2; fb[nf] = j2_for; nf++;
        int j1_b = gbnd(j1);
        int j2_b = gbnd(j2);
        int j2_b_for = fwd(j2_b), j2_b_bac = bwd(j2_b);
        if (next(j1_b, 1) == j2_b) {
            fa[nf] = j2_b; fb[nf] = j2_b_for; nf++;
        }
        else if (exists_bound(j2_for) && exists_bound(j2_b_bac) && gbnd(j2_for) == j2_b_bac) {
            fa[nf] = j2_b; fb[nf] = j2_b_for; nf++;
        }
        else if (exists_bound(j2_for) && exists_bound(j2_b_for) && gbnd(j2_for) == j2_b_for) {
            fa[nf] = j2_b; fb[nf] = j2_b_bac; nf++;
        }
        else {
            fa[nf] = j2_b; fb[nf] = j2_b_for; nf++;
            fa[nf] = j2_b; fb[nf] = j2_b_bac; nf++;
        }
        #pragma unroll 1
        for (int a = 0; a < nf; ++a) {
            int k1 = fa[a], k2 = fb[a];
            if (!exists_bound(k2)) continue;
            if (pair_stacked(k1, k2)) continue;
            int* sa = F.sa;
            int* sb = F.sb;
            int ns_ = 0;
            int dir = sd[k2] - sd[k1];
            int k2_next = next(k2, dir);
            sa[ns_] = k2; sb[ns_] = k2_next; ns_++;
            int k2_b = gbnd(k2);
            int k2_b_for = fwd(k2_b), k2_b_bac = bwd(k2_b);
            if (exists_bound(k2_next)) {
                int kn_b = gbnd(k2_next);
                if (k2_b_for != kn_b) { sa[ns_] = k2_b; sb[ns_] = k2_b_for; ns_++; }
                if (k2_b_bac != kn_b) { sa[ns_] = k2_b; sb[ns_] = k2_b_bac; ns_++; }
            }
            else {
                sa[ns_] = k2_b; sb[ns_] = k2_b_for; ns_++;
                sa[ns_] = k2_b; sb[ns_] = k2_b_bac; ns_++;
            }
            #pragma unroll 1
            for (int b = 0; b < ns_; ++b) {
                int j3 = sa[b], j4 = sb[b];
                if (!exists_bound(j4)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    __device__ __noinline__ void central_single_junction(int c1, int c2) {   // :846
        int k1 = c1, k2 = c2;
        int kb1 = gbnd(k1), kb2 = gbnd(k2);
        int dd = sd[kb1] - sd[kb2];
        if (scs[kb1] == scs[kb2] && (dd == 1 || dd == -1)) return;
        FBState& F = fbst();
        int* fa = F.fa;
        int* fb = F.fb;
        int nf = 0;
        int k1_bac = bwd(k1);
        fa[nf] = k1; fb[nf] = k1_bac; nf++;
        int k1_b_for = fwd(kb1), k1_b_bac = bwd(kb1);
        if (exists_bound(k1_bac)) {
            int kbb = gbnd(k1_bac);
            if (k1_b_for != kbb) { fa[nf] = kb1; fb[nf] = k1_b_for; nf++; }
            if (k1_b_bac != kbb) { fa[nf] = kb1; fb[nf] = k1_b_bac; nf++; }
        }
        else {
            fa[nf] = kb1; fb[nf] = k1_b_for; nf++;
            fa[nf] = kb1; fb[nf] = k1_b_bac; nf++;
        }
        #pragma unroll 1
        for (int a = 0; a < nf; ++a) {
            int j2 = fa[a], j1 = fb[a];
            if (!exists_bound(j1)) continue;
            int* sa = F.sa;
            int* sb = F.sb;
            int ns_ = 0;
            int k2_for = fwd(k2);
            sa[ns_] = k2; sb[ns_] = k2_for; ns_++;
            int k2_b_for = fwd(kb2), k2_b_bac = bwd(kb2);
            if (exists_bound(k2_for)) {
                int kfb = gbnd(k2_for);
                if (k2_b_for != kfb) { sa[ns_] = kb2; sb[ns_] = k2_b_for; ns_++; }
                if (k2_b_bac != kfb) { sa[ns_] = kb2; sb[ns_] = k2_b_bac; ns_++; }
            }
            else {
                sa[ns_] = kb2; sb[ns_] = k2_b_for; ns_++;
                sa[ns_] = kb2; sb[ns_] = k2_b_bac; ns_++;
            }
            #pragma unroll 1
            for (int b = 0; b < ns_; ++b) {
                int j3 = sa[b], j4 = sb[b];
                if (!exists_bound(j4)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    // OrigamiPotential::bind_domain (:1282) with BindingPotential::bind_domains
    // (:131) and the misbinding potentials (:938, :947)
    __device__ __noinline__ Delta bind_domain(int i) {
        fbst().viol = false;
        int j = gbnd(i);
        Delta dc;
        dc.e = 0;
        dc.stacked = 0;
        if (did[i] == -did[j]) {
            fbst().pd.e = 0;
            fbst().pd.stacked = 0;
            if (gore(i) != (gore(j) ^ 1)) {
                fbst().viol = true;
                return dc;
            }
            stacking_and_steric(i, j);
            if (fbst().viol) return dc;
            fbst().pd.e += hyb(i, j);
            dc = fbst().pd;
        }
        else {
            fbst().viol = true;
            if (sys->mis_disallowed) return dc;
            if (gore(i) != (gore(j) ^ 1)) return dc;
            fbst().viol = false;
            dc.e += hyb(i, j);
        }
        return dc;
    }
    __device__ __noinline__ Delta check_stacking(int i, int j) {   // :149
        fbst().pd.e = 0;
        fbst().pd.stacked = 0;
        fbst().viol = false;
        stacking_and_steric(i, j);
        return fbst().pd;
    }

    // ======================================== order parameters / biases ===
    __device__ __noinline__ bool staple_type_fully_bound(int type) const {
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 1; c < nc; ++c) {
            int cs = chain_order[c];
            if (chain_type[cs] != type) continue;
            int len = chain_len(cs);
            bool full = true;
            #pragma unroll 1
            for (int d = 0; d < len; ++d)
                if (st[slot_of(cs, d)] != BOUND) { full = false; break; }
            if (full) return true;
        }
        return false;
    }
    // SystemOrderParams::update_move_params (src/order_params.cpp:595)
    __device__ __noinline__ void update_move_params() {
        const LdoSys* s = sys;
        #pragma unroll 1
        for (int q = 0; q < s->n_ops; ++q) {
            int v = 0;
            int defined = 1;
            switch (s->op_kind[q]) {
            case LDO_OP_NUMSTAPLES: v = hdr.num_staples; break;
            case LDO_OP_NUMSTAPLESTYPE: v = type_count[s->op_arg[q]]; break;
            case LDO_OP_STAPLETYPEFULLYBOUND: v = staple_type_fully_bound(s->op_arg[q]) ? 1 : 0; break;
            case LDO_OP_NUMBOUND: v = hdr.num_fully; break;
            case LDO_OP_NUMMISBOUND: v = hdr.num_bound - hdr.num_fully; break;
            case LDO_OP_NUMSTACKED: v = hdr.num_stacked; break;
            case LDO_OP_ZERO: v = 0; break;
            case LDO_OP_SUM: {
                #pragma unroll 1
                for (int p = 0; p < s->op_nparts[q]; ++p) {
                    int part = s->op_parts[q][p];
                    if (op[2 * part + 1]) v += op[2 * part];
                    else { defined = 0; v = op[2 * q]; break; }
                }
                break;
            }
            case LDO_OP_DIST:
            case LDO_OP_ADJACENT: {
                // DistOrderParam / AdjacentSiteOrderParam::calc_param
                // (src/order_params.cpp:35, :84): defined while both domains
                // are assigned; the value is kept while undefined
                int a = s->op_parts[q][0], b = s->op_parts[q][1];
                if (st[a] != UNASSIGNED && st[b] != UNASSIGNED) {
                    V3 d = sub(pos(b), pos(a));
                    int l1 = abs(vx(d)) + abs(vy(d)) + abs(vz(d));
                    v = s->op_kind[q] == LDO_OP_DIST ? l1 : (l1 == 1 ? 1 : 0);
                }
                else {
                    defined = 0;
                    v = op[2 * q];
                }
                break;
            }
            }
            op[2 * q] = v;
            op[2 * q + 1] = defined;
        }
    }
    __device__ __noinline__ double bias_value(int b) const {
        const LdoSys* s = sys;
        int oq = s->bias_op[b];
        if (!op[2 * oq + 1]) return 0;
        int x = op[2 * oq];
        switch (s->bias_kind[b]) {
        case LDO_B_LINEARSTEPWELL: {   // src/bias_functions.cpp:139
            int mn = ctl->win_min[b], mx = ctl->win_max[b];
            if (x < mn) return s->bias_slope[b] * (mn - x - 1) + s->bias_minb[b];
            if (x > mx) return s->bias_slope[b] * (x - mx - 1) + s->bias_minb[b];
            return s->bias_well[b];
        }
        case LDO_B_SQUAREWELL: {   // :194
            int mn = ctl->win_min[b], mx = ctl->win_max[b];
            if (x < mn || x > mx) return s->bias_outside[b];
            return s->bias_well[b];
        }
        case LDO_B_GRID: {   // :242
            int off = ctl->grid_off[b];
            if (off >= 0 && x >= 0 && x < s->bias_grid_len[b]) return grid[off + x];
            return 0.0;
        }
        case LDO_B_HARMONIC: {
            double dx = x - ctl->centre[b];
            return 0.5 * s->bias_k[b] * dx * dx;
        }
        }
        return 0;
    }
    // SystemBiases::calc_move (src/bias_functions.cpp:475)
    __device__ __noinline__ double calc_move() {
        double diff = 0;
        #pragma unroll 1
        for (int b = 0; b < sys->n_biases; ++b) {
            double prev = bias[b];
            double nb = bias_value(b);
            bias[b] = nb;
            diff += nb - prev;
        }
        hdr.move_bias += diff;
        return diff * c_bias_mult;
    }
    __device__ __noinline__ void init_biases() {
        update_move_params();
        hdr.move_bias = 0;
        #pragma unroll 1
        for (int b = 0; b < sys->n_biases; ++b) {
            bias[b] = bias_value(b);
            hdr.move_bias += bias[b];
        }
    }

    // ============================================================ moves ===
    __device__ void reset_internal() {   // src/movetypes.cpp:242
        m.n_mod = 0;
        m.n_asg = 0;
        m.added_cs = -1;
        rejected = false;
        modifier = 1;
        delta_e = 0;
        w_bias = 1;
        w_new_bias = 1;
        new_modifier = 1;
        regrow_old = false;
        dirty = true;
        phase = 0;
    }

    __device__ __noinline__ void reset_origami() {   // src/movetypes.cpp:53
        #pragma unroll 1
        for (int n = 0; n < m.n_asg; ++n) unassign_domain(m.asg[n]);
        if (m.added_cs >= 0) {
            delete_chain(m.added_cs);
            hdr.current_c_i -= 1;
        }
        #pragma unroll 1
        for (int n = 0; n < m.n_mod; ++n) set_checked(m.mod[n], m.mod_pos[n], m.mod_ore[n]);
        hdr.violated = 0;
    }

    __device__ __noinline__ bool test_acceptance(double p) {   // src/movetypes.cpp:142
        double pa = fmin(1.0, p) * modifier;
        if (pa == 1) return true;
        return pa > rng.uniform_real();
    }

    __device__ __noinline__ int select_random_domain() {   // src/movetypes.cpp:98
        int idx = rng.uniform_int(0, hdr.num_domains - 1);
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            if (idx < len) return slot_of(cs, idx);
            idx -= len;
        }
        return -1;
    }

    // staple_is_connector / scan_for_scaffold_domain (src/movetypes.cpp:160-232):
    // reachability of the scaffold from the partner chain, not passing through
    // the staple, over bound and misbound pairs.
    __device__ __noinline__ bool staple_is_connector(int cs) {
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int i = slot_of(cs, d);
            if (st[i] == UNBOUND) continue;
            int b = bnd[i];
            if (b < 0) {
                fail(LDO_RS_INVARIANT);
                return false;
            }
            if (chain_c[scs[b]] == 0) continue;
            if (!reaches_scaffold(scs[b], cs)) return true;
        }
        return false;
    }
    __device__ __noinline__ bool reaches_scaffold(int start, int excluded) {
        unsigned long long seen = (1ull << excluded) | (1ull << start);
        uint8_t* stack_ = dfs_stack;
        int sp = 0;
        stack_[sp++] = (uint8_t)start;
        #pragma unroll 1
        while (sp > 0) {
            int x = stack_[--sp];
            int len = chain_len(x);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int b = bnd[slot_of(x, d)];
                if (b < 0) continue;
                int cx = scs[b];
                if (cx == x) continue;
                if (chain_c[cx] == 0) return true;
                if (seen & (1ull << cx)) continue;
                seen |= 1ull << cx;
                stack_[sp++] = (uint8_t)cx;
            }
        }
        return false;
    }

    __device__ __noinline__ int num_bound_staple_domains(int cs) const {   // src/movetypes.cpp:395
        int n = 0, len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int o = st[slot_of(cs, d)];
            if (o == BOUND || o == MISBOUND) n++;
        }
        return n;
    }

    __device__ __noinline__ void find_bound_domains(int cs) {   // src/movetypes.cpp:258
        m.n_bd = 0;
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int i = slot_of(cs, d);
            int b = bnd[i];
            if (b >= 0 && scs[b] != cs) {
                m.bd_new[m.n_bd] = i;
                m.bd_old[m.n_bd] = b;
                m.n_bd++;
            }
        }
        if (m.n_bd == 0) fail(LDO_RS_INVARIANT);   // "System has unbound staple"
    }

    __device__ __noinline__ void unassign_domains(int cs) {   // src/met_movetypes.cpp:77
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int i = slot_of(cs, d);
            m.mod[m.n_mod] = i;
            m.mod_pos[m.n_mod] = pos(i);
            m.mod_ore[m.n_mod] = ore[i];
            m.n_mod++;
            double de = unassign_domain(i);
            delta_e += de;
        }
    }

    // RegrowthMCMovetype::set_growth_point (src/movetypes.cpp:322)
    __device__ __noinline__ double set_growth_point(int gnew, int gold) {
        double de = set_domain_config(gnew, pos(gold), ore[gold] ^ 1);
        if (hdr.violated) rejected = true;
        else m.asg[m.n_asg++] = gnew;
        return de;
    }

    // MetMCMovetype::grow_chain (src/met_movetypes.cpp:50) over the domains
    // d0, d0+dir, ... of chain slot cs (count of them, including d0).
    __device__ __noinline__ void met_grow_chain(int cs, int d0, int dir, int count) {
        #pragma unroll 1
        for (int n = 1; n < count; ++n) {
            int i = slot_of(cs, d0 + dir * n);
            int prev = slot_of(cs, d0 + dir * (n - 1));
            V3 p = add(pos(prev), unit(rng.uniform_int(0, 5)));
            int o = rng.uniform_int(0, 5);
            delta_e += set_domain_config(i, p, o);
            if (hdr.violated) {
                rejected = true;
                break;
            }
            m.asg[m.n_asg++] = i;
        }
    }

    // RegrowthMCMovetype::grow_staple (src/movetypes.cpp:343)
    __device__ __noinline__ void grow_staple(int d_i, int cs, bool cb) {
        int len = chain_len(cs);
        int n3 = len - d_i;
        if (n3 > 1) {
            if (cb) cb_grow_chain(cs, d_i, 1, n3);
            else met_grow_chain(cs, d_i, 1, n3);
        }
        if (rejected || bad()) return;
        int n5 = d_i + 1;
        if (n5 > 1) {
            if (cb) cb_grow_chain(cs, d_i, -1, n5);
            else met_grow_chain(cs, d_i, -1, n5);
        }
    }

    __device__ void add_external_bias_met() {   // src/met_movetypes.cpp:69
        update_move_params();
        delta_e += calc_move();
    }

    __device__ __noinline__ bool exchange_accept_common(int type, double pratio) {   // src/met_movetypes.cpp:227-252
        if (staple_bound) {
            modifier *= sys->exchange_mults[type - 1];
            if (modifier * fmin(1.0, pratio) > 1) {
                if (sys->adaptive_exchange) return false;
                if (sys->allow_nonsensical) return true;
                fail(LDO_RS_INVARIANT);   // "Nonsensical exchange probability detected"
                return false;
            }
        }
        return test_acceptance(pratio);
    }

    // MetStapleExchangeMCMovetype::insert_staple (src/met_movetypes.cpp:303)
    __device__ __noinline__ bool insert_staple() {
        int S = sys->n_types - 1;
        int type = rng.uniform_int(1, S);
        if (hdr.num_staples == sys->max_total_staples || type_count[type] == sys->max_type_staples) {
            dirty = false;
            return false;
        }
        int cs = add_chain(type);
        if (cs < 0) return false;
        if (mean_field) delta_e += log6;
        delta_e += t_init_e;
        m.added_cs = cs;
        int len = chain_len(cs);
        int gi = rng.uniform_int(0, len - 1);
        int gnew = slot_of(cs, gi);
        int gold = select_random_domain();
        int guard = 0;
        #pragma unroll 1
        while (scs[gold] == cs) {
            gold = select_random_domain();
            if (++guard > LDO_GROWTHPOINT_CAP) {
                fail(LDO_RS_ITERCAP);
                return false;
            }
        }
        delta_e += set_growth_point(gnew, gold);
        if (rejected || bad()) return false;
        grow_staple(gi, cs, false);
        if (rejected || bad()) return false;
        #pragma unroll 1
        for (int d = 0; d < len; ++d)
            if (st[slot_of(cs, d)] == BOUND) { staple_bound = true; break; }
        int nbd = num_bound_staple_domains(cs);
        add_external_bias_met();
        double boltz = dexp(-delta_e);
        int ni = type_count[type];
        double pratio = (double)len / 6.0 / ni * boltz;
        pratio *= insertion_sites * c_staple_M;
        pratio /= nbd;
        return exchange_accept_common(type, pratio);
    }

    // MetStapleExchangeMCMovetype::delete_staple (src/met_movetypes.cpp:361)
    __device__ __noinline__ bool delete_staple() {
        int S = sys->n_types - 1;
        int type = rng.uniform_int(1, S);
        int n = type_count[type];
        if (n == 0) {
            rejected = true;
            dirty = false;
            return false;
        }
        int which = rng.uniform_int(0, n - 1);
        int cs = -1;
        #pragma unroll 1
        for (int c = 1; c < hdr.n_chains; ++c) {
            int x = chain_order[c];
            if (chain_type[x] == type) {
                if (which == 0) { cs = x; break; }
                --which;
            }
        }
        if (cs < 0) {
            fail(LDO_RS_INVARIANT);
            return false;
        }
        if (staple_is_connector(cs)) {
            dirty = false;
            return false;
        }
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d)
            if (st[slot_of(cs, d)] == BOUND) { staple_bound = true; break; }
        int nbd = num_bound_staple_domains(cs);
        unassign_domains(cs);
        if (mean_field) delta_e -= log6;
        delta_e -= t_init_e;
        hdr.num_staples--;
        add_external_bias_met();
        hdr.num_staples++;
        double boltz = dexp(-delta_e);
        int ni = type_count[type];
        double pratio = ni * 6.0 / (double)len * boltz;
        pratio /= c_staple_M * (double)(unsigned long long)(insertion_sites - len);
        pratio *= nbd;
        bool acc = exchange_accept_common(type, pratio);
        if (acc) delete_chain(cs);
        return acc;
    }

    __device__ __noinline__ bool met_exchange() {   // src/met_movetypes.cpp:192
        insertion_sites = hdr.num_domains;
        staple_bound = false;
        if (rng.uniform_real() < 0.5) return insert_staple();
        return delete_staple();
    }


    // ================================ learned insertion proposal (engine) ===
    // LearnedStapleExchange: the reference's staple exchange with a proposal
    // for insertion targets learned from the plain sampler.  An insertion
    // picks the growth-point target g with probability
    //   q(g) = eps / N + (1 - eps) * [g unbound scaffold domain] w(g) / Z,
    // Z = sum of w over the unbound scaffold domains (q = 1/N when Z = 0),
    // w(g) = exp(network logit) of g's neighbourhood
    // (ldo_learn.h), then the staple type and domain complementary to g with
    // probability 1 - eps_t (uniform type and domain otherwise); the other
    // domains grow with the learned directions (lr_grow).  The forward
    // probability of the new configuration sums q(partner) q(type, d) G(d)
    // over the staple's bound domains d (each could have been the growth
    // point; G the growth factor), so the Metropolis-Hastings ratio is the
    // reference's (src/met_movetypes.cpp:212-301) with its uniform proposal
    // factor n_bd / (S L N) replaced by that sum.  Deletions choose the staple
    // by del_q (weighted towards partly bound staples) instead of the
    // reference's 1 / (S N_i); both ratios use del_q for the staple that the
    // deletion removes or the reverse deletion would remove.

    // Neighbour-state code: 0 none, 1 unbound or unassigned, 2 bound,
    // 3 misbound; a domain bound to chain `fresh` (the staple being inserted)
    // counts as unbound, its state before the insertion.
    __device__ __forceinline__ int learn_code(int n, int fresh) const {
        if (n < 0) return 0;
        int s = st[n];
        if (s == BOUND || s == MISBOUND) {
            if (fresh >= 0 && scs[bnd[n]] == fresh) return 1;
            return s == BOUND ? 2 : 3;
        }
        return 1;
    }
    __device__ __noinline__ double learn_weight(int g, int fresh) const {
        int p1 = bwd(g), n1 = fwd(g);
        int p2 = p1 >= 0 ? bwd(p1) : -1;
        int n2 = n1 >= 0 ? fwd(n1) : -1;
        int combo = learn_code(p2, fresh) | (learn_code(p1, fresh) << 2) | (learn_code(n1, fresh) << 4) |
                    (learn_code(n2, fresh) << 6);
        int ts = scs[g] == 0 ? (int)sys->learn_tslot[sd[g]] : 0;
        return __ldg(learn_w + ldo_learn_index(learn_tb, ts, combo));
    }
    // Training data for the network: every bound (label 1) or unbound
    // (label 0) domain, counted at its network input (FP64 counters: exact
    // integers past the 2^24 where single-precision increments stop).
    __device__ __noinline__ void learn_collect(double* cnt_b, double* cnt_t) const {
        int nc = hdr.n_chains;
        #pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int g = slot_of(cs, d);
                int s = st[g];
                if (s != BOUND && s != UNBOUND) continue;
                int p1 = bwd(g), n1 = fwd(g);
                int p2 = p1 >= 0 ? bwd(p1) : -1;
                int n2 = n1 >= 0 ? fwd(n1) : -1;
                int combo = learn_code(p2, -1) | (learn_code(p1, -1) << 2) | (learn_code(n1, -1) << 4) |
                            (learn_code(n2, -1) << 6);
                int ts = cs == 0 ? (int)sys->learn_tslot[d] : 0;
                int k = ldo_learn_index(learn_tb, ts, combo);
                atomicAdd(cnt_t + k, 1.0);
                if (s == BOUND) atomicAdd(cnt_b + k, 1.0);
            }
        }
        // regrowth directions: for every placed staple domain next to a
        // placed chain neighbour, the six sites next to that neighbour as
        // they would be without the domain, labelled by where it is
        #pragma unroll 1
        for (int c = 1; c < nc; ++c) {
            int cs = chain_order[c];
            int len = chain_len(cs);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) {
                int i = slot_of(cs, d);
                if (st[i] == UNASSIGNED) continue;
                #pragma unroll 1
                for (int side = 0; side < 2; ++side) {
                    int prev = side == 0 ? bwd(i) : fwd(i);
                    if (prev < 0 || st[prev] == UNASSIGNED) continue;
                    int vstar = unit_index(sub(pos(i), pos(prev)));
                    #pragma unroll 1
                    for (int v = 0; v < 6; ++v) {
                        int f;
                        if (v == vstar) {
                            int j = bnd[i];
                            f = (st[i] == UNBOUND || j < 0) ? 0 : (did[i] == -did[j] ? 1 : 2);
                        }
                        else {
                            f = lr_site_class(i, add(pos(prev), unit(v)), nullptr);
                        }
                        int k = ldo_learn_dir_index(learn_tb, f);
                        atomicAdd(cnt_t + k, 1.0);
                        if (v == vstar) atomicAdd(cnt_b + k, 1.0);
                    }
                }
            }
        }
    }
    // Class of site p for growing domain i: 0 empty, 1 an unbound domain
    // complementary to i, 2 another unbound domain, 3 a bound pair; *ob (if
    // given) the orientation that binds to the unbound domain, else -1.
    __device__ int lr_site_class(int i, V3 p, int* ob) const {
        int occ = occupancy(p);
        if (ob) *ob = -1;
        if (occ == UNASSIGNED) return 0;
        if (occ == UNBOUND) {
            int j = unbound_at(p);
            if (ob) *ob = ore[j] ^ 1;
            return did[i] == -did[j] ? 1 : 2;
        }
        return 3;
    }
    // The learned direction and orientation proposal of domain i grown from
    // its placed chain neighbour prev: q(v) = eps_d/6 + (1 - eps_d) w(v)/Z over
    // the six sites, then q(o | v) = eps_o/6 + (1 - eps_o)[o binds] at a site
    // with an unbound domain, 1/6 elsewhere.  With sample set it draws (v, o)
    // (one uniform real for v, then at an unbound site one for the binding
    // choice and, if not taken, a uniform orientation); it returns q(v) q(o|v)
    // of (*v, *o).
    __device__ __noinline__ double lr_propose(int i, int prev, bool sample, int* vo, int* oo) {
        double w[6];
        int ob[6];
        double z = 0;
        V3 base = pos(prev);
        #pragma unroll 1
        for (int v = 0; v < 6; ++v) {
            int f = lr_site_class(i, add(base, unit(v)), &ob[v]);
            w[v] = __ldg(learn_w + ldo_learn_dir_index(learn_tb, f));
            z += w[v];
        }
        int v = *vo;
        if (sample) {
            double r = rng.uniform_real();
            double cum = 0;
            v = 5;
            #pragma unroll 1
            for (int k = 0; k < 6; ++k) {
                cum += z > 0 ? LDO_LEARN_EPS_D / 6.0 + (1.0 - LDO_LEARN_EPS_D) * (w[k] / z) : 1.0 / 6.0;
                if (r < cum) {
                    v = k;
                    break;
                }
            }
            int o;
            if (ob[v] >= 0) {
                double r2 = rng.uniform_real();
                o = r2 < 1.0 - LDO_LEARN_EPS_O ? ob[v] : rng.uniform_int(0, 5);
            }
            else {
                o = rng.uniform_int(0, 5);
            }
            *vo = v;
            *oo = o;
        }
        double qv = z > 0 ? LDO_LEARN_EPS_D / 6.0 + (1.0 - LDO_LEARN_EPS_D) * (w[v] / z) : 1.0 / 6.0;
        double qo = ob[v] >= 0 ? (*oo == ob[v] ? (1.0 - LDO_LEARN_EPS_O) + LDO_LEARN_EPS_O / 6.0
                                               : LDO_LEARN_EPS_O / 6.0)
                               : 1.0 / 6.0;
        return qv * qo;
    }
    // Z over the unbound scaffold domains, in scaffold order.
    // Weights of the unbound scaffold domains in scaffold order.  With pick
    // null: their sum Z.  Otherwise: the first domain at which the running
    // sum exceeds target goes to *pick (the last unbound domain if rounding
    // leaves target at or above Z, -1 if none is unbound).  The scaffold's
    // domains hold slots 0..ns-1 in chain order, so the neighbour codes of
    // learn_weight are kept in a sliding window instead of being looked up
    // four times per domain; the sums are the same, term by term.
    __device__ __noinline__ double learn_scan(double target, int* pick) const {
        if (ns < 5) {
            double z = 0;
            int last = -1;
            #pragma unroll 1
            for (int g = 0; g < ns; ++g) {
                if (st[g] != UNBOUND) continue;
                z += learn_weight(g, -1);
                last = g;
                if (pick && target < z) {
                    *pick = g;
                    return z;
                }
            }
            if (pick) *pick = last;
            return z;
        }
        bool cyc = sys->cyclic;
        auto code_at = [&](int x) {
            if (x < 0 || x >= ns) {
                if (!cyc) return 0;
                x = x < 0 ? x + ns : x - ns;
            }
            return learn_code(x, -1);
        };
        int cm2 = code_at(-2), cm1 = code_at(-1), c0 = code_at(0), cp1 = code_at(1), cp2 = code_at(2);
        const double* tab = learn_w + ldo_learn_index(learn_tb, 0, 0);
        double z = 0;
        int last = -1;
        #pragma unroll 1
        for (int g = 0; g < ns; ++g) {
            if (st[g] == UNBOUND) {
                int combo = cm2 | (cm1 << 2) | (cp1 << 4) | (cp2 << 6);
                z += __ldg(tab + (int)sys->learn_tslot[g] * LDO_LEARN_NCOMBO + combo);
                last = g;
                if (pick && target < z) {
                    *pick = g;
                    return z;
                }
            }
            cm2 = cm1;
            cm1 = c0;
            c0 = cp1;
            cp1 = cp2;
            cp2 = code_at(g + 3);
        }
        if (pick) *pick = last;
        return z;
    }
    // Z of the current state, cached in the header until a scaffold domain's
    // state or the table changes.
    __device__ double learn_z() {
        if (hdr.z_valid) return hdr.z_cache;
        double z = learn_scan(0.0, nullptr);
        hdr.z_cache = z;
        hdr.z_valid = 1;
        return z;
    }
    // q(g) for a target that was unbound in the state the proposal is made in.
    __device__ double learn_q_target(int g, double z, int n_sites, int fresh) const {
        if (z == 0) return 1.0 / n_sites;
        double q = LDO_LEARN_EPS / n_sites;
        if (scs[g] == 0) q += (1.0 - LDO_LEARN_EPS) * (learn_weight(g, fresh) / z);
        return q;
    }
    // q(type, domain d | target g)
    __device__ double learn_q_type(int g, int type, int d) const {
        int S = sys->n_types - 1;
        double u = 1.0 / ((double)S * sys->type_len[type]);
        int ct = scs[g] == 0 ? (int)sys->comp_type[sd[g]] : 0;
        if (ct == 0) return u;
        double q = LDO_LEARN_EPS_T * u;
        if (ct == type && (int)sys->comp_dom[sd[g]] == d) q += 1.0 - LDO_LEARN_EPS_T;
        return q;
    }
    // Sum over the domains d of chain cs bound to another chain of
    // q(partner) q(type, d | partner) G(d), G(d) the growth factor of the
    // chain's other domains grown from d (lr_q_old with scale 36).
    __device__ __noinline__ double learn_forward(int cs, int type, double z, int n_sites, int fresh) {
        double f = 0;
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int b = slot_of(cs, d);
            int p = bnd[b];
            if (p < 0 || scs[p] == cs) continue;
            f += learn_q_target(p, z, n_sites, fresh) * learn_q_type(p, type, d) * lr_q_old(cs, d, 36.0);
        }
        return f;
    }

    // Learned deletion choice: weight of staple chain cs, the weights' sum
    // over the staples in chain order, and the probability of choosing cs.
    __device__ double del_weight(int cs) const {
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d)
            if (st[slot_of(cs, d)] != BOUND) return LDO_LEARN_DEL_PART;
        return 1.0;
    }
    __device__ __noinline__ double del_total() const {
        double u = 0;
        #pragma unroll 1
        for (int c = 1; c < hdr.n_chains; ++c) u += del_weight(chain_order[c]);
        return u;
    }
    __device__ double del_q(int cs, double u) const {
        return LDO_LEARN_EPS_DEL / (double)hdr.num_staples + (1.0 - LDO_LEARN_EPS_DEL) * (del_weight(cs) / u);
    }

    __device__ __noinline__ bool learned_insert() {
        int S = sys->n_types - 1;
        int n_sites = hdr.num_domains;
        double z = learn_z();
        int g = -1;
        double u1 = rng.uniform_real();
        if (z == 0 || u1 < LDO_LEARN_EPS) {
            g = select_random_domain();
        }
        else {
            double target = rng.uniform_real() * z;
            learn_scan(target, &g);
        }
        if (g < 0) {
            fail(LDO_RS_INVARIANT);
            return false;
        }
        int ct = scs[g] == 0 ? (int)sys->comp_type[sd[g]] : 0;
        int type, gi;
        double u3 = rng.uniform_real();
        if (ct != 0 && u3 < 1.0 - LDO_LEARN_EPS_T) {
            type = ct;
            gi = sys->comp_dom[sd[g]];
        }
        else {
            type = rng.uniform_int(1, S);
            gi = rng.uniform_int(0, sys->type_len[type] - 1);
        }
        if (hdr.num_staples == sys->max_total_staples || type_count[type] == sys->max_type_staples) {
            dirty = false;
            return false;
        }
        int cs = add_chain(type);
        if (cs < 0) return false;
        if (mean_field) delta_e += log6;
        delta_e += t_init_e;
        m.added_cs = cs;
        int len = chain_len(cs);
        int gnew = slot_of(cs, gi);
        delta_e += set_growth_point(gnew, g);
        if (rejected || bad()) return false;
        lr_grow(cs, gi);
        if (rejected || bad()) return false;
        #pragma unroll 1
        for (int d = 0; d < len; ++d)
            if (st[slot_of(cs, d)] == BOUND) { staple_bound = true; break; }
        double f = learn_forward(cs, type, z, n_sites, cs);
        add_external_bias_met();
        double boltz = dexp(-delta_e);
        // reverse move: the learned deletion choosing this staple
        double qd = del_q(cs, del_total());
        double pratio = boltz * c_staple_M;
        pratio *= qd;
        pratio /= 6.0 * f;
        return exchange_accept_common(type, pratio);
    }

    __device__ __noinline__ bool learned_delete() {
        if (hdr.num_staples == 0) {
            rejected = true;
            dirty = false;
            return false;
        }
        // the staple: uniform with probability eps, else by deletion weight
        double u_tot = del_total();
        int cs = -1;
        if (rng.uniform_real() < LDO_LEARN_EPS_DEL) {
            cs = pick_staple_chain();
        }
        else {
            double target = rng.uniform_real() * u_tot;
            double cum = 0;
            #pragma unroll 1
            for (int c = 1; c < hdr.n_chains; ++c) {
                cs = chain_order[c];
                cum += del_weight(cs);
                if (target < cum) break;
            }
        }
        if (cs < 0) {
            fail(LDO_RS_INVARIANT);
            return false;
        }
        int type = chain_type[cs];
        double qd = del_q(cs, u_tot);
        if (staple_is_connector(cs)) {
            dirty = false;
            return false;
        }
        int len = chain_len(cs);
        #pragma unroll 1
        for (int d = 0; d < len; ++d)
            if (st[slot_of(cs, d)] == BOUND) { staple_bound = true; break; }
        // growth-point alternatives of the reverse insertion: (domain,
        // partner) and the growth factor of the other domains from there
        int na = 0;
        double gf[LDO_MAX_LEN];
        #pragma unroll 1
        for (int d = 0; d < len; ++d) {
            int b = slot_of(cs, d);
            int p = bnd[b];
            if (p < 0 || scs[p] == cs) continue;
            m.bd_new[na] = d;
            m.bd_old[na] = p;
            gf[na] = lr_q_old(cs, d, 36.0);
            na++;
        }
        if (bad()) return false;
        unassign_domains(cs);
        if (mean_field) delta_e -= log6;
        delta_e -= t_init_e;
        hdr.num_staples--;
        add_external_bias_met();
        hdr.num_staples++;
        double boltz = dexp(-delta_e);
        int n_sites = insertion_sites - len;
        double z = learn_z();
        double f = 0;
        #pragma unroll 1
        for (int a = 0; a < na; ++a)
            f += learn_q_target(m.bd_old[a], z, n_sites, -1) * learn_q_type(m.bd_old[a], type, m.bd_new[a]) * gf[a];
        double pratio = 6.0 * boltz;
        pratio *= f;
        pratio /= qd;
        pratio /= c_staple_M;
        bool acc = exchange_accept_common(type, pratio);
        if (acc) delete_chain(cs);
        return acc;
    }

    __device__ __noinline__ bool learned_exchange() {
        insertion_sites = hdr.num_domains;
        staple_bound = false;
        if (rng.uniform_real() < 0.5) return learned_insert();
        return learned_delete();
    }

    __device__ __noinline__ int pick_staple_chain() {   // uniform_int(1, num_staples) -> get_chains()[i]
        int ci = rng.uniform_int(1, hdr.num_staples);
        return chain_order[ci];
    }

    // LearnedStapleRegrowth (engine extension): MetStapleRegrowthMCMovetype
    // (src/met_movetypes.cpp:470) whose grown domains take direction and
    // orientation from the learned proposal (lr_propose).  The reverse move
    // picks the same growth point among the new configuration's bound pairs
    // and grows the old configuration, so the acceptance is the reference's
    // e^-dE n_bd,old / n_bd,new times Q(old) / Q(new), the products of the
    // proposal probabilities along each growth.

    // Class of site p in a partial growth of staple cs from the state before
    // the move: the staple's domains in `placed` (bit = index in chain) are
    // where they are, the others absent (a partner left behind is unbound).
    __device__ int lr_site_class_partial(int i, V3 p, int cs, unsigned placed, int* ob) const {
        int len = chain_len(cs);
        #pragma unroll 1
        for (int k = 0; k < len; ++k) {
            int x = slot_of(cs, k);
            if (st[x] == UNASSIGNED || pos(x) != p) continue;
            int y = bnd[x];
            bool y_gone = y >= 0 && scs[y] == cs && !(placed >> sd[y] & 1u);
            int alone;   // the domain left alone at p, or -1 for an empty site
            if (placed >> k & 1u) {
                if (st[x] != UNBOUND && !y_gone) {
                    *ob = -1;
                    return 3;
                }
                alone = x;
            }
            else {
                alone = (st[x] == UNBOUND || y_gone) ? -1 : y;
            }
            if (alone < 0) {
                *ob = -1;
                return 0;
            }
            *ob = ore[alone] ^ 1;
            return did[i] == -did[alone] ? 1 : 2;
        }
        return lr_site_class(i, p, ob);
    }
    // Q(old): the proposal probability of growing the current configuration
    // of staple cs from its domain d0, evaluated in the partial states of
    // that growth without building them: the product over the grown domains
    // of scale q(v) q(o | v).
    __device__ __noinline__ double lr_q_old(int cs, int d0, double scale) {
        int len = chain_len(cs);
        unsigned placed = 1u << d0;
        double q = 1;
        #pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            int dir = pass == 0 ? 1 : -1;
            int n = pass == 0 ? len - d0 : d0 + 1;
            #pragma unroll 1
            for (int k = 1; k < n; ++k) {
                int di = d0 + dir * k;
                int i = slot_of(cs, di), prev = slot_of(cs, di - dir);
                double w[6];
                int ob[6];
                double z = 0;
                V3 base = pos(prev);
                #pragma unroll 1
                for (int v = 0; v < 6; ++v) {
                    int f = lr_site_class_partial(i, add(base, unit(v)), cs, placed, &ob[v]);
                    w[v] = __ldg(learn_w + ldo_learn_dir_index(learn_tb, f));
                    z += w[v];
                }
                int v = unit_index(sub(pos(i), base));
                int o = ore[i];
                if (v < 0) {
                    fail(LDO_RS_INVARIANT);
                    return 1;
                }
                double qv = z > 0 ? LDO_LEARN_EPS_D / 6.0 + (1.0 - LDO_LEARN_EPS_D) * (w[v] / z) : 1.0 / 6.0;
                double qo = ob[v] >= 0 ? (o == ob[v] ? (1.0 - LDO_LEARN_EPS_O) + LDO_LEARN_EPS_O / 6.0
                                                     : LDO_LEARN_EPS_O / 6.0)
                                       : 1.0 / 6.0;
                q *= scale * (qv * qo);
                placed |= 1u << di;
            }
        }
        return q;
    }
    // Grows the domains of staple cs other than its placed domain d0 with
    // the learned direction proposal (forward to the chain's end, then
    // backward to its start, as grow_staple does); returns the product of the
    // proposal probabilities, or sets rejected on a constraint violation.
    __device__ __noinline__ double lr_grow(int cs, int d0) {
        double q = 1;
        int len = chain_len(cs);
        #pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            int dir = pass == 0 ? 1 : -1;
            int n = pass == 0 ? len - d0 : d0 + 1;
            #pragma unroll 1
            for (int k = 1; k < n; ++k) {
                int i = slot_of(cs, d0 + dir * k), prev = slot_of(cs, d0 + dir * (k - 1));
                int v = 0, o = 0;
                q *= lr_propose(i, prev, true, &v, &o);
                delta_e += set_domain_config(i, add(pos(prev), unit(v)), o);
                if (hdr.violated) {
                    rejected = true;
                    return 0;
                }
                if (bad()) return 0;
            }
        }
        return q;
    }
    __device__ __noinline__ bool learned_regrowth() {
        dirty = false;
        if (hdr.num_staples == 0) return false;
        int cs = pick_staple_chain();
        if (staple_is_connector(cs)) return false;
        dirty = true;
        find_bound_domains(cs);
        if (bad()) return false;
        int g = rng.uniform_int(0, m.n_bd - 1);
        int gnew = m.bd_new[g], gold = m.bd_old[g];
        int d0 = sd[gnew];
        double q_old = lr_q_old(cs, d0, 1.0);
        unassign_domains(cs);
        delta_e += set_growth_point(gnew, gold);
        if (rejected || bad()) return false;
        double q_new = lr_grow(cs, d0);
        if (rejected || bad()) return false;
        add_external_bias_met();
        int nbd = num_bound_staple_domains(cs);
        double boltz = dexp(-(delta_e));
        double pratio = boltz * (double)(unsigned long long)m.n_bd / nbd;
        pratio *= q_old / q_new;
        return test_acceptance(pratio);
    }

    // MetStapleRegrowthMCMovetype::internal_attempt_move (src/met_movetypes.cpp:470)
    __device__ __noinline__ bool met_regrowth() {
        dirty = false;
        if (hdr.num_staples == 0) return false;
        int cs = pick_staple_chain();
        if (staple_is_connector(cs)) return false;
        dirty = true;
        find_bound_domains(cs);
        if (bad()) return false;
        int g = rng.uniform_int(0, m.n_bd - 1);
        int gnew = m.bd_new[g], gold = m.bd_old[g];
        unassign_domains(cs);
        delta_e += set_growth_point(gnew, gold);
        if (rejected || bad()) return false;
        grow_staple(sd[gnew], cs, false);
        if (rejected || bad()) return false;
        add_external_bias_met();
        int nbd = num_bound_staple_domains(cs);
        double boltz = dexp(-(delta_e));
        double pratio = boltz * (double)(unsigned long long)m.n_bd / nbd;
        return test_acceptance(pratio);
    }

    // CBMCMovetype::select_and_set_config (src/cb_movetypes.cpp:104) with
    // calc_biases (:58) and CBStapleRegrowthMCMovetype::calc_bias (:363)
    __device__ __noinline__ void cb_select_and_set(int dom, int prev) {
        V3 p_prev = pos(prev);
        V3* cpos = cb_pos;
        int* core = cb_ore;
        double* bf = cb_bf;
        int nc = 0;
        // The six neighbour sites in the reference's order: unbound ones are
        // probed, empty ones weigh 6 (no potential is evaluated there:
        // 6 * exp(-0), src/cb_movetypes.cpp:92-99), occupied ones are skipped.
#pragma unroll 1
        for (int v = 0; v < 6; ++v) {
            V3 p = add(p_prev, unit(v));
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND) continue;
            if (occ == UNBOUND) {
                int ud = unbound_at(p);
                int o = ore[ud] ^ 1;
                Delta dc = probe_domain(dom, p, o);
                if (bad()) return;
                if (!hdr.violated) {
                    cpos[nc] = p;
                    core[nc] = o;
                    cb_de[nc] = dc.e;
                    cb_stk[nc] = dc.stacked;
                    double b = 1;
                    b *= dexp(-dc.e);
                    bf[nc] = b;
                    nc++;
                }
                else {
                    hdr.violated = 0;
                }
            }
            else {
                cpos[nc] = p;
                core[nc] = -1;
                bf[nc] = 6.0;
                nc++;
            }
        }
        double ros = 0;
        #pragma unroll 1
        for (int n = 0; n < nc; ++n) ros += bf[n];
        if (ros == 0) {
            rejected = true;
            return;
        }
        w_bias *= ros;
        if (!regrow_old) {
            V3 p = mk(0, 0, 0);
            int o = -1;
            int chosen = -1;
            double cum = 0;
            double r = rng.uniform_real();
            #pragma unroll 1
            for (int n = 0; n < nc; ++n) {
                cum += bf[n] / ros;
                if (r < cum) {
                    p = cpos[n];
                    o = core[n];
                    chosen = n;
                    break;
                }
            }
            if (o < 0) {
                o = rng.uniform_int(0, 5);
                set_checked(dom, p, o);
            }
            else {
                set_checked_probed(dom, p, o, cb_de[chosen], cb_stk[chosen]);
            }
        }
        else {
            int n = 0;
            #pragma unroll 1
            while (n < m.n_old && m.old_slot[n] != dom) ++n;
            V3 p = m.old_pos[n];
            int o = m.old_ore[n];
            int c = 0;
            #pragma unroll 1
            while (c < nc && !(core[c] == o && eq(cpos[c], p))) ++c;
            if (c < nc) set_checked_probed(dom, p, o, cb_de[c], cb_stk[c]);
            else set_checked(dom, p, o);
        }
        m.asg[m.n_asg++] = dom;
    }

    __device__ __noinline__ void cb_grow_chain(int cs, int d0, int dir, int count) {   // src/cb_movetypes.cpp:354
        #pragma unroll 1
        for (int n = 1; n < count; ++n) {
            cb_select_and_set(slot_of(cs, d0 + dir * n), slot_of(cs, d0 + dir * (n - 1)));
            if (rejected || bad()) break;
        }
    }

    __device__ __noinline__ void cb_set_gp_and_grow(int gnew, int gold, int cs) {   // src/cb_movetypes.cpp:389
        if (regrow_old) {
            int n = 0;
            #pragma unroll 1
            while (n < m.n_old && m.old_slot[n] != gnew) ++n;
            double de = 0;
            de += set_checked(gnew, pos(gold), m.old_ore[n]);
            w_bias *= dexp(-de);
            m.asg[m.n_asg++] = gnew;
        }
        else {
            double de = set_growth_point(gnew, gold);
            w_bias *= dexp(-de);
        }
        if (!rejected && !bad()) grow_staple(sd[gnew], cs, true);
    }

    // CBStapleRegrowthMCMovetype::internal_attempt_move (src/cb_movetypes.cpp:292)
    // in three phases around two snapshots: 1 = the staple unassigned, 2 = the
    // staple in its new configuration.  The reference's second
    // unassign_domains (before regrowing the old configuration, :215) becomes
    // a restore of snapshot 1, and its reset_origami on acceptance a restore
    // of snapshot 2: the same lattice states, reached without re-evaluating
    // the binding energies.
    __device__ __noinline__ int cb_begin() {
        dirty = false;
        if (hdr.num_staples == 0) return finish_move(false, 0);
        int cs = pick_staple_chain();
        if (staple_is_connector(cs)) return finish_move(false, 0);
        dirty = true;
        find_bound_domains(cs);
        if (bad()) return finish_move(false, 0);
        w_bias *= (double)(unsigned long long)m.n_bd;
        int g = rng.uniform_int(0, m.n_bd - 1);
        unassign_domains(cs);
        cb_cs = cs;
        m.cb_g = g;
        phase = PH_CB2;
        return CMD_SNAP(1) | CMD_MORE;
    }
    __device__ __noinline__ int cb_mid() {
        int cs = cb_cs, g = m.cb_g;
        cb_set_gp_and_grow(m.bd_new[g], m.bd_old[g], cs);
        if (rejected || bad()) return finish_move(false, 0);
        w_bias /= num_bound_staple_domains(cs);
        update_move_params();
        double tb = calc_move();
        w_bias *= dexp(-tb);
        // setup_for_regrow_old (:215)
        regrow_old = true;
        w_new_bias = w_bias;
        new_modifier = modifier;
        w_bias = 1;
        m.n_old = m.n_mod;
        #pragma unroll 1
        for (int n = 0; n < m.n_mod; ++n) {
            m.old_slot[n] = m.mod[n];
            m.old_pos[n] = m.mod_pos[n];
            m.old_ore[n] = m.mod_ore[n];
        }
        m.n_mod = 0;
        m.n_asg = 0;
        phase = PH_CB3;
        return CMD_SNAP(2) | CMD_REST(1) | CMD_MORE;
    }
    __device__ __noinline__ int cb_end() {
        int cs = cb_cs;
        int g = rng.uniform_int(0, m.n_bd - 1);
        cb_set_gp_and_grow(m.bd_new[g], m.bd_old[g], cs);
        if (bad()) return finish_move(false, 0);
        modifier = new_modifier;
        // test_cb_acceptance (:182)
        double ratio = w_new_bias / w_bias;
        bool acc = test_acceptance(ratio);
        return finish_move(acc, acc ? 2 : 0);
    }

    // OrientationRotationMCMovetype::internal_attempt_move (src/orientation_movetype.cpp:30)
    __device__ __noinline__ bool orientation_rotation() {
        int dom = select_random_domain();
        int o_new = rng.uniform_int(0, 5);
        bool acc = false;
        if (st[dom] == BOUND || st[dom] == MISBOUND) {
            double de = 0;
            int o_old = ore[dom];
            int bd = bnd[dom];
            de += unassign_domain(bd);
            set_domain_orientation(dom, o_new);
            V3 p = pos(dom);
            de += set_domain_config(bd, p, o_new ^ 1);
            if (!hdr.violated) acc = test_acceptance(dexp(-de));
            // a rejection (reference: unassign, old orientation, set_checked
            // of the partner, :55-62) restores the move's snapshot
            (void)o_old;
        }
        else {
            set_domain_orientation(dom, o_new);
            acc = true;
        }
        return acc;
    }

    // ================================ conserved-topology scaffold regrowth ===
    // Constraintpoints / StapleNetwork (src/top_constraint_points.cpp), the
    // segment selection of CTRegrowthMCMovetype (src/movetypes.cpp:469-720),
    // recoil growth (src/rg_movetypes.cpp) and configurational bias
    // (src/cb_movetypes.cpp:406-984).  No staple is ever excluded: the
    // reference's movetype factories pass num_excluded_staples = 0
    // (src/simulation.cpp:409,538).  The maps of the reference are arrays over
    // domain slots in the replica's working memory (LdoCtWork); endpoint lists
    // keep the reference's insertion order.  Reversal goes through the move
    // snapshots: 1 = the regrown domains unassigned, 2 = the new configuration.
    static constexpr unsigned long long CT_ALL36 = (1ull << 36) - 1ull;
    // index of a domain within its chain (scaffold slots are their index)
    __device__ int didx(int i) const { return scs[i] == 0 ? i : sd[i]; }

    __device__ __noinline__ void ct_clear() {   // Constraintpoints::reset_internal (:208)
        LdoCtWork<C>& w = *ct;
        int dc = sys->dcap;
        #pragma unroll 1
        for (int s = 0; s < dc && s < C::DCAP; ++s) {
            w.seg[s] = -1;
            w.gp_to[s] = -1;
            w.stem_of[s] = -1;
            w.inact[s] = -1;
            w.nssegs[s] = 0;
            w.in_scaf[s] = 0;
            w.in_ds[s] = 0;
            w.in_sel[s] = 0;
        }
        #pragma unroll 1
        for (int k = 0; k < LDO_CT_MAX_SEGS; ++k) w.sdir[k] = 0;
        w.checked = 0;
        w.regrow = 0;
        w.n_rd = 0;
        w.n_ep = 0;
        w.n_ep0 = 0;
        w.n_er = 0;
        w.n_eq = 0;
        w.eq_off[0] = 0;
        w.n_segs = 0;
        w.seg_off[0] = 0;
        w.n_stems = 0;
        w.pair_off[0] = 0;
        w.n_fr = 0;
    }

    // ------------------------------------------------------- endpoints ---
    __device__ void ct_add_ep(int cs, int seg, int d, V3 p) {
        LdoCtWork<C>& w = *ct;
        if (w.n_ep >= LdoCtWork<C>::EPC) {
            fail(LDO_RS_CAPACITY);
            return;
        }
        LdoCtEp& e = w.ep[w.n_ep++];
        e.pos = p;
        e.cs = (int16_t)cs;
        e.seg = (int8_t)seg;
        e.d = (int16_t)d;
    }
    // add_active_endpoint(domain, pos, seg) (:280)
    __device__ void ct_add_ep_seg(int i, V3 p, int seg) { ct_add_ep(scs[i], seg, didx(i), p); }
    // add_active_endpoint(domain, pos) (:272): the segment of the domain
    __device__ int ct_seg_at(int i) {   // m_segs.at (throws for a domain without one)
        int sg = ct->seg[i];
        if (sg < 0) fail(LDO_RS_INVARIANT);
        return sg;
    }
    __device__ void ct_add_ep_at(int i, V3 p) { ct_add_ep_seg(i, p, ct_seg_at(i)); }
    // remove_active_endpoint (:300): every endpoint on the domain, kept in m_erased_endpoints
    __device__ __noinline__ void ct_remove_ep(int i) {
        LdoCtWork<C>& w = *ct;
        w.n_er = 0;
        int seg = ct_seg_at(i), cs = scs[i], d = didx(i);
        int k = 0;
        #pragma unroll 1
        for (int j = 0; j < w.n_ep; ++j) {
            LdoCtEp e = w.ep[j];
            if (e.cs == cs && e.seg == seg && e.d == d) w.er[w.n_er++] = e.pos;
            else w.ep[k++] = e;
        }
        w.n_ep = k;
    }
    // remove_activated_endpoint (:325): the first endpoint the domain activated
    __device__ __noinline__ void ct_remove_activated(int i) {
        LdoCtWork<C>& w = *ct;
        int ed = w.inact[i];
        if (ed < 0) return;
        int seg = ct_seg_at(ed), cs = scs[ed], d = didx(ed);
        #pragma unroll 1
        for (int j = 0; j < w.n_ep; ++j) {
            if (w.ep[j].cs == cs && w.ep[j].seg == seg && w.ep[j].d == d) {
                #pragma unroll 1
                for (int q = j; q + 1 < w.n_ep; ++q) w.ep[q] = w.ep[q + 1];
                w.n_ep--;
                break;
            }
        }
    }
    // update_endpoints (:345)
    __device__ __noinline__ void ct_update_endpoints(int i) {
        ct_remove_ep(i);
        int ed = ct->inact[i];
        if (ed >= 0) ct_add_ep_at(ed, pos(i));
    }
    // endpoint_reached (:363)
    __device__ __noinline__ bool ct_endpoint_reached(int i, V3 p) {
        LdoCtWork<C>& w = *ct;
        int seg = ct_seg_at(i), cs = scs[i], d = didx(i);
        #pragma unroll 1
        for (int j = 0; j < w.n_ep; ++j)
            if (w.ep[j].cs == cs && w.ep[j].seg == seg && w.ep[j].d == d && w.ep[j].pos == p) return true;
        return false;
    }
    __device__ void ct_reset_endpoints() {   // reset_active_endpoints (:293)
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int j = 0; j < w.n_ep0; ++j) w.ep[j] = w.ep0[j];
        w.n_ep = w.n_ep0;
    }
    __device__ void ct_push_erased() {   // m_erased_endpoints_q.push_back(get_erased_endpoints())
        LdoCtWork<C>& w = *ct;
        if (w.n_eq + 1 >= C::DCAP + 2 || w.eq_off[w.n_eq] + w.n_er > LdoCtWork<C>::EQC) {
            fail(LDO_RS_CAPACITY);
            return;
        }
        int o = w.eq_off[w.n_eq];
        #pragma unroll 1
        for (int k = 0; k < w.n_er; ++k) w.eq[o + k] = w.er[k];
        w.eq_off[w.n_eq + 1] = (int16_t)(o + w.n_er);
        w.n_eq++;
    }
    // CTRGRegrowthMCMovetype::restore_endpoints (src/rg_movetypes.cpp:289)
    __device__ __noinline__ void ct_restore_endpoints(int i) {
        LdoCtWork<C>& w = *ct;
        ct_remove_activated(i);
        if (w.n_eq <= 0) {
            fail(LDO_RS_INVARIANT);
            return;
        }
        w.n_eq--;
        #pragma unroll 1
        for (int k = w.eq_off[w.n_eq]; k < w.eq_off[w.n_eq + 1]; ++k) ct_add_ep_at(i, w.eq[k]);
    }
    // direction of growth of a (chain, segment): the scaffold's from the
    // selection, a staple's +1 (3' segment 0) or -1 (5' segment 1)
    __device__ int ct_dir_of(int cs, int seg) const {
        if (cs == 0) return (seg >= 0 && seg < LDO_CT_MAX_SEGS) ? ct->sdir[seg] : 0;
        return seg == 0 ? 1 : seg == 1 ? -1 : 0;
    }
    __device__ int ct_get_dir(int i) {   // Constraintpoints::get_dir (:190)
        int sg = ct->seg[i];
        if (sg < 0) {
            ct->seg[i] = 0;
            sg = 0;
        }
        return ct_dir_of(scs[i], sg);
    }
    // calc_remaining_steps (:569)
    __device__ int ct_remaining(int end_d, int i, int dir) const {
        int dd = didx(i);
        if (cyclic && scs[i] == 0) {
            if (dir > 0 && end_d < dd) return ns + end_d - dd;
            if (dir < 0 && end_d > dd) return dd + ns - end_d;
            if (dir == 0 || end_d == dd) return 0;
        }
        return end_d > dd ? end_d - dd : dd - end_d;
    }
    // walks_remain (:398, :424).  IdealRandomWalks::num_walks
    // (src/ideal_random_walk.cpp:14) is zero exactly when the lattice distance
    // exceeds the remaining steps or differs from them in parity, and that
    // is the only use the reference makes of it here.
    __device__ __noinline__ bool ct_walks_ok(int i, V3 p) {
        LdoCtWork<C>& w = *ct;
        int segs_[2];
        int n;
        if (w.stem_of[i] >= 0) {
            n = w.nssegs[i];
            segs_[0] = w.ssegs[i][0];
            segs_[1] = w.ssegs[i][1];
        }
        else {
            n = 1;
            segs_[0] = ct_seg_at(i);
        }
        int cs = scs[i];
        #pragma unroll 1
        for (int k = 0; k < n; ++k) {
            int seg = segs_[k];
            int dir = ct_dir_of(cs, seg);
            #pragma unroll 1
            for (int j = 0; j < w.n_ep; ++j) {
                if (w.ep[j].cs != cs || w.ep[j].seg != seg) continue;
                int steps = ct_remaining(w.ep[j].d, i, dir);
                V3 dr = sub(w.ep[j].pos, p);
                int x = vx(dr), y = vy(dr), z = vz(dr);
                int l1 = (x < 0 ? -x : x) + (y < 0 ? -y : y) + (z < 0 ? -z : z);
                if (l1 > steps || ((steps - l1) & 1)) return false;
            }
        }
        return true;
    }

    // ------------------------------------------------- staple networks ---
    // StapleNetwork::scan_network / scan_staple_topology (:35, :91): a depth-
    // first walk over the staples bound to one another, in the reference's
    // recursion order (frames: chain slot, growth domain, next stack index).
    __device__ __noinline__ void ct_scan(int growth) {
        LdoCtWork<C>& w = *ct;
        w.external = 0;
        w.net_cs = 1ull;
        w.n_gps = 0;
        w.n_iaes = 0;
        w.n_nds = 0;
        int top = 0;
        w.net_cs |= 1ull << scs[growth];
        w.nds[w.n_nds++] = (int16_t)growth;
        w.in_ds[growth] = 1;
        {
            int cs = scs[growth], len = chain_len(cs), gd = didx(growth);
            #pragma unroll 1
            for (int d = 0; d < len; ++d) w.nseg[slot_of(cs, d)] = (int8_t)(d < gd ? 1 : 0);
        }
        w.scan_cs[0] = (int16_t)scs[growth];
        w.scan_g[0] = (int16_t)didx(growth);
        w.scan_k[0] = 0;
        top = 1;
        #pragma unroll 1
        while (top > 0 && !bad()) {
            int f = top - 1;
            int cs = w.scan_cs[f], gd = w.scan_g[f], len = chain_len(cs);
            if (w.scan_k[f] >= len - 1) {
                --top;
                continue;
            }
            int k = w.scan_k[f]++;
            int n3 = len - 1 - gd;
            int di = k < n3 ? gd + 1 + k : gd - 1 - (k - n3);
            int d = slot_of(cs, di);
            if (w.n_nds >= C::DCAP) {
                fail(LDO_RS_CAPACITY);
                return;
            }
            w.nds[w.n_nds++] = (int16_t)d;
            w.in_ds[d] = 1;
            int bd = bnd[d];
            if (bd < 0 || scs[bd] == cs) continue;
            int bcs = scs[bd];
            if (w.net_cs & (1ull << bcs)) {
                bool external = false;
                if (bcs == 0) external = !w.in_scaf[bd];
                if (!external) {   // add_potential_inactive_endpoint (:166)
                    if (w.in_ds[bd]) {
                        w.ia_a[w.n_iaes] = (int16_t)bd;
                        w.ia_b[w.n_iaes] = (int16_t)d;
                    }
                    else {
                        w.ia_a[w.n_iaes] = (int16_t)d;
                        w.ia_b[w.n_iaes] = (int16_t)bd;
                    }
                    w.n_iaes++;
                }
                if (external) w.external = 1;
            }
            else {
                w.gps_a[w.n_gps] = (int16_t)d;
                w.gps_b[w.n_gps] = (int16_t)bd;
                w.n_gps++;
                if (top >= C::KMAX + 2 || w.n_nds >= C::DCAP) {
                    fail(LDO_RS_CAPACITY);
                    return;
                }
                w.net_cs |= 1ull << bcs;
                w.nds[w.n_nds++] = (int16_t)bd;
                w.in_ds[bd] = 1;
                int blen = chain_len(bcs), bg = didx(bd);
                #pragma unroll 1
                for (int q = 0; q < blen; ++q) w.nseg[slot_of(bcs, q)] = (int8_t)(q < bg ? 1 : 0);
                w.scan_cs[top] = (int16_t)bcs;
                w.scan_g[top] = (int16_t)bg;
                w.scan_k[top] = 0;
                ++top;
            }
        }
    }
    // Constraintpoints::find_growthpoints_endpoints (:461) over the scaffold
    // domains seg_dom[off .. off + n) of segment `seg`
    __device__ __noinline__ void ct_find_gp_ep(const int16_t* list, int n, int seg) {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int t = 0; t < n && !bad(); ++t) {
            int d = list[t];
            if (w.n_rd >= C::DCAP) {
                fail(LDO_RS_CAPACITY);
                return;
            }
            w.rd[w.n_rd++] = (int16_t)d;
            w.seg[d] = (int8_t)seg;
            int bd = bnd[d];
            if (bd < 0 || scs[bd] == scs[d] || (w.checked & (1ull << scs[bd]))) continue;
            ct_scan(bd);
            if (bad()) return;
            w.gps_a[w.n_gps] = (int16_t)d;
            w.gps_b[w.n_gps] = (int16_t)bd;
            w.n_gps++;
            if (w.external) {   // add_active_endpoints_on_scaffold (:547)
                #pragma unroll 1
                for (int q = 0; q < w.n_gps; ++q)
                    if (scs[w.gps_a[q]] == 0) ct_add_ep_seg(w.gps_a[q], pos(w.gps_a[q]), seg);
                #pragma unroll 1
                for (int q = 0; q < w.n_iaes; ++q)
                    if (scs[w.ia_b[q]] == 0) ct_add_ep_seg(w.ia_a[q], pos(w.ia_b[q]), seg);
            }
            else {
                #pragma unroll 1
                for (int q = 0; q < w.n_gps; ++q) {   // add_growthpoints (:506)
                    w.gp_to[w.gps_a[q]] = w.gps_b[q];
                    w.stem_of[w.gps_b[q]] = w.gps_a[q];
                }
                #pragma unroll 1
                for (int q = 0; q < w.n_iaes; ++q) w.inact[w.ia_a[q]] = w.ia_b[q];
                w.regrow |= w.net_cs & ~1ull;
                if (w.n_rd + w.n_nds > C::DCAP) {
                    fail(LDO_RS_CAPACITY);
                    return;
                }
                #pragma unroll 1
                for (int q = 0; q < w.n_nds; ++q) {
                    int x = w.nds[q];
                    w.rd[w.n_rd++] = (int16_t)x;
                    if (w.seg[x] < 0) w.seg[x] = w.nseg[x];
                }
            }
            w.checked |= w.net_cs;
            #pragma unroll 1
            for (int q = 0; q < w.n_nds; ++q) w.in_ds[w.nds[q]] = 0;
        }
    }
    // calculate_constraintpoints over the selected segments (:225, :241)
    __device__ __noinline__ void ct_calc_constraintpoints() {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int k = w.seg_off[0]; k < w.seg_off[w.n_segs]; ++k) w.in_scaf[w.seg_dom[k]] = 1;
        #pragma unroll 1
        for (int k = 0; k < w.n_segs && !bad(); ++k) {
            int n = w.seg_off[k + 1] - w.seg_off[k];
            if (n == 0) continue;
            w.sdir[k] = w.seg_dirin[k];
            ct_find_gp_ep(w.seg_dom + w.seg_off[k], n, k);
        }
        #pragma unroll 1
        for (int j = 0; j < w.n_ep; ++j) w.ep0[j] = w.ep[j];
        w.n_ep0 = w.n_ep;
    }

    // ------------------------------------------------ segment selection ---
    // CTRegrowthMCMovetype::select_indices (src/movetypes.cpp:469): min
    // length 2 for the scaffold regrowth movetypes, 1 for the linker ones
    __device__ __noinline__ void ct_select_indices(int max_regrowth, int min_length = 2) {
        LdoCtWork<C>& w = *ct;
        int max_length = ns < max_regrowth ? ns : max_regrowth;
        #pragma unroll 1
        for (int guard = 0; guard < 1000; ++guard) {
            int sel = rng.uniform_int(min_length, max_length);
            int start = rng.uniform_int(0, ns - 1);
            int dir = rng.uniform_int(0, 1) == 0 ? -1 : 1;
            // forward from the start in dir, then backward from before it
            int nf = 0, cur = start;
            #pragma unroll 1
            while (cur >= 0 && nf != sel) {
                ++nf;
                cur = next(cur, dir);
            }
            int nb = 0, back = next(start, -dir);
            #pragma unroll 1
            while (back >= 0 && nf + nb != sel) {
                ++nb;
                back = next(back, -dir);
            }
            if (nf + nb < min_length) continue;
            w.dir = dir;
            int x = start;
            #pragma unroll 1
            for (int t = 0; t < nf; ++t) {
                w.seg_dom[nb + t] = (int16_t)x;
                x = next(x, dir);
            }
            x = next(start, -dir);
            #pragma unroll 1
            for (int t = 0; t < nb; ++t) {
                w.seg_dom[nb - 1 - t] = (int16_t)x;
                x = next(x, -dir);
            }
            w.n_segs = 1;
            w.seg_off[0] = 0;
            w.seg_off[1] = (int16_t)(nf + nb);
            w.seg_dirin[0] = (int8_t)dir;
            if (cur >= 0) ct_add_ep_seg(cur, pos(cur), 0);
            return;
        }
        fail(LDO_RS_ITERCAP);
    }
    // check_for_stemds (src/movetypes.cpp:702)
    __device__ void ct_check_stems(int cur, int& qt) {
        LdoCtWork<C>& w = *ct;
        if (st[cur] != BOUND) return;
        int b = bnd[cur];
        #pragma unroll 1
        for (int sdir = -1; sdir <= 1; sdir += 2) {
            int nb = next(b, sdir);
            if (nb >= 0 && st[nb] == BOUND) {
                int bn = bnd[nb];
                if (scs[bn] == 0) {
                    if (qt >= 4 * C::DCAP) {
                        fail(LDO_RS_CAPACITY);
                        return;
                    }
                    w.stemq[qt++] = (int16_t)bn;
                }
            }
        }
    }
    // fill_seg (src/movetypes.cpp:669): appends to out[*n] (and to out2 if
    // given) a segment that already holds cnt0 domains
    __device__ bool ct_fill_seg(int start, int max_length, int seg_max, int dir, int& n_in, int& qt, int16_t* out,
                                int* n, int16_t* out2, int* n2, int cnt0) {
        LdoCtWork<C>& w = *ct;
        int cur = start;
        ct_check_stems(cur, qt);
        int nd = start;
        int cnt = cnt0;
        #pragma unroll 1
        while (cnt != seg_max && nd >= 0 && !bad()) {
            nd = next(cur, dir);
            if (nd < 0) break;
            int nn = next(nd, dir);
            if (nn >= 0 && w.in_sel[nn]) break;
            out[(*n)++] = (int16_t)nd;
            if (out2) out2[(*n2)++] = (int16_t)nd;
            cnt++;
            w.in_sel[nd] = 1;
            n_in++;
            if (n_in == max_length) return true;
            cur = nd;
            ct_check_stems(cur, qt);
        }
        return false;
    }
    // CTRegrowthMCMovetype::select_noncontig_segs (src/movetypes.cpp:540)
    __device__ __noinline__ void ct_select_noncontig(int max_regrowth, int max_seg_regrowth) {
        LdoCtWork<C>& w = *ct;
        int max_length = rng.uniform_int(2, max_regrowth);
        int seg_max = rng.uniform_int(2, max_seg_regrowth + 1);
        int start = rng.uniform_int(0, ns - 1);
        int dir = rng.uniform_int(0, 1) == 0 ? -1 : 1;
        if (next(start, dir) < 0) dir = -dir;
        int n_in = 1, qh = 0, qt = 0;
        w.in_sel[start] = 1;
        int nd_ = 0;   // domains written to seg_dom
        int np = 0;    // domains written to pair_dom
        w.seg_dom[nd_++] = (int16_t)start;
        w.seg_dirin[0] = (int8_t)dir;
        bool reached = ct_fill_seg(start, max_length, seg_max, dir, n_in, qt, w.seg_dom, &nd_, nullptr, nullptr, 1);
        w.n_segs = 1;
        w.seg_off[1] = (int16_t)nd_;
        w.n_stems = 0;
        #pragma unroll 1
        while (!reached && qh < qt && !bad()) {
            int stemd = w.stemq[qh++];
            if (w.in_sel[stemd]) continue;
            int a = next(stemd, -1), b = next(stemd, 1);
            if ((a >= 0 && w.in_sel[a]) || (b >= 0 && w.in_sel[b])) continue;
            if (w.n_segs + 2 > LDO_CT_MAX_SEGS) {
                fail(LDO_RS_CAPACITY);
                return;
            }
            w.in_sel[stemd] = 1;
            n_in++;
            int si = w.n_stems++;
            w.stems[si] = (int16_t)stemd;
            if (n_in == max_length) {
                reached = true;
                w.seg_dom[nd_++] = (int16_t)stemd;
                w.seg_dirin[w.n_segs] = 1;
                w.seg_off[++w.n_segs] = (int16_t)nd_;
                w.seg_dirin[w.n_segs] = -1;
                w.seg_off[++w.n_segs] = (int16_t)nd_;
                w.pair_off[2 * si + 1] = (int16_t)np;
                w.pair_off[2 * si + 2] = (int16_t)np;
                break;
            }
            int dir1 = rng.uniform_int(0, 1) == 0 ? -1 : 1;
            int dp[2] = {dir1, -dir1};
            // segment a: the stem, then its fill in dir1; segment b: the fill in -dir1
            int ka = w.n_segs, kb = w.n_segs + 1;
            w.seg_dirin[ka] = (int8_t)dp[0];
            w.seg_dirin[kb] = (int8_t)dp[1];
            w.seg_dom[nd_++] = (int16_t)stemd;
            bool done_b = false;
            #pragma unroll 1
            for (int i = 0; i < 2; ++i) {
                int smax = rng.uniform_int(0, max_seg_regrowth);
                if (i == 0) max_length++;
                reached = ct_fill_seg(stemd, max_length, smax, dp[i], n_in, qt, w.seg_dom, &nd_, w.pair_dom, &np, 0);
                w.pair_off[2 * si + 1 + i] = (int16_t)np;
                if (i == 0) w.seg_off[ka + 1] = (int16_t)nd_;
                else {
                    w.seg_off[kb + 1] = (int16_t)nd_;
                    done_b = true;
                }
                if (reached) break;
            }
            if (!done_b) {
                w.seg_off[kb + 1] = (int16_t)nd_;
                w.pair_off[2 * si + 2] = (int16_t)np;
            }
            w.n_segs += 2;
        }
        // endpoints past the ends of the segments, growth points of the stems
        int last = w.seg_dom[w.seg_off[1] - 1];
        int nx = next(last, w.seg_dirin[0]);
        if (nx >= 0) ct_add_ep_seg(nx, pos(nx), 0);
        int seg_i = 1;
        #pragma unroll 1
        for (int i = 0; i < w.n_stems; ++i) {
            int stem = w.stems[i];
            int gp = bnd[stem];
            if (gp < 0) {
                fail(LDO_RS_INVARIANT);
                return;
            }
            w.gp_to[gp] = (int16_t)stem;
            w.stem_of[stem] = (int16_t)gp;
            w.ssegs[stem][0] = (int8_t)seg_i;
            w.ssegs[stem][1] = (int8_t)(seg_i + 1);
            w.nssegs[stem] = 2;
            #pragma unroll 1
            for (int k = 0; k < 2; ++k) {
                int d = w.seg_dirin[seg_i];
                int a0 = w.pair_off[2 * i + k], a1 = w.pair_off[2 * i + k + 1];
                int l = a1 > a0 ? w.pair_dom[a1 - 1] : stem;
                int n2 = next(l, d);
                if (n2 >= 0) ct_add_ep_seg(n2, pos(n2), seg_i);
                seg_i++;
            }
        }
    }

    // ---------------------------------------------------- recoil growth ---
    __device__ __noinline__ void rg_prepare_for_growth() {   // src/rg_movetypes.cpp:245
        LdoCtWork<C>& w = *ct;
        w.di++;
        int d = w.rd[w.di];
        w.d = d;
        w.stemd = w.stem_of[d] >= 0;
        w.dir = ct_get_dir(d);
        w.catt = 0;
        if (w.stemd) {
            w.dmax = 1;
            w.avail = 0;
            w.ref = w.stem_of[d];
        }
        else {
            w.dmax = w.max_c_attempts;
            w.avail = CT_ALL36;
            w.ref = next(d, -w.dir);
            if (w.ref < 0) fail(LDO_RS_INVARIANT);
        }
    }
    __device__ __noinline__ double rg_prepare_for_regrowth() {   // :263
        LdoCtWork<C>& w = *ct;
        w.di--;
        int d = w.rd[w.di];
        w.d = d;
        w.dir = ct_get_dir(d);
        double de = unassign_domain(d);
        ct_restore_endpoints(d);
        w.stemd = w.stem_of[d] >= 0;
        if (w.stemd) {
            w.dmax = 1;
            w.catt = 1;
            w.avail = 0;
            w.ref = w.stem_of[d];
        }
        else {
            w.dmax = w.max_c_attempts;
            w.catt = w.catt_q[w.di];
            w.avail = w.av_q[w.di];
            w.ref = next(d, -w.dir);
            if (w.ref < 0) fail(LDO_RS_INVARIANT);
        }
        return de;
    }
    // select_trial_config (:298): configuration ci = 6 * step + orientation,
    // the k-th of the untried ones (ascending, as the reference's list)
    __device__ __noinline__ void rg_select_trial(V3& p, int& o) {
        LdoCtWork<C>& w = *ct;
        if (w.stemd) {
            p = pos(w.ref);
            o = ore[w.ref] ^ 1;
            return;
        }
        unsigned long long av = w.avail;
        int n = __popcll(av);
        if (n == 0) {
            fail(LDO_RS_INVARIANT);
            p = pos(w.ref);
            o = 0;
            return;
        }
        int k = rng.uniform_int(0, n - 1);
        // the k-th set bit (0-based) of the mask, by halving (k < popcount)
        int ci = 0;
        int c = __popc((unsigned)av);
        if (k >= c) {
            k -= c;
            av >>= 32;
            ci = 32;
        }
        unsigned v = (unsigned)av;
        #pragma unroll
        for (int half = 16; half >= 1; half >>= 1) {
            c = __popc(v & ((1u << half) - 1u));
            if (k >= c) {
                k -= c;
                v >>= half;
                ci += half;
            }
        }
        w.avail &= ~(1ull << ci);
        p = add(pos(w.ref), unit(ci / 6));
        o = ci % 6;
    }
    // calc_p_config_open (:316)
    __device__ __noinline__ double rg_p_open(V3 p, int o) {
        LdoCtWork<C>& w = *ct;
        int d = w.d;
        Delta dc = probe_domain(d, p, o);
        if (bad()) return 0;
        if (hdr.violated) {
            hdr.violated = 0;
            return 0;
        }
        if (!ct_walks_ok(d, p)) return 0;
        if (occupancy(p) == UNBOUND) {
            int od = unbound_at(p);
            bool same = scs[od] == scs[d];
            bool endpoint = ct_endpoint_reached(d, p);
            if (!(same || endpoint || w.stemd)) return 0;
        }
        return fmin(1.0, dexp(-dc.e));
    }
    // calc_p_config_open of the configurations of one trial loop, evaluated
    // per neighbour site: the trials of a loop all see the same state (an
    // open trial that grows feelers restores it), and of the six
    // orientations at a site only one can bind.  An empty site is open for
    // every orientation when its walks remain (no potential is evaluated:
    // e^-0); an occupied one is closed; an unbound one is open at most for the
    // orientation opposite to its domain's, and only if the domain is on the
    // same chain or at an active endpoint (the FourBody probe runs only
    // then).  The same values as probing every configuration, with at most
    // six walk checks and six probes per loop.
    struct RgSites {
        int8_t kind[6];        // -1 unknown, 0 closed, 1 open (p = 1), 2 open for orientation opp only
        int8_t opp[6];
        double pv[6];
    };
    __device__ static void rg_sites_reset(RgSites& c) {
        #pragma unroll
        for (int k = 0; k < 6; ++k) c.kind[k] = -1;
    }
    __device__ __noinline__ double rg_p_open_site(V3 p, int o, int k, RgSites& c) {
        LdoCtWork<C>& w = *ct;
        if (w.stemd) return rg_p_open(p, o);
        if (c.kind[k] < 0) {
            int d = w.d;
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND || !ct_walks_ok(d, p)) {
                c.kind[k] = 0;
            }
            else if (occ == UNBOUND) {
                int od = unbound_at(p);
                bool same = scs[od] == scs[d];
                if (!(same || ct_endpoint_reached(d, p))) {
                    c.kind[k] = 0;
                }
                else {
                    int op = ore[od] ^ 1;
                    c.kind[k] = 2;
                    c.opp[k] = (int8_t)op;
                    Delta dc = probe_domain(d, p, op);
                    if (hdr.violated) {
                        hdr.violated = 0;
                        c.pv[k] = 0;
                    }
                    else {
                        c.pv[k] = fmin(1.0, dexp(-dc.e));
                    }
                }
            }
            else {
                c.kind[k] = 1;
            }
        }
        if (c.kind[k] == 0) return 0;
        if (c.kind[k] == 1) return 1.0;
        return o == c.opp[k] ? c.pv[k] : 0;
    }
    __device__ __noinline__ void rg_select_trial_site(V3& p, int& o, int& k) {
        LdoCtWork<C>& w = *ct;
        if (w.stemd) {
            rg_select_trial(p, o);
            k = 0;
            return;
        }
        rg_select_trial(p, o);
        k = unit_index(sub(p, pos(w.ref)));
    }
    __device__ bool rg_test_open(double p) {   // test_config_open (:346)
        p = fmin(1.0, p);
        if (p == 1) return true;
        return p > rng.uniform_real();
    }
    __device__ __noinline__ double rg_set_config(int d, V3 p, int o) {   // set_config (:233)
        double de = set_checked(d, p, o);
        ct_update_endpoints(ct->d);
        ct_push_erased();
        return de;
    }
    // recoil_regrow (:177)
    __device__ __noinline__ double rg_recoil_regrow() {
        LdoCtWork<C>& w = *ct;
        double de = 0;
        w.di = 0;
        w.d = w.rd[0];
        w.dir = ct_get_dir(w.d);
        #pragma unroll 1
        for (int k = 0; k < w.n_rd; ++k) {
            w.catt_q[k] = 0;
            w.av_q[k] = 0;
            w.c_open[k] = 0;
        }
        w.c_open[0] = 1;
        rg_prepare_for_growth();
        int recoils = 0;
        #pragma unroll 1
        for (int guard = 0; guard < (1 << 22); ++guard) {
            if (bad()) return de;
            V3 p = 0;
            int o = 0;
            double pc = 0;
            bool open = false;
            RgSites sc;
            rg_sites_reset(sc);
            #pragma unroll 1
            while (!open && w.catt != w.dmax && !bad()) {
                w.catt++;
                int k;
                rg_select_trial_site(p, o, k);
                pc = rg_p_open_site(p, o, k, sc);
                open = rg_test_open(pc);
            }
            if (open) {
                if (recoils != 0) recoils--;
                de += rg_set_config(w.d, p, o);
                w.catt_q[w.di] = (uint8_t)w.catt;
                w.av_q[w.di] = w.avail;
                w.c_open[w.di] = pc;
                if (w.di == w.n_rd - 1) return de;
                rg_prepare_for_growth();
            }
            else {
                if (recoils == w.max_recoils || w.di == 1) {
                    rejected = true;
                    return de;
                }
                recoils++;
                de += rg_prepare_for_regrowth();
            }
        }
        fail(LDO_RS_ITERCAP);
        return de;
    }
    // test_config_avail (:418)
    __device__ __noinline__ bool rg_test_avail() {
        LdoCtWork<C>& w = *ct;
        int feels = 0;
        if (feels == w.max_recoils || w.di == w.n_rd - 1) return true;
        rg_prepare_for_growth();
        bool avail = false;
        #pragma unroll 1
        for (int guard = 0; guard < (1 << 22); ++guard) {
            if (bad()) return false;
            V3 p = 0;
            int o = 0;
            bool open = false;
            RgSites sc;
            rg_sites_reset(sc);
            #pragma unroll 1
            while (!open && w.catt != w.dmax && !bad()) {
                w.catt++;
                int k;
                rg_select_trial_site(p, o, k);
                double pc = rg_p_open_site(p, o, k, sc);
                open = rg_test_open(pc);
            }
            if (open) {
                feels++;
                if (feels == w.max_recoils || w.di == w.n_rd - 1) {
                    feels--;
                    avail = true;
                    break;
                }
                rg_set_config(w.d, p, o);
                w.catt_q[w.di] = (uint8_t)w.catt;
                w.av_q[w.di] = w.avail;
                rg_prepare_for_growth();
            }
            else {
                if (feels == 0) {
                    avail = false;
                    break;
                }
                feels--;
                rg_prepare_for_regrowth();
            }
            if (guard + 1 == (1 << 22)) fail(LDO_RS_ITERCAP);
        }
        #pragma unroll 1
        while (feels != 0 && !bad()) {
            w.di--;
            feels--;
            w.d = w.rd[w.di];
            unassign_domain(w.d);
            ct_restore_endpoints(w.d);
        }
        w.di--;
        w.d = w.rd[w.di];
        return avail;
    }
    // calc_weights (:363) of the configuration src_p / src_o
    __device__ __noinline__ void rg_calc_weights(const long long* src_p, const uint8_t* src_o) {
        LdoCtWork<C>& w = *ct;
        w.di = 0;
        w.d = w.rd[0];
        #pragma unroll 1
        while (w.di != w.n_rd - 1 && !bad()) {
            w.di++;
            int d = w.rd[w.di];
            w.d = d;
            w.stemd = w.stem_of[d] >= 0;
            w.dir = ct_get_dir(d);
            int avail_cs = 1;
            if (!w.stemd) {
                w.ref = next(d, -w.dir);
                int catt = w.catt_wq[w.di];
                w.avail = w.av_wq[w.di];
                RgSites sc;
                rg_sites_reset(sc);
                #pragma unroll 1
                while (catt != w.max_c_attempts && !bad()) {
                    catt++;
                    V3 p;
                    int o, k;
                    rg_select_trial_site(p, o, k);
                    double pc = rg_p_open_site(p, o, k, sc);
                    if (rg_test_open(pc)) {
                        set_checked(d, p, o);
                        ct_update_endpoints(d);
                        ct_push_erased();
                        int dir_s = w.dir, ref_s = w.ref, stem_s = w.stemd;
                        unsigned long long av_s = w.avail;
                        avail_cs += rg_test_avail();
                        w.avail = av_s;
                        w.stemd = stem_s;
                        w.ref = ref_s;
                        w.dir = dir_s;
                        unassign_domain(d);
                        ct_restore_endpoints(d);
                    }
                }
            }
            w.weight *= avail_cs / w.c_open[w.di - 1];
            set_checked(d, src_p[d], src_o[d]);
            ct_update_endpoints(d);
            ct_push_erased();
        }
        w.weight /= w.c_open[w.di];
    }
    // calc_old_c_opens (:481)
    __device__ __noinline__ void rg_calc_old_c_opens() {
        LdoCtWork<C>& w = *ct;
        w.di = 0;
        w.c_open[0] = 1;
        #pragma unroll 1
        while (w.di != w.n_rd - 1 && !bad()) {
            w.di++;
            int d = w.rd[w.di];
            w.d = d;
            w.catt_q[w.di] = 1;
            V3 p = w.p_old[d];
            int o = w.o_old[d];
            w.stemd = w.stem_of[d] >= 0;
            w.c_open[w.di] = rg_p_open(p, o);
            rg_set_config(d, p, o);
            if (w.stemd) {
                w.av_q[w.di] = 0;
            }
            else {
                w.dir = ct_get_dir(d);
                int ref = next(d, -w.dir);
                w.ref = ref;
                int k = ref >= 0 ? unit_index(sub(p, w.p_old[ref])) : -1;
                if (k < 0) {
                    fail(LDO_RS_INVARIANT);   // m_config_to_i.at: not a neighbour step
                    return;
                }
                w.av_q[w.di] = CT_ALL36 & ~(1ull << (6 * k + o));
            }
        }
    }
    // The first phase of both recoil-growth movetypes: segments, constraint
    // points, the regrowth stack, and unassign_and_save_domains (:81).
    __device__ __noinline__ int rg_begin(int kind) {
        LdoCtWork<C>& w = *ct;
        ct_clear();
        w.kind = kind;
        w.delta_e = 0;
        w.weight = 1;
        w.weight_new = 1;
        const int* mo = sys->move_opt[cur_mv];
        w.max_recoils = mo[LDO_MO_MAX_RECOILS];
        w.max_c_attempts = mo[LDO_MO_MAX_C_ATTEMPTS];
        if (kind == LDO_MV_CTRG) {   // CTRGScaffoldRegrowthMCMovetype (:629)
            ct_select_indices(mo[LDO_MO_MAX_REGROWTH]);
            if (bad()) return finish_move(false, 0);
            ct_calc_constraintpoints();
            int nsel = w.seg_off[1];
            bool whole = cyclic && nsel == ns;
            if (!whole) ct_remove_ep(w.seg_dom[0]);
            bool whole_ds = cyclic && w.n_rd == ns;
            w.remove_first[0] = !whole_ds;
            w.remove_first[1] = !cyclic && w.n_rd == ns;   // the reference's condition at :673
            w.remove_first[2] = !whole_ds;
        }
        else {   // CTRGJumpScaffoldRegrowthMCMovetype (:792)
            ct_select_noncontig(mo[LDO_MO_MAX_REGROWTH], mo[LDO_MO_MAX_SEG_REGROWTH]);
            if (bad()) return finish_move(false, 0);
            ct_calc_constraintpoints();
            ct_remove_ep(w.seg_dom[0]);
            #pragma unroll 1
            for (int i = 0; i < w.n_stems; ++i) {
                int stem = w.stems[i];
                w.gp_to[bnd[stem]] = (int16_t)stem;
                w.stem_of[stem] = (int16_t)bnd[stem];
            }
            w.remove_first[0] = w.remove_first[1] = w.remove_first[2] = 1;
        }
        if (bad()) return finish_move(false, 0);
        // a single domain to regrow (a two-domain cyclic scaffold) leaves the
        // reference reading past its regrowth stack; the move is rejected
        if (w.n_rd < 2) return finish_move(false, 0);
        #pragma unroll 1
        for (int k = 0; k < w.n_rd; ++k) {
            int d = w.rd[k];
            w.p_old[d] = pos(d);
            w.o_old[d] = ore[d];
        }
        #pragma unroll 1
        for (int k = 1; k < w.n_rd; ++k) w.delta_e += unassign_domain(w.rd[k]);
        w.n_eq = 0;
        phase = PH_RG2;
        return CMD_SNAP(1) | CMD_MORE;
    }
    __device__ __noinline__ int rg_grow() {
        LdoCtWork<C>& w = *ct;
        w.delta_e += rg_recoil_regrow();
        if (rejected || bad()) return finish_move(false, 0);
        // add_external_bias (:76)
        update_move_params();
        w.delta_e += calc_move();
        // setup_for_calc_new_weights (:137); the new configuration is kept
        // for the weight pass and as snapshot 2
        #pragma unroll 1
        for (int k = 0; k < w.n_rd; ++k) {
            int d = w.rd[k];
            w.p_new[d] = pos(d);
            w.o_new[d] = ore[d];
            w.catt_wq[k] = w.catt_q[k];
            w.av_wq[k] = w.av_q[k];
        }
        w.n_eq = 0;
        phase = PH_RG3;
        return CMD_SNAP(2) | CMD_REST(1) | CMD_MORE;
    }
    __device__ __noinline__ int rg_weigh_new() {
        LdoCtWork<C>& w = *ct;
        ct_reset_endpoints();
        if (w.remove_first[0]) ct_remove_ep(w.rd[0]);
        rg_calc_weights(w.p_new, w.o_new);
        if (bad()) return finish_move(false, 0);
        phase = PH_RG4;
        return CMD_REST(1) | CMD_MORE;   // unassign_domains (:116)
    }
    __device__ __noinline__ int rg_old_opens() {
        LdoCtWork<C>& w = *ct;
        w.n_eq = 0;
        ct_reset_endpoints();
        if (w.remove_first[1]) ct_remove_ep(w.rd[0]);
        rg_calc_old_c_opens();
        if (bad()) return finish_move(false, 0);
        // setup_for_calc_old_weights (:146)
        w.weight_new = w.weight;
        w.weight = 1;
        #pragma unroll 1
        for (int k = 0; k < w.n_rd; ++k) {
            w.catt_wq[k] = w.catt_q[k];
            w.av_wq[k] = w.av_q[k];
        }
        phase = PH_RG5;
        return CMD_REST(1) | CMD_MORE;   // unassign_and_save_domains
    }
    __device__ __noinline__ int rg_weigh_old() {
        LdoCtWork<C>& w = *ct;
        w.n_eq = 0;
        ct_reset_endpoints();
        if (w.remove_first[2]) ct_remove_ep(w.rd[0]);
        rg_calc_weights(w.p_old, w.o_old);
        if (bad()) return finish_move(false, 0);
        // test_rg_acceptance (:515): accepted, the new configuration
        double ratio = w.weight_new / w.weight * dexp(-w.delta_e);
        bool acc = test_acceptance(ratio);
        return finish_move(acc, acc ? 2 : 0);
    }

    // ------------------------------------------- configurational bias ---
    // RegrowthMCMovetype::set_growth_point (src/movetypes.cpp:322) without
    // the reversal list
    __device__ double ct_set_growth_point(int gnew, int gold) {
        double de = set_domain_config(gnew, pos(gold), ore[gold] ^ 1);
        if (hdr.violated) rejected = true;
        return de;
    }
    // CBMCMovetype::select_and_set_config (:104) with calc_biases (:58) and
    // CTCBRegrowthMCMovetype::calc_bias (:480)
    __device__ __noinline__ void ctcb_select_and_set(int dom, int prev) {
        LdoCtWork<C>& w = *ct;
        V3 p_prev = pos(prev);
        int nc = 0;
        // calc_biases (:58) and the zero weights of calc_bias (:480): a site
        // whose weight calc_bias sets to zero is not probed (its weight
        // would be zero either way; zero terms leave the sum and the
        // selection unchanged)
        #pragma unroll 1
        for (int v = 0; v < 6; ++v) {
            V3 p = add(p_prev, unit(v));
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND) continue;
            bool zero = !ct_walks_ok(dom, p);
            if (occ == UNBOUND) {
                int ud = unbound_at(p);
                int o = ore[ud] ^ 1;
                if (!zero && !(scs[ud] == scs[dom] || ct_endpoint_reached(dom, p))) zero = true;
                if (zero) continue;
                Delta dc = probe_domain(dom, p, o);
                if (bad()) return;
                if (!hdr.violated) {
                    cb_pos[nc] = p;
                    cb_ore[nc] = o;
                    cb_de[nc] = dc.e;
                    cb_stk[nc] = dc.stacked;
                    double b = 1;
                    b *= dexp(-dc.e);
                    cb_bf[nc] = b;
                    nc++;
                }
                else {
                    hdr.violated = 0;
                }
            }
            else {
                if (zero) continue;
                cb_pos[nc] = p;
                cb_ore[nc] = -1;
                cb_bf[nc] = 6.0;
                nc++;
            }
        }
        double sum = 0;
        #pragma unroll 1
        for (int n = 0; n < nc; ++n) sum += cb_bf[n];
        // a dead end rejects; a rejection from before (the old
        // configuration's staple growth) still multiplies in this weight
        if (sum == 0) rejected = true;
        else w_bias *= sum;
        if (rejected) return;
        if (!regrow_old) {
            V3 p = mk(0, 0, 0);
            int o = -1, chosen = -1;
            double cum = 0;
            double r = rng.uniform_real();
            #pragma unroll 1
            for (int n = 0; n < nc; ++n) {
                cum += cb_bf[n] / sum;
                if (r < cum) {
                    p = cb_pos[n];
                    o = cb_ore[n];
                    chosen = n;
                    break;
                }
            }
            if (o < 0) {
                o = rng.uniform_int(0, 5);
                set_checked(dom, p, o);
            }
            else {
                set_checked_probed(dom, p, o, cb_de[chosen], cb_stk[chosen]);
            }
        }
        else {
            V3 p = w.p_old[dom];
            int o = w.o_old[dom];
            int c = 0;
            #pragma unroll 1
            while (c < nc && !(cb_ore[c] == o && eq(cb_pos[c], p))) ++c;
            if (c < nc) set_checked_probed(dom, p, o, cb_de[c], cb_stk[c]);
            else set_checked(dom, p, o);
        }
    }
    __device__ bool ct_push_frame(int kind, int a, int b, int dir, int n) {
        LdoCtWork<C>& w = *ct;
        if (w.n_fr >= LdoCtWork<C>::FR) {
            fail(LDO_RS_CAPACITY);
            return false;
        }
        int f = w.n_fr++;
        w.fr_kind[f] = (int8_t)kind;
        w.fr_a[f] = (int16_t)a;
        w.fr_b[f] = (int16_t)b;
        w.fr_dir[f] = (int8_t)dir;
        w.fr_n[f] = (int16_t)n;
        w.fr_i[f] = (int16_t)(kind == 2 ? 0 : 1);
        return true;
    }
    __device__ int ct_frame_elem(int f, int i) const {
        const LdoCtWork<C>& w = *ct;
        if (w.fr_kind[f] == 1) return slot_of(w.fr_a[f], w.fr_b[f] + w.fr_dir[f] * i);
        return (w.fr_a[f] == 0 ? w.seg_dom : w.fr_a[f] == 1 ? w.list : w.lk)[w.fr_b[f] + i];
    }
    // CTCBRegrowthMCMovetype::grow_staple_and_update_endpoints (:533) up to
    // the growth of the staple, which the frame loop does
    __device__ __noinline__ void ct_start_staple(int gold) {
        LdoCtWork<C>& w = *ct;
        int gnew = w.gp_to[gold];
        if (gnew < 0) {
            fail(LDO_RS_INVARIANT);
            return;
        }
        if (scs[gnew] == 0) return;   // the reference's guard against scaffold segments
        double de;
        if (regrow_old) de = set_checked(gnew, pos(gold), w.o_old[gnew]);   // set_old_growth_point (:168)
        else de = ct_set_growth_point(gnew, gold);
        w_bias *= dexp(-de);
        if (rejected || bad()) return;
        ct_update_endpoints(gnew);
        ct_push_frame(2, gnew, 0, 0, 0);
    }
    // CTCBRegrowthMCMovetype::grow_chain (:463) and RegrowthMCMovetype::
    // grow_staple (src/movetypes.cpp:343), their recursion as a frame stack:
    // kind 0 a list of slots, 1 a staple's domains from its growth domain in
    // one direction, 2 a staple whose 3' then 5' runs are still to grow.
    __device__ __noinline__ void ct_grow_frames() {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        while (w.n_fr > 0) {
            if (bad()) {
                w.n_fr = 0;
                return;
            }
            int f = w.n_fr - 1;
            if (w.fr_kind[f] != 2) {
                if (w.fr_i[f] >= w.fr_n[f]) {
                    w.n_fr--;
                    continue;
                }
                int i = w.fr_i[f]++;
                int d = ct_frame_elem(f, i), prev = ct_frame_elem(f, i - 1);
                w.dir = ct_get_dir(d);
                ctcb_select_and_set(d, prev);
                if (rejected || bad()) {
                    w.n_fr = 0;
                    return;
                }
                ct_update_endpoints(d);
                if (w.gp_to[d] >= 0) {
                    ct_start_staple(d);
                    if (rejected || bad()) {
                        w.n_fr = 0;
                        return;
                    }
                }
            }
            else {
                int g = w.fr_a[f];
                int cs = scs[g], di = didx(g), len = chain_len(cs);
                int stage = w.fr_i[f]++;
                if (stage == 0) {
                    if (len - di > 1) ct_push_frame(1, cs, di, 1, len - di);
                }
                else if (stage == 1) {
                    if (di + 1 > 1) ct_push_frame(1, cs, di, -1, di + 1);
                }
                else {
                    w.n_fr--;
                }
            }
        }
    }
    __device__ void ct_grow_list(int base, int off, int n) {   // grow_chain over a list of slots
        if (ct_push_frame(0, base, off, 0, n)) ct_grow_frames();
    }
    __device__ void ct_grow_from(int gold) {   // grow_staple_and_update_endpoints
        ct_start_staple(gold);
        if (!rejected && !bad()) ct_grow_frames();
    }
    // CTCBJumpScaffoldRegrowthMCMovetype::set_first_seg_domain (:968)
    __device__ __noinline__ void ctcb_first_seg_domain(int dnew) {
        LdoCtWork<C>& w = *ct;
        int dold = w.stem_of[dnew];
        if (dold < 0) {
            fail(LDO_RS_INVARIANT);
            return;
        }
        if (!ct_walks_ok(dnew, pos(dold))) {
            rejected = true;
            return;
        }
        w.dir = ct_get_dir(dnew);
        double de = ct_set_growth_point(dnew, dold);
        w_bias *= dexp(-de);
    }
    // The growth of one configuration (new or old) of a CTCB move.
    __device__ __noinline__ bool ctcb_grow() {
        LdoCtWork<C>& w = *ct;
        int first = w.seg_dom[0];
        if (w.kind == LDO_MV_CTCB) {   // CTCBScaffoldRegrowthMCMovetype (:691)
            if (w.gp_to[first] >= 0) {
                ct_grow_from(first);
                if (rejected && !regrow_old) return false;
            }
            ct_grow_list(0, 0, w.seg_off[1]);
            return !rejected;
        }
        // CTCBJumpScaffoldRegrowthMCMovetype (:880-906)
        if (w.gp_to[first] >= 0) {
            ct_grow_from(first);
            if (rejected) return false;
        }
        ct_grow_list(0, 0, w.seg_off[1]);
        if (rejected) return false;
        #pragma unroll 1
        for (int i = 0; i < w.n_stems && !bad(); ++i) {
            int stem = w.stems[i];
            ctcb_first_seg_domain(stem);
            if (rejected) return false;
            #pragma unroll 1
            for (int k = 0; k < 2; ++k) {
                int a0 = w.pair_off[2 * i + k], a1 = w.pair_off[2 * i + k + 1];
                w.list[0] = (int16_t)stem;
                #pragma unroll 1
                for (int q = a0; q < a1; ++q) w.list[1 + q - a0] = w.pair_dom[q];
                ct_grow_list(1, 0, 1 + a1 - a0);
                if (rejected) return false;
            }
        }
        return true;
    }
    __device__ __noinline__ int ctcb_begin(int kind) {
        LdoCtWork<C>& w = *ct;
        ct_clear();
        w.kind = kind;
        const int* mo = sys->move_opt[cur_mv];
        if (kind == LDO_MV_CTCB) {
            ct_select_indices(mo[LDO_MO_MAX_REGROWTH]);
            if (bad()) return finish_move(false, 0);
            ct_calc_constraintpoints();
            bool whole = cyclic && w.seg_off[1] == ns;
            w.remove_first[0] = !whole;
            if (!whole) ct_remove_ep(w.seg_dom[0]);
            if (bad()) return finish_move(false, 0);
            // unassign the scaffold domains after the first, then the
            // staples to regrow in the order of their chain indices
            int n = w.seg_off[1];
            #pragma unroll 1
            for (int k = 1; k < n; ++k) {
                int d = w.seg_dom[k];
                w.p_old[d] = pos(d);
                w.o_old[d] = ore[d];
                unassign_domain(d);
            }
            unsigned long long left = w.regrow;
            #pragma unroll 1
            while (left) {
                int best = -1;
                #pragma unroll 1
                for (unsigned long long m = left; m; m &= m - 1ull) {
                    int cs = __ffsll((long long)m) - 1;
                    if (best < 0 || chain_c[cs] < chain_c[best]) best = cs;
                }
                left &= ~(1ull << best);
                int len = chain_len(best);
                #pragma unroll 1
                for (int q = 0; q < len; ++q) {
                    int d = slot_of(best, q);
                    w.p_old[d] = pos(d);
                    w.o_old[d] = ore[d];
                    unassign_domain(d);
                }
            }
        }
        else {
            ct_select_noncontig(mo[LDO_MO_MAX_REGROWTH], mo[LDO_MO_MAX_SEG_REGROWTH]);
            if (bad()) return finish_move(false, 0);
            ct_calc_constraintpoints();
            ct_remove_ep(w.seg_dom[0]);
            w.remove_first[0] = 1;
            if (bad()) return finish_move(false, 0);
            #pragma unroll 1
            for (int k = 1; k < w.n_rd; ++k) {
                int d = w.rd[k];
                w.p_old[d] = pos(d);
                w.o_old[d] = ore[d];
                unassign_domain(d);
            }
        }
        phase = PH_CT2;
        return CMD_SNAP(1) | CMD_MORE;
    }
    __device__ __noinline__ int ctcb_new() {
        LdoCtWork<C>& w = *ct;
        regrow_old = false;
        if (!ctcb_grow() || bad()) return finish_move(false, 0);
        update_move_params();   // add_external_bias (:52)
        w_bias *= dexp(-calc_move());
        // setup_for_regrow_old (:215)
        regrow_old = true;
        w_new_bias = w_bias;
        new_modifier = modifier;
        w_bias = 1;
        (void)w;
        phase = PH_CT3;
        return CMD_SNAP(2) | CMD_REST(1) | CMD_MORE;
    }
    __device__ __noinline__ int ctcb_old() {
        LdoCtWork<C>& w = *ct;
        ct_reset_endpoints();
        if (w.remove_first[0]) ct_remove_ep(w.seg_dom[0]);
        bool ok = ctcb_grow();
        if (bad()) return finish_move(false, 0);
        // the jump movetype gives up here with the new configuration as the
        // one to revert to (its m_prev_pos, src/cb_movetypes.cpp:927)
        if (!ok && w.kind == LDO_MV_CTCB_JUMP) return finish_move(false, 0, 2);
        modifier = 1;
        double ratio = w_new_bias / w_bias;   // test_cb_acceptance (:182)
        bool acc = test_acceptance(ratio);
        return finish_move(acc, acc ? 2 : 0);
    }

    // ================================= scaffold transforms with linkers ===
    // LinkerRegrowthMCMovetype and its variants (src/transform_movetypes.cpp):
    // a central scaffold segment, with the staples bound only within it, is
    // unassigned and placed again by a rigid lattice transformation (turns
    // about a basis axis through one of its domains, then a translation),
    // chosen among num_transforms trials by their Boltzmann factors (modified
    // Rosenbluth); the scaffold linkers on both sides and the staples bound
    // to them regrow with configurational bias (CTCB) or recoil growth
    // (CTRG).  The reverse move's weight comes from num_transforms - 1 trial
    // transformations of the new configuration plus the old one.  Snapshots:
    // CTCB 1 = everything unassigned, 2 = the new configuration; CTRG 2.

    // VectorThree::rotate(axis, turns) (src/utility.cpp:102) about basis axis
    // 0 x, 1 y, 2 z, turns > 0: an even count is a half turn (rotate_half,
    // :68), an odd one a quarter turn whose sense alternates every two turns
    __device__ static V3 lk_rot(V3 v, int axis, int turns) {
        int x = vx(v), y = vy(v), z = vz(v), t;
        if (turns % 2 == 0) {
            if (axis == 0) { y = -y; z = -z; }
            else if (axis == 1) { x = -x; z = -z; }
            else { x = -x; y = -y; }
        }
        else {
            int dir = ((turns - 1) / 2 % 2 == 0) ? 1 : -1;
            if (axis == 0) { t = y; y = -dir * z; z = dir * t; }
            else if (axis == 1) { t = x; x = -dir * z; z = dir * t; }
            else { t = x; x = -dir * y; y = dir * t; }
        }
        return mk(x, y, z);
    }
    // pos.rotate(center, axis, turns) + disp; no rotation for zero turns
    __device__ static V3 lk_place(V3 p, V3 center, int axis, int turns, V3 disp) {
        if (turns != 0) p = add(lk_rot(sub(p, center), axis, turns), center);
        return add(p, disp);
    }
    __device__ static int lk_orient(int o, int axis, int turns) {
        return turns == 0 ? o : unit_index(lk_rot(unit_c(o), axis, turns));
    }
    __device__ bool lk_in(const int16_t* list, int n, int d) const {
        #pragma unroll 1
        for (int k = 0; k < n; ++k)
            if (list[k] == d) return true;
        return false;
    }
    // LinkerRegrowthMCMovetype::domains_bound_externally (:238) with
    // scan_for_external_scaffold_domain (:262): from each central domain
    // bound to a staple, the staples reached through their other domains,
    // depth first in chain order; true at the first one bound to a scaffold
    // domain outside the central segment
    __device__ __noinline__ bool lk_bound_externally() {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int c = 0; c < w.n_cen; ++c) {
            int d = w.cen[c];
            if (st[d] == UNBOUND) continue;
            int bd = bnd[d];
            if (bd < 0) {
                fail(LDO_RS_INVARIANT);
                return false;
            }
            if (scs[bd] == 0) continue;
            unsigned long long part = (1ull << scs[d]) | (1ull << scs[bd]);
            int top = 0;
            w.fs_cs[top] = (int16_t)scs[bd];
            w.fs_d[top] = (int16_t)bd;
            w.fs_k[top] = 0;
            ++top;
            #pragma unroll 1
            while (top > 0) {
                int f = top - 1;
                int cs = w.fs_cs[f];
                if (w.fs_k[f] >= chain_len(cs)) {
                    --top;
                    continue;
                }
                int cur = slot_of(cs, w.fs_k[f]++);
                if (cur == w.fs_d[f]) continue;
                int b = bnd[cur];
                if (b < 0 || scs[b] == cs) continue;
                if (scs[b] == 0) {
                    if (!lk_in(w.cen, w.n_cen, b)) return true;
                    continue;
                }
                if (part & (1ull << scs[b])) continue;
                if (top >= C::KMAX + 2) {
                    fail(LDO_RS_CAPACITY);
                    return false;
                }
                part |= 1ull << scs[b];
                w.fs_cs[top] = (int16_t)scs[b];
                w.fs_d[top] = (int16_t)b;
                w.fs_k[top] = 0;
                ++top;
            }
        }
        return false;
    }
    // MCMovetype::find_staples (src/movetypes.cpp:179) with
    // scan_for_scaffold_domain (:191): the staples reached from the central
    // segment, depth first in chain order, each scan ending (at every level)
    // at the first domain bound to the scaffold; then the central domains:
    // the segment, then those staples' domains in chain-index order
    __device__ __noinline__ void lk_central_domains() {
        LdoCtWork<C>& w = *ct;
        unsigned long long part = 0;
        #pragma unroll 1
        for (int c = 0; c < w.n_cen; ++c) {
            int bd = bnd[w.cen[c]];
            if (bd < 0 || scs[bd] == 0) continue;
            part |= 1ull << scs[bd];
            int top = 0;
            w.fs_cs[top] = (int16_t)scs[bd];
            w.fs_d[top] = (int16_t)bd;
            w.fs_k[top] = 0;
            ++top;
            #pragma unroll 1
            while (top > 0) {
                int f = top - 1;
                int cs = w.fs_cs[f];
                if (w.fs_k[f] >= chain_len(cs)) {
                    --top;
                    continue;
                }
                int cur = slot_of(cs, w.fs_k[f]++);
                if (cur == w.fs_d[f]) continue;
                int b = bnd[cur];
                if (b < 0 || scs[b] == cs) continue;
                if (scs[b] == 0) {   // bound to the scaffold: true returns through every level
                    top = 0;
                    continue;
                }
                if (part & (1ull << scs[b])) continue;
                if (top >= C::KMAX + 2) {
                    fail(LDO_RS_CAPACITY);
                    return;
                }
                part |= 1ull << scs[b];
                w.fs_cs[top] = (int16_t)scs[b];
                w.fs_d[top] = (int16_t)b;
                w.fs_k[top] = 0;
                ++top;
            }
        }
        w.n_cdom = 0;
        #pragma unroll 1
        for (int c = 0; c < w.n_cen; ++c) w.cdom[w.n_cdom++] = w.cen[c];
        #pragma unroll 1
        while (part) {
            int best = -1;
            #pragma unroll 1
            for (unsigned long long m = part; m; m &= m - 1ull) {
                int cs = __ffsll((long long)m) - 1;
                if (best < 0 || chain_c[cs] < chain_c[best]) best = cs;
            }
            part &= ~(1ull << best);
            int len = chain_len(best);
            if (w.n_cdom + len > C::DCAP) {
                fail(LDO_RS_CAPACITY);
                return;
            }
            #pragma unroll 1
            for (int q = 0; q < len; ++q) w.cdom[w.n_cdom++] = (int16_t)slot_of(best, q);
        }
    }
    // LinkerRegrowthMCMovetype::select_and_setup_segments (:156) up to the
    // fixed-end biases: central segment by select_indices with minimum
    // length 1, linkers from its ends outwards; false: the move is rejected
    __device__ __noinline__ bool lk_select() {
        LdoCtWork<C>& w = *ct;
        const int* mo = sys->move_opt[cur_mv];
        int maxl = mo[LDO_MO_MAX_LINKER];
        bool ext = true;
        #pragma unroll 1
        for (int att = 0; ext && att != 10; ++att) {
            ct_select_indices(mo[LDO_MO_MAX_REGROWTH], 1);
            if (bad()) return false;
            int n = w.seg_off[1];
            #pragma unroll 1
            for (int k = 0; k < n; ++k) w.cen[k] = w.seg_dom[k];
            w.n_cen = n;
            int dir = w.dir;
            int len1 = rng.uniform_int(2, maxl + 1);
            int stop = next(w.cen[n - 1], 2 * dir);
            int x = w.cen[0];
            w.n_lk1 = 0;
            #pragma unroll 1
            while (w.n_lk1 != len1 && x >= 0 && x != stop) {
                w.lk[w.n_lk1++] = (int16_t)x;
                x = next(x, -dir);
            }
            if (cyclic && w.n_lk1 == 1) return false;
            int len2 = rng.uniform_int(2, maxl + 1);
            stop = next(w.lk[w.n_lk1 - 1], -dir);
            x = w.cen[n - 1];
            w.n_lk2 = 0;
            #pragma unroll 1
            while (w.n_lk2 != len2 && x >= 0 && x != stop) {
                w.lk[w.n_lk1 + w.n_lk2++] = (int16_t)x;
                x = next(x, dir);
            }
            ext = lk_bound_externally();
            if (bad()) return false;
        }
        return !ext;
    }
    // ClusteredLinkerRegrowthMCMovetype::linear_select_central_segment (:670)
    // and cyclic_select_central_segment (:734): the run of bound scaffold
    // domains at or next to a random kernel domain
    __device__ void lk_reverse_cen() {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int a = 0, b = w.n_cen - 1; a < b; ++a, --b) {
            int16_t t = w.cen[a];
            w.cen[a] = w.cen[b];
            w.cen[b] = t;
        }
    }
    __device__ __noinline__ void lk_central_run() {
        LdoCtWork<C>& w = *ct;
        w.dir = 1;
        w.n_cen = 0;
        int kd = rng.uniform_int(1, ns - 2);
        bool started = false;
        if (st[kd] == BOUND) {
            started = true;
            w.cen[w.n_cen++] = (int16_t)kd;
            int p = next(kd, -1);
            #pragma unroll 1
            while (p >= 0 && st[p] == BOUND && w.n_cen != ns - 1) {
                w.cen[w.n_cen++] = (int16_t)p;
                p = next(p, -1);
            }
        }
        if (w.n_cen == ns - 1) {
            w.n_cen = 0;
            return;
        }
        lk_reverse_cen();
        bool ended = false;
        int n = next(kd, 1);
        #pragma unroll 1
        while (!ended && n >= 0 && n != kd && w.n_cen < ns) {
            if (st[n] == BOUND) {
                started = true;
                w.cen[w.n_cen++] = (int16_t)n;
            }
            else if (started) {
                ended = true;
            }
            n = next(n, 1);
        }
        if (cyclic || started) return;
        n = next(kd, -1);
        #pragma unroll 1
        while (!ended && n >= 0 && w.n_cen < ns) {
            if (st[n] == BOUND) {
                started = true;
                w.cen[w.n_cen++] = (int16_t)n;
            }
            else if (started) {
                ended = true;
            }
            n = next(n, -1);
        }
        lk_reverse_cen();
    }
    // ClusteredLinkerRegrowthMCMovetype::select_and_setup_segments (:607):
    // linkers run outwards from the cluster over domains that are not bound
    __device__ __noinline__ bool lk_select_clustered() {
        LdoCtWork<C>& w = *ct;
        int maxl = sys->move_opt[cur_mv][LDO_MO_MAX_LINKER];
        bool ext = true;
        #pragma unroll 1
        for (int att = 0; ext && att != 10; ++att) {
            lk_central_run();
            if (w.n_cen == 0) return false;
            ext = lk_bound_externally();
            if (bad()) return false;
        }
        if (ext) return false;
        int first = w.cen[0], last = w.cen[w.n_cen - 1];
        w.n_lk1 = 0;
        w.lk[w.n_lk1++] = (int16_t)first;
        int p = next(first, -1);
        if (p != last && p != next(last, 1)) {
            int stop = next(last, 2);
            #pragma unroll 1
            while (p >= 0 && st[p] != BOUND && w.n_lk1 != maxl && p != stop) {
                w.lk[w.n_lk1++] = (int16_t)p;
                p = next(p, -1);
            }
        }
        if (w.n_lk1 == 1) return false;
        int l1end = w.lk[w.n_lk1 - 1];
        w.n_lk2 = 0;
        w.lk[w.n_lk1 + w.n_lk2++] = (int16_t)last;
        int q = next(last, 1);
        if (q != l1end) {
            int stop = next(l1end, -1);
            #pragma unroll 1
            while (q >= 0 && st[q] != BOUND && w.n_lk2 != maxl && q != stop) {
                w.lk[w.n_lk1 + w.n_lk2++] = (int16_t)q;
                q = next(q, 1);
            }
        }
        return true;
    }
    // setup_fixed_end_biases (:210): the domains past the linkers' far ends as
    // active endpoints of segments 0 and 1, then the constraint points of
    // linker 1 (without its central domain, growing against m_dir) and
    // linker 2 (along it); the recoil-growth stack starts at linker 1's
    // central domain (CTRGLinkerRegrowthMCMovetype, :1161)
    __device__ __noinline__ void lk_setup_constraints() {
        LdoCtWork<C>& w = *ct;
        int dir = w.dir;
        int e1 = next(w.lk[w.n_lk1 - 1], -dir);
        int e2 = next(w.lk[w.n_lk1 + w.n_lk2 - 1], dir);
        w.lk_end[0] = (int16_t)e1;
        w.lk_end[1] = (int16_t)e2;
        if (e1 >= 0) ct_add_ep_seg(e1, pos(e1), 0);
        if (e2 >= 0) ct_add_ep_seg(e2, pos(e2), 1);
        int n = 0;
        #pragma unroll 1
        for (int k = 1; k < w.n_lk1; ++k) w.seg_dom[n++] = w.lk[k];
        w.seg_off[0] = 0;
        w.seg_off[1] = (int16_t)n;
        #pragma unroll 1
        for (int k = 1; k < w.n_lk2; ++k) w.seg_dom[n++] = w.lk[w.n_lk1 + k];
        w.seg_off[2] = (int16_t)n;
        w.n_segs = 2;
        w.seg_dirin[0] = (int8_t)(-dir);
        w.seg_dirin[1] = (int8_t)dir;
        w.rd[0] = w.lk[0];
        w.n_rd = 1;
        ct_calc_constraintpoints();
    }
    __device__ void lk_save_unassign(int d) {
        LdoCtWork<C>& w = *ct;
        w.p_old[d] = pos(d);
        w.o_old[d] = ore[d];
        unassign_domain(d);
    }
    __device__ void lk_reset_segment(int n) {   // reset_segment (:145)
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int k = 0; k < n; ++k) unassign_domain(w.cdom[k]);
    }
    // steps_less_than_distance (:524): a linker's central end farther (in
    // lattice steps) from its far end than the linker has domains
    __device__ bool lk_steps_less() {
        LdoCtWork<C>& w = *ct;
        int dist[2] = {0, 0};
        #pragma unroll 1
        for (int k = 0; k < 2; ++k) {
            int e = w.lk_end[k];
            if (e < 0) continue;
            V3 d = sub(pos(w.lk[k == 0 ? 0 : w.n_lk1]), pos(e));
            dist[k] = abs(vx(d)) + abs(vy(d)) + abs(vz(d));
        }
        return !(dist[0] <= w.n_lk1 && dist[1] <= w.n_lk2);
    }
    // apply_transformation (:401) of the central domains from src
    __device__ __noinline__ double lk_apply(const long long* src_p, const uint8_t* src_o, V3 disp, V3 center,
                                            int axis, int turns) {
        LdoCtWork<C>& w = *ct;
        double de = 0;
        #pragma unroll 1
        for (int k = 0; k < w.n_cdom; ++k) {
            int d = w.cdom[k];
            V3 p = lk_place(src_p[d], center, axis, turns, disp);
            int o = lk_orient(src_o[d], axis, turns);
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND) {
                lk_reset_segment(k);
                return 0;
            }
            if (occ == UNBOUND) {
                int ud = unbound_at(p);
                bool scaf_mis = scs[d] == 0 && scs[ud] == 0;
                bool new_pair = !lk_in(w.cdom, w.n_cdom, ud);
                if (!scaf_mis && new_pair) {
                    lk_reset_segment(k);
                    return 0;
                }
                if (scaf_mis && new_pair) {   // check_domain_constraints
                    probe_domain(d, p, o);
                    if (bad()) return 0;
                    if (hdr.violated) {
                        hdr.violated = 0;
                        lk_reset_segment(k);
                        return 0;
                    }
                }
            }
            de += set_checked(d, p, o);
            if (bad()) return 0;
        }
        return dexp(-de);
    }
    // transform_segment (:316), and with rev revert_transformation (:467):
    // the trial transformations of the central domains from src (centre: a
    // central segment domain's src position), each counted with its
    // Boltzmann factor when both linkers can still reach their ends; the
    // forward move then places one chosen by those weights, the reverse
    // places the old configuration and adds its per-domain factors
    __device__ __noinline__ double lk_transform(const long long* src_p, const uint8_t* src_o, bool rev) {
        LdoCtWork<C>& w = *ct;
        const int* mo = sys->move_opt[cur_mv];
        int K = mo[LDO_MO_NUM_TRANSFORMS] - (rev ? 1 : 0);
        int maxt = mo[LDO_MO_MAX_TURNS], maxd = mo[LDO_MO_MAX_DISP];
        double bias = 0;
        w.n_tr = 0;
        #pragma unroll 1
        for (int k = 0; k < K && !bad(); ++k) {
            int ci = rng.uniform_int(0, w.n_cen - 1);
            V3 center = src_p[w.cen[ci]];
            int axis = rng.uniform_int(0, 2);
            int turns = rng.uniform_int(0, maxt);
            int dx = rng.uniform_int(-maxd, maxd);
            int dy = rng.uniform_int(-maxd, maxd);
            int dz = rng.uniform_int(-maxd, maxd);
            V3 disp = mk(dx, dy, dz);
            double bf = lk_apply(src_p, src_o, disp, center, axis, turns);
            if (bf == 0) continue;
            if (!lk_steps_less()) {
                if (rev) {
                    bias += bf;
                }
                else {
                    int t = w.n_tr++;
                    w.tr_center[t] = center;
                    w.tr_disp[t] = disp;
                    w.tr_axis[t] = (int8_t)axis;
                    w.tr_turns[t] = (int8_t)turns;
                    w.tr_bf[t] = bf;
                }
            }
            lk_reset_segment(w.n_cdom);
        }
        if (bad()) return 0;
        if (rev) {
            #pragma unroll 1
            for (int k = 0; k < w.n_cdom; ++k) {
                int d = w.cdom[k];
                bias += dexp(-set_checked(d, w.p_old[d], w.o_old[d]));
            }
            return bias;
        }
        #pragma unroll 1
        for (int t = 0; t < w.n_tr; ++t) bias += w.tr_bf[t];
        if (bias == 0) {
            rejected = true;
            return bias;
        }
        double r = bias * rng.uniform_real();
        double cum = 0;
        int t = 0;
        #pragma unroll 1
        for (; t < w.n_tr - 1; ++t) {
            cum += w.tr_bf[t];
            if (r < cum) break;
        }
        lk_apply(src_p, src_o, w.tr_disp[t], w.tr_center[t], w.tr_axis[t], w.tr_turns[t]);
        return bias;
    }
    // The first phase of the linker movetypes: selection, constraint points,
    // the central domains, and the unassignment of everything that moves
    // (CTCB: linkers, regrown staples, central domains, then snapshot 1;
    // CTRG: the regrowth stack and the central domains, then the new
    // configuration's transformation and recoil growth).
    __device__ __noinline__ int lk_begin(int kind) {
        LdoCtWork<C>& w = *ct;
        ct_clear();
        w.kind = kind;
        w.delta_e = 0;
        w.weight = 1;
        w.weight_new = 1;
        const int* mo = sys->move_opt[cur_mv];
        w.max_recoils = mo[LDO_MO_MAX_RECOILS];
        w.max_c_attempts = mo[LDO_MO_MAX_C_ATTEMPTS];
        bool ok = kind == LDO_MV_CTCB_CLINKER ? lk_select_clustered() : lk_select();
        if (!ok || bad()) return finish_move(false, 0);
        lk_setup_constraints();
        if (bad()) return finish_move(false, 0);
        lk_central_domains();
        if (bad()) return finish_move(false, 0);
        if (kind == LDO_MV_CTRG_LINKER) {   // CTRGLinkerRegrowthMCMovetype::internal_attempt_move (:1148)
            if (w.n_rd < 2) return finish_move(false, 0);   // nothing to regrow: the reference reads past its stack
            w.p_old[w.rd[0]] = pos(w.rd[0]);
            w.o_old[w.rd[0]] = ore[w.rd[0]];
            #pragma unroll 1
            for (int k = 1; k < w.n_rd; ++k) {
                int d = w.rd[k];
                w.p_old[d] = pos(d);
                w.o_old[d] = ore[d];
                w.delta_e += unassign_domain(d);
            }
            w.n_eq = 0;
            #pragma unroll 1
            for (int k = 0; k < w.n_cdom; ++k) lk_save_unassign(w.cdom[k]);
            w.weight *= lk_transform(w.p_old, w.o_old, false);
            if (rejected || bad()) return finish_move(false, 0);
            w.delta_e += rg_recoil_regrow();
            if (rejected || bad()) return finish_move(false, 0);
            update_move_params();   // add_external_bias (:84)
            w.delta_e += calc_move();
            // setup_for_calc_new_weights (:137): the new configuration
            #pragma unroll 1
            for (int k = 0; k < w.n_rd; ++k) {
                int d = w.rd[k];
                w.p_new[d] = pos(d);
                w.o_new[d] = ore[d];
                w.catt_wq[k] = w.catt_q[k];
                w.av_wq[k] = w.av_q[k];
            }
            #pragma unroll 1
            for (int k = 0; k < w.n_cdom; ++k) {
                int d = w.cdom[k];
                w.p_new[d] = pos(d);
                w.o_new[d] = ore[d];
            }
            phase = PH_LKR2;
            return CMD_SNAP(2) | CMD_MORE;
        }
        // CTCBLinkerRegrowthMCMovetype::internal_attempt_move (:859)
        #pragma unroll 1
        for (int k = 1; k < w.n_lk1; ++k) lk_save_unassign(w.lk[k]);
        #pragma unroll 1
        for (int k = 1; k < w.n_lk2; ++k) lk_save_unassign(w.lk[w.n_lk1 + k]);
        unsigned long long left = w.regrow;
        #pragma unroll 1
        while (left) {
            int best = -1;
            #pragma unroll 1
            for (unsigned long long m = left; m; m &= m - 1ull) {
                int cs = __ffsll((long long)m) - 1;
                if (best < 0 || chain_c[cs] < chain_c[best]) best = cs;
            }
            left &= ~(1ull << best);
            int len = chain_len(best);
            #pragma unroll 1
            for (int q = 0; q < len; ++q) lk_save_unassign(slot_of(best, q));
        }
        #pragma unroll 1
        for (int k = 0; k < w.n_cdom; ++k) lk_save_unassign(w.cdom[k]);
        phase = PH_LK2;
        return CMD_SNAP(1) | CMD_MORE;
    }
    __device__ __noinline__ int lk_cb_new() {
        LdoCtWork<C>& w = *ct;
        regrow_old = false;
        w_bias *= lk_transform(w.p_old, w.o_old, false);
        if (rejected || bad()) return finish_move(false, 0);
        ct_grow_list(2, 0, w.n_lk1);
        if (rejected || bad()) return finish_move(false, 0);
        ct_grow_list(2, w.n_lk1, w.n_lk2);
        if (rejected || bad()) return finish_move(false, 0);
        update_move_params();   // add_external_bias (:52)
        w_bias *= dexp(-calc_move());
        // setup_for_regrow_old (:215); the transformations of the old pass
        // start from the central domains' new configuration
        regrow_old = true;
        w_new_bias = w_bias;
        new_modifier = modifier;
        w_bias = 1;
        #pragma unroll 1
        for (int k = 0; k < w.n_cdom; ++k) {
            int d = w.cdom[k];
            w.p_new[d] = pos(d);
            w.o_new[d] = ore[d];
        }
        phase = PH_LK3;
        return CMD_SNAP(2) | CMD_REST(1) | CMD_MORE;
    }
    __device__ __noinline__ int lk_cb_old() {
        LdoCtWork<C>& w = *ct;
        ct_reset_endpoints();
        w_bias *= lk_transform(w.p_new, w.o_new, true);
        if (bad()) return finish_move(false, 0);
        // both linkers grow in the old configuration whatever the first did
        ct_grow_list(2, 0, w.n_lk1);
        ct_grow_list(2, w.n_lk1, w.n_lk2);
        if (bad()) return finish_move(false, 0);
        modifier = 1;
        double ratio = w_new_bias / w_bias;   // test_cb_acceptance (:182)
        bool acc = test_acceptance(ratio);
        return finish_move(acc, acc ? 2 : 0);
    }
    // CTRGLinkerRegrowthMCMovetype, from the weights of the new configuration
    // to the acceptance test (:1181-1211)
    __device__ __noinline__ int lk_rg_weigh() {
        LdoCtWork<C>& w = *ct;
        #pragma unroll 1
        for (int k = 1; k < w.n_rd; ++k) unassign_domain(w.rd[k]);   // unassign_and_save_domains
        w.n_eq = 0;
        ct_reset_endpoints();
        rg_calc_weights(w.p_new, w.o_new);
        if (bad()) return finish_move(false, 0);
        #pragma unroll 1
        for (int k = 1; k < w.n_rd; ++k) unassign_domain(w.rd[k]);   // unassign_domains
        w.n_eq = 0;
        #pragma unroll 1
        for (int k = 0; k < w.n_cdom; ++k) unassign_domain(w.cdom[k]);
        w.weight /= lk_transform(w.p_new, w.o_new, true);
        if (bad()) return finish_move(false, 0);
        ct_reset_endpoints();
        rg_calc_old_c_opens();
        if (bad()) return finish_move(false, 0);
        // setup_for_calc_old_weights (:146)
        w.weight_new = w.weight;
        w.weight = 1;
        #pragma unroll 1
        for (int k = 0; k < w.n_rd; ++k) {
            w.catt_wq[k] = w.catt_q[k];
            w.av_wq[k] = w.av_q[k];
        }
        #pragma unroll 1
        for (int k = 1; k < w.n_rd; ++k) unassign_domain(w.rd[k]);   // unassign_and_save_domains
        w.n_eq = 0;
        ct_reset_endpoints();
        rg_calc_weights(w.p_old, w.o_old);
        if (bad()) return finish_move(false, 0);
        double ratio = w.weight_new / w.weight * dexp(-w.delta_e);   // test_rg_acceptance (:515)
        bool acc = test_acceptance(ratio);
        return finish_move(acc, acc ? 2 : 0);
    }

    // GCMCSimulation::simulate, one step (src/simulation.cpp:575-619), as a
    // state machine: step_begin runs the move until it needs the warp to copy
    // snapshots, step_resume continues it, and each returns the next CMD_*
    // (0 = step done).  Snapshot 0 always holds the state at the start of the
    // move.  A rejected move is undone by restoring it instead of the
    // reference's reset_origami + update_move_params + calc_move: the same
    // lattice state, order parameters and biases; the energy and bias totals
    // come back exactly instead of through the reversal's roundings.
    // CT: the kernel is built with the scaffold regrowth movetypes (a kernel
    // without them keeps their code out of its instruction stream).
    template <bool CT>
    __device__ __noinline__ int step_begin(long long s) {
        cur_s = s;
        double r = rng.uniform_real();
        int nm = sys->n_moves;
        int mv = 0;
        #pragma unroll 1
        while (mv < nm && !(r < sys->move_cum[mv])) ++mv;
        if (mv == nm) {
            fail(LDO_RS_INVARIANT);
            return 0;
        }
        cur_mv = mv;
        reset_internal();
        int kind = sys->move_kind[mv];
        if (kind >= LDO_MV_CTRG && kind <= LDO_MV_CTCB_JUMP) {   // scaffold regrowth
            if constexpr (CT) {
                if (ct) return kind <= LDO_MV_CTRG_JUMP ? rg_begin(kind) : ctcb_begin(kind);
            }
            fail(LDO_RS_INVARIANT);
            return 0;
        }
        if constexpr (CT) {   // scaffold transforms with linker regrowth
            if (kind >= LDO_MV_CTCB_LINKER && kind <= LDO_MV_CTRG_LINKER) {
                if (ct) return lk_begin(kind);
                fail(LDO_RS_INVARIANT);
                return 0;
            }
        }
        bool acc = false;
        switch (kind) {
        case LDO_MV_ORIENT: acc = orientation_rotation(); break;
        case LDO_MV_MET_EXCHANGE: acc = met_exchange(); break;
        case LDO_MV_MET_REGROWTH: acc = met_regrowth(); break;
        case LDO_MV_LEARNED_EXCHANGE: acc = learned_exchange(); break;
        case LDO_MV_LEARNED_REGROWTH: acc = learned_regrowth(); break;
        case LDO_MV_CB_REGROWTH: return cb_begin();
        }
        return finish_move(acc, 0);
    }

    // Move statistics, then the snapshot work: an accepted move refreshes
    // snapshot 0 (CB: restore snapshot `from` first), a rejected move that
    // changed anything restores it, or, with rej_from, keeps the state of
    // snapshot rej_from (a rejection that the reference reverts to it).
    __device__ __noinline__ int finish_move(bool acc, int from, int rej_from = 0) {
        if (bad()) return 0;
        mstat[2 * cur_mv] += 1;
        int cmd = 0;
        recalc = false;
        if (acc) {
            mstat[2 * cur_mv + 1] += 1;
            cmd = from ? (CMD_REST(from) | CMD_SNAP(0) | CMD_REST_FIRST) : CMD_SNAP(0);
        }
        else if (rej_from) {
            cmd = CMD_REST(rej_from) | CMD_SNAP(0) | CMD_REST_FIRST;
            if (sys->n_biases > 0) recalc = true;
        }
        else {
            // With bias functions the reference's trailing update_move_params
            // + calc_move also fold in a grid or window change made since
            // the last calc_move, so they still run after the restore.
            if (dirty) cmd = CMD_REST(0);
            if (sys->n_biases > 0) {
                if (dirty) recalc = true;
                else {
                    update_move_params();
                    calc_move();
                }
            }
        }
        long long s = cur_s;
        if (recalc || (sys->centering_freq != 0 && s % sys->centering_freq == 0) ||
            (sys->constraint_check_freq != 0 && s % sys->constraint_check_freq == 0)) {
            phase = PH_POST;
            cmd |= CMD_MORE;
        }
        return cmd;
    }

    template <bool CT>
    __device__ __noinline__ int step_resume() {
        if (bad()) return 0;
        if (phase == PH_CB2) return cb_mid();
        if (phase == PH_CB3) return cb_end();
        if constexpr (CT) {
            if (phase == PH_RG2) return rg_grow();
            if (phase == PH_RG3) return rg_weigh_new();
            if (phase == PH_RG4) return rg_old_opens();
            if (phase == PH_RG5) return rg_weigh_old();
            if (phase == PH_CT2) return ctcb_new();
            if (phase == PH_CT3) return ctcb_old();
            if (phase == PH_LK2) return lk_cb_new();
            if (phase == PH_LK3) return lk_cb_old();
            if (phase == PH_LKR2) return lk_rg_weigh();
        }
        phase = 0;
        if (recalc) {
            recalc = false;
            update_move_params();
            calc_move();
        }
        long long s = cur_s;
        int cmd = 0;
        if (sys->centering_freq != 0 && s % sys->centering_freq == 0) {
            center(sys->centering_domain);
            cmd = CMD_SNAP(0);
        }
        if (sys->constraint_check_freq != 0 && s % sys->constraint_check_freq == 0) check_all_constraints();
        return cmd;
    }
};

} // namespace ldo
