// Learned proposals: feature encoding and network shape, shared by the MC
// kernel, the network kernels, the host library and the oracle.
//
// Insertion: the network scores a candidate growth-point domain g from its
// local neighbourhood along its chain: the states of the domains two and one
// step before and after g (none / unbound / bound / misbound), the type slot
// of the staple complementary to g, and the temperature bin; exp(logit)
// weighs g among the unbound domains (LDO_LEARN_INS entries).
// Regrowth directions: the same network, with a task flag in its input,
// scores the six lattice sites next to a growing staple domain's chain
// neighbour by what the site holds (empty / an unbound domain complementary
// to the growing one / another unbound domain / a bound pair) and the
// temperature bin (LDO_LEARN_DIRS entries after the insertion entries).
// LearnedStapleRegrowth grows staples with these directions, and so does
// LearnedStapleExchange after placing an inserted staple's growth point.
// The input space is finite (LDO_LEARN_TABLE entries), so the network is
// evaluated once for every input on the tensor cores and the MC kernel reads
// the weights from that table: the proposals are exact functions of the
// current state, as the Metropolis-Hastings ratio requires.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define LDO_LHD __host__ __device__
#else
#define LDO_LHD
#endif

enum {
    LDO_LEARN_DIN = 64,       // network input width
    LDO_LEARN_H = 256,        // hidden width (three GELU layers)
    LDO_LEARN_NTYPE = 32,     // type slots: 0 = no complementary staple
    LDO_LEARN_NTB = 64,       // temperature bins of 1 K from 300 K
    LDO_LEARN_NCOMBO = 256,   // 4 neighbour states x 4 positions
    LDO_LEARN_NDIRF = 4,      // regrowth site classes
    LDO_LEARN_INS = LDO_LEARN_NTB * LDO_LEARN_NTYPE * LDO_LEARN_NCOMBO,
    LDO_LEARN_DIRS = LDO_LEARN_NTB * LDO_LEARN_NDIRF,
    LDO_LEARN_TABLE = LDO_LEARN_INS + LDO_LEARN_DIRS,
    // parameter vector: W1[64][256] b1[256] W2[256][256] b2 W3[256][256] b3 w4[256] b4
    LDO_LEARN_OFF_W1 = 0,
    LDO_LEARN_OFF_B1 = LDO_LEARN_OFF_W1 + LDO_LEARN_DIN * LDO_LEARN_H,
    LDO_LEARN_OFF_W2 = LDO_LEARN_OFF_B1 + LDO_LEARN_H,
    LDO_LEARN_OFF_B2 = LDO_LEARN_OFF_W2 + LDO_LEARN_H * LDO_LEARN_H,
    LDO_LEARN_OFF_W3 = LDO_LEARN_OFF_B2 + LDO_LEARN_H,
    LDO_LEARN_OFF_B3 = LDO_LEARN_OFF_W3 + LDO_LEARN_H * LDO_LEARN_H,
    LDO_LEARN_OFF_W4 = LDO_LEARN_OFF_B3 + LDO_LEARN_H,
    LDO_LEARN_OFF_B4 = LDO_LEARN_OFF_W4 + LDO_LEARN_H,
    LDO_LEARN_NPARAM = LDO_LEARN_OFF_B4 + 1
};

// Proposal mixture weights: with probability LDO_LEARN_EPS the target is
// uniform over all domains, and with LDO_LEARN_EPS_T the staple type and
// domain are uniform; both keep every insertion the reference can make
// possible.
#define LDO_LEARN_EPS 0.05
#define LDO_LEARN_EPS_T 0.05
// Regrowth: with probability LDO_LEARN_EPS_D the direction is uniform over
// the six sites, with LDO_LEARN_EPS_O the orientation at a site holding an
// unbound domain is uniform (otherwise the one opposite to that domain's);
// every configuration the reference's uniform regrowth makes stays possible.
#define LDO_LEARN_EPS_D 0.05
#define LDO_LEARN_EPS_O 0.05
// Deletion: with probability LDO_LEARN_EPS_DEL the staple is uniform over the
// staples, otherwise it is drawn with weight LDO_LEARN_DEL_PART when one of
// its domains is not fully bound (unbound or misbound) and 1 when all are.
#define LDO_LEARN_EPS_DEL 0.05
#define LDO_LEARN_DEL_PART 8.0
#define LDO_LEARN_LOGIT_CLAMP 30.0f

LDO_LHD inline int ldo_learn_tbin(double temp) {
    int b = (int)floor(temp - 300.0 + 0.5);
    return b < 0 ? 0 : (b >= LDO_LEARN_NTB ? LDO_LEARN_NTB - 1 : b);
}
LDO_LHD inline int ldo_learn_index(int tbin, int tslot, int combo) {
    return (tbin * LDO_LEARN_NTYPE + tslot) * LDO_LEARN_NCOMBO + combo;
}
// Regrowth site class f (0 empty, 1 unbound complementary, 2 unbound other,
// 3 bound or misbound) at temperature bin tbin.
LDO_LHD inline int ldo_learn_dir_index(int tbin, int f) { return LDO_LEARN_INS + tbin * LDO_LEARN_NDIRF + f; }
// Type slot of staple type t (1..S) in the one-hot (types above 31 share slots).
LDO_LHD inline int ldo_learn_tslot(int t) { return t <= 0 ? 0 : 1 + (t - 1) % (LDO_LEARN_NTYPE - 1); }
// Input vector of table entry k (written as floats; the kernels round to bf16):
// insertion entries: [0,16) one-hot neighbour states (position-major: two
// before, one before, one after, two after), [16,48) type-slot one-hot,
// [48] (T - 335 K) / 15 K, [49] 1, the rest 0; regrowth entries: [0,4)
// one-hot site class, [48] and [49] as above, [50] 1 (the task flag).
LDO_LHD inline void ldo_learn_input(int k, float* x) {
    for (int i = 0; i < LDO_LEARN_DIN; ++i) x[i] = 0.f;
    if (k >= LDO_LEARN_INS) {
        int kk = k - LDO_LEARN_INS;
        int tb = kk / LDO_LEARN_NDIRF;
        x[kk % LDO_LEARN_NDIRF] = 1.f;
        x[48] = (float)(tb - 35) / 15.f;
        x[49] = 1.f;
        x[50] = 1.f;
        return;
    }
    int combo = k % LDO_LEARN_NCOMBO;
    int tslot = (k / LDO_LEARN_NCOMBO) % LDO_LEARN_NTYPE;
    int tbin = k / (LDO_LEARN_NCOMBO * LDO_LEARN_NTYPE);
    for (int o = 0; o < 4; ++o) x[4 * o + ((combo >> (2 * o)) & 3)] = 1.f;
    x[16 + tslot] = 1.f;
    x[48] = (float)(tbin - 35) / 15.f;
    x[49] = 1.f;
}
