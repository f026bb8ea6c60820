// Exact staple-only enumeration on the GPU (StapleConformationalEnumerator,
// src/enumerate.cpp:666-811, with the base ConformationalEnumerator's
// enumerate_domain / set_growthpoint_domains / set_bound_domain,
// :378-550, and the overcount calculators, :83-159).
//
// The host lists the independent work units the reference walks through in
// series -- each staple set (StapleEnumerator::recurse, :1103) times each
// distinct growth-point set (GrowthpointEnumerator, :819-1067) -- and one
// thread per unit runs the reference's conformational recursion on its own
// replica state in shared memory, with the engine's set_domain_config /
// unassign_domain (the same energies as the MC moves), and writes the
// Boltzmann weight of every configuration into its own row of a histogram
// over two order parameters.  The host adds the rows in unit order.
//
// Orientations: the staple-only recursion places an unbound staple domain
// with the orientation (0, 0, 0) (:781-791), which the engine's orientation
// indices cannot hold.  Such a domain is stored with index 0 and marked; a
// domain that later binds to it takes the opposite index, so the reference's
// test that paired orientations are opposite (-0 == 0) passes as it does
// there.  Only misbound pairs can form at such a site (staple domains are
// not complementary to each other), and misbound pairs are not read by the
// stacking and twist terms, so no energy depends on the stand-in index.
#pragma once
#include "ldo_engine.cuh"
#include "ldo_kernels.h"

namespace ldo {

template <class C>
struct EnumWork {
    int16_t stack[C::DCAP];       // m_domains
    int sp;
    long long pgp[C::DCAP];       // m_prev_growthpoint_ps
    int npgp;
    int16_t gp_of[C::DCAP];       // m_growthpoints
    int16_t inv_gp[C::DCAP];      // m_inverse_growthpoints
    uint8_t zero_ore[C::DCAP];    // orientation (0, 0, 0) in the reference
    double E, E_lo, mult, prefix;     // E + E_lo: the running energy, summed without rounding drift
    double part, nconf, sumE;
    double part_c, sumE_c;        // compensations of part and sumE
    double* row;                  // this part's histogram row, then its compensations
    int op1, op2, n1, n2;         // key order parameters and histogram shape
    int overcount;                // 0 MaxTwoDomain, 1 MisbindingOnly
    int bad;                      // a key outside the histogram
    int full;                     // ConformationalEnumerator::enumerate: the scaffold enumerated too
    int depth, npre;              // choice loops around the current call; levels fixed by the prefix
    int8_t pre[LDO_ENUM_MAX_SPLIT];   // the branch taken at each fixed level
    int16_t cnt[2 * LDO_ENUM_MAX_IDENT + 1];   // m_identities_to_num_unassigned
};

template <class C>
struct Enumerator {
    Rep<C>& R;
    EnumWork<C>& W;

    __device__ void push(int d) { W.stack[W.sp++] = (int16_t)d; }
    __device__ int pop() { return W.stack[--W.sp]; }

    __device__ double set(int d, V3 p, int o) {
        W.zero_ore[d] = 0;
        return R.set_domain_config(d, p, o);
    }
    __device__ double unset(int d) { return R.unassign_domain(d); }
    // m_energy (long double in the reference) as a two-term sum: a traversal
    // adds and removes millions of domain energies, whose FP64 roundings would
    // otherwise drift (TwoSum, Knuth; the error term collects each rounding)
    __device__ void addE(double x) {
        double s = W.E + x;
        double bp = s - W.E;
        W.E_lo += (W.E - (s - bp)) + (x - bp);
        W.E = s;
    }
    __device__ double energy() const { return W.E + W.E_lo; }
    // Neumaier's compensated summation: s + c is the sum of the added terms
    // without the drift a running double sum picks up over millions of terms
    __device__ static void acc(double& s, double& c, double x) {
        double t = s + x;
        c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    __device__ int16_t& count(int ident) { return W.cnt[ident + LDO_ENUM_MAX_IDENT]; }
    // a unit split by a prefix follows only its branch at the first levels
    __device__ bool skip(int level, int k) const { return level < W.npre && k != W.pre[level]; }

    // ConformationalEnumerator::calc_and_save_weights (:639)
    __device__ __noinline__ void save() {
        W.nconf += W.mult;
        R.update_move_params();
        double e = energy();
        double w = W.prefix * exp(-e) * W.mult;
        acc(W.part, W.part_c, w);
        acc(W.sumE, W.sumE_c, e * w);
        int k1 = R.op[2 * W.op1], k2 = R.op[2 * W.op2];
        if (k1 < 0 || k1 >= W.n1 || k2 < 0 || k2 >= W.n2) {
            W.bad = 1;
            return;
        }
        int k = k1 * W.n2 + k2;
        acc(W.row[k], W.row[W.n1 * W.n2 + k], w);
    }

    // MaxTwoDomainOvercountCalculator::count_involved_staples (:131)
    __device__ int involved(int d) {
        if (R.scs[d] == 0) return 0;
        int n = 1;
        int x = d;
        #pragma unroll 1
        for (int guard = 0; guard < C::DCAP; ++guard) {
            int nx = R.nxt[x] < 0 ? R.prv[x] : R.nxt[x];
            if (nx < 0) break;
            x = R.bnd[nx];
            if (x < 0 || R.scs[x] == 0) break;
            ++n;
        }
        return n;
    }

    // OvercountCalculator::calc_multiplier (:83, :112)
    __device__ __noinline__ double overcount(int d, int other) {
        if (W.overcount == 0) {
            if (R.scs[d] == R.scs[other]) return 1.0;
            double m = 1.0;
            m /= (involved(d) + involved(other) + 1);
            return m;
        }
        double m = 1.0;
        #pragma unroll 1
        for (int x = R.nxt[d]; x >= 0; x = R.nxt[x]) {
            if (R.st[x] == BOUND) m += 1;
            else if (R.st[x] == UNASSIGNED) return 1.0;
        }
        #pragma unroll 1
        for (int x = R.prv[d]; x >= 0; x = R.prv[x]) {
            if (R.st[x] == BOUND) m += 1;
            else if (R.st[x] == UNASSIGNED) return 1.0;
        }
        return m;
    }

    // ConformationalEnumerator::create_staple_stack (:610)
    __device__ __noinline__ void staple_stack(int d) {
        push(d);
        int cs = R.scs[d], len = R.clen[cs], di = R.sd[d];
        #pragma unroll 1
        for (int k = di + 1; k < len; ++k) {
            int x = R.slot_of(cs, k);
            push(x);
            if (W.gp_of[x] >= 0) staple_stack(W.gp_of[x]);
        }
        #pragma unroll 1
        for (int k = di - 1; k >= 0; --k) {
            int x = R.slot_of(cs, k);
            push(x);
            if (W.gp_of[x] >= 0) staple_stack(W.gp_of[x]);
        }
    }

    // StapleConformationalEnumerator::create_domains_stack (:793)
    __device__ void domains_stack() {
        W.sp = 0;
        #pragma unroll 1
        for (int d = 0; d < R.ns; ++d) {
            if (W.gp_of[d] >= 0) {
                W.inv_gp[W.gp_of[d]] = (int16_t)d;
                staple_stack(W.gp_of[d]);
            }
        }
        #pragma unroll 1
        for (int a = 0, b = W.sp - 1; a < b; ++a, --b) {
            int16_t t = W.stack[a];
            W.stack[a] = W.stack[b];
            W.stack[b] = t;
        }
    }

    __device__ void next_from(int nd, V3 p) {
        if (W.inv_gp[nd] >= 0) grow_off_scaffold(nd);
        else enumerate_domain(nd, p);
    }

    // StapleConformationalEnumerator::grow_next_domain (:729), or the base
    // ConformationalEnumerator::grow_next_domain (:550) when the scaffold is
    // enumerated too
    __device__ __noinline__ void grow_next(int d, V3 p) {
        if (W.full) {
            grow_next_full(d, p);
            return;
        }
        if (W.sp != 0) next_from(pop(), p);
        else save();
        addE(unset(d));
    }
    __device__ __noinline__ void grow_next_full(int d, V3 p) {
        if (W.sp != 0) {
            int nd = pop();
            bool terminal = R.scs[d] != R.scs[nd];
            V3 np = p;
            if (terminal) {
                if (W.npgp == 0) {   // no growth point to return to: not a stack the reference builds
                    R.fail(LDO_RS_INVARIANT);
                    return;
                }
                np = W.pgp[--W.npgp];
            }
            enumerate_domain(nd, np);
            if (terminal) W.pgp[W.npgp++] = np;
        }
        else if (R.cyclic) {   // a closed scaffold must close
            V3 e = sub(R.pos(0), R.pos(R.ns - 1));
            if (abs(vx(e)) + abs(vy(e)) + abs(vz(e)) == 1) save();
        }
        else {
            save();
        }
        addE(unset(d));
    }

    // StapleConformationalEnumerator::grow_off_scaffold (:754)
    __device__ __noinline__ void grow_off_scaffold(int nd) {
        int g = W.inv_gp[nd];
        V3 p = R.pos(g);
        addE(set(nd, p, R.ore[g] ^ 1));
        if (R.hdr.violated) {
            R.hdr.violated = 0;
            push(nd);
        }
        else {
            if (W.sp != 0) {
                next_from(pop(), p);
                push(nd);
            }
            addE(unset(nd));
        }
    }

    // StapleConformationalEnumerator::set_unbound_domain (:781)
    __device__ __noinline__ void set_unbound(int d, V3 p) {
        addE(set(d, p, 0));
        W.zero_ore[d] = 1;
        double mult0 = W.mult;   // restored, not divided back: no drift over a traversal
        W.mult *= 6.0;
        grow_next(d, p);
        W.mult = mult0;
    }

    // ConformationalEnumerator::set_unbound_domain (:523): every orientation
    // while a complementary domain is still unassigned, else the (0, 0, 0)
    // stand-in counted six times
    __device__ __noinline__ void set_unbound_full(int d, V3 p) {
        int id = R.did[d];
        if (count(-id) == 0) {
            count(id) -= 1;
            addE(set(d, p, 0));
            W.zero_ore[d] = 1;
            double mult0 = W.mult;   // restored, not divided back: no drift over a traversal
            W.mult *= 6.0;
            grow_next_full(d, p);
            count(id) += 1;
            W.mult = mult0;
            return;
        }
        int level = W.depth++;
        #pragma unroll 1
        for (int o = 0; o < 6; ++o) {
            if (skip(level, o)) continue;
            addE(set(d, p, o));
            if (R.hdr.violated) {
                R.hdr.violated = 0;
                continue;
            }
            count(id) -= 1;
            grow_next_full(d, p);
            count(id) += 1;
        }
        W.depth--;
    }

    // ConformationalEnumerator::set_bound_domain (:499)
    __device__ __noinline__ void set_bound(int d, V3 p) {
        int occ = R.unbound_at(p);
        int zero = W.zero_ore[occ];
        addE(set(d, p, R.ore[occ] ^ 1));
        W.zero_ore[d] = (uint8_t)zero;
        if (R.hdr.violated) {
            R.hdr.violated = 0;
            return;
        }
        double m = overcount(d, occ);
        double mult0 = W.mult;   // restored, not divided back: no drift over a traversal
        W.mult *= m;
        count(R.did[d]) -= 1;
        grow_next(d, p);
        count(R.did[d]) += 1;
        W.mult = mult0;
    }

    // ConformationalEnumerator::set_comp_growthpoint_domains (:451)
    __device__ __noinline__ void set_comp_gp(int d, int bd, V3 p) {
        int level = W.depth++;
        #pragma unroll 1
        for (int o = 0; o < 6; ++o) {
            if (skip(level, o)) continue;
            addE(set(d, p, o));
            addE(set(bd, p, o ^ 1));
            if (R.hdr.violated) {
                R.hdr.violated = 0;
                addE(unset(d));
                continue;
            }
            count(R.did[d]) -= 1;
            count(R.did[bd]) -= 1;
            grow_next(bd, p);
            count(R.did[d]) += 1;
            count(R.did[bd]) += 1;
            addE(unset(d));
        }
        W.depth--;
    }

    // ConformationalEnumerator::set_mis_growthpoint_domains (:477)
    __device__ __noinline__ void set_mis_gp(int d, int bd, V3 p) {
        addE(set(d, p, 0));
        addE(set(bd, p, 1));
        double mult0 = W.mult;   // restored, not divided back: no drift over a traversal
        W.mult *= 6.0;
        count(R.did[d]) -= 1;
        count(R.did[bd]) -= 1;
        grow_next(bd, p);
        count(R.did[d]) += 1;
        count(R.did[bd]) += 1;
        addE(unset(d));
        W.mult = mult0;
    }

    // ConformationalEnumerator::set_growthpoint_domains (:413)
    __device__ __noinline__ void set_gp(int d, V3 p) {
        bool terminal = false;
        int f = R.nxt[d], b = R.prv[d];
        if (f >= 0 && R.st[f] == UNASSIGNED) {
            if (b >= 0) terminal = true;
        }
        else if (f >= 0) {
            terminal = true;
        }
        if (terminal) W.pgp[W.npgp++] = p;
        int bd = pop();
        if (R.did[d] == -R.did[bd]) set_comp_gp(d, bd, p);
        else set_mis_gp(d, bd, p);
        push(bd);
        if (terminal) --W.npgp;
    }

    // ConformationalEnumerator::enumerate_domain (:378)
    __device__ __noinline__ void enumerate_domain(int d, V3 p_prev) {
        int level = W.depth++;
        #pragma unroll 1
        for (int k = 0; k < 6 && !R.bad(); ++k) {
            if (skip(level, k)) continue;
            V3 p = add(p_prev, unit(k));
            bool is_gp = W.gp_of[d] >= 0;
            int occ = R.occupancy(p);
            bool occupied = occ == UNBOUND;
            bool bound = occ == BOUND || occ == MISBOUND;
            if ((is_gp && occupied) || bound) continue;
            if (is_gp) set_gp(d, p);
            else if (occupied) set_bound(d, p);
            else if (W.full) set_unbound_full(d, p);
            else set_unbound(d, p);
        }
        W.depth--;
        push(d);
    }

    // ConformationalEnumerator::create_domains_stack (:578): scaffold domains
    // in order, each growth point followed by its staple's stack; reversed
    __device__ void domains_stack_full() {
        W.sp = 0;
        #pragma unroll 1
        for (int d = 0; d < R.ns; ++d) {
            push(d);
            if (W.gp_of[d] >= 0) {
                W.inv_gp[W.gp_of[d]] = (int16_t)d;
                staple_stack(W.gp_of[d]);
            }
        }
        #pragma unroll 1
        for (int a = 0, b = W.sp - 1; a < b; ++a, --b) {
            int16_t t = W.stack[a];
            W.stack[a] = W.stack[b];
            W.stack[b] = t;
        }
    }
    // ConformationalEnumerator::enumerate (:218), after the constructor's
    // unassignment of the scaffold (:188): the first domain at the origin
    // along +x, its staple first when it is a growth point
    __device__ void run_full() {
        #pragma unroll 1
        for (int d = 0; d < R.ns; ++d) unset(d);
        domains_stack_full();
        if (W.sp < 2) return;
        int start = pop();
        V3 p = mk(0, 0, 0);
        count(R.did[start]) -= 1;
        set(start, p, 0);
        int nd = pop();
        if (W.gp_of[start] >= 0) {
            W.pgp[W.npgp++] = p;
            count(R.did[nd]) -= 1;
            addE(set(nd, p, 1));
            if (W.sp > 0) {
                int nn = pop();
                enumerate_domain(nn, p);
            }
            count(R.did[nd]) += 1;
            addE(unset(nd));
            W.npgp--;
        }
        else {
            enumerate_domain(nd, p);
        }
        count(R.did[start]) += 1;
        unset(start);
    }

    // StapleConformationalEnumerator::enumerate (:687)
    __device__ void run() {
        domains_stack();
        if (W.sp == 0) {
            save();
            return;
        }
        int start = pop();
        int g = W.inv_gp[start];
        V3 p = R.pos(g);
        addE(set(start, p, R.ore[g] ^ 1));
        if (W.sp != 0) {
            int nd = pop();
            next_from(nd, p);
        }
        else {
            save();
        }
        if (R.st[start] != UNASSIGNED) addE(unset(start));
    }
};

} // namespace ldo
