// Oracle (test infrastructure only): lattice state, FourBody potential, moves.
//
// CPU restatement of the reference's staple-move path, used by tests/, by
// smoke() and by bench.py's CPU-baseline leg to check and time the CUDA
// engine.  It is never linked into the engine.  Each member cites the
// reference function it restates.  The traversal order of the FourBody terms
// and of every energy accumulation follows the reference so that energies
// agree bit for bit and every random draw happens at the same point.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <deque>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "oracle_philox.hpp"
#include "oracle_thermo.hpp"
#include "../latticednaorigami_gb300/csrc/ldo_learn.h"
#include "../latticednaorigami_gb300/csrc/ldo_math.h"

namespace oracle {

enum Occ : int { UNASSIGNED = 0, UNBOUND = 1, BOUND = 2, MISBOUND = 3 };

struct V3 {
    int x {0}, y {0}, z {0};
    V3() = default;
    V3(int a, int b, int c): x(a), y(b), z(c) {}
    V3 operator+(const V3& o) const { return {x + o.x, y + o.y, z + o.z}; }
    V3 operator-(const V3& o) const { return {x - o.x, y - o.y, z - o.z}; }
    V3 operator-() const { return {-x, -y, -z}; }
    bool operator==(const V3& o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const V3& o) const { return !(*this == o); }
    V3 absv() const { return {std::abs(x), std::abs(y), std::abs(z)}; }
    int abssum() const { return std::abs(x) + std::abs(y) + std::abs(z); }
};

// Order matters: random index -> direction (include/.../utility.hpp:156-162).
static const V3 kUnit[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
// utility::basis_vectors (include/.../utility.hpp)
static const V3 kBasis[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

// VectorThree::rotate_half (src/utility.cpp:68)
inline V3 rotate_half(V3 v, V3 axis) {
    axis = axis.absv();
    if (axis == V3(1, 0, 0)) { v.y = -v.y; v.z = -v.z; }
    else if (axis == V3(0, 1, 0)) { v.x = -v.x; v.z = -v.z; }
    else if (axis == V3(0, 0, 1)) { v.x = -v.x; v.y = -v.y; }
    return v;
}

// VectorThree::rotate(axis, turns) (src/utility.cpp:102)
inline V3 rotate_quarter(V3 v, V3 axis, int turns) {
    if (turns % 2 == 0) return rotate_half(v, axis);
    bool odd_even = (turns - 1) / 2 % 2 == 0;
    int dir = (turns >= 0 && odd_even) ? 1 : -1;
    V3 a = axis.absv();
    if (axis != a) dir *= -1;
    if (a == V3(1, 0, 0)) { std::swap(v.y, v.z); v.y *= -dir; v.z *= dir; }
    else if (a == V3(0, 1, 0)) { std::swap(v.x, v.z); v.x *= -dir; v.z *= dir; }
    else if (a == V3(0, 0, 1)) { std::swap(v.x, v.y); v.x *= -dir; v.y *= dir; }
    return v;
}

inline uint64_t pos_key(const V3& p) {
    return ((uint64_t)(uint32_t)(p.x + (1 << 20)) << 42) | ((uint64_t)(uint32_t)(p.y + (1 << 20)) << 21) |
           (uint64_t)(uint32_t)(p.z + (1 << 20));
}

struct Dom {
    int c, cident, d, dident, clen;
    int fwd {-1}, bwd {-1};
    V3 pos, ore;
    int state {UNASSIGNED};
    int bound {-1};
};

struct Delta {
    double e {0};
    int stacked {0};
};

// A Rosenbluth weight.  The reference keeps CBMCMovetype::m_bias and
// m_new_bias in long double (include/.../cb_movetypes.hpp:126-127), whose
// width depends on the platform (x87 80-bit on x86-64, 128-bit on AArch64);
// the engine computes them in FP64.  With `ld` set the oracle follows the
// reference's long double, otherwise the engine's FP64.  The two choose the
// same configurations and accept the same moves except where a weight ratio
// lies within a rounding of 1 (then one side may skip the acceptance draw).
// The same holds for the exponential: the reference's is the C library's,
// the engine's is ldo_math::exp, identical on the GPU and the host.
struct Wt {
    long double v {1};
    bool ld {false};
    void set(long double x) { v = ld ? x : (long double)(double)x; }
    void mul(long double b) { v = ld ? v * b : (long double)((double)v * (double)b); }
    void div(long double b) { v = ld ? v / b : (long double)((double)v / (double)b); }
    long double over(const Wt& b) const { return ld ? v / b.v : (long double)((double)v / (double)b.v); }
};

struct SiteRec {
    int occ;
    int unbound_dom;   // valid when occ == UNBOUND
};

// State touches of the reference's algorithm, counted only in the build with
// ORACLE_COUNT_TOUCHES (liboracle_touch.so): every access to a domain record
// and every operation on the occupancy map, per thread.  They give the
// algorithmic bytes per move attempt of the engine's throughput roofline.
// In the normal build the containers below are plain std containers.
#ifdef ORACLE_COUNT_TOUCHES
struct TouchCounts {
    long long dom {0}, site {0};
};
inline thread_local TouchCounts g_touch;
#define ORACLE_TOUCH(field) (++g_touch.field)
#else
#define ORACLE_TOUCH(field) ((void)0)
#endif

template <class T>
struct DomVec : std::vector<T> {
    using std::vector<T>::vector;
    T& operator[](size_t i) {
        ORACLE_TOUCH(dom);
        return std::vector<T>::operator[](i);
    }
    const T& operator[](size_t i) const {
        ORACLE_TOUCH(dom);
        return std::vector<T>::operator[](i);
    }
};

struct SiteMap : std::unordered_map<uint64_t, SiteRec> {
    using Base = std::unordered_map<uint64_t, SiteRec>;
    iterator find(uint64_t k) {
        ORACLE_TOUCH(site);
        return Base::find(k);
    }
    const_iterator find(uint64_t k) const {
        ORACLE_TOUCH(site);
        return Base::find(k);
    }
    SiteRec& at(uint64_t k) {
        ORACLE_TOUCH(site);
        return Base::at(k);
    }
    const SiteRec& at(uint64_t k) const {
        ORACLE_TOUCH(site);
        return Base::at(k);
    }
    SiteRec& operator[](uint64_t k) {
        ORACLE_TOUCH(site);
        return Base::operator[](k);
    }
    size_t erase(uint64_t k) {
        ORACLE_TOUCH(site);
        return Base::erase(k);
    }
};

// ------------------------------------------------------- order params ----
enum OpKind { OP_NUMSTAPLES, OP_NUMSTAPLESTYPE, OP_STAPLETYPEFULLYBOUND, OP_NUMBOUND, OP_NUMMISBOUND,
              OP_NUMSTACKED, OP_NUMLINEARHELICES, OP_NUMSTACKEDJUNCTS, OP_SUM, OP_DIST, OP_ADJACENT };

struct OpRec {
    OpKind kind;
    std::string tag;
    int arg {0};
    std::vector<int> parts;   // Sum
    int param {0};
    bool defined {true};
};

enum BiasKind { B_LINEARSTEPWELL, B_SQUAREWELL, B_GRID, B_HARMONIC };

struct BiasRec {
    BiasKind kind;
    std::string tag;
    std::vector<int> ops;
    int min_op {0}, max_op {0};
    double well_bias {0}, min_bias {0}, slope {0}, outside_bias {0};
    double k {0}, centre {0};
    std::vector<double> grid;   // 1-D grid over op value 0..grid.size()-1
    bool grid_set {false};
    double off_grid {0};
    double bias {0};
};

enum MoveKind { MV_ORIENTATION = 0, MV_MET_EXCHANGE = 1, MV_MET_REGROWTH = 2, MV_CB_REGROWTH = 3, MV_LEARNED_EXCHANGE = 4,
                MV_CTRG_SCAFFOLD = 5, MV_CTRG_JUMP = 6, MV_CTCB_SCAFFOLD = 7, MV_CTCB_JUMP = 8,
                MV_LEARNED_REGROWTH = 9, MV_CTCB_LINKER = 10, MV_CTCB_CLINKER = 11, MV_CTRG_LINKER = 12 };

// Options of a scaffold regrowth movetype (src/simulation.cpp:400-560).
struct ScaffoldMoveOpts {
    int max_regrowth {0};
    int max_seg_regrowth {0};
    int max_num_recoils {0};
    int max_c_attempts {0};
    // linker movetypes (src/simulation.cpp:445)
    int max_disp {0};
    int max_turns {0};
    int max_linker_length {0};
    int num_transforms {0};
};

// IdealRandomWalks::num_walks (src/ideal_random_walk.cpp:14): the number of
// nearest-neighbour walks of `steps` steps on the cubic lattice between two
// sites, summed over the numbers of negative x and y steps.
inline long double ideal_walks(int dx, int dy, int dz, int steps) {
    int d[3] = {std::abs(dx), std::abs(dy), std::abs(dz)};
    std::sort(d, d + 3);
    int DX = d[0], DY = d[1], DZ = d[2];
    int sum = DX + DY + DZ;
    if (sum > steps || (steps - sum) % 2 != 0) return 0;
    int n_minus = (steps - sum) / 2;
    int n_plus = (steps - DX - DY + DZ) / 2;
    auto fact = [](int n) {
        long double f = 1;
        for (int k = 2; k <= n; ++k) f *= k;
        return f;
    };
    long double walks = 0;
    for (int yb = 0; yb <= n_minus; ++yb)
        for (int xb = 0; xb <= n_minus - yb; ++xb) {
            if (n_plus - xb - yb < 0) continue;
            walks += fact(steps) / (fact(xb) * fact(xb + DX) * fact(yb) * fact(yb + DY) *
                                    fact(n_minus - xb - yb) * fact(n_plus - xb - yb));
        }
    return walks;
}

struct Config {
    // chain-type identities, index 0 is the scaffold
    std::vector<std::vector<int>> identities;
    bool cyclic {false};
    bool three_quarter {false};
    bool misbinding_disallowed {false};
    bool mean_field {false};
    double staple_M {1};
    int max_total_staples {999};
    int max_type_staples {999};
    std::vector<int> move_kinds;
    std::vector<double> move_cum;
    std::vector<ScaffoldMoveOpts> move_opts;   // per movetype (scaffold regrowth options)
    std::vector<double> exchange_mults;
    bool adaptive_exchange {false};
    bool allow_nonsensical_ps {false};
    double bias_mult {1};
    int centering_freq {0};
    int centering_domain {0};
    int constraint_check_freq {0};
};

struct ChainInit {
    int index, identity;
    std::vector<V3> pos, ore;
};

class System {
  public:
    Config cfg;
    EnergyTables tab;
    Stream rng;

    // Bookkeeping (OrigamiSystem members, include/.../origami_system.hpp:175-205)
    DomVec<Dom> doms;
    std::vector<int> free_doms;
    std::vector<std::vector<int>> chains;   // domain ids, m_domains order
    std::vector<int> chain_index;           // unique chain index per chain
    std::vector<int> chain_ident;
    std::vector<std::vector<int>> ident_to_index;
    SiteMap sites;
    int num_domains {0}, num_staples {0}, num_bound {0}, num_fully {0}, num_self {0}, num_unassigned {0},
        num_stacked {0};
    int current_c_i {0};
    double energy {0};
    bool violated {false};

    std::vector<OpRec> ops;
    std::vector<BiasRec> biases;
    double move_bias {0};

    // move-loop statistics
    std::vector<long long> attempts, accepts;
    // state touches per movetype (ORACLE_COUNT_TOUCHES build)
    std::vector<long long> touch_dom, touch_site;

    // ---------------------------------------------------- construction ---
    void init(const Config& c, const EnergyTables& t, const std::vector<ChainInit>& config) {
        cfg = c;
        tab = t;
        ident_to_index.assign(cfg.identities.size(), {});
        attempts.assign(cfg.move_kinds.size(), 0);
        accepts.assign(cfg.move_kinds.size(), 0);
        touch_dom.assign(cfg.move_kinds.size(), 0);
        touch_site.assign(cfg.move_kinds.size(), 0);
        // initialize_scaffold (src/origami_system.cpp:680)
        add_chain_with_index(config[0].identity, config[0].index);
        num_staples--;
        if (cfg.cyclic) {
            auto& sc = chains[0];
            doms[sc.back()].fwd = sc.front();
            doms[sc.front()].bwd = sc.back();
        }
        // initialize_staples (src/origami_system.cpp:659)
        for (size_t i = 1; i < config.size(); ++i) add_chain_with_index(config[i].identity, config[i].index);
        if (cfg.mean_field) energy += (config.size() - 1) * std::log(6);
        energy += (chains.size() - 1) * tab.init_e;
        current_c_i = chain_index[0];
        for (int ci : chain_index) current_c_i = std::max(current_c_i, ci);
        // set_all_domains(config) (src/origami_system.cpp:588)
        for (size_t i = 0; i < config.size(); ++i)
            for (size_t d = 0; d < chains[i].size(); ++d) {
                doms[chains[i][d]].pos = config[i].pos[d];
                doms[chains[i][d]].ore = config[i].ore[d];
            }
        set_all_current();
    }

    void set_all_current() {
        for (size_t i = 0; i < chains.size(); ++i)
            for (int id : chains[i]) {
                set_domain_config(id, doms[id].pos, doms[id].ore);
                if (violated) throw std::runtime_error("Constaints in violation after move complete");
            }
        for (auto& ch : chains)
            for (int id : ch) {
                int nx = next(id, 1);
                if (nx >= 0 && (doms[nx].pos - doms[id].pos).abssum() != 1)
                    throw std::runtime_error("Contiguous domains not on adjacent sites");
            }
    }

    // ------------------------------------------------------ accessors ---
    int next(int id, int incr) const {   // Domain::operator+ (src/domain.cpp:9)
        while (id >= 0 && incr > 0) { id = doms[id].fwd; --incr; }
        while (id >= 0 && incr < 0) { id = doms[id].bwd; ++incr; }
        return id;
    }
    int chain_pos(int c_i) const {
        for (size_t i = 0; i < chain_index.size(); ++i)
            if (chain_index[i] == c_i) return (int)i;
        throw std::runtime_error("no chain with index " + std::to_string(c_i));
    }
    const std::vector<int>& get_chain(int c_i) const { return chains[chain_pos(c_i)]; }
    int occupancy(const V3& p) const {
        auto it = sites.find(pos_key(p));
        return it == sites.end() ? UNASSIGNED : it->second.occ;
    }
    int unbound_at(const V3& p) const { return sites.at(pos_key(p)).unbound_dom; }
    int num_staples_of_ident(int t) const { return (int)ident_to_index[t].size(); }
    double hyb(int i, int j) const { return tab.hyb_e[tab.at(doms[i].dident, doms[j].dident)]; }
    double hyb_h(int i, int j) const { return tab.hyb_h[tab.at(doms[i].dident, doms[j].dident)]; }
    double hyb_s(int i, int j) const { return tab.hyb_s[tab.at(doms[i].dident, doms[j].dident)]; }
    double stack(int i, int j) const { return tab.stack_e[tab.at(doms[i].dident, doms[j].dident)]; }

    // --------------------------------------------------- chain add/del ---
    int add_chain_with_index(int ident, int c_i) {   // src/origami_system.cpp:402
        if (ident < 0 || ident >= (int)cfg.identities.size()) throw std::runtime_error("bad chain identity");
        ident_to_index[ident].push_back(c_i);
        chain_index.push_back(c_i);
        chain_ident.push_back(ident);
        const auto& ids = cfg.identities[ident];
        int len = (int)ids.size();
        chains.push_back({});
        num_staples++;
        int prev = -1;
        for (int d = 0; d < len; ++d) {
            int id;
            if (!free_doms.empty()) {
                id = free_doms.back();
                free_doms.pop_back();
            }
            else {
                id = (int)doms.size();
                doms.push_back({});
            }
            Dom dm {c_i, ident, d, ids[d], len};
            dm.bwd = prev;
            dm.fwd = -1;
            doms[id] = dm;
            if (prev >= 0) doms[prev].fwd = id;
            chains.back().push_back(id);
            prev = id;
            num_domains++;
            num_unassigned++;
        }
        return c_i;
    }
    int add_chain(int ident) {   // src/origami_system.cpp:387
        current_c_i += 1;
        if (cfg.mean_field) energy += std::log(6);
        energy += tab.init_e;
        return add_chain_with_index(ident, current_c_i);
    }
    void delete_chain(int c_i) {   // src/origami_system.cpp:445
        int k = chain_pos(c_i);
        int ident = chain_ident[k];
        auto& lst = ident_to_index[ident];
        lst.erase(std::find(lst.begin(), lst.end(), c_i));
        chain_index.erase(chain_index.begin() + k);
        chain_ident.erase(chain_ident.begin() + k);
        num_domains -= (int)chains[k].size();
        num_staples--;
        for (int id : chains[k]) {
            free_doms.push_back(id);
            num_unassigned--;
        }
        chains.erase(chains.begin() + k);
        if (cfg.mean_field) energy -= std::log(6);
        energy -= tab.init_e;
    }

    // ------------------------------------------------ state transitions ---
    // update_occupancies (src/origami_system.cpp:770)
    void update_occupancies(int i, const V3& p) {
        uint64_t key = pos_key(p);
        auto it = sites.find(key);
        int occ = it == sites.end() ? UNASSIGNED : it->second.occ;
        if (occ == UNBOUND) {
            int j = it->second.unbound_dom;
            num_bound += 1;
            int ns;
            if (doms[i].dident == -doms[j].dident) {
                ns = BOUND;
                num_fully += 1;
            }
            else {
                if (doms[i].c == doms[j].c) num_self += 1;
                ns = MISBOUND;
            }
            doms[i].state = ns;
            doms[j].state = ns;
            it->second = {ns, -1};
            doms[j].bound = i;
            doms[i].bound = j;
        }
        else if (occ == UNASSIGNED) {
            doms[i].state = UNBOUND;
            sites[key] = {UNBOUND, i};
        }
        else {
            throw std::runtime_error("Trying to bind to an already bound domain");
        }
    }

    // unassign_bound_domain (src/origami_system.cpp:741)
    double unassign_bound(int i) {
        int j = doms[i].bound;
        double de = -hyb(i, j);
        doms[i].bound = -1;
        doms[j].bound = -1;
        doms[i].state = UNASSIGNED;
        sites[pos_key(doms[i].pos)] = {UNBOUND, j};
        doms[j].state = UNBOUND;
        return de;
    }

    // internal_unassign_domain (src/origami_system.cpp:695)
    Delta internal_unassign(int i) {
        int occ = doms[i].state;
        int j = doms[i].bound;
        Delta dc;
        switch (occ) {
        case BOUND:
            num_fully -= 1;
            num_bound -= 1;
            dc = check_stacking(i, j);
            dc.e *= -1;
            dc.stacked *= -1;
            dc.e += unassign_bound(i);
            break;
        case MISBOUND:
            num_bound -= 1;
            if (doms[j].c == doms[i].c) num_self -= 1;
            dc.e += unassign_bound(i);
            break;
        case UNBOUND:
            sites.erase(pos_key(doms[i].pos));
            doms[i].state = UNASSIGNED;
            break;
        case UNASSIGNED:
            num_unassigned--;
            break;
        }
        if (cfg.mean_field && occ == BOUND) {
            if (num_fully == 0) dc.e -= 2 * std::log(6);
            else if (num_fully == 1) dc.e -= std::log(3);
        }
        return dc;
    }

    // internal_check_domain_constraints (src/origami_system.cpp:828)
    Delta internal_check(int i, const V3& p, const V3& o) {
        int occ = occupancy(p);
        Delta dc;
        switch (occ) {
        case BOUND:
        case MISBOUND:
            violated = true;
            num_unassigned++;
            break;
        case UNBOUND:
            doms[i].pos = p;
            doms[i].ore = o;
            update_occupancies(i, p);
            dc = bind_domain(i);
            violated = pot_violated;
            break;
        case UNASSIGNED:
            doms[i].pos = p;
            doms[i].ore = o;
            update_occupancies(i, p);
            break;
        }
        if (cfg.mean_field && !violated && doms[i].state == BOUND) {
            if (num_fully == 1) dc.e += 2 * std::log(6);
            else if (num_fully == 2) dc.e += std::log(3);
        }
        return dc;
    }

    // set_domain_config (src/origami_system.cpp:517)
    double set_domain_config(int i, V3 p, V3 o) {
        if (doms[i].state != UNASSIGNED) throw std::runtime_error("Trying to set an already assigned domain");
        Delta dc = internal_check(i, p, o);
        if (violated) {
            internal_unassign(i);
        }
        else {
            energy += dc.e;
            num_stacked += dc.stacked;
            num_unassigned--;
        }
        return dc.e;
    }

    // set_checked_domain_config (src/origami_system.cpp:478)
    double set_checked(int i, V3 p, V3 o) {
        doms[i].pos = p;
        doms[i].ore = o;
        update_occupancies(i, p);
        double de = 0;
        if (doms[i].state == MISBOUND) {
            de += hyb(i, doms[i].bound);
        }
        else if (doms[i].state == BOUND) {
            de += hyb(i, doms[i].bound);
            Delta dc = check_stacking(i, doms[i].bound);
            de += dc.e;
            num_stacked += dc.stacked;
        }
        if (cfg.mean_field && doms[i].state == BOUND) {
            if (num_fully == 1) de += 2 * std::log(6);
            else if (num_fully == 2) de += std::log(3);
        }
        energy += de;
        num_unassigned--;
        return de;
    }

    // unassign_domain (src/origami_system.cpp:375)
    double unassign_domain(int i) {
        Delta dc = internal_unassign(i);
        energy += dc.e;
        num_stacked += dc.stacked;
        num_unassigned++;
        return dc.e;
    }

    // check_domain_constraints (src/origami_system.cpp:343)
    double check_domain_constraints(int i, V3 p, V3 o) {
        Delta dc = internal_check(i, p, o);
        internal_unassign(i);
        return dc.e;
    }

    // set_domain_orientation (src/origami_system.cpp:543)
    void set_domain_orientation(int i, V3 o) {
        if (doms[i].state == BOUND) violated = true;
        else doms[i].ore = o;
    }

    // center (src/origami_system.cpp:553)
    void center(int cd) {
        V3 ref = doms[chains[0][cd]].pos;
        std::unordered_map<uint64_t, SiteRec> ns;
        for (auto& ch : chains)
            for (int id : ch) {
                V3 np = doms[id].pos - ref;
                auto it = sites.find(pos_key(doms[id].pos));
                if (it != sites.end()) ns[pos_key(np)] = it->second;
                else ns[pos_key(np)] = {UNASSIGNED, -1};
                doms[id].pos = np;
            }
        sites.clear();
        for (auto& kv : ns)
            if (kv.second.occ != UNASSIGNED) sites.insert(kv);
    }

    // check_all_constraints (src/origami_system.cpp:267)
    void check_all_constraints() {
        if (num_unassigned != 0) throw std::runtime_error("Number of unassigned domains is no zero on constraint check");
        for (size_t c = 0; c < chains.size(); ++c)
            for (int id : chains[c]) {
                if (doms[id].state == UNASSIGNED) throw std::runtime_error("Domain unassigned after move complete");
                unassign_domain(id);
            }
        if (cfg.mean_field) energy -= (chains.size() - 1) * std::log(6);
        energy -= (chains.size() - 1) * tab.init_e;
        if (num_stacked != 0) {
            int sp = num_stacked;
            set_all_current();
            throw std::runtime_error("Stack count inconsistency: " + std::to_string(sp));
        }
        double eps = 0.000001;
        if (energy < -eps || energy > eps) {
            double e = energy;
            set_all_current();
            throw std::runtime_error("System energy inconsistency: " + std::to_string(e));
        }
        energy = 0;
        set_all_current();
        if (cfg.mean_field) energy += (chains.size() - 1) * std::log(6);
        energy += (chains.size() - 1) * tab.init_e;
    }

    // update_energy (src/origami_system.cpp:808), after a table change
    void recompute_energy() {
        for (size_t c = 0; c < chains.size(); ++c)
            for (int id : chains[c]) unassign_domain(id);
        energy = 0;
        if (cfg.mean_field) energy += (chains.size() - 1) * std::log(6);
        energy += (chains.size() - 1) * tab.init_e;
        set_all_current();
    }

    // update_enthalpy_and_entropy (src/origami_system.cpp:204)
    void enthalpy_entropy(double& H, double& S, double& stacking) const {
        H = 0;
        S = 0;
        std::set<int> acc;
        for (auto& ch : chains)
            for (int id : ch) {
                int st = doms[id].state;
                if (st == BOUND || st == MISBOUND) {
                    if (acc.find(id) == acc.end()) {
                        int b = doms[id].bound;
                        H += hyb_h(id, b);
                        S += hyb_s(id, b);
                        acc.insert(b);
                    }
                }
            }
        if (cfg.mean_field) {
            S -= (chains.size() - 1) * std::log(6);
            if (num_fully >= 1) S -= 2 * std::log(6);
            if (num_fully >= 2) S -= std::log(3);
        }
        H += (chains.size() - 1) * tab.init_h;
        S += (chains.size() - 1) * tab.init_s;
        stacking = energy - (H - S);
    }

    // ================================================== FourBody potential ===
    // JunctionBindingPotential, src/origami_potential.cpp:51-934.
    bool pot_violated {false};
    Delta pd;   // m_delta_config

    bool exists_bound(int id) const { return id >= 0 && doms[id].state == BOUND; }

    bool twist_ok(int i1, V3 ndr, int i2) const {   // src/domain.cpp:33,69
        V3 r = cfg.three_quarter ? rotate_quarter(doms[i1].ore, ndr, -1) : rotate_half(doms[i1].ore, ndr);
        return r == doms[i2].ore;
    }
    bool kink_ok(int i1, V3 ndr, int i2) const {   // src/domain.cpp:42,80
        const V3& o1 = doms[i1].ore;
        const V3& o2 = doms[i2].ore;
        if (ndr == -o1) return false;
        if (ndr == o1) {
            if (cfg.three_quarter) return !(o1 == o2 || o1 == -o2);
            return !(o2 == -o1);
        }
        if (ndr == o2 || ndr == -o2) return false;
        return true;
    }
    bool junction_ok(int j1, int j2, int j3, int j4, int k1, int k2) const {   // src/domain.cpp:59,99
        (void)j3;
        (void)j4;
        if (!cfg.three_quarter) return true;
        V3 ndr_k = doms[k2].pos - doms[k1].pos;
        if (ndr_k == doms[k1].ore) {
            V3 ndr1 = doms[j2].pos - doms[j1].pos;
            if (doms[j1].d > doms[j2].d) ndr1 = -ndr1;
            if (!twist_ok(k1, ndr1, k2)) return false;
        }
        return true;
    }
    bool doubly_contig(int a, int b) const {   // :51
        if (doms[a].c != doms[b].c || doms[b].d != doms[a].d + 1) return false;
        int ba = doms[a].bound, bb = doms[b].bound;
        if (doms[ba].c != doms[bb].c) return false;
        return std::abs(doms[bb].d - doms[ba].d) == 1;
    }
    bool pair_stacked(int a, int b) const {   // :70
        if (doms[a].d > doms[b].d) std::swap(a, b);
        V3 ndr = doms[b].pos - doms[a].pos;
        if (ndr != doms[a].ore && ndr != -doms[a].ore) return twist_ok(a, ndr, b);
        return false;
    }
    int junction_penalty(int j1, int j2, int j3, int j4, int k1, int k2) const {   // :85
        V3 ndr_k = doms[k2].pos - doms[k1].pos;
        if (!(ndr_k == doms[k1].ore)) return 0;
        V3 n1 = doms[j2].pos - doms[j1].pos;
        if (doms[j1].d > doms[j2].d) n1 = -n1;
        V3 n3 = doms[j4].pos - doms[j3].pos;
        if (doms[j3].d > doms[j4].d) n3 = -n3;
        if (n1 == n3) return 2;
        if (n1 == -n3) return 0;
        return 1;
    }
    void triplet_single(int h1, int h2, int h3) {   // :158
        V3 n1 = doms[h2].pos - doms[h1].pos;
        if (n1 == doms[h1].ore) return;
        V3 n2 = doms[h3].pos - doms[h2].pos;
        if (n1 != n2) {
            pd.e -= stack(h2, h3);
            pd.stacked -= 1;
        }
    }
    void triplet_double(int h1, int h2, int h3) {   // :181
        V3 n1 = doms[h2].pos - doms[h1].pos;
        V3 n2 = doms[h3].pos - doms[h2].pos;
        if (n1 != n2) {
            pd.e -= stack(h1, h2) / 2;
            pd.e -= stack(h2, h3) / 2;
            pd.stacked -= 1;
        }
    }
    void triply_contig_helix(int h1, int h2, int h3) {   // :200
        V3 n1 = doms[h2].pos - doms[h1].pos;
        V3 n2 = doms[h3].pos - doms[h2].pos;
        if (n1 != n2) pot_violated = true;
    }

    void stacking_and_steric(int i, int j) {   // :212
        int jj = 0;
        for (int cd : {i, j}) {
            constraints_around(cd, jj);
            if (pot_violated) return;
            jj++;
        }
        central_triplets(i, j);
    }

    void constraints_around(int cd, int jj) {   // :231
        for (int k : {-1, 0}) {
            int c1 = next(cd, k);
            int c2 = next(cd, k + 1);
            if (!(exists_bound(c1) && exists_bound(c2))) continue;
            int b1 = doms[c1].bound, b2 = doms[c2].bound;
            if (doms[b1].c == doms[b2].c) {
                if (doms[b1].d == doms[b2].d - 1) doubly_contig_helix_pair(c1, c2, k, jj);
                else if (doms[b1].d == doms[b2].d + 1) doubly_contig_junction_pair(c1, c2, jj);
                else regular_pair(c1, c2, k);
            }
            else {
                regular_pair(c1, c2, k);
            }
            if (pot_violated) return;
        }
        int prev = next(cd, -1);
        int forw = next(cd, 1);
        if (exists_bound(prev) && exists_bound(forw)) {
            if (pair_stacked(cd, forw)) {
                if (pair_stacked(prev, cd)) {
                    if (doubly_contig(prev, cd) && doubly_contig(cd, forw)) {
                        triply_contig_helix(prev, cd, forw);
                        if (pot_violated) return;
                    }
                    triplet_double(prev, cd, forw);
                }
                else {
                    triplet_single(prev, cd, forw);
                }
            }
        }
    }

    void regular_pair(int c1, int c2, int k) {   // :288
        V3 ndr = doms[c2].pos - doms[c1].pos;
        if (!kink_ok(c1, ndr, c2)) {
            pot_violated = true;
            return;
        }
        if (pair_stacked(c1, c2)) {
            pd.e += stack(c1, c2);
            pd.stacked += 1;
            if (k == -1) backward_single_junction(c1, c2);
            else forward_single_junction(c1, c2);
        }
        else {
            central_single_junction(c1, c2);
        }
        if (k == -1) backward_triplets(c1, c2);
        else forward_triplets(c1, c2);
    }

    void doubly_contig_helix_pair(int c1, int c2, int k, int jj) {   // :322
        if (jj == 1) return;
        V3 ndr = doms[c2].pos - doms[c1].pos;
        if (ndr == doms[c1].ore || ndr == -doms[c1].ore) {
            pot_violated = true;
            return;
        }
        if (twist_ok(c1, ndr, c2)) {
            pd.e += stack(c1, c2);
            pd.stacked += 1;
        }
        else {
            pot_violated = true;
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

    void doubly_contig_junction_pair(int c1, int c2, int jj) {   // :359
        int k1 = c1, k2 = c2;
        V3 ndr = doms[k2].pos - doms[k1].pos;
        if (doms[k1].ore != ndr) {
            pot_violated = true;
            return;
        }
        if (jj == 1) return;
        int sel[2][2] = {{next(c1, -1), c1}, {next(doms[c1].bound, 1), doms[c1].bound}};
        for (auto& s : sel) {
            int j1 = s[0], j2 = s[1];
            int j3 = k2, j4 = next(k2, 1);
            if (exists_bound(j4) && exists_bound(j1)) junction(j1, j2, j3, j4, k1, k2);
            j3 = doms[k2].bound;
            j4 = next(j3, -1);
            if (exists_bound(j4) && exists_bound(j1)) junction(j1, j2, j3, j4, k1, k2);
        }
    }

    void junction(int j1, int j2, int j3, int j4, int k1, int k2) {   // :419
        if (doms[k1].d > doms[k2].d) {
            std::swap(k1, k2);
            std::swap(j1, j4);
            std::swap(j2, j3);
        }
        if (!(pair_stacked(j1, j2) && pair_stacked(j3, j4))) return;
        if (!junction_ok(j1, j2, j3, j4, k1, k2)) {
            pot_violated = true;
            return;
        }
        int pen = junction_penalty(j1, j2, j3, j4, k1, k2);
        if (pen == 1) {
            pd.e -= stack(j1, j2) / 2;
            pd.e -= stack(j3, j4) / 2;
            pd.stacked -= 1;
        }
        else if (pen == 2) {
            pd.e -= stack(j1, j2);
            pd.e -= stack(j3, j4);
            pd.stacked -= 2;
        }
    }

    void backward_triplets(int c1, int c2) {   // :464
        int h2 = c1, h3 = c2;
        if (!pair_stacked(h2, h3)) return;
        int h1 = next(c1, -1);
        bool h23_dc = doubly_contig(h2, h3);
        if (exists_bound(h1)) {
            bool h12_dc = doubly_contig(h1, h2);
            if (pair_stacked(h1, h2)) {
                if (h12_dc && h23_dc) {
                    triply_contig_helix(h1, h2, h3);
                    if (pot_violated) return;
                }
                triplet_double(h1, h2, h3);
            }
            else {
                triplet_single(h1, h2, h3);
            }
        }
        int h2_prev = h1;
        int b1 = doms[c1].bound;
        h1 = next(b1, 1);
        if (exists_bound(h1) && doms[h1].bound != h2_prev && doms[h1].bound != h3) {
            if (pair_stacked(b1, h1)) triplet_double(h1, h2, h3);
        }
        h1 = next(b1, -1);
        if (exists_bound(h1) && doms[h1].bound != h2_prev && doms[h1].bound != h3) {
            if (pair_stacked(h1, b1)) triplet_double(h1, h2, h3);
            else triplet_single(h1, b1, h3);
        }
    }

    void forward_triplets(int c1, int c2) {   // :521
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
                    if (pot_violated) return;
                }
                triplet_double(h1, h2, h3);
            }
            else if (second) {
                triplet_single(h1, h2, h3);
            }
        }
        int h2_next = h3;
        int b2 = doms[c2].bound;
        h3 = next(b2, 1);
        if (exists_bound(h3) && doms[h3].bound != h2_next && doms[h3].bound != h1) {
            if (pair_stacked(b2, h3)) {
                if (first) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
        }
        h3 = next(b2, -1);
        if (exists_bound(h3) && doms[h3].bound != h2_next && doms[h3].bound != h1) {
            if (pair_stacked(h3, b2)) {
                if (first) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
            else if (first) {
                triplet_single(h3, b2, h1);
            }
        }
    }

    void central_triplets(int i, int j) {   // :587
        int h1 = next(i, -1);
        int h2 = i;
        int h3 = next(j, 1);
        int h2_next = next(i, 1);
        if (exists_bound(h1) && exists_bound(h3) && doms[h3].bound != h2_next && !doubly_contig(h1, h2)) {
            if (pair_stacked(j, h3)) {
                if (pair_stacked(h1, h2)) triplet_double(h1, h2, h3);
                else triplet_single(h1, h2, h3);
            }
        }
        h3 = next(j, -1);
        if (exists_bound(h1) && exists_bound(h3) && doms[h3].bound != h1 && !doubly_contig(h1, h2)) {
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
        if (exists_bound(h1) && exists_bound(h3) && doms[h1].bound != h3 && !doubly_contig(h2, h3)) {
            if (pair_stacked(j, h1) && pair_stacked(h2, h3)) triplet_double(h1, h2, h3);
        }
        h1 = next(j, -1);
        if (exists_bound(h1) && exists_bound(h3) && doms[h1].bound != h2_prev && !doubly_contig(h2, h3)) {
            if (pair_stacked(h2, h3)) {
                if (pair_stacked(h1, j)) triplet_double(h1, h2, h3);
                else triplet_single(h1, j, h3);
            }
        }
    }

    void backward_single_junction(int c1, int c2) {   // :654
        int j3 = c1, j4 = c2;
        int first[3][2];
        int nf = 0;
        int j3_bac = doms[j3].bwd;
        first[nf][0] = j3;
        first[nf][1] = j3_bac;
        nf++;
        int j3_b = doms[j3].bound;
        int j3_b_for = doms[j3_b].fwd;
        int j3_b_bac = doms[j3_b].bwd;
        if (j3_b_for == doms[j4].bound) {
            first[nf][0] = j3_b; first[nf][1] = j3_b_bac; nf++;
        }
        else if (exists_bound(j3_bac) && exists_bound(j3_b_bac) && doms[j3_bac].bound == j3_b_bac) {
            first[nf][0] = j3_b; first[nf][1] = j3_b_for; nf++;
        }
        else if (exists_bound(j3_bac) && exists_bound(j3_b_for) && doms[j3_bac].bound == j3_b_for) {
            first[nf][0] = j3_b; first[nf][1] = j3_b_bac; nf++;
        }
        else {
            first[nf][0] = j3_b; first[nf][1] = j3_b_for; nf++;
            first[nf][0] = j3_b; first[nf][1] = j3_b_bac; nf++;
        }
        for (int a = 0; a < nf; ++a) {
            int k2 = first[a][0], k1 = first[a][1];
            if (!exists_bound(k1)) continue;
            if (pair_stacked(k1, k2)) continue;
            int second[3][2];
            int ns = 0;
            int dir = doms[k1].d - doms[k2].d;
            int k1_next = next(k1, dir);
            second[ns][0] = k1; second[ns][1] = k1_next; ns++;
            int k1_b = doms[k1].bound;
            int k1_b_for = doms[k1_b].fwd, k1_b_bac = doms[k1_b].bwd;
            if (exists_bound(k1_next)) {
                int kn_b = doms[k1_next].bound;
                if (k1_b_for != kn_b) { second[ns][0] = k1_b; second[ns][1] = k1_b_for; ns++; }
                if (k1_b_bac != kn_b) { second[ns][0] = k1_b; second[ns][1] = k1_b_bac; ns++; }
            }
            else {
                second[ns][0] = k1_b; second[ns][1] = k1_b_for; ns++;
                second[ns][0] = k1_b; second[ns][1] = k1_b_bac; ns++;
            }
            for (int b = 0; b < ns; ++b) {
                int j2 = second[b][0], j1 = second[b][1];
                if (!exists_bound(j1)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    void forward_single_junction(int c1, int c2) {   // :750
        int j1 = c1, j2 = c2;
        int first[3][2];
        int nf = 0;
        int j2_for = doms[j2].fwd;
        first[nf][0] = j2; first[nf][1] = j2_for; nf++;
        int j1_b = doms[j1].bound;
        int j2_b = doms[j2].bound;
        int j2_b_for = doms[j2_b].fwd, j2_b_bac = doms[j2_b].bwd;
        if (next(j1_b, 1) == j2_b) {
            first[nf][0] = j2_b; first[nf][1] = j2_b_for; nf++;
        }
        else if (exists_bound(j2_for) && exists_bound(j2_b_bac) && doms[j2_for].bound == j2_b_bac) {
            first[nf][0] = j2_b; first[nf][1] = j2_b_for; nf++;
        }
        else if (exists_bound(j2_for) && exists_bound(j2_b_for) && doms[j2_for].bound == j2_b_for) {
            first[nf][0] = j2_b; first[nf][1] = j2_b_bac; nf++;
        }
        else {
            first[nf][0] = j2_b; first[nf][1] = j2_b_for; nf++;
            first[nf][0] = j2_b; first[nf][1] = j2_b_bac; nf++;
        }
        for (int a = 0; a < nf; ++a) {
            int k1 = first[a][0], k2 = first[a][1];
            if (!exists_bound(k2)) continue;
            if (pair_stacked(k1, k2)) continue;
            int second[3][2];
            int ns = 0;
            int dir = doms[k2].d - doms[k1].d;
            int k2_next = next(k2, dir);
            second[ns][0] = k2; second[ns][1] = k2_next; ns++;
            int k2_b = doms[k2].bound;
            int k2_b_for = doms[k2_b].fwd, k2_b_bac = doms[k2_b].bwd;
            if (exists_bound(k2_next)) {
                int kn_b = doms[k2_next].bound;
                if (k2_b_for != kn_b) { second[ns][0] = k2_b; second[ns][1] = k2_b_for; ns++; }
                if (k2_b_bac != kn_b) { second[ns][0] = k2_b; second[ns][1] = k2_b_bac; ns++; }
            }
            else {
                second[ns][0] = k2_b; second[ns][1] = k2_b_for; ns++;
                second[ns][0] = k2_b; second[ns][1] = k2_b_bac; ns++;
            }
            for (int b = 0; b < ns; ++b) {
                int j3 = second[b][0], j4 = second[b][1];
                if (!exists_bound(j4)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    void central_single_junction(int c1, int c2) {   // :846
        int k1 = c1, k2 = c2;
        int kb1 = doms[k1].bound, kb2 = doms[k2].bound;
        if (doms[kb1].c == doms[kb2].c && std::abs(doms[kb1].d - doms[kb2].d) == 1) return;
        int first[3][2];
        int nf = 0;
        int k1_bac = doms[k1].bwd;
        first[nf][0] = k1; first[nf][1] = k1_bac; nf++;
        int k1_b = kb1;
        int k1_b_for = doms[k1_b].fwd, k1_b_bac = doms[k1_b].bwd;
        if (exists_bound(k1_bac)) {
            int kbb = doms[k1_bac].bound;
            if (k1_b_for != kbb) { first[nf][0] = k1_b; first[nf][1] = k1_b_for; nf++; }
            if (k1_b_bac != kbb) { first[nf][0] = k1_b; first[nf][1] = k1_b_bac; nf++; }
        }
        else {
            first[nf][0] = k1_b; first[nf][1] = k1_b_for; nf++;
            first[nf][0] = k1_b; first[nf][1] = k1_b_bac; nf++;
        }
        for (int a = 0; a < nf; ++a) {
            int j2 = first[a][0], j1 = first[a][1];
            if (!exists_bound(j1)) continue;
            int second[3][2];
            int ns = 0;
            int k2_for = doms[k2].fwd;
            second[ns][0] = k2; second[ns][1] = k2_for; ns++;
            int k2_b = kb2;
            int k2_b_for = doms[k2_b].fwd, k2_b_bac = doms[k2_b].bwd;
            if (exists_bound(k2_for)) {
                int kfb = doms[k2_for].bound;
                if (k2_b_for != kfb) { second[ns][0] = k2_b; second[ns][1] = k2_b_for; ns++; }
                if (k2_b_bac != kfb) { second[ns][0] = k2_b; second[ns][1] = k2_b_bac; ns++; }
            }
            else {
                second[ns][0] = k2_b; second[ns][1] = k2_b_for; ns++;
                second[ns][0] = k2_b; second[ns][1] = k2_b_bac; ns++;
            }
            for (int b = 0; b < ns; ++b) {
                int j3 = second[b][0], j4 = second[b][1];
                if (!exists_bound(j4)) continue;
                junction(j1, j2, j3, j4, k1, k2);
            }
        }
    }

    // BindingPotential::bind_domains (:131) / check_stacking (:149),
    // OrigamiPotential::bind_domain (:1282), misbinding (:938, :947)
    Delta bind_domain(int i) {
        pot_violated = false;
        int j = doms[i].bound;
        Delta dc;
        if (doms[i].dident == -doms[j].dident) {
            pd = {};
            if (doms[i].ore != -doms[j].ore) {
                pot_violated = true;
                return {};
            }
            stacking_and_steric(i, j);
            if (pot_violated) return {};
            pd.e += hyb(i, j);
            dc = pd;
        }
        else {
            if (cfg.misbinding_disallowed) {
                pot_violated = true;
                return dc;
            }
            pot_violated = true;
            if (doms[i].ore != -doms[j].ore) return dc;
            pot_violated = false;
            dc.e += hyb(i, j);
        }
        return dc;
    }
    Delta check_stacking(int i, int j) {
        pd = {};
        pot_violated = false;
        stacking_and_steric(i, j);
        return pd;
    }

    // =========================================== order params / biases ===
    // SystemOrderParams::update_move_params (src/order_params.cpp:595)
    void update_move_params() {
        for (auto& op : ops) {
            switch (op.kind) {
            case OP_NUMSTAPLES: op.param = num_staples; break;
            case OP_NUMSTAPLESTYPE: op.param = num_staples_of_ident(op.arg); break;
            case OP_STAPLETYPEFULLYBOUND: {
                op.param = 0;
                for (int c_i : ident_to_index[op.arg]) {
                    bool full = true;
                    for (int id : get_chain(c_i))
                        if (doms[id].state != BOUND) { full = false; break; }
                    if (full) { op.param = 1; break; }
                }
                break;
            }
            case OP_NUMBOUND: op.param = num_fully; break;
            case OP_NUMMISBOUND: op.param = num_bound - num_fully; break;
            case OP_NUMSTACKED: op.param = num_stacked; break;
            case OP_NUMLINEARHELICES: op.param = 0; break;
            case OP_NUMSTACKEDJUNCTS: op.param = 0; break;
            case OP_SUM: {
                int s = 0;
                op.defined = true;
                for (int p : op.parts) {
                    if (ops[p].defined) s += ops[p].param;
                    else { op.defined = false; s = op.param; break; }
                }
                op.param = s;
                break;
            }
            case OP_DIST:            // DistOrderParam::calc_param (src/order_params.cpp:35)
            case OP_ADJACENT: {      // AdjacentSiteOrderParam::calc_param (:84)
                const Dom& a = doms[chains[0][op.parts[0]]];
                const Dom& b = doms[chains[0][op.parts[1]]];
                if (a.state != UNASSIGNED && b.state != UNASSIGNED) {
                    op.defined = true;
                    int l1 = (b.pos - a.pos).abssum();
                    op.param = op.kind == OP_DIST ? l1 : (l1 == 1 ? 1 : 0);
                }
                else {
                    op.defined = false;
                }
                break;
            }
            }
        }
    }

    double bias_value(BiasRec& b) {
        for (int o : b.ops)
            if (!ops[o].defined) return 0;
        int x = ops[b.ops[0]].param;
        switch (b.kind) {
        case B_LINEARSTEPWELL:   // src/bias_functions.cpp:139
            if (x < b.min_op) return b.slope * (b.min_op - x - 1) + b.min_bias;
            if (x > b.max_op) return b.slope * (x - b.max_op - 1) + b.min_bias;
            return b.well_bias;
        case B_SQUAREWELL:   // :194
            if (x < b.min_op || x > b.max_op) return b.outside_bias;
            return b.well_bias;
        case B_GRID:   // :242
            if (x >= 0 && x < (int)b.grid.size() && b.grid_set) return b.grid[x];
            return b.off_grid;
        case B_HARMONIC: {
            double dx = x - b.centre;
            return 0.5 * b.k * dx * dx;
        }
        }
        return 0;
    }

    // SystemBiases::calc_move (src/bias_functions.cpp:475)
    double calc_move() {
        double diff = 0;
        for (auto& b : biases) {
            double prev = b.bias;
            double nb = bias_value(b);
            b.bias = nb;
            diff += nb - prev;
        }
        move_bias += diff;
        return diff * cfg.bias_mult;
    }
    double total_bias() const { return move_bias * cfg.bias_mult; }

    void init_biases() {
        update_move_params();
        move_bias = 0;
        for (auto& b : biases) {
            b.bias = bias_value(b);
            move_bias += b.bias;
        }
    }

    // ================================================================ moves ===
    // MCMovetype bookkeeping (include/.../movetypes.hpp:141-169)
    struct Key { int c, d; };
    std::vector<Key> modified, assigned;
    std::vector<V3> prev_pos, prev_ore;   // parallel to `modified`
    std::vector<int> added;
    bool rejected {false};
    double modifier {1};
    double delta_e {0};
    // CB state (include/.../cb_movetypes.hpp:126-130)
    Wt w_bias, w_new_bias;
    double new_modifier {1};
    // The reference's own arithmetic (long double Rosenbluth weights and the
    // C library's exp) instead of the engine's (FP64, ldo_math::exp).
    bool ld_weights {false};
    double xexp(double x) const { return ld_weights ? xexp(x) : ldo_math::exp(x); }
    bool regrow_old {false};
    std::vector<Key> old_keys;
    std::vector<V3> old_pos, old_ore;

    int dom_of(Key k) const { return get_chain(k.c)[k.d]; }
    Key key_of(int id) const { return {doms[id].c, doms[id].d}; }

    void reset_internal() {   // src/movetypes.cpp:242
        modified.clear();
        assigned.clear();
        prev_pos.clear();
        prev_ore.clear();
        added.clear();
        rejected = false;
        modifier = 1;
        delta_e = 0;
        w_bias.ld = w_new_bias.ld = ld_weights;
        w_bias.set(1);
        w_new_bias.set(1);
        new_modifier = 1;
        regrow_old = false;
    }

    void reset_origami() {   // src/movetypes.cpp:53
        for (auto& k : assigned) unassign_domain(dom_of(k));
        for (int c_i : added) {
            delete_chain(c_i);
            current_c_i -= 1;
        }
        for (size_t n = 0; n < modified.size(); ++n) set_checked(dom_of(modified[n]), prev_pos[n], prev_ore[n]);
        violated = false;
    }

    bool test_acceptance(double p) {   // src/movetypes.cpp:142
        double pa = std::fmin(1.0, p) * modifier;
        if (pa == 1) return true;
        return pa > rng.uniform_real();
    }

    int select_random_domain() {   // src/movetypes.cpp:98
        int idx = rng.uniform_int(0, num_domains - 1);
        int cnt = 0;
        for (auto& ch : chains)
            for (int id : ch) {
                if (cnt == idx) return id;
                cnt++;
            }
        return -1;
    }

    bool staple_is_connector(const std::vector<int>& st) {   // src/movetypes.cpp:160
        for (int id : st) {
            if (doms[id].state != UNBOUND) {
                int b = doms[id].bound;
                if (doms[b].c == scaffold_c()) continue;
                std::set<int> part {doms[id].c};
                if (!scan_for_scaffold(b, part)) return true;
            }
        }
        return false;
    }
    bool scan_for_scaffold(int dom, std::set<int>& part) {   // src/movetypes.cpp:191
        int c_i = doms[dom].c;
        part.insert(c_i);
        std::vector<int> st = get_chain(c_i);
        for (int cur : st) {
            if (cur == dom) continue;
            int b = doms[cur].bound;
            if (b >= 0) {
                if (doms[b].c == doms[dom].c) continue;
                if (doms[b].c == scaffold_c()) return true;
                if (part.count(doms[b].c) > 0) continue;
                if (scan_for_scaffold(b, part)) return true;
            }
        }
        return false;
    }
    int scaffold_c() const { return 0; }

    int num_bound_staple_domains(const std::vector<int>& st) const {   // src/movetypes.cpp:395
        int n = 0;
        for (int id : st)
            if (doms[id].state == BOUND || doms[id].state == MISBOUND) n++;
        return n;
    }

    std::vector<std::pair<int, int>> find_bound_domains(const std::vector<int>& st) const {   // :258
        std::vector<std::pair<int, int>> out;
        int c = doms[st[0]].c;
        for (int id : st)
            if (doms[id].bound >= 0 && doms[doms[id].bound].c != c) out.push_back({id, doms[id].bound});
        if (out.empty()) throw std::runtime_error("System has unbound staple");
        return out;
    }

    void unassign_domains(const std::vector<int>& st) {   // src/met_movetypes.cpp:77, src/cb_movetypes.cpp:200
        for (int id : st) {
            modified.push_back(key_of(id));
            prev_pos.push_back(doms[id].pos);
            prev_ore.push_back(doms[id].ore);
            double de = unassign_domain(id);
            delta_e += de;
        }
    }

    // RegrowthMCMovetype::set_growth_point (src/movetypes.cpp:322)
    double set_growth_point(int gnew, int gold) {
        V3 o = -doms[gold].ore;
        double de = set_domain_config(gnew, doms[gold].pos, o);
        if (violated) rejected = true;
        else assigned.push_back(key_of(gnew));
        return de;
    }

    // MetMCMovetype::grow_chain (src/met_movetypes.cpp:50)
    void met_grow_chain(const std::vector<int>& ds) {
        for (size_t i = 1; i < ds.size(); ++i) {
            int id = ds[i], prev = ds[i - 1];
            V3 p = doms[prev].pos + kUnit[rng.uniform_int(0, 5)];
            V3 o = kUnit[rng.uniform_int(0, 5)];
            delta_e += set_domain_config(id, p, o);
            if (violated) {
                rejected = true;
                break;
            }
            assigned.push_back(key_of(id));
        }
    }

    // RegrowthMCMovetype::grow_staple (src/movetypes.cpp:343)
    void grow_staple(int d_i, const std::vector<int>& ch, bool cb) {
        std::vector<int> three(ch.begin() + d_i, ch.end());
        if (three.size() > 1) {
            if (cb) cb_grow_chain(three);
            else met_grow_chain(three);
        }
        if (rejected) return;
        std::vector<int> five(ch.begin(), ch.begin() + d_i + 1);
        std::reverse(five.begin(), five.end());
        if (five.size() > 1) {
            if (cb) cb_grow_chain(five);
            else met_grow_chain(five);
        }
    }

    double add_external_bias_met() {   // src/met_movetypes.cpp:69
        update_move_params();
        double b = calc_move();
        delta_e += b;
        return b;
    }

    // MetStapleExchangeMCMovetype (src/met_movetypes.cpp:192-403)
    int insertion_sites {0};
    bool staple_bound {false};

    bool exchange_accept_common(int ident, double pratio) {
        if (staple_bound) {
            modifier *= cfg.exchange_mults[ident - 1];
            if (modifier * std::fmin(1.0, pratio) > 1) {
                if (cfg.adaptive_exchange) {
                    cfg.exchange_mults[ident - 1] /= 10;
                    return false;
                }
                if (cfg.allow_nonsensical_ps) return true;
                throw std::runtime_error("Nonsensical exchange probability detected");
            }
            return test_acceptance(pratio);
        }
        return test_acceptance(pratio);
    }

    bool insert_staple() {
        int S = (int)cfg.identities.size() - 1;
        int ident = rng.uniform_int(1, S);
        if (num_staples == cfg.max_total_staples) return false;
        if (num_staples_of_ident(ident) == cfg.max_type_staples) return false;
        int c_i = add_chain(ident);
        if (cfg.mean_field) delta_e += std::log(6);
        delta_e += tab.init_e;
        added.push_back(c_i);
        std::vector<int> ch = chains.back();
        int gi = rng.uniform_int(0, (int)ch.size() - 1);
        int gnew = ch[gi];
        int gold = select_random_domain();
        long guard = 0;
        while (doms[gold].c == doms[gnew].c) {
            gold = select_random_domain();
            if (++guard > 100000000L) throw std::runtime_error("growth point selection did not terminate");
        }
        delta_e += set_growth_point(gnew, gold);
        if (rejected) return false;
        grow_staple(doms[gnew].d, ch, false);
        if (rejected) return false;
        std::vector<int> st = get_chain(c_i);
        for (int id : st)
            if (doms[id].state == BOUND) { staple_bound = true; break; }
        int nbd = num_bound_staple_domains(st);
        add_external_bias_met();
        double boltz = xexp(-delta_e);
        int ni = num_staples_of_ident(ident);
        size_t L = cfg.identities[ident].size();
        double pratio = static_cast<double>(L) / 6.0 / ni * boltz;
        pratio *= insertion_sites * cfg.staple_M;
        pratio /= nbd;
        return exchange_accept_common(ident, pratio);
    }

    bool delete_staple() {
        int S = (int)cfg.identities.size() - 1;
        int ident = rng.uniform_int(1, S);
        int n = num_staples_of_ident(ident);
        if (n == 0) {
            rejected = true;
            return false;
        }
        int c_i = ident_to_index[ident][rng.uniform_int(0, n - 1)];
        std::vector<int> st = get_chain(c_i);
        if (staple_is_connector(st)) return false;
        for (int id : st)
            if (doms[id].state == BOUND) { staple_bound = true; break; }
        int nbd = num_bound_staple_domains(st);
        unassign_domains(st);
        if (cfg.mean_field) delta_e -= std::log(6);
        delta_e -= tab.init_e;
        num_staples--;
        add_external_bias_met();
        num_staples++;
        double boltz = xexp(-delta_e);
        int ni = num_staples_of_ident(ident);
        size_t L = cfg.identities[ident].size();
        double pratio = ni * 6.0 / static_cast<double>(L) * boltz;
        pratio /= cfg.staple_M * (double)(size_t)(insertion_sites - L);
        pratio *= nbd;
        bool acc = exchange_accept_common(ident, pratio);
        if (acc) delete_chain(c_i);
        return acc;
    }

    bool met_exchange() {
        insertion_sites = num_domains;
        staple_bound = false;
        if (rng.uniform_real() < 0.5) return insert_staple();
        return delete_staple();
    }

    // ---------------------------- learned insertion proposal (engine only) ---
    // CPU restatement of the engine's LearnedStapleExchange (no reference
    // counterpart): the same targets, the same weights (the engine's table),
    // the same order of every sum, so trajectories agree exactly.
    const double* learn_w {nullptr};
    int learn_tb {0};

    int learn_code(int n, int fresh_c) const {
        if (n < 0) return 0;
        int s = doms[n].state;
        if (s == BOUND || s == MISBOUND) {
            if (fresh_c >= 0 && doms[doms[n].bound].c == fresh_c) return 1;
            return s == BOUND ? 2 : 3;
        }
        return 1;
    }
    // complementary staple type / domain of scaffold domain index k (0: none)
    std::pair<int, int> learn_comp(int k) const {
        int id = cfg.identities[0][k];
        for (size_t t = 1; t < cfg.identities.size(); ++t)
            for (size_t q = 0; q < cfg.identities[t].size(); ++q)
                if (cfg.identities[t][q] == -id) return {(int)t, (int)q};
        return {0, 0};
    }
    double learn_weight(int g, int fresh_c) const {
        int p1 = doms[g].bwd, n1 = doms[g].fwd;
        int p2 = p1 >= 0 ? doms[p1].bwd : -1;
        int n2 = n1 >= 0 ? doms[n1].fwd : -1;
        int combo = learn_code(p2, fresh_c) | (learn_code(p1, fresh_c) << 2) | (learn_code(n1, fresh_c) << 4) |
                    (learn_code(n2, fresh_c) << 6);
        int ts = doms[g].cident == 0 ? ldo_learn_tslot(learn_comp(doms[g].d).first) : 0;
        return learn_w[ldo_learn_index(learn_tb, ts, combo)];
    }
    double learn_z() const {
        double z = 0;
        for (int g : chains[0])
            if (doms[g].state == UNBOUND) z += learn_weight(g, -1);
        return z;
    }
    double learn_q_target(int g, double z, int n_sites, int fresh_c) const {
        if (z == 0) return 1.0 / n_sites;
        double q = LDO_LEARN_EPS / n_sites;
        if (doms[g].cident == 0) q += (1.0 - LDO_LEARN_EPS) * (learn_weight(g, fresh_c) / z);
        return q;
    }
    double learn_q_type(int g, int type, int d) const {
        int S = (int)cfg.identities.size() - 1;
        double u = 1.0 / ((double)S * cfg.identities[type].size());
        int ct = 0, cd = 0;
        if (doms[g].cident == 0) {
            auto cc = learn_comp(doms[g].d);
            ct = cc.first;
            cd = cc.second;
        }
        if (ct == 0) return u;
        double q = LDO_LEARN_EPS_T * u;
        if (ct == type && cd == d) q += 1.0 - LDO_LEARN_EPS_T;
        return q;
    }

    // learned deletion choice (the engine's del_weight / del_total / del_q)
    double del_weight(int c_i) const {
        for (int id : get_chain(c_i))
            if (doms[id].state != BOUND) return LDO_LEARN_DEL_PART;
        return 1.0;
    }
    double del_total() const {
        double u = 0;
        for (size_t c = 1; c < chains.size(); ++c) u += del_weight(doms[chains[c][0]].c);
        return u;
    }
    double del_q(int c_i, double u) const {
        return LDO_LEARN_EPS_DEL / (double)num_staples + (1.0 - LDO_LEARN_EPS_DEL) * (del_weight(c_i) / u);
    }

    bool learned_insert() {
        if (!learn_w) throw std::runtime_error("LearnedStapleExchange needs the weight table");
        int S = (int)cfg.identities.size() - 1;
        int n_sites = num_domains;
        double z = learn_z();
        int g = -1;
        double u1 = rng.uniform_real();
        if (z == 0 || u1 < LDO_LEARN_EPS) {
            g = select_random_domain();
        }
        else {
            double target = rng.uniform_real() * z;
            double cum = 0;
            int last = -1;
            for (int x : chains[0]) {
                if (doms[x].state != UNBOUND) continue;
                cum += learn_weight(x, -1);
                last = x;
                if (target < cum) {
                    g = x;
                    break;
                }
            }
            if (g < 0) g = last;
        }
        int ct = 0, cd = 0;
        if (doms[g].cident == 0) {
            auto cc = learn_comp(doms[g].d);
            ct = cc.first;
            cd = cc.second;
        }
        int ident, gi;
        double u3 = rng.uniform_real();
        if (ct != 0 && u3 < 1.0 - LDO_LEARN_EPS_T) {
            ident = ct;
            gi = cd;
        }
        else {
            ident = rng.uniform_int(1, S);
            gi = rng.uniform_int(0, (int)cfg.identities[ident].size() - 1);
        }
        if (num_staples == cfg.max_total_staples) return false;
        if (num_staples_of_ident(ident) == cfg.max_type_staples) return false;
        int c_i = add_chain(ident);
        if (cfg.mean_field) delta_e += std::log(6);
        delta_e += tab.init_e;
        added.push_back(c_i);
        std::vector<int> ch = chains.back();
        int gnew = ch[gi];
        delta_e += set_growth_point(gnew, g);
        if (rejected) return false;
        // the other domains grown with the learned direction proposal
        for (auto& gk : growth_order(gi, (int)ch.size())) {
            int i = ch[gk.first], prev = ch[gk.second];
            int v = 0;
            V3 o;
            lr_propose(i, prev, true, v, o);
            delta_e += set_domain_config(i, doms[prev].pos + kUnit[v], o);
            if (violated) {
                rejected = true;
                return false;
            }
            assigned.push_back(key_of(i));
        }
        std::vector<int> st = get_chain(c_i);
        for (int id : st)
            if (doms[id].state == BOUND) { staple_bound = true; break; }
        double f = 0;
        for (size_t d = 0; d < st.size(); ++d) {
            int b = st[d];
            int p = doms[b].bound;
            if (p < 0 || doms[p].c == c_i) continue;
            f += learn_q_target(p, z, n_sites, c_i) * learn_q_type(p, ident, (int)d) * lr_growth_literal(st, (int)d);
        }
        add_external_bias_met();
        double boltz = xexp(-delta_e);
        double qd = del_q(c_i, del_total());
        double pratio = boltz * cfg.staple_M;
        pratio *= qd;
        pratio /= 6.0 * f;
        return exchange_accept_common(ident, pratio);
    }

    bool learned_delete() {
        if (num_staples == 0) {
            rejected = true;
            return false;
        }
        double u_tot = del_total();
        int c_i = -1;
        if (rng.uniform_real() < LDO_LEARN_EPS_DEL) {
            c_i = doms[chains[rng.uniform_int(1, num_staples)][0]].c;
        }
        else {
            double target = rng.uniform_real() * u_tot;
            double cum = 0;
            for (size_t c = 1; c < chains.size(); ++c) {
                c_i = doms[chains[c][0]].c;
                cum += del_weight(c_i);
                if (target < cum) break;
            }
        }
        int ident = doms[chains[chain_pos(c_i)][0]].cident;
        double qd = del_q(c_i, u_tot);
        std::vector<int> st = get_chain(c_i);
        if (staple_is_connector(st)) return false;
        for (int id : st)
            if (doms[id].state == BOUND) { staple_bound = true; break; }
        std::vector<std::pair<int, int>> alt;   // (domain index, partner)
        std::vector<double> gf;                 // growth factor from that domain
        for (size_t d = 0; d < st.size(); ++d) {
            int p = doms[st[d]].bound;
            if (p < 0 || doms[p].c == c_i) continue;
            alt.push_back({(int)d, p});
            gf.push_back(lr_growth_literal(st, (int)d));
        }
        unassign_domains(st);
        if (cfg.mean_field) delta_e -= std::log(6);
        delta_e -= tab.init_e;
        num_staples--;
        add_external_bias_met();
        num_staples++;
        double boltz = xexp(-delta_e);
        int n_sites = insertion_sites - (int)st.size();
        double z = learn_z();
        double f = 0;
        for (size_t a = 0; a < alt.size(); ++a)
            f += learn_q_target(alt[a].second, z, n_sites, -1) * learn_q_type(alt[a].second, ident, alt[a].first) *
                 gf[a];
        double pratio = 6.0 * boltz;
        pratio *= f;
        pratio /= qd;
        pratio /= cfg.staple_M;
        bool acc = exchange_accept_common(ident, pratio);
        if (acc) delete_chain(c_i);
        return acc;
    }

    bool learned_exchange() {
        insertion_sites = num_domains;
        staple_bound = false;
        if (rng.uniform_real() < 0.5) return learned_insert();
        return learned_delete();
    }

    // ----------------------------- learned regrowth directions (engine only) ---
    // CPU restatement of the engine's LearnedStapleRegrowth: the same site
    // classes, weights (the engine's table), sums in the same order, draws at
    // the same points.
    int lr_site_class(int i, V3 p, V3* ob, bool* has_ob) const {
        *has_ob = false;
        int occ = occupancy(p);
        if (occ == UNASSIGNED) return 0;
        if (occ == UNBOUND) {
            int j = unbound_at(p);
            *ob = -doms[j].ore;
            *has_ob = true;
            return doms[i].dident == -doms[j].dident ? 1 : 2;
        }
        return 3;
    }
    double lr_propose(int i, int prev, bool sample, int& v, V3& o) {
        if (!learn_w) throw std::runtime_error("LearnedStapleRegrowth needs the weight table");
        double w[6];
        V3 ob[6];
        bool hob[6];
        double z = 0;
        for (int k = 0; k < 6; ++k) {
            int f = lr_site_class(i, doms[prev].pos + kUnit[k], &ob[k], &hob[k]);
            w[k] = learn_w[ldo_learn_dir_index(learn_tb, f)];
            z += w[k];
        }
        if (sample) {
            double r = rng.uniform_real();
            double cum = 0;
            v = 5;
            for (int k = 0; k < 6; ++k) {
                cum += z > 0 ? LDO_LEARN_EPS_D / 6.0 + (1.0 - LDO_LEARN_EPS_D) * (w[k] / z) : 1.0 / 6.0;
                if (r < cum) {
                    v = k;
                    break;
                }
            }
            if (hob[v]) {
                double r2 = rng.uniform_real();
                o = r2 < 1.0 - LDO_LEARN_EPS_O ? ob[v] : kUnit[rng.uniform_int(0, 5)];
            }
            else {
                o = kUnit[rng.uniform_int(0, 5)];
            }
        }
        double qv = z > 0 ? LDO_LEARN_EPS_D / 6.0 + (1.0 - LDO_LEARN_EPS_D) * (w[v] / z) : 1.0 / 6.0;
        double qo = hob[v] ? (o == ob[v] ? (1.0 - LDO_LEARN_EPS_O) + LDO_LEARN_EPS_O / 6.0 : LDO_LEARN_EPS_O / 6.0)
                           : 1.0 / 6.0;
        return qv * qo;
    }
    // Growth order of a staple of len domains from domain d0, as grow_staple
    // grows it: (domain index, previous domain index), forward to the end,
    // then backward to the start.
    static std::vector<std::pair<int, int>> growth_order(int d0, int len) {
        std::vector<std::pair<int, int>> g;
        for (int k = d0 + 1; k < len; ++k) g.push_back({k, k - 1});
        for (int k = d0 - 1; k >= 0; --k) g.push_back({k, k + 1});
        return g;
    }
    // Growth factor of staple st grown from its domain d0 by the learned
    // direction proposal: the product over the grown domains of 36 q(v) q(o|v)
    // (36: the uniform growth's 1/36 per domain), evaluated literally by
    // removing the other domains and setting them again one by one in growth
    // order.  The state, energy and counters are left as they were.
    double lr_growth_literal(const std::vector<int>& st, int d0) {
        double e0 = energy;
        int nst0 = num_stacked, nu0 = num_unassigned;
        int len = (int)st.size();
        std::vector<V3> p(len), o(len);
        for (int k = 0; k < len; ++k) {
            p[k] = doms[st[k]].pos;
            o[k] = doms[st[k]].ore;
        }
        auto order = growth_order(d0, len);
        for (size_t n = order.size(); n-- > 0;) unassign_domain(st[order[n].first]);
        double g = 1;
        for (auto& gk : order) {
            int i = st[gk.first], prev = st[gk.second];
            V3 dv = p[gk.first] - doms[prev].pos;
            int v = 0;
            while (v < 6 && !(kUnit[v] == dv)) ++v;
            if (v == 6) throw std::runtime_error("staple configuration is not a chain of neighbours");
            V3 ov = o[gk.first];
            g *= 36.0 * lr_propose(i, prev, false, v, ov);
            set_checked(i, p[gk.first], o[gk.first]);
        }
        energy = e0;
        num_stacked = nst0;
        num_unassigned = nu0;
        return g;
    }
    bool learned_regrowth() {
        if (num_staples == 0) return false;
        int ci = rng.uniform_int(1, num_staples);
        std::vector<int> sel = chains[ci];
        if (staple_is_connector(sel)) return false;
        auto bds = find_bound_domains(sel);
        auto gp = bds[rng.uniform_int(0, (int)bds.size() - 1)];
        std::vector<V3> old_pos, old_ore;
        for (int id : sel) {
            old_pos.push_back(doms[id].pos);
            old_ore.push_back(doms[id].ore);
        }
        unassign_domains(sel);
        delta_e += set_growth_point(gp.first, gp.second);
        if (rejected) return false;
        int d0 = doms[gp.first].d, len = (int)sel.size();
        std::vector<std::pair<int, int>> grown;   // (domain index, previous domain index) in growth order
        for (int k = d0 + 1; k < len; ++k) grown.push_back({k, k - 1});
        for (int k = d0 - 1; k >= 0; --k) grown.push_back({k, k + 1});
        double qn = 1;
        for (auto& gk : grown) {
            int i = sel[gk.first], prev = sel[gk.second];
            int v = 0;
            V3 o;
            qn *= lr_propose(i, prev, true, v, o);
            delta_e += set_domain_config(i, doms[prev].pos + kUnit[v], o);
            if (violated) {
                rejected = true;
                return false;
            }
            assigned.push_back(key_of(i));
        }
        add_external_bias_met();
        int nbd = num_bound_staple_domains(sel);
        // Q(old): the old configuration grown again from the growth point
        std::vector<V3> new_pos, new_ore;
        for (auto& gk : grown) {
            new_pos.push_back(doms[sel[gk.first]].pos);
            new_ore.push_back(doms[sel[gk.first]].ore);
        }
        for (size_t n = grown.size(); n-- > 0;) unassign_domain(sel[grown[n].first]);
        double qo = 1;
        for (auto& gk : grown) {
            int i = sel[gk.first], prev = sel[gk.second];
            V3 dv = old_pos[gk.first] - doms[prev].pos;
            int v = 0;
            while (v < 6 && !(kUnit[v] == dv)) ++v;
            if (v == 6) throw std::runtime_error("old staple configuration is not a chain of neighbours");
            V3 o = old_ore[gk.first];
            qo *= lr_propose(i, prev, false, v, o);
            set_checked(i, old_pos[gk.first], o);
        }
        for (size_t n = grown.size(); n-- > 0;) unassign_domain(sel[grown[n].first]);
        for (size_t n = 0; n < grown.size(); ++n) set_checked(sel[grown[n].first], new_pos[n], new_ore[n]);
        double boltz = xexp(-(delta_e));
        double pratio = boltz * (double)bds.size() / nbd;
        pratio *= qo / qn;
        return test_acceptance(pratio);
    }

    // MetStapleRegrowthMCMovetype (src/met_movetypes.cpp:470)
    bool met_regrowth() {
        if (num_staples == 0) return false;
        int ci = rng.uniform_int(1, num_staples);
        std::vector<int> sel = chains[ci];
        if (staple_is_connector(sel)) return false;
        auto bds = find_bound_domains(sel);
        auto gp = bds[rng.uniform_int(0, (int)bds.size() - 1)];
        unassign_domains(sel);
        delta_e += set_growth_point(gp.first, gp.second);
        if (rejected) return false;
        grow_staple(doms[gp.first].d, sel, false);
        if (rejected) return false;
        add_external_bias_met();
        int nbd = num_bound_staple_domains(sel);
        double boltz = xexp(-(delta_e));
        double pratio = boltz * bds.size() / nbd;
        return test_acceptance(pratio);
    }

    // CBMCMovetype helpers (src/cb_movetypes.cpp:58-225)
    void calc_biases(V3 p_prev, int dom, std::vector<V3>& cpos, std::vector<V3>& core,
                     std::vector<double>& bf) {
        for (int v = 0; v < 6; ++v) {
            V3 p = p_prev + kUnit[v];
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND) continue;
            if (occ == UNBOUND) {
                int ud = unbound_at(p);
                V3 o = -doms[ud].ore;
                double de = check_domain_constraints(dom, p, o);
                if (!violated) {
                    cpos.push_back(p);
                    core.push_back(o);
                    double b = 1;
                    b *= xexp(-de);
                    bf.push_back(b);
                }
                else {
                    violated = false;
                }
            }
            else {
                cpos.push_back(p);
                core.push_back(V3(0, 0, 0));
                double de = check_domain_constraints(dom, p, V3(1, 0, 0));
                bf.push_back(6 * xexp(-de));
            }
        }
    }

    void cb_select_and_set(int i, const std::vector<int>& ds) {
        int dom = ds[i];
        int prev = ds[i - 1];
        V3 p_prev = doms[prev].pos;
        std::vector<V3> cpos, core;
        std::vector<double> bf;
        calc_biases(p_prev, dom, cpos, core, bf);
        double ros = 0;
        for (double b : bf) ros += b;
        std::vector<double> w;
        if (ros == 0) {
            rejected = true;
            return;
        }
        w_bias.mul(ros);
        for (double b : bf) w.push_back(b / ros);
        if (!regrow_old) {
            V3 p(0, 0, 0), o(0, 0, 0);
            double cum = 0;
            double r = rng.uniform_real();
            for (size_t n = 0; n < w.size(); ++n) {
                cum += w[n];
                if (r < cum) {
                    p = cpos[n];
                    o = core[n];
                    break;
                }
            }
            if (o == V3(0, 0, 0)) o = kUnit[rng.uniform_int(0, 5)];
            set_checked(dom, p, o);
        }
        else {
            Key k = key_of(dom);
            size_t n = 0;
            while (!(old_keys[n].c == k.c && old_keys[n].d == k.d)) ++n;
            set_checked(dom, old_pos[n], old_ore[n]);
        }
        assigned.push_back(key_of(dom));
    }

    void cb_grow_chain(const std::vector<int>& ds) {   // src/cb_movetypes.cpp:354
        for (size_t i = 1; i < ds.size(); ++i) {
            cb_select_and_set((int)i, ds);
            if (rejected) break;
        }
    }

    void cb_set_gp_and_grow(std::pair<int, int> gp, const std::vector<int>& sel) {   // :389
        if (regrow_old) {
            Key k = key_of(gp.first);
            size_t n = 0;
            while (!(old_keys[n].c == k.c && old_keys[n].d == k.d)) ++n;
            double de = 0;
            de += set_checked(gp.first, doms[gp.second].pos, old_ore[n]);
            w_bias.mul(xexp(-de));
            assigned.push_back(k);
        }
        else {
            double de = set_growth_point(gp.first, gp.second);
            w_bias.mul(xexp(-de));
        }
        if (!rejected) grow_staple(doms[gp.first].d, sel, true);
    }

    // CBStapleRegrowthMCMovetype::internal_attempt_move (src/cb_movetypes.cpp:292)
    bool cb_regrowth() {
        if (num_staples == 0) return false;
        int ci = rng.uniform_int(1, num_staples);
        std::vector<int> sel = chains[ci];
        if (staple_is_connector(sel)) return false;
        auto bds = find_bound_domains(sel);
        w_bias.mul((long double)bds.size());
        auto gp = bds[rng.uniform_int(0, (int)bds.size() - 1)];
        unassign_domains(sel);
        cb_set_gp_and_grow(gp, sel);
        if (rejected) return false;
        w_bias.div((long double)num_bound_staple_domains(sel));
        update_move_params();
        double tb = calc_move();
        w_bias.mul(xexp(-tb));
        // setup_for_regrow_old (:215)
        regrow_old = true;
        w_new_bias = w_bias;
        new_modifier = modifier;
        w_bias.set(1);
        old_keys = modified;
        old_pos = prev_pos;
        old_ore = prev_ore;
        modified.clear();
        assigned.clear();
        prev_pos.clear();
        prev_ore.clear();
        gp = bds[rng.uniform_int(0, (int)bds.size() - 1)];
        unassign_domains(sel);
        cb_set_gp_and_grow(gp, sel);
        modifier = new_modifier;
        // test_cb_acceptance (:182)
        if (test_acceptance_ld(w_new_bias.over(w_bias))) {
            reset_origami();
            update_move_params();
            calc_move();
            return true;
        }
        modified.clear();
        assigned.clear();
        prev_pos.clear();
        prev_ore.clear();
        return false;
    }

    // ============================== conserved-topology scaffold regrowth ===
    // topConstraintPoints::StapleNetwork and Constraintpoints
    // (src/top_constraint_points.cpp:26-602), CTRegrowthMCMovetype
    // (src/movetypes.cpp:429-720), the recoil-growth movetypes
    // (src/rg_movetypes.cpp) and the configurational-bias ones
    // (src/cb_movetypes.cpp:406-984).  The reference's movetype factories
    // always pass num_excluded_staples = 0 (src/simulation.cpp:409,538), so no
    // staple is ever excluded and the excluded-staple branches drop out.
    // Domains are keyed by domain id here (a chain never changes during these
    // moves); a (chain, segment) key is (chain index, segment number).
    using CKey = std::pair<int, int>;
    using Ep = std::pair<int, V3>;   // (domain index in its chain, position)
    struct CtPoints {
        std::vector<int> scaffold_domains;
        std::set<int> regrowth_staples;
        std::vector<int> d_stack;
        std::set<int> checked;
        std::vector<V3> erased;
        std::map<int, int> segs;
        std::map<CKey, int> dirs;
        std::map<int, int> growthpoints, stemdomains, inactive;
        std::map<CKey, std::vector<Ep>> active, initial_active;
        std::map<int, std::vector<int>> stemd_to_segs;
        void clear() {   // Constraintpoints::reset_internal (:208)
            scaffold_domains.clear();
            regrowth_staples.clear();
            d_stack.clear();
            checked.clear();
            erased.clear();
            segs.clear();
            dirs.clear();
            growthpoints.clear();
            stemdomains.clear();
            inactive.clear();
            active.clear();
            initial_active.clear();
            stemd_to_segs.clear();
        }
    } cp;
    // StapleNetwork::m_domain_to_dir: never cleared by the reference; it only
    // ever gains (staple, 0) -> +1 and (staple, 1) -> -1.
    std::map<CKey, int> net_dirs;
    struct Net {   // one StapleNetwork::scan_network result
        bool external {false};
        std::set<int> cs;
        std::vector<std::pair<int, int>> gps, iaes;
        std::vector<int> ds;
        std::map<int, int> segs;
    };

    int scaffold_len() const { return (int)chains[0].size(); }
    static bool has(const std::vector<int>& v, int x) { return std::find(v.begin(), v.end(), x) != v.end(); }

    // StapleNetwork::scan_staple_topology (:91) and make_staple_stack (:141)
    void net_scan(Net& n, int growth_d) {
        int ci = doms[growth_d].c;
        n.cs.insert(ci);
        n.ds.push_back(growth_d);
        std::vector<int> st = get_chain(ci);
        int gd = doms[growth_d].d;
        std::vector<int> stack_;
        n.segs[growth_d] = 0;
        net_dirs[{ci, 0}] = 1;
        for (size_t di = gd + 1; di < st.size(); ++di) {
            stack_.push_back(st[di]);
            n.segs[st[di]] = 0;
        }
        net_dirs[{ci, 1}] = -1;
        for (int di = gd - 1; di >= 0; --di) {
            stack_.push_back(st[di]);
            n.segs[st[di]] = 1;
        }
        for (int d : stack_) {
            n.ds.push_back(d);
            int bd = doms[d].bound;
            if (bd < 0 || doms[bd].c == ci) continue;
            int bci = doms[bd].c;
            if (n.cs.count(bci)) {
                bool external = false;
                if (bci == 0) external = !has(cp.scaffold_domains, bd);
                if (!external) {   // add_potential_inactive_endpoint (:166)
                    if (has(n.ds, bd)) n.iaes.push_back({bd, d});
                    else n.iaes.push_back({d, bd});
                }
                if (external) n.external = true;
            }
            else {
                n.gps.push_back({d, bd});
                net_scan(n, bd);
            }
        }
    }

    // Constraintpoints::find_growthpoints_endpoints (:461) with its helpers
    void find_growthpoints_endpoints(const std::vector<int>& sds, int seg) {
        for (int d : sds) {
            cp.d_stack.push_back(d);
            cp.segs[d] = seg;
            int bd = doms[d].bound;
            if (bd < 0 || doms[bd].c == doms[d].c || cp.checked.count(doms[bd].c)) continue;
            Net n;
            n.cs.insert(0);
            net_scan(n, bd);
            n.gps.push_back({d, bd});
            if (n.external) {
                // add_active_endpoints_on_scaffold (:547): note that the
                // inactive-endpoint entries go under the staple's key
                for (auto& g : n.gps)
                    if (doms[g.first].c == 0) add_active_endpoint_seg(g.first, doms[g.first].pos, seg);
                for (auto& e : n.iaes)
                    if (doms[e.second].c == 0) add_active_endpoint_seg(e.first, doms[e.second].pos, seg);
            }
            else {
                for (auto& g : n.gps) {   // add_growthpoints (:506)
                    cp.growthpoints[g.first] = g.second;
                    cp.stemdomains[g.second] = g.first;
                }
                for (auto& e : n.iaes) cp.inactive[e.first] = e.second;
                for (int c : n.cs)
                    if (c != 0) cp.regrowth_staples.insert(c);
                cp.d_stack.insert(cp.d_stack.end(), n.ds.begin(), n.ds.end());
                for (auto& kv : n.segs) cp.segs.insert(kv);
                for (auto& kv : net_dirs) cp.dirs.insert(kv);
            }
            for (int c : n.cs) cp.checked.insert(c);
        }
    }

    // Constraintpoints::calculate_constraintpoints, one segment (:225) or
    // several (:241)
    void calculate_constraintpoints(const std::vector<int>& sds, int dir) {
        cp.scaffold_domains = sds;
        cp.dirs[{doms[sds[0]].c, 0}] = dir;
        find_growthpoints_endpoints(sds, 0);
        cp.initial_active = cp.active;
    }
    void calculate_constraintpoints(const std::vector<std::vector<int>>& segs, const std::vector<int>& dirs_) {
        for (auto& sg : segs) cp.scaffold_domains.insert(cp.scaffold_domains.end(), sg.begin(), sg.end());
        int seg = 0;
        for (size_t i = 0; i < segs.size(); ++i) {
            if (!segs[i].empty()) {
                cp.dirs[{doms[segs[i][0]].c, seg}] = dirs_[i];
                find_growthpoints_endpoints(segs[i], seg);
            }
            seg++;
        }
        cp.initial_active = cp.active;
    }

    void add_active_endpoint_seg(int d, V3 pos, int seg) { cp.active[{doms[d].c, seg}].push_back({doms[d].d, pos}); }
    void add_active_endpoint(int d, V3 pos) { add_active_endpoint_seg(d, pos, cp.segs.at(d)); }
    void add_growthpoint(int gp, int stem) {
        cp.growthpoints[gp] = stem;
        cp.stemdomains[stem] = gp;
    }

    // Constraintpoints::remove_active_endpoint (:300)
    void remove_active_endpoint(int d) {
        cp.erased.clear();
        auto& lst = cp.active[{doms[d].c, cp.segs.at(d)}];
        std::vector<Ep> keep;
        for (auto& e : lst) {
            if (e.first == doms[d].d) cp.erased.push_back(e.second);
            else keep.push_back(e);
        }
        lst = keep;
    }
    // remove_activated_endpoint (:325)
    void remove_activated_endpoint(int d) {
        auto it = cp.inactive.find(d);
        if (it == cp.inactive.end()) return;
        int ed = it->second;
        auto& lst = cp.active[{doms[ed].c, cp.segs.at(ed)}];
        for (size_t j = 0; j < lst.size(); ++j)
            if (lst[j].first == doms[ed].d) {
                lst.erase(lst.begin() + j);
                break;
            }
    }
    // update_endpoints (:345)
    void update_endpoints(int d) {
        remove_active_endpoint(d);
        auto it = cp.inactive.find(d);
        if (it != cp.inactive.end()) add_active_endpoint(it->second, doms[d].pos);
    }
    bool is_growthpoint(int d) const { return cp.growthpoints.count(d) > 0; }
    bool is_stemdomain(int d) const { return cp.stemdomains.count(d) > 0; }
    int get_dir(int d) {   // Constraintpoints::get_dir (:190)
        int seg = cp.segs[d];
        return cp.dirs[{doms[d].c, seg}];
    }
    // endpoint_reached (:363)
    bool endpoint_reached(int d, V3 pos) {
        for (auto& e : cp.active[{doms[d].c, cp.segs.at(d)}])
            if (e.first == doms[d].d && e.second == pos) return true;
        return false;
    }
    // calc_remaining_steps (:569)
    int remaining_steps(int end_d, int d, int dir) const {
        int steps;
        int dd = doms[d].d;
        if (cfg.cyclic && doms[d].c == 0) {
            int N = scaffold_len();
            if (dir > 0 && end_d < dd) steps = N + end_d - dd;
            else if (dir < 0 && end_d > dd) steps = dd + N - end_d;
            else if (dir == 0 || end_d == dd) steps = 0;
            else steps = std::abs(end_d - dd);
        }
        else {
            steps = std::abs(end_d - dd);
        }
        return steps;
    }
    // walks_remain (:398, :424)
    bool walks_remain(int d, V3 pos) {
        std::vector<int> sl;
        if (is_stemdomain(d)) sl = cp.stemd_to_segs[d];
        else sl = {cp.segs.at(d)};
        for (int seg : sl) {
            CKey key {doms[d].c, seg};
            int dir = cp.dirs[key];
            for (auto& e : cp.active[key]) {
                int steps = remaining_steps(e.first, d, dir);
                V3 dr = e.second - pos;
                if (ideal_walks(dr.x, dr.y, dr.z, steps) == 0) return false;
            }
        }
        return true;
    }

    // ---------------------------------------------- segment selection ---
    std::map<int, V3> ct_prev_pos, ct_prev_ore;   // MCMovetype::m_prev_pos/m_prev_ore (keyed)
    int ct_dir {0};                                // CTRegrowthMCMovetype::m_dir

    // CTRegrowthMCMovetype::select_indices (src/movetypes.cpp:479)
    std::vector<int> select_indices(int min_length, int seg, int max_regrowth) {
        const std::vector<int>& sc = chains[0];
        int seg_length = (int)sc.size();
        int max_length = std::min(seg_length, max_regrowth);
        int sel_length = rng.uniform_int(min_length, max_length);
        int start_i = rng.uniform_int(0, seg_length - 1);
        ct_dir = rng.uniform_int(0, 1);
        if (ct_dir == 0) ct_dir = -1;
        int cur = sc[start_i];
        std::vector<int> out;
        while (cur >= 0 && (int)out.size() != sel_length) {
            out.push_back(cur);
            cur = next(cur, ct_dir);
        }
        int back = next(sc[start_i], -ct_dir);
        while (back >= 0 && (int)out.size() != sel_length) {
            out.insert(out.begin(), back);
            back = next(back, -ct_dir);
        }
        if ((int)out.size() < min_length) return select_indices(min_length, seg, max_regrowth);
        if (cur >= 0) add_active_endpoint_seg(cur, doms[cur].pos, seg);
        return out;
    }

    // CTRegrowthMCMovetype::check_for_stemds (src/movetypes.cpp:702)
    void check_for_stemds(int cur, std::deque<int>& stems) {
        if (doms[cur].state != BOUND) return;
        int b = doms[cur].bound;
        for (int sdir : {-1, 1}) {
            int nb = next(b, sdir);
            if (nb >= 0 && doms[nb].state == BOUND) {
                int bn = doms[nb].bound;
                if (doms[bn].c == 0) stems.push_back(bn);
            }
        }
    }
    // fill_seg (src/movetypes.cpp:669)
    bool fill_seg(int start, int max_length, int seg_max, int dir, std::set<int>& in, std::deque<int>& stems,
                  std::vector<int>& seg) {
        int cur = start;
        check_for_stemds(cur, stems);
        int nd = start;
        bool reached = false;
        while ((int)seg.size() != seg_max && nd >= 0) {
            nd = next(cur, dir);
            if (nd < 0) break;
            int nn = next(nd, dir);
            if (nn >= 0 && in.count(nn)) break;
            seg.push_back(nd);
            in.insert(nd);
            if ((int)in.size() == max_length) {
                reached = true;
                break;
            }
            cur = nd;
            check_for_stemds(cur, stems);
        }
        return reached;
    }
    // select_noncontig_segs (src/movetypes.cpp:540)
    void select_noncontig_segs(const ScaffoldMoveOpts& mo, std::vector<std::vector<int>>& segs,
                               std::vector<std::vector<std::vector<int>>>& paired, std::vector<int>& stems_sel,
                               std::vector<int>& dirs_) {
        const std::vector<int>& sc = chains[0];
        std::set<int> in;
        int max_length = rng.uniform_int(2, mo.max_regrowth);
        int seg_max = rng.uniform_int(2, mo.max_seg_regrowth + 1);
        int start_i = rng.uniform_int(0, (int)sc.size() - 1);
        int sd0 = sc[start_i];
        int dir = rng.uniform_int(0, 1);
        if (dir == 0) dir = -1;
        if (next(sd0, dir) < 0) dir *= -1;
        std::vector<int> cur_seg {sd0};
        in.insert(sd0);
        std::deque<int> stems;
        dirs_.push_back(dir);
        bool reached = fill_seg(sd0, max_length, seg_max, dir, in, stems, cur_seg);
        segs.push_back(cur_seg);
        while (!reached && !stems.empty()) {
            cur_seg.clear();
            int stemd = stems.front();
            stems.pop_front();
            if (in.count(stemd)) continue;
            bool adjacent = false;
            for (int td : {-1, 1}) {
                int nd = next(stemd, td);
                if (nd >= 0 && in.count(nd)) {
                    adjacent = true;
                    break;
                }
            }
            if (adjacent) continue;
            cur_seg.push_back(stemd);
            in.insert(stemd);
            stems_sel.push_back(stemd);
            if ((int)in.size() == max_length) {
                reached = true;
                segs.push_back(cur_seg);
                segs.push_back({});
                paired.push_back({{}, {}});
                dirs_.push_back(1);
                dirs_.push_back(-1);
                break;
            }
            int dir1 = rng.uniform_int(0, 1);
            if (dir1 == 0) dir1 = -1;
            int dp[2] = {dir1, -dir1};
            dirs_.push_back(dp[0]);
            dirs_.push_back(dp[1]);
            std::vector<std::vector<int>> pair_ {{}, {}};
            segs.push_back({});
            segs.push_back({});
            for (int i = 0; i < 2; ++i) {
                dir = dp[i];
                seg_max = rng.uniform_int(0, mo.max_seg_regrowth);
                if (i == 0) max_length++;
                std::vector<int> sg;
                reached = fill_seg(stemd, max_length, seg_max, dir, in, stems, sg);
                pair_[i] = sg;
                if (!cur_seg.empty()) sg.insert(sg.begin(), cur_seg[0]);
                segs[segs.size() - 2 + i] = sg;
                if (reached) break;
                cur_seg.clear();
            }
            paired.push_back(pair_);
        }
        int last = segs[0].back();
        int nd = next(last, dirs_[0]);
        if (nd >= 0) add_active_endpoint_seg(nd, doms[nd].pos, 0);
        int seg_i = 1;
        for (size_t i = 0; i < paired.size(); ++i) {
            int stem = stems_sel[i];
            add_growthpoint(doms[stem].bound, stem);
            cp.stemd_to_segs[stem] = {seg_i, seg_i + 1};
            for (auto& sg : paired[i]) {
                int d = dirs_[seg_i];
                int l = sg.empty() ? stem : sg.back();
                int n2 = next(l, d);
                if (n2 >= 0) add_active_endpoint_seg(n2, doms[n2].pos, seg_i);
                seg_i++;
            }
        }
    }

    // Reference-side bookkeeping of the keyed maps, for reset_origami.
    void ct_sync_prev() {
        prev_pos.clear();
        prev_ore.clear();
        for (auto& k : modified) {
            int id = dom_of(k);
            prev_pos.push_back(ct_prev_pos.at(id));
            prev_ore.push_back(ct_prev_ore.at(id));
        }
    }
    void ct_save_unassign(int id, double* de) {
        ct_prev_pos[id] = doms[id].pos;
        ct_prev_ore[id] = doms[id].ore;
        modified.push_back(key_of(id));
        double e = unassign_domain(id);
        if (de) *de += e;
    }

    // ------------------------------------------------------ recoil growth ---
    // CTRGRegrowthMCMovetype state (include/.../rg_movetypes.hpp:73-108)
    std::vector<int> rg_ds;
    std::vector<int> catt_q, catt_wq;
    std::vector<std::vector<int>> avail_q, avail_wq;
    std::vector<double> c_opens;
    std::map<int, V3> rg_old_pos, rg_old_ore, rg_new_pos, rg_new_ore;
    std::vector<std::vector<V3>> erased_q;
    double rg_delta_e {0}, rg_weight {1}, rg_weight_new {1};
    int rg_di {0}, rg_d {0}, rg_ref {0};
    bool rg_stemd {false};
    int rg_catt {0}, rg_dmax {0};
    std::vector<int> rg_avail;
    int rg_max_recoils {0}, rg_max_c_attempts {0};

    void rg_reset() {   // CTRGRegrowthMCMovetype::reset_internal (:63)
        cp.clear();
        ct_prev_pos.clear();
        ct_prev_ore.clear();
        rg_ds.clear();
        catt_q.clear();
        catt_wq.clear();
        avail_q.clear();
        avail_wq.clear();
        c_opens.clear();
        erased_q.clear();
        rg_delta_e = 0;
        rg_weight = 1;
        rg_weight_new = 1;
    }
    static std::vector<int> all_cis() {
        std::vector<int> v(36);
        for (int i = 0; i < 36; ++i) v[i] = i;
        return v;
    }
    // unassign_and_save_domains (:81)
    double rg_unassign_and_save() {
        double de = 0;
        int d0 = rg_ds[0];
        ct_prev_pos[d0] = doms[d0].pos;
        ct_prev_ore[d0] = doms[d0].ore;
        for (size_t i = 1; i < rg_ds.size(); ++i) ct_save_unassign(rg_ds[i], &de);
        erased_q.clear();
        return de;
    }
    void rg_unassign_domains() {   // :116
        for (size_t i = 1; i < rg_ds.size(); ++i) unassign_domain(rg_ds[i]);
        erased_q.clear();
    }
    double rg_set_config(int d, V3 p, V3 o) {   // set_config (:233)
        double de = set_checked(d, p, o);
        assigned.push_back(key_of(d));
        update_endpoints(rg_d);
        erased_q.push_back(cp.erased);
        return de;
    }
    void rg_prepare_for_growth() {   // :245
        rg_di++;
        rg_d = rg_ds[rg_di];
        rg_stemd = is_stemdomain(rg_d);
        ct_dir = get_dir(rg_d);
        rg_catt = 0;
        if (rg_stemd) {
            rg_dmax = 1;
            rg_avail.clear();
            rg_ref = cp.stemdomains[rg_d];
        }
        else {
            rg_dmax = rg_max_c_attempts;
            rg_avail = all_cis();
            rg_ref = next(rg_d, -ct_dir);
        }
    }
    void rg_restore_endpoints() {   // :289
        remove_activated_endpoint(rg_d);
        std::vector<V3> er = erased_q.back();
        erased_q.pop_back();
        for (auto& p : er) add_active_endpoint(rg_d, p);
    }
    double rg_prepare_for_regrowth() {   // :263
        rg_di--;
        rg_d = rg_ds[rg_di];
        ct_dir = get_dir(rg_d);
        double de = unassign_domain(rg_d);
        assigned.pop_back();
        rg_restore_endpoints();
        rg_stemd = is_stemdomain(rg_d);
        if (rg_stemd) {
            rg_dmax = 1;
            rg_catt = 1;
            rg_avail.clear();
            rg_ref = cp.stemdomains[rg_d];
        }
        else {
            rg_dmax = rg_max_c_attempts;
            rg_catt = catt_q[rg_di];
            rg_avail = avail_q[rg_di];
            rg_ref = next(rg_d, -ct_dir);
        }
        return de;
    }
    // select_trial_config (:298): configuration ci = 6 * (position step) + orientation
    void rg_select_trial(V3& p, V3& o) {
        if (rg_stemd) {
            p = doms[rg_ref].pos;
            o = -doms[rg_ref].ore;
        }
        else {
            int k = rng.uniform_int(0, (int)rg_avail.size() - 1);
            int i = rg_avail[k];
            rg_avail.erase(rg_avail.begin() + k);
            p = kUnit[i / 6] + doms[rg_ref].pos;
            o = kUnit[i % 6];
        }
    }
    // calc_p_config_open (:316)
    double rg_p_open(V3 p, V3 o) {
        double de = check_domain_constraints(rg_d, p, o);
        if (violated) {
            violated = false;
            return 0;
        }
        if (!walks_remain(rg_d, p)) return 0;
        if (occupancy(p) == UNBOUND) {
            int od = unbound_at(p);
            bool same = doms[od].c == doms[rg_d].c;
            bool endpoint = endpoint_reached(rg_d, p);
            if (!(same || endpoint || rg_stemd)) return 0;
        }
        return std::fmin(1, xexp(-de));
    }
    bool rg_test_open(double p) {   // test_config_open (:346)
        p = std::fmin(1, p);
        if (p == 1) return true;
        return p > rng.uniform_real();
    }
    // recoil_regrow (:177)
    double recoil_regrow() {
        double de = 0;
        rg_di = 0;
        rg_d = rg_ds[0];
        ct_dir = get_dir(rg_d);
        catt_q.assign(rg_ds.size(), 0);
        avail_q.assign(rg_ds.size(), {});
        c_opens.assign(rg_ds.size(), 0);
        c_opens[0] = 1;
        rg_prepare_for_growth();
        int recoils = 0;
        while (true) {
            V3 p, o;
            double pc = 0;
            bool open = false;
            while (!open && rg_catt != rg_dmax) {
                rg_catt++;
                rg_select_trial(p, o);
                pc = rg_p_open(p, o);
                open = rg_test_open(pc);
            }
            if (open) {
                if (recoils != 0) recoils--;
                de += rg_set_config(rg_d, p, o);
                catt_q[rg_di] = rg_catt;
                avail_q[rg_di] = rg_avail;
                c_opens[rg_di] = pc;
                if (rg_di == (int)rg_ds.size() - 1) break;
                rg_prepare_for_growth();
            }
            else {
                if (recoils == rg_max_recoils || rg_di == 1) {
                    rejected = true;
                    break;
                }
                recoils++;
                de += rg_prepare_for_regrowth();
            }
        }
        return de;
    }
    // test_config_avail (:418)
    bool rg_test_avail() {
        int feels = 0;
        if (feels == rg_max_recoils || rg_di == (int)rg_ds.size() - 1) return true;
        rg_prepare_for_growth();
        bool avail;
        while (true) {
            V3 p, o;
            bool open = false;
            while (!open && rg_catt != rg_dmax) {
                rg_catt++;
                rg_select_trial(p, o);
                double pc = rg_p_open(p, o);
                open = rg_test_open(pc);
            }
            if (open) {
                feels++;
                if (feels == rg_max_recoils || rg_di == (int)rg_ds.size() - 1) {
                    feels--;
                    avail = true;
                    break;
                }
                rg_set_config(rg_d, p, o);
                catt_q[rg_di] = rg_catt;
                avail_q[rg_di] = rg_avail;
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
        }
        while (feels != 0) {
            rg_di--;
            feels--;
            rg_d = rg_ds[rg_di];
            unassign_domain(rg_d);
            rg_restore_endpoints();
        }
        rg_di--;
        rg_d = rg_ds[rg_di];
        return avail;
    }
    // calc_weights (:363): `pos`/`ore` hold the configuration being weighed
    void rg_calc_weights() {
        rg_di = 0;
        rg_d = rg_ds[0];
        while (rg_di != (int)rg_ds.size() - 1) {
            rg_di++;
            rg_d = rg_ds[rg_di];
            rg_stemd = is_stemdomain(rg_d);
            ct_dir = get_dir(rg_d);
            int avail_cs = 1;
            if (!rg_stemd) {
                rg_ref = next(rg_d, -ct_dir);
                int catt = catt_wq[rg_di];
                rg_avail = avail_wq[rg_di];
                while (catt != rg_max_c_attempts) {
                    catt++;
                    V3 p, o;
                    rg_select_trial(p, o);
                    double pc = rg_p_open(p, o);
                    if (rg_test_open(pc)) {
                        set_checked(rg_d, p, o);
                        update_endpoints(rg_d);
                        erased_q.push_back(cp.erased);
                        int dir_s = ct_dir, ref_s = rg_ref;
                        bool stem_s = rg_stemd;
                        std::vector<int> avail_s = rg_avail;
                        avail_cs += rg_test_avail();
                        rg_avail = avail_s;
                        rg_stemd = stem_s;
                        rg_ref = ref_s;
                        ct_dir = dir_s;
                        unassign_domain(rg_d);
                        rg_restore_endpoints();
                    }
                }
            }
            rg_weight *= avail_cs / c_opens[rg_di - 1];
            set_checked(rg_d, ct_prev_pos.at(rg_d), ct_prev_ore.at(rg_d));
            update_endpoints(rg_d);
            erased_q.push_back(cp.erased);
        }
        rg_weight /= c_opens[rg_di];
    }
    // calc_old_c_opens (:481)
    void rg_calc_old_c_opens() {
        rg_di = 0;
        c_opens[0] = 1;
        while (rg_di != (int)rg_ds.size() - 1) {
            rg_di++;
            rg_d = rg_ds[rg_di];
            catt_q[rg_di] = 1;
            V3 p = rg_old_pos.at(rg_d), o = rg_old_ore.at(rg_d);
            rg_stemd = is_stemdomain(rg_d);
            c_opens[rg_di] = rg_p_open(p, o);
            rg_set_config(rg_d, p, o);
            if (rg_stemd) {
                avail_q[rg_di].clear();
            }
            else {
                avail_q[rg_di] = all_cis();
                ct_dir = get_dir(rg_d);
                rg_ref = next(rg_d, -ct_dir);
                V3 dp = p - rg_old_pos.at(rg_ref);
                int k = 0;
                while (k < 6 && !(kUnit[k] == dp)) ++k;
                int ko = 0;
                while (ko < 6 && !(kUnit[ko] == o)) ++ko;
                if (k == 6 || ko == 6) throw std::runtime_error("old configuration is not a neighbour step");
                int ci = 6 * k + ko;
                auto& av = avail_q[rg_di];
                av.erase(std::remove(av.begin(), av.end(), ci), av.end());
            }
        }
    }
    // test_rg_acceptance (:515)
    bool rg_test_acceptance() {
        long double ratio = rg_weight_new / rg_weight * xexp(-rg_delta_e);
        if (test_acceptance_ld(ratio)) {
            ct_prev_pos = rg_new_pos;
            ct_prev_ore = rg_new_ore;
            ct_sync_prev();
            reset_origami();
            return true;
        }
        modified.clear();
        assigned.clear();
        prev_pos.clear();
        prev_ore.clear();
        return false;
    }
    bool test_acceptance_ld(long double p) {   // MCMovetype::test_acceptance (src/movetypes.cpp:142)
        if (!ld_weights) return test_acceptance((double)p);
        double pa = (double)(std::fmin((long double)1, p) * (long double)modifier);
        if (pa == 1) return true;
        return pa > rng.uniform_real();
    }
    // The weights of the new and old configurations and the acceptance test,
    // common to both recoil-growth movetypes.  remove_first(k) says whether
    // the k-th endpoint reset also drops the endpoints of the first domain.
    bool rg_weigh_and_test(bool remove_first[3]) {
        update_move_params();   // add_external_bias (:76)
        rg_delta_e += calc_move();
        // setup_for_calc_new_weights (:137)
        catt_wq = catt_q;
        avail_wq = avail_q;
        rg_old_pos = ct_prev_pos;
        rg_old_ore = ct_prev_ore;
        modified.clear();
        rg_unassign_and_save();
        cp.active = cp.initial_active;
        if (remove_first[0]) remove_active_endpoint(rg_ds[0]);
        rg_calc_weights();
        rg_unassign_domains();
        cp.active = cp.initial_active;
        if (remove_first[1]) remove_active_endpoint(rg_ds[0]);
        rg_calc_old_c_opens();
        // setup_for_calc_old_weights (:146)
        rg_weight_new = rg_weight;
        rg_weight = 1;
        catt_wq = catt_q;
        avail_wq = avail_q;
        rg_new_pos = ct_prev_pos;
        rg_new_ore = ct_prev_ore;
        modified.clear();
        rg_unassign_and_save();
        cp.active = cp.initial_active;
        if (remove_first[2]) remove_active_endpoint(rg_ds[0]);
        rg_calc_weights();
        return rg_test_acceptance();
    }
    // CTRGScaffoldRegrowthMCMovetype::internal_attempt_move (:629)
    bool ctrg_scaffold(const ScaffoldMoveOpts& mo) {
        rg_reset();
        rg_max_recoils = mo.max_num_recoils;
        rg_max_c_attempts = mo.max_c_attempts;
        std::vector<int> sel = select_indices(2, 0, mo.max_regrowth);
        calculate_constraintpoints(sel, ct_dir);   // setup_constraints (:126)
        bool whole = cfg.cyclic && (int)sel.size() == scaffold_len();
        if (!whole) remove_active_endpoint(sel[0]);
        rg_ds = cp.d_stack;
        rg_delta_e += rg_unassign_and_save();
        rg_delta_e += recoil_regrow();
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        bool whole_ds = cfg.cyclic && (int)rg_ds.size() == scaffold_len();
        // the second reset's condition reads differently in the reference (:673)
        bool rf[3] = {!whole_ds, !cfg.cyclic && (int)rg_ds.size() == scaffold_len(), !whole_ds};
        return rg_weigh_and_test(rf);
    }
    // CTRGJumpScaffoldRegrowthMCMovetype::internal_attempt_move (:792)
    bool ctrg_jump(const ScaffoldMoveOpts& mo) {
        rg_reset();
        rg_max_recoils = mo.max_num_recoils;
        rg_max_c_attempts = mo.max_c_attempts;
        std::vector<std::vector<int>> segs;
        std::vector<std::vector<std::vector<int>>> paired;
        std::vector<int> stems, dirs_;
        select_noncontig_segs(mo, segs, paired, stems, dirs_);
        calculate_constraintpoints(segs, dirs_);
        remove_active_endpoint(segs[0][0]);
        for (int st : stems) add_growthpoint(doms[st].bound, st);
        rg_ds = cp.d_stack;
        rg_delta_e += rg_unassign_and_save();
        rg_delta_e += recoil_regrow();
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        bool rf[3] = {true, true, true};
        return rg_weigh_and_test(rf);
    }

    // --------------------------------------------- configurational bias ---
    std::map<int, V3> cb_old_pos, cb_old_ore;

    void ctcb_unassign(const std::vector<int>& ds) {   // CBMCMovetype::unassign_domains (:200)
        for (int id : ds) ct_save_unassign(id, nullptr);
    }
    // CTCBRegrowthMCMovetype::calc_bias (:480) after CBMCMovetype::calc_biases (:58)
    void ctcb_select_and_set(int i, const std::vector<int>& ds) {
        int dom = ds[i];
        V3 p_prev = doms[ds[i - 1]].pos;
        std::vector<V3> cpos, core;
        std::vector<double> bf;
        calc_biases(p_prev, dom, cpos, core, bf);
        std::vector<long double> w(bf.begin(), bf.end());   // FP64 values unless ld_weights
        for (size_t k = 0; k < cpos.size(); ++k) {
            V3 p = cpos[k];
            if (occupancy(p) == UNBOUND) {
                int od = unbound_at(p);
                bool same = doms[od].c == doms[dom].c;
                bool endpoint = endpoint_reached(dom, p);
                if (!(same || endpoint)) w[k] = 0;
            }
            if (!walks_remain(dom, p)) w[k] = 0;
        }
        long double sum = 0;
        for (auto x : w) sum = ld_weights ? sum + x : (long double)((double)sum + (double)x);
        // a dead end rejects; a rejection from before (the old configuration's
        // staple growth, :717) still multiplies in this domain's weight
        // (CBMCMovetype::select_and_set_config, :113-116)
        if (sum == 0) rejected = true;
        else w_bias.mul(sum);
        if (rejected) return;
        std::vector<double> nw;
        for (auto x : w) nw.push_back(ld_weights ? (double)(x / sum) : (double)x / (double)sum);
        if (!regrow_old) {   // select_and_set_new_config (:132)
            V3 p(0, 0, 0), o(0, 0, 0);
            double cum = 0;
            double r = rng.uniform_real();
            for (size_t n = 0; n < nw.size(); ++n) {
                cum += nw[n];
                if (r < cum) {
                    p = cpos[n];
                    o = core[n];
                    break;
                }
            }
            if (o == V3(0, 0, 0)) o = kUnit[rng.uniform_int(0, 5)];
            set_checked(dom, p, o);
        }
        else {
            set_checked(dom, cb_old_pos.at(dom), cb_old_ore.at(dom));
        }
        assigned.push_back(key_of(dom));
    }
    // CTCBRegrowthMCMovetype::grow_chain (:463)
    void ctcb_grow_chain(const std::vector<int>& ds) {
        if (ds.size() <= 1) return;
        for (size_t i = 1; i < ds.size(); ++i) {
            int d = ds[i];
            ct_dir = get_dir(d);
            ctcb_select_and_set((int)i, ds);
            if (rejected) break;
            update_endpoints(d);
            if (is_growthpoint(d)) {
                ctcb_grow_staple_and_update(d);
                if (rejected) break;
            }
        }
    }
    // grow_staple_and_update_endpoints (:533) with RegrowthMCMovetype::grow_staple
    void ctcb_grow_staple_and_update(int gold) {
        int gnew = cp.growthpoints[gold];
        int c_i = doms[gnew].c;
        if (c_i == 0) return;
        if (regrow_old) {   // set_old_growth_point (:168)
            double de = set_checked(gnew, doms[gold].pos, cb_old_ore.at(gnew));
            w_bias.mul(xexp(-de));
            assigned.push_back(key_of(gnew));
        }
        else {
            double de = set_growth_point(gnew, gold);
            w_bias.mul(xexp(-de));
        }
        if (rejected) return;
        update_endpoints(gnew);
        std::vector<int> ch = get_chain(c_i);
        int d_i = doms[gnew].d;
        std::vector<int> three(ch.begin() + d_i, ch.end());
        if (three.size() > 1) ctcb_grow_chain(three);
        if (rejected) return;
        std::vector<int> five(ch.begin(), ch.begin() + d_i + 1);
        std::reverse(five.begin(), five.end());
        if (five.size() > 1) ctcb_grow_chain(five);
    }
    void ctcb_reset() {   // CTCBRegrowthMCMovetype::reset_internal (:459)
        cp.clear();
        ct_prev_pos.clear();
        ct_prev_ore.clear();
    }
    void ctcb_setup_regrow_old() {   // CBMCMovetype::setup_for_regrow_old (:215)
        regrow_old = true;
        w_new_bias = w_bias;
        new_modifier = modifier;
        w_bias.set(1);
        modified.clear();
        assigned.clear();
        cb_old_pos = ct_prev_pos;
        cb_old_ore = ct_prev_ore;
    }
    // test_cb_acceptance (:182) with the long double weights
    bool ctcb_test_acceptance() {
        if (test_acceptance_ld(w_new_bias.over(w_bias))) {
            ct_sync_prev();
            reset_origami();
            update_move_params();
            calc_move();
            return true;
        }
        modified.clear();
        assigned.clear();
        prev_pos.clear();
        prev_ore.clear();
        return false;
    }
    // CTCBScaffoldRegrowthMCMovetype::internal_attempt_move (:691)
    bool ctcb_scaffold(const ScaffoldMoveOpts& mo) {
        ctcb_reset();
        std::vector<int> sd = select_indices(2, 0, mo.max_regrowth);
        calculate_constraintpoints(sd, ct_dir);
        bool whole = cfg.cyclic && (int)sd.size() == scaffold_len();
        if (!whole) remove_active_endpoint(sd[0]);
        std::set<int> staples = cp.regrowth_staples;
        std::vector<int> unassign_sc(sd.begin() + 1, sd.end());
        ctcb_unassign(unassign_sc);
        for (int c : staples) ctcb_unassign(get_chain(c));
        if (is_growthpoint(sd[0])) {
            ctcb_grow_staple_and_update(sd[0]);
            if (rejected) {
                ct_sync_prev();
                return false;
            }
        }
        ctcb_grow_chain(sd);
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        update_move_params();   // add_external_bias (:52)
        w_bias.mul(xexp(-calc_move()));
        ctcb_setup_regrow_old();
        cp.active = cp.initial_active;
        if (!whole) remove_active_endpoint(sd[0]);
        ctcb_unassign(unassign_sc);
        for (int c : staples) ctcb_unassign(get_chain(c));
        if (is_growthpoint(sd[0])) ctcb_grow_staple_and_update(sd[0]);
        ctcb_grow_chain(sd);
        modifier = 1;
        return ctcb_test_acceptance();
    }
    // CTCBJumpScaffoldRegrowthMCMovetype::set_first_seg_domain (:968)
    void ctcb_first_seg_domain(int dnew) {
        int dold = cp.stemdomains[dnew];
        if (!walks_remain(dnew, doms[dold].pos)) {
            rejected = true;
            return;
        }
        ct_dir = get_dir(dnew);
        double de = set_growth_point(dnew, dold);
        w_bias.mul(xexp(-de));
    }
    // the growth sequence of CTCBJumpScaffoldRegrowthMCMovetype (:880-906)
    bool ctcb_jump_grow(const std::vector<std::vector<int>>& segs,
                        const std::vector<std::vector<std::vector<int>>>& paired, const std::vector<int>& stems) {
        if (is_growthpoint(segs[0][0])) {
            ctcb_grow_staple_and_update(segs[0][0]);
            if (rejected) return false;
        }
        ctcb_grow_chain(segs[0]);
        if (rejected) return false;
        for (size_t i = 0; i < stems.size(); ++i) {
            ctcb_first_seg_domain(stems[i]);
            if (rejected) return false;
            for (auto sg : paired[i]) {
                sg.insert(sg.begin(), stems[i]);
                ctcb_grow_chain(sg);
                if (rejected) return false;
            }
        }
        return true;
    }
    // CTCBJumpScaffoldRegrowthMCMovetype::internal_attempt_move (:864)
    bool ctcb_jump(const ScaffoldMoveOpts& mo) {
        ctcb_reset();
        std::vector<std::vector<int>> segs;
        std::vector<std::vector<std::vector<int>>> paired;
        std::vector<int> stems, dirs_;
        select_noncontig_segs(mo, segs, paired, stems, dirs_);
        calculate_constraintpoints(segs, dirs_);
        remove_active_endpoint(segs[0][0]);
        std::vector<int> rd = cp.d_stack;
        std::vector<int> to_unassign(rd.begin() + 1, rd.end());
        ctcb_unassign(to_unassign);
        if (!ctcb_jump_grow(segs, paired, stems)) {
            ct_sync_prev();
            return false;
        }
        update_move_params();   // add_external_bias
        w_bias.mul(xexp(-calc_move()));
        ctcb_setup_regrow_old();
        cp.active = cp.initial_active;
        remove_active_endpoint(segs[0][0]);
        ctcb_unassign(to_unassign);
        if (!ctcb_jump_grow(segs, paired, stems)) {
            // the reference returns here with the new configuration saved as
            // the one to revert to (m_prev_pos, :927)
            ct_sync_prev();
            return false;
        }
        modifier = 1;
        return ctcb_test_acceptance();
    }


    // ================================= scaffold transforms with linkers ===
    // LinkerRegrowthMCMovetype, ClusteredLinkerRegrowthMCMovetype and the
    // CTCB / CTRG linker movetypes (src/transform_movetypes.cpp).
    std::vector<int> lk1, lk2, lk_cen, lk_cdom;
    int lk_end[2] {-1, -1};   // m_linker_endpoints

    // scan_for_external_scaffold_domain (:262)
    bool lk_scan_external(int dom, std::set<int>& part) {
        bool ext = false;
        int c_i = doms[dom].c;
        part.insert(c_i);
        for (int cur : get_chain(c_i)) {
            if (cur == dom) continue;
            int b = doms[cur].bound;
            if (b < 0) continue;
            if (doms[b].c == doms[dom].c) continue;
            if (doms[b].c == scaffold_c()) {
                if (!has(lk_cen, b)) {
                    ext = true;
                    break;
                }
                continue;
            }
            if (part.count(doms[b].c)) continue;
            ext = lk_scan_external(b, part);
            if (ext) break;
        }
        return ext;
    }
    bool lk_bound_externally() {   // domains_bound_externally (:238)
        for (int d : lk_cen) {
            if (doms[d].state == UNBOUND) continue;
            int b = doms[d].bound;
            if (doms[b].c == scaffold_c()) continue;
            std::set<int> part {doms[d].c};
            if (lk_scan_external(b, part)) return true;
        }
        return false;
    }
    // LinkerRegrowthMCMovetype::select_and_setup_segments (:156)
    bool lk_select(const ScaffoldMoveOpts& mo) {
        bool ext = true;
        int attempts = 0;
        while (ext && attempts != 10) {
            lk1.clear();
            lk2.clear();
            lk_cen = select_indices(1, 0, mo.max_regrowth);
            int len1 = rng.uniform_int(2, mo.max_linker_length + 1);
            int d = lk_cen.front();
            int stop = next(lk_cen.back(), 2 * ct_dir);
            while ((int)lk1.size() != len1 && d >= 0 && d != stop) {
                lk1.push_back(d);
                d = next(d, -ct_dir);
            }
            if (cfg.cyclic && lk1.size() == 1) return false;
            int len2 = rng.uniform_int(2, mo.max_linker_length + 1);
            d = lk_cen.back();
            stop = next(lk1.back(), -ct_dir);
            while ((int)lk2.size() != len2 && d >= 0 && d != stop) {
                lk2.push_back(d);
                d = next(d, ct_dir);
            }
            ext = lk_bound_externally();
            attempts++;
        }
        return !ext;
    }
    // ClusteredLinkerRegrowthMCMovetype::linear_select_central_segment (:670)
    std::vector<int> lk_linear_central() {
        ct_dir = 1;
        std::vector<int> cen;
        const std::vector<int>& sc = chains[0];
        int kernel = rng.uniform_int(1, (int)sc.size() - 2);
        bool started = false;
        int kd = sc[kernel];
        if (doms[kd].state == BOUND) {
            started = true;
            cen.push_back(kd);
            int p = next(kd, -1);
            while (p >= 0 && doms[p].state == BOUND && cen.size() != sc.size() - 1) {
                cen.push_back(p);
                p = next(p, -1);
            }
        }
        if (cen.size() == sc.size() - 1) return {};
        std::reverse(cen.begin(), cen.end());
        int n = next(kd, 1);
        bool ended = false;
        while (!ended && n >= 0) {
            if (doms[n].state == BOUND) {
                started = true;
                cen.push_back(n);
            }
            else if (started) {
                ended = true;
            }
            n = next(n, 1);
        }
        n = next(kd, -1);
        if (!started) {
            while (!ended && n >= 0) {
                if (doms[n].state == BOUND) {
                    started = true;
                    cen.push_back(n);
                }
                else if (started) {
                    ended = true;
                }
                n = next(n, -1);
            }
            std::reverse(cen.begin(), cen.end());
        }
        return cen;
    }
    // ClusteredLinkerRegrowthMCMovetype::cyclic_select_central_segment (:734)
    std::vector<int> lk_cyclic_central() {
        ct_dir = 1;
        std::vector<int> cen;
        const std::vector<int>& sc = chains[0];
        int kernel = rng.uniform_int(1, (int)sc.size() - 2);
        bool started = false;
        int kd = sc[kernel];
        if (doms[kd].state == BOUND) {
            started = true;
            cen.push_back(kd);
            int p = next(kd, -1);
            while (doms[p].state == BOUND && cen.size() != sc.size() - 1) {
                cen.push_back(p);
                p = next(p, -1);
            }
        }
        if (cen.size() == sc.size() - 1) return {};
        std::reverse(cen.begin(), cen.end());
        int n = next(kd, 1);
        bool ended = false;
        while (!ended && n != kd) {
            if (doms[n].state == BOUND) {
                started = true;
                cen.push_back(n);
            }
            else if (started) {
                ended = true;
            }
            n = next(n, 1);
        }
        return cen;
    }
    // ClusteredLinkerRegrowthMCMovetype::select_and_setup_segments (:607)
    bool lk_select_clustered(const ScaffoldMoveOpts& mo) {
        bool ext = true;
        int attempts = 0;
        while (ext && attempts != 10) {
            lk_cen = cfg.cyclic ? lk_cyclic_central() : lk_linear_central();
            if (lk_cen.empty()) return false;
            ext = lk_bound_externally();
            attempts++;
        }
        if (ext) return false;
        lk1.clear();
        lk2.clear();
        int maxl = mo.max_linker_length;
        lk1.push_back(lk_cen[0]);
        int p = next(lk_cen[0], -1);
        if (p != lk_cen.back() && p != next(lk_cen.back(), 1)) {
            while (p >= 0 && doms[p].state != BOUND && (int)lk1.size() != maxl && p != next(lk_cen.back(), 2)) {
                lk1.push_back(p);
                p = next(p, -1);
            }
        }
        if (lk1.size() == 1) return false;
        lk2.push_back(lk_cen.back());
        int n = next(lk_cen.back(), 1);
        if (n != lk1.back()) {
            while (n >= 0 && doms[n].state != BOUND && (int)lk2.size() != maxl && n != next(lk1.back(), -1)) {
                lk2.push_back(n);
                n = next(n, 1);
            }
        }
        return true;
    }
    // setup_fixed_end_biases (:210)
    void lk_setup_fixed_ends() {
        lk_end[0] = next(lk1.back(), -ct_dir);
        lk_end[1] = next(lk2.back(), ct_dir);
        for (int seg = 0; seg < 2; ++seg)
            if (lk_end[seg] >= 0) add_active_endpoint_seg(lk_end[seg], doms[lk_end[seg]].pos, seg);
        std::vector<std::vector<int>> segs {{lk1.begin() + 1, lk1.end()}, {lk2.begin() + 1, lk2.end()}};
        calculate_constraintpoints(segs, {-ct_dir, ct_dir});
    }
    // the central segment and the staples bound within it (find_staples, src/movetypes.cpp:179)
    void lk_central_domains() {
        std::set<int> staples;
        for (int d : lk_cen) {
            int b = doms[d].bound;
            if (b >= 0 && doms[b].c != 0) scan_for_scaffold(b, staples);
        }
        lk_cdom = lk_cen;
        for (int c : staples)
            for (int id : get_chain(c)) lk_cdom.push_back(id);
    }
    void lk_reset_segment(size_t n) {   // reset_segment (:145)
        for (size_t k = 0; k < n; ++k) {
            unassign_domain(lk_cdom[k]);
            assigned.pop_back();
        }
    }
    bool lk_steps_less() {   // steps_less_than_distance (:524)
        int d1 = lk_end[0] >= 0 ? (doms[lk1[0]].pos - doms[lk_end[0]].pos).abssum() : 0;
        int d2 = lk_end[1] >= 0 ? (doms[lk2[0]].pos - doms[lk_end[1]].pos).abssum() : 0;
        return !(d1 <= (int)lk1.size() && d2 <= (int)lk2.size());
    }
    static V3 lk_rot(V3 v, V3 origin, V3 axis, int turns) {   // VectorThree::rotate(origin, axis, turns)
        if (turns == 0) return v;
        return rotate_quarter(v - origin, axis, turns) + origin;
    }
    // apply_transformation (:401) from the positions in ct_prev_pos
    double lk_apply(V3 disp, V3 center, V3 axis, int turns) {
        double bf = 1, de = 0;
        for (size_t di = 0; di < lk_cdom.size(); ++di) {
            int d = lk_cdom[di];
            V3 p = lk_rot(ct_prev_pos.at(d), center, axis, turns) + disp;
            V3 o = lk_rot(ct_prev_ore.at(d), V3(0, 0, 0), axis, turns);
            int occ = occupancy(p);
            if (occ == BOUND || occ == MISBOUND) {
                lk_reset_segment(di);
                bf = 0;
                break;
            }
            if (occ == UNBOUND) {
                int ud = unbound_at(p);
                bool scaf_mis = doms[d].c == scaffold_c() && doms[ud].c == scaffold_c();
                bool new_pair = !has(lk_cdom, ud);
                if (!scaf_mis && new_pair) {
                    lk_reset_segment(di);
                    bf = 0;
                    break;
                }
                if (scaf_mis && new_pair) {
                    check_domain_constraints(d, p, o);
                    if (violated) {
                        bf = 0;
                        violated = false;
                        lk_reset_segment(di);
                        break;
                    }
                }
            }
            de += set_checked(d, p, o);
            assigned.push_back(key_of(d));
        }
        if (bf != 0) bf = xexp(-de);
        return bf;
    }
    // transform_segment (:316); with rev, revert_transformation (:467)
    double lk_transform(const ScaffoldMoveOpts& mo, bool rev) {
        std::vector<V3> centers, axes, disps;
        std::vector<int> turnss;
        std::vector<double> bfs;
        double bias = 0;
        int K = mo.num_transforms - (rev ? 1 : 0);
        for (int k = 0; k < K; ++k) {
            int ci = rng.uniform_int(0, (int)lk_cen.size() - 1);
            V3 center = ct_prev_pos.at(lk_cen[ci]);
            V3 axis = kBasis[rng.uniform_int(0, 2)];
            int turns = rng.uniform_int(0, mo.max_turns);
            V3 disp;
            disp.x = rng.uniform_int(-mo.max_disp, mo.max_disp);
            disp.y = rng.uniform_int(-mo.max_disp, mo.max_disp);
            disp.z = rng.uniform_int(-mo.max_disp, mo.max_disp);
            double bf = lk_apply(disp, center, axis, turns);
            if (bf != 0) {
                if (!lk_steps_less()) {
                    if (rev) {
                        bias += bf;
                    }
                    else {
                        centers.push_back(center);
                        axes.push_back(axis);
                        turnss.push_back(turns);
                        disps.push_back(disp);
                        bfs.push_back(bf);
                    }
                }
                lk_reset_segment(lk_cdom.size());
            }
        }
        if (rev) {
            for (int d : lk_cdom) {
                double de = set_checked(d, cb_old_pos.at(d), cb_old_ore.at(d));
                bias += xexp(-de);
                assigned.push_back(key_of(d));
            }
            return bias;
        }
        for (double b : bfs) bias += b;
        if (bias == 0) {
            rejected = true;
            return bias;
        }
        double r = bias * rng.uniform_real();
        double cum = 0;
        size_t t = 0;
        for (; t + 1 < bfs.size(); ++t) {
            cum += bfs[t];
            if (r < cum) break;
        }
        lk_apply(disps[t], centers[t], axes[t], turnss[t]);
        return bias;
    }
    // CTCBLinkerRegrowthMCMovetype::internal_attempt_move (:859), also the
    // clustered variant (its selection differs)
    bool ctcb_linker(const ScaffoldMoveOpts& mo, bool clustered) {
        ctcb_reset();
        lk_end[0] = lk_end[1] = -1;
        bool ok = clustered ? lk_select_clustered(mo) : lk_select(mo);
        if (!ok) return false;
        lk_setup_fixed_ends();
        std::set<int> staples = cp.regrowth_staples;
        lk_central_domains();
        std::vector<int> u1(lk1.begin() + 1, lk1.end()), u2(lk2.begin() + 1, lk2.end());
        ctcb_unassign(u1);
        ctcb_unassign(u2);
        for (int c : staples) ctcb_unassign(get_chain(c));
        ctcb_unassign(lk_cdom);
        w_bias.mul(lk_transform(mo, false));
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        ctcb_grow_chain(lk1);
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        ctcb_grow_chain(lk2);
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        update_move_params();   // add_external_bias (:52)
        w_bias.mul(xexp(-calc_move()));
        ctcb_setup_regrow_old();
        cp.active = cp.initial_active;
        ctcb_unassign(u1);
        ctcb_unassign(u2);
        for (int c : staples) ctcb_unassign(get_chain(c));
        ctcb_unassign(lk_cdom);
        w_bias.mul(lk_transform(mo, true));
        ctcb_grow_chain(lk1);
        ctcb_grow_chain(lk2);
        modifier = 1;
        return ctcb_test_acceptance();
    }
    // CTRGLinkerRegrowthMCMovetype::internal_attempt_move (:1148)
    bool ctrg_linker(const ScaffoldMoveOpts& mo) {
        rg_reset();
        lk_end[0] = lk_end[1] = -1;
        rg_max_recoils = mo.max_num_recoils;
        rg_max_c_attempts = mo.max_c_attempts;
        if (!lk_select(mo)) return false;
        lk_setup_fixed_ends();
        lk_central_domains();
        rg_ds = cp.d_stack;
        rg_ds.insert(rg_ds.begin(), lk1.front());
        if (rg_ds.size() < 2) throw std::runtime_error("linker regrowth with nothing to regrow");
        rg_delta_e += rg_unassign_and_save();
        for (int d : lk_cdom) ct_save_unassign(d, nullptr);
        rg_weight *= lk_transform(mo, false);
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        rg_delta_e += recoil_regrow();
        if (rejected) {
            ct_sync_prev();
            return false;
        }
        update_move_params();   // add_external_bias
        rg_delta_e += calc_move();
        // setup_for_calc_new_weights (:137)
        catt_wq = catt_q;
        avail_wq = avail_q;
        rg_old_pos = ct_prev_pos;
        rg_old_ore = ct_prev_ore;
        cb_old_pos = ct_prev_pos;   // the old configuration revert_transformation places
        cb_old_ore = ct_prev_ore;
        modified.clear();
        rg_unassign_and_save();
        cp.active = cp.initial_active;
        rg_calc_weights();
        // old weights
        rg_unassign_domains();
        for (int d : lk_cdom) ct_save_unassign(d, nullptr);
        rg_weight /= lk_transform(mo, true);
        cp.active = cp.initial_active;
        rg_calc_old_c_opens();
        // setup_for_calc_old_weights (:146)
        rg_weight_new = rg_weight;
        rg_weight = 1;
        catt_wq = catt_q;
        avail_wq = avail_q;
        rg_new_pos = ct_prev_pos;
        rg_new_ore = ct_prev_ore;
        modified.clear();
        rg_unassign_and_save();
        for (int d : lk_cdom) modified.push_back(key_of(d));
        cp.active = cp.initial_active;
        rg_calc_weights();
        return rg_test_acceptance();
    }

    // OrientationRotationMCMovetype::internal_attempt_move (src/orientation_movetype.cpp:30)
    bool orientation_rotation() {
        int dom = select_random_domain();
        V3 o_new = kUnit[rng.uniform_int(0, 5)];
        bool acc = false;
        if (doms[dom].state == BOUND || doms[dom].state == MISBOUND) {
            double de = 0;
            V3 o_old = doms[dom].ore;
            int bd = doms[dom].bound;
            de += unassign_domain(bd);
            set_domain_orientation(dom, o_new);
            V3 p = doms[dom].pos;
            de += set_domain_config(bd, p, -o_new);
            if (!violated) acc = test_acceptance(xexp(-de));
            if (!acc) {
                unassign_domain(bd);
                set_domain_orientation(dom, o_old);
                set_checked(bd, p, -o_old);
            }
        }
        else {
            set_domain_orientation(dom, o_new);
            acc = true;
        }
        return acc;
    }

    // GCMCSimulation::simulate step body (src/simulation.cpp:575-619)
    bool step(long long s) {
        double r = rng.uniform_real();
        size_t m = 0;
        for (m = 0; m < cfg.move_cum.size(); ++m)
            if (r < cfg.move_cum[m]) break;
        if (m == cfg.move_cum.size()) throw std::runtime_error("movetype selection fell off the end");
#ifdef ORACLE_COUNT_TOUCHES
        TouchCounts t0 = g_touch;
#endif
        reset_internal();
        bool acc = false;
        switch (cfg.move_kinds[m]) {
        case MV_ORIENTATION: acc = orientation_rotation(); break;
        case MV_MET_EXCHANGE: acc = met_exchange(); break;
        case MV_MET_REGROWTH: acc = met_regrowth(); break;
        case MV_CB_REGROWTH: acc = cb_regrowth(); break;
        case MV_LEARNED_EXCHANGE: acc = learned_exchange(); break;
        case MV_LEARNED_REGROWTH: acc = learned_regrowth(); break;
        case MV_CTRG_SCAFFOLD: acc = ctrg_scaffold(cfg.move_opts[m]); break;
        case MV_CTRG_JUMP: acc = ctrg_jump(cfg.move_opts[m]); break;
        case MV_CTCB_SCAFFOLD: acc = ctcb_scaffold(cfg.move_opts[m]); break;
        case MV_CTCB_JUMP: acc = ctcb_jump(cfg.move_opts[m]); break;
        case MV_CTCB_LINKER: acc = ctcb_linker(cfg.move_opts[m], false); break;
        case MV_CTCB_CLINKER: acc = ctcb_linker(cfg.move_opts[m], true); break;
        case MV_CTRG_LINKER: acc = ctrg_linker(cfg.move_opts[m]); break;
        }
        attempts[m]++;
        if (acc) accepts[m]++;
        if (!acc) {
            reset_origami();
            update_move_params();
            calc_move();
        }
#ifdef ORACLE_COUNT_TOUCHES
        touch_dom[m] += g_touch.dom - t0.dom;
        touch_site[m] += g_touch.site - t0.site;
#endif
        if (cfg.centering_freq != 0 && s % cfg.centering_freq == 0) center(cfg.centering_domain);
        if (cfg.constraint_check_freq != 0 && s % cfg.constraint_check_freq == 0) check_all_constraints();
        return acc;
    }
};

} // namespace oracle
