// Host side of the engine: reads the reference's input files, builds the
// device descriptors and energy tables, lays out one state region per
// replica, launches the kernels and implements the C ABI of include/ldo.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <iterator>
#include <tuple>
#include <vector>

#include "../../include/ldo.h"
#include "ldo_io.hpp"
#include "ldo_kernels.h"
#include "ldo_mlp.h"
#include "ldo_output.hpp"
#include "ldo_tables.hpp"

namespace {

using std::string;
using std::vector;

thread_local string g_create_err;

struct LdoError : std::runtime_error {
    ldo_status code;
    LdoError(ldo_status c, const string& m): std::runtime_error(m), code(c) {}
};

#define CU(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) throw LdoError(LDO_ECUDA, string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
struct DevBuf {
    T* p {nullptr};
    size_t n {0};
    void alloc(size_t count) {
        free();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw LdoError(LDO_ENOMEM, string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        n = count;
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { free(); }
};

int move_kind(const string& t) {
    if (t == "OrientationRotation") return LDO_MV_ORIENT;
    if (t == "MetStapleExchange") return LDO_MV_MET_EXCHANGE;
    if (t == "MetStapleRegrowth") return LDO_MV_MET_REGROWTH;
    if (t == "CBStapleRegrowth") return LDO_MV_CB_REGROWTH;
    if (t == "LearnedStapleExchange") return LDO_MV_LEARNED_EXCHANGE;
    if (t == "LearnedStapleRegrowth") return LDO_MV_LEARNED_REGROWTH;
    if (t == "CTRGScaffoldRegrowth") return LDO_MV_CTRG;
    if (t == "CTRGJumpScaffoldRegrowth") return LDO_MV_CTRG_JUMP;
    if (t == "CTCBScaffoldRegrowth") return LDO_MV_CTCB;
    if (t == "CTCBJumpScaffoldRegrowth") return LDO_MV_CTCB_JUMP;
    if (t == "CTCBLinkerRegrowth") return LDO_MV_CTCB_LINKER;
    if (t == "CTCBClusteredLinkerRegrowth") return LDO_MV_CTCB_CLINKER;
    if (t == "CTRGLinkerRegrowth") return LDO_MV_CTRG_LINKER;
    // accepted by the reference's type check but never constructed there
    // (GCMCSimulation::setup_scaffold_transform_movetype, src/simulation.cpp:445)
    if (t == "CTRGClusteredLinkerRegrowth")
        throw LdoError(LDO_EINVAL, t + ": the reference builds no such movetype");
    throw LdoError(LDO_EINVAL, t + ": no such movetype");
}

// One input system (one .inp file) on the host.
struct HostSystem {
    ldo_io::Params p;
    ldo_io::SystemFile sf;
    vector<ldo_io::MoveSpec> moves;
    vector<ldo_io::OpSpec> ops;
    vector<ldo_io::BiasSpec> biases;
    LdoSys desc {};
    ldo_host::EnergyInputs energy;
};

HostSystem load_system(const string& inp, const string& overrides) {
    HostSystem hs;
    ldo_io::Params& p = hs.p;
    try {
        p = ldo_io::read_inp(inp);
        if (!overrides.empty()) {
            std::istringstream is(overrides);
            string line;
            while (std::getline(is, line)) {
                auto h = line.find('#');
                if (h != string::npos) line = line.substr(0, h);
                auto eq = line.find('=');
                if (eq == string::npos) continue;
                ldo_io::set_param(p, ldo_io::trim(line.substr(0, eq)), ldo_io::trim(line.substr(eq + 1)));
            }
        }
        hs.sf = ldo_io::read_system(ldo_io::resolve(p, p.origami_input_filename));
        // setup_origami (src/origami_system.cpp:1000-1003): the configuration
        // of frame restart_step of a trajectory replaces the system file's
        if (!p.restart_traj_file.empty())
            hs.sf.chains = ldo_io::read_trj_frame(ldo_io::resolve(p, p.restart_traj_file), p.restart_step);
        hs.moves = ldo_io::read_movetypes(ldo_io::resolve(p, p.movetype_file));
        if (!p.order_parameter_file.empty()) hs.ops = ldo_io::read_ops(ldo_io::resolve(p, p.order_parameter_file));
        if (!p.bias_functions_file.empty())
            hs.biases = ldo_io::read_biases(ldo_io::resolve(p, p.bias_functions_file));
    } catch (LdoError&) {
        throw;
    } catch (std::exception& e) {
        throw LdoError(LDO_EINVAL, e.what());
    }
    if (p.domain_type != "HalfTurn" && p.domain_type != "ThreeQuarterTurn")
        throw LdoError(LDO_EINVAL, p.domain_type + ": No such domain type");
    if (p.binding_pot != "FourBody") throw LdoError(LDO_EINVAL, p.binding_pot + ": No such binding potential");
    if (p.misbinding_pot != "Opposing" && p.misbinding_pot != "Disallowed")
        throw LdoError(LDO_EINVAL, p.misbinding_pot + ": No such misbinding potential");
    if (p.domain_update_biases_present)
        throw LdoError(LDO_EINVAL, "domain_update_biases_present: per-domain biases are not implemented by this engine");

    const auto& ids = hs.sf.identities;
    if (ids.size() < 2) throw LdoError(LDO_EINVAL, "system needs a scaffold and at least one staple type");
    if (ids.size() > LDO_MAX_TYPES) throw LdoError(LDO_EINVAL, "too many staple types");
    if (hs.sf.chains.empty() || hs.sf.chains[0].identity != 0)
        throw LdoError(LDO_EINVAL, "first configuration chain must be the scaffold");
    LdoSys& d = hs.desc;
    std::memset(&d, 0, sizeof d);
    d.n_types = (int)ids.size();
    d.ns = (int)ids[0].size();
    d.lmax = 1;
    int noff = 0;
    for (size_t t = 0; t < ids.size(); ++t) {
        d.type_len[t] = (int)ids[t].size();
        d.type_off[t] = noff;
        if (t > 0) d.lmax = std::max(d.lmax, (int)ids[t].size());
        for (int x : ids[t]) {
            if (noff >= LDO_MAX_IDENTS) throw LdoError(LDO_EINVAL, "too many domain identities");
            d.idents[noff++] = (int16_t)x;
            d.imax = std::max(d.imax, std::abs(x));
        }
    }
    if (d.lmax > LDO_MAX_LEN) throw LdoError(LDO_EINVAL, "staples longer than 4 domains are not supported");
    d.dim = 2 * d.imax + 1;
    int kmax_default = std::min(LDO_MAX_KMAX, d.ns * 2);
    d.kmax = std::min(p.max_total_staples, LDO_MAX_KMAX);
    if (p.max_total_staples > LDO_MAX_KMAX) d.kmax = kmax_default;
    if ((int)hs.sf.chains.size() - 1 > d.kmax)
        throw LdoError(LDO_ECAPACITY, "initial configuration has more staples than staple slots");
    d.dcap = d.ns + d.kmax * d.lmax;
    if (d.dcap > 4000) throw LdoError(LDO_EINVAL, "system too large");
    d.cyclic = hs.sf.cyclic;
    d.tqt = p.domain_type == "ThreeQuarterTurn";
    d.mis_disallowed = p.misbinding_pot == "Disallowed";
    d.mean_field = p.apply_mean_field_cor;
    d.max_total_staples = p.max_total_staples;
    d.max_type_staples = p.max_type_staples;
    if ((int)hs.moves.size() > LDO_MAX_MOVES) throw LdoError(LDO_EINVAL, "too many movetypes");
    d.n_moves = (int)hs.moves.size();
    double cum = 0;
    for (int t = 0; t < LDO_MAX_TYPES; ++t) d.exchange_mults[t] = 1;
    for (size_t m = 0; m < hs.moves.size(); ++m) {
        d.move_kind[m] = move_kind(hs.moves[m].type);
        cum += hs.moves[m].freq;
        d.move_cum[m] = cum;
        const ldo_io::MoveSpec& ms = hs.moves[m];
        d.move_opt[m][LDO_MO_MAX_REGROWTH] = ms.max_regrowth;
        d.move_opt[m][LDO_MO_MAX_SEG_REGROWTH] = ms.max_seg_regrowth;
        d.move_opt[m][LDO_MO_MAX_RECOILS] = ms.max_num_recoils;
        d.move_opt[m][LDO_MO_MAX_C_ATTEMPTS] = ms.max_c_attempts;
        d.move_opt[m][LDO_MO_MAX_DISP] = ms.max_disp;
        d.move_opt[m][LDO_MO_MAX_TURNS] = ms.max_turns;
        d.move_opt[m][LDO_MO_MAX_LINKER] = ms.max_linker_length;
        d.move_opt[m][LDO_MO_NUM_TRANSFORMS] = ms.num_transforms;
        int k = d.move_kind[m];
        if (k >= LDO_MV_CTCB_LINKER && k <= LDO_MV_CTRG_LINKER) {
            d.has_ct = 1;
            // uniform_int(2, max_linker_length + 1) for the linker lengths,
            // uniform_int(1, min(ns, max_regrowth)) for the central segment
            // (src/transform_movetypes.cpp:156, src/movetypes.cpp:469), and
            // the clustered kernel domain uniform_int(1, ns - 2) (:670)
            if (ms.num_transforms < 1 || ms.num_transforms > LDO_CT_MAX_TRANSFORMS)
                throw LdoError(LDO_EINVAL, ms.type + ": num_transforms must be 1.." +
                                               std::to_string(LDO_CT_MAX_TRANSFORMS));
            if (ms.max_disp < 0 || ms.max_turns < 0 || ms.max_linker_length < 1)
                throw LdoError(LDO_EINVAL, ms.type + ": max_disp and max_turns must not be negative and "
                                                     "max_linker_length must be positive");
            if (d.ns < 3) throw LdoError(LDO_EINVAL, ms.type + ": the scaffold needs at least 3 domains");
            if (k != LDO_MV_CTCB_CLINKER && ms.max_regrowth < 1)
                throw LdoError(LDO_EINVAL, ms.type + ": max_regrowth must be at least 1");
            if (k == LDO_MV_CTRG_LINKER && (ms.max_c_attempts < 1 || ms.max_c_attempts > 36 || ms.max_num_recoils < 0))
                throw LdoError(LDO_EINVAL, ms.type + ": max_c_attempts must be 1..36 and max_num_recoils >= 0");
        }
        if (k >= LDO_MV_CTRG && k <= LDO_MV_CTCB_JUMP) {
            d.has_ct = 1;
            // the reference draws uniform_int(2, max_regrowth) and keeps at
            // most 36 untried configurations per domain (src/movetypes.cpp:479,
            // src/rg_movetypes.cpp:298)
            if (ms.max_regrowth < 2) throw LdoError(LDO_EINVAL, ms.type + ": max_regrowth must be at least 2");
            if (d.ns < 2) throw LdoError(LDO_EINVAL, ms.type + ": the scaffold needs at least 2 domains");
            if ((k == LDO_MV_CTRG_JUMP || k == LDO_MV_CTCB_JUMP) && ms.max_seg_regrowth < 0)
                throw LdoError(LDO_EINVAL, ms.type + ": max_seg_regrowth must not be negative");
            if ((k == LDO_MV_CTRG || k == LDO_MV_CTRG_JUMP) &&
                (ms.max_c_attempts < 1 || ms.max_c_attempts > 36 || ms.max_num_recoils < 0))
                throw LdoError(LDO_EINVAL, ms.type + ": max_c_attempts must be 1..36 and max_num_recoils >= 0");
        }
        if (d.move_kind[m] == LDO_MV_LEARNED_EXCHANGE && d.ns > LDO_MAX_SCAF)
            throw LdoError(LDO_EINVAL, "LearnedStapleExchange: scaffold longer than 320 domains");
        if (d.move_kind[m] == LDO_MV_MET_EXCHANGE || d.move_kind[m] == LDO_MV_LEARNED_EXCHANGE) {
            for (size_t t = 0; t < hs.moves[m].exchange_mults.size() && t < LDO_MAX_TYPES; ++t)
                d.exchange_mults[t] = hs.moves[m].exchange_mults[t];
            d.adaptive_exchange = hs.moves[m].adaptive_exchange;
            if (d.adaptive_exchange)
                for (size_t t = 0; t < hs.moves[m].exchange_mults.size(); ++t)
                    if (hs.moves[m].exchange_mults[t] != 1)
                        throw LdoError(LDO_EINVAL, "adaptive_exchange with exchange multipliers is not implemented");
        }
    }
    d.allow_nonsensical = p.allow_nonsensical_ps;
    // complementary staple domain of each scaffold domain (first in type order)
    for (int k = 0; k < d.ns && k < LDO_MAX_SCAF; ++k) {
        int id = ids[0][k];
        for (size_t t = 1; t < ids.size() && !d.comp_type[k]; ++t)
            for (size_t q = 0; q < ids[t].size(); ++q)
                if (ids[t][q] == -id) {
                    d.comp_type[k] = (uint8_t)t;
                    d.comp_dom[k] = (uint8_t)q;
                    d.learn_tslot[k] = (uint8_t)ldo_learn_tslot((int)t);
                    break;
                }
    }
    if (hs.ops.size() > LDO_MAX_OPS) throw LdoError(LDO_EINVAL, "too many order parameters");
    d.n_ops = (int)hs.ops.size();
    d.fully_op = -1;
    for (size_t q = 0; q < hs.ops.size(); ++q) {
        const auto& o = hs.ops[q];
        int k;
        if (o.type == "NumStaples") k = LDO_OP_NUMSTAPLES;
        else if (o.type == "NumStaplesType") k = LDO_OP_NUMSTAPLESTYPE;
        else if (o.type == "StapleTypeFullyBound") k = LDO_OP_STAPLETYPEFULLYBOUND;
        else if (o.type == "NumBoundDomainPairs") k = LDO_OP_NUMBOUND;
        else if (o.type == "NumMisboundDomainPairs") k = LDO_OP_NUMMISBOUND;
        else if (o.type == "NumStackedPairs") k = LDO_OP_NUMSTACKED;
        else if (o.type == "NumLinearHelices" || o.type == "NumStackedJuncts") k = LDO_OP_ZERO;
        else if (o.type == "Sum") k = LDO_OP_SUM;
        else if (o.type == "Dist") k = LDO_OP_DIST;
        else if (o.type == "AdjacentSite") k = LDO_OP_ADJACENT;
        else throw LdoError(LDO_EINVAL, o.type + ": order parameter type does not exist");
        d.op_kind[q] = k;
        d.op_arg[q] = o.staple;
        if (k == LDO_OP_NUMSTAPLESTYPE || k == LDO_OP_STAPLETYPEFULLYBOUND)
            if (o.staple < 1 || o.staple >= d.n_types) throw LdoError(LDO_EINVAL, "order parameter staple out of range");
        if (k == LDO_OP_NUMBOUND && d.fully_op < 0) d.fully_op = (int)q;
        if (k == LDO_OP_DIST || k == LDO_OP_ADJACENT) {
            // the pair of domains (chain index, domain index) the reference
            // looks up once at set-up (SystemOrderParams::setup_ops,
            // src/order_params.cpp:495-512); this engine takes scaffold domains
            // and the move-level update (update_per_domain false)
            int sc = hs.sf.chains.empty() ? 0 : hs.sf.chains[0].index;
            if (o.update_per_domain)
                throw LdoError(LDO_EINVAL, o.type + " order parameter " + o.tag +
                                                   ": update_per_domain is not supported by this engine");
            if (o.chain1 != sc || o.chain2 != sc)
                throw LdoError(LDO_EINVAL, o.type + " order parameter " + o.tag +
                                                   ": this engine takes scaffold domains only");
            if (o.domain1 < 0 || o.domain1 >= d.ns || o.domain2 < 0 || o.domain2 >= d.ns)
                throw LdoError(LDO_EINVAL, o.type + " order parameter " + o.tag + ": domain out of range");
            d.op_nparts[q] = 2;
            d.op_parts[q][0] = o.domain1;
            d.op_parts[q][1] = o.domain2;
        }
        if (k == LDO_OP_SUM) {
            if (o.ops.size() > LDO_MAX_PARTS) throw LdoError(LDO_EINVAL, "Sum over too many order parameters");
            d.op_nparts[q] = (int)o.ops.size();
            for (size_t a = 0; a < o.ops.size(); ++a) {
                int idx = -1;
                for (size_t r = 0; r < q; ++r)
                    if (hs.ops[r].tag == o.ops[a]) idx = (int)r;
                if (idx < 0) throw LdoError(LDO_EINVAL, "Sum order parameter: unknown tag " + o.ops[a]);
                d.op_parts[q][a] = idx;
            }
        }
    }
    if (hs.biases.size() > LDO_MAX_BIASES) throw LdoError(LDO_EINVAL, "too many bias functions");
    d.n_biases = (int)hs.biases.size();
    for (size_t b = 0; b < hs.biases.size(); ++b) {
        const auto& s = hs.biases[b];
        if (s.type == "LinearStepWell") d.bias_kind[b] = LDO_B_LINEARSTEPWELL;
        else if (s.type == "SquareWell") d.bias_kind[b] = LDO_B_SQUAREWELL;
        else if (s.type == "Grid") d.bias_kind[b] = LDO_B_GRID;
        else if (s.type == "Harmonic") d.bias_kind[b] = LDO_B_HARMONIC;
        else throw LdoError(LDO_EINVAL, s.type + "; no such bias function type");
        if (s.ops.size() != 1) throw LdoError(LDO_EINVAL, "bias functions over several order parameters are not implemented");
        int idx = -1;
        for (size_t r = 0; r < hs.ops.size(); ++r)
            if (hs.ops[r].tag == s.ops[0]) idx = (int)r;
        if (idx < 0) throw LdoError(LDO_EINVAL, "bias function " + s.tag + ": unknown order parameter " + s.ops[0]);
        d.bias_op[b] = idx;
        d.bias_nops[b] = 1;
        d.bias_min[b] = s.min_op;
        d.bias_max[b] = s.max_op;
        d.bias_well[b] = s.well_bias;
        d.bias_minb[b] = s.min_bias;
        d.bias_slope[b] = s.slope;
        d.bias_outside[b] = s.outside_bias;
        d.bias_k[b] = s.k;
        d.bias_centre[b] = s.centre;
        d.bias_grid_len[b] = d.bias_kind[b] == LDO_B_GRID ? (d.ns + d.kmax * d.lmax + 1) : 0;
    }
    d.bias_mult = p.bias_functions_mult;
    d.centering_freq = p.centering_freq;
    d.centering_domain = p.centering_domain;
    if (p.centering_domain < 0 || p.centering_domain >= d.ns) throw LdoError(LDO_EINVAL, "centering_domain out of range");
    d.constraint_check_freq = p.constraint_check_freq;

    ldo_host::EnergyInputs& en = hs.energy;
    en.hybridization_pot = p.hybridization_pot;
    en.stacking_pot = p.stacking_pot;
    en.mean_field = p.apply_mean_field_cor;
    en.temp = p.temp;
    en.cation_M = p.cation_M;
    en.stacking_ene = p.stacking_ene;
    en.binding_h = p.binding_h;
    en.binding_s = p.binding_s;
    en.misbinding_h = p.misbinding_h;
    en.misbinding_s = p.misbinding_s;
    en.enthalpies = hs.sf.enthalpies;
    en.entropies = hs.sf.entropies;
    return hs;
}

int next_pow2(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

template <class C>
LdoLayout layout_of(int cls) {
    using S = LdoState<C>;
    LdoLayout y {};
    y.cls = cls;
    y.bytes = (int)sizeof(S);
    y.o_hdr = (int)offsetof(S, hdr);
    y.o_hash = (int)offsetof(S, hash);
    y.o_bias = (int)offsetof(S, bias);
    y.o_mstat = (int)offsetof(S, mstat);
    y.o_chain_c = (int)offsetof(S, chain_c);
    y.o_op = (int)offsetof(S, op);
    y.o_pp = (int)offsetof(S, pp);
    y.o_nxt = (int)offsetof(S, nxt);
    y.o_prv = (int)offsetof(S, prv);
    y.o_bound = (int)offsetof(S, bnd);
    y.o_dident = (int)offsetof(S, did);
    y.o_type_count = (int)offsetof(S, type_count);
    y.o_ore = (int)offsetof(S, ore);
    y.o_state = (int)offsetof(S, st);
    y.o_slot_cs = (int)offsetof(S, scs);
    y.o_slot_d = (int)offsetof(S, sd);
    y.o_chain_type = (int)offsetof(S, chain_type);
    y.o_chain_order = (int)offsetof(S, chain_order);
    y.o_clen = (int)offsetof(S, clen);
    y.dcap = C::DCAP;
    y.kmax = C::KMAX;
    y.hcap = C::HCAP;
    y.ntypes = C::NT;
    y.nb = C::NB;
    y.nop = C::NOP;
    y.nmv = C::NMV;
    return y;
}

// Smallest capacity class that holds every system of the batch (the occupancy
// hash gets at least twice as many entries as domain slots).
LdoLayout make_layout(int dcap, int kmax, int ntypes, int nb, int nop, int nmv) {
    if (ntypes > LDO_MAX_TYPES || nb > LDO_MAX_BIASES || nop > LDO_MAX_OPS || nmv > LDO_MAX_MOVES)
        throw LdoError(LDO_EINVAL, "system exceeds the engine's descriptor limits");
    if (dcap <= LdoCapS::DCAP && kmax <= LdoCapS::KMAX && 2 * dcap <= LdoCapS::HCAP) return layout_of<LdoCapS>(LDO_CLASS_S);
    if (dcap <= LdoCapM::DCAP && kmax <= LdoCapM::KMAX && 2 * dcap <= LdoCapM::HCAP) return layout_of<LdoCapM>(LDO_CLASS_M);
    if (dcap <= LdoCapL::DCAP && kmax <= LdoCapL::KMAX && 2 * dcap <= LdoCapL::HCAP) return layout_of<LdoCapL>(LDO_CLASS_L);
    throw LdoError(LDO_ECAPACITY, "system needs more domain or staple slots than the largest capacity class");
}

} // namespace

// Seeded initial network parameters: uniform(-a, a) with a = sqrt(6 / (fan_in
// + fan_out)) for the weight matrices, zero biases (splitmix64 stream).
vector<float> ldo_learn_init_params(uint32_t seed) {
    vector<float> p(LDO_LEARN_NPARAM, 0.f);
    unsigned long long x = 0x9E3779B97F4A7C15ull * (seed + 1ull);
    auto next = [&]() {
        x += 0x9E3779B97F4A7C15ull;
        unsigned long long z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * 0x1.0p-53;
    };
    auto fill = [&](int off, int fan_in, int fan_out) {
        double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int i = 0; i < fan_in * fan_out; ++i) p[off + i] = (float)((2 * next() - 1) * a);
    };
    fill(LDO_LEARN_OFF_W1, LDO_LEARN_DIN, LDO_LEARN_H);
    fill(LDO_LEARN_OFF_W2, LDO_LEARN_H, LDO_LEARN_H);
    fill(LDO_LEARN_OFF_W3, LDO_LEARN_H, LDO_LEARN_H);
    fill(LDO_LEARN_OFF_W4, LDO_LEARN_H, 1);
    return p;
}

// Neumaier's compensated summation (value() is the sum without the drift a
// running double sum accumulates)
struct CompSum {
    double s = 0, c = 0;
    void add(double x) {
        double t = s + x;
        c += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    double value() const { return s + c; }
};

// Work units of the exact staple-only enumeration, in the order the reference
// walks them: StapleEnumerator::enumerate / recurse (src/enumerate.cpp:1082,
// :1103) over staple sets, and for each set GrowthpointEnumerator::enumerate
// (:819) with the misbinding (:869-966) or no-misbinding (:968-1067) rules,
// skipping growth-point sets enumerated before (growthpoints_repeated).  Each
// unit is one call of the reference's conformational enumeration.
struct EnumBuilder {
    typedef std::pair<int, int> DRef;                  // (chain, domain); chain -1: scaffold
    typedef std::tuple<int, int, int, int> GP;         // (staple identity, domain, old chain, old domain)
    const vector<vector<int>>& ids;                    // identities of each chain type (0: scaffold)
    int S;
    bool misbinding;
    size_t max_units;
    vector<LdoEnumUnit> units;
    vector<int> chains;                                // identity of the k-th added staple
    std::map<int, vector<int>> id_to_idx;              // m_identity_to_indices
    vector<std::pair<int, int>> staples;               // m_staples
    vector<DRef> usd;                                  // misbinding: m_unbound_system_domains
    vector<vector<DRef>> usd_nm;                       // no misbinding: per staple identity
    std::map<DRef, DRef> gmap;                         // m_growthpoints
    vector<GP> gp;                                     // m_growthpoints of the growth-point enumerator
    // m_enumerated_growthpoints, each set sorted.  The reference tests a new
    // set against every enumerated one of its size for containment; the
    // growth points of one set are distinct (each old domain is taken out of
    // the candidates while it is in use), so containment at equal size is
    // set equality, looked up here in logarithmic time
    std::set<vector<GP>> enumerated;

    EnumBuilder(const vector<vector<int>>& identities, bool mis, size_t cap)
        : ids(identities), S((int)identities.size() - 1), misbinding(mis), max_units(cap) {
        int ns = (int)ids[0].size();
        for (int d = 0; d < ns; ++d) usd.push_back({-1, d});
        // OrigamiSystem::initialize_complementary_associations (src/origami_system.cpp:630)
        usd_nm.resize(S);
        for (int t = 1; t <= S; ++t)
            for (int di : ids[t]) {
                auto it = std::find(ids[0].begin(), ids[0].end(), -di);
                if (it != ids[0].end()) usd_nm[t - 1].push_back({-1, (int)(it - ids[0].begin())});
            }
    }

    void emit() {
        if (units.size() >= max_units) throw LdoError(LDO_EINVAL, "enumeration: too many growth-point sets");
        if (gmap.size() > LDO_ENUM_MAX_STAPLES) throw LdoError(LDO_EINVAL, "enumeration: too many growth points");
        LdoEnumUnit u {};
        u.n_chains = (int)chains.size();
        for (size_t k = 0; k < chains.size(); ++k) u.ident[k] = chains[k];
        u.n_gp = 0;
        for (auto& kv : gmap) {
            u.gp_old_chain[u.n_gp] = kv.first.first;
            u.gp_old_dom[u.n_gp] = kv.first.second;
            u.gp_new_chain[u.n_gp] = kv.second.first;
            u.gp_new_dom[u.n_gp] = kv.second.second;
            ++u.n_gp;
        }
        units.push_back(u);
    }

    vector<GP> sorted_gp() const {
        vector<GP> key(gp);
        std::sort(key.begin(), key.end());
        return key;
    }
    bool repeated() const { return enumerated.count(sorted_gp()) != 0; }   // growthpoints_repeated (:944, :1046)

    void recurse_or_enumerate(int ident, int d_i, DRef old) {
        int L = (int)ids[ident].size();
        gp.push_back(GP {ident, d_i, old.first < 0 ? -1 : old.first + 1, old.second});
        // ConformationalEnumerator::add_growthpoint (:317)
        int k = id_to_idx[ident].back();
        id_to_idx[ident].pop_back();
        gmap[old] = DRef {k, d_i};
        if (!staples.empty()) {
            if (misbinding) {
                for (int d = 0; d < L; ++d)
                    if (d != d_i) usd.push_back({k, d});
            }
            iterate_staple_identities();
            if (misbinding)
                for (int d = 0; d + 1 < L; ++d) usd.pop_back();
        }
        else if (!repeated()) {
            emit();
            enumerated.insert(sorted_gp());
        }
        // remove_growthpoint (:336)
        DRef nw = gmap[old];
        gmap.erase(old);
        id_to_idx[chains[nw.first]].push_back(nw.first);
        gp.pop_back();
    }

    void iterate_domain_growthpoints(int ident) {
        int L = (int)ids[ident].size();
        vector<DRef>& lst = misbinding ? usd : usd_nm[ident - 1];
        for (size_t j = 0; j != lst.size(); ++j) {
            DRef old = lst[j];
            lst.erase(lst.begin() + j);
            for (int d_i = 0; d_i < L; ++d_i) {
                if (!misbinding && ids[ident][d_i] != -ids[0][old.second]) continue;
                recurse_or_enumerate(ident, d_i, old);
            }
            lst.insert(lst.begin() + j, old);
        }
    }

    void iterate_staple_identities() {   // :834
        for (size_t i = 0; i != staples.size(); ++i) {
            int ident = staples[i].first;
            int rem = staples[i].second - 1;
            if (rem == 0) staples.erase(staples.begin() + i);
            else staples[i] = {ident, rem};
            iterate_domain_growthpoints(ident);
            bool found = false;
            for (auto& st : staples)
                if (st.first == ident) {
                    st.second++;
                    found = true;
                    break;
                }
            if (!found) staples.insert(staples.begin() + i, {ident, rem + 1});
        }
    }

    void growthpoints() {   // GrowthpointEnumerator::enumerate (:819)
        enumerated.clear();
        staples.clear();
        for (int t = 1; t <= S; ++t) {
            int n = (int)std::count(chains.begin(), chains.end(), t);
            if (n) staples.push_back({t, n});
        }
        iterate_staple_identities();
    }

    void recurse(int cur, int type_i, int cur_i, int cur_max, int max_type) {   // :1103
        if (cur == cur_max) {
            growthpoints();
            return;
        }
        while (type_i != S + 1) {
            if (cur_i < max_type) {
                chains.push_back(type_i);
                id_to_idx[type_i].push_back((int)chains.size() - 1);
                recurse(cur + 1, type_i, cur_i + 1, cur_max, max_type);
                id_to_idx[type_i].pop_back();
                chains.pop_back();
            }
            type_i++;
            cur_i = 0;
        }
    }

    void run(int min_total, int max_total, int max_type) {   // :1082
        if (max_total > LDO_ENUM_MAX_STAPLES) throw LdoError(LDO_EINVAL, "enumeration: at most 8 staples");
        int cur_max;
        if (min_total == 0) {
            emit();
            cur_max = 1;
        }
        else {
            cur_max = min_total;
        }
        for (; cur_max <= max_total; ++cur_max) recurse(0, 1, 0, cur_max, max_type);
    }
};

struct ldo_engine {
    string err;
    vector<HostSystem> systems;
    vector<int> sys_of;
    int n_rep {0};
    uint32_t seed {0};
    LdoLayout lay {};
    int wpb {1};
    int smem_pad {0};
    cudaStream_t stream {nullptr};
    cudaEvent_t ev0 {nullptr}, ev1 {nullptr};
    // Every host-device copy of the engine is ordered on its stream and
    // complete when this returns.  The stream is non-blocking, so a copy on
    // the legacy default stream (plain cudaMemcpy) would be ordered with none
    // of the engine's kernels, and a pageable host-to-device cudaMemcpy may
    // return before its transfer has finished.
    cudaError_t copy(void* dst, const void* src, size_t n, cudaMemcpyKind kind) {
        if (n == 0) return cudaSuccess;
        count_copy(n, kind);
        cudaError_t err = cudaMemcpyAsync(dst, src, n, kind, stream);
        if (err != cudaSuccess) return err;
        return cudaStreamSynchronize(stream);
    }

    // Counters of the engine's own work (ldo_get_counters): kernel launches
    // (the MC, exchange, status and enumeration kernels; a replayed graph
    // counts its kernels) and bytes copied between host and device.
    long long n_launches {0}, bytes_h2d {0}, bytes_d2h {0};
    bool capturing {false};
    void count_copy(size_t n, cudaMemcpyKind kind) {
        if (kind == cudaMemcpyHostToDevice) bytes_h2d += (long long)n;
        else if (kind == cudaMemcpyDeviceToHost) bytes_d2h += (long long)n;
    }
    void count_launch(int k = 1) {
        if (!capturing) n_launches += k;
    }
    cudaError_t launch_mc(const LdoLaunch& L) {
        count_launch();
        return ldo_launch_mc(L, stream);
    }

    vector<LdoSys> h_sys;
    vector<LdoTab> h_tabs;
    vector<double> h_bank;
    std::map<std::tuple<int, double, double>, int> tab_index;
    vector<LdoRepCtl> h_ctl;
    vector<double> h_grid;
    vector<double> temps, stack_mults, u_mults;

    DevBuf<LdoSys> d_sys;
    DevBuf<LdoTab> d_tabs;
    DevBuf<double> d_bank;
    DevBuf<LdoRepCtl> d_ctl;
    DevBuf<double> d_grid;
    DevBuf<unsigned char> d_arena;
    DevBuf<unsigned char> d_snap;   // move snapshots (run mode)
    DevBuf<unsigned char> d_ct;     // scaffold regrowth working memory
    size_t ct_stride {0};
    // learned insertion proposal: weight table, training counts, network
    DevBuf<double> d_learn_w;
    DevBuf<double> d_cnt_b, d_cnt_t;
    LdoMlp mlp;
    bool mlp_init {false};
    DevBuf<int> d_status;
    DevBuf<int> d_rep_map;          // autotuner's replica order (warp -> replica)
    bool use_rep_map {false};
    DevBuf<int16_t> d_samples;
    DevBuf<double> d_trace;
    int sample_interval {0}, sample_cap {0};
    int n_trace {0}, trace_max {0};

    // parallel tempering
    int pt_rungs {0}, pt_q {0};
    long long pt_swap_i {0};
    DevBuf<double> d_slot_q, d_red_u, d_rep_q;
    DevBuf<int> d_perm, d_tab_slot;
    DevBuf<unsigned long long> d_pt_draws;
    DevBuf<long long> d_pt_att, d_pt_acc;
    DevBuf<int> d_pt_sched;
    int pt_dim2 {0}, pt_nctr {0};
    vector<double> pt_slot_q;          // host copy of the slots' controls (4 x n_rungs)
    // swap history (.swp): ring of hist_cap rows per ladder
    DevBuf<int> d_hist_perm;
    DevBuf<long long> d_hist_step, d_hist_n;
    long long hist_cap {0};
    cudaGraphExec_t pt_graph {nullptr};
    LdoPT pt {};

    // umbrella sampling (one SimpleUS state per window)
    struct USWindow {
        int min_op {0}, max_op {0};
        std::vector<double> E_w;        // bias per grid point (0 off grid)
        std::vector<char> in_S;         // point visited in an earlier iteration (m_S_n)
        std::vector<char> in_file;      // point read from a .biases file (an entry of m_E_w)
    };
    std::vector<USWindow> us_win;
    string us_tag;                      // grid bias of the current US state (empty: none)
    long long us_iters_done {0};
    std::vector<int> us_window_of;      // replica -> window
    std::vector<int> us_replica_of;     // window -> replica
    DevBuf<int> d_us_hist, d_us_window;
    int us_bias {-1}, us_len {0}, us_sq_bias {-1};
    unsigned long long us_swap_draws {0};
    std::vector<long long> us_att, us_acc;

    ~ldo_engine() {
        ldo_mlp_free(mlp);
        if (pt_graph) cudaGraphExecDestroy(pt_graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int table_for(int s, double temp, double mult) {
        auto key = std::make_tuple(s, temp, mult);
        auto it = tab_index.find(key);
        if (it != tab_index.end()) return it->second;
        HostSystem& hs = systems[s];
        ldo_host::EnergyInputs in = hs.energy;
        in.temp = temp;
        in.stacking_mult = mult;
        ldo_host::Tables t;
        try {
            t = ldo_host::build_tables(hs.sf.identities, hs.sf.sequences, in);
        } catch (std::exception& e) {
            throw LdoError(LDO_EINVAL, e.what());
        }
        LdoTab d {};
        d.dense = t.dense;
        d.stack_dense = t.stack_dense;
        d.off_e = (long long)h_bank.size();
        h_bank.insert(h_bank.end(), t.e.begin(), t.e.end());
        d.off_h = (long long)h_bank.size();
        h_bank.insert(h_bank.end(), t.h.begin(), t.h.end());
        d.off_s = (long long)h_bank.size();
        h_bank.insert(h_bank.end(), t.s.begin(), t.s.end());
        d.off_stack = -1;
        if (t.stack_dense) {
            d.off_stack = (long long)h_bank.size();
            h_bank.insert(h_bank.end(), t.stack.begin(), t.stack.end());
        }
        d.stack_const = t.stack_const;
        d.init_e = t.init_e;
        d.init_h = t.init_h;
        d.init_s = t.init_s;
        d.temp = temp;
        int idx = (int)h_tabs.size();
        h_tabs.push_back(d);
        tab_index[key] = idx;
        return idx;
    }

    void upload_tables() {
        d_tabs.alloc(h_tabs.size());
        CU(copy(d_tabs.p, h_tabs.data(), h_tabs.size() * sizeof(LdoTab), cudaMemcpyHostToDevice));
        d_bank.alloc(h_bank.size());
        CU(copy(d_bank.p, h_bank.data(), h_bank.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    void upload_ctl() {
        CU(copy(d_ctl.p, h_ctl.data(), h_ctl.size() * sizeof(LdoRepCtl), cudaMemcpyHostToDevice));
    }
    void upload_grid() {
        if (h_grid.empty()) return;
        CU(copy(d_grid.p, h_grid.data(), h_grid.size() * sizeof(double), cudaMemcpyHostToDevice));
    }

    LdoLaunch launch_params(int mode, long long steps) {
        LdoLaunch L {};
        L.sys = d_sys.p;
        L.tabs = d_tabs.p;
        L.bank = d_bank.p;
        L.ctl = d_ctl.p;
        L.grid = d_grid.p;
        L.arena = d_arena.p;
        L.snap = d_snap.p;
        L.ct_ws = d_ct.p;
        L.ct_stride = ct_stride;
        L.lay = lay;
        L.n_rep = n_rep;
        L.only_rep = -1;
        L.warps_per_block = wpb;
        L.smem_pad = smem_pad;
        L.mode = mode;
        L.want_dep = 0;
        L.n_steps = steps;
        L.sample_interval = sample_interval;
        L.sample_cap = sample_cap;
        L.samples = d_samples.p;
        L.n_trace = n_trace;
        L.trace_max = trace_max;
        L.trace = d_trace.p;
        L.us_hist = nullptr;
        L.us_window = nullptr;
        L.learn_w = d_learn_w.p;
        L.learn_cnt_b = d_cnt_b.p;
        L.learn_cnt_t = d_cnt_t.p;
        L.rep_map = use_rep_map ? d_rep_map.p : nullptr;
        return L;
    }

    // ------------------------------------------------------- autotuner ---
    // The engine's own autotuner of the MC kernel's launch shape (no
    // counterpart in the reference).  Knobs: warps (replicas) per block, the
    // number of resident blocks per SM (set through extra dynamic shared
    // memory per block), and the replica order (as given, or interleaved over
    // the systems so that every block and SM holds a mix of sizes).  Every
    // candidate is timed on probe_sweeps sweeps of the engine's own batch,
    // best of two, and the replicas' state is restored after every probe, so
    // tuning leaves the trajectories exactly those of an untuned engine.  The
    // choice is kept per (capacity class, kernel variant, systems, replica
    // count) for the life of the process.
    struct TuneCand {
        int wpb, pad, blocks, order;
        double ms;
    };
    vector<TuneCand> tune_log;
    TuneCand tune_default {};
    static std::map<string, TuneCand>& tune_cache() {
        static std::map<string, TuneCand> c;
        return c;
    }

    vector<int> interleaved_order() const {
        std::map<int, vector<int>> by_sys;
        for (int r = 0; r < n_rep; ++r) by_sys[sys_of[r]].push_back(r);
        vector<int> order;
        for (size_t k = 0; order.size() < (size_t)n_rep; ++k)
            for (auto& kv : by_sys)
                if (k < kv.second.size()) order.push_back(kv.second[k]);
        return order;
    }

    double probe(int sweeps) {
        LdoLaunch L = launch_params(LDO_MODE_RUN, sweeps);
        L.sweep_units = 1;
        L.sample_interval = 0;
        L.n_trace = 0;
        CU(cudaEventRecord(ev0, stream));
        CU(launch_mc(L));
        CU(cudaEventRecord(ev1, stream));
        CU(cudaStreamSynchronize(stream));
        float f = 0;
        CU(cudaEventElapsedTime(&f, ev0, ev1));
        return f;
    }

    TuneCand autotune(int probe_sweeps, bool use_cache) {
        int wb = ldo_warp_smem_bytes(lay.cls);
        int ct = d_ct.p ? 1 : 0;
        std::ostringstream key;
        key << lay.cls << "/" << ct << "/" << systems_hash() << "/" << n_rep;
        tune_default = TuneCand {wpb, smem_pad, 0, use_rep_map ? 1 : 0, 0.0};
        if (use_cache) {
            auto it = tune_cache().find(key.str());
            if (it != tune_cache().end()) {
                apply_tune(it->second);
                return it->second;
            }
        }
        // candidates: (warps per block, resident blocks per SM) pairs that the
        // occupancy calculator confirms, each with the smallest padding
        vector<TuneCand> cands;
        const size_t kMaxSmem = 227 * 1024;
        for (int w : {1, 2, 4}) {
            size_t base = (size_t)w * wb;
            if (base > kMaxSmem) continue;
            int full = 0;
            CU(ldo_mc_occupancy(lay.cls, ct, w, base, &full));
            for (int want = full; want >= 1; --want) {
                if (w * want > 32 || (w * want) % 4 != 0) continue;
                size_t lo = 0, hi = kMaxSmem - base;
                int occ = 0;
                CU(ldo_mc_occupancy(lay.cls, ct, w, base + hi, &occ));
                if (occ > want) continue;
                while (lo < hi) {   // smallest padding with at most `want` blocks per SM
                    size_t mid = (lo + hi) / 2;
                    CU(ldo_mc_occupancy(lay.cls, ct, w, base + mid, &occ));
                    if (occ <= want) hi = mid;
                    else lo = mid + 1;
                }
                CU(ldo_mc_occupancy(lay.cls, ct, w, base + lo, &occ));
                if (occ == want) cands.push_back(TuneCand {w, (int)lo, want, 0, 0.0});
            }
        }
        bool multi = false;
        for (int r = 1; r < n_rep; ++r) multi = multi || sys_of[r] != sys_of[0];
        if (multi) {
            size_t n = cands.size();
            for (size_t i = 0; i < n; ++i) {
                TuneCand c = cands[i];
                c.order = 1;
                cands.push_back(c);
            }
        }
        vector<int> order = interleaved_order();
        d_rep_map.alloc(n_rep);
        CU(copy(d_rep_map.p, order.data(), n_rep * sizeof(int), cudaMemcpyHostToDevice));
        DevBuf<unsigned char> saved;
        saved.alloc(d_arena.n);
        CU(cudaMemcpyAsync(saved.p, d_arena.p, d_arena.n, cudaMemcpyDeviceToDevice, stream));
        auto restore = [&]() {
            CU(cudaMemcpyAsync(d_arena.p, saved.p, d_arena.n, cudaMemcpyDeviceToDevice, stream));
            CU(cudaStreamSynchronize(stream));
        };
        TuneCand keep = tune_default;
        // the default shape, timed the same way
        apply_tune(keep);
        probe(probe_sweeps);
        restore();
        tune_default.ms = probe(probe_sweeps);
        restore();
        tune_default.ms = std::min(tune_default.ms, probe(probe_sweeps));
        restore();
        tune_log.clear();
        TuneCand best = tune_default;
        for (auto& c : cands) {
            apply_tune(c);
            double t = probe(probe_sweeps);
            restore();
            t = std::min(t, probe(probe_sweeps));
            restore();
            c.ms = t;
            tune_log.push_back(c);
            if (c.ms < best.ms) best = c;
        }
        check_status();
        apply_tune(best);
        tune_cache()[key.str()] = best;
        return best;
    }

    void apply_tune(const TuneCand& c) {
        wpb = c.wpb;
        smem_pad = c.pad;
        use_rep_map = c.order == 1 && d_rep_map.p;
        if (c.order == 1 && !d_rep_map.p) {
            vector<int> order = interleaved_order();
            d_rep_map.alloc(n_rep);
            CU(copy(d_rep_map.p, order.data(), n_rep * sizeof(int), cudaMemcpyHostToDevice));
            use_rep_map = true;
        }
        // a captured PT cycle graph holds the launch shape: pt_run compares
        // the launch parameters and captures again
    }

    void check_status() {
        CU(cudaMemsetAsync(d_status.p, 0, sizeof(int), stream));
        count_launch();
        CU(ldo_launch_status(d_arena.p, lay.bytes, lay.o_hdr, n_rep, d_status.p, stream));
        int st = 0;
        count_copy(sizeof(int), cudaMemcpyDeviceToHost);
        CU(cudaMemcpyAsync(&st, d_status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CU(cudaStreamSynchronize(stream));
        if (st != 0) {
            const char* what = st == LDO_EINVARIANT  ? "a replica reached a state the reference rejects (invariant)"
                               : st == LDO_EITERCAP  ? "a replica hit an iteration cap"
                               : st == LDO_ECAPACITY ? "a replica ran out of staple or lattice slots"
                                                     : "replica error";
            throw LdoError((ldo_status)st, what);
        }
    }

    // Replica r's state bytes (b: lay.bytes zero bytes) for configuration
    // `chains`, as the OrigamiSystem constructor leaves them before
    // set_all_domains (src/origami_system.cpp:659-678); the kernel's init
    // mode then sets every domain.
    void fill_replica(int r, const vector<ldo_io::ChainConf>& chains, unsigned char* b) {
        {
            const HostSystem& hs = systems[sys_of[r]];
            const LdoSys& d = hs.desc;
            auto* h = reinterpret_cast<LdoHdr*>(b + lay.o_hdr);
            auto* pp = reinterpret_cast<long long*>(b + lay.o_pp);
            auto* nxt = reinterpret_cast<int16_t*>(b + lay.o_nxt);
            auto* prv = reinterpret_cast<int16_t*>(b + lay.o_prv);
            auto* bnd = reinterpret_cast<int16_t*>(b + lay.o_bound);
            auto* did = reinterpret_cast<int16_t*>(b + lay.o_dident);
            unsigned char* ore = b + lay.o_ore;
            unsigned char* st = b + lay.o_state;
            unsigned char* scs = b + lay.o_slot_cs;
            unsigned char* sd = b + lay.o_slot_d;
            auto* chain_c = reinterpret_cast<int32_t*>(b + lay.o_chain_c);
            unsigned char* chain_type = b + lay.o_chain_type;
            unsigned char* chain_order = b + lay.o_chain_order;
            unsigned char* clen = b + lay.o_clen;
            auto* type_count = reinterpret_cast<int16_t*>(b + lay.o_type_count);
            for (int s = 0; s < lay.dcap; ++s) {
                bnd[s] = -1;
                nxt[s] = -1;
                prv[s] = -1;
                if (s < d.ns) {
                    scs[s] = 0;
                    sd[s] = (unsigned char)s;
                }
                else if (s < d.dcap) {
                    scs[s] = (unsigned char)(1 + (s - d.ns) / d.lmax);
                    sd[s] = (unsigned char)((s - d.ns) % d.lmax);
                }
                else {
                    scs[s] = 0xff;
                    sd[s] = 0;
                }
            }
            for (int k = 0; k <= lay.kmax; ++k) chain_type[k] = 0xff;
            if (chains.empty() || (int)chains.size() - 1 > d.kmax)
                throw LdoError(LDO_ECAPACITY, "configuration has more staples than staple slots");
            int total = 0;
            int maxc = 0;
            for (size_t c = 0; c < chains.size(); ++c) {
                const auto& ch = chains[c];
                int cs = (int)c;
                int type = ch.identity;
                if (type < 0 || type >= d.n_types) throw LdoError(LDO_EINVAL, "chain identity out of range");
                if (c == 0 && type != 0) throw LdoError(LDO_EINVAL, "first chain must be the scaffold");
                if (c > 0 && type == 0) throw LdoError(LDO_EINVAL, "only the first chain may be the scaffold");
                int len = d.type_len[type];
                if ((int)ch.positions.size() != len) throw LdoError(LDO_EINVAL, "chain length does not match identity");
                chain_c[cs] = ch.index;
                // the reference's scaffold moves identify the scaffold by chain index 0
                if (c == 0 && d.has_ct && ch.index != 0)
                    throw LdoError(LDO_EINVAL, "scaffold regrowth movetypes need the scaffold's chain index to be 0");
                chain_type[cs] = (unsigned char)type;
                clen[cs] = (unsigned char)len;
                chain_order[c] = (unsigned char)cs;
                type_count[type]++;
                maxc = std::max(maxc, ch.index);
                for (int dd = 0; dd < len; ++dd) {
                    int s = cs == 0 ? dd : d.ns + (cs - 1) * d.lmax + dd;
                    for (int q = 0; q < 3; ++q)
                        if (ch.positions[dd][q] < -32000 || ch.positions[dd][q] > 32000)
                            throw LdoError(LDO_ECAPACITY, "position coordinate outside +-32000");
                    pp[s] = (long long)ch.positions[dd][0] + (long long)ch.positions[dd][1] * 65536ll +
                            (long long)ch.positions[dd][2] * 4294967296ll;
                    nxt[s] = (int16_t)(dd + 1 < len ? s + 1 : -1);
                    prv[s] = (int16_t)(dd > 0 ? s - 1 : -1);
                    if (cs == 0 && d.cyclic) {
                        if (dd + 1 == len) nxt[s] = 0;
                        if (dd == 0) prv[s] = (int16_t)(len - 1);
                    }
                    const auto& o = ch.orientations[dd];
                    int oi;
                    if (o[0] == 1 && o[1] == 0 && o[2] == 0) oi = 0;
                    else if (o[0] == -1 && o[1] == 0 && o[2] == 0) oi = 1;
                    else if (o[0] == 0 && o[1] == 1 && o[2] == 0) oi = 2;
                    else if (o[0] == 0 && o[1] == -1 && o[2] == 0) oi = 3;
                    else if (o[0] == 0 && o[1] == 0 && o[2] == 1) oi = 4;
                    else if (o[0] == 0 && o[1] == 0 && o[2] == -1) oi = 5;
                    else throw LdoError(LDO_EINVAL, "orientation is not a unit lattice vector");
                    ore[s] = (unsigned char)oi;
                    st[s] = 0;
                    did[s] = d.idents[d.type_off[type] + dd];
                }
                total += len;
            }
            // OrigamiSystem constructor bookkeeping before set_all_domains
            // (src/origami_system.cpp:659-678)
            h->n_chains = (int)chains.size();
            h->num_domains = total;
            h->num_unassigned = total;
            h->num_staples = (int)chains.size() - 1;
            h->current_c_i = maxc;
            h->energy = 0;
            unsigned long long nst = (unsigned long long)(chains.size() - 1);
            if (d.mean_field) h->energy += nst * std::log(6);
            h->energy += nst * h_tabs[h_ctl[r].tab].init_e;
            h->tab = h_ctl[r].tab;
        }
    }

    void init_arena() {
        vector<unsigned char> host((size_t)n_rep * lay.bytes, 0);
        for (int r = 0; r < n_rep; ++r)
            fill_replica(r, systems[sys_of[r]].sf.chains, host.data() + (size_t)r * lay.bytes);
        d_arena.alloc(host.size());
        CU(copy(d_arena.p, host.data(), host.size(), cudaMemcpyHostToDevice));
    }

    // Philox stream key of each replica (ldo_batch: its index in the whole
    // batch); empty: the replica's own index.
    vector<uint32_t> rep_ids;

    void create(const vector<string>& inps, const string& overrides, const vector<int>& sys_of_replica,
                uint32_t seed_) {
        seed = seed_;
        for (auto& f : inps) systems.push_back(load_system(f, overrides));
        sys_of = sys_of_replica;
        n_rep = (int)sys_of.size();
        if (n_rep <= 0) throw LdoError(LDO_EINVAL, "need at least one replica");
        int dcap = 0, kmax = 0, ntypes = 0, nb = 0, nop = 0, nmv = 0;
        for (auto& hs : systems) {
            dcap = std::max(dcap, hs.desc.dcap);
            kmax = std::max(kmax, hs.desc.kmax);
            ntypes = std::max(ntypes, hs.desc.n_types);
            nb = std::max(nb, hs.desc.n_biases);
            nop = std::max(nop, hs.desc.n_ops);
            nmv = std::max(nmv, hs.desc.n_moves);
        }
        lay = make_layout(dcap, kmax, ntypes, nb, nop, nmv);
        CU(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CU(cudaEventCreate(&ev0));
        CU(cudaEventCreate(&ev1));
        // Four replicas (warps) per block by default; the kernel's launch
        // bounds allow seven such blocks per SM.  Tuning keys (engine-only,
        // not reference options): gpu_warps_per_block (1..4) and
        // gpu_smem_pad_bytes (extra shared memory per block, to lower the
        // number of resident blocks).
        wpb = 4;
        smem_pad = 0;
        for (auto& hs : systems) {
            auto it = hs.p.extra.find("gpu_warps_per_block");
            if (it != hs.p.extra.end()) wpb = std::max(1, std::min(4, std::atoi(it->second.c_str())));
            it = hs.p.extra.find("gpu_smem_pad_bytes");
            if (it != hs.p.extra.end()) smem_pad = std::max(0, std::atoi(it->second.c_str()));
        }
        for (auto& hs : systems) h_sys.push_back(hs.desc);
        d_sys.alloc(h_sys.size());
        CU(copy(d_sys.p, h_sys.data(), h_sys.size() * sizeof(LdoSys), cudaMemcpyHostToDevice));
        h_ctl.resize(n_rep);
        temps.resize(n_rep);
        stack_mults.assign(n_rep, 1.0);
        u_mults.resize(n_rep);
        size_t grid_total = 0;
        for (int r = 0; r < n_rep; ++r) {
            int s = sys_of[r];
            if (s < 0 || s >= (int)systems.size()) throw LdoError(LDO_EINVAL, "sys_of_replica out of range");
            const HostSystem& hs = systems[s];
            LdoRepCtl& c = h_ctl[r];
            std::memset(&c, 0, sizeof c);
            c.sys = s;
            temps[r] = hs.p.temp;
            u_mults[r] = hs.p.staple_u_mult;
            c.tab = table_for(s, hs.p.temp, 1.0);
            c.staple_M = hs.p.staple_M;
            c.staple_u_mult = hs.p.staple_u_mult;
            c.bias_mult = hs.p.bias_functions_mult;
            for (int b = 0; b < LDO_MAX_BIASES; ++b) {
                c.win_min[b] = hs.desc.bias_min[b];
                c.win_max[b] = hs.desc.bias_max[b];
                c.centre[b] = hs.desc.bias_centre[b];
                c.grid_off[b] = -1;
                if (b < hs.desc.n_biases && hs.desc.bias_kind[b] == LDO_B_GRID) {
                    c.grid_off[b] = (int)grid_total;
                    grid_total += hs.desc.bias_grid_len[b];
                }
            }
            c.seed = seed;
            c.rep = rep_ids.empty() ? (uint32_t)r : rep_ids[r];
        }
        h_grid.assign(std::max<size_t>(grid_total, 1), 0.0);
        d_grid.alloc(h_grid.size());
        upload_grid();
        d_ctl.alloc(n_rep);
        upload_ctl();
        upload_tables();
        d_status.alloc(1);
        init_arena();
        d_snap.alloc((size_t)n_rep * LDO_N_SNAPSHOTS * ldo_snapshot_stride(lay.bytes));
        bool any_ct = false;
        for (auto& d : h_sys) any_ct = any_ct || d.has_ct;
        if (any_ct) {
            ct_stride = ldo_ct_work_bytes(lay.cls);
            d_ct.alloc((size_t)n_rep * ct_stride);
        }
        // untrained proposal: every unbound domain weighs 1
        {
            vector<double> ones(LDO_LEARN_TABLE, 1.0);
            d_learn_w.alloc(LDO_LEARN_TABLE);
            CU(copy(d_learn_w.p, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice));
            d_cnt_b.alloc(LDO_LEARN_TABLE);
            d_cnt_t.alloc(LDO_LEARN_TABLE);
            CU(cudaMemsetAsync(d_cnt_b.p, 0, LDO_LEARN_TABLE * sizeof(double), stream));
            CU(cudaMemsetAsync(d_cnt_t.p, 0, LDO_LEARN_TABLE * sizeof(double), stream));
        }
        LdoLaunch L = launch_params(LDO_MODE_INIT, 0);
        CU(launch_mc(L));
        CU(cudaStreamSynchronize(stream));
        check_status();
    }

    void run(long long steps, double* ms, int sweeps = 0) {
        LdoLaunch L = launch_params(LDO_MODE_RUN, steps);
        L.sweep_units = sweeps;
        CU(cudaEventRecord(ev0, stream));
        CU(launch_mc(L));
        CU(cudaEventRecord(ev1, stream));
        CU(cudaStreamSynchronize(stream));
        if (ms) {
            float f = 0;
            CU(cudaEventElapsedTime(&f, ev0, ev1));
            *ms = f;
        }
        check_status();
    }

    // ---------------------------------------- configuration import ---
    // Chains of a configuration buffer in ldo_get_config's format (n_chains,
    // then per chain index, identity, length, length x (x, y, z, ox, oy, oz,
    // state)); the states are ignored.
    static vector<ldo_io::ChainConf> parse_config(const int32_t* buf, int n) {
        int p = 0;
        auto next = [&]() {
            if (p >= n) throw LdoError(LDO_EINVAL, "configuration buffer ends early");
            return buf[p++];
        };
        int nc = next();
        if (nc < 1 || nc > 100000) throw LdoError(LDO_EINVAL, "configuration: bad number of chains");
        vector<ldo_io::ChainConf> chains(nc);
        for (auto& c : chains) {
            c.index = next();
            c.identity = next();
            int len = next();
            if (len < 1 || len > 100000) throw LdoError(LDO_EINVAL, "configuration: bad chain length");
            for (int d = 0; d < len; ++d) {
                std::array<int, 3> pos, ore;
                for (int q = 0; q < 3; ++q) pos[q] = next();
                for (int q = 0; q < 3; ++q) ore[q] = next();
                next();
                c.positions.push_back(pos);
                c.orientations.push_back(ore);
            }
        }
        if (p != n) throw LdoError(LDO_EINVAL, "configuration buffer has trailing values");
        return chains;
    }

    // Replaces replica r's configuration, as the OrigamiSystem constructor
    // builds a system from given chains (src/origami_system.cpp:991-1003):
    // energy, counters, order parameters and biases become those of the new
    // configuration; the replica keeps its random-number position, step
    // counter, sample count and move statistics.  A configuration that
    // violates a constraint leaves the replica as it was
    // (set_all_domains: "Constaints in violation after move complete").
    void set_config(int r, const int32_t* buf, int n) {
        if (r < 0 || r >= n_rep) throw LdoError(LDO_EINVAL, "replica out of range");
        vector<ldo_io::ChainConf> chains = parse_config(buf, n);
        size_t off = (size_t)r * lay.bytes;
        vector<unsigned char> old(lay.bytes), fresh(lay.bytes, 0);
        CU(copy(old.data(), d_arena.p + off, lay.bytes, cudaMemcpyDeviceToHost));
        fill_replica(r, chains, fresh.data());
        const auto* ho = reinterpret_cast<const LdoHdr*>(old.data() + lay.o_hdr);
        auto* hn = reinterpret_cast<LdoHdr*>(fresh.data() + lay.o_hdr);
        hn->draws = ho->draws;
        hn->steps_done = ho->steps_done;
        hn->sample_count = ho->sample_count;
        std::memcpy(fresh.data() + lay.o_mstat, old.data() + lay.o_mstat, 2 * lay.nmv * sizeof(long long));
        CU(copy(d_arena.p + off, fresh.data(), lay.bytes, cudaMemcpyHostToDevice));
        LdoLaunch L = launch_params(LDO_MODE_INIT, 0);
        L.only_rep = r;
        CU(launch_mc(L));
        CU(cudaStreamSynchronize(stream));
        LdoHdr h;
        CU(copy(&h, d_arena.p + off + lay.o_hdr, sizeof h, cudaMemcpyDeviceToHost));
        if (h.status != 0) {
            CU(copy(d_arena.p + off, old.data(), lay.bytes, cudaMemcpyHostToDevice));
            throw LdoError(LDO_EINVAL, h.status == LDO_RS_INVARIANT
                                           ? "Constaints in violation after move complete"
                                           : "configuration does not fit the replica's capacity");
        }
    }

    // Every replica's configuration at once (ldo_set_configs): bufs holds
    // n_rep configurations, replica r's at [off[r], off[r+1]).  One init
    // launch for the batch; all or nothing.
    void set_configs(const int32_t* bufs, const int32_t* off) {
        vector<unsigned char> old((size_t)n_rep * lay.bytes), fresh((size_t)n_rep * lay.bytes, 0);
        CU(copy(old.data(), d_arena.p, old.size(), cudaMemcpyDeviceToHost));
        for (int r = 0; r < n_rep; ++r) {
            if (off[r] < 0 || off[r + 1] < off[r]) throw LdoError(LDO_EINVAL, "configuration offsets not increasing");
            vector<ldo_io::ChainConf> chains = parse_config(bufs + off[r], off[r + 1] - off[r]);
            unsigned char* b = fresh.data() + (size_t)r * lay.bytes;
            fill_replica(r, chains, b);
            const unsigned char* o = old.data() + (size_t)r * lay.bytes;
            const auto* ho = reinterpret_cast<const LdoHdr*>(o + lay.o_hdr);
            auto* hn = reinterpret_cast<LdoHdr*>(b + lay.o_hdr);
            hn->draws = ho->draws;
            hn->steps_done = ho->steps_done;
            hn->sample_count = ho->sample_count;
            std::memcpy(b + lay.o_mstat, o + lay.o_mstat, 2 * lay.nmv * sizeof(long long));
        }
        CU(copy(d_arena.p, fresh.data(), fresh.size(), cudaMemcpyHostToDevice));
        LdoLaunch L = launch_params(LDO_MODE_INIT, 0);
        CU(launch_mc(L));
        CU(cudaStreamSynchronize(stream));
        CU(copy(fresh.data(), d_arena.p, fresh.size(), cudaMemcpyDeviceToHost));
        for (int r = 0; r < n_rep; ++r) {
            const auto* h = reinterpret_cast<const LdoHdr*>(fresh.data() + (size_t)r * lay.bytes + lay.o_hdr);
            if (h->status != 0) {
                CU(copy(d_arena.p, old.data(), old.size(), cudaMemcpyHostToDevice));
                throw LdoError(LDO_EINVAL, "replica " + std::to_string(r) + ": " +
                                               (h->status == LDO_RS_INVARIANT
                                                    ? "Constaints in violation after move complete"
                                                    : "configuration does not fit the replica's capacity"));
            }
        }
    }

    // ---------------------------------------- checkpoint / resume ---
    // One binary file from which a run continues bit for bit: every
    // replica's state (configuration, counters, random-number position,
    // move statistics), its controls (temperature, chemical-potential and
    // stacking multipliers, windows, centres, grid biases, seed), the
    // learned proposal's weight table and network, and a parallel-tempering
    // ladder's permutation, swap counter, swap random-number positions and
    // statistics.  It stands for the reference's restart pieces: the .trj
    // configuration (src/origami_system.cpp:1000), the .randstate file
    // (src/simulation.cpp:204-212) and the permutation of the last .swp line
    // (src/ptmc_simulation.cpp:62-83).  Energy-table indices are stored as
    // (system, temperature, stacking multiplier) keys and rebuilt, so any
    // engine created from the same input files and replica count can load
    // it.  Not stored: sample and trace buffers, the .swp history, the
    // network optimiser's moments, umbrella-sampling iterations.
    struct CkptHead {
        char magic[8];
        uint32_t version, n_rep, n_sys, seed;
        uint64_t sys_hash;
        uint32_t n_tabs, has_mlp;
        uint64_t n_grid;
        int32_t pt_rungs, pt_q, pt_dim2, pt_nctr;
        int64_t pt_swap_i;
        LdoLayout lay;
        uint64_t payload_bytes, payload_hash;   // everything after the header (FNV-1a)
    };
    struct CkptTab {
        int32_t sys, pad;
        double temp, mult;
    };

    static uint64_t fnv1a(const unsigned char* b, size_t n) {
        uint64_t h = 1469598103934665603ull;
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
        return h;
    }
    uint64_t systems_hash() const {
        uint64_t h = 1469598103934665603ull;   // FNV-1a
        const unsigned char* b = reinterpret_cast<const unsigned char*>(h_sys.data());
        for (size_t i = 0; i < h_sys.size() * sizeof(LdoSys); ++i) h = (h ^ b[i]) * 1099511628211ull;
        for (int s : sys_of) h = (h ^ (uint64_t)(uint32_t)s) * 1099511628211ull;
        return h;
    }

    void checkpoint_save(const string& path) {
        CkptHead H;
        std::memset(&H, 0, sizeof H);
        std::memcpy(H.magic, "LDOCKPT", 8);
        H.version = 3;
        H.n_rep = (uint32_t)n_rep;
        H.n_sys = (uint32_t)systems.size();
        H.seed = seed;
        H.sys_hash = systems_hash();
        H.n_tabs = (uint32_t)h_tabs.size();
        H.has_mlp = mlp_init ? 1 : 0;
        H.n_grid = h_grid.size();
        H.pt_rungs = pt_rungs;
        H.pt_q = pt_q;
        H.pt_dim2 = pt_dim2;
        H.pt_nctr = pt_nctr;
        H.pt_swap_i = pt_swap_i;
        H.lay = lay;
        vector<CkptTab> keys(h_tabs.size());
        for (auto& kv : tab_index) {
            CkptTab& k = keys[kv.second];
            std::memset(&k, 0, sizeof k);
            k.sys = std::get<0>(kv.first);
            k.temp = std::get<1>(kv.first);
            k.mult = std::get<2>(kv.first);
        }
        vector<unsigned char> arena((size_t)n_rep * lay.bytes);
        CU(copy(arena.data(), d_arena.p, arena.size(), cudaMemcpyDeviceToHost));
        vector<double> table(LDO_LEARN_TABLE);
        CU(copy(table.data(), d_learn_w.p, table.size() * sizeof(double), cudaMemcpyDeviceToHost));
        std::string out(sizeof H, '\0');
        auto put = [&](const void* p, size_t bytes) { out.append(reinterpret_cast<const char*>(p), bytes); };
        put(keys.data(), keys.size() * sizeof(CkptTab));
        put(h_ctl.data(), h_ctl.size() * sizeof(LdoRepCtl));
        put(temps.data(), n_rep * sizeof(double));
        put(stack_mults.data(), n_rep * sizeof(double));
        put(u_mults.data(), n_rep * sizeof(double));
        put(h_grid.data(), h_grid.size() * sizeof(double));
        put(arena.data(), arena.size());
        put(table.data(), table.size() * sizeof(double));
        if (mlp_init) {
            vector<float> params(LDO_LEARN_NPARAM);
            CU(copy(params.data(), mlp.params, params.size() * sizeof(float), cudaMemcpyDeviceToHost));
            put(params.data(), params.size() * sizeof(float));
        }
        if (pt_rungs) {
            int nl = n_rep / pt_rungs;
            vector<int> perm(n_rep);
            vector<double> rep_q(4 * (size_t)n_rep);
            vector<unsigned long long> draws(nl);
            vector<long long> att(std::max(pt_nctr, 1)), acc(std::max(pt_nctr, 1));
            CU(copy(perm.data(), d_perm.p, perm.size() * sizeof(int), cudaMemcpyDeviceToHost));
            CU(copy(rep_q.data(), d_rep_q.p, rep_q.size() * sizeof(double), cudaMemcpyDeviceToHost));
            CU(copy(draws.data(), d_pt_draws.p, draws.size() * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost));
            CU(copy(att.data(), d_pt_att.p, att.size() * sizeof(long long), cudaMemcpyDeviceToHost));
            CU(copy(acc.data(), d_pt_acc.p, acc.size() * sizeof(long long), cudaMemcpyDeviceToHost));
            put(perm.data(), perm.size() * sizeof(int));
            put(rep_q.data(), rep_q.size() * sizeof(double));
            put(draws.data(), draws.size() * sizeof(unsigned long long));
            put(att.data(), att.size() * sizeof(long long));
            put(acc.data(), acc.size() * sizeof(long long));
        }
        // umbrella sampling between iterations (what the reference restarts
        // from its .S_n/.s_i/.f_i archives and .biases files,
        // src/us_simulation.cpp:192-344): windows, biases, visited points
        int32_t us_on = us_win.empty() ? 0 : 1;
        put(&us_on, sizeof us_on);
        if (us_on) {
            int32_t nw = (int32_t)us_win.size(), tl = (int32_t)us_tag.size();
            int32_t ints[5] = {tl, us_bias, us_len, us_sq_bias, nw};
            put(ints, sizeof ints);
            put(us_tag.data(), us_tag.size());
            for (auto& w : us_win) {
                int32_t mm[2] = {w.min_op, w.max_op};
                put(mm, sizeof mm);
                put(w.E_w.data(), us_len * sizeof(double));
                put(w.in_S.data(), us_len);
                put(w.in_file.data(), us_len);
            }
            put(us_window_of.data(), n_rep * sizeof(int));
            put(us_replica_of.data(), nw * sizeof(int));
            put(us_att.data(), us_att.size() * sizeof(long long));
            put(us_acc.data(), us_acc.size() * sizeof(long long));
            put(&us_swap_draws, sizeof us_swap_draws);
            put(&us_iters_done, sizeof us_iters_done);
        }
        H.payload_bytes = out.size() - sizeof H;
        H.payload_hash = fnv1a(reinterpret_cast<const unsigned char*>(out.data()) + sizeof H, H.payload_bytes);
        std::memcpy(&out[0], &H, sizeof H);
        std::ofstream f(path, std::ios::binary);
        if (!f) throw LdoError(LDO_EINVAL, path + ": cannot open checkpoint file for writing");
        f.write(out.data(), (std::streamsize)out.size());
        f.flush();
        if (!f) throw LdoError(LDO_EINVAL, path + ": writing the checkpoint failed");
    }

    void checkpoint_load(const string& path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw LdoError(LDO_EINVAL, path + ": checkpoint file does not exist");
        std::string in((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        size_t cur = 0;
        auto get = [&](void* p, size_t bytes) {
            if (in.size() - cur < bytes) throw LdoError(LDO_EINVAL, path + ": checkpoint file is truncated");
            std::memcpy(p, in.data() + cur, bytes);
            cur += bytes;
        };
        CkptHead H;
        get(&H, sizeof H);
        if (std::memcmp(H.magic, "LDOCKPT", 8) != 0 || H.version != 3)
            throw LdoError(LDO_EINVAL, path + ": not a checkpoint of this engine");
        if (H.payload_bytes != in.size() - sizeof H ||
            H.payload_hash != fnv1a(reinterpret_cast<const unsigned char*>(in.data()) + sizeof H, H.payload_bytes))
            throw LdoError(LDO_EINVAL, path + ": checkpoint file is truncated or corrupt");
        if (H.n_rep != (uint32_t)n_rep || H.n_sys != systems.size() || H.sys_hash != systems_hash() ||
            std::memcmp(&H.lay, &lay, sizeof lay) != 0 || H.n_grid != h_grid.size())
            throw LdoError(LDO_EINVAL, path + ": checkpoint of other systems or another replica count");
        if (H.n_tabs == 0 || H.n_tabs > 1000000) throw LdoError(LDO_EINVAL, path + ": bad table count");
        if (H.pt_rungs < 0 || (H.pt_rungs && (H.pt_rungs < 2 || n_rep % H.pt_rungs != 0)))
            throw LdoError(LDO_EINVAL, path + ": bad ladder shape");
        vector<CkptTab> keys(H.n_tabs);
        get(keys.data(), keys.size() * sizeof(CkptTab));
        vector<LdoRepCtl> ctl(n_rep);
        get(ctl.data(), ctl.size() * sizeof(LdoRepCtl));
        vector<double> t(n_rep), sm(n_rep), um(n_rep), grid(h_grid.size());
        get(t.data(), n_rep * sizeof(double));
        get(sm.data(), n_rep * sizeof(double));
        get(um.data(), n_rep * sizeof(double));
        get(grid.data(), grid.size() * sizeof(double));
        vector<unsigned char> arena((size_t)n_rep * lay.bytes);
        get(arena.data(), arena.size());
        vector<double> table(LDO_LEARN_TABLE);
        get(table.data(), table.size() * sizeof(double));
        vector<float> params;
        if (H.has_mlp) {
            params.resize(LDO_LEARN_NPARAM);
            get(params.data(), params.size() * sizeof(float));
        }
        // ladder payload, read and checked before anything of the engine changes
        vector<int> perm;
        vector<double> rep_q;
        vector<unsigned long long> draws;
        vector<long long> att, acc;
        if (H.pt_rungs) {
            if (pt_check(H.pt_rungs, H.pt_q, H.pt_dim2) != H.pt_nctr)
                throw LdoError(LDO_EINVAL, path + ": ladder does not match the input files");
            int nl = n_rep / H.pt_rungs;
            perm.resize(n_rep);
            rep_q.resize(4 * (size_t)n_rep);
            draws.resize(nl);
            att.resize(std::max(H.pt_nctr, 1));
            acc.resize(std::max(H.pt_nctr, 1));
            get(perm.data(), perm.size() * sizeof(int));
            get(rep_q.data(), rep_q.size() * sizeof(double));
            get(draws.data(), draws.size() * sizeof(unsigned long long));
            get(att.data(), att.size() * sizeof(long long));
            get(acc.data(), acc.size() * sizeof(long long));
            vector<char> seen(n_rep, 0);
            for (int r : perm) {
                if (r < 0 || r >= n_rep || seen[r]) throw LdoError(LDO_EINVAL, path + ": bad ladder permutation");
                seen[r] = 1;
            }
        }
        // umbrella-sampling section
        int32_t us_on = 0;
        get(&us_on, sizeof us_on);
        vector<USWindow> uw;
        string utag;
        int32_t uints[5] = {0, -1, 0, -1, 0};
        vector<int> u_wof, u_rof;
        vector<long long> u_att, u_acc;
        unsigned long long u_draws = 0;
        long long u_iters = 0;
        if (us_on) {
            get(uints, sizeof uints);
            int32_t tl = uints[0], ub = uints[1], ul = uints[2], nw = uints[4];
            if (tl < 1 || tl > 4096 || nw != n_rep || ul < 1 || ul > 1 << 20)
                throw LdoError(LDO_EINVAL, path + ": bad umbrella-sampling section");
            utag.resize(tl);
            get(&utag[0], tl);
            const HostSystem& hs = systems[sys_of[0]];
            if (ub < 0 || ub >= hs.desc.n_biases || hs.biases[ub].tag != utag || hs.desc.bias_kind[ub] != LDO_B_GRID ||
                hs.desc.bias_grid_len[ub] != ul || uints[3] >= hs.desc.n_biases)
                throw LdoError(LDO_EINVAL, path + ": umbrella-sampling grid does not match the input files");
            uw.resize(nw);
            for (auto& w : uw) {
                int32_t mm[2];
                get(mm, sizeof mm);
                w.min_op = mm[0];
                w.max_op = mm[1];
                w.E_w.resize(ul);
                w.in_S.resize(ul);
                w.in_file.resize(ul);
                get(w.E_w.data(), ul * sizeof(double));
                get(w.in_S.data(), ul);
                get(w.in_file.data(), ul);
            }
            u_wof.resize(n_rep);
            u_rof.resize(nw);
            u_att.resize(std::max(nw - 1, 1));
            u_acc.resize(std::max(nw - 1, 1));
            get(u_wof.data(), n_rep * sizeof(int));
            get(u_rof.data(), nw * sizeof(int));
            get(u_att.data(), u_att.size() * sizeof(long long));
            get(u_acc.data(), u_acc.size() * sizeof(long long));
            get(&u_draws, sizeof u_draws);
            get(&u_iters, sizeof u_iters);
            for (int r = 0; r < n_rep; ++r)
                if (u_wof[r] < 0 || u_wof[r] >= nw || u_rof[u_wof[r]] != r)
                    throw LdoError(LDO_EINVAL, path + ": bad umbrella window assignment");
        }
        if (cur != in.size()) throw LdoError(LDO_EINVAL, path + ": checkpoint file has trailing bytes");
        for (size_t i = 0; i < keys.size(); ++i)
            if (keys[i].sys < 0 || keys[i].sys >= (int)systems.size())
                throw LdoError(LDO_EINVAL, path + ": bad table key");
        auto check_tab = [&](int k) {
            if (k < 0 || k >= (int)keys.size()) throw LdoError(LDO_EINVAL, path + ": bad table index");
        };
        for (int r = 0; r < n_rep; ++r) {
            if (ctl[r].sys != sys_of[r] || ctl[r].rep != h_ctl[r].rep)
                throw LdoError(LDO_EINVAL, path + ": replica controls do not match this engine");
            for (int b = 0; b < LDO_MAX_BIASES; ++b)
                if (ctl[r].grid_off[b] != h_ctl[r].grid_off[b])
                    throw LdoError(LDO_EINVAL, path + ": grid layout does not match this engine");
            check_tab(ctl[r].tab);
            check_tab(reinterpret_cast<const LdoHdr*>(arena.data() + (size_t)r * lay.bytes + lay.o_hdr)->tab);
        }
        // Every check has passed: from here on the engine takes the file's
        // state.  Energy tables of the saved keys, in this engine's numbering.
        vector<int> remap(H.n_tabs);
        for (size_t i = 0; i < keys.size(); ++i) remap[i] = table_for(keys[i].sys, keys[i].temp, keys[i].mult);
        for (int r = 0; r < n_rep; ++r) {
            ctl[r].tab = remap[ctl[r].tab];
            auto* h = reinterpret_cast<LdoHdr*>(arena.data() + (size_t)r * lay.bytes + lay.o_hdr);
            h->tab = remap[h->tab];
        }
        // ladder: set up its shape, then the saved permutation and counters
        if (pt_graph) {
            cudaGraphExecDestroy(pt_graph);
            pt_graph = nullptr;
        }
        seed = H.seed;
        pt_rungs = 0;
        if (H.pt_rungs) {
            pt_setup(H.pt_rungs, H.pt_q, H.pt_dim2);
            CU(copy(d_perm.p, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice));
            CU(copy(d_rep_q.p, rep_q.data(), rep_q.size() * sizeof(double), cudaMemcpyHostToDevice));
            CU(copy(d_pt_draws.p, draws.data(), draws.size() * sizeof(unsigned long long),
                          cudaMemcpyHostToDevice));
            CU(copy(d_pt_att.p, att.data(), att.size() * sizeof(long long), cudaMemcpyHostToDevice));
            CU(copy(d_pt_acc.p, acc.data(), acc.size() * sizeof(long long), cudaMemcpyHostToDevice));
            pt_swap_i = H.pt_swap_i;
        }
        h_ctl = ctl;
        temps = t;
        stack_mults = sm;
        u_mults = um;
        h_grid = grid;
        us_win.clear();
        us_tag.clear();
        if (us_on) {
            us_win = std::move(uw);
            us_tag = utag;
            us_bias = uints[1];
            us_len = uints[2];
            us_sq_bias = uints[3];
            us_window_of = u_wof;
            us_replica_of = u_rof;
            us_att = u_att;
            us_acc = u_acc;
            us_swap_draws = u_draws;
            us_iters_done = u_iters;
            d_us_hist.alloc(us_win.size() * (size_t)us_len);
            d_us_window.alloc(n_rep);
            CU(copy(d_us_window.p, us_window_of.data(), n_rep * sizeof(int), cudaMemcpyHostToDevice));
        }
        upload_tables();
        upload_ctl();
        upload_grid();
        CU(copy(d_arena.p, arena.data(), arena.size(), cudaMemcpyHostToDevice));
        CU(copy(d_learn_w.p, table.data(), table.size() * sizeof(double), cudaMemcpyHostToDevice));
        if (H.has_mlp) {
            mlp_ensure(0);
            CU(copy(mlp.params, params.data(), params.size() * sizeof(float), cudaMemcpyHostToDevice));
            CU(ldo_mlp_sync_weights(mlp, stream));
        }
        CU(cudaStreamSynchronize(stream));
    }

    // ---------------------------------------- learned insertion proposal ---
    static constexpr int kMlpCap = 1 << 17;

    void mlp_ensure(uint32_t seed) {
        if (!mlp.params) CU(ldo_mlp_alloc(mlp, kMlpCap));
        if (!mlp_init) {
            vector<float> p = ldo_learn_init_params(seed);
            CU(copy(mlp.params, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice));
            CU(ldo_mlp_sync_weights(mlp, stream));
            mlp_init = true;
        }
    }

    void learn_collect() {
        LdoLaunch L = launch_params(LDO_MODE_COLLECT, 0);
        CU(launch_mc(L));
        CU(cudaStreamSynchronize(stream));
        check_status();
    }

    // Adam on the weighted logistic loss over the collected counts (full
    // batch), then the weight table.
    void learn_train(int iters, double lr, uint32_t seed, double* loss0, double* loss1) {
        vector<double> cb(LDO_LEARN_TABLE), ct(LDO_LEARN_TABLE);
        CU(copy(cb.data(), d_cnt_b.p, cb.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CU(copy(ct.data(), d_cnt_t.p, ct.size() * sizeof(double), cudaMemcpyDeviceToHost));
        vector<int32_t> idx;
        vector<float> bb, tt;
        double norm = 0;
        for (int k = 0; k < LDO_LEARN_TABLE; ++k)
            if (ct[k] > 0) {
                idx.push_back(k);
                bb.push_back((float)cb[k]);
                tt.push_back((float)ct[k]);
                norm += (float)ct[k];
            }
        if (idx.empty()) throw LdoError(LDO_EINVAL, "no training data collected");
        if ((int)idx.size() > kMlpCap) throw LdoError(LDO_EINVAL, "too many distinct network inputs");
        mlp_ensure(seed);
        int n = (int)idx.size();
        CU(copy(mlp.idx, idx.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice));
        CU(copy(mlp.cnt_b, bb.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        CU(copy(mlp.cnt_t, tt.data(), n * sizeof(float), cudaMemcpyHostToDevice));
        for (int it = 0; it < iters; ++it) {
            CU(ldo_mlp_loss_grad(mlp, n, norm, stream));
            if (it == 0 && loss0) CU(cudaMemcpyAsync(loss0, mlp.loss, sizeof(double), cudaMemcpyDeviceToHost, stream));
            CU(ldo_mlp_adam(mlp, (float)lr, stream));
        }
        CU(ldo_mlp_loss_grad(mlp, n, norm, stream));
        if (loss1) CU(cudaMemcpyAsync(loss1, mlp.loss, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CU(ldo_mlp_table(mlp, d_learn_w.p, stream));
        mlp_check();
    }

    void mlp_check() {
        bool timed_out = false;
        CU(ldo_mlp_check(mlp, stream, &timed_out));
        if (timed_out) throw LdoError(LDO_ECUDA, "network product: a tensor-core completion wait ran out");
    }

    // PTGCMCSimulation constructor + OneDPTGCMCSimulation::initialize_control_qs
    // (src/ptmc_simulation.cpp:24-90, 337-358) for n_rep / n_rungs ladders.
    // dim2 = 0: one-dimensional ladder over the .inp's temps (and the other
    // per-rung lists).  dim2 > 0: TwoDPTGCMCSimulation's grid of temps x
    // stacking_mults (dim2 = number of stacking multipliers), slot
    // k = i * dim2 + j, exchanging temperature, staple chemical potential and
    // stacking multiplier (src/ptmc_simulation.cpp:428-481).
    // The checks of pt_setup, without changing the engine: throws for a
    // ladder these input files cannot form, else returns its number of
    // attempt/accept counters.
    int pt_check(int n_rungs, int exchange_q, int dim2) const {
        if (n_rungs < 2 || n_rep % n_rungs != 0) throw LdoError(LDO_EINVAL, "replicas must form whole ladders of n_rungs");
        if (!(exchange_q & 1)) throw LdoError(LDO_EINVAL, "every exchange variant exchanges the temperature");
        for (int r = 0; r < n_rep; ++r)
            if (sys_of[r] != sys_of[(r / n_rungs) * n_rungs])
                throw LdoError(LDO_EINVAL, "replicas of one ladder must share a system");
        const HostSystem& hs = systems[sys_of[0]];
        for (auto& s : systems)
            if (&s != &hs && s.desc.n_types != hs.desc.n_types)
                throw LdoError(LDO_EINVAL, "ladders must have the same staple types");
        const ldo_io::Params& p = hs.p;
        if (dim2 == 0) {
            if ((int)p.temps.size() != n_rungs) throw LdoError(LDO_EINVAL, "temps must list one temperature per rung");
            for (auto* v : {&p.chem_pot_mults, &p.bias_mults, &p.stacking_mults})
                if (!v->empty() && (int)v->size() != n_rungs)
                    throw LdoError(LDO_EINVAL, "chem_pot_mults, bias_mults and stacking_mults must list one value per rung");
            return n_rungs - 1;
        }
        int d1 = (int)p.temps.size(), d2 = (int)p.stacking_mults.size();
        if (d2 != dim2 || d1 * d2 != n_rungs || d1 < 1 || d2 < 1)
            throw LdoError(LDO_EINVAL, "a 2-D ladder needs temps x stacking_mults slots");
        return 2 * d1 * d2;
    }

    void pt_setup(int n_rungs, int exchange_q, int dim2 = 0) {
        pt_check(n_rungs, exchange_q, dim2);
        int nl = n_rep / n_rungs;
        const HostSystem& hs = systems[sys_of[0]];
        const ldo_io::Params& p = hs.p;
        vector<double> tq, uq, bq, sq;
        // pair schedule: sets of (slot a, slot b, counter) in the reference's loop order
        vector<vector<std::tuple<int, int, int>>> sets;
        int n_ctr = 0;
        if (dim2 == 0) {
            if ((int)p.temps.size() != n_rungs) throw LdoError(LDO_EINVAL, "temps must list one temperature per rung");
            auto fill = [&](const vector<double>& v, const char* what) {
                if (v.empty()) return vector<double>(n_rungs, 1.0);
                if ((int)v.size() != n_rungs)
                    throw LdoError(LDO_EINVAL, string(what) + " must list one value per rung");
                return v;
            };
            tq = p.temps;
            uq = fill(p.chem_pot_mults, "chem_pot_mults");
            bq = fill(p.bias_mults, "bias_mults");
            sq = fill(p.stacking_mults, "stacking_mults");
            // OneDPTGCMCSimulation::attempt_exchange (:360): i = swap_i % 2, i + 2, ...
            sets.resize(2);
            for (int set = 0; set < 2; ++set)
                for (int i = set; i < n_rungs - 1; i += 2) sets[set].push_back(std::make_tuple(i, i + 1, i));
            n_ctr = n_rungs - 1;
        }
        else {
            int d1 = (int)p.temps.size(), d2 = (int)p.stacking_mults.size();
            if (d2 != dim2 || d1 * d2 != n_rungs || d1 < 1 || d2 < 1)
                throw LdoError(LDO_EINVAL, "a 2-D ladder needs temps x stacking_mults slots");
            for (int i = 0; i < d1; ++i)
                for (int j = 0; j < d2; ++j) {
                    tq.push_back(p.temps[i]);
                    uq.push_back(p.staple_u_mult);
                    bq.push_back(1.0);
                    sq.push_back(p.stacking_mults[j]);
                }
            // TwoDPTGCMCSimulation::attempt_exchange (:495) with the set tables
            // of include/.../ptmc_simulation.hpp:158-164
            const int i_start[4] = {0, 0, 1, 0}, j_start[4] = {0, 0, 0, 1};
            const int i_incr[4] = {2, 1, 2, 1}, j_incr[4] = {1, 2, 1, 2};
            const int i_end[4] = {d1 - 1, d1, d1 - 1, d1}, j_end[4] = {d2, d2 - 1, d2, d2 - 1};
            const int rep_incr[4] = {d2, 1, d2, 1};
            sets.resize(4);
            for (int set = 0; set < 4; ++set) {
                int v = set % 2;
                for (int i = i_start[set]; i < i_end[set]; i += i_incr[set])
                    for (int j = j_start[set]; j < j_end[set]; j += j_incr[set]) {
                        int a = i * d2 + j;
                        sets[set].push_back(std::make_tuple(a, a + rep_incr[set], v * d1 * d2 + i * d2 + j));
                    }
            }
            n_ctr = 2 * d1 * d2;
        }
        vector<double> slot(4 * n_rungs);
        for (int k = 0; k < n_rungs; ++k) {
            slot[k] = tq[k];
            slot[n_rungs + k] = uq[k];
            slot[2 * n_rungs + k] = bq[k];
            slot[3 * n_rungs + k] = sq[k];
        }
        // m_reduced_staple_us from molarity_to_chempots at the input temperature
        // (src/origami_system.cpp:965-989)
        int S = hs.desc.n_types - 1;
        vector<double> red(std::max(S, 1));
        for (int t = 1; t <= S; ++t) {
            double n = (double)hs.sf.identities[t].size();
            double extra = (2 * n - 1) * std::log(6);
            double u = p.temp * (std::log(p.staple_M) - extra);
            red[t - 1] = u / p.temp;
        }
        vector<int> tab_slot(n_rungs);
        for (int k = 0; k < n_rungs; ++k) tab_slot[k] = table_for(sys_of[0], tq[k], (exchange_q & 8) ? sq[k] : 1.0);
        vector<double> rep_q(4 * n_rep);
        vector<int> perm(n_rep);
        for (int l = 0; l < nl; ++l)
            for (int k = 0; k < n_rungs; ++k) {
                int r = l * n_rungs + k;
                perm[r] = r;
                rep_q[4 * r] = tq[k];
                rep_q[4 * r + 1] = uq[k];
                rep_q[4 * r + 2] = bq[k];
                rep_q[4 * r + 3] = sq[k];
                temps[r] = tq[k];
                stack_mults[r] = (exchange_q & 8) ? sq[k] : 1.0;
                h_ctl[r].tab = tab_slot[k];
                h_ctl[r].staple_u_mult = uq[k];
            }
        upload_tables();
        upload_ctl();
        d_slot_q.alloc(slot.size());
        CU(copy(d_slot_q.p, slot.data(), slot.size() * sizeof(double), cudaMemcpyHostToDevice));
        d_red_u.alloc(red.size());
        CU(copy(d_red_u.p, red.data(), red.size() * sizeof(double), cudaMemcpyHostToDevice));
        d_rep_q.alloc(rep_q.size());
        CU(copy(d_rep_q.p, rep_q.data(), rep_q.size() * sizeof(double), cudaMemcpyHostToDevice));
        d_perm.alloc(perm.size());
        CU(copy(d_perm.p, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice));
        d_tab_slot.alloc(n_rungs);
        CU(copy(d_tab_slot.p, tab_slot.data(), n_rungs * sizeof(int), cudaMemcpyHostToDevice));
        d_pt_draws.alloc(nl);
        CU(cudaMemsetAsync(d_pt_draws.p, 0, nl * sizeof(unsigned long long), stream));
        d_pt_att.alloc(std::max(n_ctr, 1));
        d_pt_acc.alloc(std::max(n_ctr, 1));
        CU(cudaMemsetAsync(d_pt_att.p, 0, std::max(n_ctr, 1) * sizeof(long long), stream));
        CU(cudaMemsetAsync(d_pt_acc.p, 0, std::max(n_ctr, 1) * sizeof(long long), stream));
        vector<int> set_start(1, 0), pa, pb, pc;
        for (auto& st : sets) {
            for (auto& t : st) {
                pa.push_back(std::get<0>(t));
                pb.push_back(std::get<1>(t));
                pc.push_back(std::get<2>(t));
            }
            set_start.push_back((int)pa.size());
        }
        vector<int> sched(set_start);
        sched.insert(sched.end(), pa.begin(), pa.end());
        sched.insert(sched.end(), pb.begin(), pb.end());
        sched.insert(sched.end(), pc.begin(), pc.end());
        d_pt_sched.alloc(std::max<size_t>(sched.size(), 1));
        CU(copy(d_pt_sched.p, sched.data(), sched.size() * sizeof(int), cudaMemcpyHostToDevice));
        pt = LdoPT {};
        pt.n_ladders = nl;
        pt.n_rungs = n_rungs;
        pt.exchange_q = exchange_q;
        pt.n_types = hs.desc.n_types;
        pt.slot_temp = d_slot_q.p;
        pt.slot_u = d_slot_q.p + n_rungs;
        pt.slot_bias = d_slot_q.p + 2 * n_rungs;
        pt.slot_stack = d_slot_q.p + 3 * n_rungs;
        pt.red_u = d_red_u.p;
        pt.perm = d_perm.p;
        pt.rep_q = d_rep_q.p;
        pt.tab_slot = d_tab_slot.p;
        pt.ctl = d_ctl.p;
        pt.arena = d_arena.p;
        pt.lay = lay;
        pt.draws = d_pt_draws.p;
        pt.att = d_pt_att.p;
        pt.acc = d_pt_acc.p;
        pt.seed = seed;
        pt.n_sets = (int)sets.size();
        pt.set_start = d_pt_sched.p;
        pt.pair_a = d_pt_sched.p + set_start.size();
        pt.pair_b = pt.pair_a + pa.size();
        pt.pair_ctr = pt.pair_b + pb.size();
        pt_rungs = n_rungs;
        pt_q = exchange_q;
        pt_dim2 = dim2;
        pt_nctr = n_ctr;
        pt_swap_i = 0;
        pt_slot_q = slot;
        hist_cap = 0;   // a new ladder shape drops the swap history
        if (pt_graph) {
            cudaGraphExecDestroy(pt_graph);
            pt_graph = nullptr;
        }
    }

    // Record the pre-exchange permutation of every round (ring of cap rows
    // per ladder, the .swp rows).
    void pt_record_swaps(long long cap) {
        int nl = n_rep / pt_rungs;
        d_hist_perm.alloc((size_t)cap * nl * pt_rungs);
        d_hist_step.alloc((size_t)cap * nl);
        d_hist_n.alloc(nl);
        CU(cudaMemsetAsync(d_hist_n.p, 0, nl * sizeof(long long), stream));
        hist_cap = cap;
        pt.hist_perm = d_hist_perm.p;
        pt.hist_step = d_hist_step.p;
        pt.hist_n = d_hist_n.p;
        pt.hist_cap = cap;
    }

    // One PTGCMCSimulation::run iteration (src/ptmc_simulation.cpp:110-141):
    // update_control_qs (energy recomputed with the slot's tables), simulate,
    // update_dependent_qs, attempt_exchange.
    void pt_round(long long swap_i, int exchange_interval) {
        LdoLaunch L = launch_params(LDO_MODE_RUN, exchange_interval);
        L.force_recompute = 1;
        L.want_dep = 1;
        CU(launch_mc(L));
        LdoPT P = pt;
        P.swap_i = (int)(swap_i % pt.n_sets);
        count_launch();
        CU(ldo_launch_pt_swap(P, stream));
    }

    void pt_run(int n_rungs, long long swaps, int exchange_interval, int exchange_q, double* ms, int dim2 = 0) {
        if (n_rungs != pt_rungs || exchange_q != pt_q || dim2 != pt_dim2) {
            if (pt_graph) {
                cudaGraphExecDestroy(pt_graph);
                pt_graph = nullptr;
            }
            pt_setup(n_rungs, exchange_q, dim2);
        }
        if (swaps < 0 || exchange_interval < 0) throw LdoError(LDO_EINVAL, "negative swaps or interval");
        CU(cudaEventRecord(ev0, stream));
        long long done = 0;
        // Rounds cycle through the pair sets; one cycle of rounds (swap
        // counters 1..n_sets) forms one CUDA graph.
        int period = pt.n_sets;
        if (swaps >= 2 * period) {
            // the graph holds the launch parameters by value (interval,
            // sampling and trace buffers): capture again when they changed
            LdoLaunch now = launch_params(LDO_MODE_RUN, exchange_interval);
            if (pt_graph && (std::memcmp(&now, &pt_graph_L, sizeof(LdoLaunch)) != 0 ||
                             std::memcmp(&pt, &pt_graph_P, sizeof(LdoPT)) != 0)) {
                cudaGraphExecDestroy(pt_graph);
                pt_graph = nullptr;
            }
            if (!pt_graph) {
                cudaGraph_t g;
                CU(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                {
                    // captured launches run (and count) when the graph is launched
                    struct Flag {
                        bool& f;
                        ~Flag() { f = false; }
                    } flag {capturing};
                    capturing = true;
                    for (int k = 1; k <= period; ++k) pt_round(k, exchange_interval);
                }
                CU(cudaStreamEndCapture(stream, &g));
                CU(cudaGraphInstantiate(&pt_graph, g, 0));
                cudaGraphDestroy(g);
                pt_graph_L = now;
                pt_graph_P = pt;
            }
            // the graph starts with swap counter 1 (mod period): align
            while (pt_swap_i % period != 0 && done < swaps) {
                pt_round(pt_swap_i + 1, exchange_interval);
                ++pt_swap_i;
                ++done;
            }
            while (swaps - done >= period) {
                CU(cudaGraphLaunch(pt_graph, stream));
                count_launch(2 * period);
                pt_swap_i += period;
                done += period;
            }
        }
        while (done < swaps) {
            pt_round(pt_swap_i + 1, exchange_interval);
            ++pt_swap_i;
            ++done;
        }
        CU(cudaEventRecord(ev1, stream));
        CU(cudaStreamSynchronize(stream));
        if (ms) {
            float f = 0;
            CU(cudaEventElapsedTime(&f, ev0, ev1));
            *ms = f;
        }
        // host mirror of the replicas' current temperatures
        vector<double> rq(4 * n_rep);
        CU(copy(rq.data(), d_rep_q.p, rq.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (int r = 0; r < n_rep; ++r) temps[r] = rq[4 * r];
        CU(copy(h_ctl.data(), d_ctl.p, h_ctl.size() * sizeof(LdoRepCtl), cudaMemcpyDeviceToHost));
        check_status();
    }
    LdoLaunch pt_graph_L {};
    LdoPT pt_graph_P {};

    // ------------------------------------------------ umbrella sampling ----
    static uint64_t host_philox_word(uint32_t seed, uint32_t key1, uint32_t stream, unsigned long long draw) {
        unsigned long long b = draw >> 1;
        uint32_t c0 = (uint32_t)b, c1 = (uint32_t)(b >> 32), c2 = stream, c3 = 0, k0 = seed, k1 = key1;
        for (int r = 0; r < 10; ++r) {
            uint64_t p0 = (uint64_t)0xD2511F53u * c0;
            uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
            uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
            uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
            c0 = n0; c1 = n1; c2 = n2; c3 = n3;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t w[4] = {c0, c1, c2, c3};
        int j = (int)(draw & 1) * 2;
        return ((uint64_t)w[j] << 32) | w[j + 1];
    }
    double us_uniform() {   // window-exchange stream: key (seed, 0), stream 2
        uint64_t x = host_philox_word(seed, 0u, 2u, us_swap_draws++);
        return (double)(x >> 11) * 0x1.0p-53;
    }

    void us_setup(const string& grid_tag) {
        const HostSystem& hs = systems[sys_of[0]];
        for (int r = 0; r < n_rep; ++r)
            if (sys_of[r] != sys_of[0]) throw LdoError(LDO_EINVAL, "umbrella windows must share one system");
        us_bias = -1;
        for (int b = 0; b < hs.desc.n_biases; ++b)
            if (hs.biases[b].tag == grid_tag && hs.desc.bias_kind[b] == LDO_B_GRID) us_bias = b;
        if (us_bias < 0) throw LdoError(LDO_EINVAL, "us_grid_bias_tag " + grid_tag + " is not a Grid bias function");
        us_len = hs.desc.bias_grid_len[us_bias];
        int nw = n_rep;
        us_win.assign(nw, USWindow {});
        us_sq_bias = -1;
        if (!hs.p.windows_file.empty()) {
            ldo_io::Windows w;
            try {
                w = ldo_io::read_windows(ldo_io::resolve(hs.p, hs.p.windows_file));
            } catch (std::exception& x) {
                throw LdoError(LDO_EINVAL, x.what());
            }
            if ((int)w.bounds.size() != nw)
                throw LdoError(LDO_EINVAL, "number of windows must equal the number of replicas");
            for (int b = 0; b < hs.desc.n_biases; ++b)
                if (hs.biases[b].tag == w.bias_tag) us_sq_bias = b;
            if (us_sq_bias < 0) throw LdoError(LDO_EINVAL, "window bias function " + w.bias_tag + " not found");
            for (int i = 0; i < nw; ++i) {
                us_win[i].min_op = w.bounds[i].first;
                us_win[i].max_op = w.bounds[i].second;
            }
        }
        else {
            for (int i = 0; i < nw; ++i) {
                us_win[i].min_op = 0;
                us_win[i].max_op = us_len - 1;
            }
        }
        for (auto& w : us_win) {
            w.E_w.assign(us_len, 0.0);
            w.in_S.assign(us_len, 0);
            w.in_file.assign(us_len, 0);
        }
        // read_biases (USGCMCSimulation constructor, src/us_simulation.cpp:48-66,
        // with the window's file name of MWUSGCMCSimulation::setup_window_sims,
        // :527-531): each window's grid biases from a .biases file
        if (hs.p.read_biases) {
            for (int i = 0; i < nw; ++i) {
                string f = hs.p.windows_file.empty()
                                   ? hs.p.biases_file
                                   : hs.p.biases_filebase +
                                             ldo_io::window_postfix({us_win[i].min_op}, {us_win[i].max_op}) +
                                             ".biases";
                us_read_biases(i, ldo_io::resolve(hs.p, f));
            }
        }
        us_window_of.resize(n_rep);
        us_replica_of.resize(nw);
        for (int r = 0; r < n_rep; ++r) {
            us_window_of[r] = r;
            us_replica_of[r] = r;
        }
        us_att.assign(std::max(nw - 1, 1), 0);
        us_acc.assign(std::max(nw - 1, 1), 0);
        us_swap_draws = 0;
        us_iters_done = 0;
        us_tag = grid_tag;
        d_us_hist.alloc((size_t)nw * us_len);
        d_us_window.alloc(n_rep);
        us_apply_windows();
    }

    // USGCMCSimulation::read_weights (src/us_simulation.cpp:192) into window
    // w: every 1-D grid point of the file becomes an entry of its biases.
    void us_read_biases(int w, const string& path) {
        vector<ldo_io::GridBias> g;
        try {
            if (!ldo_io::file_exists(path)) throw std::runtime_error("Restart bias file " + path + " does not exist");
            g = ldo_io::read_biases_json(path);
        } catch (std::exception& x) {
            throw LdoError(LDO_EINVAL, x.what());
        }
        USWindow& W = us_win.at(w);
        for (auto& e : g) {
            if (e.point.size() != 1) throw LdoError(LDO_EINVAL, path + ": the grid order parameter is one-dimensional");
            int x = e.point[0];
            if (x < 0 || x >= us_len) throw LdoError(LDO_EINVAL, path + ": grid point outside the order parameter's range");
            W.E_w[x] = e.bias;
            W.in_file[x] = 1;
        }
    }

    // USGCMCSimulation::output_weights (src/us_simulation.cpp:208) of window
    // w: the points that have a bias entry (visited or read), in ascending
    // order.
    void us_write_biases(int w, const string& path) const {
        const USWindow& W = us_win.at(w);
        vector<ldo_io::GridBias> g;
        for (int x = 0; x < us_len; ++x)
            if (W.in_S[x] || W.in_file[x]) g.push_back(ldo_io::GridBias {{x}, W.E_w[x]});
        std::ofstream f(path);
        if (!f) throw LdoError(LDO_EINVAL, path + ": cannot open for writing");
        f << ldo_io::biases_json_text(g);
        if (!f) throw LdoError(LDO_EINVAL, path + ": writing failed");
    }

    // Window restraint and grid values of every replica follow the window it holds
    // (MWUSGCMCSimulation::setup_window_restraints, src/us_simulation.cpp:503).
    void us_apply_windows() {
        for (int r = 0; r < n_rep; ++r) {
            const USWindow& w = us_win[us_window_of[r]];
            if (us_sq_bias >= 0) {
                h_ctl[r].win_min[us_sq_bias] = w.min_op;
                h_ctl[r].win_max[us_sq_bias] = w.max_op;
            }
            int off = h_ctl[r].grid_off[us_bias];
            for (int x = 0; x < us_len; ++x) h_grid[off + x] = w.E_w[x];
        }
        upload_ctl();
        upload_grid();
        CU(copy(d_us_window.p, us_window_of.data(), n_rep * sizeof(int), cudaMemcpyHostToDevice));
    }

    void us_launch(long long steps, bool record) {
        LdoLaunch L = launch_params(LDO_MODE_RUN, steps);
        if (record) {
            L.us_hist = d_us_hist.p;
            L.us_window = d_us_window.p;
            L.us_bias = us_bias;
            L.us_len = us_len;
        }
        CU(launch_mc(L));
    }

    // PTMWUSGCMCSimulation::attempt_exchange (src/us_simulation.cpp:770-864):
    // neighbouring windows of parity swap_i % 2 exchange when both grid points
    // lie in the other window, with probability min(1, exp(bias difference)).
    void us_exchange(int swap_i) {
        int nw = (int)us_win.size();
        vector<int> point(nw, -1);
        auto host = download_arena();
        const HostSystem& hs = systems[sys_of[0]];
        int oq = hs.desc.bias_op[us_bias];
        for (int w = 0; w < nw; ++w) {
            int r = us_replica_of[w];
            const auto* op = reinterpret_cast<const int32_t*>(host.data() + (size_t)r * lay.bytes + lay.o_op);
            point[w] = op[2 * oq];
        }
        for (int i = swap_i % 2; i < nw - 1; i += 2) {
            us_att[i]++;
            int w1 = i, w2 = i + 1;
            int p1 = point[w1], p2 = point[w2];
            bool inside = !(p2 < us_win[w1].min_op || p2 > us_win[w1].max_op) &&
                          !(p1 < us_win[w2].min_op || p1 > us_win[w2].max_op);
            if (!inside) continue;
            bool accepted = true;
            if (p1 != p2) {
                auto bias_at = [&](int w, int p) { return (p >= 0 && p < us_len) ? us_win[w].E_w[p] : 0.0; };
                double d1 = bias_at(w1, p1) - bias_at(w2, p1);
                double d2 = bias_at(w2, p2) - bias_at(w1, p2);
                double pa = std::min(1.0, std::exp(d1 + d2));
                accepted = (pa == 1) ? true : (pa > us_uniform());
            }
            if (accepted) {
                us_acc[i]++;
                int r1 = us_replica_of[w1], r2 = us_replica_of[w2];
                us_replica_of[w1] = r2;
                us_replica_of[w2] = r1;
                us_window_of[r1] = w2;
                us_window_of[r2] = w1;
            }
        }
        us_apply_windows();
    }

    // SimpleUSGCMCSimulation::process_iteration (src/us_simulation.cpp:154,
    // 286-416): reweight this iteration's visits by the biases it ran with,
    // set each visited point's bias to ln p (a point seen before but not now
    // loses max_D_bias), and limit every change to max_D_bias.
    void us_process_iteration(const vector<int>& hist, double max_D) {
        int nw = (int)us_win.size();
        for (int w = 0; w < nw; ++w) {
            USWindow& W = us_win[w];
            const int* f = hist.data() + (size_t)w * us_len;
            double ave = 0;
            for (int x = 0; x < us_len; ++x)
                if (f[x] > 0) ave += f[x] * std::exp(W.E_w[x]);
            vector<double> p(us_len, 0.0);
            for (int x = 0; x < us_len; ++x)
                if (f[x] > 0) p[x] = f[x] * std::exp(W.E_w[x]) / ave;
            for (int x = 0; x < us_len; ++x)
                if (f[x] > 0) W.in_S[x] = 1;
            for (int x = 0; x < us_len; ++x) {
                if (!W.in_S[x]) continue;
                double old_bias = W.E_w[x];
                double D, nb;
                if (p[x] == 0) {
                    D = -max_D;
                    nb = old_bias + D;
                }
                else {
                    nb = std::log(p[x]);
                    D = nb - old_bias;
                }
                double upd = nb;
                if (std::abs(D) > max_D) upd = D > 0 ? old_bias + max_D : old_bias - max_D;
                W.E_w[x] = upd;
            }
        }
        us_apply_windows();
    }

    void us_run(const string& tag, int n_iters, long long equil_steps, long long iter_steps, double max_D,
                int exchange_interval, double* ms) {
        // A second run with the same grid bias continues the iterations (the
        // reference restarts them from its archives, :312-344); equil_steps
        // run before this call's first iteration.
        if (us_tag != tag || us_win.empty()) us_setup(tag);
        CU(cudaEventRecord(ev0, stream));
        // USGCMCSimulation::run_equilibration
        if (equil_steps > 0) us_launch(equil_steps, false);
        int nw = (int)us_win.size();
        vector<int> hist((size_t)nw * us_len);
        for (int n = 0; n < n_iters; ++n) {
            CU(cudaMemsetAsync(d_us_hist.p, 0, hist.size() * sizeof(int), stream));
            if (exchange_interval > 0) {
                long long swaps = iter_steps / exchange_interval;
                for (long long s = 1; s <= swaps; ++s) {
                    us_launch(exchange_interval, true);
                    us_exchange((int)s);
                }
            }
            else {
                us_launch(iter_steps, true);
            }
            count_copy(hist.size() * sizeof(int), cudaMemcpyDeviceToHost);
            CU(cudaMemcpyAsync(hist.data(), d_us_hist.p, hist.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
            CU(cudaStreamSynchronize(stream));
            check_status();
            us_process_iteration(hist, max_D);
            ++us_iters_done;
        }
        CU(cudaEventRecord(ev1, stream));
        CU(cudaStreamSynchronize(stream));
        if (ms) {
            float f = 0;
            CU(cudaEventElapsedTime(&f, ev0, ev1));
            *ms = f;
        }
        check_status();
    }

    vector<double> enum_units;   // last enumeration: (partition sum, configurations) per unit
    vector<double> enum_unit_w;  // last enumeration: per unit, its (op1, op2) weights before normalisation
    int enum_n1 {0}, enum_n2 {0};

    // Exact staple-only enumeration (enumerate_main with
    // enumerate_staples_only, src/enumerate.cpp:19) of replica 0's system at
    // its temperature: normalised weights over (op1, op2) into w[n1 * n2].
    void enumerate(int min_total, int max_total, int max_type, int op1, int op2, int n1, int n2, double* w,
                   double* num_configs, int* n_units, double* ms, int full = 0, int split = 0) {
        const HostSystem& hs = systems[sys_of[0]];
        if (split < 0 || split > LDO_ENUM_MAX_SPLIT) throw LdoError(LDO_EINVAL, "enumeration: split levels 0.." + std::to_string(LDO_ENUM_MAX_SPLIT));
        for (auto& ids : hs.sf.identities)
            for (int d : ids)
                if (d > LDO_ENUM_MAX_IDENT || d < -LDO_ENUM_MAX_IDENT)
                    throw LdoError(LDO_EINVAL, "enumeration: domain identities beyond +-64");
        if (hs.desc.n_biases != 0) throw LdoError(LDO_EINVAL, "enumeration: bias functions are not supported");
        if (hs.desc.has_ct) throw LdoError(LDO_EINVAL, "enumeration: the scaffold must stay fixed");
        if (op1 < 0 || op1 >= hs.desc.n_ops || op2 < 0 || op2 >= hs.desc.n_ops || n1 < 1 || n2 < 1)
            throw LdoError(LDO_EINVAL, "enumeration: bad order parameters or histogram shape");
        if (hs.sf.chains.size() != 1) throw LdoError(LDO_EINVAL, "enumeration: the system must start without staples");
        if (max_total > hs.desc.kmax)
            throw LdoError(LDO_EINVAL, "enumeration: more staples than the system's max_total_staples");
        LdoHdr h0 {};
        CU(copy(&h0, d_arena.p + lay.o_hdr, sizeof h0, cudaMemcpyDeviceToHost));
        if (h0.num_staples != 0 || h0.n_chains != 1)
            throw LdoError(LDO_EINVAL, "enumeration: replica 0 must hold the scaffold only (enumerate before any run)");
        int overcount;
        if (hs.p.max_staple_size == 2) overcount = 0;
        else if (hs.p.misbinding_pot == "Disallowed") overcount = 1;
        else throw LdoError(LDO_EINVAL, "No enumerator available for system");
        EnumBuilder b(hs.sf.identities, hs.p.misbinding_pot != "Disallowed", 1u << 22);
        b.run(min_total, max_total, max_type);
        int nu = (int)b.units.size();
        int parts = 1;
        for (int k = 0; k < split; ++k) parts *= 6;
        size_t nb = (size_t)nu * parts;   // one block per part of a unit
        size_t stride = ldo_enum_work_bytes(lay.cls);
        if (nb * (stride + 2 * (size_t)n1 * n2 * sizeof(double)) > ((size_t)8 << 30))
            throw LdoError(LDO_ECAPACITY, "enumeration: more than 8 GiB of per-part working memory");
        DevBuf<LdoEnumUnit> d_units;
        d_units.alloc(nu);
        CU(copy(d_units.p, b.units.data(), nu * sizeof(LdoEnumUnit), cudaMemcpyHostToDevice));
        DevBuf<unsigned char> d_work;
        d_work.alloc(nb * stride);
        DevBuf<double> d_hist, d_stats;
        d_hist.alloc(nb * 2 * n1 * n2);   // per part: weights, then the compensations of their sums
        d_stats.alloc(nb * 4);
        LdoEnumLaunch E {};
        E.L = launch_params(LDO_MODE_RUN, 0);
        E.state = d_arena.p;
        E.units = d_units.p;
        E.n_units = nu;
        E.full = full;
        E.split = split;
        E.work = d_work.p;
        E.work_stride = stride;
        E.hist = d_hist.p;
        E.stats = d_stats.p;
        E.op1 = op1;
        E.op2 = op2;
        E.n1 = n1;
        E.n2 = n2;
        E.overcount = overcount;
        // the recursion is deep: a larger per-thread stack for this launch
        size_t old_stack = 0;
        CU(cudaDeviceGetLimit(&old_stack, cudaLimitStackSize));
        CU(cudaDeviceSetLimit(cudaLimitStackSize, 16384));
        CU(cudaEventRecord(ev0, stream));
        count_launch();
        cudaError_t err = ldo_launch_enum(E, stream);
        if (err == cudaSuccess) err = cudaEventRecord(ev1, stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
        cudaDeviceSetLimit(cudaLimitStackSize, old_stack);
        CU(err);
        if (ms) {
            float f = 0;
            CU(cudaEventElapsedTime(&f, ev0, ev1));
            *ms = f;
        }
        const size_t nk = (size_t)n1 * n2;
        vector<double> hist(nb * 2 * nk), stats(nb * 4);
        CU(copy(hist.data(), d_hist.p, hist.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CU(copy(stats.data(), d_stats.p, stats.size() * sizeof(double), cudaMemcpyDeviceToHost));
        // every sum over parts compensated, as the parts' own sums are
        CompSum part, nconf;
        vector<CompSum> wt(nk), uw(nk);
        enum_units.assign(2 * (size_t)nu, 0.0);
        enum_unit_w.assign((size_t)nu * nk, 0.0);
        enum_n1 = n1;
        enum_n2 = n2;
        CompSum upart, uconf;
        for (size_t q = 0; q < nb; ++q) {   // parts in unit order, each unit's parts in branch order
            if (stats[4 * q + 3] < 0) throw LdoError(LDO_EINVAL, "enumeration: an order parameter value outside the histogram");
            if (stats[4 * q + 3] > 0) throw LdoError((ldo_status)(int)stats[4 * q + 3], "enumeration: a unit failed");
            part.add(stats[4 * q]);
            nconf.add(stats[4 * q + 1]);
            upart.add(stats[4 * q]);
            uconf.add(stats[4 * q + 1]);
            const double* h = hist.data() + q * 2 * nk;   // the folded sums; the scratch half follows
            for (size_t k = 0; k < nk; ++k) {
                wt[k].add(h[k]);
                uw[k].add(h[k]);
            }
            if ((q + 1) % parts == 0) {   // the unit's last part
                size_t u = q / parts;
                enum_units[2 * u] = upart.value();
                enum_units[2 * u + 1] = uconf.value();
                for (size_t k = 0; k < nk; ++k) enum_unit_w[u * nk + k] = uw[k].value();
                upart = uconf = CompSum {};
                for (auto& c : uw) c = CompSum {};
            }
        }
        // ConformationalEnumerator::normalize_weights (:344)
        for (size_t k = 0; k < nk; ++k) w[k] = wt[k].value() / part.value();
        if (num_configs) *num_configs = nconf.value();
        if (n_units) *n_units = nu;
    }

    // replica 0's sample counter; replica r's is lay.bytes * r further
    unsigned char* sample_count_ptr() {
        return reinterpret_cast<unsigned char*>(d_arena.p) + lay.o_hdr + offsetof(LdoHdr, sample_count);
    }

    vector<unsigned char> download_arena() {
        vector<unsigned char> host((size_t)n_rep * lay.bytes);
        CU(copy(host.data(), d_arena.p, host.size(), cudaMemcpyDeviceToHost));
        return host;
    }
};

namespace {

ldo_status guard(ldo_engine* e, const std::function<void()>& f) {
    try {
        f();
        if (e) e->err.clear();
        return LDO_OK;
    } catch (LdoError& x) {
        if (e) e->err = x.what();
        else g_create_err = x.what();
        return x.code;
    } catch (std::exception& x) {
        if (e) e->err = x.what();
        else g_create_err = x.what();
        return LDO_EINVAL;
    }
}

} // namespace

extern "C" {

ldo_status ldo_create_multi(const char* const* inp_paths, int n_systems, const char* overrides,
                            const int* sys_of_replica, int n_replicas, uint32_t seed, ldo_engine** out) {
    if (!out || !inp_paths || n_systems <= 0 || n_replicas <= 0) {
        g_create_err = "invalid arguments";
        return LDO_EINVAL;
    }
    *out = nullptr;
    auto* e = new ldo_engine;
    vector<string> inps;
    for (int i = 0; i < n_systems; ++i) inps.push_back(inp_paths[i]);
    vector<int> so(n_replicas, 0);
    if (sys_of_replica)
        for (int r = 0; r < n_replicas; ++r) so[r] = sys_of_replica[r];
    ldo_status st = guard(nullptr, [&]() { e->create(inps, overrides ? overrides : "", so, seed); });
    if (st != LDO_OK) {
        delete e;
        return st;
    }
    *out = e;
    return LDO_OK;
}

ldo_status ldo_create_from_inp(const char* inp_path, const char* overrides, int n_replicas, uint32_t seed,
                               ldo_engine** out) {
    const char* p[1] = {inp_path};
    return ldo_create_multi(p, 1, overrides, nullptr, n_replicas, seed, out);
}

void ldo_destroy(ldo_engine* e) { delete e; }

const char* ldo_last_error(const ldo_engine* e) { return e ? e->err.c_str() : g_create_err.c_str(); }

int ldo_num_replicas(const ldo_engine* e) { return e ? e->n_rep : 0; }

ldo_status ldo_run(ldo_engine* e, int64_t n_steps, double* device_ms) {
    if (!e || n_steps < 0) return LDO_EINVAL;
    return guard(e, [&]() { e->run(n_steps, device_ms); });
}

ldo_status ldo_run_sweeps(ldo_engine* e, int64_t n_sweeps, double* device_ms) {
    if (!e || n_sweeps < 0) return LDO_EINVAL;
    return guard(e, [&]() { e->run(n_sweeps, device_ms, 1); });
}

int ldo_state_bytes(const ldo_engine* e) { return e ? e->lay.bytes : 0; }

namespace {
ldo_status enumerate_call(ldo_engine* e, int32_t min_total, int32_t max_total, int32_t max_type, const char* op1_tag,
                          const char* op2_tag, int32_t n1, int32_t n2, double* weights, double* num_configs,
                          int32_t* n_units, double* device_ms, int full, int split) {
    if (!e || !op1_tag || !op2_tag || !weights || min_total < 0 || max_total < min_total || max_type < 1)
        return LDO_EINVAL;
    return guard(e, [&]() {
        const HostSystem& hs = e->systems[e->sys_of[0]];
        auto find = [&](const char* tag) {
            for (size_t q = 0; q < hs.ops.size(); ++q)
                if (hs.ops[q].tag == tag) return (int)q;
            throw LdoError(LDO_EINVAL, string("enumeration: no order parameter ") + tag);
        };
        int nu = 0;
        e->enumerate(min_total, max_total, max_type, find(op1_tag), find(op2_tag), n1, n2, weights, num_configs, &nu,
                     device_ms, full, split);
        if (n_units) *n_units = nu;
    });
}
} // namespace

ldo_status ldo_enumerate(ldo_engine* e, int32_t min_total, int32_t max_total, int32_t max_type, const char* op1_tag,
                         const char* op2_tag, int32_t n1, int32_t n2, double* weights, double* num_configs,
                         int32_t* n_units, double* device_ms) {
    return enumerate_call(e, min_total, max_total, max_type, op1_tag, op2_tag, n1, n2, weights, num_configs, n_units,
                          device_ms, 0, 0);
}

ldo_status ldo_enumerate_full(ldo_engine* e, int32_t min_total, int32_t max_total, int32_t max_type,
                              const char* op1_tag, const char* op2_tag, int32_t n1, int32_t n2, int32_t split_levels,
                              double* weights, double* num_configs, int32_t* n_units, double* device_ms) {
    return enumerate_call(e, min_total, max_total, max_type, op1_tag, op2_tag, n1, n2, weights, num_configs, n_units,
                          device_ms, 1, split_levels);
}

ldo_status ldo_enumerate_unit_weights(ldo_engine* e, double* out, int64_t cap, int32_t* n_units) {
    if (!e || !n_units) return LDO_EINVAL;
    int nu = (int)(e->enum_units.size() / 2);
    *n_units = nu;
    if (!out) return LDO_OK;
    if (cap < (int64_t)e->enum_unit_w.size()) return LDO_EINVAL;
    std::copy(e->enum_unit_w.begin(), e->enum_unit_w.end(), out);
    return LDO_OK;
}

ldo_status ldo_enumerate_units(ldo_engine* e, double* out, int32_t cap, int32_t* n_units) {
    if (!e || !n_units) return LDO_EINVAL;
    int nu = (int)(e->enum_units.size() / 2);
    *n_units = nu;
    if (!out) return LDO_OK;
    if (cap < nu) return LDO_EINVAL;
    std::copy(e->enum_units.begin(), e->enum_units.end(), out);
    return LDO_OK;
}

ldo_status ldo_autotune(ldo_engine* e, int32_t probe_sweeps, int32_t use_cache, ldo_tune_report* out) {
    if (!e || probe_sweeps < 1 || !out) return LDO_EINVAL;
    return guard(e, [&]() {
        auto best = e->autotune(probe_sweeps, use_cache != 0);
        out->warps_per_block = best.wpb;
        out->smem_pad_bytes = best.pad;
        out->blocks_per_sm = best.blocks;
        out->interleaved = best.order;
        out->best_ms = best.ms;
        out->default_ms = e->tune_default.ms;
        out->n_candidates = (int32_t)e->tune_log.size();
    });
}

ldo_status ldo_autotune_candidates(ldo_engine* e, int32_t* shape, double* ms, int32_t cap) {
    if (!e || !shape || !ms || cap < (int32_t)e->tune_log.size()) return LDO_EINVAL;
    for (size_t k = 0; k < e->tune_log.size(); ++k) {
        const auto& c = e->tune_log[k];
        shape[4 * k] = c.wpb;
        shape[4 * k + 1] = c.pad;
        shape[4 * k + 2] = c.blocks;
        shape[4 * k + 3] = c.order;
        ms[k] = c.ms;
    }
    return LDO_OK;
}

ldo_status ldo_set_controls(ldo_engine* e, const double* temps, const double* stacking_mults,
                            const double* staple_u_mults, int n) {
    if (!e || n != e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() {
        for (int r = 0; r < n; ++r) {
            if (temps) e->temps[r] = temps[r];
            if (stacking_mults) e->stack_mults[r] = stacking_mults[r];
            if (staple_u_mults) e->u_mults[r] = staple_u_mults[r];
            if (!(e->temps[r] > 0)) throw LdoError(LDO_EINVAL, "temperature must be positive");
            e->h_ctl[r].tab = e->table_for(e->sys_of[r], e->temps[r], e->stack_mults[r]);
            e->h_ctl[r].staple_u_mult = e->u_mults[r];
        }
        e->upload_tables();
        e->upload_ctl();
        LdoLaunch L = e->launch_params(LDO_MODE_RECOMPUTE, 0);
        CU(e->launch_mc(L));
        CU(cudaStreamSynchronize(e->stream));
        e->check_status();
    });
}

ldo_status ldo_get_observables(ldo_engine* e, ldo_observables* out, int n) {
    if (!e || !out || n > e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() {
        LdoLaunch L = e->launch_params(LDO_MODE_OBSERVE, 0);
        L.want_dep = 1;
        CU(e->launch_mc(L));
        CU(cudaStreamSynchronize(e->stream));
        auto host = e->download_arena();
        for (int r = 0; r < n; ++r) {
            const auto* h = reinterpret_cast<const LdoHdr*>(host.data() + (size_t)r * e->lay.bytes + e->lay.o_hdr);
            ldo_observables& o = out[r];
            o.energy = h->energy;
            o.total_bias = h->move_bias * e->h_ctl[r].bias_mult;
            o.temp = e->temps[r];
            o.enthalpy = h->H;
            o.entropy = h->S;
            o.stacking = h->stacking;
            o.draws = (int64_t)h->draws;
            o.num_staples = h->num_staples;
            o.num_fully_bound = h->num_fully;
            o.num_bound = h->num_bound;
            o.num_self_bound = h->num_self;
            o.num_stacked = h->num_stacked;
            o.num_unassigned = h->num_unassigned;
            o.current_c_i = h->current_c_i;
            o.status = h->status;
        }
    });
}

ldo_status ldo_get_config(ldo_engine* e, int replica, int32_t* buf, int cap, int* written) {
    if (!e || replica < 0 || replica >= e->n_rep || !buf) return LDO_EINVAL;
    return guard(e, [&]() {
        vector<unsigned char> b(e->lay.bytes);
        CU(e->copy(b.data(), e->d_arena.p + (size_t)replica * e->lay.bytes, b.size(), cudaMemcpyDeviceToHost));
        const LdoLayout& y = e->lay;
        const LdoSys& d = e->systems[e->sys_of[replica]].desc;
        const auto* h = reinterpret_cast<const LdoHdr*>(b.data() + y.o_hdr);
        const auto* pp = reinterpret_cast<const long long*>(b.data() + y.o_pp);
        const unsigned char* ore = b.data() + y.o_ore;
        const unsigned char* st = b.data() + y.o_state;
        const auto* chain_c = reinterpret_cast<const int32_t*>(b.data() + y.o_chain_c);
        const unsigned char* chain_type = b.data() + y.o_chain_type;
        const unsigned char* chain_order = b.data() + y.o_chain_order;
        static const int U[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        vector<int32_t> out;
        out.push_back(h->n_chains);
        for (int c = 0; c < h->n_chains; ++c) {
            int cs = chain_order[c];
            int type = cs == 0 ? 0 : chain_type[cs];
            int len = d.type_len[type];
            out.push_back(chain_c[cs]);
            out.push_back(type);
            out.push_back(len);
            for (int dd = 0; dd < len; ++dd) {
                int s = cs == 0 ? dd : d.ns + (cs - 1) * d.lmax + dd;
                long long p = pp[s];
                int x = (int)(short)(unsigned short)(p & 0xffff);
                long long r1 = (p - x) >> 16;
                int yy = (int)(short)(unsigned short)(r1 & 0xffff);
                int z = (int)((r1 - yy) >> 16);
                out.push_back(x);
                out.push_back(yy);
                out.push_back(z);
                out.push_back(U[ore[s]][0]);
                out.push_back(U[ore[s]][1]);
                out.push_back(U[ore[s]][2]);
                out.push_back(st[s]);
            }
        }
        if ((int)out.size() > cap) throw LdoError(LDO_EINVAL, "config buffer too small");
        std::memcpy(buf, out.data(), out.size() * sizeof(int32_t));
        if (written) *written = (int)out.size();
    });
}

ldo_status ldo_set_config(ldo_engine* e, int replica, const int32_t* buf, int n) {
    if (!e || !buf || n <= 0) return LDO_EINVAL;
    return guard(e, [&]() { e->set_config(replica, buf, n); });
}

// AnnealingGCMCSimulation (src/annealing_simulation.cpp:12-50): from
// max_temp down to min_temp in steps of temp_interval, every replica is set to
// the temperature (update_temp with stacking multiplier 1; update_staple_us
// with multiplier 1 unless the staple concentration is held constant) and
// runs steps_per_temp steps; step numbers continue across temperatures.
ldo_status ldo_anneal_run(ldo_engine* e, double max_temp, double min_temp, double temp_interval,
                          int64_t steps_per_temp, int constant_staple_M, double* device_ms) {
    if (!e) return LDO_EINVAL;
    return guard(e, [&]() {
        if (!(temp_interval > 0) || steps_per_temp < 0)
            throw LdoError(LDO_EINVAL, "temp_interval must be positive and steps_per_temp not negative");
        if (std::fmod(max_temp - min_temp, temp_interval) != 0) throw LdoError(LDO_EINVAL, "Bad temperature interval");
        double total = 0;
        double temp = max_temp;
        while (temp >= min_temp) {
            for (int r = 0; r < e->n_rep; ++r) {
                e->temps[r] = temp;
                e->stack_mults[r] = 1.0;
                if (!constant_staple_M) e->u_mults[r] = 1.0;
                e->h_ctl[r].tab = e->table_for(e->sys_of[r], temp, 1.0);
                e->h_ctl[r].staple_u_mult = e->u_mults[r];
            }
            e->upload_tables();
            e->upload_ctl();
            double ms = 0;
            e->run(steps_per_temp, &ms);   // recomputes the energy with the new tables first
            total += ms;
            temp -= temp_interval;
        }
        if (device_ms) *device_ms = total;
    });
}

ldo_status ldo_set_configs(ldo_engine* e, const int32_t* bufs, const int32_t* offsets, int n_replicas) {
    if (!e || !bufs || !offsets || n_replicas != e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() { e->set_configs(bufs, offsets); });
}

ldo_status ldo_read_trj_frame(const char* path, int frame, int32_t* buf, int cap, int* written) {
    if (!path || !buf || cap < 0) {
        g_create_err = "invalid arguments";
        return LDO_EINVAL;
    }
    return guard(nullptr, [&]() {
        vector<ldo_io::ChainConf> chains = ldo_io::read_trj_frame(path, frame);
        vector<int32_t> out;
        out.push_back((int32_t)chains.size());
        for (auto& c : chains) {
            out.push_back(c.index);
            out.push_back(c.identity);
            out.push_back((int32_t)c.positions.size());
            for (size_t d = 0; d < c.positions.size(); ++d) {
                for (int q = 0; q < 3; ++q) out.push_back(c.positions[d][q]);
                for (int q = 0; q < 3; ++q) out.push_back(c.orientations[d][q]);
                out.push_back(0);
            }
        }
        if ((int)out.size() > cap) throw LdoError(LDO_EINVAL, "config buffer too small");
        std::memcpy(buf, out.data(), out.size() * sizeof(int32_t));
        if (written) *written = (int)out.size();
    });
}

ldo_status ldo_checkpoint_save(ldo_engine* e, const char* path) {
    if (!e || !path) return LDO_EINVAL;
    return guard(e, [&]() { e->checkpoint_save(path); });
}

ldo_status ldo_checkpoint_load(ldo_engine* e, const char* path) {
    if (!e || !path) return LDO_EINVAL;
    return guard(e, [&]() { e->checkpoint_load(path); });
}

ldo_status ldo_set_sampling(ldo_engine* e, int interval, int capacity) {
    if (!e || interval < 0 || capacity < 0) return LDO_EINVAL;
    return guard(e, [&]() {
        e->sample_interval = interval;
        e->sample_cap = capacity;
        e->d_samples.alloc((size_t)e->n_rep * std::max(capacity, 1) * 2);
        CU(cudaMemsetAsync(e->d_samples.p, 0, e->d_samples.n * sizeof(int16_t), e->stream));
        // restart the per-replica sample counters: one int in each replica's
        // header, a strided set over the arena
        CU(cudaMemset2DAsync(e->sample_count_ptr(), e->lay.bytes, 0, sizeof(int), e->n_rep, e->stream));
        CU(cudaStreamSynchronize(e->stream));
    });
}

ldo_status ldo_get_samples(ldo_engine* e, int16_t* out, int capacity, int* count) {
    if (!e || !out || capacity != e->sample_cap) return LDO_EINVAL;
    return guard(e, [&]() {
        CU(e->copy(out, e->d_samples.p, (size_t)e->n_rep * capacity * 2 * sizeof(int16_t), cudaMemcpyDeviceToHost));
        if (count) {
            // the counters alone: a strided copy of one int per replica
            e->count_copy(sizeof(int) * e->n_rep, cudaMemcpyDeviceToHost);
            CU(cudaMemcpy2DAsync(count, sizeof(int), e->sample_count_ptr(), e->lay.bytes, sizeof(int), e->n_rep,
                                 cudaMemcpyDeviceToHost, e->stream));
            CU(cudaStreamSynchronize(e->stream));
        }
    });
}

ldo_status ldo_get_counters(ldo_engine* e, int64_t* launches, int64_t* h2d_bytes, int64_t* d2h_bytes) {
    if (!e) return LDO_EINVAL;
    if (launches) *launches = e->n_launches;
    if (h2d_bytes) *h2d_bytes = e->bytes_h2d;
    if (d2h_bytes) *d2h_bytes = e->bytes_d2h;
    return LDO_OK;
}

ldo_status ldo_set_trace(ldo_engine* e, int n_trace, int max_steps) {
    if (!e || n_trace < 0 || max_steps < 0) return LDO_EINVAL;
    return guard(e, [&]() {
        e->n_trace = std::min(n_trace, e->n_rep);
        e->trace_max = max_steps;
        e->d_trace.alloc((size_t)std::max(e->n_trace, 1) * std::max(max_steps, 1) * 8);
        CU(cudaMemsetAsync(e->d_trace.p, 0, e->d_trace.n * sizeof(double), e->stream));
    });
}

ldo_status ldo_get_trace(ldo_engine* e, double* out, int n_trace, int max_steps) {
    if (!e || !out || n_trace != e->n_trace || max_steps != e->trace_max) return LDO_EINVAL;
    return guard(e, [&]() {
        CU(e->copy(out, e->d_trace.p, (size_t)n_trace * max_steps * 8 * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

ldo_status ldo_get_move_stats(ldo_engine* e, int64_t* out, int n_moves) {
    if (!e || !out) return LDO_EINVAL;
    return guard(e, [&]() {
        auto host = e->download_arena();
        for (int m = 0; m < 2 * n_moves; ++m) out[m] = 0;
        for (int r = 0; r < e->n_rep; ++r) {
            const auto* ms = reinterpret_cast<const long long*>(host.data() + (size_t)r * e->lay.bytes + e->lay.o_mstat);
            int nm = std::min(n_moves, e->lay.nmv);
            for (int m = 0; m < 2 * nm; ++m) out[m] += ms[m];
        }
    });
}

ldo_status ldo_set_grid_bias(ldo_engine* e, const char* tag, int replica, const double* values, int n) {
    if (!e || !tag || !values || replica >= e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() {
        int r0 = replica < 0 ? 0 : replica, r1 = replica < 0 ? e->n_rep : replica + 1;
        bool found = false;
        for (int r = r0; r < r1; ++r) {
            const HostSystem& hs = e->systems[e->sys_of[r]];
            for (int b = 0; b < hs.desc.n_biases; ++b)
                if (hs.biases[b].tag == tag && hs.desc.bias_kind[b] == LDO_B_GRID) {
                    found = true;
                    int len = hs.desc.bias_grid_len[b];
                    for (int k = 0; k < len; ++k) e->h_grid[e->h_ctl[r].grid_off[b] + k] = k < n ? values[k] : 0.0;
                }
        }
        if (!found) throw LdoError(LDO_EINVAL, string("no Grid bias function tagged ") + tag);
        e->upload_grid();
        // Bias state follows the new grid at the next move (SystemBiases::calc_move).
    });
}

ldo_status ldo_pt_run(ldo_engine* e, int n_rungs, int64_t swaps, int exchange_interval, int exchange_q,
                      double* device_ms) {
    if (!e) return LDO_EINVAL;
    return guard(e, [&]() { e->pt_run(n_rungs, swaps, exchange_interval, exchange_q, device_ms); });
}

ldo_status ldo_pt_get_permutation(ldo_engine* e, int32_t* out, int n) {
    if (!e || !out || e->pt_rungs == 0 || n != e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() { CU(e->copy(out, e->d_perm.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost)); });
}

ldo_status ldo_pt2d_run(ldo_engine* e, int n_temps, int n_stacking, int64_t swaps, int exchange_interval,
                        double* device_ms) {
    if (!e || n_temps < 1 || n_stacking < 1) return LDO_EINVAL;
    return guard(e, [&]() {
        e->pt_run(n_temps * n_stacking, swaps, exchange_interval, 1 | 2 | 8, device_ms, n_stacking);
    });
}

ldo_status ldo_pt_get_stats(ldo_engine* e, int64_t* attempts, int64_t* accepts, int n_pairs) {
    if (!e || !attempts || !accepts || e->pt_rungs == 0 || n_pairs != e->pt_nctr) return LDO_EINVAL;
    return guard(e, [&]() {
        CU(e->copy(attempts, e->d_pt_att.p, n_pairs * sizeof(int64_t), cudaMemcpyDeviceToHost));
        CU(e->copy(accepts, e->d_pt_acc.p, n_pairs * sizeof(int64_t), cudaMemcpyDeviceToHost));
    });
}

ldo_status ldo_us_run(ldo_engine* e, const char* grid_tag, int n_iters, int64_t equil_steps, int64_t iter_steps,
                      double max_D_bias, int exchange_interval, double* device_ms) {
    if (!e || !grid_tag || n_iters < 0 || equil_steps < 0 || iter_steps < 0 || exchange_interval < 0)
        return LDO_EINVAL;
    return guard(e, [&]() {
        e->us_run(grid_tag, n_iters, equil_steps, iter_steps, max_D_bias, exchange_interval, device_ms);
    });
}

ldo_status ldo_us_write_biases(ldo_engine* e, int window, const char* path) {
    if (!e || !path) return LDO_EINVAL;
    return guard(e, [&]() {
        if (e->us_win.empty()) throw LdoError(LDO_EINVAL, "no umbrella-sampling state: run ldo_us_run first");
        if (window < 0 || window >= (int)e->us_win.size()) throw LdoError(LDO_EINVAL, "no such window");
        e->us_write_biases(window, path);
    });
}

ldo_status ldo_us_read_biases(ldo_engine* e, const char* grid_tag, int window, const char* path) {
    if (!e || !grid_tag || !path) return LDO_EINVAL;
    return guard(e, [&]() {
        if (e->us_tag != grid_tag || e->us_win.empty()) e->us_setup(grid_tag);
        if (window < 0 || window >= (int)e->us_win.size()) throw LdoError(LDO_EINVAL, "no such window");
        e->us_read_biases(window, path);
        e->us_apply_windows();
    });
}

ldo_status ldo_us_reset(ldo_engine* e) {
    if (!e) return LDO_EINVAL;
    return guard(e, [&]() {
        e->us_win.clear();
        e->us_tag.clear();
    });
}

ldo_status ldo_read_biases(const char* path, int32_t* points, double* biases, int cap, int* n, int* dim) {
    if (!path || !n || !dim) return LDO_EINVAL;
    return guard(nullptr, [&]() {
        auto g = ldo_io::read_biases_json(path);
        *n = (int)g.size();
        *dim = g.empty() ? 0 : (int)g[0].point.size();
        for (auto& x : g)
            if ((int)x.point.size() != *dim) throw LdoError(LDO_EINVAL, string(path) + ": points of mixed dimension");
        if (!points || !biases) return;
        if (cap < *n) throw LdoError(LDO_EINVAL, "output buffers too small");
        for (int i = 0; i < *n; ++i) {
            for (int j = 0; j < *dim; ++j) points[(size_t)i * *dim + j] = g[i].point[j];
            biases[i] = g[i].bias;
        }
    });
}

ldo_status ldo_us_get_biases(ldo_engine* e, double* out, int n_windows, int grid_len) {
    if (!e || !out || n_windows != (int)e->us_win.size() || grid_len != e->us_len) return LDO_EINVAL;
    return guard(e, [&]() {
        for (int w = 0; w < n_windows; ++w)
            for (int x = 0; x < grid_len; ++x) out[(size_t)w * grid_len + x] = e->us_win[w].E_w[x];
    });
}

ldo_status ldo_us_get_windows(ldo_engine* e, int32_t* window_of_replica, int n, int* grid_len) {
    if (!e || !window_of_replica || n != e->n_rep || e->us_win.empty()) return LDO_EINVAL;
    return guard(e, [&]() {
        for (int r = 0; r < n; ++r) window_of_replica[r] = e->us_window_of[r];
        if (grid_len) *grid_len = e->us_len;
    });
}

// Status read-out for callers that may not allocate device memory (a program
// whose pool allocator owns all device memory, a step loop that must not stall
// the device on cudaMalloc/cudaFree).  The scratch is a fixed device array of
// the library, whose device address is looked up on every call; nothing is
// allocated on the success path, on the device or the host.
ldo_status ldo_replica_status_noalloc(ldo_engine* e, int32_t* status_of_replica, int n, int32_t* worst,
                                      int32_t* n_bad) {
    if (!e || !worst || !n_bad) return LDO_EINVAL;
    if (n != e->n_rep) {
        e->err = "ldo_replica_status_noalloc: n must equal the engine's replica count";
        return LDO_EINVAL;
    }
    if (n > LDO_NOALLOC_MAX_REPLICAS) {
        e->err = "ldo_replica_status_noalloc: more replicas than the fixed status scratch holds (limit 65536)";
        return LDO_EINVAL;
    }
    // The scratch address is per device: make the engine's device current.
    cudaPointerAttributes attr {};
    cudaError_t err = cudaPointerGetAttributes(&attr, e->d_arena.p);
    int prev = 0;
    if (err == cudaSuccess) err = cudaGetDevice(&prev);
    if (err == cudaSuccess && attr.device != prev) err = cudaSetDevice(attr.device);
    if (err == cudaSuccess) {
        err = ldo_status_noalloc(e->d_arena.p, e->lay.bytes, e->lay.o_hdr, n, e->stream, status_of_replica, worst,
                                 n_bad);
        if (attr.device != prev) {
            cudaError_t back = cudaSetDevice(prev);
            if (err == cudaSuccess) err = back;
        }
    }
    if (err != cudaSuccess) {
        e->err = std::string("ldo_replica_status_noalloc: ") + cudaGetErrorString(err);
        return LDO_ECUDA;
    }
    return LDO_OK;
}

// The engine's exponential evaluated by the GPU, for host tools that need
// its exact bits (the same function as ldo_math::exp on the host).
ldo_status ldo_engine_exp(const double* x, double* y, int n) {
    if (n < 0 || (n > 0 && (!x || !y))) return LDO_EINVAL;
    if (n == 0) return LDO_OK;
    double *dx = nullptr, *dy = nullptr;
    cudaError_t err = cudaMalloc(&dx, (size_t)n * sizeof(double));
    if (err == cudaSuccess) err = cudaMalloc(&dy, (size_t)n * sizeof(double));
    if (err == cudaSuccess) err = cudaMemcpy(dx, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = ldo_launch_exp(dx, dy, n, 0);
    if (err == cudaSuccess) err = cudaMemcpy(y, dy, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
    if (dx) cudaFree(dx);
    if (dy) cudaFree(dy);
    return err == cudaSuccess ? LDO_OK : LDO_ECUDA;
}

ldo_status ldo_set_window(ldo_engine* e, const char* tag, int replica, int min_op, int max_op) {
    if (!e || !tag || replica < 0 || replica >= e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() {
        const HostSystem& hs = e->systems[e->sys_of[replica]];
        bool found = false;
        for (int b = 0; b < hs.desc.n_biases; ++b)
            if (hs.biases[b].tag == tag) {
                found = true;
                e->h_ctl[replica].win_min[b] = min_op;
                e->h_ctl[replica].win_max[b] = max_op;
            }
        if (!found) throw LdoError(LDO_EINVAL, string("no bias function tagged ") + tag);
        e->upload_ctl();
    });
}

ldo_status ldo_set_bias_centre(ldo_engine* e, const char* tag, int replica, double centre) {
    if (!e || !tag || replica < 0 || replica >= e->n_rep) return LDO_EINVAL;
    return guard(e, [&]() {
        const HostSystem& hs = e->systems[e->sys_of[replica]];
        bool found = false;
        for (int b = 0; b < hs.desc.n_biases; ++b)
            if (hs.biases[b].tag == tag) {
                if (hs.desc.bias_kind[b] != LDO_B_HARMONIC)
                    throw LdoError(LDO_EINVAL, string("bias function ") + tag + " is not Harmonic");
                found = true;
                e->h_ctl[replica].centre[b] = centre;
            }
        if (!found) throw LdoError(LDO_EINVAL, string("no bias function tagged ") + tag);
        e->upload_ctl();
    });
}

} // extern "C"

extern "C" {

ldo_status ldo_nn_duplex_thermo(const char* seq, double temp, double cation_M, double* h, double* s) {
    if (!seq || !h || !s || !(temp > 0) || !(cation_M > 0)) return LDO_EINVAL;
    return guard(nullptr, [&]() {
        static const ldo_host::NNParams P;
        ldo_host::HS x = ldo_host::reduce(ldo_host::duplex_hs(P, seq, cation_M), temp);
        *h = x.h;
        *s = x.s;
    });
}

ldo_status ldo_enumeration_plan(const char* inp_path, const char* overrides, int32_t min_total, int32_t max_total,
                                int32_t max_type, int32_t* out, int32_t cap, int32_t* n_units) {
    if (!inp_path || !n_units || min_total < 0 || max_total < min_total || max_type < 1) return LDO_EINVAL;
    return guard(nullptr, [&]() {
        HostSystem hs = load_system(inp_path, overrides ? overrides : "");
        if (hs.p.max_staple_size != 2 && hs.p.misbinding_pot != "Disallowed")
            throw LdoError(LDO_EINVAL, "No enumerator available for system");
        EnumBuilder b(hs.sf.identities, hs.p.misbinding_pot != "Disallowed", 1u << 22);
        b.run(min_total, max_total, max_type);
        *n_units = (int32_t)b.units.size();
        if (!out) return;
        if ((size_t)cap < 2 * b.units.size()) throw LdoError(LDO_EINVAL, "unit buffer too small");
        for (size_t u = 0; u < b.units.size(); ++u) {
            out[2 * u] = b.units[u].n_chains;
            out[2 * u + 1] = b.units[u].n_gp;
        }
    });
}

ldo_status ldo_energy_tables(const char* inp_path, double temp, double stacking_mult, int* imax, double* hyb_e,
                             double* hyb_h, double* hyb_s, double* stack, double* init, int cap) {
    if (!inp_path || !imax) return LDO_EINVAL;
    return guard(nullptr, [&]() {
        HostSystem hs = load_system(inp_path, "");
        ldo_host::EnergyInputs in = hs.energy;
        in.temp = temp;
        in.stacking_mult = stacking_mult;
        ldo_host::Tables t = ldo_host::build_tables(hs.sf.identities, hs.sf.sequences, in);
        *imax = t.imax;
        int dim = t.dim;
        if (!hyb_e) return;
        if (dim * dim > cap) throw LdoError(LDO_EINVAL, "table buffer too small");
        for (int a = -t.imax; a <= t.imax; ++a)
            for (int b = -t.imax; b <= t.imax; ++b) {
                size_t k = (size_t)(a + t.imax) * dim + (size_t)(b + t.imax);
                size_t src = t.dense ? k : (a == -b ? (size_t)std::abs(a) : (size_t)t.imax + 1);
                hyb_e[k] = t.e[src];
                if (hyb_h) hyb_h[k] = t.h[src];
                if (hyb_s) hyb_s[k] = t.s[src];
                if (stack) stack[k] = t.stack_dense ? t.stack[k] : t.stack_const;
            }
        if (init) {
            init[0] = t.init_h;
            init[1] = t.init_s;
            init[2] = t.init_e;
        }
    });
}

// ------------------------------------------------ learned proposal ABI ---

ldo_status ldo_learn_collect(ldo_engine* e) {
    if (!e) return LDO_EINVAL;
    return guard(e, [&]() { e->learn_collect(); });
}

ldo_status ldo_learn_reset_counts(ldo_engine* e) {
    if (!e) return LDO_EINVAL;
    return guard(e, [&]() {
        CU(cudaMemsetAsync(e->d_cnt_b.p, 0, LDO_LEARN_TABLE * sizeof(double), e->stream));
        CU(cudaMemsetAsync(e->d_cnt_t.p, 0, LDO_LEARN_TABLE * sizeof(double), e->stream));
    });
}

ldo_status ldo_learn_get_counts(ldo_engine* e, float* cnt_bound, float* cnt_total, int n) {
    if (!e || !cnt_bound || !cnt_total || n != LDO_LEARN_TABLE) return LDO_EINVAL;
    return guard(e, [&]() {
        vector<double> b(n), t(n);
        CU(e->copy(b.data(), e->d_cnt_b.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        CU(e->copy(t.data(), e->d_cnt_t.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        for (int k = 0; k < n; ++k) {
            cnt_bound[k] = (float)b[k];
            cnt_total[k] = (float)t[k];
        }
    });
}

ldo_status ldo_learn_train(ldo_engine* e, int iters, double lr, uint32_t seed, double* loss_first, double* loss_last) {
    if (!e || iters < 0 || !(lr > 0)) return LDO_EINVAL;
    return guard(e, [&]() { e->learn_train(iters, lr, seed, loss_first, loss_last); });
}

ldo_status ldo_learn_set_params(ldo_engine* e, const float* params, int n) {
    if (!e || !params || n != LDO_LEARN_NPARAM) return LDO_EINVAL;
    return guard(e, [&]() {
        e->mlp_ensure(0);
        CU(e->copy(e->mlp.params, params, n * sizeof(float), cudaMemcpyHostToDevice));
        CU(ldo_mlp_sync_weights(e->mlp, e->stream));
        CU(ldo_mlp_table(e->mlp, e->d_learn_w.p, e->stream));
        e->mlp_check();
    });
}

ldo_status ldo_learn_get_params(ldo_engine* e, float* params, int n) {
    if (!e || !params || n != LDO_LEARN_NPARAM) return LDO_EINVAL;
    return guard(e, [&]() {
        e->mlp_ensure(0);
        CU(e->copy(params, e->mlp.params, n * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

ldo_status ldo_learn_get_table(ldo_engine* e, double* weights, int n) {
    if (!e || !weights || n != LDO_LEARN_TABLE) return LDO_EINVAL;
    return guard(e, [&]() { CU(e->copy(weights, e->d_learn_w.p, n * sizeof(double), cudaMemcpyDeviceToHost)); });
}

ldo_status ldo_learn_set_table(ldo_engine* e, const double* weights, int n) {
    if (!e || !weights || n != LDO_LEARN_TABLE) return LDO_EINVAL;
    return guard(e, [&]() { CU(e->copy(e->d_learn_w.p, weights, n * sizeof(double), cudaMemcpyHostToDevice)); });
}

ldo_status ldo_learn_loss_grad(const float* params, const int32_t* idx, const float* cnt_bound, const float* cnt_total,
                             int n, double* loss, float* grad) {
    if (!params || !idx || !cnt_bound || !cnt_total || n <= 0 || !loss || !grad) return LDO_EINVAL;
    return guard(nullptr, [&]() {
        LdoMlp m;
        struct Free {
            LdoMlp& m;
            ~Free() { ldo_mlp_free(m); }
        } hold {m};
        CU(ldo_mlp_alloc(m, n));
        double norm = 0;
        for (int i = 0; i < n; ++i) norm += cnt_total[i];
        CU(cudaMemcpy(m.params, params, LDO_LEARN_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.idx, idx, n * sizeof(int32_t), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.cnt_b, cnt_bound, n * sizeof(float), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.cnt_t, cnt_total, n * sizeof(float), cudaMemcpyHostToDevice));
        CU(ldo_mlp_sync_weights(m, 0));
        CU(ldo_mlp_loss_grad(m, n, norm, 0));
        bool timed_out = false;
        CU(ldo_mlp_check(m, 0, &timed_out));
        if (timed_out) throw LdoError(LDO_ECUDA, "network product: a tensor-core completion wait ran out");
        CU(cudaMemcpy(loss, m.loss, sizeof(double), cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(grad, m.grad, LDO_LEARN_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

} // extern "C"

// ------------------------------------------------------ output writers ---

struct ldo_writer {
    ldo_engine* e {nullptr};
    int replica {0};
    std::unique_ptr<ldo_out::Writer> w;
    vector<int> op_index;
    // .swp writer of one ladder (PTGCMCSimulation::initialize_swap_file /
    // write_swap_entry, src/ptmc_simulation.cpp:91,315)
    int swp_ladder {-1};
    long long swp_freq {0};
    long long swp_read {0};
    std::ofstream swp;
};

namespace {

ldo_out::Snapshot replica_snapshot(ldo_engine* e, int replica, const vector<int>& op_index) {
    LdoLaunch L = e->launch_params(LDO_MODE_OBSERVE, 0);
    L.want_dep = 1;
    CU(e->launch_mc(L));
    CU(cudaStreamSynchronize(e->stream));
    vector<unsigned char> b(e->lay.bytes);
    CU(e->copy(b.data(), e->d_arena.p + (size_t)replica * e->lay.bytes, b.size(), cudaMemcpyDeviceToHost));
    const LdoLayout& y = e->lay;
    const LdoSys& d = e->systems[e->sys_of[replica]].desc;
    const auto* h = reinterpret_cast<const LdoHdr*>(b.data() + y.o_hdr);
    const auto* pp = reinterpret_cast<const long long*>(b.data() + y.o_pp);
    const unsigned char* ore = b.data() + y.o_ore;
    const unsigned char* st = b.data() + y.o_state;
    const auto* chain_c = reinterpret_cast<const int32_t*>(b.data() + y.o_chain_c);
    const unsigned char* chain_type = b.data() + y.o_chain_type;
    const unsigned char* chain_order = b.data() + y.o_chain_order;
    const auto* op = reinterpret_cast<const int32_t*>(b.data() + y.o_op);
    static const int U[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    ldo_out::Snapshot s;
    for (int c = 0; c < h->n_chains; ++c) {
        int cs = chain_order[c];
        int type = cs == 0 ? 0 : chain_type[cs];
        ldo_out::Snapshot::Chain ch;
        ch.index = chain_c[cs];
        ch.identity = type;
        for (int dd = 0; dd < d.type_len[type]; ++dd) {
            int sl = cs == 0 ? dd : d.ns + (cs - 1) * d.lmax + dd;
            long long p = pp[sl];
            int x = (int)(short)(unsigned short)(p & 0xffff);
            long long r1 = (p - x) >> 16;
            int yy = (int)(short)(unsigned short)(r1 & 0xffff);
            int z = (int)((r1 - yy) >> 16);
            ldo_out::Snapshot::Dom dm {{x, yy, z}, {U[ore[sl]][0], U[ore[sl]][1], U[ore[sl]][2]}, st[sl]};
            ch.doms.push_back(dm);
        }
        s.chains.push_back(std::move(ch));
    }
    s.n_types = d.n_types - 1;
    s.num_staples = h->num_staples;
    s.num_bound = h->num_bound;
    s.num_fully = h->num_fully;
    s.energy = h->energy;
    s.enthalpy = h->H;
    s.entropy = h->S;
    s.stacking = h->stacking;
    s.bias = h->move_bias * e->h_ctl[replica].bias_mult;
    for (int q : op_index) s.op_values.push_back(op[2 * q]);
    return s;
}

} // namespace

extern "C" {

ldo_status ldo_writer_open(ldo_engine* e, int replica, const char* filebase, uint32_t kinds, ldo_writer** out) {
    if (!e || !filebase || !out || replica < 0 || replica >= e->n_rep) return LDO_EINVAL;
    *out = nullptr;
    return guard(e, [&]() {
        const HostSystem& hs = e->systems[e->sys_of[replica]];
        auto wr = std::make_unique<ldo_writer>();
        wr->e = e;
        wr->replica = replica;
        vector<string> tags = hs.p.ops_to_output;
        if (tags.empty())
            for (auto& o : hs.ops) tags.push_back(o.tag);
        for (auto& t : tags) {
            int q = -1;
            for (size_t k = 0; k < hs.ops.size(); ++k)
                if (hs.ops[k].tag == t) q = (int)k;
            if (q < 0) throw LdoError(LDO_EINVAL, t + ": no such order parameter to output");
            wr->op_index.push_back(q);
        }
        try {
            wr->w = std::make_unique<ldo_out::Writer>(filebase, kinds, hs.desc.ns, hs.p.max_total_staples,
                                                      hs.p.max_staple_size, tags);
        } catch (std::runtime_error& x) {
            throw LdoError(LDO_EINVAL, x.what());
        }
        *out = wr.release();
    });
}

// .swp of one ladder: the header of PTGCMCSimulation::initialize_swap_file
// (the exchanged controls of every slot, "v1/v2/ " per slot), then the rows
// that pt runs record.
ldo_status ldo_swap_writer_open(ldo_engine* e, int n_rungs, int exchange_q, int ladder, const char* filebase,
                                int64_t freq, ldo_writer** out) {
    if (!e || !filebase || !out || n_rungs < 2 || freq <= 0) return LDO_EINVAL;
    *out = nullptr;
    return guard(e, [&]() {
        if (n_rungs != e->pt_rungs || exchange_q != e->pt_q || e->pt_dim2 != 0) {
            if (e->pt_graph) {
                cudaGraphExecDestroy(e->pt_graph);
                e->pt_graph = nullptr;
            }
            e->pt_setup(n_rungs, exchange_q, 0);
        }
        int nl = e->n_rep / n_rungs;
        if (ladder < 0 || ladder >= nl) throw LdoError(LDO_EINVAL, "ladder out of range");
        if (e->hist_cap == 0) e->pt_record_swaps(4096);
        auto wr = std::make_unique<ldo_writer>();
        wr->e = e;
        wr->swp_ladder = ladder;
        wr->swp_freq = freq;
        long long n = 0;
        CU(e->copy(&n, e->d_hist_n.p + ladder, sizeof(long long), cudaMemcpyDeviceToHost));
        wr->swp_read = n;
        string name = string(filebase) + ".swp";
        wr->swp.open(name);
        if (!wr->swp.good()) throw LdoError(LDO_EINVAL, name + ": output path does not exist");
        for (int rep = 0; rep < n_rungs; ++rep) {
            for (int q = 0; q < 4; ++q)
                if (exchange_q & (1 << q)) wr->swp << e->pt_slot_q[(size_t)q * n_rungs + rep] << "/";
            wr->swp << " ";
        }
        wr->swp << "\n";
        wr->swp.flush();
        *out = wr.release();
    });
}

namespace {
// write_swap_entry rows: the rows recorded since the last call whose step is
// a multiple of the frequency, then (step >= 0) the current permutation as
// the end-of-run row at `step`.
void swap_writer_write(ldo_writer* w, int64_t step) {
    ldo_engine* e = w->e;
    int R = e->pt_rungs, nl = e->n_rep / R, lad = w->swp_ladder;
    if (e->hist_cap == 0) throw LdoError(LDO_EINVAL, "the swap history was dropped (the ladder was set up again)");
    long long n = 0;
    CU(e->copy(&n, e->d_hist_n.p + lad, sizeof(long long), cudaMemcpyDeviceToHost));
    if (n - w->swp_read > e->hist_cap)
        throw LdoError(LDO_EINVAL, "swap history overflow: write the .swp file at least every 4096 exchanges");
    vector<int> row(R);
    for (long long k = w->swp_read; k < n; ++k) {
        size_t r = (size_t)(k % e->hist_cap) * nl + lad;
        long long st = 0;
        CU(e->copy(&st, e->d_hist_step.p + r, sizeof(long long), cudaMemcpyDeviceToHost));
        if (st % w->swp_freq != 0) continue;
        CU(e->copy(row.data(), e->d_hist_perm.p + r * R, R * sizeof(int), cudaMemcpyDeviceToHost));
        for (int q = 0; q < R; ++q) w->swp << row[q] - lad * R << " ";
        w->swp << "\n";
    }
    w->swp_read = n;
    if (step >= 0 && step % w->swp_freq == 0) {
        CU(e->copy(row.data(), e->d_perm.p + (size_t)lad * R, R * sizeof(int), cudaMemcpyDeviceToHost));
        for (int q = 0; q < R; ++q) w->swp << row[q] - lad * R << " ";
        w->swp << "\n";
    }
    w->swp.flush();
}
} // namespace

ldo_status ldo_writer_write(ldo_writer* w, int64_t step) {
    if (!w || !w->e) return LDO_EINVAL;
    if (w->swp_ladder >= 0) return guard(w->e, [&]() { swap_writer_write(w, step); });
    return guard(w->e, [&]() { w->w->write(step, replica_snapshot(w->e, w->replica, w->op_index)); });
}

void ldo_writer_close(ldo_writer* w) { delete w; }

} // extern "C"

// ------------------------------------------------------------ batches ---
// A batch of replicas over systems of different sizes, split by capacity
// class: one engine per class, each with its own state layout, kernel
// instantiation and launch shape, launched together (their streams fork
// from and join into the batch's stream).  Replica r keeps the Philox
// stream key r of the whole batch, so every trajectory equals that of one
// engine holding all the replicas in the largest class.
struct ldo_batch {
    string err;
    int n_rep {0};
    vector<ldo_engine*> groups;
    vector<int> cls;
    vector<vector<int>> reps;          // batch indices of each group's replicas
    vector<int> group_of, local_of;    // per batch replica
    cudaStream_t stream {nullptr};
    cudaEvent_t ev0 {nullptr}, ev1 {nullptr};
    vector<cudaEvent_t> done;

    ~ldo_batch() {
        for (auto ev : done) cudaEventDestroy(ev);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
        for (auto* g : groups) delete g;
    }

    void create(const vector<string>& inps, const string& overrides, const vector<int>& sys_of, uint32_t seed) {
        n_rep = (int)sys_of.size();
        if (n_rep <= 0) throw LdoError(LDO_EINVAL, "need at least one replica");
        vector<int> sys_cls(inps.size());
        for (size_t i = 0; i < inps.size(); ++i) {
            HostSystem hs = load_system(inps[i], overrides);
            sys_cls[i] = make_layout(hs.desc.dcap, hs.desc.kmax, hs.desc.n_types, hs.desc.n_biases, hs.desc.n_ops,
                                     hs.desc.n_moves).cls;
        }
        for (int r = 0; r < n_rep; ++r)
            if (sys_of[r] < 0 || sys_of[r] >= (int)inps.size())
                throw LdoError(LDO_EINVAL, "sys_of_replica out of range");
        group_of.assign(n_rep, -1);
        local_of.assign(n_rep, -1);
        CU(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CU(cudaEventCreate(&ev0));
        CU(cudaEventCreate(&ev1));
        for (int c = LDO_CLASS_S; c <= LDO_CLASS_L; ++c) {
            vector<int> sys_map(inps.size(), -1), so, rr;
            vector<string> sub;
            vector<uint32_t> ids;
            for (int r = 0; r < n_rep; ++r) {
                int s = sys_of[r];
                if (sys_cls[s] != c) continue;
                if (sys_map[s] < 0) {
                    sys_map[s] = (int)sub.size();
                    sub.push_back(inps[s]);
                }
                group_of[r] = (int)groups.size();
                local_of[r] = (int)rr.size();
                so.push_back(sys_map[s]);
                ids.push_back((uint32_t)r);
                rr.push_back(r);
            }
            if (rr.empty()) continue;
            auto* e = new ldo_engine;
            groups.push_back(e);
            e->rep_ids = ids;
            e->create(sub, overrides, so, seed);
            if (e->lay.cls != c) throw LdoError(LDO_EINVAL, "batch: a group's layout class differs from its systems'");
            cls.push_back(c);
            reps.push_back(rr);
            cudaEvent_t ev;
            CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            done.push_back(ev);
        }
    }

    // One MC launch per group on the group's stream, all forked from and
    // joined into the batch's stream; device_ms spans the whole fork/join.
    void run(long long steps, int sweeps, double* ms) {
        CU(cudaEventRecord(ev0, stream));
        for (size_t g = 0; g < groups.size(); ++g) {
            ldo_engine& e = *groups[g];
            CU(cudaStreamWaitEvent(e.stream, ev0, 0));
            LdoLaunch L = e.launch_params(LDO_MODE_RUN, steps);
            L.sweep_units = sweeps;
            CU(e.launch_mc(L));
            CU(cudaEventRecord(done[g], e.stream));
            CU(cudaStreamWaitEvent(stream, done[g], 0));
        }
        CU(cudaEventRecord(ev1, stream));
        CU(cudaStreamSynchronize(stream));
        if (ms) {
            float f = 0;
            CU(cudaEventElapsedTime(&f, ev0, ev1));
            *ms = f;
        }
        for (auto* g : groups) g->check_status();
    }
};

namespace {

ldo_status bguard(ldo_batch* b, const std::function<void()>& f) {
    try {
        f();
        if (b) b->err.clear();
        return LDO_OK;
    } catch (LdoError& x) {
        if (b) b->err = x.what();
        else g_create_err = x.what();
        return x.code;
    } catch (std::exception& x) {
        if (b) b->err = x.what();
        else g_create_err = x.what();
        return LDO_EINVAL;
    }
}

// a group engine's call inside a batch call: its error becomes the batch's
void group_ok(ldo_engine* e, ldo_status st) {
    if (st != LDO_OK) throw LdoError(st, e->err);
}

} // namespace

extern "C" {

ldo_status ldo_batch_create(const char* const* inp_paths, int n_systems, const char* overrides,
                            const int* sys_of_replica, int n_replicas, uint32_t seed, ldo_batch** out) {
    if (!out || !inp_paths || n_systems <= 0 || n_replicas <= 0) {
        g_create_err = "invalid arguments";
        return LDO_EINVAL;
    }
    *out = nullptr;
    auto* b = new ldo_batch;
    vector<string> inps;
    for (int i = 0; i < n_systems; ++i) inps.push_back(inp_paths[i]);
    vector<int> so(n_replicas, 0);
    if (sys_of_replica)
        for (int r = 0; r < n_replicas; ++r) so[r] = sys_of_replica[r];
    ldo_status st = bguard(nullptr, [&]() { b->create(inps, overrides ? overrides : "", so, seed); });
    if (st != LDO_OK) {
        delete b;
        return st;
    }
    *out = b;
    return LDO_OK;
}

void ldo_batch_destroy(ldo_batch* b) { delete b; }

const char* ldo_batch_last_error(const ldo_batch* b) { return b ? b->err.c_str() : g_create_err.c_str(); }

int ldo_batch_num_groups(const ldo_batch* b) { return b ? (int)b->groups.size() : 0; }

ldo_status ldo_batch_group(ldo_batch* b, int g, int* cls, int* n_rep, int32_t* replicas, ldo_engine** engine) {
    if (!b || g < 0 || g >= (int)b->groups.size()) return LDO_EINVAL;
    if (cls) *cls = b->cls[g];
    if (n_rep) *n_rep = (int)b->reps[g].size();
    if (replicas)
        for (size_t k = 0; k < b->reps[g].size(); ++k) replicas[k] = b->reps[g][k];
    if (engine) *engine = b->groups[g];
    return LDO_OK;
}

ldo_status ldo_batch_set_controls(ldo_batch* b, const double* temps, const double* stacking_mults,
                                  const double* staple_u_mults, int n) {
    if (!b || n != b->n_rep) return LDO_EINVAL;
    return bguard(b, [&]() {
        for (size_t g = 0; g < b->groups.size(); ++g) {
            const auto& rr = b->reps[g];
            vector<double> t(rr.size()), s(rr.size()), u(rr.size());
            for (size_t k = 0; k < rr.size(); ++k) {
                if (temps) t[k] = temps[rr[k]];
                if (stacking_mults) s[k] = stacking_mults[rr[k]];
                if (staple_u_mults) u[k] = staple_u_mults[rr[k]];
            }
            group_ok(b->groups[g], ldo_set_controls(b->groups[g], temps ? t.data() : nullptr,
                                                    stacking_mults ? s.data() : nullptr,
                                                    staple_u_mults ? u.data() : nullptr, (int)rr.size()));
        }
    });
}

ldo_status ldo_batch_run(ldo_batch* b, int64_t n_steps, double* device_ms) {
    if (!b || n_steps < 0) return LDO_EINVAL;
    return bguard(b, [&]() { b->run(n_steps, 0, device_ms); });
}

ldo_status ldo_batch_run_sweeps(ldo_batch* b, int64_t n_sweeps, double* device_ms) {
    if (!b || n_sweeps < 0) return LDO_EINVAL;
    return bguard(b, [&]() { b->run(n_sweeps, 1, device_ms); });
}

ldo_status ldo_batch_set_sampling(ldo_batch* b, int interval, int capacity) {
    if (!b || interval < 0 || capacity < 0) return LDO_EINVAL;
    return bguard(b, [&]() {
        for (auto* g : b->groups) group_ok(g, ldo_set_sampling(g, interval, capacity));
    });
}

ldo_status ldo_batch_get_samples(ldo_batch* b, int16_t* out, int capacity, int* count) {
    if (!b || !out) return LDO_EINVAL;
    return bguard(b, [&]() {
        for (size_t g = 0; g < b->groups.size(); ++g) {
            const auto& rr = b->reps[g];
            vector<int16_t> part(rr.size() * (size_t)capacity * 2);
            vector<int> cnt(rr.size());
            group_ok(b->groups[g], ldo_get_samples(b->groups[g], part.data(), capacity, cnt.data()));
            for (size_t k = 0; k < rr.size(); ++k) {
                std::memcpy(out + (size_t)rr[k] * capacity * 2, part.data() + k * (size_t)capacity * 2,
                            (size_t)capacity * 2 * sizeof(int16_t));
                if (count) count[rr[k]] = cnt[k];
            }
        }
    });
}

ldo_status ldo_batch_autotune(ldo_batch* b, int32_t probe_sweeps, int32_t use_cache, ldo_tune_report* out, int n) {
    if (!b || probe_sweeps < 1 || !out || n < (int)b->groups.size()) return LDO_EINVAL;
    return bguard(b, [&]() {
        for (size_t g = 0; g < b->groups.size(); ++g)
            group_ok(b->groups[g], ldo_autotune(b->groups[g], probe_sweeps, use_cache, out + g));
    });
}

ldo_status ldo_batch_get_counters(ldo_batch* b, int64_t* launches, int64_t* h2d_bytes, int64_t* d2h_bytes) {
    if (!b) return LDO_EINVAL;
    int64_t l = 0, h = 0, d = 0;
    for (auto* g : b->groups) {
        l += g->n_launches;
        h += g->bytes_h2d;
        d += g->bytes_d2h;
    }
    if (launches) *launches = l;
    if (h2d_bytes) *h2d_bytes = h;
    if (d2h_bytes) *d2h_bytes = d;
    return LDO_OK;
}

} // extern "C"
