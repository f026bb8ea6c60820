// Exchange driver for the reference build.  Test infrastructure only: it
// records golden vectors for the parallel-tempering and umbrella-sampling
// restatements in tests/.
//
// The reference's own exchange code (src/ptmc_simulation.cpp,
// src/us_simulation.cpp) is compiled from its sources with the single-process
// MPI stand-in of stubs/boost/mpi.  This process is the master rank: it posts
// the messages the other ranks would have sent, calls the reference's member
// functions, and collects what the master sends back.  Random numbers come
// from the Philox replacement of src/random_gens.cpp, keyed as the engine keys
// its exchange streams, so the reference's acceptance draws are the engine's.
//
// Usage: ref_exchange <params>, a key=value file as for ref_trace plus
//   exchange_mode = pt | us_update | us_exchange
// Commands are read from standard input, one per line.  Answers are written
// to standard output on lines that start with "@@ " (the reference itself
// prints progress messages there too).
//
// pt (PTGCMCSimulation and its variants): pt_variant = T | UT | HUT | ST | 2D,
// temps, chem_pot_mults, bias_mults, stacking_mults (space-separated lists),
// num_reps, staple_u_mult; the swap stream is (trace_seed, trace_replica,
// stream 1).
//   redu -> "@@ redu <m_reduced_staple_us>" (origami_system.cpp:57)
//   acc t1 t2 sm1 sm2 H1 H2 b1 b2 st1 st2 u1[S] u2[S] N1[S] N2[S]
//       -> "@@ p <p>": PTGCMCSimulation::calc_acceptance_p (:275) on these
//          quantities (each per-type vector is passed with one trailing zero,
//          so that its loop over identities.size() entries reads no memory
//          past the S staple types)
//   round <swap_i>, then num_reps lines "H bias stacking N_1 .. N_S" for ranks
//       0 .. R-1 -> update_control_qs of the master (:595-680), then
//          attempt_exchange (OneD :360, TwoD :495) with master_receive /
//          master_send; "@@ perm <q_to_repi> draws <n> ctl <T u b s per rank>"
//   counts -> "@@ att <..> acc <..>" (attempt and swap counts, row-major)
//
// us_update (USGCMCSimulation / SimpleUSGCMCSimulation): num_windows W
// independent window simulations, us_grid_bias_tag, max_D_bias.
//   iter <n>, then W lines "k x_1 c_1 .. x_k c_k" (visit counts of a 1-D grid
//       order parameter) -> process_iteration(n) (:160: fill_grid_sets,
//       estimate_current_weights :286, update_grids, update_bias :385) of each
//       window; "@@ E <w> <k> x_1 E_1 .. x_k E_k" per window
//
// us_exchange (PTMWUSGCMCSimulation): windows_file, the master of num_windows
// windows; the exchange stream is (trace_seed, 0, stream 2).
//   point0 -> "@@ point0 <x>": the grid point of window 0, the master's own
//       configuration (it never changes: a configuration the master receives
//       in an exchange is its own, sent back)
//   round <swap_i>, then W lines "x k y_1 E_1 .. y_k E_k" (grid point and
//       grid biases of windows 0 .. W-1) -> attempt_exchange (:770);
//       "@@ w2w <win_to_win> configi <win_to_configi> draws <n>"
//   counts -> "@@ att <..> acc <..>"
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "LatticeDNAOrigami/ptmc_simulation.hpp"
#include "LatticeDNAOrigami/us_simulation.hpp"

#include "ref_params.h"

extern "C" void ldo_ref_rng_configure(uint32_t seed, uint32_t replica, uint32_t stream);
extern "C" uint64_t ldo_ref_rng_draws();

char const* const GIT_COMMIT = "oracle-build";

using std::pair;
using std::string;
using std::vector;

namespace {

// Access to the reference's protected and private members without changing
// its sources: an explicit template instantiation may name any member, and
// the friend function it defines hands out the member pointer.
template <class Tag, typename Tag::type M>
struct Grant {
    friend typename Tag::type member(Tag) { return M; }
};
#define LDO_GRANT(NAME, TYPE, MEMBER)        \
    struct NAME {                            \
        using type = TYPE;                   \
        friend type member(NAME);            \
    };                                       \
    template struct Grant<NAME, &MEMBER>;

using PT = ptmc::PTGCMCSimulation;
using OneD = ptmc::OneDPTGCMCSimulation;
using TwoD = ptmc::TwoDPTGCMCSimulation;
using PairVec = vector<pair<double, double>>;
using PerStaple = vector<pair<vector<double>, vector<double>>>;
LDO_GRANT(PtQToRep, vector<int> PT::*, PT::m_q_to_repi)
LDO_GRANT(PtCtl, vector<double> PT::*, PT::m_replica_control_qs)
LDO_GRANT(PtDep, vector<double> PT::*, PT::m_replica_dependent_qs)
LDO_GRANT(PtExQ, vector<int> PT::*, PT::m_exchange_q_is)
LDO_GRANT(PtUpdateCtl, void (PT::*)(), PT::update_control_qs)
LDO_GRANT(PtAttempt, void (PT::*)(int), PT::attempt_exchange)
LDO_GRANT(PtAccP, double (PT::*)(PairVec, PairVec, PerStaple), PT::calc_acceptance_p)
LDO_GRANT(OneAtt, vector<int> OneD::*, OneD::m_attempt_count)
LDO_GRANT(OneAcc, vector<int> OneD::*, OneD::m_swap_count)
LDO_GRANT(TwoAtt, vector<vector<vector<int>>> TwoD::*, TwoD::m_attempt_count)
LDO_GRANT(TwoAcc, vector<vector<vector<int>>> TwoD::*, TwoD::m_swap_count)

using US = us::USGCMCSimulation;
using MWUS = us::MWUSGCMCSimulation;
using PTMWUS = us::PTMWUSGCMCSimulation;
LDO_GRANT(UsSi, us::SetOfGridPoints US::*, US::m_s_i)
LDO_GRANT(UsFi, us::GridInts US::*, US::m_f_i)
LDO_GRANT(UsBase, string US::*, US::m_output_filebase)
LDO_GRANT(SimLog, std::ostream* simulation::GCMCSimulation::*, simulation::GCMCSimulation::m_logging_stream)
LDO_GRANT(MwSim, US* MWUS::*, MWUS::m_us_sim)
LDO_GRANT(MwAttempt, void (PTMWUS::*)(int), PTMWUS::attempt_exchange)
LDO_GRANT(MwConfigi, vector<int> PTMWUS::*, PTMWUS::m_win_to_configi)
LDO_GRANT(MwAtt, vector<int> PTMWUS::*, PTMWUS::m_attempt_count)
LDO_GRANT(MwAcc, vector<int> PTMWUS::*, PTMWUS::m_swap_count)

vector<double> doubles(const string& s) {
    vector<double> v;
    std::istringstream is(s);
    double x;
    while (is >> x) v.push_back(x);
    return v;
}

void answer(const string& s) { std::cout << "@@ " << s << std::endl; }

string fmt(double x) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", x);
    return b;
}

template <class V> string join(const V& v) {
    std::ostringstream os;
    for (size_t i = 0; i < v.size(); ++i) os << (i ? " " : "") << v[i];
    return os.str();
}

// ------------------------------------------------------------------ PT ---

// The master's own staple counts (get_staple_counts counts its chains): the
// system files used here hold the scaffold only, so the counts are made by
// adding unplaced staple chains, which are deleted again before the next
// update_control_qs (its energy update places every chain of the system).
struct MasterStaples {
    vector<int> added;
    void clear(origami::OrigamiSystem& o) {
        for (int c : added) o.delete_chain(c);
        added.clear();
    }
    void set(origami::OrigamiSystem& o, const vector<int>& want) {
        vector<int> have = o.get_staple_counts();
        for (size_t t = 0; t < want.size(); ++t) {
            if (want[t] < have[t]) throw std::runtime_error("round: fewer staples than the master's system holds");
            for (int k = have[t]; k < want[t]; ++k) added.push_back(o.add_chain((int)t + 1));
        }
    }
};

int run_pt(origami::OrigamiSystem& o, parser::InputParameters& p, std::map<string, string>& kv) {
    string variant = kv.count("pt_variant") ? kv["pt_variant"] : string("T");
    PT* sim = nullptr;
    auto& ops = o.get_system_order_params();
    auto& biases = o.get_system_biases();
    if (variant == "T") sim = new ptmc::TPTGCMCSimulation(o, ops, biases, p);
    else if (variant == "UT") sim = new ptmc::UTPTGCMCSimulation(o, ops, biases, p);
    else if (variant == "HUT") sim = new ptmc::HUTPTGCMCSimulation(o, ops, biases, p);
    else if (variant == "ST") sim = new ptmc::STPTGCMCSimulation(o, ops, biases, p);
    else if (variant == "2D") sim = new ptmc::TwoDPTGCMCSimulation(o, ops, biases, p);
    else throw std::runtime_error("unknown pt_variant " + variant);
    bool two_d = variant == "2D";
    uint32_t seed = kv.count("trace_seed") ? (uint32_t)std::stoul(kv["trace_seed"]) : 0u;
    uint32_t ladder = kv.count("trace_replica") ? (uint32_t)std::stoul(kv["trace_replica"]) : 0u;
    ldo_ref_rng_configure(seed, ladder, 1);
    int R = p.m_num_reps;
    int S = (int)o.m_identities.size() - 1;
    // control quantities of every rank as its initialize_control_qs sets
    // them.  Both versions (1-D :375-392, 2-D :428-470) store the rank's bias
    // multiplier at index m_bias_i = 1, a dependent-quantity index, which is
    // the staple-u slot of the control vector: until its first exchange a
    // rank's staple u multiplier is its bias multiplier (bias_mults[r]; 1 in
    // 2-D) and its bias multiplier stays 0.
    vector<vector<double>> ctl(R, vector<double>(4));
    for (int r = 0; r < R; ++r) {
        if (two_d) {
            int d2 = (int)p.m_stacking_mults.size();
            ctl[r] = {p.m_temps[r / d2], 1.0, 0.0, p.m_stacking_mults[r % d2]};
        }
        else {
            ctl[r] = {p.m_temps[r], p.m_bias_mults[r], 0.0, p.m_stacking_mults[r]};
        }
    }
    if ((sim->*member(PtCtl {})) != ctl[0]) throw std::runtime_error("the master's controls are not the expected ones");
    auto& mb = boost::mpi::Mailbox::get();
    MasterStaples staples;
    string line;
    while (std::getline(std::cin, line)) {
        std::istringstream is(line);
        string cmd;
        is >> cmd;
        if (cmd == "quit") break;
        if (cmd == "redu") {
            std::ostringstream os;
            os << "redu";
            for (double u : o.m_reduced_staple_us) os << " " << fmt(u);
            answer(os.str());
        }
        else if (cmd == "acc") {
            vector<double> v = doubles(line.substr(3));
            if ((int)v.size() != 10 + 4 * S) throw std::runtime_error("acc: wrong number of values");
            PairVec cq = {{v[0], v[1]}, {1.0, 1.0}, {1.0, 1.0}, {v[2], v[3]}};
            PairVec dq = {{v[4], v[5]}, {v[6], v[7]}, {v[8], v[9]}};
            vector<double> u1(v.begin() + 10, v.begin() + 10 + S), u2(v.begin() + 10 + S, v.begin() + 10 + 2 * S);
            vector<double> n1(v.begin() + 10 + 2 * S, v.begin() + 10 + 3 * S);
            vector<double> n2(v.begin() + 10 + 3 * S, v.begin() + 10 + 4 * S);
            for (auto* x : {&u1, &u2, &n1, &n2}) x->push_back(0.0);
            PerStaple ps = {{u1, u2}, {n1, n2}};
            double pa = (sim->*member(PtAccP {}))(cq, dq, ps);
            answer("p " + fmt(pa));
        }
        else if (cmd == "round") {
            int swap_i;
            is >> swap_i;
            vector<vector<double>> dep(R);
            for (int r = 0; r < R; ++r) {
                std::getline(std::cin, line);
                dep[r] = doubles(line);
                if ((int)dep[r].size() != 3 + S) throw std::runtime_error("round: wrong number of values");
            }
            // the master's own part: its controls into its system, its
            // dependent quantities and staple counts
            staples.clear(o);
            (sim->*member(PtUpdateCtl {}))();
            (sim->*member(PtDep {})) = {dep[0][0], dep[0][1], dep[0][2], 0.0};
            vector<int> n0;
            for (int t = 0; t < S; ++t) n0.push_back((int)dep[0][3 + t]);
            staples.set(o, n0);
            // slave_send of every other rank (:163): four dependent
            // quantities, its staple chemical potentials (update_staple_us of
            // its controls, origami_system.cpp:624), its staple counts
            for (int r = 1; r < R; ++r) {
                for (int q = 0; q < 3; ++q) mb.post(r, 0, swap_i, dep[r][q]);
                mb.post(r, 0, swap_i, 0.0);
                for (int t = 0; t < S; ++t) mb.post(r, 0, swap_i, o.m_reduced_staple_us[t] * ctl[r][0] * ctl[r][1]);
                for (int t = 0; t < S; ++t) mb.post(r, 0, swap_i, dep[r][3 + t]);
            }
            (sim->*member(PtAttempt {}))(swap_i);
            // slave_receive of every other rank (:177)
            const vector<int>& exq = sim->*member(PtExQ {});
            for (int r = 1; r < R; ++r)
                for (int q : exq)
                    if (!mb.take(0, r, swap_i, ctl[r][q])) throw std::runtime_error("round: no controls for a rank");
            ctl[0] = sim->*member(PtCtl {});
            std::ostringstream os;
            os << "perm " << join(sim->*member(PtQToRep {})) << " draws " << ldo_ref_rng_draws() << " ctl";
            for (int r = 0; r < R; ++r)
                for (int q = 0; q < 4; ++q) os << " " << fmt(ctl[r][q]);
            answer(os.str());
        }
        else if (cmd == "counts") {
            vector<int> att, acc;
            if (two_d) {
                for (auto& a : static_cast<TwoD*>(sim)->*member(TwoAtt {}))
                    for (auto& b : a) att.insert(att.end(), b.begin(), b.end());
                for (auto& a : static_cast<TwoD*>(sim)->*member(TwoAcc {}))
                    for (auto& b : a) acc.insert(acc.end(), b.begin(), b.end());
            }
            else {
                att = static_cast<OneD*>(sim)->*member(OneAtt {});
                acc = static_cast<OneD*>(sim)->*member(OneAcc {});
            }
            answer("att " + join(att) + " acc " + join(acc));
        }
        else if (!cmd.empty()) throw std::runtime_error("unknown command " + cmd);
    }
    return 0;
}

// ------------------------------------------------------------------ US ---

int run_us_update(parser::InputParameters& p, std::map<string, string>& kv) {
    int W = kv.count("num_windows") ? std::stoi(kv["num_windows"]) : 1;
    vector<origami::OrigamiSystem*> sys;
    vector<US*> sims;
    vector<parser::InputParameters> ps(W, p);
    std::ostringstream sink;
    for (int w = 0; w < W; ++w) {
        ps[w].m_output_filebase = p.m_output_filebase + "_win" + std::to_string(w);
        sys.push_back(origami::setup_origami(ps[w]));
        sims.push_back(new us::SimpleUSGCMCSimulation(*sys[w], sys[w]->get_system_order_params(),
                                                       sys[w]->get_system_biases(), ps[w]));
        sims[w]->set_output_stream(&sink);
        sims[w]->*member(UsBase {}) = ps[w].m_output_filebase;
    }
    string line;
    while (std::getline(std::cin, line)) {
        std::istringstream is(line);
        string cmd;
        is >> cmd;
        if (cmd == "quit") break;
        if (cmd != "iter") {
            if (!cmd.empty()) throw std::runtime_error("unknown command " + cmd);
            continue;
        }
        int n;
        is >> n;
        for (int w = 0; w < W; ++w) {
            std::getline(std::cin, line);
            vector<double> v = doubles(line);
            US* s = sims[w];
            auto& si = s->*member(UsSi {});
            auto& fi = s->*member(UsFi {});
            long long total = 0;
            int k = (int)v.at(0);
            // what update_internal (:262) leaves after the iteration's steps
            for (int j = 0; j < k; ++j) {
                us::GridPoint pt {(int)v.at(1 + 2 * j)};
                long long c = (long long)v.at(2 + 2 * j);
                si.insert(pt);
                fi[pt] += c;
                total += c;
            }
            s->m_steps = total;
            s->*member(SimLog {}) = new std::ostringstream;   // process_iteration deletes it
            s->process_iteration(n);
        }
        for (int w = 0; w < W; ++w) {
            std::map<int, double> e;
            for (auto& kv2 : sims[w]->m_E_w) e[kv2.first.at(0)] = kv2.second;
            std::ostringstream os;
            os << "E " << w << " " << e.size();
            for (auto& x : e) os << " " << x.first << " " << fmt(x.second);
            answer(os.str());
        }
    }
    return 0;
}

int run_us_exchange(origami::OrigamiSystem& o, parser::InputParameters& p, std::map<string, string>& kv) {
    auto& mb = boost::mpi::Mailbox::get();
    PTMWUS sim(o, o.get_system_order_params(), o.get_system_biases(), p);
    US* us_sim = sim.*member(MwSim {});
    uint32_t seed = kv.count("trace_seed") ? (uint32_t)std::stoul(kv["trace_seed"]) : 0u;
    ldo_ref_rng_configure(seed, 0, 2);
    int W = mb.size;
    // a configuration the master would receive in an exchange is its own
    origami::Chains own = sim.get_chains();
    mb.on_empty = [&](int src, int dst, int tag) { mb.post(src, dst, tag, own); };
    string line;
    while (std::getline(std::cin, line)) {
        std::istringstream is(line);
        string cmd;
        is >> cmd;
        if (cmd == "quit") break;
        if (cmd == "point0") {
            answer("point0 " + std::to_string(us_sim->get_current_point().at(0)));
        }
        else if (cmd == "round") {
            int swap_i;
            is >> swap_i;
            for (int w = 0; w < W; ++w) {
                std::getline(std::cin, line);
                vector<double> v = doubles(line);
                us::GridPoint pt {(int)v.at(0)};
                us::GridFloats E;
                int k = (int)v.at(1);
                for (int j = 0; j < k; ++j) E[us::GridPoint {(int)v.at(2 + 2 * j)}] = v.at(3 + 2 * j);
                if (w == 0) {
                    if (pt != us_sim->get_current_point()) throw std::runtime_error("round: window 0 point differs");
                    us_sim->m_E_w = E;
                }
                else {
                    mb.post(w, 0, swap_i, pt);   // slave_send_ops (:709)
                    mb.post(w, 0, swap_i, E);
                }
            }
            (sim.*member(MwAttempt {}))(swap_i);
            vector<int> w2w(W, 0);
            for (int w = 1; w < W; ++w)
                if (!mb.take(0, w, swap_i, w2w[w])) throw std::runtime_error("round: no window for a rank");
            for (int w = 1; w < W; ++w) {
                origami::Chains c;
                mb.take(0, w, swap_i, c);   // the master's configuration, if it was exchanged
            }
            w2w[0] = 0;
            for (int w = 1; w < W; ++w)
                if (w2w[w] == 0) w2w[0] = w;
            answer("w2w " + join(w2w) + " configi " + join(sim.*member(MwConfigi {})) + " draws " +
                   std::to_string(ldo_ref_rng_draws()));
        }
        else if (cmd == "counts") {
            answer("att " + join(sim.*member(MwAtt {})) + " acc " + join(sim.*member(MwAcc {})));
        }
        else if (!cmd.empty()) throw std::runtime_error("unknown command " + cmd);
    }
    return 0;
}

} // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: ref_exchange <params>\n";
        return 2;
    }
    auto kv = ldo_refdrv::read_kv(argv[1]);
    parser::InputParameters params;
    ldo_refdrv::fill_params(params, kv);
    auto list = [&](const char* k) { return kv.count(k) ? doubles(kv[k]) : vector<double> {}; };
    params.m_temps = list("temps");
    params.m_chem_pot_mults = list("chem_pot_mults");
    params.m_bias_mults = list("bias_mults");
    params.m_stacking_mults = list("stacking_mults");
    params.m_num_reps = kv.count("num_reps") ? std::stoi(kv["num_reps"]) : (int)params.m_temps.size();
    params.m_swaps = 0;
    params.m_configs_output_freq = 1;
    params.m_us_grid_bias_tag = kv.count("us_grid_bias_tag") ? kv["us_grid_bias_tag"] : string();
    params.m_max_D_bias = kv.count("max_D_bias") ? std::stod(kv["max_D_bias"]) : 0.0;
    params.m_windows_file = kv.count("windows_file") ? kv["windows_file"] : string();
    params.m_iter_swaps = 0;
    string mode = kv.count("exchange_mode") ? kv["exchange_mode"] : string("pt");
    auto& mb = boost::mpi::Mailbox::get();
    mb.rank = 0;
    mb.size = mode == "us_exchange" ? (kv.count("num_windows") ? std::stoi(kv["num_windows"]) : 1)
                                    : params.m_num_reps;
    try {
        if (mode == "us_update") return run_us_update(params, kv);
        origami::OrigamiSystem* o = origami::setup_origami(params);
        if (mode == "pt") return run_pt(*o, params, kv);
        if (mode == "us_exchange") return run_us_exchange(*o, params, kv);
        throw std::runtime_error("unknown exchange_mode " + mode);
    } catch (std::exception& e) {
        std::cout << "@@ error " << e.what() << std::endl;
        return 3;
    }
}
