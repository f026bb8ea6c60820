// Oracle (test infrastructure only): C entry points over the CPU restatement
// in oracle_system.hpp, loaded by tests/ and bench.py through ctypes.  The
// engine never links or calls anything in this directory.
#include <atomic>
#include <chrono>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../latticednaorigami_gb300/csrc/ldo_io.hpp"
#include "oracle_system.hpp"

using namespace oracle;

namespace {

thread_local std::string g_err;

struct Replica {
    ldo_io::Params params;
    ldo_io::SystemFile sf;
    EnergyModel model;
    System sys;
    std::vector<double> learn_w;   // learned-proposal weight table (engine's)
};

int move_kind(const std::string& t) {
    if (t == "OrientationRotation") return MV_ORIENTATION;
    if (t == "MetStapleExchange") return MV_MET_EXCHANGE;
    if (t == "MetStapleRegrowth") return MV_MET_REGROWTH;
    if (t == "CBStapleRegrowth") return MV_CB_REGROWTH;
    if (t == "LearnedStapleExchange") return MV_LEARNED_EXCHANGE;
    if (t == "LearnedStapleRegrowth") return MV_LEARNED_REGROWTH;
    if (t == "CTRGScaffoldRegrowth") return MV_CTRG_SCAFFOLD;
    if (t == "CTRGJumpScaffoldRegrowth") return MV_CTRG_JUMP;
    if (t == "CTCBScaffoldRegrowth") return MV_CTCB_SCAFFOLD;
    if (t == "CTCBJumpScaffoldRegrowth") return MV_CTCB_JUMP;
    if (t == "CTCBLinkerRegrowth") return MV_CTCB_LINKER;
    if (t == "CTCBClusteredLinkerRegrowth") return MV_CTCB_CLINKER;
    if (t == "CTRGLinkerRegrowth") return MV_CTRG_LINKER;
    throw std::runtime_error(t + ": movetype not supported by the oracle");
}

Replica* build(const char* inp_path, const char* overrides, uint32_t seed, uint32_t replica) {
    auto* r = new Replica;
    try {
        ldo_io::Params& p = r->params;
        p = ldo_io::read_inp(inp_path);
        if (overrides && *overrides) {
            ldo_io::Params o = ldo_io::parse_inp_text(overrides);
            (void)o;
            std::istringstream is(overrides);
            std::string line;
            while (std::getline(is, line)) {
                auto eq = line.find('=');
                if (eq == std::string::npos) continue;
                ldo_io::set_param(p, ldo_io::trim(line.substr(0, eq)), ldo_io::trim(line.substr(eq + 1)));
            }
        }
        r->sf = ldo_io::read_system(ldo_io::resolve(p, p.origami_input_filename));
        // setup_origami (src/origami_system.cpp:1000-1003)
        if (!p.restart_traj_file.empty())
            r->sf.chains = ldo_io::read_trj_frame(ldo_io::resolve(p, p.restart_traj_file), p.restart_step);
        if (p.domain_type != "HalfTurn" && p.domain_type != "ThreeQuarterTurn")
            throw std::runtime_error(p.domain_type + ": No such domain type");
        if (p.binding_pot != "FourBody") throw std::runtime_error(p.binding_pot + ": No such binding potential");
        if (p.misbinding_pot != "Opposing" && p.misbinding_pot != "Disallowed")
            throw std::runtime_error(p.misbinding_pot + ": No such misbinding potential");
        EnergyModel& m = r->model;
        m.hybridization_pot = p.hybridization_pot;
        m.stacking_pot = p.stacking_pot;
        m.mean_field = p.apply_mean_field_cor;
        m.temp = p.temp;
        m.cation_M = p.cation_M;
        m.stacking_ene = p.stacking_ene;
        m.binding_h = p.binding_h;
        m.binding_s = p.binding_s;
        m.misbinding_h = p.misbinding_h;
        m.misbinding_s = p.misbinding_s;
        m.enthalpies = r->sf.enthalpies;
        m.entropies = r->sf.entropies;
        EnergyTables tab = build_tables(r->sf.identities, r->sf.sequences, m);

        Config c;
        c.identities = r->sf.identities;
        c.cyclic = r->sf.cyclic;
        c.three_quarter = p.domain_type == "ThreeQuarterTurn";
        c.misbinding_disallowed = p.misbinding_pot == "Disallowed";
        c.mean_field = p.apply_mean_field_cor;
        c.staple_M = p.staple_M;
        c.max_total_staples = p.max_total_staples;
        c.max_type_staples = p.max_type_staples;
        c.allow_nonsensical_ps = p.allow_nonsensical_ps;
        c.bias_mult = p.bias_functions_mult;
        c.centering_freq = p.centering_freq;
        c.centering_domain = p.centering_domain;
        c.constraint_check_freq = p.constraint_check_freq;
        auto moves = ldo_io::read_movetypes(ldo_io::resolve(p, p.movetype_file));
        double cum = 0;
        size_t S = c.identities.size() - 1;
        for (auto& mv : moves) {
            c.move_kinds.push_back(move_kind(mv.type));
            c.move_opts.push_back({mv.max_regrowth, mv.max_seg_regrowth, mv.max_num_recoils, mv.max_c_attempts,
                                   mv.max_disp, mv.max_turns, mv.max_linker_length, mv.num_transforms});
            cum += mv.freq;
            c.move_cum.push_back(cum);
            if (mv.type == "MetStapleExchange" || mv.type == "LearnedStapleExchange") {
                c.exchange_mults = mv.exchange_mults;
                while (c.exchange_mults.size() < S) c.exchange_mults.push_back(1);
                c.adaptive_exchange = mv.adaptive_exchange;
            }
        }
        std::vector<ChainInit> init;
        for (auto& ch : r->sf.chains) {
            ChainInit ci {ch.index, ch.identity, {}, {}};
            for (size_t d = 0; d < ch.positions.size(); ++d) {
                ci.pos.push_back(V3(ch.positions[d][0], ch.positions[d][1], ch.positions[d][2]));
                ci.ore.push_back(V3(ch.orientations[d][0], ch.orientations[d][1], ch.orientations[d][2]));
            }
            init.push_back(ci);
        }
        System& s = r->sys;
        s.rng.key[0] = seed;
        s.rng.key[1] = replica;
        s.rng.stream = 0;
        s.rng.draws = 0;
        s.init(c, tab, init);
        s.learn_tb = ldo_learn_tbin(m.temp);

        if (!p.order_parameter_file.empty()) {
            auto ops = ldo_io::read_ops(ldo_io::resolve(p, p.order_parameter_file));
            for (auto& o : ops) {
                OpRec rec;
                rec.tag = o.tag;
                if (o.type == "NumStaples") rec.kind = OP_NUMSTAPLES;
                else if (o.type == "NumStaplesType") { rec.kind = OP_NUMSTAPLESTYPE; rec.arg = o.staple; }
                else if (o.type == "StapleTypeFullyBound") { rec.kind = OP_STAPLETYPEFULLYBOUND; rec.arg = o.staple; }
                else if (o.type == "NumBoundDomainPairs") rec.kind = OP_NUMBOUND;
                else if (o.type == "NumMisboundDomainPairs") rec.kind = OP_NUMMISBOUND;
                else if (o.type == "NumStackedPairs") rec.kind = OP_NUMSTACKED;
                else if (o.type == "NumLinearHelices") rec.kind = OP_NUMLINEARHELICES;
                else if (o.type == "NumStackedJuncts") rec.kind = OP_NUMSTACKEDJUNCTS;
                else if (o.type == "Dist" || o.type == "AdjacentSite") {
                    // scaffold domains, updated per move (update_per_domain false)
                    rec.kind = o.type == "Dist" ? OP_DIST : OP_ADJACENT;
                    if (o.update_per_domain) throw std::runtime_error(o.type + ": update_per_domain not supported");
                    rec.parts = {o.domain1, o.domain2};
                }
                else if (o.type == "Sum") {
                    rec.kind = OP_SUM;
                    for (auto& t : o.ops) {
                        int idx = -1;
                        for (size_t q = 0; q < s.ops.size(); ++q)
                            if (s.ops[q].tag == t) idx = (int)q;
                        if (idx < 0) throw std::runtime_error("Sum order parameter: unknown tag " + t);
                        rec.parts.push_back(idx);
                    }
                }
                else throw std::runtime_error(o.type + ": order parameter type not supported by the oracle");
                s.ops.push_back(rec);
            }
        }
        if (!p.bias_functions_file.empty()) {
            auto bs = ldo_io::read_biases(ldo_io::resolve(p, p.bias_functions_file));
            for (auto& b : bs) {
                BiasRec rec;
                rec.tag = b.tag;
                for (auto& t : b.ops) {
                    int idx = -1;
                    for (size_t q = 0; q < s.ops.size(); ++q)
                        if (s.ops[q].tag == t) idx = (int)q;
                    if (idx < 0) throw std::runtime_error("bias function " + b.tag + ": unknown order parameter " + t);
                    rec.ops.push_back(idx);
                }
                rec.min_op = b.min_op;
                rec.max_op = b.max_op;
                rec.well_bias = b.well_bias;
                rec.min_bias = b.min_bias;
                rec.slope = b.slope;
                rec.outside_bias = b.outside_bias;
                rec.k = b.k;
                rec.centre = b.centre;
                if (b.type == "LinearStepWell") rec.kind = B_LINEARSTEPWELL;
                else if (b.type == "SquareWell") rec.kind = B_SQUAREWELL;
                else if (b.type == "Grid") rec.kind = B_GRID;
                else if (b.type == "Harmonic") rec.kind = B_HARMONIC;
                else throw std::runtime_error(b.type + "; no such bias function type");
                if (rec.ops.empty()) throw std::runtime_error("bias function " + b.tag + " has no order parameter");
                s.biases.push_back(rec);
            }
        }
        s.init_biases();
    } catch (std::exception& e) {
        g_err = e.what();
        delete r;
        return nullptr;
    }
    return r;
}

} // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

void* oracle_create(const char* inp_path, const char* overrides, uint32_t seed, uint32_t replica) {
    return build(inp_path, overrides, seed, replica);
}

void oracle_destroy(void* h) { delete static_cast<Replica*>(h); }

// Runs `steps` move attempts.  If trace != nullptr, writes 8 doubles per step:
// step, energy, staples, fully bound pairs, bound pairs, stacked pairs,
// total bias, random draws so far.
int oracle_run(void* h, long long steps, long long start_step, double* trace) {
    auto* r = static_cast<Replica*>(h);
    try {
        for (long long k = 0; k < steps; ++k) {
            long long st = start_step + k + 1;
            r->sys.step(st);
            if (trace) {
                double* t = trace + 8 * k;
                System& s = r->sys;
                t[0] = (double)st;
                t[1] = s.energy;
                t[2] = s.num_staples;
                t[3] = s.num_fully;
                t[4] = s.num_bound;
                t[5] = s.num_stacked;
                t[6] = s.total_bias();
                t[7] = (double)s.rng.draws;
            }
        }
    } catch (std::exception& e) {
        g_err = e.what();
        return -1;
    }
    return 0;
}

// Flattened configuration: n_chains, then per chain: index, identity, length,
// and length x (x, y, z, ox, oy, oz, state).  Returns ints written or -needed.
int oracle_get_config(void* h, int* buf, int cap) {
    auto* r = static_cast<Replica*>(h);
    System& s = r->sys;
    std::vector<int> out;
    out.push_back((int)s.chains.size());
    for (size_t c = 0; c < s.chains.size(); ++c) {
        out.push_back(s.chain_index[c]);
        out.push_back(s.chain_ident[c]);
        out.push_back((int)s.chains[c].size());
        for (int id : s.chains[c]) {
            const Dom& d = s.doms[id];
            int v[7] = {d.pos.x, d.pos.y, d.pos.z, d.ore.x, d.ore.y, d.ore.z, d.state};
            out.insert(out.end(), v, v + 7);
        }
    }
    if ((int)out.size() > cap) return -(int)out.size();
    std::memcpy(buf, out.data(), out.size() * sizeof(int));
    return (int)out.size();
}

// energy, staples, fully, bound, self, stacked, unassigned, total bias, draws, current_c_i
void oracle_observables(void* h, double* out) {
    System& s = static_cast<Replica*>(h)->sys;
    out[0] = s.energy;
    out[1] = s.num_staples;
    out[2] = s.num_fully;
    out[3] = s.num_bound;
    out[4] = s.num_self;
    out[5] = s.num_stacked;
    out[6] = s.num_unassigned;
    out[7] = s.total_bias();
    out[8] = (double)s.rng.draws;
    out[9] = s.current_c_i;
}

// IdealRandomWalks::num_walks between sites dr apart in `steps` steps.
double oracle_ideal_walks(int dx, int dy, int dz, int steps) { return (double)ideal_walks(dx, dy, dz, steps); }

// The reference's own arithmetic (long double Rosenbluth weights, the C
// library's exp) instead of the engine's (FP64, ldo_math::exp).
void oracle_set_reference_arithmetic(void* h, int on) { static_cast<Replica*>(h)->sys.ld_weights = on != 0; }

// The engine's exponential on the host (ldo_math::exp), n values.
void oracle_engine_exp(const double* x, double* y, int n) {
    for (int i = 0; i < n; ++i) y[i] = ldo_math::exp(x[i]);
}

// Per-move attempts/accepts, 2 x n_moves.
// Per movetype: attempts, domain-record accesses, occupancy-map operations
// (the ORACLE_COUNT_TOUCHES build; -1 in the normal one).
int oracle_touch_counts(void* h, long long* out, int cap) {
#ifdef ORACLE_COUNT_TOUCHES
    auto& sy = static_cast<Replica*>(h)->sys;
    int n = (int)sy.attempts.size();
    if (cap < 3 * n) return -1;
    for (int m = 0; m < n; ++m) {
        out[3 * m] = sy.attempts[m];
        out[3 * m + 1] = sy.touch_dom[m];
        out[3 * m + 2] = sy.touch_site[m];
    }
    return n;
#else
    (void)h;
    (void)out;
    (void)cap;
    return -1;
#endif
}

int oracle_move_stats(void* h, long long* out, int cap) {
    System& s = static_cast<Replica*>(h)->sys;
    int n = (int)s.attempts.size();
    if (2 * n > cap) return -2 * n;
    for (int i = 0; i < n; ++i) {
        out[2 * i] = s.attempts[i];
        out[2 * i + 1] = s.accepts[i];
    }
    return n;
}

// Energy tables: returns imax; fills (2 imax + 1)^2 entries each if non-null.
int oracle_tables(void* h, double* hyb_e, double* hyb_h, double* hyb_s, double* stack_e, double* init3) {
    const EnergyTables& t = static_cast<Replica*>(h)->sys.tab;
    size_t n = t.hyb_e.size();
    if (hyb_e) std::memcpy(hyb_e, t.hyb_e.data(), n * sizeof(double));
    if (hyb_h) std::memcpy(hyb_h, t.hyb_h.data(), n * sizeof(double));
    if (hyb_s) std::memcpy(hyb_s, t.hyb_s.data(), n * sizeof(double));
    if (stack_e) std::memcpy(stack_e, t.stack_e.data(), n * sizeof(double));
    if (init3) {
        init3[0] = t.init_h;
        init3[1] = t.init_s;
        init3[2] = t.init_e;
    }
    return t.imax;
}

// OrigamiSystem::update_temp (src/origami_system.cpp:618): new tables, full
// energy recomputation.
// Weight table of the learned insertion proposal (the engine's, LDO_LEARN_TABLE
// doubles), used by LearnedStapleExchange.
int oracle_set_learn_table(void* h, const double* w, int n) {
    auto* r = static_cast<Replica*>(h);
    if (n != LDO_LEARN_TABLE) {
        g_err = "learn table size";
        return -1;
    }
    r->learn_w.assign(w, w + n);
    r->sys.learn_w = r->learn_w.data();
    return 0;
}

int oracle_update_temp(void* h, double temp, double stacking_mult) {
    auto* r = static_cast<Replica*>(h);
    try {
        EnergyModel m = r->model;
        m.temp = temp;
        m.stacking_mult = stacking_mult;
        r->sys.tab = build_tables(r->sf.identities, r->sf.sequences, m);
        r->sys.learn_tb = ldo_learn_tbin(temp);
        r->sys.recompute_energy();
    } catch (std::exception& e) {
        g_err = e.what();
        return -1;
    }
    return 0;
}

// H, S, stacking as the PTMC driver's dependent quantities
// (PTGCMCSimulation::update_dependent_qs, src/ptmc_simulation.cpp:152).
void oracle_dependent_qs(void* h, double* out) {
    System& s = static_cast<Replica*>(h)->sys;
    double H, S, st;
    s.enthalpy_entropy(H, S, st);
    out[0] = H;
    out[1] = S;
    out[2] = st;
    out[3] = s.total_bias();
}

// SquareWellBiasFunction::set_min_op / set_max_op (src/bias_functions.cpp:218-220)
int oracle_set_window(void* h, const char* tag, int min_op, int max_op) {
    System& s = static_cast<Replica*>(h)->sys;
    for (auto& b : s.biases)
        if (b.tag == tag) {
            b.min_op = min_op;
            b.max_op = max_op;
            return 0;
        }
    g_err = std::string("no bias ") + tag;
    return -1;
}

int oracle_set_bias_centre(void* h, const char* tag, double centre) {
    System& s = static_cast<Replica*>(h)->sys;
    for (auto& b : s.biases)
        if (b.tag == tag && b.kind == B_HARMONIC) {
            b.centre = centre;
            return 0;
        }
    g_err = std::string("no harmonic bias ") + tag;
    return -1;
}

// `count` uniform reals of Philox key (seed, key1), stream `stream`, from draw `first`.
void oracle_uniforms(uint32_t seed, uint32_t key1, uint32_t stream, unsigned long long first, int count, double* out) {
    Stream st;
    st.key[0] = seed;
    st.key[1] = key1;
    st.stream = stream;
    st.draws = first;
    for (int i = 0; i < count; ++i) out[i] = st.uniform_real();
}

// Staple counts per chain type (index 0 = scaffold, always 0 here), as
// OrigamiSystem::get_staple_counts (src/origami_system.cpp:153).
int oracle_staple_counts(void* h, int* out, int cap) {
    System& s = static_cast<Replica*>(h)->sys;
    int n = (int)s.cfg.identities.size();
    if (n > cap) return -n;
    for (int t = 0; t < n; ++t) out[t] = t == 0 ? 0 : s.num_staples_of_ident(t);
    return n;
}

// Uniform reals of the swap stream: `count` draws of Philox key (seed,
// ladder), stream 1, starting at draw index `first`.
void oracle_swap_uniforms(uint32_t seed, uint32_t ladder, unsigned long long first, int count, double* out) {
    Stream st;
    st.key[0] = seed;
    st.key[1] = ladder;
    st.stream = 1;
    st.draws = first;
    for (int i = 0; i < count; ++i) out[i] = st.uniform_real();
}

// Grid bias values (1-D, index = order-parameter value) for bias `tag`.
int oracle_set_grid(void* h, const char* tag, const double* vals, int n) {
    System& s = static_cast<Replica*>(h)->sys;
    for (auto& b : s.biases)
        if (b.tag == tag && b.kind == B_GRID) {
            // GridBiasFunction::replace_biases (src/bias_functions.cpp:237): the
            // cached bias value changes only at the next update.
            b.grid.assign(vals, vals + n);
            b.grid_set = true;
            return 0;
        }
    g_err = std::string("no grid bias ") + tag;
    return -1;
}

// CPU baseline: n_rep independent replicas of one system, seeds seed0+i,
// each for `steps` move attempts, on `threads` host threads.  Returns the
// wall time in seconds, or a negative value on error.
double oracle_run_batch(const char* inp_path, const char* overrides, uint32_t seed0, int n_rep, long long steps,
                        int threads) {
    std::vector<Replica*> reps(n_rep, nullptr);
    for (int i = 0; i < n_rep; ++i) {
        reps[i] = build(inp_path, overrides, seed0, (uint32_t)i);
        if (!reps[i]) {
            for (auto* r : reps) delete r;
            return -1;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    std::atomic<int> next {0};
    std::atomic<int> failed {0};
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                int i = next.fetch_add(1);
                if (i >= n_rep) break;
                try {
                    for (long long k = 0; k < steps; ++k) reps[i]->sys.step(k + 1);
                } catch (...) {
                    failed.store(1);
                }
            }
        });
    for (auto& th : pool) th.join();
    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (auto* r : reps) delete r;
    return failed.load() ? -2 : dt;
}

// Independent replicas (key (seed0, r)) with an optional learned-proposal
// weight table: after `burn` steps, n_snaps snapshots `gap` steps apart of
// (staples, fully bound pairs) into out[(r * n_snaps + k) * 2].  Returns 0, or
// -1 if a replica failed.
int oracle_run_batch_states(const char* inp_path, const char* overrides, uint32_t seed0, int n_rep, long long burn,
                            long long gap, int n_snaps, int threads, const double* learn_w, int* out) {
    std::vector<Replica*> reps(n_rep, nullptr);
    for (int i = 0; i < n_rep; ++i) {
        reps[i] = build(inp_path, overrides, seed0, (uint32_t)i);
        if (!reps[i]) {
            for (auto* r : reps) delete r;
            return -1;
        }
        reps[i]->sys.learn_w = learn_w;   // shared, read-only
    }
    std::vector<std::thread> pool;
    std::atomic<int> next {0};
    std::atomic<int> failed {0};
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                int i = next.fetch_add(1);
                if (i >= n_rep) break;
                try {
                    long long st = 0;
                    for (long long k = 0; k < burn; ++k) reps[i]->sys.step(++st);
                    for (int s = 0; s < n_snaps; ++s) {
                        for (long long k = 0; k < gap; ++k) reps[i]->sys.step(++st);
                        out[((size_t)i * n_snaps + s) * 2] = reps[i]->sys.num_staples;
                        out[((size_t)i * n_snaps + s) * 2 + 1] = reps[i]->sys.num_fully;
                    }
                } catch (std::exception& e) {
                    failed.store(1);
                }
            }
        });
    for (auto& th : pool) th.join();
    for (auto* r : reps) delete r;
    return failed.load() ? -1 : 0;
}

// CPU baseline with order-parameter samples: n_rep replicas (key (seed0, r)),
// each `sweeps` sweeps of sweep_len steps; after every sweep the number of
// fully bound domain pairs goes to out[r * sweeps + k].  Returns wall seconds.
double oracle_run_batch_sampled_centres(const char* inp_path, const char* overrides, uint32_t seed0, int n_rep,
                                        long long sweeps, int sweep_len, int threads, const double* temps,
                                        const char* centre_tag, const double* centres, short* out) {
    std::vector<Replica*> reps(n_rep, nullptr);
    for (int i = 0; i < n_rep; ++i) {
        reps[i] = build(inp_path, overrides, seed0, (uint32_t)i);
        if (!reps[i] || (temps && oracle_update_temp(reps[i], temps[i], 1.0) != 0) ||
            (centres && oracle_set_bias_centre(reps[i], centre_tag, centres[i]) != 0)) {
            for (auto* r : reps) delete r;
            return -1;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    std::atomic<int> next {0};
    std::atomic<int> failed {0};
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                int i = next.fetch_add(1);
                if (i >= n_rep) break;
                try {
                    long long st = 0;
                    for (long long k = 0; k < sweeps; ++k) {
                        for (int q = 0; q < sweep_len; ++q) reps[i]->sys.step(++st);
                        out[(size_t)i * sweeps + k] = (short)reps[i]->sys.num_fully;
                    }
                } catch (...) {
                    failed.store(1);
                }
            }
        });
    for (auto& th : pool) th.join();
    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (auto* r : reps) delete r;
    return failed.load() ? -2 : dt;
}

double oracle_run_batch_sampled(const char* inp_path, const char* overrides, uint32_t seed0, int n_rep,
                                long long sweeps, int sweep_len, int threads, const double* temps, short* out) {
    return oracle_run_batch_sampled_centres(inp_path, overrides, seed0, n_rep, sweeps, sweep_len, threads, temps,
                                            nullptr, nullptr, out);
}

} // extern "C"
