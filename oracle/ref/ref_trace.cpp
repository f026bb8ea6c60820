// Trace driver for the reference compiled from its own sources.
//
// Reads a parameter file in the reference's key=value (.inp) format plus a few
// trace_* keys, builds the system with origami::setup_origami
// (src/origami_system.cpp:991), and runs the reference's own move loop
// GCMCSimulation::simulate (src/simulation.cpp:568) with the Philox RNG of
// ref_random_gens.cpp.  After every step it records the energy and counters,
// and every trace_every steps the full configuration, as JSON on stdout.
//
// Extra keys: trace_steps, trace_seed, trace_replica, trace_every,
//             trace_mode (simulate | enumerate | anneal: the reference's
//             annealing loop over max_temp .. min_temp)
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "LatticeDNAOrigami/annealing_simulation.hpp"
#include "LatticeDNAOrigami/bias_functions.hpp"
#include "LatticeDNAOrigami/enumerate.hpp"
#include "LatticeDNAOrigami/order_params.hpp"
#include "LatticeDNAOrigami/origami_system.hpp"
#include "LatticeDNAOrigami/parser.hpp"
#include "LatticeDNAOrigami/simulation.hpp"

extern "C" void ldo_ref_rng_configure(uint32_t seed, uint32_t replica, uint32_t stream);
extern "C" uint64_t ldo_ref_rng_draws();

char const* const GIT_COMMIT = "oracle-build";

using std::string;
using std::vector;

#include "ref_params.h"

namespace {

using ldo_refdrv::dump_config;
using ldo_refdrv::fill_params;
using ldo_refdrv::read_kv;

// The staple-only enumerator with the partition-function increment of every
// conformational enumeration (one growth-point set) recorded in order.
class UnitStapleEnum : public enumerator::StapleConformationalEnumerator {
  public:
    using StapleConformationalEnumerator::StapleConformationalEnumerator;
    void enumerate() override {
        long double z0 = m_partition_f, n0 = m_num_configs;
        StapleConformationalEnumerator::enumerate();
        units.push_back({(double)(m_partition_f - z0), (double)(m_num_configs - n0)});
    }
    vector<std::pair<double, double>> units;
};

// The same for the full conformational enumeration (the scaffold
// enumerated too, ConformationalEnumerator::enumerate, src/enumerate.cpp:218),
// with the change of the running energy m_energy over the unit, which every
// set and unassign leaves balanced in exact arithmetic (its rounding drift).
class UnitConfEnum : public enumerator::ConformationalEnumerator {
  public:
    using ConformationalEnumerator::ConformationalEnumerator;
    void enumerate() override {
        long double z0 = m_partition_f, n0 = m_num_configs, e0 = m_energy;
        std::map<vector<int>, double> w0(m_state_weights.begin(), m_state_weights.end());
        ConformationalEnumerator::enumerate();
        units.push_back({(double)(m_partition_f - z0), (double)(m_num_configs - n0)});
        drift.push_back((double)(m_energy - e0));
        // each bin's increment over the unit (its double running sum's)
        std::map<vector<int>, double> inc;
        for (auto& kv : m_state_weights) {
            double before = w0.count(kv.first) ? w0[kv.first] : 0.0;
            if (kv.second != before) inc[kv.first] = kv.second - before;
        }
        bins.push_back(inc);
    }

    // With exact_bins set, the weight of every configuration, as
    // calc_and_save_weights (src/enumerate.cpp:639) computes and adds it, is
    // also summed into a compensated long-double sum per bin.  The reference
    // keeps each bin of m_state_weights as a running double sum, whose
    // roundings accumulate over the millions of configurations of a bin; the
    // compensated sums are the same weights summed without that error.  The
    // weight is read off m_partition_f (zeroed before the configuration is
    // saved, so that it holds exactly the added weight) and m_partition_f is
    // then given the value the reference's own addition gives.
    void grow_next_domain(domainContainer::Domain* domain, utility::VectorThree p_new) override {
        if (!exact_bins || !m_domains.empty()) {
            ConformationalEnumerator::grow_next_domain(domain, p_new);
            return;
        }
        m_ops.update_move_params();   // recomputes from the system: the key calc_and_save_weights reads
        vector<int> key;
        for (auto op : m_ops_to_output) key.push_back(op.get().get_param());
        long double z = m_partition_f, n = m_num_configs;
        m_partition_f = 0;
        ConformationalEnumerator::grow_next_domain(domain, p_new);
        long double w = m_partition_f;
        m_partition_f = z + w;
        if (m_num_configs != n) {
            ++exact_calls;
            if (key.size() == 2 && key[0] >= 0 && key[0] < 64 && key[1] >= 0 && key[1] < 64) flat[key[0] * 64 + key[1]].add(w);
            else other[key].add(w);
        }
    }
    // Neumaier's compensated summation in long double
    struct Acc {
        long double s = 0, c = 0;
        long long n = 0;
        void add(long double x) {
            long double t = s + x;
            c += (fabsl(s) >= fabsl(x)) ? (s - t) + x : (x - t) + s;
            s = t;
            ++n;
        }
        long double value() const { return s + c; }
    };
    std::map<vector<int>, Acc> exact() const {
        std::map<vector<int>, Acc> out(other.begin(), other.end());
        for (int k = 0; k < 64 * 64; ++k)
            if (flat[k].n) out[{k / 64, k % 64}] = flat[k];
        return out;
    }
    bool exact_bins = false;
    long long exact_calls = 0;
    vector<Acc> flat = vector<Acc>(64 * 64);
    std::map<vector<int>, Acc> other;

    vector<std::pair<double, double>> units;
    vector<double> drift;
    vector<std::map<vector<int>, double>> bins;
};

class TraceSim : public simulation::GCMCSimulation {
  public:
    TraceSim(origami::OrigamiSystem& o, orderParams::SystemOrderParams& ops,
             biasFunctions::SystemBiases& b, parser::InputParameters& p, long every,
             std::ostream& out)
        : GCMCSimulation(o, ops, b, p), m_every(every), m_out(out) {
        m_logging_stream = &std::cerr;
        if (p.m_configs_output_freq || p.m_vtf_output_freq || p.m_counts_output_freq || p.m_energies_output_freq ||
            p.m_order_params_output_freq)
            m_output_files = simulation::setup_output_files(p, p.m_output_filebase, o, ops, b, m_random_gens);
    }
    void run() override {}
    bool m_first {true};

    bool m_quiet {false};

  protected:
    void update_internal(long long int step) override {
        if (m_quiet) return;
        auto& o = m_origami_system;
        char buf[512];
        std::snprintf(buf, sizeof buf, "%s[%lld,%.17g,%d,%d,%d,%d,%.17g,%llu]",
                      m_first ? "" : ",", step, o.energy(), o.num_staples(),
                      o.num_fully_bound_domain_pairs(), o.num_bound_domain_pairs(),
                      o.num_stacked_domain_pairs(), m_biases.get_total_bias(),
                      (unsigned long long)ldo_ref_rng_draws());
        m_out << buf;
        m_first = false;
        if (m_every > 0 && step % m_every == 0) {
            std::ostringstream d;
            d << "[" << step << ",";
            dump_config(o, d);
            d << "]";
            m_dumps.push_back(d.str());
        }
    }

  public:
    long m_every;
    std::ostream& m_out;
    vector<string> m_dumps;
    // attempts and accepts of every movetype, in the movetype file's order
    string move_stats() {
        std::ostringstream s;
        s << "[";
        for (size_t i = 0; i < m_movetypes.size(); ++i)
            s << (i ? "," : "") << "[" << m_movetypes[i]->get_attempts() << "," << m_movetypes[i]->get_accepts()
              << "]";
        s << "]";
        return s.str();
    }
};

// The reference's own annealing loop (AnnealingGCMCSimulation::run,
// src/annealing_simulation.cpp:40) with the per-step record of TraceSim.
class TraceAnneal : public annealing::AnnealingGCMCSimulation {
  public:
    TraceAnneal(origami::OrigamiSystem& o, orderParams::SystemOrderParams& ops, biasFunctions::SystemBiases& b,
                parser::InputParameters& p, std::ostream& out)
        : AnnealingGCMCSimulation(o, ops, b, p), m_out(out) {
        m_logging_stream = &std::cerr;
    }

  private:
    bool m_first {true};
    std::ostream& m_out;
    void update_internal(long long int step) override {
        auto& o = m_origami_system;
        char buf[512];
        std::snprintf(buf, sizeof buf, "%s[%lld,%.17g,%d,%d,%d,%d,%.17g,%llu]",
                      m_first ? "" : ",", step, o.energy(), o.num_staples(),
                      o.num_fully_bound_domain_pairs(), o.num_bound_domain_pairs(),
                      o.num_stacked_domain_pairs(), m_biases.get_total_bias(),
                      (unsigned long long)ldo_ref_rng_draws());
        m_out << buf;
        m_first = false;
    }
};

} // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: ref_trace <params>\n";
        return 2;
    }
    auto kv = read_kv(argv[1]);
    parser::InputParameters params;
    fill_params(params, kv);
    long long steps = kv.count("trace_steps") ? std::stoll(kv["trace_steps"]) : 0;
    uint32_t seed = kv.count("trace_seed") ? (uint32_t)std::stoul(kv["trace_seed"]) : 0u;
    uint32_t rep = kv.count("trace_replica") ? (uint32_t)std::stoul(kv["trace_replica"]) : 0u;
    long every = kv.count("trace_every") ? std::stol(kv["trace_every"]) : 0;
    string mode = kv.count("trace_mode") ? kv["trace_mode"] : string("simulate");
    try {
        origami::OrigamiSystem* o = origami::setup_origami(params);
        if (mode == "enumerate") {
            // enumerate_main (src/enumerate.cpp:19) with the weights printed
            // at full precision instead of print_weights' six digits
            auto& ops = o->get_system_order_params();
            auto& biases = o->get_system_biases();
            enumerator::OvercountCalculator* oc;
            if (params.m_max_staple_size == 2) oc = new enumerator::MaxTwoDomainOvercountCalculator {};
            else if (params.m_misbinding_pot == "Disallowed") oc = new enumerator::MisbindingOnlyOvercountCalculator {};
            else throw std::runtime_error("No enumerator available for system");
            enumerator::ConformationalEnumerator* ce;
            if (params.m_enumerate_staples_only)
                ce = new UnitStapleEnum {*o, *oc, ops, biases, params.m_ops_to_output, params.m_apply_mean_field_cor};
            else {
                auto* uc = new UnitConfEnum {*o, *oc, ops, biases, params.m_ops_to_output, params.m_apply_mean_field_cor};
                uc->exact_bins = kv.count("trace_exact_bins") && kv["trace_exact_bins"] == "1";
                ce = uc;
            }
            enumerator::GrowthpointEnumerator* ge;
            if (params.m_misbinding_pot == "Disallowed")
                ge = new enumerator::NoMisbindingGrowthpointEnumerator {*ce, *o};
            else
                ge = new enumerator::MisbindingGrowthpointEnumerator {*ce, *o};
            enumerator::StapleEnumerator se {*ge, *ce, *o, params.m_excluded_staples};
            auto t0 = std::chrono::steady_clock::now();
            se.enumerate(params.m_min_total_staples, params.m_max_total_staples, params.m_max_type_staples);
            double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            ce->normalize_weights();
            std::map<vector<int>, double> sorted(ce->m_normalized_weights.begin(), ce->m_normalized_weights.end());
            std::ostringstream js;
            js << "@@{\"weights\": {";
            bool first = true;
            for (auto& kv : sorted) {
                js << (first ? "" : ", ") << "\"";
                for (size_t i = 0; i < kv.first.size(); ++i) js << (i ? " " : "") << kv.first[i];
                char b[64];
                std::snprintf(b, sizeof b, "\": %.17g", kv.second);
                js << b;
                first = false;
            }
            char b[128];
            std::snprintf(b, sizeof b, "}, \"num_configs\": %.17Lg, \"seconds\": %.6f", ce->num_configs(), secs);
            js << b;
            // trace_exact_bins=1: every bin summed without rounding drift
            // (compensated), normalised by the compensated partition function,
            // with the number of configurations saved into the bin
            if (!params.m_enumerate_staples_only && static_cast<UnitConfEnum*>(ce)->exact_bins) {
                auto* uc = static_cast<UnitConfEnum*>(ce);
                auto ex = uc->exact();
                UnitConfEnum::Acc z;
                for (auto& e : ex) z.add(e.second.value());
                js << ", \"weights_exact\": {";
                bool f = true;
                for (auto& e : ex) {
                    js << (f ? "\"" : ", \"");
                    for (size_t i = 0; i < e.first.size(); ++i) js << (i ? " " : "") << e.first[i];
                    std::snprintf(b, sizeof b, "\": %.17g", (double)(e.second.value() / z.value()));
                    js << b;
                    f = false;
                }
                js << "}, \"bin_configs\": {";
                f = true;
                for (auto& e : ex) {
                    js << (f ? "\"" : ", \"");
                    for (size_t i = 0; i < e.first.size(); ++i) js << (i ? " " : "") << e.first[i];
                    js << "\": " << e.second.n;
                    f = false;
                }
                std::snprintf(b, sizeof b, "}, \"saved_configs\": %lld", uc->exact_calls);
                js << b;
            }
            // trace_units=1: the partition-function increment of every
            // growth-point set, in enumeration order
            if (kv.count("trace_units") && kv["trace_units"] == "1") {
                js << ", \"units\": [";
                auto& us = params.m_enumerate_staples_only ? static_cast<UnitStapleEnum*>(ce)->units
                                                           : static_cast<UnitConfEnum*>(ce)->units;
                for (size_t i = 0; i < us.size(); ++i) {
                    std::snprintf(b, sizeof b, "%s[%.17g, %.17g]", i ? ", " : "", us[i].first, us[i].second);
                    js << b;
                }
                js << "]";
                if (!params.m_enumerate_staples_only && kv.count("trace_unit_bins") && kv["trace_unit_bins"] == "1") {
                    js << ", \"unit_bins\": [";
                    auto& bs = static_cast<UnitConfEnum*>(ce)->bins;
                    for (size_t i = 0; i < bs.size(); ++i) {
                        js << (i ? ", {" : "{");
                        bool f = true;
                        for (auto& e : bs[i]) {
                            std::snprintf(b, sizeof b, "%s\"%d %d\": %.17g", f ? "" : ", ", e.first[0], e.first[1],
                                          e.second);
                            js << b;
                            f = false;
                        }
                        js << "}";
                    }
                    js << "]";
                }
                if (!params.m_enumerate_staples_only) {
                    js << ", \"unit_energy_drift\": [";
                    auto& dr = static_cast<UnitConfEnum*>(ce)->drift;
                    for (size_t i = 0; i < dr.size(); ++i) {
                        std::snprintf(b, sizeof b, "%s%.17g", i ? ", " : "", dr[i]);
                        js << b;
                    }
                    js << "]";
                }
            }
            js << "}";
            std::cout << "\n" << js.str() << "\n";
            delete ge;
            delete ce;
            delete oc;
            return 0;
        }
        ldo_ref_rng_configure(seed, rep, 0);
        auto& ops = o->get_system_order_params();
        auto& biases = o->get_system_biases();
        std::cout << "{\"initial\": ";
        dump_config(*o, std::cout);
        char buf[256];
        std::snprintf(buf, sizeof buf, ", \"initial_energy\": %.17g, \"steps\": [", o->energy());
        std::cout << buf;
        auto t0 = std::chrono::steady_clock::now();
        if (mode == "anneal") {
            TraceAnneal sim(*o, ops, biases, params, std::cout);
            sim.run();
            std::cout << "], \"dumps\": [[-1,";
            dump_config(*o, std::cout);
            std::cout << "]";
        }
        else {
            TraceSim sim(*o, ops, biases, params, every, std::cout);
            // trace_quiet=1: no per-step records (for timing the move loop)
            sim.m_quiet = kv.count("trace_quiet") && kv["trace_quiet"] == "1";
            sim.simulate(steps, 0, false);
            std::cout << "], \"move_stats\": " << sim.move_stats() << ", \"dumps\": [";
            for (size_t i = 0; i < sim.m_dumps.size(); ++i) std::cout << (i ? "," : "") << sim.m_dumps[i];
        }
        double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::snprintf(buf, sizeof buf, "], \"final_energy\": %.17g, \"draws\": %llu, \"seconds\": %.6f}\n",
                      o->energy(), (unsigned long long)ldo_ref_rng_draws(), secs);
        std::cout << buf;
        delete o;
    } catch (std::exception& e) {
        std::cout << "{\"error\": \"" << e.what() << "\"}\n";
        return 3;
    }
    return 0;
}
