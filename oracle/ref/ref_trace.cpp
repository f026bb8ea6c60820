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

namespace {

std::map<string, string> read_kv(const string& fname) {
    std::ifstream f(fname);
    if (!f) {
        std::cerr << "cannot open " << fname << "\n";
        std::exit(2);
    }
    std::map<string, string> kv;
    string line;
    while (std::getline(f, line)) {
        auto h = line.find('#');
        if (h != string::npos) line = line.substr(0, h);
        auto eq = line.find('=');
        if (eq == string::npos) continue;
        auto trim = [](string s) {
            size_t a = s.find_first_not_of(" \t\r");
            size_t b = s.find_last_not_of(" \t\r");
            return a == string::npos ? string() : s.substr(a, b - a + 1);
        };
        kv[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return kv;
}

vector<string> split_ws(const string& s) {
    std::istringstream is(s);
    vector<string> out;
    string t;
    while (is >> t) out.push_back(t);
    return out;
}

// Defaults are those of src/parser.cpp:33-449.
void fill_params(parser::InputParameters& p, std::map<string, string>& kv) {
    auto S = [&](const char* k, const char* d) { return kv.count(k) ? kv[k] : string(d); };
    auto D = [&](const char* k, double d) { return kv.count(k) ? std::stod(kv[k]) : d; };
    auto I = [&](const char* k, long long d) { return kv.count(k) ? std::stoll(kv[k]) : d; };
    auto B = [&](const char* k, bool d) {
        if (!kv.count(k)) return d;
        string v = kv[k];
        return v == "true" || v == "1" || v == "yes" || v == "on";
    };
    p.m_origami_input_filename = S("origami_input_filename", "");
    p.m_domain_type = S("domain_type", "Halfturn");
    p.m_binding_pot = S("binding_pot", "FourBody");
    p.m_misbinding_pot = S("misbinding_pot", "Opposing");
    p.m_stacking_pot = S("stacking_pot", "Constant");
    p.m_hybridization_pot = S("hybridization_pot", "NearestNeighbour");
    p.m_apply_mean_field_cor = B("apply_mean_field_cor", false);
    p.m_temp = D("temp", 300);
    p.m_staple_M = D("staple_M", 1);
    p.m_cation_M = D("cation_M", 1);
    p.m_temp_for_staple_u = p.m_temp;
    p.m_staple_u_mult = D("staple_u_mult", 1);
    p.m_constant_staple_M = B("constant_staple_M", true);
    p.m_stacking_ene = D("stacking_ene", 1);
    p.m_binding_h = D("binding_h", 0);
    p.m_binding_s = D("binding_s", 0);
    p.m_misbinding_h = D("misbinding_h", 0);
    p.m_misbinding_s = D("misbinding_s", 0);
    p.m_min_total_staples = (int)I("min_total_staples", 0);
    p.m_max_total_staples = (int)I("max_total_staples", 999);
    p.m_max_type_staples = (int)I("max_type_staples", 999);
    p.m_max_staple_size = (int)I("max_staple_size", 2);
    p.m_domain_update_biases_present = B("domain_update_biases_present", false);
    p.m_ops_filename = S("order_parameter_file", "");
    p.m_bias_funcs_filename = S("bias_functions_file", "");
    p.m_bias_funcs_mult = D("bias_functions_mult", 1);
    p.m_energy_filebase = S("energy_filebase", "");
    p.m_simulation_type = S("simulation_type", "constant_temp");
    p.m_enumerate_staples_only = B("enumerate_staples_only", false);
    p.m_random_seed = -1;
    p.m_movetype_filename = S("movetype_file", "");
    p.m_read_num_walks = false;
    p.m_num_walks_filename = "";
    p.m_restart_from_config = false;
    p.m_restart_traj_file = S("restart_traj_file", "");
    p.m_restart_traj_filebase = "";
    p.m_restart_traj_postfix = ".trj";
    p.m_restart_us_iter = false;
    p.m_restart_us_filebase = "";
    p.m_restart_step = (int)I("restart_step", 0);
    p.m_restart_from_swap = false;
    p.m_read_rand_engine_state = false;
    p.m_rand_engine_state_file = "";
    p.m_vmd_file_dir = "";
    p.m_logging_freq = 0;
    p.m_centering_freq = (int)I("centering_freq", 0);
    p.m_centering_domain = (int)I("centering_domain", 0);
    p.m_constraint_check_freq = (int)I("constraint_check_freq", 0);
    p.m_allow_nonsensical_ps = B("allow_nonsensical_ps", false);
    p.m_max_duration = 10e9;
    p.m_ct_steps = 0;
    p.m_max_temp = D("max_temp", 400);
    p.m_min_temp = D("min_temp", 300);
    p.m_temp_interval = D("temp_interval", 1);
    p.m_steps_per_temp = I("steps_per_temp", 0);
    p.m_num_reps = 1;
    p.m_exchange_interval = 0;
    p.m_swaps = 0;
    p.m_max_pt_dur = 10e9;
    p.m_us_grid_bias_tag = "";
    p.m_max_num_iters = 0;
    p.m_max_D_bias = 0;
    p.m_equil_steps = 0;
    p.m_max_equil_dur = 0;
    p.m_iter_steps = 0;
    p.m_iter_swaps = 0;
    p.m_max_iter_dur = 0;
    p.m_max_rel_P_diff = 0.1;
    p.m_read_biases = false;
    p.m_multi_window = false;
    p.m_output_filebase = S("output_filebase", "/tmp/ldo_ref_trace");
    // the reference's output writers (src/simulation.cpp:47), when asked for
    p.m_configs_output_freq = (int)I("configs_output_freq", 0);
    p.m_vtf_output_freq = (int)I("vtf_output_freq", 0);
    p.m_vcf_per_domain = false;
    p.m_counts_output_freq = (int)I("counts_output_freq", 0);
    p.m_times_output_freq = 0;
    p.m_energies_output_freq = (int)I("energies_output_freq", 0);
    p.m_order_params_output_freq = (int)I("order_params_output_freq", 0);
    p.m_rand_engine_state_output_freq = 0;
    p.m_vmd_pipe_freq = 0;
    p.m_create_vmd_instance = false;
    if (kv.count("ops_to_output")) p.m_ops_to_output = split_ws(kv["ops_to_output"]);
}

void dump_config(origami::OrigamiSystem& o, std::ostream& out) {
    out << "[";
    bool firstc = true;
    for (auto& chain : o.get_chains()) {
        out << (firstc ? "" : ",") << "[" << chain[0]->m_c << "," << chain[0]->m_c_ident << ",[";
        firstc = false;
        bool firstd = true;
        for (auto* d : chain) {
            out << (firstd ? "" : ",") << "[" << d->m_pos.at(0) << "," << d->m_pos.at(1) << ","
                << d->m_pos.at(2) << "," << d->m_ore.at(0) << "," << d->m_ore.at(1) << ","
                << d->m_ore.at(2) << "," << static_cast<int>(d->m_state) << "]";
            firstd = false;
        }
        out << "]]";
    }
    out << "]";
}

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
            enumerator::enumerate_main(*o, o->get_system_order_params(), o->get_system_biases(), params);
            std::cout << "{\"enumerated\": true}\n";
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
            std::cout << "], \"dumps\": [";
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
