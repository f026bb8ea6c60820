// Helpers shared by the drivers around the reference build (ref_trace.cpp,
// ref_exchange.cpp): the reference's key=value parameter files read into
// parser::InputParameters through its test constructor, with the defaults of
// src/parser.cpp:33-449, and a JSON dump of a configuration.
#pragma once
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "LatticeDNAOrigami/origami_system.hpp"
#include "LatticeDNAOrigami/parser.hpp"

namespace ldo_refdrv {

using std::string;
using std::vector;

inline std::map<string, string> read_kv(const string& fname) {
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

inline vector<string> split_ws(const string& s) {
    std::istringstream is(s);
    vector<string> out;
    string t;
    while (is >> t) out.push_back(t);
    return out;
}

// Defaults are those of src/parser.cpp:33-449.
inline void fill_params(parser::InputParameters& p, std::map<string, string>& kv) {
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
    p.m_output_filebase = S("output_filebase", "ref_trace_out");
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

inline void dump_config(origami::OrigamiSystem& o, std::ostream& out) {
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

} // namespace ldo_refdrv
