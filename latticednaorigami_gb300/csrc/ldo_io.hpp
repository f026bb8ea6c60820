// Readers for the reference's user-facing input files.
//
//   .inp key=value parameter file  -> Params   (option names and defaults of
//                                               src/parser.cpp:33-449)
//   system JSON                     -> SystemFile (src/files.cpp:36-104)
//   movetype JSON                   -> MoveSpec list (src/files.cpp:264-314)
//   order-parameter JSON            -> OpSpec list, grouped by level
//                                      (src/files.cpp:376-413)
//   bias-function JSON              -> BiasSpec list, grouped by level
//                                      (src/files.cpp:430-482)
//   umbrella .windows file          -> windows (src/us_simulation.cpp:555)
//
// Header-only so that the engine's host library and the test oracle read the
// same files the same way.  Errors are reported through std::runtime_error
// with the reference's messages where it has one.
#pragma once

#include <array>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ldo_io {

using std::string;
using std::vector;

// ---------------------------------------------------------------- JSON ----
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind {Null};
    bool b {false};
    double num {0};
    string str;
    vector<JVal> arr;
    vector<std::pair<string, JVal>> obj;

    bool has(const string& k) const {
        for (auto& kv : obj)
            if (kv.first == k) return true;
        return false;
    }
    const JVal& operator[](const string& k) const {
        static const JVal null_val;
        for (auto& kv : obj)
            if (kv.first == k) return kv.second;
        return null_val;
    }
    const JVal& operator[](size_t i) const {
        static const JVal null_val;
        return i < arr.size() ? arr[i] : null_val;
    }
    size_t size() const { return kind == Arr ? arr.size() : (kind == Obj ? obj.size() : 0); }
    int as_int() const {
        if (kind == Num) return (int)num;
        if (kind == Bool) return b ? 1 : 0;
        if (kind == Str) return std::stoi(str);
        return 0;
    }
    double as_double() const {
        if (kind == Num) return num;
        if (kind == Bool) return b ? 1.0 : 0.0;
        if (kind == Str) return std::stod(str);
        return 0.0;
    }
    bool as_bool() const {
        if (kind == Bool) return b;
        if (kind == Num) return num != 0;
        return false;
    }
    string as_string() const {
        if (kind == Str) return str;
        if (kind == Bool) return b ? "true" : "false";
        if (kind == Num) {
            char buf[64];
            std::snprintf(buf, sizeof buf, "%.17g", num);
            return buf;
        }
        return "";
    }
};

class JParser {
  public:
    explicit JParser(const string& s): m_s(s) {}
    JVal parse() {
        JVal v = value();
        ws();
        if (m_i != m_s.size()) fail("trailing characters");
        return v;
    }

  private:
    const string& m_s;
    size_t m_i {0};
    [[noreturn]] void fail(const string& what) {
        throw std::runtime_error("JSON parse error at offset " + std::to_string(m_i) + ": " + what);
    }
    void ws() {
        while (m_i < m_s.size()) {
            char c = m_s[m_i];
            if (c == ' ' || c == '\t' || c == '\n' || c == '\r') {
                ++m_i;
            }
            else if (c == '/' && m_i + 1 < m_s.size() && m_s[m_i + 1] == '/') {
                while (m_i < m_s.size() && m_s[m_i] != '\n') ++m_i;
            }
            else {
                break;
            }
        }
    }
    JVal value() {
        ws();
        if (m_i >= m_s.size()) fail("unexpected end");
        char c = m_s[m_i];
        JVal v;
        if (c == '{') {
            v.kind = JVal::Obj;
            ++m_i;
            ws();
            if (peek() == '}') {
                ++m_i;
                return v;
            }
            for (;;) {
                ws();
                if (peek() != '"') fail("expected key");
                string k = string_lit();
                ws();
                if (peek() != ':') fail("expected ':'");
                ++m_i;
                JVal x = value();
                v.obj.emplace_back(k, std::move(x));
                ws();
                if (peek() == ',') {
                    ++m_i;
                    continue;
                }
                if (peek() == '}') {
                    ++m_i;
                    break;
                }
                fail("expected ',' or '}'");
            }
        }
        else if (c == '[') {
            v.kind = JVal::Arr;
            ++m_i;
            ws();
            if (peek() == ']') {
                ++m_i;
                return v;
            }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (peek() == ',') {
                    ++m_i;
                    continue;
                }
                if (peek() == ']') {
                    ++m_i;
                    break;
                }
                fail("expected ',' or ']'");
            }
        }
        else if (c == '"') {
            v.kind = JVal::Str;
            v.str = string_lit();
        }
        else if (m_s.compare(m_i, 4, "true") == 0) {
            v.kind = JVal::Bool;
            v.b = true;
            m_i += 4;
        }
        else if (m_s.compare(m_i, 5, "false") == 0) {
            v.kind = JVal::Bool;
            m_i += 5;
        }
        else if (m_s.compare(m_i, 4, "null") == 0) {
            m_i += 4;
        }
        else {
            size_t st = m_i;
            while (m_i < m_s.size() && (std::isdigit((unsigned char)m_s[m_i]) || m_s[m_i] == '-' ||
                                        m_s[m_i] == '+' || m_s[m_i] == '.' || m_s[m_i] == 'e' ||
                                        m_s[m_i] == 'E'))
                ++m_i;
            if (st == m_i) fail("unexpected character");
            v.kind = JVal::Num;
            v.num = std::strtod(m_s.substr(st, m_i - st).c_str(), nullptr);
        }
        return v;
    }
    char peek() const { return m_i < m_s.size() ? m_s[m_i] : '\0'; }
    string string_lit() {
        ++m_i;
        string out;
        while (m_i < m_s.size() && m_s[m_i] != '"') {
            char c = m_s[m_i++];
            if (c == '\\' && m_i < m_s.size()) {
                char e = m_s[m_i++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': m_i += 4; out += '?'; break;
                default: out += e;
                }
            }
            else {
                out += c;
            }
        }
        if (m_i >= m_s.size()) fail("unterminated string");
        ++m_i;
        return out;
    }
};

inline string read_text(const string& fname, const string& what) {
    std::ifstream f(fname, std::ios::binary);
    if (!f) throw std::runtime_error(what + " " + fname + " does not exist");
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

inline JVal read_json(const string& fname, const string& what) {
    string text = read_text(fname, what);
    try {
        return JParser(text).parse();
    } catch (std::exception& e) {
        throw std::runtime_error(what + " " + fname + " is not well formed:\n" + e.what());
    }
}

// --------------------------------------------------------------- .inp ----
// Option names and defaults follow src/parser.cpp:33-449.
struct Params {
    string origami_input_filename;
    string domain_type {"Halfturn"};
    string binding_pot {"FourBody"};
    string misbinding_pot {"Opposing"};
    string stacking_pot {"Constant"};
    string hybridization_pot {"NearestNeighbour"};
    bool apply_mean_field_cor {false};
    double temp {300};
    double staple_M {1};
    double cation_M {1};
    double staple_u_mult {1};
    double stacking_ene {1};
    double binding_h {0};
    double binding_s {0};
    double misbinding_h {0};
    double misbinding_s {0};
    int min_total_staples {0};
    int max_total_staples {999};
    int max_type_staples {999};
    int max_staple_size {2};
    bool domain_update_biases_present {false};
    string order_parameter_file;
    string bias_functions_file;
    double bias_functions_mult {1};
    string simulation_type {"constant_temp"};
    bool enumerate_staples_only {false};
    long long random_seed {-1};
    string movetype_file;
    string restart_traj_file;
    int restart_step {0};
    int centering_freq {0};
    int centering_domain {0};
    int constraint_check_freq {0};
    bool allow_nonsensical_ps {false};
    double max_duration {10e9};
    long long ct_steps {0};
    bool constant_staple_M {true};
    double max_temp {400};
    double min_temp {300};
    double temp_interval {1};
    long long steps_per_temp {0};
    vector<double> temps;
    int num_reps {1};
    long long swaps {0};
    double max_pt_dur {10e9};
    int exchange_interval {0};
    vector<double> chem_pot_mults;
    vector<double> bias_mults;
    vector<double> stacking_mults;
    string us_grid_bias_tag;
    int max_num_iters {0};
    double max_D_bias {0};
    long long equil_steps {0};
    long long iter_steps {0};
    long long iter_swaps {0};
    double max_rel_P_diff {0.1};
    bool multi_window {false};
    string windows_file;
    // umbrella-sampling restart (USGCMCSimulation constructor,
    // src/us_simulation.cpp:48-87): grid biases read from .biases files
    bool read_biases {false};
    string biases_file;
    string biases_filebase;
    string output_filebase;
    int logging_freq {0};
    int configs_output_freq {0};
    int counts_output_freq {0};
    int energies_output_freq {0};
    int order_params_output_freq {0};
    vector<string> ops_to_output;
    // Keys the engine adds for batching; the reference has no such options.
    std::map<string, string> extra;
    // Directory of the .inp file: relative file names resolve against it.
    string base_dir;
};

inline string trim(const string& s) {
    size_t a = s.find_first_not_of(" \t\r\n");
    size_t b = s.find_last_not_of(" \t\r\n");
    return a == string::npos ? string() : s.substr(a, b - a + 1);
}

inline vector<string> split_ws(const string& s) {
    std::istringstream is(s);
    vector<string> out;
    string t;
    while (is >> t) out.push_back(t);
    return out;
}

inline vector<double> split_doubles(const string& s) {
    vector<double> out;
    for (auto& t : split_ws(s)) out.push_back(std::stod(t));
    return out;
}

inline bool parse_bool(const string& v) {
    if (v == "true" || v == "1" || v == "yes" || v == "on") return true;
    if (v == "false" || v == "0" || v == "no" || v == "off") return false;
    throw std::runtime_error("invalid boolean value: " + v);
}

inline void set_param(Params& p, const string& k, const string& v) {
    auto D = [&]() { return std::stod(v); };
    auto I = [&]() { return (int)std::stoll(v); };
    auto L = [&]() { return std::stoll(v); };
    if (k == "origami_input_filename") p.origami_input_filename = v;
    else if (k == "domain_type") p.domain_type = v;
    else if (k == "binding_pot") p.binding_pot = v;
    else if (k == "misbinding_pot") p.misbinding_pot = v;
    else if (k == "stacking_pot") p.stacking_pot = v;
    else if (k == "hybridization_pot") p.hybridization_pot = v;
    else if (k == "apply_mean_field_cor") p.apply_mean_field_cor = parse_bool(v);
    else if (k == "temp") p.temp = D();
    else if (k == "staple_M") p.staple_M = D();
    else if (k == "cation_M") p.cation_M = D();
    else if (k == "staple_u_mult") p.staple_u_mult = D();
    else if (k == "stacking_ene") p.stacking_ene = D();
    else if (k == "binding_h") p.binding_h = D();
    else if (k == "binding_s") p.binding_s = D();
    else if (k == "misbinding_h") p.misbinding_h = D();
    else if (k == "misbinding_s") p.misbinding_s = D();
    else if (k == "min_total_staples") p.min_total_staples = I();
    else if (k == "max_total_staples") p.max_total_staples = I();
    else if (k == "max_type_staples") p.max_type_staples = I();
    else if (k == "max_staple_size") p.max_staple_size = I();
    else if (k == "domain_update_biases_present") p.domain_update_biases_present = parse_bool(v);
    else if (k == "order_parameter_file") p.order_parameter_file = v;
    else if (k == "bias_functions_file") p.bias_functions_file = v;
    else if (k == "bias_functions_mult") p.bias_functions_mult = D();
    else if (k == "simulation_type") p.simulation_type = v;
    else if (k == "enumerate_staples_only") p.enumerate_staples_only = parse_bool(v);
    else if (k == "random_seed") p.random_seed = L();
    else if (k == "movetype_file") p.movetype_file = v;
    else if (k == "restart_traj_file") p.restart_traj_file = v;
    else if (k == "restart_step") p.restart_step = I();
    else if (k == "centering_freq") p.centering_freq = I();
    else if (k == "centering_domain") p.centering_domain = I();
    else if (k == "constraint_check_freq") p.constraint_check_freq = I();
    else if (k == "allow_nonsensical_ps") p.allow_nonsensical_ps = parse_bool(v);
    else if (k == "max_duration") p.max_duration = D();
    else if (k == "ct_steps") p.ct_steps = L();
    else if (k == "constant_staple_M") p.constant_staple_M = parse_bool(v);
    else if (k == "max_temp") p.max_temp = D();
    else if (k == "min_temp") p.min_temp = D();
    else if (k == "temp_interval") p.temp_interval = D();
    else if (k == "steps_per_temp") p.steps_per_temp = L();
    else if (k == "temps") p.temps = split_doubles(v);
    else if (k == "num_reps") p.num_reps = I();
    else if (k == "swaps") p.swaps = L();
    else if (k == "max_pt_dur") p.max_pt_dur = D();
    else if (k == "exchange_interval") p.exchange_interval = I();
    else if (k == "chem_pot_mults") p.chem_pot_mults = split_doubles(v);
    else if (k == "bias_mults") p.bias_mults = split_doubles(v);
    else if (k == "stacking_mults") p.stacking_mults = split_doubles(v);
    else if (k == "us_grid_bias_tag") p.us_grid_bias_tag = v;
    else if (k == "max_num_iters") p.max_num_iters = I();
    else if (k == "max_D_bias") p.max_D_bias = D();
    else if (k == "equil_steps") p.equil_steps = L();
    else if (k == "iter_steps") p.iter_steps = L();
    else if (k == "iter_swaps") p.iter_swaps = L();
    else if (k == "max_rel_P_diff") p.max_rel_P_diff = D();
    else if (k == "multi_window") p.multi_window = parse_bool(v);
    else if (k == "windows_file") p.windows_file = v;
    else if (k == "read_biases") p.read_biases = parse_bool(v);
    else if (k == "biases_file") p.biases_file = v;
    else if (k == "biases_filebase") p.biases_filebase = v;
    else if (k == "output_filebase") p.output_filebase = v;
    else if (k == "logging_freq") p.logging_freq = I();
    else if (k == "configs_output_freq") p.configs_output_freq = I();
    else if (k == "counts_output_freq") p.counts_output_freq = I();
    else if (k == "energies_output_freq") p.energies_output_freq = I();
    else if (k == "order_params_output_freq") p.order_params_output_freq = I();
    else if (k == "ops_to_output") p.ops_to_output = split_ws(v);
    else p.extra[k] = v;
}

// Parses key=value lines ('#' starts a comment), like Boost's config-file
// reader used by src/parser.cpp:476-479.
inline Params parse_inp_text(const string& text, const string& base_dir = "") {
    Params p;
    p.base_dir = base_dir;
    std::istringstream is(text);
    string line;
    int lineno = 0;
    while (std::getline(is, line)) {
        ++lineno;
        auto h = line.find('#');
        if (h != string::npos) line = line.substr(0, h);
        line = trim(line);
        if (line.empty()) continue;
        auto eq = line.find('=');
        if (eq == string::npos)
            throw std::runtime_error("parameter file line " + std::to_string(lineno) + ": expected key=value");
        string k = trim(line.substr(0, eq));
        string v = trim(line.substr(eq + 1));
        try {
            set_param(p, k, v);
        } catch (std::invalid_argument&) {
            throw std::runtime_error("parameter " + k + ": invalid value '" + v + "'");
        } catch (std::out_of_range&) {
            throw std::runtime_error("parameter " + k + ": value out of range '" + v + "'");
        }
    }
    return p;
}

inline string dir_of(const string& path) {
    auto s = path.find_last_of('/');
    return s == string::npos ? string() : path.substr(0, s + 1);
}

inline bool file_exists(const string& f) {
    std::ifstream in(f);
    return (bool)in;
}

inline string resolve(const Params& p, const string& f) {
    if (f.empty() || f[0] == '/' || p.base_dir.empty()) return f;
    return p.base_dir + f;
}

inline Params read_inp(const string& fname) {
    return parse_inp_text(read_text(fname, "Parameter file"), dir_of(fname));
}

// -------------------------------------------------------- system JSON ----
struct ChainConf {
    int index {0};
    int identity {0};
    vector<std::array<int, 3>> positions;
    vector<std::array<int, 3>> orientations;
};

struct SystemFile {
    vector<vector<int>> identities;
    vector<vector<string>> sequences;
    vector<double> enthalpies;
    vector<double> entropies;
    vector<ChainConf> chains;
    bool cyclic {false};
};

inline SystemFile system_from_json(const JVal& root) {
    SystemFile s;
    const JVal& o = root["origami"];
    if (o.has("sequences")) {
        const JVal& seqs = o["sequences"];
        for (size_t i = 0; i < seqs.size(); ++i) {
            s.sequences.push_back({});
            for (size_t j = 0; j < seqs[i].size(); ++j) s.sequences[i].push_back(seqs[i][j].as_string());
        }
    }
    if (o.has("enthalpies"))
        for (size_t i = 0; i < o["enthalpies"].size(); ++i) s.enthalpies.push_back(o["enthalpies"][i].as_double());
    if (o.has("entropies"))
        for (size_t i = 0; i < o["entropies"].size(); ++i) s.entropies.push_back(o["entropies"][i].as_double());
    const JVal& idents = o["identities"];
    for (size_t i = 0; i < idents.size(); ++i) {
        s.identities.push_back({});
        for (size_t j = 0; j < idents[i].size(); ++j) s.identities[i].push_back(idents[i][j].as_int());
    }
    const JVal& chains = o["configurations"][0]["chains"];
    for (size_t i = 0; i < chains.size(); ++i) {
        const JVal& c = chains[i];
        ChainConf cc;
        cc.index = c["index"].as_int();
        cc.identity = c["identity"].as_int();
        for (size_t j = 0; j < c["positions"].size(); ++j) {
            cc.positions.push_back({c["positions"][j][0].as_int(), c["positions"][j][1].as_int(),
                                    c["positions"][j][2].as_int()});
            cc.orientations.push_back({c["orientations"][j][0].as_int(), c["orientations"][j][1].as_int(),
                                       c["orientations"][j][2].as_int()});
        }
        s.chains.push_back(cc);
    }
    s.cyclic = o["cyclic"].as_bool();
    return s;
}

inline SystemFile read_system(const string& fname) {
    return system_from_json(read_json(fname, "Origami input file"));
}

// ------------------------------------------------------ trajectory ----
// Configuration of frame `frame` (0 = the first configuration written) of a
// .trj file (OrigamiTrajInputFile::read_config, src/files.cpp:129-189): frames
// are separated by an empty line; a frame is its step line, then per chain a
// line "index identity", a line of x y z triples and a line of orientation
// triples.  The reference's reader appends one (0, 0, 0) triple for the
// trailing space of each line, which its constructor never reads (it takes
// as many triples as the chain's identity has domains); this reader keeps
// every whole triple and leaves the length check to the caller.
inline vector<ChainConf> read_trj_frame(const string& fname, int frame) {
    std::ifstream f(fname);
    if (!f) throw std::runtime_error("Trajectory input file " + fname + " does not exist");
    if (frame < 0) throw std::runtime_error("restart_step must not be negative");
    string line;
    // OrigamiTrajInputFile::go_to_step (src/files.cpp:191): skip `frame` frames
    for (int i = 0; i < frame; ++i) {
        while (true) {
            bool got = (bool)std::getline(f, line);
            if (!got || f.eof())
                throw std::runtime_error("Step " + std::to_string(frame) + " not found in trajectory input file" +
                                         fname);
            if (line.empty()) break;
        }
    }
    if (!std::getline(f, line)) throw std::runtime_error("Step " + std::to_string(frame) +
                                                         " not found in trajectory input file" + fname);
    auto triples = [&](const string& s) {
        std::istringstream is(s);
        vector<std::array<int, 3>> v;
        long long a, b, c;
        while (is >> a >> b >> c) v.push_back({(int)a, (int)b, (int)c});
        return v;
    };
    vector<ChainConf> chains;
    while (std::getline(f, line) && !line.empty()) {
        std::istringstream id(line);
        ChainConf cc;
        if (!(id >> cc.index >> cc.identity))
            throw std::runtime_error("Trajetory input file " + fname + " is not well formed: chain line '" + line +
                                     "'");
        string pos, ore;
        std::getline(f, pos);
        std::getline(f, ore);
        cc.positions = triples(pos);
        cc.orientations = triples(ore);
        if (cc.positions.size() != cc.orientations.size())
            throw std::runtime_error("Trajetory input file " + fname +
                                     " is not well formed: positions and orientations differ in number");
        chains.push_back(cc);
    }
    if (chains.empty())
        throw std::runtime_error("Trajetory input file " + fname + " is not well formed: frame " +
                                 std::to_string(frame) + " has no chains");
    return chains;
}

// ------------------------------------------------------ movetype JSON ----
struct MoveSpec {
    string type;
    string label;
    double freq {0};
    vector<double> exchange_mults;
    bool adaptive_exchange {false};
    int max_regrowth {0};
    int max_seg_regrowth {0};
    int max_num_recoils {0};
    int max_c_attempts {0};
    int max_disp {0};
    int max_turns {0};
    int max_linker_length {0};
    int num_transforms {0};
};

// utility::Fraction (src/utility.cpp:266): "a/b" or a plain real number.
inline double parse_fraction(const string& s) {
    auto d = s.find('/');
    if (d == string::npos) return std::stod(s);
    double num = std::stod(s.substr(0, d));
    double den = std::stod(s.substr(d + 1));
    return num / den;
}

inline vector<MoveSpec> movetypes_from_json(const JVal& root) {
    vector<MoveSpec> out;
    const JVal& mts = root["origami"]["movetypes"];
    for (size_t i = 0; i < mts.size(); ++i) {
        const JVal& m = mts[i];
        MoveSpec ms;
        ms.type = m["type"].as_string();
        ms.label = m["label"].as_string();
        ms.freq = parse_fraction(m["freq"].as_string());
        for (size_t j = 0; j < m["exchange_mults"].size(); ++j)
            ms.exchange_mults.push_back(m["exchange_mults"][j].as_double());
        ms.adaptive_exchange = m["adaptive_exchange"].as_bool();
        ms.max_regrowth = m["max_regrowth"].as_int();
        ms.max_seg_regrowth = m["max_seg_regrowth"].as_int();
        ms.max_num_recoils = m["max_num_recoils"].as_int();
        ms.max_c_attempts = m["max_c_attempts"].as_int();
        ms.max_disp = m["max_disp"].as_int();
        ms.max_turns = m["max_turns"].as_int();
        ms.max_linker_length = m["max_linker_length"].as_int();
        ms.num_transforms = m["num_transforms"].as_int();
        out.push_back(ms);
    }
    return out;
}

inline vector<MoveSpec> read_movetypes(const string& fname) {
    return movetypes_from_json(read_json(fname, "Move type file"));
}

// ------------------------------------------- order parameter JSON ----
struct OpSpec {
    string type, label, tag;
    int level {0};
    int staple {0};                 // NumStaplesType / StapleTypeFullyBound
    int chain1 {0}, domain1 {0}, chain2 {0}, domain2 {0};  // Dist / AdjacentSite
    bool update_per_domain {false};
    vector<string> ops;             // Sum
};

// Returns the specs in level-major order, i.e. the order in which
// SystemOrderParams::setup_ops (src/order_params.cpp:471) creates them.
inline vector<OpSpec> ops_from_json(const JVal& root) {
    const JVal& arr = root["origami"]["order_params"];
    vector<OpSpec> all;
    int max_level = 0;
    for (size_t i = 0; i < arr.size(); ++i) {
        const JVal& j = arr[i];
        OpSpec s;
        s.type = j["type"].as_string();
        s.label = j["label"].as_string();
        s.tag = j["tag"].as_string();
        s.level = j["level"].as_int();
        s.staple = j["staple"].as_int();
        s.chain1 = j["chain1"].as_int();
        s.domain1 = j["domain1"].as_int();
        s.chain2 = j["chain2"].as_int();
        s.domain2 = j["domain2"].as_int();
        s.update_per_domain = j["update_per_domain"].as_bool();
        for (size_t k = 0; k < j["ops"].size(); ++k) s.ops.push_back(j["ops"][k].as_string());
        if (s.level > max_level) max_level = s.level;
        all.push_back(s);
    }
    vector<OpSpec> out;
    for (int l = 0; l <= max_level; ++l)
        for (auto& s : all)
            if (s.level == l) out.push_back(s);
    return out;
}

inline vector<OpSpec> read_ops(const string& fname) {
    return ops_from_json(read_json(fname, "Order parameter file"));
}

// --------------------------------------------- bias function JSON ----
struct BiasSpec {
    string type, label, tag;
    int level {0};
    vector<string> ops;
    vector<string> bias_funcs;
    int min_op {0}, max_op {0};
    double max_bias {0}, well_bias {0}, min_bias {0}, slope {0}, outside_bias {0};
    // Engine extension "Harmonic": bias = 0.5 * k * (op - centre)^2
    double k {0}, centre {0};
};

inline vector<BiasSpec> biases_from_json(const JVal& root) {
    const JVal& arr = root["origami"]["bias_functions"];
    vector<BiasSpec> all;
    int max_level = 0;
    for (size_t i = 0; i < arr.size(); ++i) {
        const JVal& j = arr[i];
        BiasSpec s;
        s.type = j["type"].as_string();
        s.label = j["label"].as_string();
        s.tag = j["tag"].as_string();
        s.level = j["level"].as_int();
        for (size_t k = 0; k < j["ops"].size(); ++k) s.ops.push_back(j["ops"][k].as_string());
        s.bias_funcs = split_ws(j["bias_funcs"].as_string());
        s.min_op = j["min_op"].as_int();
        s.max_op = j["max_op"].as_int();
        s.max_bias = j["max_bias"].as_double();
        s.well_bias = j["well_bias"].as_double();
        s.min_bias = j["min_bias"].as_double();
        s.slope = j["slope"].as_double();
        s.outside_bias = j["outside_bias"].as_double();
        s.k = j["k"].as_double();
        s.centre = j["centre"].as_double();
        if (s.level > max_level) max_level = s.level;
        all.push_back(s);
    }
    vector<BiasSpec> out;
    for (int l = 0; l <= max_level; ++l)
        for (auto& s : all)
            if (s.level == l) out.push_back(s);
    return out;
}

inline vector<BiasSpec> read_biases(const string& fname) {
    return biases_from_json(read_json(fname, "Bias functions file"));
}

// --------------------------------------------------- .windows file ----
// First line: tag of the square-well bias; then one "min, max" tuple pair per
// window (src/us_simulation.cpp:555-601, 1-D order parameters).
struct Windows {
    string bias_tag;
    vector<std::pair<int, int>> bounds;
};

inline Windows read_windows(const string& fname) {
    string text = read_text(fname, "Windows file");
    std::istringstream is(text);
    Windows w;
    string line;
    bool first = true;
    while (std::getline(is, line)) {
        line = trim(line);
        if (line.empty()) continue;
        if (first) {
            w.bias_tag = line;
            first = false;
            continue;
        }
        for (auto& c : line)
            if (c == ',' || c == '(' || c == ')') c = ' ';
        auto t = split_ws(line);
        if (t.size() < 2) throw std::runtime_error("Windows file " + fname + ": malformed window line");
        w.bounds.push_back({std::stoi(t[0]), std::stoi(t[1])});
    }
    return w;
}

// ------------------------------------------------------ .biases files ----
// Grid biases of an umbrella-sampling window: {"biases": [{"point": [..],
// "bias": x}, ..]}, read by USGCMCSimulation::read_weights
// (src/us_simulation.cpp:192) and written by output_weights (:208).
struct GridBias {
    vector<int> point;
    double bias;
};

inline vector<GridBias> read_biases_json(const string& fname) {
    JVal root = read_json(fname, "Restart bias file");
    const JVal& arr = root["biases"];
    if (arr.kind != JVal::Arr) throw std::runtime_error("Restart bias file " + fname + " has no biases array");
    vector<GridBias> out;
    for (size_t i = 0; i < arr.size(); ++i) {
        const JVal& e = arr[i];
        GridBias g;
        for (size_t j = 0; j < e["point"].size(); ++j) g.point.push_back(e["point"][j].as_int());
        if (g.point.empty()) throw std::runtime_error("Restart bias file " + fname + ": an entry has no point");
        g.bias = e["bias"].as_double();
        out.push_back(g);
    }
    return out;
}

// output_weights' layout: one entry per grid point, each bias printed by
// std::to_string (six decimals), no trailing comma.
inline string biases_json_text(const vector<GridBias>& entries) {
    std::ostringstream os;
    os << "{\n";
    os << "    \"biases\": [";
    for (size_t i = 0; i < entries.size(); ++i) {
        os << (i == 0 ? "\n" : ",\n");
        const auto& g = entries[i];
        os << "        {\n";
        os << "            \"point\": [\n";
        for (size_t j = 0; j + 1 < g.point.size(); ++j) os << "                " << std::to_string(g.point[j]) << ",\n";
        os << "                " << std::to_string(g.point.back()) << "\n";
        os << "            ],\n";
        os << "            \"bias\": " << std::to_string(g.bias) << "\n";
        os << "        }";
    }
    os << "\n    ]\n";
    os << "}\n";
    return os.str();
}

// MWUSGCMCSimulation::setup_window_variables (src/us_simulation.cpp:487):
// the file-name postfix of a window, "_win-" + each min + "-", then "-" +
// each max (a 1-D window 0..8 gives "_win-0--8").
inline string window_postfix(const vector<int>& mins, const vector<int>& maxs) {
    string s = "_win-";
    for (int j : mins) s += std::to_string(j) + "-";
    for (int j : maxs) s += "-" + std::to_string(j);
    return s;
}

} // namespace ldo_io
