// Oracle (test infrastructure only): energy tables.
//
// CPU restatement of the reference's table builder, used to check the engine:
//   - SantaLucia 2004 nearest-neighbour thermodynamics
//     (src/nearest_neighbour.cpp:34-115, tables include/.../nearest_neighbour.hpp:32-92)
//   - longest contiguous complement search (src/nearest_neighbour.cpp:117-160)
//   - per identity-pair hybridisation / stacking tables
//     (OrigamiPotential::calc_energies and helpers, src/origami_potential.cpp:1057-1221)
// Arithmetic is done in the reference's order so table entries agree bit for bit.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle {

using std::string;
using std::vector;

constexpr double kGasR = 8.3144598;
constexpr double kJoulePerCal = 4.184;

inline int base_index(char b) {
    switch (b) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    }
    throw std::runtime_error(string("invalid base ") + b);
}

inline char complement(char b) {
    switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'G': return 'C';
    case 'C': return 'G';
    }
    throw std::runtime_error(string("invalid base ") + b);
}

inline string complement_seq(const string& s) {
    string o;
    for (char c : s) o += complement(c);
    return o;
}

// Nearest-neighbour stack "XY/X'Y'" is determined by the top dinucleotide XY.
// kcal/mol and kcal/mol/K, SantaLucia & Hicks 2004.
inline void nn_stack(char x, char y, double& dh, double& ds) {
    static const double H[4][4] = {
        // A      C      G      T     (second base)
        {-7.6, -8.4, -7.8, -7.2},   // A
        {-8.5, -8.0, -10.6, -7.8},  // C
        {-8.2, -9.8, -8.0, -8.4},   // G
        {-7.2, -8.2, -8.5, -7.6}};  // T
    static const double S[4][4] = {
        {-0.0213, -0.0224, -0.0210, -0.0204},
        {-0.0227, -0.0199, -0.0272, -0.0210},
        {-0.0222, -0.0244, -0.0199, -0.0224},
        {-0.0213, -0.0222, -0.0227, -0.0213}};
    dh = H[base_index(x)][base_index(y)];
    ds = S[base_index(x)][base_index(y)];
}

// Kilchherr 2016 stacking free energies, kcal/mol, by dinucleotide XY.
inline double stack_free_energy(char x, char y) {
    static const double G[4][4] = {
        {-1.36, -2.03, -1.60, -2.35},
        {-0.81, -1.64, -2.06, -1.39},
        {-1.39, -3.42, -1.64, -0.81},
        {-1.01, -1.60, -2.03, -1.36}};
    return G[base_index(x)][base_index(y)];
}

constexpr double kInitH = 0.2;
constexpr double kInitS = -0.0057;
constexpr double kTerminalAtH = 2.2;
constexpr double kTerminalAtS = 0.0069;
constexpr double kSymmetryS = -0.0014;

struct Thermo {
    double h;
    double s;
};

inline bool palindromic(const string& s) {
    string rc = complement_seq(s);
    string r(rc.rbegin(), rc.rend());
    return r == s;
}

inline Thermo hybrid_h_and_s(const string& seq, double cation_M) {
    double dh_init = kInitH;
    double ds_init = kInitS;
    double ds_sym = palindromic(seq) ? kSymmetryS : 0.0;
    double dh_stack = 0, ds_stack = 0;
    for (size_t i = 0; i + 1 < seq.size(); ++i) {
        double h, s;
        nn_stack(seq[i], seq[i + 1], h, s);
        dh_stack += h;
        ds_stack += s;
    }
    int at = 0;
    if (seq.front() == 'A' || seq.front() == 'T') at += 1;
    if (seq.back() == 'A' || seq.back() == 'T') at += 1;
    double dh_at = kTerminalAtH * at;
    double ds_at = kTerminalAtS * at;
    double dh = dh_init + dh_stack + dh_at;
    double ds = ds_init + ds_sym + ds_stack + ds_at;
    ds += 0.368 * seq.size() * std::log(cation_M) / 1000;
    return {dh, ds};
}

inline Thermo unitless_hybrid(const string& seq, double temp, double cation_M) {
    Thermo t = hybrid_h_and_s(seq, cation_M);
    t.h = t.h * kJoulePerCal * 1000 / kGasR / temp;
    t.s = t.s * kJoulePerCal * 1000 / kGasR;
    return t;
}

inline Thermo unitless_init(double temp) {
    Thermo t {kInitH, kInitS};
    t.h = t.h * kJoulePerCal * 1000 / kGasR / temp;
    t.s = t.s * kJoulePerCal * 1000 / kGasR;
    return t;
}

// All longest substrings of seq_i that pair with seq_j, with multiplicity.
inline vector<string> longest_complements(const string& seq_i, const string& seq_j) {
    string three, five;
    if (seq_i.size() <= seq_j.size()) {
        three.assign(seq_j.rbegin(), seq_j.rend());
        five = seq_i;
    }
    else {
        three.assign(seq_i.rbegin(), seq_i.rend());
        five = seq_j;
    }
    three = complement_seq(three);
    vector<string> found;
    for (int len = (int)three.size(); len != 0; --len) {
        for (size_t st = 0; st + len <= three.size(); ++st) {
            string sub = three.substr(st, len);
            size_t at = five.find(sub);
            while (at != string::npos) {
                found.push_back(sub);
                at = five.find(sub, at + 1);
            }
        }
        if (!found.empty()) return found;
    }
    return found;
}

struct EnergyModel {
    string hybridization_pot;   // NearestNeighbour | Uniform | Specified
    string stacking_pot;        // Constant | SequenceSpecific
    bool mean_field {false};
    double temp {300};
    double cation_M {1};
    double stacking_ene {1};
    double stacking_mult {1};
    double binding_h {0}, binding_s {0}, misbinding_h {0}, misbinding_s {0};
    vector<double> enthalpies, entropies;
};

// Dense tables over identity pairs (i, j), i, j in [-imax, imax].
struct EnergyTables {
    int imax {0};
    int dim {1};
    vector<double> hyb_e, hyb_h, hyb_s, stack_e;
    double init_h {0}, init_s {0}, init_e {0};
    size_t at(int a, int b) const { return (size_t)(a + imax) * dim + (size_t)(b + imax); }
};

inline EnergyTables build_tables(const vector<vector<int>>& idents, const vector<vector<string>>& seqs,
                                 const EnergyModel& m) {
    EnergyTables t;
    for (auto& c : idents)
        for (int x : c) t.imax = std::max(t.imax, std::abs(x));
    t.dim = 2 * t.imax + 1;
    size_t n = (size_t)t.dim * t.dim;
    t.hyb_e.assign(n, 0.0);
    t.hyb_h.assign(n, 0.0);
    t.hyb_s.assign(n, 0.0);
    t.stack_e.assign(n, 0.0);
    Thermo init = unitless_init(m.temp);
    t.init_h = init.h;
    t.init_s = init.s;
    t.init_e = init.h - init.s;
    // Constant stacking uses the multiplied energy (OrigamiPotential::update_temp,
    // src/origami_potential.cpp:1019-1035).
    double stack_ene = m.stacking_ene * m.stacking_mult;
    for (size_t ci = 0; ci < idents.size(); ++ci) {
        for (size_t cj = 0; cj < idents.size(); ++cj) {
            for (size_t di = 0; di < idents[ci].size(); ++di) {
                for (size_t dj = 0; dj < idents[cj].size(); ++dj) {
                    int a = idents[ci][di];
                    int b = idents[cj][dj];
                    double H = 0, S = 0;
                    if (m.hybridization_pot == "NearestNeighbour") {
                        const string& si = seqs.at(ci).at(di);
                        const string& sj = seqs.at(cj).at(dj);
                        vector<string> comps = longest_complements(si, sj);
                        if (!comps.empty()) {
                            int N = 0;
                            for (auto& c : comps) {
                                Thermo th = unitless_hybrid(c, m.temp, m.cation_M);
                                H += th.h - init.h;
                                S += th.s - init.s;
                                ++N;
                            }
                            H /= N;
                            S /= N;
                            S += std::log(6);
                            if (a == -b) {
                                if (m.mean_field) S += 3 * std::log(6);
                                if (comps[0].size() != si.size() && si.size() == sj.size())
                                    throw std::runtime_error("Sequences that should be complementary are not: \n" + si +
                                                             "\n" + sj);
                            }
                            else if (comps[0].size() == si.size() && si.size() == sj.size()) {
                                throw std::runtime_error("Sequences that should not be complementary are: \n" + si +
                                                         "\n" + sj);
                            }
                        }
                    }
                    else if (m.hybridization_pot == "Uniform" || m.hybridization_pot == "Specified") {
                        if (a == -b) {
                            if (m.hybridization_pot == "Uniform") {
                                H = m.binding_h / m.temp;
                                S = m.binding_s;
                            }
                            else {
                                int i = std::abs(a) - 1;
                                H = m.enthalpies.at(i) / m.temp;
                                S = m.entropies.at(i);
                            }
                            if (m.mean_field) S += 3 * std::log(6);
                        }
                        else {
                            H = m.misbinding_h / m.temp;
                            S = m.misbinding_s;
                        }
                        S += std::log(6);
                    }
                    else {
                        throw std::runtime_error(m.stacking_pot + ": No such hybridization potential");
                    }
                    size_t k = t.at(a, b);
                    t.hyb_h[k] = H;
                    t.hyb_s[k] = S;
                    t.hyb_e[k] = H - S;
                    if (m.stacking_pot == "SequenceSpecific") {
                        const string& si = seqs.at(ci).at(di);
                        const string& sj = seqs.at(cj).at(dj);
                        t.stack_e[k] = stack_free_energy(si.back(), sj.front());
                    }
                    else if (m.stacking_pot == "Constant") {
                        t.stack_e[k] = stack_ene / m.temp;
                    }
                    else {
                        throw std::runtime_error(m.stacking_pot + ": No such stacking potential");
                    }
                }
            }
        }
    }
    return t;
}

} // namespace oracle
