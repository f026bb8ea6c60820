// Energy tables for the engine, built on the host once per (temperature,
// stacking multiplier) the way OrigamiPotential::calc_energies does
// (src/origami_potential.cpp:1057-1221) with the nearest-neighbour model of
// src/nearest_neighbour.cpp:34-160 (SantaLucia 2004; Kilchherr 2016 stacking).
// Every sum is formed in the reference's order so each entry is bit-identical.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

namespace ldo_host {

using std::string;
using std::vector;

struct NNParams {
    // Dinucleotide XY on the top strand; index 4*X+Y with A,C,G,T = 0..3.
    double dh[16], ds[16], stack_g[16];
    double init_h, init_s, term_at_h, term_at_s, sym_s;
    NNParams() {
        const double h[16] = {-7.6, -8.4, -7.8, -7.2, -8.5, -8.0, -10.6, -7.8,
                              -8.2, -9.8, -8.0, -8.4, -7.2, -8.2, -8.5, -7.6};
        const double s[16] = {-0.0213, -0.0224, -0.0210, -0.0204, -0.0227, -0.0199, -0.0272, -0.0210,
                              -0.0222, -0.0244, -0.0199, -0.0224, -0.0213, -0.0222, -0.0227, -0.0213};
        const double g[16] = {-1.36, -2.03, -1.60, -2.35, -0.81, -1.64, -2.06, -1.39,
                              -1.39, -3.42, -1.64, -0.81, -1.01, -1.60, -2.03, -1.36};
        for (int k = 0; k < 16; ++k) {
            dh[k] = h[k];
            ds[k] = s[k];
            stack_g[k] = g[k];
        }
        init_h = 0.2;
        init_s = -0.0057;
        term_at_h = 2.2;
        term_at_s = 0.0069;
        sym_s = -0.0014;
    }
};

inline int nuc(char b) {
    switch (b) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    }
    throw std::runtime_error(string("invalid nucleotide '") + b + "'");
}
inline char comp_nuc(char b) { return "TGCA"[nuc(b)]; }
inline string comp_strand(const string& s) {
    string o(s.size(), ' ');
    for (size_t i = 0; i < s.size(); ++i) o[i] = comp_nuc(s[i]);
    return o;
}

struct HS {
    double h, s;
};

// calc_hybridization_H_and_S (src/nearest_neighbour.cpp:66), kcal/mol(/K)
inline HS duplex_hs(const NNParams& P, const string& seq, double cation_M) {
    string rc = comp_strand(seq);
    string rrc(rc.rbegin(), rc.rend());
    double ds_sym = (rrc == seq) ? P.sym_s : 0.0;
    double h_st = 0, s_st = 0;
    for (size_t i = 0; i + 1 < seq.size(); ++i) {
        int k = 4 * nuc(seq[i]) + nuc(seq[i + 1]);
        h_st += P.dh[k];
        s_st += P.ds[k];
    }
    int n_at = (seq.front() == 'A' || seq.front() == 'T') + (seq.back() == 'A' || seq.back() == 'T');
    double h_at = P.term_at_h * n_at;
    double s_at = P.term_at_s * n_at;
    HS r;
    r.h = P.init_h + h_st + h_at;
    r.s = P.init_s + ds_sym + s_st + s_at;
    r.s += 0.368 * seq.size() * std::log(cation_M) / 1000;
    return r;
}

constexpr double kR = 8.3144598;
constexpr double kCal = 4.184;

// Reduced units: H / (R T) and S / R.
inline HS reduce(HS x, double temp) {
    x.h = x.h * kCal * 1000 / kR / temp;
    x.s = x.s * kCal * 1000 / kR;
    return x;
}

// find_longest_contig_complement (src/nearest_neighbour.cpp:117)
inline vector<string> longest_pairing(const string& a, const string& b) {
    const string& longer = a.size() <= b.size() ? b : a;
    const string& shorter = a.size() <= b.size() ? a : b;
    string three = comp_strand(string(longer.rbegin(), longer.rend()));
    vector<string> out;
    for (size_t len = three.size(); len > 0; --len) {
        for (size_t st = 0; st + len <= three.size(); ++st) {
            string sub = three.substr(st, len);
            for (size_t at = shorter.find(sub); at != string::npos; at = shorter.find(sub, at + 1)) out.push_back(sub);
        }
        if (!out.empty()) break;
    }
    return out;
}

struct EnergyInputs {
    string hybridization_pot, stacking_pot;
    bool mean_field {false};
    double temp {300}, cation_M {1}, stacking_ene {1}, stacking_mult {1};
    double binding_h {0}, binding_s {0}, misbinding_h {0}, misbinding_s {0};
    vector<double> enthalpies, entropies;
};

struct Tables {
    int imax {0}, dim {1};
    bool dense {true};
    // dense: dim*dim each; compact: imax+2 each (by |identity|, then mismatch)
    vector<double> e, h, s;
    bool stack_dense {false};
    vector<double> stack;   // dense sequence-specific stacking, dim*dim
    double stack_const {0};
    double init_e {0}, init_h {0}, init_s {0};
};

inline Tables build_tables(const vector<vector<int>>& idents, const vector<vector<string>>& seqs,
                           const EnergyInputs& in) {
    static const NNParams P;
    Tables t;
    for (auto& c : idents)
        for (int x : c) t.imax = std::max(t.imax, std::abs(x));
    t.dim = 2 * t.imax + 1;
    HS init = reduce(HS {P.init_h, P.init_s}, in.temp);
    t.init_h = init.h;
    t.init_s = init.s;
    t.init_e = init.h - init.s;
    const bool nn = in.hybridization_pot == "NearestNeighbour";
    const bool uni = in.hybridization_pot == "Uniform";
    const bool spec = in.hybridization_pot == "Specified";
    if (!nn && !uni && !spec) throw std::runtime_error(in.stacking_pot + ": No such hybridization potential");
    const bool seqstack = in.stacking_pot == "SequenceSpecific";
    if (!seqstack && in.stacking_pot != "Constant")
        throw std::runtime_error(in.stacking_pot + ": No such stacking potential");
    t.dense = nn;
    t.stack_dense = seqstack;
    t.stack_const = in.stacking_ene * in.stacking_mult / in.temp;
    size_t n = t.dense ? (size_t)t.dim * t.dim : (size_t)t.imax + 2;
    t.e.assign(n, 0.0);
    t.h.assign(n, 0.0);
    t.s.assign(n, 0.0);
    if (seqstack) t.stack.assign((size_t)t.dim * t.dim, 0.0);
    auto uniform_hs = [&](int a, int b, double& H, double& S) {
        if (a == -b) {
            if (uni) {
                H = in.binding_h / in.temp;
                S = in.binding_s;
            }
            else {
                int i = std::abs(a) - 1;
                H = in.enthalpies.at(i) / in.temp;
                S = in.entropies.at(i);
            }
            if (in.mean_field) S += 3 * std::log(6);
        }
        else {
            H = in.misbinding_h / in.temp;
            S = in.misbinding_s;
        }
        S += std::log(6);
    };
    for (size_t ci = 0; ci < idents.size(); ++ci)
        for (size_t cj = 0; cj < idents.size(); ++cj)
            for (size_t di = 0; di < idents[ci].size(); ++di)
                for (size_t dj = 0; dj < idents[cj].size(); ++dj) {
                    int a = idents[ci][di], b = idents[cj][dj];
                    double H = 0, S = 0;
                    if (nn) {
                        const string& si = seqs.at(ci).at(di);
                        const string& sj = seqs.at(cj).at(dj);
                        vector<string> cs = longest_pairing(si, sj);
                        if (!cs.empty()) {
                            for (auto& c : cs) {
                                HS x = reduce(duplex_hs(P, c, in.cation_M), in.temp);
                                H += x.h - init.h;
                                S += x.s - init.s;
                            }
                            int N = (int)cs.size();
                            H /= N;
                            S /= N;
                            S += std::log(6);
                            bool full = cs[0].size() == si.size() && si.size() == sj.size();
                            bool partial = cs[0].size() != si.size() && si.size() == sj.size();
                            if (a == -b) {
                                if (in.mean_field) S += 3 * std::log(6);
                                if (partial)
                                    throw std::runtime_error("Sequences that should be complementary are not: \n" + si +
                                                             "\n" + sj);
                            }
                            else if (full) {
                                throw std::runtime_error("Sequences that should not be complementary are: \n" + si +
                                                         "\n" + sj);
                            }
                        }
                        size_t k = (size_t)(a + t.imax) * t.dim + (size_t)(b + t.imax);
                        t.h[k] = H;
                        t.s[k] = S;
                        t.e[k] = H - S;
                    }
                    else {
                        uniform_hs(a, b, H, S);
                        size_t k = (a == -b) ? (size_t)std::abs(a) : (size_t)t.imax + 1;
                        t.h[k] = H;
                        t.s[k] = S;
                        t.e[k] = H - S;
                    }
                    if (seqstack) {
                        const string& si = seqs.at(ci).at(di);
                        const string& sj = seqs.at(cj).at(dj);
                        t.stack[(size_t)(a + t.imax) * t.dim + (size_t)(b + t.imax)] =
                            P.stack_g[4 * nuc(si.back()) + nuc(sj.front())];
                    }
                }
    return t;
}

} // namespace ldo_host
