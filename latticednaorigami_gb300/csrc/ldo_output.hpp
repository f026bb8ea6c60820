// Output files of one replica in the reference's formats (OrigamiOutputFile
// subclasses, src/files.cpp:519-789, opened by setup_output_files,
// src/simulation.cpp:47-147), written from a host copy of the replica's
// state.  Host code only.
#pragma once
#include <chrono>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace ldo_out {

// One replica's state as the writers need it.
struct Snapshot {
    struct Dom {
        int pos[3], ore[3], state;   // state: 0 unassigned, 1 unbound, 2 bound, 3 misbound
    };
    struct Chain {
        int index, identity;
        std::vector<Dom> doms;
    };
    std::vector<Chain> chains;       // m_domains order
    int n_types {0};                 // staple types (identities 1..n_types)
    int num_staples {0}, num_bound {0}, num_fully {0};
    double energy {0}, enthalpy {0}, entropy {0}, stacking {0}, bias {0};
    std::vector<int> op_values;      // order parameters to output, in order
};

enum Kind : unsigned {
    TRJ = 1,       // .trj
    VTF = 2,       // .vcf .states .ores
    COUNTS = 4,    // .counts .staples .staplestates
    ENE = 8,       // .ene
    OPS = 16,      // .ops
    TIMES = 32     // .times (seconds since the writer was opened)
};

class Writer {
  public:
    // max_total_staples / max_staple_size give the padded domain count of
    // the VMD files (m_max_num_domains, src/files.cpp:503-505).
    Writer(const std::string& base, unsigned kinds, int scaffold_len, int max_total_staples, int max_staple_size,
           const std::vector<std::string>& op_tags)
        : m_kinds(kinds),
          m_max_staple_size(max_staple_size),
          m_max_num_domains(max_staple_size * max_total_staples + scaffold_len) {
        // OrigamiVSFOutputFile, always written (src/simulation.cpp:56-62)
        {
            std::ofstream vsf(base + ".vsf");
            if (!vsf.good()) throw std::runtime_error(base + ".vsf: output path does not exist");
            vsf << "atom 0:" << scaffold_len << " radius 0.25 type scaffold\n";
            vsf << "atom " << scaffold_len << ":" << m_max_num_domains - 1 << " radius 0.25 type staple";
        }
        if (kinds & TRJ) open(m_trj, base + ".trj");
        if (kinds & VTF) {
            open(m_vcf, base + ".vcf");
            open(m_states, base + ".states");
            open(m_ores, base + ".ores");
        }
        if (kinds & COUNTS) {
            open(m_counts, base + ".counts");
            open(m_staples, base + ".staples");
            open(m_staplestates, base + ".staplestates");
        }
        if (kinds & ENE) {
            open(m_ene, base + ".ene");
            m_ene << "step tenergy henthalpy hentropy stacking bias\n";
            m_ene.precision(10);
        }
        if (kinds & TIMES) {
            // OrigamiTimesOutputFile (src/files.cpp:723)
            open(m_times, base + ".times");
            m_times << "step time\n";
            m_start = std::chrono::steady_clock::now();
        }
        if (kinds & OPS) {
            open(m_ops, base + ".ops");
            for (auto& t : op_tags) {
                m_ops << t << ", ";
                m_ops.precision(10);
            }
            m_ops << "\n";
            m_ops.flush();
        }
    }

    void write(long long step, const Snapshot& s) {
        if (m_kinds & TRJ) write_trj(step, s);
        if (m_kinds & VTF) {
            write_vcf(s);
            write_states(s);
            write_ores(s);
        }
        if (m_kinds & COUNTS) write_counts(step, s);
        if (m_kinds & ENE) {
            m_ene << step << " " << s.energy << " " << s.enthalpy << " " << s.entropy << " " << s.stacking << " "
                  << s.bias << " \n";
            m_ene.flush();
        }
        if (m_kinds & TIMES) {   // OrigamiTimesOutputFile::write (src/files.cpp:739)
            std::chrono::duration<double> dt {std::chrono::steady_clock::now() - m_start};
            m_times << step << " ";
            m_times << dt.count();
            m_times << "\n";
            m_times.flush();
        }
        if (m_kinds & OPS) {
            m_ops << step;
            for (int v : s.op_values) m_ops << " " << v;
            m_ops << "\n";
            m_ops.flush();
        }
    }

  private:
    static void open(std::ofstream& f, const std::string& name) {
        f.open(name);
        if (!f.good()) throw std::runtime_error(name + ": output path does not exist");
    }

    // OrigamiTrajOutputFile::write (src/files.cpp:529)
    void write_trj(long long step, const Snapshot& s) {
        m_trj << step << "\n";
        for (auto& c : s.chains) {
            m_trj << c.index << " " << c.identity << "\n";
            for (auto& d : c.doms)
                for (int i = 0; i < 3; ++i) m_trj << d.pos[i] << " ";
            m_trj << "\n";
            for (auto& d : c.doms)
                for (int i = 0; i < 3; ++i) m_trj << d.ore[i] << " ";
            m_trj << "\n";
        }
        m_trj << "\n";
        m_trj.flush();
    }

    // OrigamiVCFOutputFile::write (src/files.cpp:552)
    void write_vcf(const Snapshot& s) {
        m_vcf << "timestep\n";
        int written = 0;
        for (auto& c : s.chains) {
            int n = 0;
            for (auto& d : c.doms) {
                ++n;
                for (int i = 0; i < 3; ++i) m_vcf << d.pos[i] << " ";
                m_vcf << "\n";
            }
            for (; n < m_max_staple_size; ++n) m_vcf << "0 0 0 \n";
            written += n;
        }
        for (int k = written; k < m_max_num_domains; ++k) m_vcf << "0 0 0 \n";
        m_vcf << "\n";
        m_vcf.flush();
    }

    // OrigamiStateOutputFile::write (src/files.cpp:617)
    void write_states(const Snapshot& s) {
        int written = 0;
        for (auto& c : s.chains) {
            int n = 0;
            for (auto& d : c.doms) {
                ++n;
                m_states << (d.state >= 1 && d.state <= 3 ? d.state : 0) << " ";
            }
            for (; n < m_max_staple_size; ++n) m_states << "-1 ";
            written += n;
        }
        for (int k = written; k < m_max_num_domains; ++k) m_states << "-1 ";
        m_states << "\n";
        m_states.flush();
    }

    // OrigamiOrientationOutputFile::write (src/files.cpp:586)
    void write_ores(const Snapshot& s) {
        int written = 0;
        for (auto& c : s.chains) {
            int n = 0;
            for (auto& d : c.doms) {
                ++n;
                for (int i = 0; i < 3; ++i) m_ores << (d.state != 0 ? d.ore[i] : 0) << " ";
            }
            for (; n < m_max_staple_size; ++n) m_ores << "0 0 0 ";
            written += n;
        }
        for (int k = written; k < m_max_num_domains; ++k) m_ores << "0 0 0 ";
        m_ores << "\n";
        m_ores.flush();
    }

    // OrigamiCountsOutputFile, OrigamiStaplesBoundOutputFile,
    // OrigamiStaplesFullyBoundOutputFile (src/files.cpp:651-697)
    void write_counts(long long step, const Snapshot& s) {
        std::vector<int> per_type(s.n_types, 0), fully(s.n_types, 0);
        for (size_t c = 1; c < s.chains.size(); ++c) {
            int t = s.chains[c].identity;
            if (t < 1 || t > s.n_types) continue;
            per_type[t - 1]++;
            bool all = true;
            for (auto& d : s.chains[c].doms) all = all && d.state == 2;
            if (all) fully[t - 1] = 1;
        }
        int unique = 0;
        for (int n : per_type) unique += n > 0;
        m_counts << step << " " << s.num_staples << " " << unique << " " << s.num_bound << " " << s.num_fully << " "
                 << s.num_bound - s.num_fully << " \n";
        m_counts.flush();
        m_staples << step << " ";
        for (int n : per_type) m_staples << n << " ";
        m_staples << "\n";
        m_staples.flush();
        m_staplestates << step << " ";
        for (int f : fully) m_staplestates << f << " ";
        m_staplestates << "\n";
        m_staplestates.flush();
    }

    unsigned m_kinds;
    int m_max_staple_size, m_max_num_domains;
    std::ofstream m_trj, m_vcf, m_states, m_ores, m_counts, m_staples, m_staplestates, m_ene, m_ops, m_times;
    std::chrono::steady_clock::time_point m_start;
};

} // namespace ldo_out
