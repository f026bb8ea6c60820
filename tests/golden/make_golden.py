"""Generates the golden fixtures in this directory by running the reference
itself, compiled from its own sources with the recipe in oracle/ref (Philox
RNG in place of std::mt19937_64), on the synthetic systems of tests/systems.py.

Needs the reference sources (only present where the fixtures are made):
    make -C oracle/ref REF=<reference checkout> && python tests/golden/make_golden.py

Each fixture <case>_s<seed>.json.gz holds the per-step trace (step, energy,
staples, fully bound pairs, bound pairs, stacked pairs, total bias, random
draws) and the final configuration (chains: index, identity, per domain
x y z ox oy oz state); <case>_r<frame>_s<seed> starts from a frame of a
reference-written trajectory under outputs/, <case>_anneal_s<seed> runs the
reference's annealing loop.  <name>_enumeration.json holds the reference's
exact staple-only enumerations, outputs/ the reference's own output files.

pt_<variant>_<case>.json: parallel-tempering runs whose exchanges are made by
the reference's own PTGCMCSimulation code (oracle/_ref/ref_exchange acting as
each ladder's master rank) on the per-replica quantities of the oracle's MC
between exchanges: per round the reference's acceptance probabilities of the
pairs tried, permutations, draw counts and controls, and the final attempt and
swap counts.  us_update_<case>.json: umbrella-sampling runs whose bias updates
are made by the reference's SimpleUSGCMCSimulation::process_iteration on the
oracle's visit counts.  us_exchange.json: window exchanges made by the
reference's PTMWUSGCMCSimulation::attempt_exchange on seeded points and biases."""
import gzip
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import systems  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ref_trace")
REF_X = os.path.join(ROOT, "oracle", "_ref", "ref_exchange")

# case, seed, steps
RUNS = [("c1", 1, 20000), ("c1", 2, 20000), ("g24a", 3, 20000), ("g24b", 4, 20000), ("g24c", 5, 20000),
        ("g24d", 6, 10000), ("g24e", 7, 20000), ("c3", 8, 10000),
        # scaffold regrowth (conserved topology, recoil growth and configurational bias)
        ("s24a", 3, 20000), ("s24b", 4, 20000), ("s24c", 5, 20000), ("r24", 6, 20000), ("s48", 7, 10000),
        # the 96-domain ThreeQuarterTurn design with two- and three-domain staples
        ("c4", 9, 20000),
        # a run with a weight ratio within a rounding of 1 at step 19885 (long double vs FP64)
        ("s24a", 11, 20000),
        # Dist / AdjacentSite order parameters with biases, on a moving scaffold
        ("d24", 12, 20000),
        # scaffold transforms with linker regrowth (CTCB, clustered CTCB, CTRG)
        ("l24a", 13, 20000), ("l24b", 14, 20000), ("l24c", 18, 20000), ("l24r", 16, 20000),
        # three-domain staples with misbinding disallowed
        ("m8", 19, 20000)]


def ref_trace(inp, seed, steps, replica=0):
    with open(inp) as f:
        text = f.read()
    tmp = inp + ".trace.inp"
    with open(tmp, "w") as f:
        f.write(text + "trace_steps=%d\ntrace_seed=%d\ntrace_replica=%d\ntrace_every=%d\n"
                % (steps, seed, replica, steps))
    out = subprocess.run([REF, tmp], capture_output=True, text=True, cwd=os.path.dirname(inp))
    os.remove(tmp)
    d = json.loads(out.stdout)
    if "error" in d:
        raise RuntimeError(d["error"])
    return d


def flatten(chains):
    flat = [len(chains)]
    for idx, ident, doms in chains:
        flat += [idx, ident, len(doms)]
        for d in doms:
            flat += d
    return flat


# exact enumerations: fixture name, case (the 4-domain system, whose staples
# never bind both domains; the capped 8-domain system, where they do)
ENUMERATIONS = [("c1_enumeration", "c1"), ("e8_enumeration", "e8"), ("e8s3_enumeration", "e8"),
                # every staple set of the 8-domain system (38 min on one core)
                ("e8s4_enumeration", "e8"),
                # three-domain staples, misbinding disallowed: the no-misbinding
                # growth-point enumerator and the misbinding-only overcount
                ("m8_enumeration", "m8"),
                # the full conformational enumeration (scaffold enumerated too, src/enumerate.cpp:218)
                ("c1full_enumeration", "c1"), ("c1full3_enumeration", "c1")]
# extra .inp options of an enumeration (defaults: the case's own)
ENUM_OPTS = {"e8s3_enumeration": {"max_total_staples": 3}, "e8s4_enumeration": {"max_total_staples": 4},
             "c1full_enumeration": {"enumerate_staples_only": "false", "max_total_staples": 2},
             "c1full3_enumeration": {"enumerate_staples_only": "false", "max_total_staples": 3}}
# enumerations recorded with the partition sum of every growth-point set
ENUM_UNITS = {"e8_enumeration", "m8_enumeration", "c1full_enumeration", "c1full3_enumeration"}
# enumerations recorded with their number of growth-point sets only
ENUM_UNIT_COUNT = {"c1_enumeration", "e8s3_enumeration", "e8s4_enumeration"}
# full enumerations recorded also with every bin summed without rounding drift
# (the reference's weights, compensated sums; ref_trace.cpp's exact_bins)
ENUM_EXACT = {"c1full_enumeration", "c1full3_enumeration"}


def enumerate_case(tmp, name, case):
    """Exact enumeration of a small system with the reference's enumerator
    (staple-only, src/enumerate.cpp:687, or with the scaffold enumerated too,
    :218, as enumerate_staples_only says), weights over (numstaples,
    numfulldomains) at full precision (oracle/ref/ref_trace.cpp's enumerate
    mode runs enumerate_main's sequence and prints the normalised weights)."""
    base = os.path.join(tmp, name)
    opts = dict(simulation_type="enumerate", enumerate_staples_only="true",
                ops_to_output="numstaples numfulldomains", output_filebase=base)
    opts.update(ENUM_OPTS.get(name, {}))
    inp = systems.write_case(tmp, case, extra=opts)
    with open(inp, "a") as f:
        f.write("trace_mode=enumerate\n")
        if name in ENUM_UNITS or name in ENUM_UNIT_COUNT:
            f.write("trace_units=1\n")
        if name in ENUM_EXACT:
            f.write("trace_exact_bins=1\n")
    out = subprocess.run([REF, inp], capture_output=True, text=True, cwd=tmp, check=True).stdout
    d = json.loads([x for x in out.splitlines() if x.startswith("@@")][-1][2:])
    path = os.path.join(HERE, name + ".json")
    with open(path, "w") as f:
        json.dump({"case": case, "ops": ["numstaples", "numfulldomains"], "options": ENUM_OPTS.get(name, {}),
                   "weights": d["weights"], "num_configs": d["num_configs"],
                   **({"units": d["units"]} if "units" in d and name in ENUM_UNITS else {}),
                   **({"n_units": len(d["units"])} if "units" in d and name in ENUM_UNIT_COUNT else {}),
                   **({"unit_energy_drift": d["unit_energy_drift"]} if "unit_energy_drift" in d else {}),
                   **({k: d[k] for k in ("weights_exact", "bin_configs", "saved_configs") if k in d})},
                  f, sort_keys=True)
    print(path, d["weights"], "%.1f s" % d["seconds"])


# restarts from a frame of a reference-written trajectory (restart_traj_file /
# restart_step, src/origami_system.cpp:1000): case, trajectory under
# outputs/, frame, seed, steps
RESTART_RUNS = [("g24a", "g24a_s3.trj", 3, 21, 10000), ("c3", "c3_s8.trj", 4, 22, 10000),
                ("g24b", "g24b_s4.trj", 0, 23, 10000)]


def restart_overrides(trj, frame):
    """The .inp lines of a restart from frame `frame` of outputs/<trj>."""
    return "restart_traj_file=%s\nrestart_step=%d\n" % (os.path.join(HERE, "outputs", trj), frame)


def make_restarts(tmp, only=None):
    for case, trj, frame, seed, steps in RESTART_RUNS:
        if only and case not in only:
            continue
        inp = systems.write_case(tmp, case)
        with open(inp, "a") as f:
            f.write(restart_overrides(trj, frame))
        d = ref_trace(inp, seed, steps)
        fx = {"case": case, "seed": seed, "steps": steps, "restart": [trj, frame],
              "initial_energy": d["initial_energy"], "trace": d["steps"], "final_config": flatten(d["dumps"][-1][1]),
              "draws": d["draws"]}
        path = os.path.join(HERE, "%s_r%d_s%d.json.gz" % (case, frame, seed))
        with gzip.open(path, "wt") as f:
            json.dump(fx, f)
        print(path, len(d["steps"]), "steps, draws", d["draws"])


# the reference's annealing loop (AnnealingGCMCSimulation::run,
# src/annealing_simulation.cpp:40): case, seed, max_temp, min_temp,
# temp_interval, steps_per_temp, constant_staple_M
ANNEAL_RUNS = [("g24a", 31, 350.0, 330.0, 5.0, 1500, True), ("c3", 32, 350.0, 335.0, 5.0, 2000, False)]


def anneal_options(run):
    case, seed, tmax, tmin, dt, steps, const = run
    return dict(max_temp=tmax, min_temp=tmin, temp_interval=dt, steps_per_temp=steps,
                constant_staple_M="true" if const else "false")


def make_anneals(tmp, only=None):
    for run in ANNEAL_RUNS:
        case, seed = run[0], run[1]
        if only and case not in only:
            continue
        opts = anneal_options(run)
        opts["output_filebase"] = os.path.join(tmp, "%s_anneal" % case)
        inp = systems.write_case(tmp, case, extra=opts)
        with open(inp, "a") as f:
            f.write("trace_mode=anneal\n")
        d = ref_trace(inp, seed, 0)
        fx = {"case": case, "seed": seed, "steps": len(d["steps"]), "anneal": list(run[2:]),
              "initial_energy": d["initial_energy"], "trace": d["steps"], "final_config": flatten(d["dumps"][-1][1]),
              "draws": d["draws"]}
        path = os.path.join(HERE, "%s_anneal_s%d.json.gz" % (case, seed))
        with gzip.open(path, "wt") as f:
            json.dump(fx, f)
        print(path, len(d["steps"]), "steps, draws", d["draws"])


# reference output files: case, seed, steps, write frequency
OUTPUT_RUNS = [("g24a", 3, 2000, 400), ("g24b", 4, 2000, 400), ("c3", 8, 2000, 400)]
OUTPUT_EXTS = [".vsf", ".trj", ".vcf", ".states", ".ores", ".counts", ".staples", ".staplestates", ".ene", ".ops"]


def make_outputs(tmp, only=None):
    """The reference's own output writers (setup_output_files,
    src/simulation.cpp:47) on the traced runs: every file of every kind the
    engine's ldo_writer_* reproduces, written every `freq` steps."""
    out_dir = os.path.join(HERE, "outputs")
    os.makedirs(out_dir, exist_ok=True)
    for case, seed, steps, freq in OUTPUT_RUNS:
        if only and case not in only:
            continue
        base = os.path.join(tmp, "%s_out" % case)
        inp = systems.write_case(tmp, case, extra=dict(
            configs_output_freq=freq, vtf_output_freq=freq, counts_output_freq=freq, energies_output_freq=freq,
            order_params_output_freq=freq, ops_to_output="numstaples numfulldomains", output_filebase=base))
        ref_trace(inp, seed, steps)
        for ext in OUTPUT_EXTS:
            with open(base + ext) as f, open(os.path.join(out_dir, "%s_s%d%s" % (case, seed, ext)), "w") as g:
                g.write(f.read())
        print(out_dir, case, "outputs")


class RefExchange:
    """One ref_exchange process: the reference's exchange code as a master
    rank, fed and read line by line (answers start with "@@ ")."""

    def __init__(self, params_path, extra_lines=""):
        tmp = params_path + ".x.inp"
        with open(params_path) as f:
            text = f.read()
        with open(tmp, "w") as f:
            f.write(text + extra_lines)
        self.p = subprocess.Popen([REF_X, tmp], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True,
                                  cwd=os.path.dirname(params_path))

    def ask(self, lines):
        self.p.stdin.write("\n".join(lines) + "\n")
        self.p.stdin.flush()
        while True:
            line = self.p.stdout.readline()
            if not line:
                raise RuntimeError("ref_exchange ended")
            if line.startswith("@@ "):
                if line.startswith("@@ error"):
                    raise RuntimeError(line)
                return line[3:].split()

    def close(self):
        self.p.stdin.write("quit\n")
        self.p.stdin.close()
        self.p.wait()


def fields(words, key, conv=float):
    i = words.index(key) + 1
    out = []
    while i < len(words) and not words[i].isalpha():
        out.append(conv(words[i]))
        i += 1
    return out


# name, case, PT parameters, reference variant, exchange_q bits / 2-D size,
# ladders, seed, rounds, steps between exchanges, oracle parameters
PT_RUNS = [
    ("pt_ut_g24a", "g24a", dict(temps=[325.0, 330.0, 336.0, 343.0], chem_pot_mults=[1.0, 1.3, 0.9, 1.1]),
     "UT", 3, 0, 2, 31, 12, 150, dict(temp=335.0, staple_M=1e-3, staple_lengths=[2] * 12)),
    ("pt_st_g24a", "g24a", dict(temps=[325.0, 330.0, 336.0, 343.0], stacking_mults=[1.0, 0.85, 1.1, 1.25]),
     "ST", 9, 0, 2, 37, 12, 150, dict(temp=335.0, staple_M=1e-3, staple_lengths=[2] * 12)),
    ("pt_t_c3", "c3", dict(temps=[310.0 * (370.0 / 310.0) ** (k / 7.0) for k in range(8)]),
     "T", 1, 0, 2, 41, 8, 500, dict(temp=340.0, staple_M=1e-6, staple_lengths=[2] * 24)),
    ("pt_2d_g24a", "g24a", dict(temps=[325.0, 333.0, 342.0], stacking_mults=[0.8, 1.0, 1.25]),
     "2D", 0, 3, 2, 53, 14, 150, dict(temp=335.0, staple_M=1e-3, staple_lengths=[2] * 12)),
]


def pt_inp_extra(pt, dim2):
    """.inp keys of a PT run (the engine's and the reference's)."""
    temps = pt["temps"]
    R = len(temps) * (dim2 or 1)
    extra = dict(temps=" ".join(repr(t) for t in temps), num_reps=R)
    for k in ("chem_pot_mults", "bias_mults", "stacking_mults"):
        if k in pt:
            extra[k] = " ".join(repr(x) for x in pt[k])
    return extra, R


def make_pt_exchanges(tmp, only=None):
    from pt_oracle import PTOracle
    for name, case, pt, variant, q, dim2, n_lad, seed, swaps, interval, oparams in PT_RUNS:
        if only and name not in only and case not in only:
            continue
        extra, R = pt_inp_extra(pt, dim2)
        inp = systems.write_case(os.path.join(tmp, name), case, extra=extra)
        op = dict(oparams)
        op.update({k: v for k, v in pt.items()})
        if not dim2:
            for k in ("chem_pot_mults", "bias_mults", "stacking_mults"):
                op.setdefault(k, [1.0] * R)
        # the reference needs every per-rank list; 1-D lists default to 1
        ref_lists = "".join("%s = %s\n" % (k, " ".join(repr(x) for x in op[k]))
                            for k in ("chem_pot_mults", "bias_mults", "stacking_mults") if not dim2)
        refs = [RefExchange(inp, "exchange_mode = pt\npt_variant = %s\ntrace_seed = %d\ntrace_replica = %d\n%s"
                            % (variant, seed, l, ref_lists)) for l in range(n_lad)]
        red_ref = [float(x) for x in refs[0].ask(["redu"])[1:]]
        rounds = []

        class RefPT(PTOracle):
            def exchange(self, l, deps):
                R_ = self.n_rungs
                ref = refs[l]
                perm = self.perm[l]
                S = len(deps[0][3]) - 1
                ps = []
                for i, i2, _ in self.pairs():
                    r1, r2 = perm[i], perm[i2]
                    H1, st1, b1, n1 = deps[r1]
                    H2, st2, b2, n2 = deps[r2]
                    vals = [self.slot["temp"][i], self.slot["temp"][i2], self.slot["stack"][i], self.slot["stack"][i2],
                            H1, H2, b1, b2, st1, st2]
                    vals += [red_ref[t - 1] * self.ctrl[r1]["temp"] * self.ctrl[r1]["u"] for t in range(1, S + 1)]
                    vals += [red_ref[t - 1] * self.ctrl[r2]["temp"] * self.ctrl[r2]["u"] for t in range(1, S + 1)]
                    vals += [float(n1[t]) for t in range(1, S + 1)] + [float(n2[t]) for t in range(1, S + 1)]
                    ps.append(float(ref.ask(["acc " + " ".join(repr(float(v)) for v in vals)])[1]))
                lines = ["round %d" % self.swap_i]
                for k in range(R_):
                    H, st, b, n = deps[l * R_ + k]
                    lines.append(" ".join(repr(float(v)) for v in [H, b, st] + [float(x) for x in n[1:]]))
                w = ref.ask(lines)
                qperm = fields(w, "perm", int)
                self.perm[l] = [l * R_ + x for x in qperm]
                self.draws[l] = int(fields(w, "draws", int)[0])
                ctl = fields(w, "ctl")
                for k in range(R_):
                    c = self.ctrl[l * R_ + k]
                    c["temp"], c["u"], c["bias"], c["stack"] = ctl[4 * k:4 * k + 4]
                rounds.append({"ladder": l, "swap_i": self.swap_i, "p": ps, "perm": self.perm[l],
                               "draws": self.draws[l], "ctl": ctl})

        ora = RefPT(inp, op, n_lad, seed, exchange_q=q or 1, dim2=dim2, reference_initial_controls=True)
        for _ in range(swaps):
            ora.round(interval)
        att, acc = [0] * len(ora.att), [0] * len(ora.acc)
        for ref in refs:
            w = ref.ask(["counts"])
            for i, x in enumerate(fields(w, "att", int)):
                att[i] += x
            for i, x in enumerate(fields(w, "acc", int)):
                acc[i] += x
            ref.close()
        fx = {"name": name, "case": case, "extra": extra, "oracle_params": op, "variant": variant, "q": q,
              "dim2": dim2, "n_ladders": n_lad, "seed": seed, "swaps": swaps, "interval": interval,
              "red_u": red_ref, "rounds": rounds, "att": att, "acc": acc,
              "final_perm": [x for p in ora.perm for x in p]}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(fx, f)
        print(name, "accepted", sum(acc), "of", sum(att))


US_WINDOWS = systems.US_WINDOWS
write_us_case = systems.write_us_case


def make_us_update(tmp, only=None):
    """Umbrella iterations without window exchange: the oracle's MC per
    window, the reference's SimpleUSGCMCSimulation::process_iteration for the
    bias updates of every window."""
    if only and "us_update" not in only:
        return
    from us_oracle import USOracle
    seed, iters, equil, steps, max_D = 17, 4, 400, 600, 2.0
    inp = write_us_case(os.path.join(tmp, "us_update"))
    ref = RefExchange(inp, "exchange_mode = us_update\nnum_windows = %d\nmax_D_bias = %r\n"
                      % (len(US_WINDOWS), max_D))
    record = []

    class RefUS(USOracle):
        def process(self, hist, max_D_):
            lines = ["iter %d" % len(record)]
            for w in range(self.nw):
                pts = [(x, c) for x, c in enumerate(hist[w]) if c > 0]
                lines.append(" ".join([str(len(pts))] + ["%d %d" % pc for pc in pts]))
            ref.p.stdin.write("\n".join(lines) + "\n")
            ref.p.stdin.flush()
            it = {"hist": [list(map(int, h)) for h in hist], "E": []}
            for w in range(self.nw):
                while True:
                    line = ref.p.stdout.readline()
                    if line.startswith("@@ "):
                        break
                words = line[3:].split()
                assert words[0] == "E" and int(words[1]) == w, words
                k = int(words[2])
                E = np.zeros(self.len)
                self.inS[w][:] = False
                for j in range(k):
                    x, e = int(words[3 + 2 * j]), float(words[4 + 2 * j])
                    E[x] = e
                    self.inS[w][x] = True
                self.E[w] = E
                it["E"].append(E.tolist())
            record.append(it)
            self.apply()

    ora = RefUS(inp, seed, US_WINDOWS, "grid", "win", 25)
    ora.run(iters, equil, steps, max_D, 0)
    ref.close()
    # the .biases file the reference's output_weights wrote for window 1
    # after the last iteration (process_iteration, src/us_simulation.cpp:169)
    with open(os.path.join(os.path.dirname(inp), "ref_trace_out_win1.biases")) as f, \
            open(os.path.join(HERE, "outputs", "us_update_win1.biases"), "w") as g:
        g.write(f.read())
    fx = {"seed": seed, "iters": iters, "equil": equil, "steps": steps, "max_D": max_D, "windows": US_WINDOWS,
          "grid_len": 25, "iterations": record, "window_of": ora.window_of,
          "draws": [int(r.observables()["draws"]) for r in ora.reps]}
    with open(os.path.join(HERE, "us_update_g24a.json"), "w") as f:
        json.dump(fx, f)
    print("us_update_g24a", iters, "iterations")


def make_us_exchange(tmp, only=None):
    """Window exchanges of PTMWUSGCMCSimulation::attempt_exchange on seeded
    grid points and biases (window 0's point is the master's own, fixed)."""
    if only and "us_exchange" not in only:
        return
    import random
    rng = random.Random(7)
    seed, rounds = 23, 60
    inp = write_us_case(os.path.join(tmp, "us_exchange"))
    W = len(US_WINDOWS)
    ref = RefExchange(inp, "exchange_mode = us_exchange\nnum_windows = %d\ntrace_seed = %d\n" % (W, seed))
    p0 = int(ref.ask(["point0"])[1])
    rec = []
    E = [[rng.gauss(0.0, 1.5) for _ in range(25)] for _ in range(W)]
    for swap_i in range(1, rounds + 1):
        pts = [p0] + [rng.randint(US_WINDOWS[w][0], US_WINDOWS[w][1]) for w in range(1, W)]
        if swap_i % 7 == 0:
            pts[2] = pts[1] = min(max(pts[1], US_WINDOWS[2][0]), US_WINDOWS[1][1])   # equal points
        if swap_i % 5 == 0:
            E = [[e + rng.gauss(0.0, 0.5) for e in Ew] for Ew in E]
        lines = ["round %d" % swap_i]
        for w in range(W):
            lines.append(" ".join([str(pts[w]), "25"] + ["%d %r" % (x, E[w][x]) for x in range(25)]))
        words = ref.ask(lines)
        rec.append({"swap_i": swap_i, "points": pts, "E": [list(e) for e in E],
                    "w2w": fields(words, "w2w", int), "configi": fields(words, "configi", int),
                    "draws": int(fields(words, "draws", int)[0])})
    words = ref.ask(["counts"])
    fx = {"seed": seed, "windows": US_WINDOWS, "rounds": rec, "att": fields(words, "att", int),
          "acc": fields(words, "acc", int)}
    ref.close()
    with open(os.path.join(HERE, "us_exchange.json"), "w") as f:
        json.dump(fx, f)
    print("us_exchange accepted", sum(fx["acc"]), "of", sum(fx["att"]))


def main(only=None):
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -C oracle/ref REF=<reference checkout>")
    with tempfile.TemporaryDirectory() as tmp:
        for case, seed, steps in RUNS:
            if only and case not in only:
                continue
            inp = systems.write_case(tmp, case)
            d = ref_trace(inp, seed, steps)
            fx = {"case": case, "seed": seed, "steps": steps, "initial_energy": d["initial_energy"],
                  "trace": d["steps"], "final_config": flatten(d["dumps"][-1][1]), "draws": d["draws"]}
            path = os.path.join(HERE, "%s_s%d.json.gz" % (case, seed))
            with gzip.open(path, "wt") as f:
                json.dump(fx, f)
            print(path, len(d["steps"]), "steps, draws", d["draws"])
        for name, case in ENUMERATIONS:
            if not only or case in only:
                enumerate_case(tmp, name, case)
        make_outputs(tmp, only)
        make_restarts(tmp, only)
        make_anneals(tmp, only)
        make_pt_exchanges(tmp, only)
        make_us_update(tmp, only)
        make_us_exchange(tmp, only)


if __name__ == "__main__":
    # python tests/golden/make_golden.py [case ...]   (default: every run)
    main(sys.argv[1:] or None)
