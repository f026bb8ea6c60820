"""Generates the golden fixtures in this directory by running the reference
itself, compiled from its own sources with the recipe in oracle/ref (Philox
RNG in place of std::mt19937_64), on the synthetic systems of tests/systems.py.

Needs the reference sources (only present where the fixtures are made):
    make -C oracle/ref && python tests/golden/make_golden.py

Each fixture <case>_s<seed>.json.gz holds the per-step trace (step, energy,
staples, fully bound pairs, bound pairs, stacked pairs, total bias, random
draws) and the final configuration (chains: index, identity, per domain
x y z ox oy oz state); <case>_r<frame>_s<seed> starts from a frame of a
reference-written trajectory under outputs/, <case>_anneal_s<seed> runs the
reference's annealing loop.  <name>_enumeration.json holds the reference's
exact staple-only enumerations, outputs/ the reference's own output files."""
import gzip
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import systems  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ref_trace")

# case, seed, steps
RUNS = [("c1", 1, 20000), ("c1", 2, 20000), ("g24a", 3, 20000), ("g24b", 4, 20000), ("g24c", 5, 20000),
        ("g24d", 6, 10000), ("g24e", 7, 20000), ("c3", 8, 10000),
        # scaffold regrowth (conserved topology, recoil growth and configurational bias)
        ("s24a", 3, 20000), ("s24b", 4, 20000), ("s24c", 5, 20000), ("r24", 6, 20000), ("s48", 7, 10000),
        # the 96-domain ThreeQuarterTurn design with two- and three-domain staples
        ("c4", 9, 20000),
        # a run with a weight ratio within a rounding of 1 at step 19885 (long double vs FP64)
        ("s24a", 11, 20000)]


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
ENUMERATIONS = [("c1_enumeration", "c1"), ("e8_enumeration", "e8")]


def enumerate_case(tmp, name, case):
    """Exact staple-only enumeration of a small system with the reference's
    enumerator (src/enumerate.cpp:687), weights over (numstaples,
    numfulldomains)."""
    base = os.path.join(tmp, name)
    opts = dict(simulation_type="enumerate", enumerate_staples_only="true",
                ops_to_output="numstaples numfulldomains", output_filebase=base)
    inp = systems.write_case(tmp, case, extra=opts)
    with open(inp, "a") as f:
        f.write("trace_mode=enumerate\n")
    subprocess.run([REF, inp], capture_output=True, text=True, cwd=tmp, check=True)
    weights = {}
    with open(base + ".weights") as f:
        tags = f.readline().split()
        for line in f:
            line = line.strip()
            if not line:
                continue
            key, w = line.rsplit(" ", 1)
            weights[" ".join(key.strip("()").split())] = float(w)
    path = os.path.join(HERE, name + ".json")
    with open(path, "w") as f:
        json.dump({"case": case, "ops": tags, "weights": weights}, f, indent=1, sort_keys=True)
    print(path, weights)


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


def main(only=None):
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -C oracle/ref")
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


if __name__ == "__main__":
    # python tests/golden/make_golden.py [case ...]   (default: every run)
    main(sys.argv[1:] or None)
