"""Benchmark of the batched MC workload (4096 independent constant-T chains
of uneven size) on one GB300: learned-proposal MC against plain MC.

Workload: scaffolds of 8/12/16/24 domains (1024 replicas each, serpentine
layout, n/2 two-domain staple types), uniform hybridisation dH = -120 kcal/mol
and dS = -0.33 kcal/mol/K per bound domain, T ~ U[320, 350] K (seeded),
1 uM staples, FourBody, Opposing misbinding, constant stacking 1000 K.  Plain
moveset: Met exchange / Met regrowth / CB regrowth at 1/3 each; learned
moveset: the exchange and the Met regrowth replaced by LearnedStapleExchange
and LearnedStapleRegrowth, whose network is trained (on the GPU) on states of
the plain run.  Philox seeds: replica r uses
key (0, r).  Inputs are synthetic (tests/systems.py).

A step is one launch of SWEEPS sweeps of every replica (a sweep = n_scaffold
move attempts).  `value` is effective samples per second of the number of
fully bound domains (one sample per replica per sweep, tau_int by Sokal
windowing) of the learned moveset, from the device-timed region; `plain`
holds the same figures for the plain moveset; `e2e` repeats the timed loop
through the C ABI with host buffers (temperatures in, samples out every step).

Under torchrun (N > 1) every rank runs the same per-GPU workload on its own
GPU with its own seed (replicas only); value = effective samples of all ranks
/ the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

# 250 sweeps per step: the default 20 timed steps record 5000 sweeps per
# replica, more than 50 integrated autocorrelation times of the slowest
# (24-domain) plain chains, so that tau_int and its confidence interval are
# settled (the tau_vs_length fields of the line show it).
SWEEPS_PER_STEP = 250
N_REP = 4096
SIZES = [8, 12, 16, 24]
R_KCAL = 8.3144598 / 4184.0


def write_c2(d):
    import systems
    files = []
    bh = -120.0 / R_KCAL
    bs = -0.33 / R_KCAL
    for n in SIZES:
        sysj = systems.make_system(n, systems.staple_pairs(n), seed=100 + n, positions=systems.serpentine(n, 4))
        with open(os.path.join(d, "c2_%d.json" % n), "w") as f:
            json.dump(sysj, f)
        with open(os.path.join(d, "moves.json"), "w") as f:
            json.dump(systems.moves_json("met3"), f)
        with open(os.path.join(d, "ops.json"), "w") as f:
            json.dump({"origami": {"order_params": [
                {"label": "Number of bound staples", "tag": "numstaples", "type": "NumStaples", "level": 0},
                {"label": "Number of fully bound domain pairs", "tag": "numfulldomains",
                 "type": "NumBoundDomainPairs", "level": 0}]}}, f)
        opts = dict(systems.BASE)
        opts.update(origami_input_filename="c2_%d.json" % n, movetype_file="moves.json",
                    hybridization_pot="Uniform", binding_h=repr(bh), binding_s=repr(bs), stacking_ene=1000,
                    temp=335, staple_M=1e-6, max_total_staples=n, max_type_staples=2)
        p = os.path.join(d, "c2_%d.inp" % n)
        systems.write_inp(p, opts)
        files.append(p)
    return files


class nvtx_range:
    """An NVTX push/pop range around a timed region, so that a profiler can
    select exactly its launches (`ncu --nvtx --nvtx-include "<name>/"`)."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        import torch
        torch.cuda.nvtx.range_push(self.name)

    def __exit__(self, *exc):
        import torch
        torch.cuda.nvtx.range_pop()
        return False


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for i, nme in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nme)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


class Ranks:
    """One process per GPU under torchrun (replicas only: no data-path
    collective).  Each rank takes the GPU of its LOCAL_RANK (through
    CUDA_VISIBLE_DEVICES, set before the engine library initialises CUDA),
    runs the whole per-GPU workload with its own Philox seed, and meets the
    others in a host-side (gloo) group only for the barriers around the timed
    region and the reductions of its results: work is summed, time is the
    maximum over ranks."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES")
            devs = [v for v in vis.split(",") if v] if vis else [str(i) for i in range(self.world)]
            os.environ["CUDA_VISIBLE_DEVICES"] = devs[self.local % len(devs)]
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def _reduce(self, x, op):
        if not self.dist:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.dist.ReduceOp.MAX if self.dist else None)

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM if self.dist else None)

    def close(self):
        if self.dist and self.dist.is_initialized():
            self.dist.destroy_process_group()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def host_cores():
    """(threads this process may use, CPUs present on the host)."""
    try:
        usable = len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        usable = os.cpu_count() or 1
    present = usable
    try:
        with open("/sys/devices/system/cpu/present") as f:
            present = 0
            for part in f.read().strip().split(","):
                a, _, b = part.partition("-")
                present += (int(b) - int(a) + 1) if b else 1
    except OSError:
        pass
    return usable, present


# Shared-memory roofline of the MC kernel (each replica's state lives in
# shared memory for a whole launch).  Algorithmic bytes per move attempt of
# the c2 workload, from the reference's algorithm as the oracle restates it
# (oracle/touch_counts.py: 16 bytes per domain-record access, 8 per
# occupancy-map operation, after burn-in, both movesets):
B_ATTEMPT = {"plain": 8599.0, "learned": 12202.0}
# the same count on the c3 system (python oracle/touch_counts.py c3: two
# constant-temperature replicas at every ninth of the 64 temperatures)
B_ATTEMPT_C3 = {"plain": 7867.0, "learned": 12279.0}
SMEM_BYTES_PER_CLK_PER_SM = 128
N_SM = 152
KERNEL_SOURCES = ["ldo_engine.cuh", "ldo_kernels.cu", "ldo_kernels.h", "ldo_bind.cuh", "ldo_types.h",
                  "ldo_ct.h", "ldo_math.h", "ldo_learn.h"]


def kernel_source_sha():
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "latticednaorigami_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def measured_traffic(workload):
    """DRAM bytes per launch of the MC kernel from the ncu capture committed
    under profiles/ for this workload, if it was taken of the current kernel
    sources (same source hash); else None."""
    p = os.path.join(ROOT, "profiles", "ldo_mc_kernel_%s_traffic.json" % workload)
    if not os.path.exists(p):
        return None, "no capture"
    with open(p) as f:
        d = json.load(f)
    if d.get("kernel_source_sha") != kernel_source_sha():
        return None, "capture of other kernel sources"
    return d, "ncu capture of these kernel sources (%s)" % os.path.relpath(p, ROOT)


CPU_REPS_PER_SIZE = 128
# Equilibration.  From empty scaffolds the plain sampler relaxes over hundreds
# of sweeps (low temperatures, large scaffolds slowest), and tau_int of a
# series that still drifts is inflated.  The GPU arms therefore start from
# configurations relaxed for RELAX_SWEEPS sweeps by the learned moveset (which
# samples the same distribution: tests against the exact enumeration and the
# plain sampler), the CPU arms from CPU_BURN_SWEEPS sweeps of their own plain
# sampler; every arm then records only stationary sweeps.
RELAX_SWEEPS = 2000
CPU_BURN_SWEEPS = 3000
LEARN_ITERS = 400
LEARN_LR = 2e-3


def write_learned_moves(d):
    """The c2 moveset with the staple exchange and the Met regrowth replaced
    by the learned ones (insertion sites; regrowth directions)."""
    p = os.path.join(d, "moves_learned.json")
    with open(p, "w") as f:
        json.dump({"origami": {"movetypes": [
            {"label": "Learned staple exchange", "type": "LearnedStapleExchange", "freq": "1/3",
             "adaptive_exchange": False},
            {"label": "Learned staple regrowth", "type": "LearnedStapleRegrowth", "freq": "1/3"},
            {"label": "CB staple regrowth", "type": "CBStapleRegrowth", "freq": "1/3"}]}}, f)
    return p


def replica_temps():
    """T ~ U[320, 350] K per replica (seeded); replica r has scaffold size
    SIZES[r // (N_REP / 4)]."""
    return np.random.default_rng(0).uniform(320.0, 350.0, N_REP)


def cpu_temperatures(i):
    """Temperatures of the CPU sample of scaffold size SIZES[i]: the GPU
    run's temperatures of that size, stratified (every per/128-th of them in
    ascending order), so that the sample spans the same range."""
    temps = replica_temps()
    per = N_REP // len(SIZES)
    t = np.sort(temps[i * per:(i + 1) * per])
    return t[np.linspace(0, per - 1, CPU_REPS_PER_SIZE).round().astype(int)]


def cpu_effective_rate(files, cores, burn_sweeps, rec_sweeps):
    """The oracle port on all usable host cores over a bounded sample of the
    same workload: CPU_REPS_PER_SIZE replicas of each scaffold size at
    stratified GPU-run temperatures, burn_sweeps of burn-in from the empty
    scaffold, then the recorded sweeps, tau_int estimated from its own
    samples by the same estimator.  Only the recorded sweeps are timed (pro
    rata).  Returns a dict: effective samples/s with its 95 % bootstrap
    interval, sweeps/s, median tau, mean fully bound domains per size."""
    from oracle_lib import run_batch_sampled
    from latticednaorigami_gb300.analysis import replica_ess, bootstrap_sum, tau_int
    t_total, sweeps_total = 0.0, 0.0
    ess, groups, taus = [], [], []
    means = {}
    for i, f in enumerate(files):
        n = SIZES[i]
        t, smp = run_batch_sampled(f, 0, CPU_REPS_PER_SIZE, burn_sweeps + rec_sweeps, n, cores,
                                   temps=cpu_temperatures(i))
        rec = smp[:, burn_sweeps:]
        means[n] = float(rec.mean())
        series = list(rec)
        ess.append(replica_ess(series))
        groups += [i] * len(series)
        taus += [x for x in (tau_int(s_) for s_ in series) if x is not None]
        t_total += t * rec_sweeps / float(burn_sweeps + rec_sweeps)
        sweeps_total += CPU_REPS_PER_SIZE * rec_sweeps
    ess = np.concatenate(ess)
    (lo, hi), _ = bootstrap_sum(ess, groups)
    return {"value": float(ess.sum()) / t_total, "ci95": [lo / t_total, hi / t_total],
            "sweeps_per_s": sweeps_total / t_total, "tau_int_median": float(np.median(taus)) if taus else None,
            "mean_fully_bound_by_size": means}


def cpu_baseline(files, burn_sweeps, rec_sweeps):
    cores, present = host_cores()
    r = cpu_effective_rate(files, cores, burn_sweeps, rec_sweeps)
    out = {"value": r["value"], "unit": "effective samples/s", "cores": cores, "cores_present_on_host": present,
           "kind": "port",
           "sample": "%d replicas of each scaffold size (GPU-run temperatures, stratified) x %d recorded sweeps "
                     "after %d burn-in sweeps from the empty scaffold, %d threads"
                     % (CPU_REPS_PER_SIZE, rec_sweeps, burn_sweeps, cores)}
    out.update({k: v for k, v in r.items() if k != "value"})
    if present > cores:
        # the port's threads are independent replicas: linear in cores
        out["value_all_host_cores_linear"] = r["value"] * present / cores
    return out


def run_reference_arm(args):
    """Reference arm: the CPU restatement of the reference (oracle port; the
    reference itself cannot be built on the GPU machine) on all usable host cores."""
    tmp = tempfile.mkdtemp()
    files = write_c2(tmp)
    cores, present = host_cores()
    from oracle_lib import run_batch
    for _ in range(args.warmup):
        run_batch(files[0], 0, cores, 20 * SIZES[0], cores)
    burn, rec = CPU_BURN_SWEEPS, args.steps * SWEEPS_PER_STEP
    res, times = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res.append(cpu_effective_rate(files, cores, burn, rec))
        times.append(time.perf_counter() - t0)
    value = float(np.mean([r["value"] for r in res]))
    line = {"impl": "reference", "metric": "effective samples/s (tau_int of #bound domains), learned vs plain MC",
            "value": value, "unit": "effective samples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "c2: constant-T chains, scaffolds 8/12/16/24, uniform hyb, T~U[320,350] K; "
                                   "bounded CPU sample per step; plain moveset (the reference has no learned "
                                   "proposal)"},
            "cpu_baseline": {"value": value, "unit": "effective samples/s", "cores": cores,
                             "cores_present_on_host": present, "kind": "port",
                             "sample": "%d replicas of each scaffold size (GPU-run temperatures, stratified) x %d "
                                       "recorded sweeps after %d burn-in sweeps from the empty scaffold, per step"
                                       % (CPU_REPS_PER_SIZE, rec, burn)},
            "e2e": {"value": value, "unit": "effective samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "ci95_last_step": res[-1]["ci95"],
            "sweeps_per_s": float(np.mean([r["sweeps_per_s"] for r in res])),
            "tau_int_median": res[-1]["tau_int_median"]}
    print(json.dumps(line))


# ---------------------------------------------------------------- c4 ---
# The 96-domain umbrella workload: 48 harmonic windows on the number of fully
# bound domains (k = 0.5 kT/domain^2, centres 0..94 step 2) x 8 temperatures
# (320..350 K), the 96-domain ThreeQuarterTurn design with 16 three-domain and
# 24 two-domain staple types (8 bp domains, NN energies), 1 uM, and the
# reference's standard moveset (orientation rotation, Met exchange, CB staple
# regrowth, CTRG contiguous and jump scaffold regrowth).  Each replica keeps
# its window and temperature (no exchange in the timed region).
C4_WINDOWS, C4_TEMPS, C4_K = 48, 8, 0.5
C4_SWEEPS_PER_STEP = 10
C4_CPU_REPS = 48


def write_c4(d):
    import systems
    with open(os.path.join(d, "c4_windows.json"), "w") as f:
        json.dump({"origami": {"bias_functions": [
            {"label": "window", "tag": "win", "type": "Harmonic", "k": C4_K, "centre": 0,
             "ops": ["numfulldomains"], "level": 0}]}}, f)
    return systems.write_case(d, "c4", extra=dict(bias_functions_file="c4_windows.json"))


def c4_controls():
    """(temperature, window centre) of every replica: replica r holds window
    r % 48 at temperature r // 48."""
    n = C4_WINDOWS * C4_TEMPS
    temps = np.repeat(np.linspace(320.0, 350.0, C4_TEMPS), C4_WINDOWS)
    centres = np.tile(2.0 * np.arange(C4_WINDOWS), C4_TEMPS)
    return n, temps, centres


# ------------------------------------------------------------- mixed ---
# Batching across capacity classes: the c2 systems (8-24 domains, small
# class, staple moves) and the c4 design (96 domains, large class, scaffold
# regrowth) in one batch of 4096 + 384 replicas.  The per-class batch
# (ldo_batch_*: one engine per class, launched together) against one engine
# that promotes every replica to the largest class and compiles the scaffold
# moves in for all; both autotuned, the same replicas, seeds and steps (the
# trajectories are identical, only the time differs).
MIXED_STEPS_PER_STEP = 960   # 10 sweeps of the 96-domain design, 40-120 of the c2 systems


def run_mixed(args):
    from latticednaorigami_gb300 import Batch, Engine
    tmp = tempfile.mkdtemp()
    files = write_c2(tmp) + [write_c4(tmp)]
    per = N_REP // len(SIZES)
    n4, temps4, _ = c4_controls()
    sys_of = np.concatenate([np.repeat(np.arange(len(SIZES)), per), np.full(n4, len(SIZES))])
    temps = np.concatenate([replica_temps(), temps4])
    n = len(sys_of)
    steps = MIXED_STEPS_PER_STEP
    attempts = n * steps

    def arm(make):
        x = make()
        x.set_controls(temps=temps)
        tune = x.autotune(probe_sweeps=1)
        for _ in range(args.warmup):
            x.run(steps)
        clocks = ClockSampler()
        clocks.start()
        c0 = x.counters()[0]
        dev_ms = [x.run(steps) for _ in range(args.steps)]
        launches = x.counters()[0] - c0
        clk = clocks.stop()
        x.close()
        tune = tune if isinstance(tune, list) else [tune]
        return {"ms_per_step": float(np.mean(dev_ms)), "move_attempts_per_s": attempts / (np.mean(dev_ms) / 1000.0),
                "autotune": [{k: v for k, v in t.items() if k != "candidates"} for t in tune],
                "gpu_launches": launches, "clocks": clk}

    def groups():
        b = Batch(files, n, seed=0, sys_of_replica=sys_of.tolist())
        info = [{"class": g["cls"], "replicas": int(len(g["replicas"])),
                 "state_bytes": int(g["engine"].state_bytes())} for g in b.groups]
        b.close()
        return info

    batch = arm(lambda: Batch(files, n, seed=0, sys_of_replica=sys_of.tolist()))
    one = arm(lambda: Engine(files, n, seed=0, sys_of_replica=sys_of.tolist()))
    line = {"metric": "move attempts/s, mixed-class batch", "value": batch["move_attempts_per_s"],
            "unit": "move attempts/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": batch["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mixed: the c2 systems (4096 replicas, 8-24 domains) and the c4 design (384 "
                                   "replicas, 96 domains, scaffold regrowth) in one batch, %d steps of every "
                                   "replica per step" % steps, "replicas": n,
                       "l2": "state resident in shared memory; no L2 flush needed"},
            "groups": groups(), "per_class_batch": batch, "one_engine_largest_class": one,
            "gain_over_one_engine": one["ms_per_step"] / batch["ms_per_step"],
            "gpu_launches": batch["gpu_launches"], "clocks": batch["clocks"]}
    print(json.dumps(line))


def c4_cpu(inp, burn, rec):
    """The oracle port on all host cores: C4_CPU_REPS replicas spread over the
    windows and temperatures, the same burn-in and recorded sweeps."""
    from oracle_lib import run_batch_sampled_centres
    from latticednaorigami_gb300.analysis import effective_samples
    n, temps, centres = c4_controls()
    pick = np.linspace(0, n - 1, C4_CPU_REPS).astype(int)
    cores = os.cpu_count() or 1
    t, smp = run_batch_sampled_centres(inp, 0, C4_CPU_REPS, burn + rec, 96, cores, temps[pick], "win", centres[pick])
    ess, tau = effective_samples(list(smp[:, burn:]))
    t_rec = t * rec / float(burn + rec)
    return {"value": ess / t_rec, "unit": "effective samples/s", "cores": cores, "kind": "port",
            "sample": "%d replicas (every %dth window x temperature) x %d recorded sweeps after %d burn-in, "
                      "%d threads" % (C4_CPU_REPS, n // C4_CPU_REPS, rec, burn, cores),
            "sweeps_per_s": C4_CPU_REPS * rec / t_rec, "tau_int_median": tau}


def run_c4(args, impl):
    from latticednaorigami_gb300.analysis import effective_samples
    tmp = tempfile.mkdtemp()
    inp = write_c4(tmp)
    n, temps, centres = c4_controls()
    total = args.steps * C4_SWEEPS_PER_STEP
    metric = "effective samples/s (tau_int of #bound domains), umbrella windows x temperatures, scaffold regrowth"
    workload = ("c4: 96-domain ThreeQuarterTurn design (16 three- and 24 two-domain staple types, 8 bp, NN), "
                "48 harmonic windows (k=0.5, centres 0..94) x 8 temperatures 320..350 K = 384 replicas, 1 uM; "
                "reference standard moveset with CTRG contiguous and jump scaffold regrowth")
    if impl == "reference":
        cpu = c4_cpu(inp, args.warmup * C4_SWEEPS_PER_STEP, total)
        line = {"impl": "reference", "metric": metric, "value": cpu["value"], "unit": "effective samples/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": workload}, "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "effective samples/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    from latticednaorigami_gb300 import Engine
    eng = Engine(inp, n_replicas=n, seed=0)
    eng.set_controls(temps=temps)
    for r in range(n):
        eng.set_bias_centre("win", r, centres[r])
    eng.set_sampling(1, total)
    for _ in range(args.warmup):
        eng.run_sweeps(C4_SWEEPS_PER_STEP)
    eng.set_sampling(1, total)
    clocks = ClockSampler()
    clocks.start()
    n0 = eng.counters()[0]
    dev_ms = [eng.run_sweeps(C4_SWEEPS_PER_STEP) for _ in range(args.steps)]
    launches = eng.counters()[0] - n0
    clk = clocks.stop()
    t_dev = sum(dev_ms) / 1000.0
    smp, cnt = eng.samples()
    ess, tau = effective_samples([smp[r, :cnt[r], 0] for r in range(n)])
    stats = eng.move_stats(5)
    # e2e: the same loop with controls uploaded and samples read every step
    eng2 = Engine(inp, n_replicas=n, seed=1)
    for r in range(n):
        eng2.set_bias_centre("win", r, centres[r])
    eng2.set_controls(temps=temps)
    eng2.set_sampling(1, C4_SWEEPS_PER_STEP)
    for _ in range(args.warmup):
        eng2.run_sweeps(C4_SWEEPS_PER_STEP)
    series = [[] for _ in range(n)]
    c0 = eng2.counters()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng2.set_controls(temps=temps)
        eng2.set_sampling(1, C4_SWEEPS_PER_STEP)
        eng2.run_sweeps(C4_SWEEPS_PER_STEP)
        s2, c2 = eng2.samples()
        for r in range(n):
            series[r].append(s2[r, :c2[r], 0])
    t_e2e = time.perf_counter() - t0
    c1 = eng2.counters()
    e2e_ess, _ = effective_samples([np.concatenate(x) for x in series])
    lay_bytes = eng.state_bytes()
    alg_bytes = n * lay_bytes * 2 + n * C4_SWEEPS_PER_STEP * 4
    achieved = alg_bytes / (np.mean(dev_ms) / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    obs = eng.observables()
    line = {"metric": metric, "value": ess / t_dev, "unit": "effective samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(dev_ms)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "sweeps_per_step": C4_SWEEPS_PER_STEP, "replicas": n,
                       "l2": "state resident in shared memory; no L2 flush needed"},
            "sweeps_per_s": n * total / t_dev, "move_attempts_per_s": n * 96 * total / t_dev,
            "tau_int_median": tau,
            "fully_bound_mean_by_temperature": [float(np.mean([obs[r]["num_fully_bound"]
                                                               for r in range(t * C4_WINDOWS, (t + 1) * C4_WINDOWS)]))
                                                for t in range(C4_TEMPS)],
            "move_stats": stats.tolist(),
            "e2e": {"value": e2e_ess / t_e2e, "unit": "effective samples/s",
                    "h2d_bytes_per_step": (c1[1] - c0[1]) / args.steps, "d2h_bytes_per_step": (c1[2] - c0[2]) / args.steps,
                    "gpu_launches_per_step": (c1[0] - c0[0]) / args.steps},
            "gpu_launches": launches,   # counted by the engine: per step the MC kernel and the status fold
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind},
            "clocks": clk}
    if not args.no_cpu:
        line["cpu_baseline"] = c4_cpu(inp, args.warmup * C4_SWEEPS_PER_STEP, total)
    print(json.dumps(line))


# ---------------------------------------------------------------- c3 ---
# The 48-domain parallel-tempering workload (the learned proposal's target
# system): the 48-domain HalfTurn scaffold with 24 two-domain staple types,
# nearest-neighbour energies of seeded 16-mers, 1 uM; 64 temperatures
# geometric over 310-370 K x 32 independent ladders = 2048 replicas, uT
# exchange (temperature and staple chemical potential, UTPTGCMCSimulation)
# every 1000 steps.  Both arms start from the same configurations: a plain PT
# burn-in of C3_BURN_ROUNDS rounds from the empty scaffold, imported by
# temperature slot.  Samples: the number of fully bound domains every 100
# steps; effective samples are counted on the per-temperature series (the
# replica at each slot, followed through the permutations of the .swp rows).
C3_RUNGS, C3_LADDERS, C3_INTERVAL, C3_SAMPLE = 64, 32, 1000, 100
C3_TEMPS = [310.0 * (370.0 / 310.0) ** (k / 63.0) for k in range(64)]
C3_ROUNDS_PER_STEP = 25
# Burn-in: C3_BURN_ROUNDS rounds of plain PT from the empty scaffold (the
# network's first training data), then C3_RELAX_ROUNDS rounds of PT with the
# learned moveset, which samples the same distribution and assembles the
# low-temperature rungs far faster, then the network trained again on those
# states.  Both timed arms start from the result, imported by slot.
C3_BURN_ROUNDS = 200
C3_RELAX_ROUNDS = 800
C3_CPU_REPS = 128
# The network's training set: C3_TRAIN_CONFIGS configurations sampled by
# plain PT at the 64 temperatures after the burn-in (one collection of all
# 2048 replicas every C3_TRAIN_EVERY steps, exchanges at the same interval).
C3_TRAIN_CONFIGS = 10_000_000
C3_TRAIN_EVERY = 100


def write_c3(d):
    import systems
    return systems.write_case(d, "c3", extra=dict(temps=" ".join(repr(t) for t in C3_TEMPS), num_reps=C3_RUNGS,
                                                    exchange_interval=C3_INTERVAL))


def c3_slot_series(smp, rows, rounds):
    """Per-temperature-slot series: rows[l][k] is ladder l's permutation
    (slot -> replica within the ladder) during round k; every round holds
    C3_INTERVAL / C3_SAMPLE samples of each replica."""
    per = C3_INTERVAL // C3_SAMPLE
    out = {}
    for l in range(C3_LADDERS):
        for q in range(C3_RUNGS):
            parts = []
            for k in range(rounds):
                r = l * C3_RUNGS + rows[l][k][q]
                parts.append(smp[r, k * per:(k + 1) * per, 0])
            out[(l, q)] = np.concatenate(parts).astype(np.float64)
    return out


def read_swp_rows(path, rounds):
    with open(path) as f:
        lines = [x.split() for x in f.read().splitlines()]
    rows = [[int(v) for v in x] for x in lines[1:] if x]
    return rows[:rounds]


def kl_noise(p_counts, q_counts, ess_p, ess_q):
    """Expected plug-in KL of two samples of one distribution: (k - 1) / 2 x
    (1/N_p + 1/N_q), k occupied bins, N the effective sample counts (the
    first-order bias of the plug-in estimator)."""
    k = int(np.count_nonzero(np.asarray(p_counts) + np.asarray(q_counts)))
    return 0.5 * max(k - 1, 0) * (1.0 / max(ess_p, 1e-9) + 1.0 / max(ess_q, 1e-9))


def kl_divergence(p_counts, q_counts, eps=1e-9):
    p = np.asarray(p_counts, np.float64) + eps
    q = np.asarray(q_counts, np.float64) + eps
    p /= p.sum()
    q /= q.sum()
    return float(np.sum(p * np.log(p / q)))


def run_c3(args, impl):
    from latticednaorigami_gb300.analysis import replica_ess, bootstrap_sum, tau_int
    tmp = tempfile.mkdtemp()
    inp = write_c3(tmp)
    learned_over = "movetype_file = %s" % write_learned_moves(tmp)
    n = C3_RUNGS * C3_LADDERS
    rounds = args.steps * C3_ROUNDS_PER_STEP
    metric = "effective samples/s (tau_int of #bound domains per temperature), learned vs plain PTMC"
    workload = ("c3: 48-domain HalfTurn scaffold, 24 two-domain staple types, NN energies of seeded 16-mers, 1 uM; "
                "64 temperatures geometric 310-370 K x 32 ladders = 2048 replicas, uT exchange every 1000 steps; "
                "learned staple exchange + learned regrowth + CB regrowth (value) vs Met exchange + Met regrowth + "
                "CB regrowth (plain)")
    if impl == "reference":
        cpu = c3_cpu(inp, rounds)
        line = {"impl": "reference", "metric": metric, "value": cpu["value"], "unit": "effective samples/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": workload}, "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "effective samples/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    from latticednaorigami_gb300 import Engine
    t_burn0 = time.perf_counter()
    # plain PT burn-in from the empty scaffold, then the network's training data
    burn = Engine(inp, n_replicas=n, seed=900)
    burn.autotune(probe_sweeps=2)
    done = 0
    while done < C3_BURN_ROUNDS:
        k = min(100, C3_BURN_ROUNDS - done)
        burn.pt_run(C3_RUNGS, k, C3_INTERVAL, 3)
        done += k
    # the training set: plain PT configurations at the 64 temperatures
    t_collect0 = time.perf_counter()
    n_collect = -(-C3_TRAIN_CONFIGS // n)
    for _ in range(n_collect):
        burn.pt_run(C3_RUNGS, 1, C3_TRAIN_EVERY, 3)
        burn.learn_collect()
    collect_s = time.perf_counter() - t_collect0
    t_train0 = time.perf_counter()
    loss0, loss1 = burn.learn_train(LEARN_ITERS, lr=LEARN_LR, seed=0)
    table = burn.learn_table()
    train_s = time.perf_counter() - t_train0
    perm = burn.pt_permutation()
    mid = [burn.config(int(perm[s])) for s in range(n)]   # by slot
    burn.close()
    # the learned moveset relaxes the low-temperature rungs the plain burn-in
    # leaves unassembled; both timed arms start from its configurations
    relax = Engine(inp, n_replicas=n, seed=901, overrides=learned_over)
    relax.learn_set_table(table)
    relax.set_configs(mid)
    relax.autotune(probe_sweeps=2)
    done = 0
    while done < C3_RELAX_ROUNDS:
        k = min(100, C3_RELAX_ROUNDS - done)
        relax.pt_run(C3_RUNGS, k, C3_INTERVAL, 3)
        done += k
    perm = relax.pt_permutation()
    start = [relax.config(int(perm[s])) for s in range(n)]   # by slot
    relax.close()
    low_slot_configs = [start[l * C3_RUNGS] for l in range(C3_LADDERS)]
    burn_s = time.perf_counter() - t_burn0

    def arm(overrides, tab, seed):
        eng = Engine(inp, n_replicas=n, seed=seed, overrides=overrides)
        if tab is not None:
            eng.learn_set_table(tab)
        eng.set_configs(start)
        tune = eng.autotune(probe_sweeps=2)
        writers = [eng.open_swap_writer(C3_RUNGS, 3, l, os.path.join(tmp, "%d_lad%d" % (seed, l)), C3_INTERVAL)
                   for l in range(C3_LADDERS)]
        for _ in range(args.warmup):
            eng.pt_run(C3_RUNGS, C3_ROUNDS_PER_STEP, C3_INTERVAL, 3)
        for w in writers:
            w.close()
        writers = [eng.open_swap_writer(C3_RUNGS, 3, l, os.path.join(tmp, "%d_rec%d" % (seed, l)), C3_INTERVAL)
                   for l in range(C3_LADDERS)]
        eng.set_sampling(C3_SAMPLE, rounds * (C3_INTERVAL // C3_SAMPLE))
        clocks = ClockSampler()
        clocks.start()
        dev_ms = []
        n0 = eng.counters()[0]
        for _ in range(args.steps):
            dev_ms.append(eng.pt_run(C3_RUNGS, C3_ROUNDS_PER_STEP, C3_INTERVAL, 3))
            for w in writers:
                w.write(-1)
        launches = eng.counters()[0] - n0
        clk = clocks.stop()
        for w in writers:
            w.close()
        smp, cnt = eng.samples()
        rows = [read_swp_rows(os.path.join(tmp, "%d_rec%d.swp" % (seed, l)), rounds) for l in range(C3_LADDERS)]
        series = c3_slot_series(smp, rows, rounds)
        keys = sorted(series)
        ess = replica_ess([series[k] for k in keys])
        t = sum(dev_ms) / 1000.0
        (lo, hi), boot = bootstrap_sum(ess, [q for (_, q) in keys])
        hist = np.zeros((C3_RUNGS, 49))
        halves = np.zeros((2, C3_RUNGS, 49))   # ladders 0-15 and 16-31 apart
        for (l, q), x in series.items():
            hb = np.bincount(x.astype(int), minlength=49)[:49]
            hist[q] += hb
            halves[l * 2 // C3_LADDERS, q] += hb
        half = len(series[keys[0]]) // 2
        top = [series[(l, C3_RUNGS - 1)] for l in range(C3_LADDERS)]
        taus = [tau_int(series[k]) for k in keys]
        st = eng.move_stats(3)
        att, acc = eng.pt_stats(C3_RUNGS - 1)
        ess_by_rung = np.zeros(C3_RUNGS)
        for (l, q), e_ in zip(keys, ess):
            ess_by_rung[q] += e_
        res = {"value": float(ess.sum()) / t, "ci95": [lo / t, hi / t], "boot": boot / t,
               "ess_by_rung": ess_by_rung, "dev_ms": dev_ms, "attempts": float(st[:, 0].sum()),
               "launches": launches,
               "sweeps_per_s": n * rounds * C3_INTERVAL / 48.0 / t,
               "ms_per_step": float(np.mean(dev_ms)), "tau_int_median_samples": float(np.median([x for x in taus if x])),
               "mean_fully_bound_by_temperature": [float(hist[q] @ np.arange(49) / hist[q].sum()) for q in
                                                   range(C3_RUNGS)],
               "max_rung_drift_between_halves": float(max(
                   abs(np.mean([series[(l, q)][:half].mean() for l in range(C3_LADDERS)]) -
                       np.mean([series[(l, q)][half:].mean() for l in range(C3_LADDERS)]))
                   for q in range(C3_RUNGS))),
               "top_rung_mean_first_half": float(np.mean([x[:half].mean() for x in top])),
               "top_rung_mean_second_half": float(np.mean([x[half:].mean() for x in top])),
               "acceptance": {"exchange": float(st[0, 1]) / max(1.0, float(st[0, 0])),
                              "regrowth": float(st[1, 1]) / max(1.0, float(st[1, 0])),
                              "cb_regrowth": float(st[2, 1]) / max(1.0, float(st[2, 0]))},
               "swap_acceptance_mean": float(acc.sum()) / max(1.0, float(att.sum())),
               "autotune": {k: v for k, v in tune.items() if k != "candidates"}, "clocks": clk,
               "kl_between_ladder_halves": [kl_divergence(halves[0, q], halves[1, q]) for q in range(C3_RUNGS)]}
        eng.close()
        return res, hist

    def e2e_arm(overrides, tab, seed):
        """The learned arm end to end through the C ABI with host buffers:
        inside the timed region the start configurations are uploaded from
        host memory, then every step runs its rounds and reads back that
        step's samples and slot permutations (the .swp rows)."""
        eng = Engine(inp, n_replicas=n, seed=seed, overrides=overrides)
        eng.learn_set_table(tab)
        eng.autotune(probe_sweeps=2)   # the timed arm's shape (cached)
        writers = [eng.open_swap_writer(C3_RUNGS, 3, l, os.path.join(tmp, "%d_e2e%d" % (seed, l)), C3_INTERVAL)
                   for l in range(C3_LADDERS)]
        per = C3_INTERVAL // C3_SAMPLE
        flat = [np.asarray(c, np.int32) for c in start]
        parts = []
        c0 = eng.counters()
        t0 = time.perf_counter()
        eng.set_configs(flat)
        for _ in range(args.steps):
            eng.set_sampling(C3_SAMPLE, C3_ROUNDS_PER_STEP * per)
            eng.pt_run(C3_RUNGS, C3_ROUNDS_PER_STEP, C3_INTERVAL, 3)
            s_, c_ = eng.samples()
            for w in writers:
                w.write(-1)
            parts.append(s_)
        t = time.perf_counter() - t0
        c1 = eng.counters()
        for w in writers:
            w.close()
        eng.close()
        smp = np.concatenate(parts, axis=1)
        rows = [read_swp_rows(os.path.join(tmp, "%d_e2e%d.swp" % (seed, l)), rounds) for l in range(C3_LADDERS)]
        series = c3_slot_series(smp, rows, rounds)
        ess = replica_ess([series[k] for k in sorted(series)])
        return {"value": float(ess.sum()) / t, "unit": "effective samples/s",
                "h2d_bytes_per_step": (c1[1] - c0[1]) / args.steps, "d2h_bytes_per_step": (c1[2] - c0[2]) / args.steps,
                "gpu_launches_per_step": (c1[0] - c0[0]) / args.steps,
                "note": "start configurations uploaded once inside the timed region (bytes spread over the steps); "
                        "bytes and launches counted by the engine"}

    plain, h_plain = arm("", None, 0)
    learned, h_learned = arm(learned_over, table, 1)
    e2e = e2e_arm(learned_over, table, 2)
    kl = [kl_divergence(h_plain[q], h_learned[q]) for q in range(C3_RUNGS)]
    noise = [kl_noise(h_plain[q], h_learned[q], plain["ess_by_rung"][q], learned["ess_by_rung"][q])
             for q in range(C3_RUNGS)]
    q_max = int(np.argmax(kl))
    ratio_boot = learned.pop("boot") / plain.pop("boot")

    def roofline(res, kind):
        # shared-memory roofline as for c2: algorithmic bytes per attempt
        # (oracle touch counts on this system) x attempts per launch
        t_launch = float(np.mean(res["dev_ms"])) / 1000.0 / C3_ROUNDS_PER_STEP
        att = res["attempts"] / (rounds + args.warmup * C3_ROUNDS_PER_STEP)
        sm_mhz = res["clocks"].get("sm_mhz") or 2070.0
        peak = N_SM * SMEM_BYTES_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e9
        achieved = att * B_ATTEMPT_C3[kind] / t_launch / 1e9
        return {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": "derived: 152 SMs x 128 B/clk x median SM clock %.0f MHz" % sm_mhz,
                "bytes_per_attempt": B_ATTEMPT_C3[kind], "attempts_per_launch": att,
                "launch": "one round: 1000 steps of every replica (then the exchange kernel)",
                "traffic": None, "traffic_source": "no capture of this workload"}

    for res in (plain, learned):
        # the arm's own spread: KL between its two halves of ladders, at the
        # temperature of the largest plain-vs-learned KL and at its largest
        self_kl = res.pop("kl_between_ladder_halves")
        res["kl_between_ladder_halves"] = {"at_argmax_K": self_kl[q_max], "max": max(self_kl),
                                           "mean": float(np.mean(self_kl))}
        res["roofline"] = roofline(res, "learned" if res is learned else "plain")
        res.pop("dev_ms")
        res.pop("attempts")
        res["gpu_launches"] = res.pop("launches")
        res["ess_by_rung"] = [float(x) for x in res["ess_by_rung"]]

    # constant-temperature references at the top temperature: from the empty
    # scaffold and from the burn-in's lowest-temperature configurations
    def const_t(configs):
        e = Engine(inp, n_replicas=C3_LADDERS, seed=77)
        e.set_controls(temps=[C3_TEMPS[-1]] * C3_LADDERS)
        if configs is not None:
            e.set_configs(configs)
        e.run(rounds * C3_INTERVAL // 2)
        e.set_sampling(C3_SAMPLE, rounds * C3_INTERVAL // 2 // C3_SAMPLE)
        e.run(rounds * C3_INTERVAL // 2)
        s_, c_ = e.samples()
        e.close()
        return float(np.mean([s_[r, :c_[r], 0].mean() for r in range(C3_LADDERS)]))

    ref_empty = const_t(None)
    ref_assembled = const_t(low_slot_configs)
    value = learned["value"]
    line = {"metric": metric, "value": value, "unit": "effective samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": learned["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "rounds_per_step": C3_ROUNDS_PER_STEP, "replicas": n,
                       "start": "both arms from the same configurations: %d rounds of plain PT from the empty "
                                "scaffold, the training collection, then %d rounds of PT with the learned moveset, "
                                "imported by temperature slot" % (C3_BURN_ROUNDS, C3_RELAX_ROUNDS),
                       "l2": "state resident in shared memory; no L2 flush needed"},
            "ci95": learned["ci95"], "learned": learned, "plain": plain,
            "learned_over_plain": value / plain["value"],
            "learned_over_plain_ci95": [float(np.quantile(ratio_boot, 0.025)), float(np.quantile(ratio_boot, 0.975))],
            "kl_plain_learned_by_temperature": {"max": max(kl), "mean": float(np.mean(kl)),
                                                "top": kl[-1], "bottom": kl[0], "argmax_K": C3_TEMPS[q_max],
                                                "sampling_noise_at_argmax": noise[q_max],
                                                "max_excess_over_noise": float(max(k - z for k, z in zip(kl, noise))),
                                                "noise": "(occupied bins - 1)/2 x (1/ESS_plain + 1/ESS_learned) "
                                                         "per temperature"},
            "stationarity": {"top_rung_370K_plain": plain["mean_fully_bound_by_temperature"][-1],
                             "top_rung_370K_learned": learned["mean_fully_bound_by_temperature"][-1],
                             "constant_T_370K_from_empty": ref_empty,
                             "constant_T_370K_from_assembled": ref_assembled},
            "network": {"train_iters": LEARN_ITERS, "loss_first": loss0, "loss_last": loss1, "train_s": train_s,
                        "training_configurations": n_collect * n, "collect_s": collect_s,
                        "training_set": "plain PT at the 64 temperatures, all 2048 replicas every %d steps after "
                                        "the burn-in" % C3_TRAIN_EVERY},
            "burn_in_s": burn_s, "roofline": learned["roofline"], "e2e": e2e,
            # counted by the engine: per step C3_ROUNDS_PER_STEP rounds of the MC
            # kernel and the exchange kernel (graph replays), and the status fold
            "gpu_launches": learned["gpu_launches"]}
    if not args.no_cpu:
        line["cpu_baseline"] = c3_cpu(inp, min(rounds, 500))
    print(json.dumps(line))


def c3_cpu(inp, rounds):
    """The oracle port on all usable host cores: two constant-temperature
    chains at each of the 64 temperatures (the PT exchange is omitted, as in
    the reference's CPU baseline plan), burn-in then recorded samples every
    100 steps."""
    from oracle_lib import run_batch_sampled
    from latticednaorigami_gb300.analysis import replica_ess, bootstrap_sum
    cores, present = host_cores()
    temps = np.repeat(C3_TEMPS, C3_CPU_REPS // C3_RUNGS)
    burn = 2000
    rec = rounds * C3_INTERVAL // C3_SAMPLE
    t, smp = run_batch_sampled(inp, 0, C3_CPU_REPS, burn + rec, C3_SAMPLE, cores, temps=temps)
    ess = replica_ess(list(smp[:, burn:]))
    t_rec = t * rec / float(burn + rec)
    (lo, hi), _ = bootstrap_sum(ess)
    return {"value": float(ess.sum()) / t_rec, "ci95": [lo / t_rec, hi / t_rec], "unit": "effective samples/s",
            "cores": cores, "cores_present_on_host": present, "kind": "port",
            "sample": "%d constant-T chains (2 per temperature, no exchange) x %d samples every 100 steps after %d "
                      "burn-in samples, %d threads" % (C3_CPU_REPS, rec, burn, cores),
            "sweeps_per_s": C3_CPU_REPS * (rec * C3_SAMPLE / 48.0) / t_rec}


def main():
    global C4_SWEEPS_PER_STEP, SWEEPS_PER_STEP
    global C3_BURN_ROUNDS, C3_ROUNDS_PER_STEP, C3_RELAX_ROUNDS, C3_TRAIN_CONFIGS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "mixed"],
                    help="c2: the learned-vs-plain headline workload; c3: the 48-domain PTMC learned-vs-plain "
                         "workload; c4: the 96-domain umbrella workload; mixed: c2 and c4 in one batch, split "
                         "by capacity class against one engine")
    ap.add_argument("--c3-burn-rounds", type=int, default=0, help="c3 only: PT rounds of the plain burn-in")
    ap.add_argument("--c3-relax-rounds", type=int, default=0,
                    help="c3 only: PT rounds of the learned relaxation after the burn-in")
    ap.add_argument("--c3-rounds-per-step", type=int, default=0, help="c3 only: PT rounds per timed step")
    ap.add_argument("--c3-train-configs", type=int, default=0,
                    help="c3 only: plain-PT configurations the network is trained on (default %d)" % C3_TRAIN_CONFIGS)
    ap.add_argument("--sweeps-per-step", type=int, default=0,
                    help="sweeps per launch (default c2 %d, c4 %d); small values make short profiler captures"
                         % (SWEEPS_PER_STEP, C4_SWEEPS_PER_STEP))
    args = ap.parse_args()
    if args.sweeps_per_step > 0:
        C4_SWEEPS_PER_STEP = args.sweeps_per_step
        SWEEPS_PER_STEP = args.sweeps_per_step
    rank = int(os.environ.get("RANK", "0"))
    if args.c3_train_configs > 0:
        C3_TRAIN_CONFIGS = args.c3_train_configs
    if args.c3_burn_rounds > 0:
        C3_BURN_ROUNDS = args.c3_burn_rounds
    if args.c3_relax_rounds > 0:
        C3_RELAX_ROUNDS = args.c3_relax_rounds
    if args.c3_rounds_per_step > 0:
        C3_ROUNDS_PER_STEP = args.c3_rounds_per_step
    if args.workload == "c3":
        if rank == 0:
            run_c3(args, args.impl)
        return
    if args.workload == "c4":
        # single-GPU workload (384 replicas): other ranks have nothing to do
        if rank == 0:
            run_c4(args, args.impl)
        return
    if args.workload == "mixed":
        if rank == 0:
            if args.impl == "reference":
                print(json.dumps({"impl": "reference", "unavailable": "the reference runs one system per "
                                  "process; it has no batch to split"}))
            else:
                run_mixed(args)
        return
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args)
        return
    ranks = Ranks()
    from latticednaorigami_gb300 import Engine
    from latticednaorigami_gb300.analysis import (bootstrap_sum, effective_samples, replica_ess, tau_int,
                                                  tau_vs_length)

    tmp = tempfile.mkdtemp()
    files = write_c2(tmp)
    learned_over = "movetype_file = %s" % write_learned_moves(tmp)
    per = N_REP // len(SIZES)
    sys_of = np.repeat(np.arange(len(SIZES)), per)
    temps = replica_temps()
    ns_of = np.array(SIZES)[sys_of]
    total_sweeps = args.steps * SWEEPS_PER_STEP

    overhead = {"collect_s": 0.0, "train_s": 0.0}

    def collect_and_train(eng):
        """Network inputs and labels from 10 states 10 sweeps apart, then
        LEARN_ITERS Adam steps (untimed; their wall time is the learned
        proposal's own overhead, amortised in value_amortised)."""
        t0 = time.perf_counter()
        for _ in range(10):
            eng.run_sweeps(10)
            eng.learn_collect()
        overhead["collect_s"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        loss0, loss1 = eng.learn_train(LEARN_ITERS, lr=LEARN_LR, seed=0)
        dt = time.perf_counter() - t0
        overhead["train_s"] += dt
        return {"loss_first": loss0, "loss_last": loss1, "iters": LEARN_ITERS, "train_s": dt,
                "table": eng.learn_table()}

    def relax():
        """Stationary starting configurations: a first network trained on a
        short plain run from the empty scaffolds, RELAX_SWEEPS sweeps of the
        learned moveset with it, the network trained again on those states."""
        e0 = Engine(files, n_replicas=N_REP, seed=500 + ranks.rank, sys_of_replica=sys_of.tolist())
        e0.set_controls(temps=temps)
        for _ in range(3):
            e0.run_sweeps(100)
        table0 = collect_and_train(e0)["table"]
        e0.close()
        e1 = Engine(files, n_replicas=N_REP, seed=600 + ranks.rank, sys_of_replica=sys_of.tolist(),
                    overrides=learned_over)
        e1.set_controls(temps=temps)
        e1.learn_set_table(table0)
        for _ in range(RELAX_SWEEPS // 100):
            e1.run_sweeps(100)
        train = collect_and_train(e1)
        start = [e1.config(r) for r in range(N_REP)]
        e1.close()
        return start, train

    start, train = relax()

    def timed_arm(overrides, table, label):
        """From the relaxed configurations: W warm-up launches, then K timed
        launches of SWEEPS_PER_STEP sweeps with one numfulldomains sample per
        replica per sweep (inside the NVTX range "<label>_timed")."""
        eng = Engine(files, n_replicas=N_REP, seed=ranks.rank, sys_of_replica=sys_of.tolist(), overrides=overrides)
        eng.set_controls(temps=temps)
        if table is not None:
            eng.learn_set_table(table)
        eng.set_configs(start)
        # the engine's autotuner picks the launch shape on this batch (state
        # restored after every probe: the trajectories are unchanged)
        tune = eng.autotune(probe_sweeps=4)
        tune = {k: v for k, v in tune.items() if k != "candidates"}
        tune["gain_over_default"] = tune["default_ms"] / tune["best_ms"] if tune["best_ms"] > 0 else None
        eng.set_sampling(1, total_sweeps)
        for _ in range(args.warmup):
            eng.run_sweeps(SWEEPS_PER_STEP)
        eng.set_sampling(1, total_sweeps)
        clocks = ClockSampler()
        clocks.start()
        ranks.barrier()
        n0 = eng.counters()[0]
        with nvtx_range(label + "_timed"):
            dev_ms = [eng.run_sweeps(SWEEPS_PER_STEP) for _ in range(args.steps)]   # each call ends synchronised
        launches = eng.counters()[0] - n0
        ranks.barrier()
        clk = clocks.stop()
        t_dev = ranks.max(sum(dev_ms) / 1000.0)
        smp, cnt = eng.samples()
        series = [smp[r, :cnt[r], 0] for r in range(N_REP)]
        per_rep = replica_ess(series)
        ess = ranks.sum(float(per_rep.sum()))
        (lo, hi), boot = bootstrap_sum(per_rep, sys_of)
        taus, means = {}, {}
        for i, n in enumerate(SIZES):
            ts = [tau_int(series[r]) for r in range(i * per, (i + 1) * per)]
            ts = [t for t in ts if t is not None]
            taus[n] = float(np.median(ts)) if ts else None
            means[n] = float(np.mean(np.concatenate(series[i * per:(i + 1) * per])))
        big = [series[r] for r in range(3 * per, 4 * per)]
        tvl = tau_vs_length(big, [L for L in (500, 1000, 2000, 5000, 10000) if L <= total_sweeps])
        tau_med = float(np.median([t for t in (tau_int(x) for x in series) if t is not None]))
        st = eng.move_stats(3)
        acc = [float(st[k, 1]) / max(1.0, float(st[k, 0])) for k in range(3)]
        return {"eng": eng, "dev_ms": dev_ms, "t_dev": t_dev, "ess": ess, "boot": boot / t_dev,
                "ci95": [lo / t_dev, hi / t_dev], "tau_med": tau_med, "taus": taus, "tau_vs_length_24": tvl,
                "means": means, "clk": clk, "acc": acc, "tune": tune, "launches": launches}

    def e2e_arm(overrides, table):
        """The same loop through the C ABI with host buffers: temperatures in,
        samples out, every step."""
        eng2 = Engine(files, n_replicas=N_REP, seed=1000 + ranks.rank, sys_of_replica=sys_of.tolist(),
                      overrides=overrides)
        eng2.set_controls(temps=temps)
        if table is not None:
            eng2.learn_set_table(table)
        eng2.set_configs(start)
        eng2.autotune(probe_sweeps=4)   # the shape found for the timed arm (cached)
        eng2.set_sampling(1, SWEEPS_PER_STEP)
        for _ in range(args.warmup):
            eng2.run_sweeps(SWEEPS_PER_STEP)
        e2e_series = [[] for _ in range(N_REP)]
        ranks.barrier()
        c0 = eng2.counters()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng2.set_controls(temps=temps)
            eng2.set_sampling(1, SWEEPS_PER_STEP)
            eng2.run_sweeps(SWEEPS_PER_STEP)
            s2, c2 = eng2.samples()
            for r in range(N_REP):
                e2e_series[r].append(s2[r, :c2[r], 0])
        t_e2e = time.perf_counter() - t0
        c1 = eng2.counters()
        ranks.barrier()
        t_e2e = ranks.max(t_e2e)
        e2e_ess, _ = effective_samples([np.concatenate(x) for x in e2e_series])
        eng2.close()
        return ranks.sum(e2e_ess) / t_e2e, [(b - a) / args.steps for a, b in zip(c0, c1)]

    table = train["table"]
    plain = timed_arm("", None, "plain")
    learned = timed_arm(learned_over, table, "learned")
    value = learned["ess"] / learned["t_dev"]
    plain_value = plain["ess"] / plain["t_dev"]
    ratio_boot = learned["boot"] / plain["boot"]
    e2e_learned, e2e_counts = e2e_arm(learned_over, table)
    e2e_plain, _ = e2e_arm("", None)
    # per step, counted by the engine: the temperature upload (control
    # records and the energy tables of the replicas' temperatures), the
    # recompute and MC launches with their status folds, and the samples
    # read back with their counts
    e2e_launches, h2d, d2h = e2e_counts

    # Roofline of the MC kernel: shared memory (the replica state stays in it
    # for a whole launch).  achieved = move attempts per launch x algorithmic
    # bytes per attempt / launch time; peak = 152 SMs x 128 B/clk x the
    # median SM clock sampled during the timed launches.  HBM as a second
    # figure: state in + out + samples per launch against the measured copy
    # bandwidth.
    attempts_per_launch = float(np.sum(ns_of)) * SWEEPS_PER_STEP

    def roofline(arm, kind):
        t_launch = float(np.mean(arm["dev_ms"])) / 1000.0
        sm_mhz = arm["clk"].get("sm_mhz") or 2070.0
        peak = N_SM * SMEM_BYTES_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e9
        achieved = attempts_per_launch * B_ATTEMPT[kind] / t_launch / 1e9
        eng_ = arm["eng"]
        alg_hbm = N_REP * eng_.state_bytes() * 2 + N_REP * SWEEPS_PER_STEP * 4
        hbm_peak, hbm_kind = measured_peaks()
        hbm_ach = alg_hbm / t_launch / 1e9
        return {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": "derived: 152 SMs x 128 B/clk x median SM clock %.0f MHz" % sm_mhz,
                "bytes_per_attempt": B_ATTEMPT[kind], "attempts_per_launch": attempts_per_launch,
                "hbm": {"achieved": hbm_ach, "peak": hbm_peak, "frac": hbm_ach / hbm_peak, "peak_kind": hbm_kind,
                        "algorithmic_bytes_per_launch": alg_hbm}}

    rl = roofline(learned, "learned")
    tr_d, tr_src = measured_traffic("c2")
    rl["traffic"] = None
    rl["traffic_source"] = tr_src
    if tr_d:
        # per launch of SWEEPS_PER_STEP sweeps, scaled from the captured launch
        rl["traffic"] = tr_d["dram_bytes_per_launch"] * SWEEPS_PER_STEP / tr_d["sweeps_per_launch"]
    overhead_s = overhead["collect_s"] + overhead["train_s"]

    def rates(arm, kind):
        t = arm["t_dev"]
        W = ranks.world
        return {"value": arm["ess"] / t, "ci95": arm["ci95"], "sweeps_per_s": W * N_REP * total_sweeps / t,
                "move_attempts_per_s": W * float(np.sum(ns_of)) * total_sweeps / t,
                "ms_per_step": float(np.mean(arm["dev_ms"])), "tau_int_median": arm["tau_med"],
                "tau_int_by_size": arm["taus"], "tau_vs_record_length_24_domain": arm["tau_vs_length_24"],
                "mean_fully_bound_by_size": arm["means"],
                "acceptance": {"exchange": arm["acc"][0], "regrowth": arm["acc"][1], "cb_regrowth": arm["acc"][2]},
                "roofline_smem_frac": roofline(arm, kind)["frac"], "autotune": arm["tune"]}

    tr = train
    lrates = rates(learned, "learned")
    lrates["value_amortised"] = learned["ess"] / (learned["t_dev"] + overhead_s)
    lrates["learned_overhead_s"] = {"collect_s": overhead["collect_s"], "train_s": overhead["train_s"],
                                    "note": "two collections of 10 states and two trainings; value_amortised "
                                            "adds them to the timed region of this run"}
    line = {"metric": "effective samples/s (tau_int of #bound domains), learned vs plain MC", "value": value,
            "unit": "effective samples/s", "n_gpus": ranks.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(learned["dev_ms"])), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "c2: 4096 constant-T chains, scaffolds 8/12/16/24 (1024 each), uniform hyb "
                                   "dH=-120 kcal/mol dS=-0.33 kcal/mol/K, T~U[320,350] K, 1 uM; moveset "
                                   "learned staple exchange + learned regrowth + CB regrowth (value) vs Met "
                                   "exchange + Met regrowth + CB regrowth (plain)",
                       "sweeps_per_step": SWEEPS_PER_STEP, "replicas": N_REP * ranks.world,
                       "replicas_per_gpu": N_REP, "parallelism": "replicas only, one process per GPU",
                       "start": "both arms from the same configurations, relaxed %d sweeps by the learned "
                                "moveset, then %d warm-up sweeps" % (RELAX_SWEEPS, args.warmup * SWEEPS_PER_STEP),
                       "l2": "state resident in shared memory; no L2 flush needed"},
            "ci95": learned["ci95"],
            "learned": lrates, "plain": rates(plain, "plain"),
            "learned_over_plain": value / plain_value,
            "learned_over_plain_ci95": [float(np.quantile(ratio_boot, 0.025)), float(np.quantile(ratio_boot, 0.975))],
            "ci_method": "percentile bootstrap over replicas (resampled within scaffold size), 2000 resamples",
            "distribution_check": "tests/test_gpu_learned.py::test_learned_distribution_matches_plain_on_c2",
            "network": {"layers": "64-256-256-256-1 GELU, bf16 weights/activations, fp32 accumulation",
                        "train_iters": tr["iters"], "loss_first": tr["loss_first"], "loss_last": tr["loss_last"],
                        "train_s": tr["train_s"]},
            "sweeps_per_s": lrates["sweeps_per_s"],
            "e2e": {"value": e2e_learned, "unit": "effective samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "plain_value": e2e_plain, "gpu_launches_per_step": e2e_launches},
            "gpu_launches": learned["launches"],   # counted by the engine: per step the MC kernel and the status fold
            "roofline": rl,
            "clocks": learned["clk"], "clocks_plain": plain["clk"]}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline(files, CPU_BURN_SWEEPS, total_sweeps)
    if rank == 0:
        print(json.dumps(line))
    ranks.close()


if __name__ == "__main__":
    main()
