"""Benchmark of the batched plain-MC workload (4096 independent constant-T
chains of uneven size) on one GB300.

Workload: scaffolds of 8/12/16/24 domains (1024 replicas each, serpentine
layout, n/2 two-domain staple types), uniform hybridisation dH = -120 kcal/mol
and dS = -0.33 kcal/mol/K per bound domain, T ~ U[320, 350] K (seeded),
1 uM staples, FourBody, Opposing misbinding, constant stacking 1000 K, the
Met exchange / Met regrowth / CB regrowth moveset at 1/3 each.  Philox seeds:
replica r uses key (0, r).  Inputs are synthetic (tests/systems.py).

A step is one launch of SWEEPS sweeps of every replica (a sweep = n_scaffold
move attempts).  `value` is effective samples per second of the number of
fully bound domains (one sample per replica per sweep, tau_int by Sokal
windowing), from the device-timed region; `e2e` repeats the timed loop through
the C ABI with host buffers (temperatures in, samples out every step)."""
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

SWEEPS_PER_STEP = 100
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


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


CPU_REPS_PER_SIZE = 128


def replica_temps():
    """T ~ U[320, 350] K per replica (seeded); replica r has scaffold size
    SIZES[r // (N_REP / 4)]."""
    return np.random.default_rng(0).uniform(320.0, 350.0, N_REP)


def cpu_effective_rate(files, cores, burn_sweeps, rec_sweeps):
    """The oracle port on all host cores over a bounded sample of the same
    workload: CPU_REPS_PER_SIZE replicas of each scaffold size at the
    temperatures of the first replicas of that size in the GPU run, the same
    burn-in and recorded sweeps as the GPU run, tau_int estimated from its own
    samples by the same estimator.  Only the recorded sweeps are timed
    (pro rata).  Returns (effective samples/s, sweeps/s, median tau)."""
    from oracle_lib import run_batch_sampled
    from latticednaorigami_gb300.analysis import effective_samples
    temps = replica_temps()
    per = N_REP // len(SIZES)
    ess_total, t_total, sweeps_total = 0.0, 0.0, 0.0
    taus = []
    for i, f in enumerate(files):
        n = SIZES[i]
        tt = temps[i * per:i * per + CPU_REPS_PER_SIZE]
        t, smp = run_batch_sampled(f, 0, CPU_REPS_PER_SIZE, burn_sweeps + rec_sweeps, n, cores, temps=tt)
        rec = smp[:, burn_sweeps:]
        ess, tau = effective_samples(list(rec))
        frac = rec_sweeps / float(burn_sweeps + rec_sweeps)
        ess_total += ess
        t_total += t * frac
        sweeps_total += CPU_REPS_PER_SIZE * rec_sweeps
        if tau is not None:
            taus.append(tau)
    return ess_total / t_total, sweeps_total / t_total, (float(np.median(taus)) if taus else None)


def cpu_baseline(files, burn_sweeps, rec_sweeps):
    cores = os.cpu_count() or 1
    rate, sweeps_per_s, tau = cpu_effective_rate(files, cores, burn_sweeps, rec_sweeps)
    return {"value": rate, "unit": "effective samples/s", "cores": cores, "kind": "port",
            "sample": "%d replicas of each scaffold size (GPU-run temperatures) x %d recorded sweeps after %d "
                      "burn-in, %d threads" % (CPU_REPS_PER_SIZE, rec_sweeps, burn_sweeps, cores),
            "sweeps_per_s": sweeps_per_s, "tau_int_median": tau}


def run_reference_arm(args):
    """Reference arm: the CPU restatement of the reference (oracle port; the
    reference itself cannot be built on the GPU machine) on all host cores."""
    tmp = tempfile.mkdtemp()
    files = write_c2(tmp)
    cores = os.cpu_count() or 1
    from oracle_lib import run_batch
    for _ in range(args.warmup):
        run_batch(files[0], 0, cores, 20 * SIZES[0], cores)
    burn, rec = args.warmup * SWEEPS_PER_STEP, args.steps * SWEEPS_PER_STEP
    rates, sps, taus, times = [], [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r, s_, tau = cpu_effective_rate(files, cores, burn, rec)
        times.append(time.perf_counter() - t0)
        rates.append(r)
        sps.append(s_)
        taus.append(tau)
    value = float(np.mean(rates))
    line = {"impl": "reference", "metric": "effective samples/s (tau_int of #bound domains), plain MC",
            "value": value, "unit": "effective samples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "c2: constant-T chains, scaffolds 8/12/16/24, uniform hyb, T~U[320,350] K; "
                                   "bounded CPU sample per step"},
            "cpu_baseline": {"value": value, "unit": "effective samples/s", "cores": cores, "kind": "port",
                             "sample": "%d replicas of each scaffold size (GPU-run temperatures) x %d recorded "
                                       "sweeps after %d burn-in per step" % (CPU_REPS_PER_SIZE, rec, burn)},
            "e2e": {"value": value, "unit": "effective samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "sweeps_per_s": float(np.mean(sps)), "tau_int_median": taus[-1]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args)
        return
    from latticednaorigami_gb300 import Engine

    tmp = tempfile.mkdtemp()
    files = write_c2(tmp)
    per = N_REP // len(SIZES)
    sys_of = np.repeat(np.arange(len(SIZES)), per)
    temps = replica_temps()
    eng = Engine(files, n_replicas=N_REP, seed=0, sys_of_replica=sys_of.tolist(), overrides="")
    eng.set_controls(temps=temps)
    ns_of = np.array(SIZES)[sys_of]
    total_sweeps = args.steps * SWEEPS_PER_STEP
    eng.set_sampling(1, total_sweeps)   # one sample per sweep
    # warmup: run, then restart the sample ring
    for _ in range(args.warmup):
        eng.run_sweeps(SWEEPS_PER_STEP)
    eng.set_sampling(1, total_sweeps)
    clocks = ClockSampler()
    clocks.start()
    dev_ms = []
    for _ in range(args.steps):
        dev_ms.append(eng.run_sweeps(SWEEPS_PER_STEP))
    clk = clocks.stop()
    t_dev = sum(dev_ms) / 1000.0
    smp, cnt = eng.samples()
    series = [smp[r, :cnt[r], 0] for r in range(N_REP)]
    from latticednaorigami_gb300.analysis import effective_samples, tau_int
    ess, tau_med = effective_samples(series)
    taus_per_size = {}
    for i, n in enumerate(SIZES):
        ts = [tau_int(series[r]) for r in range(i * per, (i + 1) * per)]
        ts = [t for t in ts if t is not None]
        taus_per_size[n] = float(np.median(ts)) if ts else None
    value = ess / t_dev
    sweeps_per_s = N_REP * total_sweeps / t_dev
    moves_per_s = float(np.sum(ns_of)) * total_sweeps / t_dev

    # e2e through the C ABI with host buffers: temperatures in, samples out
    eng2 = Engine(files, n_replicas=N_REP, seed=1, sys_of_replica=sys_of.tolist())
    eng2.set_controls(temps=temps)
    eng2.set_sampling(1, SWEEPS_PER_STEP)
    for _ in range(args.warmup):
        eng2.run_sweeps(SWEEPS_PER_STEP)
    e2e_series = [[] for _ in range(N_REP)]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng2.set_controls(temps=temps)
        eng2.set_sampling(1, SWEEPS_PER_STEP)
        eng2.run_sweeps(SWEEPS_PER_STEP)
        s2, c2 = eng2.samples()
        for r in range(N_REP):
            e2e_series[r].append(s2[r, :c2[r], 0])
    t_e2e = time.perf_counter() - t0
    e2e_ess, _ = effective_samples([np.concatenate(x) for x in e2e_series])
    h2d = N_REP * 8
    d2h = N_REP * SWEEPS_PER_STEP * 2 * 2

    # roofline of the MC kernel: algorithmic DRAM bytes = state in + out + samples
    lay_bytes = eng.state_bytes()
    alg_bytes = N_REP * lay_bytes * 2 + N_REP * SWEEPS_PER_STEP * 4
    achieved = alg_bytes / (np.mean(dev_ms) / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", "c2_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    line = {"metric": "effective samples/s (tau_int of #bound domains), plain MC", "value": value,
            "unit": "effective samples/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(dev_ms)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "c2: 4096 constant-T chains, scaffolds 8/12/16/24 (1024 each), uniform hyb "
                                   "dH=-120 kcal/mol dS=-0.33 kcal/mol/K, T~U[320,350] K, 1 uM, Met exchange/"
                                   "regrowth + CB regrowth", "sweeps_per_step": SWEEPS_PER_STEP,
                       "replicas": N_REP, "l2": "state resident in shared memory; no L2 flush needed"},
            "sweeps_per_s": sweeps_per_s, "move_attempts_per_s": moves_per_s, "tau_int_median": tau_med,
            "tau_int_by_size": taus_per_size,
            "e2e": {"value": e2e_ess / t_e2e, "unit": "effective samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind},
            "clocks": clk}
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline(files, args.warmup * SWEEPS_PER_STEP, total_sweeps)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
