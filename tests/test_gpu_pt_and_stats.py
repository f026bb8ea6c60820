"""Parallel tempering and sampling distribution on the GPU.

- PT: the in-kernel exchange (CUDA graph of MC + swap launches) against the
  CPU restatement in tests/pt_oracle.py: identical permutations, swap counts,
  random-draw counts and energies.
- Distribution: order-parameter histogram of many independent GPU chains of
  the 4-domain system against the reference's exact staple-only enumeration
  (tests/golden/c1_enumeration.json), chi-square p > 0.01."""
import json
import math
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN
import systems

pytestmark = pytest.mark.gpu


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


@pytest.mark.parametrize("q", [1, 3])
def test_pt_matches_cpu_restatement(q):
    from pt_oracle import PTOracle
    temps = [325.0, 330.0, 336.0, 343.0]
    umults = [1.0, 1.3, 0.9, 1.1]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)),
                                                     chem_pot_mults=" ".join(map(str, umults)),
                                                     num_reps=4, exchange_interval=150))
    n_ladders, swaps, interval, seed = 2, 12, 150, 31
    eng = engine(inp, n_replicas=4 * n_ladders, seed=seed)
    eng.pt_run(4, swaps, interval, q)
    ora = PTOracle(inp, dict(temps=temps, chem_pot_mults=umults, temp=335.0, staple_M=1e-3,
                             staple_lengths=[2] * 12), n_ladders, seed, exchange_q=q)
    for _ in range(swaps):
        ora.round(interval)
    np.testing.assert_array_equal(eng.pt_permutation(), ora.permutation())
    att, acc = eng.pt_stats(3)
    assert att.tolist() == ora.att and acc.tolist() == ora.acc
    obs = eng.observables()
    for r, rep in enumerate(ora.reps):
        ob = rep.observables()
        assert obs[r]["draws"] == ob["draws"]
        assert obs[r]["num_fully_bound"] == ob["num_fully_bound"]
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))


def test_pt_48_domain_ladder_matches_cpu_restatement():
    """The 48-domain PTMC system's shape (nearest-neighbour energies, 24
    staple types): 8 temperatures geometric over 310-370 K, 2 ladders,
    temperature exchange every 500 steps."""
    from pt_oracle import PTOracle
    temps = [310.0 * (370.0 / 310.0) ** (k / 7.0) for k in range(8)]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "c3", extra=dict(temps=" ".join(repr(t) for t in temps), num_reps=8,
                                                   exchange_interval=500))
    n_ladders, swaps, interval, seed = 2, 8, 500, 41
    eng = engine(inp, n_replicas=8 * n_ladders, seed=seed)
    eng.pt_run(8, swaps, interval, 1)
    ora = PTOracle(inp, dict(temps=temps, chem_pot_mults=[1.0] * 8, temp=340.0, staple_M=1e-6,
                             staple_lengths=[2] * 24), n_ladders, seed, exchange_q=1)
    for _ in range(swaps):
        ora.round(interval)
    np.testing.assert_array_equal(eng.pt_permutation(), ora.permutation())
    att, acc = eng.pt_stats(7)
    assert att.tolist() == ora.att and acc.tolist() == ora.acc
    obs = eng.observables()
    for r, rep in enumerate(ora.reps):
        ob = rep.observables()
        assert obs[r]["draws"] == ob["draws"]
        assert obs[r]["num_staples"] == ob["num_staples"]
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))


def chi2_sf(x, k):
    # survival function of chi-square with k dof (series for the regularised gamma)
    a = k / 2.0
    x2 = x / 2.0
    if x2 <= 0:
        return 1.0
    s, term, n = 0.0, 1.0 / a, 0
    while term > 1e-16 * s or n < 5:
        s += term
        n += 1
        term *= x2 / (a + n)
        if n > 10000:
            break
    p_lower = math.exp(-x2 + a * math.log(x2) - math.lgamma(a)) * s
    return max(0.0, 1.0 - p_lower)


def test_distribution_matches_exact_enumeration(data_dir):
    with open(os.path.join(GOLDEN, "c1_enumeration.json")) as f:
        ref = json.load(f)["weights"]
    n_rep, burn, gap, snaps = 4096, 40000, 20000, 4
    eng = engine(os.path.join(data_dir, "c1.inp"), n_replicas=n_rep, seed=2024)
    eng.run(burn)
    counts = {}
    for _ in range(snaps):
        eng.run(gap)
        for o in eng.observables():
            k = "%d %d" % (o["num_staples"], o["num_fully_bound"])
            counts[k] = counts.get(k, 0) + 1
    total = n_rep * snaps
    keys = sorted(ref, key=lambda k: -ref[k])
    # merge the tail into one bin so every expected count is >= 5
    bins, tail = [], []
    for k in keys:
        (bins if ref[k] * total >= 5 else tail).append(k)
    obs = [counts.get(k, 0) for k in bins] + [sum(counts.get(k, 0) for k in tail)]
    exp = [ref[k] * total for k in bins] + [sum(ref[k] for k in tail) * total]
    extra = sum(v for k, v in counts.items() if k not in ref)
    assert extra == 0
    if exp[-1] < 5:
        obs[-2] += obs[-1]
        exp[-2] += exp[-1]
        obs, exp = obs[:-1], exp[:-1]
    chi2 = sum((o - e) ** 2 / e for o, e in zip(obs, exp))
    p = chi2_sf(chi2, len(obs) - 1)
    assert p > 0.01, (obs, exp, chi2, p)


def test_pt_2d_temperature_stacking_grid_matches_cpu_restatement():
    """TwoDPTGCMCSimulation's grid: 3 temperatures x 3 stacking multipliers,
    the four alternating pair sets, 2 ladders, 14 rounds (CUDA-graph cycles
    of four rounds plus alignment rounds)."""
    from pt_oracle import PTOracle
    temps = [325.0, 333.0, 342.0]
    stacks = [0.8, 1.0, 1.25]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)),
                                                     stacking_mults=" ".join(map(str, stacks)), num_reps=9,
                                                     exchange_interval=150))
    n_ladders, swaps, interval, seed = 2, 14, 150, 53
    eng = engine(inp, n_replicas=9 * n_ladders, seed=seed)
    eng.pt2d_run(3, 3, 5, interval)
    eng.pt2d_run(3, 3, swaps - 5, interval)
    ora = PTOracle(inp, dict(temps=temps, stacking_mults=stacks, temp=335.0, staple_M=1e-3,
                             staple_lengths=[2] * 12), n_ladders, seed, dim2=3)
    for _ in range(swaps):
        ora.round(interval)
    np.testing.assert_array_equal(eng.pt_permutation(), ora.permutation())
    att, acc = eng.pt_stats(18)
    assert att.tolist() == ora.att and acc.tolist() == ora.acc
    assert sum(acc) > 0
    obs = eng.observables()
    for r, rep in enumerate(ora.reps):
        ob = rep.observables()
        assert obs[r]["draws"] == ob["draws"]
        assert obs[r]["num_staples"] == ob["num_staples"]
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))


def test_pt_graph_follows_sampling_and_interval_changes():
    """The captured PT cycle holds the kernel's launch parameters: a run after
    set_sampling (or with another exchange interval) must use the new ones."""
    temps = [325.0, 330.0, 336.0, 343.0]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)), num_reps=4))
    eng = engine(inp, n_replicas=8, seed=5)
    eng.pt_run(4, 8, 100, 1)              # captures the graph without sampling
    eng.set_sampling(50, 64)
    eng.pt_run(4, 8, 100, 1)              # 800 steps: a sample every 50
    smp, cnt = eng.samples()
    assert (cnt == 16).all(), cnt
    eng.set_sampling(50, 64)
    eng.pt_run(4, 8, 150, 1)              # another interval: 1200 steps
    smp, cnt = eng.samples()
    assert (cnt == 24).all(), cnt


def test_counters_count_launches_and_copies():
    """ldo_get_counters: a run is one MC launch and the status fold; a PT run
    of k rounds is k MC and k exchange launches (graph replays counted per
    kernel) and the status fold; reading the samples copies exactly the
    sample buffer and the per-replica counters."""
    temps = [325.0, 330.0, 336.0, 343.0]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)), num_reps=4))
    eng = engine(inp, n_replicas=8, seed=5)
    eng.set_sampling(10, 32)
    l0, h0, d0 = eng.counters()
    eng.run(100)
    l1, h1, d1 = eng.counters()
    assert l1 - l0 == 2
    assert h1 == h0
    smp, cnt = eng.samples()
    l2, h2, d2 = eng.counters()
    assert (cnt == 10).all(), cnt
    assert l2 == l1 and h2 == h1
    assert d2 - d1 == smp.nbytes + cnt.nbytes
    for swaps in (3, 12):                 # below and above the graph threshold
        a = eng.counters()[0]
        eng.pt_run(4, swaps, 100, 1)
        assert eng.counters()[0] - a == 2 * swaps + 1, swaps
