"""Exact staple-only enumeration on the GPU (ldo_enumerate, csrc/ldo_enum.cuh)
against the reference's own enumerator (src/enumerate.cpp, golden weights at
full precision from tests/golden/make_golden.py): the 4-domain system with up
to four staples and the 8-domain system with up to two, three and four
staples (max_total_staples raised as in the fixtures; four is every staple
set, 38 min for the reference on one core, 0.6 s of GPU time), where staples
bind both of their domains.  The reference sums its weights in long double,
the engine in FP64 with compensated sums: weights agree to 1e-10 relative."""
import json
import os

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,case,max_total,max_type", [("c1_enumeration", "c1", 4, 4),
                                                          ("e8_enumeration", "e8", 2, 1),
                                                          ("e8s3_enumeration", "e8", 3, 1),
                                                          ("e8s4_enumeration", "e8", 4, 1),
                                                          ("m8_enumeration", "m8", 3, 1)])
def test_enumeration_matches_reference(name, case, max_total, max_type, data_dir):
    from latticednaorigami_gb300 import Engine
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    eng = Engine(os.path.join(data_dir, case + ".inp"), n_replicas=1, seed=0, overrides=over)
    w, info = eng.enumerate(0, max_total, max_type)
    assert set(w) == set(fx["weights"]), (sorted(w), sorted(fx["weights"]))
    for k, v in fx["weights"].items():
        assert abs(w[k] - v) <= 1e-10 * v, (k, w[k], v)
    assert abs(info["num_configs"] - fx["num_configs"]) <= 1e-9 * fx["num_configs"]


@pytest.mark.parametrize("name,case,max_total", [("e8_enumeration", "e8", 2), ("m8_enumeration", "m8", 3)])
def test_enumeration_units_match_reference(name, case, max_total, data_dir):
    """Unit by unit: the growth-point sets in the reference's order, each
    with its partition-function sum and number of configurations.

    The reference's per-unit sums are increments of its running partition
    function (long double, 64-bit mantissa): each configuration's weight is
    added to the total so far, so a unit's increment carries an absolute
    error of up to half an ulp of that total per configuration.  The
    tolerance is 1e-10 relative plus that bound (one ulp of the final total
    per configuration); the engine sums each unit from zero in FP64."""
    import numpy as np
    from latticednaorigami_gb300 import Engine
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    eng = Engine(os.path.join(data_dir, case + ".inp"), n_replicas=1, seed=0)
    eng.enumerate(0, max_total, 1)
    units = eng.enumerate_units()
    ref = np.array(fx["units"])
    assert units.shape == ref.shape
    np.testing.assert_array_equal(units[:, 1], ref[:, 1])
    total = ref[:, 0].sum()
    ulp = 2.0 ** -63 * 2.0 ** np.ceil(np.log2(total))
    tol = 1e-10 * np.abs(ref[:, 0]) + np.maximum(ref[:, 1], 1.0) * ulp
    bad = np.abs(units[:, 0] - ref[:, 0]) > tol
    assert not bad.any(), (np.flatnonzero(bad)[:10], units[bad][:5], ref[bad][:5])


@pytest.mark.parametrize("name,max_total,split", [("c1full_enumeration", 2, 0), ("c1full_enumeration", 2, 2),
                                                  ("c1full3_enumeration", 3, 3)])
def test_full_enumeration_matches_reference(name, max_total, split, data_dir):
    """The full conformational enumeration (the scaffold enumerated too,
    ConformationalEnumerator::enumerate) of the 4-domain system with up to
    two and three staples, against the reference's own, whole and split into
    6^split parts per unit.

    The reference adds every configuration's weight to its bin of
    m_state_weights, a running double sum (src/enumerate.cpp:658), over up to
    1e8 configurations per bin; those roundings move a bin by up to (n - 1) u
    relative (n configurations, u = 2^-53; recursive summation's bound,
    Higham, Accuracy and Stability of Numerical Algorithms, 2nd ed., eq.
    4.4), 3e-9 on the ≤3-staple system's smallest bins.  The trace driver
    therefore also sums the reference's own weights, configuration by
    configuration, without that drift (weights_exact: compensated sums,
    oracle/ref/ref_trace.cpp).  The engine's bins (compensated sums of its
    weights) match those at 1e-12, and the reference's printed weights lie
    within the running-sum bound of them.  The reference's running energy
    m_energy (long double) has no drift over a unit (unit_energy_drift)."""
    import numpy as np
    from latticednaorigami_gb300 import Engine
    path = os.path.join(GOLDEN, name + ".json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    with open(path) as f:
        fx = json.load(f)
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    eng = Engine(os.path.join(data_dir, "c1.inp"), n_replicas=1, seed=0, overrides=over)
    w, info = eng.enumerate(0, max_total, 4, full=True, split_levels=split)
    drift = np.array(fx.get("unit_energy_drift", [0.0]))
    offset = np.concatenate([[0.0], np.cumsum(drift)])
    bound = float(np.max(np.abs(offset[:-1]) + np.abs(drift)))
    rtol = 1e-12 + 2 * bound
    exact = fx["weights_exact"]
    assert set(w) == set(fx["weights"]) == set(exact), (sorted(w), sorted(fx["weights"]))
    u = 2.0 ** -53
    for k, v in exact.items():
        assert abs(w[k] - v) <= rtol * v, (k, w[k], v, rtol)
        n = fx["bin_configs"][k]
        # the bin's own running sum, the partition function's (long double,
        # over every configuration), the roundings of the output
        tol = max(n - 1, 1) * u + fx["saved_configs"] * 2.0 ** -64 + 4 * u
        assert abs(fx["weights"][k] - v) <= tol * v, (k, fx["weights"][k], v, n)
    assert abs(info["num_configs"] - fx["num_configs"]) <= 1e-12 * fx["num_configs"]
    if "units" in fx:
        units = eng.enumerate_units()
        ref = np.array(fx["units"])
        assert units.shape == ref.shape
        np.testing.assert_allclose(units[:, 1], ref[:, 1], rtol=1e-12, atol=0)
        total = ref[:, 0].sum()
        ulp = 2.0 ** -63 * 2.0 ** np.ceil(np.log2(total))
        tol = 1e-10 * np.abs(ref[:, 0]) + np.maximum(ref[:, 1], 1.0) * ulp
        bad = np.abs(units[:, 0] - ref[:, 0]) > tol
        assert not bad.any(), (np.flatnonzero(bad)[:10], units[bad][:5], ref[bad][:5])


def _chi2_against(weights, samples):
    """Chi-square p-value of (numstaples, numfulldomains) samples against
    normalised weights, with the bins of fewer than 5 expected samples merged."""
    from test_gpu_pt_and_stats import chi2_sf
    counts = {}
    for s in samples:
        counts[s] = counts.get(s, 0) + 1
    total = len(samples)
    assert all(k in weights for k in counts), sorted(set(counts) - set(weights))
    keys = sorted(weights, key=lambda k: -weights[k])
    bins = [k for k in keys if weights[k] * total >= 5]
    tail = [k for k in keys if k not in bins]
    obs = [counts.get(k, 0) for k in bins] + [sum(counts.get(k, 0) for k in tail)]
    exp = [weights[k] * total for k in bins] + [sum(weights[k] for k in tail) * total]
    if exp[-1] < 5:
        obs[-2] += obs[-1]
        exp[-2] += exp[-1]
        obs, exp = obs[:-1], exp[:-1]
    chi2 = sum((o - e) ** 2 / e for o, e in zip(obs, exp))
    return chi2_sf(chi2, len(obs) - 1), obs, exp


def _mc_samples(inp, over, moves, seed, cb=True):
    """(numstaples, numfulldomains) of 2048 replicas at 4 snapshots 20000
    steps apart after 40000 steps: the plain moveset (Met exchange, Met
    regrowth) or the learned exchange and regrowth with a strongly
    non-uniform random weight table, each with CB staple regrowth if cb."""
    import tempfile

    import numpy as np
    from latticednaorigami_gb300 import Engine
    from test_learned_oracle import learn_ref
    kinds = {"plain": [("Met staple exchange", "MetStapleExchange"), ("Met staple regrowth", "MetStapleRegrowth")],
             "learned": [("Learned staple exchange", "LearnedStapleExchange"),
                         ("Learned staple regrowth", "LearnedStapleRegrowth")]}[moves]
    if cb:
        kinds = kinds + [("CB staple regrowth", "CBStapleRegrowth")]
    mv = {"origami": {"movetypes": [{"label": l, "type": t, "freq": "1/%d" % len(kinds), "adaptive_exchange": False}
                                    for l, t in kinds]}}
    path = os.path.join(tempfile.mkdtemp(), "moves.json")
    with open(path, "w") as f:
        json.dump(mv, f)
    over = "\n".join(x for x in (over, "movetype_file = %s" % path) if x)
    n_rep, burn, gap, snaps = 2048, 40000, 20000, 4
    mc = Engine(inp, n_replicas=n_rep, seed=seed, overrides=over)
    if moves == "learned":
        mc.learn_set_table(np.exp(np.random.default_rng(21).normal(0.0, 2.0, learn_ref.TABLE)))
    mc.run(burn)
    samples = []
    for _ in range(snaps):
        mc.run(gap)
        samples += ["%d %d" % (o["num_staples"], o["num_fully_bound"]) for o in mc.observables()]
    return samples


@pytest.mark.parametrize("moves", ["plain", "learned"])
def test_mc_samples_enumeration_of_every_staple_set(moves, data_dir):
    """Every staple set of the 8-domain system (up to four staples, one per
    type; the reference's enumeration of it, 38 min on one core, is the
    fixture): the engine's MC with the plain moveset, and with the learned
    exchange and regrowth driven by a strongly non-uniform random weight
    table, samples its distribution (chi-square p > 0.01)."""
    with open(os.path.join(GOLDEN, "e8s4_enumeration.json")) as f:
        w4 = json.load(f)["weights"]
    samples = _mc_samples(os.path.join(data_dir, "e8.inp"), "max_total_staples = 4", moves, 4242)
    p, obs, exp = _chi2_against(w4, samples)
    assert p > 0.01, (obs, exp, p)


def test_learned_and_met_moves_agree_with_three_domain_staples(data_dir):
    """Three-domain staples with misbinding disallowed (m8): the learned
    exchange and regrowth sample the distribution of the reference's Met
    exchange and regrowth (two-sample chi-square p > 0.01).  Without CB
    staple regrowth: on this system the reference's CBStapleRegrowth moves
    the distribution away from the one its Met moves sample (all three
    staples bound 0.113 of the samples with it, 0.081 without; CPU
    restatement, which follows the reference's trace m8_s19 step for step),
    and the reference's staple-only enumeration (misbinding-only overcount)
    gives a third (0.133), which the engine's enumerator reproduces
    (test_enumeration_matches_reference)."""
    from test_gpu_pt_and_stats import chi2_sf
    inp = os.path.join(data_dir, "m8.inp")
    a = _mc_samples(inp, "", "plain", 4242, cb=False)
    b = _mc_samples(inp, "", "learned", 4343, cb=False)
    keys = sorted(set(a) | set(b))
    ca = [a.count(k) for k in keys]
    cb = [b.count(k) for k in keys]
    # merge bins with fewer than 10 samples in all into one
    small = [i for i in range(len(keys)) if ca[i] + cb[i] < 10]
    big = [i for i in range(len(keys)) if i not in small]
    ca = [ca[i] for i in big] + ([sum(ca[i] for i in small)] if small else [])
    cb = [cb[i] for i in big] + ([sum(cb[i] for i in small)] if small else [])
    if small and ca[-1] + cb[-1] < 10:
        ca[-2] += ca.pop()
        cb[-2] += cb.pop()
    na, nb = len(a), len(b)
    chi2 = 0.0
    for x, y in zip(ca, cb):
        t = x + y
        ex, ey = t * na / (na + nb), t * nb / (na + nb)
        chi2 += (x - ex) ** 2 / ex + (y - ey) ** 2 / ey
    p = chi2_sf(chi2, len(ca) - 1)
    assert p > 0.01, (keys, ca, cb, p)
