"""Learned proposals on the CPU (no GPU needed).

- Exactness of the Metropolis-Hastings ratios: the CPU restatements of
  LearnedStapleExchange and LearnedStapleRegrowth, driven by a strongly
  non-uniform random weight table, sample the 4-domain system's (staples,
  fully bound) distribution of the reference's exact enumeration (chi-square
  p > 0.01), as the plain moveset does.
- The numpy network (oracle/learn_ref.py) that the GPU kernels are checked
  against: its analytic gradient against central finite differences."""
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, inp
from oracle_lib import run_batch_states
from test_gpu_pt_and_stats import chi2_sf

import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import learn_ref  # noqa: E402


def learned_moves(d, regrowth=False):
    """The c2 moveset with the learned exchange (and, with regrowth, the
    learned regrowth in place of the Met regrowth)."""
    mv = {"origami": {"movetypes": [
        {"label": "Learned staple exchange", "type": "LearnedStapleExchange", "freq": "1/3",
         "adaptive_exchange": False},
        {"label": "Met staple regrowth", "type": "LearnedStapleRegrowth" if regrowth else "MetStapleRegrowth",
         "freq": "1/3"},
        {"label": "CB staple regrowth", "type": "CBStapleRegrowth", "freq": "1/3"}]}}
    p = os.path.join(d, "moves_learned%s.json" % ("_lr" if regrowth else ""))
    with open(p, "w") as f:
        json.dump(mv, f)
    return p


def chi2_against_enumeration(states, name="c1_enumeration"):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        ref = json.load(f)["weights"]
    counts = {}
    for s, fb in states.reshape(-1, 2):
        k = "%d %d" % (s, fb)
        counts[k] = counts.get(k, 0) + 1
    total = states.shape[0] * states.shape[1]
    assert sum(v for k, v in counts.items() if k not in ref) == 0
    keys = sorted(ref, key=lambda k: -ref[k])
    bins = [k for k in keys if ref[k] * total >= 5]
    tail = [k for k in keys if k not in bins]
    obs = [counts.get(k, 0) for k in bins] + [sum(counts.get(k, 0) for k in tail)]
    exp = [ref[k] * total for k in bins] + [sum(ref[k] for k in tail) * total]
    if exp[-1] < 5:
        obs[-2] += obs[-1]
        exp[-2] += exp[-1]
        obs, exp = obs[:-1], exp[:-1]
    chi2 = sum((o - e) ** 2 / e for o, e in zip(obs, exp))
    return chi2_sf(chi2, len(obs) - 1), obs, exp


def test_learned_exchange_samples_exact_distribution():
    d = tempfile.mkdtemp()
    mv = learned_moves(d)
    rng = np.random.default_rng(5)
    table = np.exp(rng.normal(0.0, 2.0, learn_ref.TABLE))
    # one state per replica after 60000 steps (the empty start has relaxed)
    states = run_batch_states(inp("c1"), 77, 1024, 60000, 1, 1, os.cpu_count() or 1,
                              overrides="movetype_file = %s" % mv, learn_w=table)
    p, obs, exp = chi2_against_enumeration(states)
    assert p > 0.01, (obs, exp, p)


@pytest.mark.parametrize("moves", ["plain", "learned"])
def test_capped_8_domain_system_samples_exact_distribution(moves):
    """The 8-domain system capped at two staples, where a third of the weight
    is one fully and one partly bound staple: the learned exchange (sites,
    growth directions, deletion choice weighted by how a staple is bound)
    with a strongly non-uniform random table, and the plain moveset, against
    the reference's exact enumeration."""
    d = tempfile.mkdtemp()
    over = "movetype_file = %s" % learned_moves(d, regrowth=True) if moves == "learned" else ""
    table = np.exp(np.random.default_rng(9).normal(0.0, 2.0, learn_ref.TABLE))
    states = run_batch_states(inp("e8"), 81, 2048, 40000, 1, 1, os.cpu_count() or 1,
                              overrides=over, learn_w=table if moves == "learned" else None)
    p, obs, exp = chi2_against_enumeration(states, "e8_enumeration")
    assert p > 0.01, (obs, exp, p)


def test_learned_regrowth_samples_exact_distribution():
    """LearnedStapleRegrowth (learned directions and orientations) with a
    strongly non-uniform random table: the enumeration's distribution."""
    d = tempfile.mkdtemp()
    mv = os.path.join(d, "moves_lr.json")
    with open(mv, "w") as f:
        json.dump({"origami": {"movetypes": [
            {"label": "Met staple exchange", "type": "MetStapleExchange", "freq": "1/3", "adaptive_exchange": False},
            {"label": "Learned staple regrowth", "type": "LearnedStapleRegrowth", "freq": "1/3"},
            {"label": "CB staple regrowth", "type": "CBStapleRegrowth", "freq": "1/3"}]}}, f)
    rng = np.random.default_rng(6)
    table = np.exp(rng.normal(0.0, 2.0, learn_ref.TABLE))
    states = run_batch_states(inp("c1"), 78, 1024, 60000, 1, 1, os.cpu_count() or 1,
                              overrides="movetype_file = %s" % mv, learn_w=table)
    p, obs, exp = chi2_against_enumeration(states)
    assert p > 0.01, (obs, exp, p)


def test_numpy_network_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    params = learn_ref.init_params(11)
    idx = rng.choice(learn_ref.TABLE, 40, replace=False).astype(np.int32)
    cnt_t = rng.integers(1, 20, 40).astype(np.float32)
    cnt_b = np.floor(cnt_t * rng.random(40)).astype(np.float32)
    # exact arithmetic (no bf16 rounding) so that differences resolve the gradient
    loss, grad = learn_ref.loss_grad(params, idx, cnt_b, cnt_t, bf16=False)
    for k in list(rng.choice(len(params), 25, replace=False)) + [learn_ref.OFF_B4, learn_ref.OFF_W4 + 3]:
        h = 1e-3
        p1 = params.astype(np.float64).copy()
        p1[k] += h
        l1, _ = learn_ref.loss_grad(p1, idx, cnt_b, cnt_t, bf16=False)
        p1[k] -= 2 * h
        l2, _ = learn_ref.loss_grad(p1, idx, cnt_b, cnt_t, bf16=False)
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, grad[k])
