"""Scaffold regrowth on the GPU (CTRG, CTRG jump, CTCB, CTCB jump):
against the reference's own traces (tests/golden, made by the reference
compiled from its sources) and against the CPU oracle with FP64 weights on
more seeds and replicas.  Lattice state, counters and random-draw counts must
agree exactly at every step, the FP64 energies within 1e-12 relative."""
import gzip
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, inp
from oracle_lib import OracleReplica, set_bias_centre
import systems

pytestmark = pytest.mark.gpu

EXACT = [0, 2, 3, 4, 5, 7]   # step, staples, fully bound, bound, stacked, draws
CASES = ["s24a", "s24b", "s24c", "r24", "s48", "c4"]
FIXTURES = ["s24a_s3", "s24b_s4", "s24c_s5", "r24_s6", "s48_s7", "c4_s9"]


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


def check_trace(tr, ref):
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(tr[:, 6], ref[:, 6], rtol=1e-12, atol=1e-12)


def load(name):
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rt") as f:
        return json.load(f)


@pytest.mark.parametrize("name", FIXTURES)
def test_scaffold_moves_match_reference_trace(name):
    fx = load(name)
    steps = fx["steps"]
    eng = engine(inp(fx["case"]), n_replicas=1, seed=fx["seed"])
    eng.set_trace(1, steps)
    eng.run(steps)
    check_trace(eng.trace()[0], np.array(fx["trace"], dtype=np.float64))
    assert eng.config(0) == fx["final_config"]


def test_fp64_weights_follow_reference_until_the_tie():
    """s24a_s11 meets a weight ratio within a rounding of 1 at step 19885; the
    engine (FP64) follows the reference (long double) up to there and the
    oracle's FP64 arithmetic over the whole run."""
    fx = load("s24a_s11")
    steps = fx["steps"]
    eng = engine(inp(fx["case"]), n_replicas=1, seed=fx["seed"])
    eng.set_trace(1, steps)
    eng.run(steps)
    tr = eng.trace()[0]
    ref = np.array(fx["trace"], dtype=np.float64)
    check_trace(tr[:19884], ref[:19884])
    o = OracleReplica(inp(fx["case"]), seed=fx["seed"], replica=0)
    check_trace(tr, o.run(steps))
    assert eng.config(0) == o.config()


@pytest.mark.parametrize("case", CASES)
def test_scaffold_moves_match_oracle_per_step(case):
    steps, n, seed = 4000, 8, 4321
    eng = engine(inp(case), n_replicas=n, seed=seed)
    eng.set_trace(n, steps)
    eng.run(steps)
    tr = eng.trace()
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        check_trace(tr[r], o.run(steps))
        assert eng.config(r) == o.config()


@pytest.mark.parametrize("case", ["s24c", "r24"])
def test_scaffold_moves_long_runs_in_chunks(case):
    n, seed, chunks, steps, n_moves = 12, 17, 4, 5000, {"s24c": 5, "r24": 7}[case]
    eng = engine(inp(case), n_replicas=n, seed=seed)
    for _ in range(chunks):
        eng.run(steps)
    obs = eng.observables()
    total = np.zeros((n_moves, 2), np.int64)
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        o.run(chunks * steps, trace=False)
        ob = o.observables()
        assert obs[r]["draws"] == ob["draws"]
        for k in ["num_staples", "num_fully_bound", "num_bound", "num_self_bound", "num_stacked"]:
            assert obs[r][k] == ob[k], (r, k)
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))
        assert eng.config(r) == o.config()
        total += o.move_stats(n_moves)
    stats = eng.move_stats(n_moves)
    np.testing.assert_array_equal(stats, total)
    # every scaffold movetype was tried and accepted
    assert (stats[3:, 1] > 0).all()


def test_engine_exp_same_bits_on_gpu_and_host():
    """ldo_math::exp: the GPU and the host give identical doubles, within one
    unit in the last place of the exact exponential."""
    from latticednaorigami_gb300.engine import engine_exp
    from oracle_lib import engine_exp as host_exp
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(-745, 709, 200000), rng.uniform(-40, 40, 200000), rng.normal(0, 1e-3, 10000),
                        [0.0, -0.0, 1.0, -1.0, 709.78, -745.1, 710.0, -746.0]])
    g = engine_exp(x)
    h = host_exp(x)
    np.testing.assert_array_equal(g.view(np.int64), h.view(np.int64))
    m = (np.abs(x) < 700)
    ulp = np.spacing(np.exp(x[m]))
    assert np.max(np.abs(g[m] - np.exp(x[m])) / ulp) <= 1.5


def test_harmonic_windows_with_scaffold_moves():
    """Umbrella windows of the 96-domain design: a Harmonic bias on the number
    of fully bound domains with a different centre per replica
    (ldo_set_bias_centre), the reference's standard moveset, two temperatures."""
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "harm.json"), "w") as f:
        json.dump({"origami": {"bias_functions": [
            {"label": "window", "tag": "win", "type": "Harmonic", "k": 0.5, "centre": 0,
             "ops": ["numfulldomains"], "level": 0}]}}, f)
    p = systems.write_case(d, "c4", extra=dict(bias_functions_file="harm.json"))
    centres = [0, 6, 14, 24, 40, 60]
    temps = [310.0, 320.0, 310.0, 320.0, 310.0, 320.0]
    n, seed, steps = len(centres), 23, 3000
    eng = engine(p, n_replicas=n, seed=seed)
    eng.set_controls(temps=np.array(temps))
    for r, c in enumerate(centres):
        eng.set_bias_centre("win", r, c)
    eng.set_trace(n, steps)
    eng.run(steps)
    tr = eng.trace()
    for r in range(n):
        o = OracleReplica(p, seed=seed, replica=r)
        o.update_temp(temps[r])
        set_bias_centre(o, "win", centres[r])
        check_trace(tr[r], o.run(steps))
        assert eng.config(r) == o.config()
    # each replica is restrained by its own centre
    assert tr[5, -1, 6] > tr[4, -1, 6] > tr[2, -1, 6]
