"""GPU engine against the CPU oracle (and, through the golden fixtures,
against the reference itself).  Same systems, same Philox streams: the lattice
state, counters and random-draw counts must agree exactly at every step and
the FP64 energies within 1e-12 relative."""
import glob
import gzip
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_overrides, inp
from oracle_lib import OracleReplica

pytestmark = pytest.mark.gpu

CASES = ["c1", "g24a", "g24b", "g24c", "g24d", "g24e", "c3"]
LINKER_ENERGY_RTOL = 2e-11
EXACT = [0, 2, 3, 4, 5, 7]   # step, staples, fully bound, bound, stacked, draws


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


def check_trace(tr, ref):
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(tr[:, 6], ref[:, 6], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_engine_matches_oracle_per_step(case):
    steps, n, seed = 3000, 6, 1234
    eng = engine(inp(case), n_replicas=n, seed=seed)
    eng.set_trace(n, steps)
    eng.run(steps)
    tr = eng.trace()
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        ref = o.run(steps)
        check_trace(tr[r], ref)
        assert eng.config(r) == o.config()


# s24a_s11 meets a weight ratio within a rounding of 1 (long double vs FP64):
# tests/test_gpu_scaffold.py compares it up to that step
# (the annealing fixtures pin the oracle's annealing to the reference's;
# tests/test_gpu_anneal.py pins the engine's to the oracle's)
@pytest.mark.parametrize("path", [p for p in sorted(glob.glob(os.path.join(GOLDEN, "*.json.gz")))
                                  if not p.endswith("s24a_s11.json.gz") and "_anneal_" not in p],
                         ids=lambda p: os.path.basename(p)[:-8])
def test_engine_matches_reference_golden(path):
    with gzip.open(path, "rt") as f:
        fx = json.load(f)
    steps = fx["steps"]
    eng = engine(inp(fx["case"]), n_replicas=1, seed=fx["seed"], overrides=golden_overrides(fx))
    eng.set_trace(1, steps)
    eng.run(steps)
    tr = eng.trace()[0]
    ref = np.array(fx["trace"], dtype=np.float64)
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    # The reference's energy is a running total of every placement and
    # removal a move makes, undone or not; the engine restores rejected and
    # intermediate states from snapshots.  Under the linker movetypes (many
    # trial transformations per move) the reference's total drifts from its
    # configuration's energy by up to 7.5e-12 relative over these runs
    # (tests/test_oracle_golden.py::test_reference_energy_drift_under_linker_moves),
    # the others by less than 2e-13.
    rtol = LINKER_ENERGY_RTOL if fx["case"].startswith("l24") else 1e-12
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=rtol, atol=1e-12)
    assert eng.config(0) == fx["final_config"]


@pytest.mark.parametrize("case", ["g24a", "g24c"])
def test_long_runs_in_chunks_match_oracle(case):
    n, seed, chunks, steps = 48, 77, 4, 5000
    eng = engine(inp(case), n_replicas=n, seed=seed)
    for _ in range(chunks):
        eng.run(steps)
    obs = eng.observables()
    for r in range(0, n, 7):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        o.run(chunks * steps, trace=False)
        ob = o.observables()
        assert obs[r]["draws"] == ob["draws"]
        for k in ["num_staples", "num_fully_bound", "num_bound", "num_self_bound", "num_stacked", "current_c_i"]:
            assert obs[r][k] == ob[k], (r, k)
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))
        assert eng.config(r) == o.config()


def test_heterogeneous_batch_matches_oracle():
    files = [inp("c1"), inp("g24a"), inp("g24c")]
    sys_of = [0, 1, 2, 1, 0, 2, 2, 1]
    steps, seed = 2000, 9
    eng = engine(files, n_replicas=len(sys_of), seed=seed, sys_of_replica=sys_of)
    eng.set_trace(len(sys_of), steps)
    eng.run(steps)
    tr = eng.trace()
    for r, s in enumerate(sys_of):
        o = OracleReplica(files[s], seed=seed, replica=r)
        check_trace(tr[r], o.run(steps))


def test_temperature_change_recomputes_energy_like_update_temp():
    n, seed = 8, 5
    eng = engine(inp("g24a"), n_replicas=n, seed=seed)
    eng.run(4000)
    temps = np.linspace(320, 350, n)
    eng.set_controls(temps=temps)
    eng.run(1000)
    obs = eng.observables()
    for r in range(n):
        o = OracleReplica(inp("g24a"), seed=seed, replica=r)
        o.run(4000, trace=False)
        o.update_temp(float(temps[r]))
        o.run(1000, trace=False)
        ob = o.observables()
        assert obs[r]["draws"] == ob["draws"]
        assert obs[r]["num_fully_bound"] == ob["num_fully_bound"]
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))
        H, S, st, b = o.dependent_qs()
        assert abs(obs[r]["enthalpy"] - H) <= 1e-12 * max(1.0, abs(H))
        assert abs(obs[r]["stacking"] - st) <= 1e-10 * max(1.0, abs(st))


def test_samples_follow_the_trace():
    n, steps, interval = 4, 2000, 50
    eng = engine(inp("g24a"), n_replicas=n, seed=3)
    eng.set_trace(n, steps)
    eng.set_sampling(interval, steps // interval)
    eng.run(steps)
    tr = eng.trace()
    smp, cnt = eng.samples()
    assert (cnt == steps // interval).all()
    for r in range(n):
        np.testing.assert_array_equal(smp[r, :, 0], tr[r, interval - 1::interval, 3])
        np.testing.assert_array_equal(smp[r, :, 1], tr[r, interval - 1::interval, 2])


def test_move_statistics_match_oracle():
    eng = engine(inp("g24a"), n_replicas=3, seed=21)
    eng.run(3000)
    tot = np.zeros((4, 2), np.int64)
    for r in range(3):
        o = OracleReplica(inp("g24a"), seed=21, replica=r)
        o.run(3000, trace=False)
        tot += o.move_stats(4)
    np.testing.assert_array_equal(eng.move_stats(4), tot)
