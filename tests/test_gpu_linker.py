"""Scaffold transforms with linker regrowth on the GPU (CTCBLinkerRegrowth,
CTCBClusteredLinkerRegrowth, CTRGLinkerRegrowth; src/transform_movetypes.cpp),
step by step against the oracle on several replicas and in chunked runs (the
reference's own traces of the same systems are checked by
tests/test_gpu_parity.py::test_engine_matches_reference_golden, fixtures
l24a/l24b/l24c/l24r, and the oracle against them by tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from conftest import inp
from oracle_lib import OracleReplica

pytestmark = pytest.mark.gpu

EXACT = [0, 2, 3, 4, 5, 7]   # step, staples, fully bound, bound, stacked, draws
CASES = ["l24a", "l24b", "l24c", "l24r"]
# The oracle, like the reference, keeps its energy as a running total of
# every placement and removal, which drifts under the linker movetypes' many
# trial transformations (up to 7.5e-12 relative over 20000 steps,
# tests/test_oracle_golden.py::test_reference_energy_drift_under_linker_moves);
# the engine restores snapshots and stays on its configuration's energy.
RTOL = 2e-11


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


def check_trace(tr, ref):
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(tr[:, 6], ref[:, 6], rtol=RTOL, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_linker_moves_match_oracle_per_step(case):
    steps, n, seed = 4000, 8, 2468
    eng = engine(inp(case), n_replicas=n, seed=seed)
    eng.set_trace(n, steps)
    eng.run(steps)
    tr = eng.trace()
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        check_trace(tr[r], o.run(steps))
        assert eng.config(r) == o.config()


@pytest.mark.parametrize("case,n_moves,first_linker", [("l24a", 5, 3), ("l24b", 4, 3), ("l24r", 5, 2)])
def test_linker_moves_long_runs_in_chunks(case, n_moves, first_linker):
    n, seed, chunks, steps = 12, 31, 4, 5000
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
        assert abs(obs[r]["energy"] - ob["energy"]) <= RTOL * max(1.0, abs(ob["energy"]))
        assert eng.config(r) == o.config()
        total += o.move_stats(n_moves)
    stats = eng.move_stats(n_moves)
    np.testing.assert_array_equal(stats, total)
    # every linker movetype was tried and accepted
    assert (stats[first_linker:, 1] > 0).all()


def test_engine_energy_stays_on_its_configuration():
    """After 20000 steps of every linker movetype the engine's running energy
    equals the energy recomputed from its configuration (set_controls at the
    same temperature recomputes it) within 1e-12 relative."""
    import re
    case = "l24r"
    temp = float(re.search(r"temp\s*=\s*([0-9.]+)", open(inp(case)).read()).group(1))
    eng = engine(inp(case), n_replicas=4, seed=16)
    eng.run(20000)
    run = [o["energy"] for o in eng.observables()]
    eng.set_controls(temps=[temp] * 4)
    rec = [o["energy"] for o in eng.observables()]
    for a, b in zip(run, rec):
        assert abs(a - b) <= 1e-12 * max(1.0, abs(b)), (a, b)
