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


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


def check_trace(tr, ref):
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(tr[:, 6], ref[:, 6], rtol=1e-12, atol=1e-12)


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
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))
        assert eng.config(r) == o.config()
        total += o.move_stats(n_moves)
    stats = eng.move_stats(n_moves)
    np.testing.assert_array_equal(stats, total)
    # every linker movetype was tried and accepted
    assert (stats[first_linker:, 1] > 0).all()
