"""Annealing driver (AnnealingGCMCSimulation::run,
src/annealing_simulation.cpp:40) on the GPU against the oracle stepping
through the same temperatures with update_temp."""
import numpy as np
import pytest

from conftest import inp
from oracle_lib import OracleReplica

pytestmark = pytest.mark.gpu


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


@pytest.mark.parametrize("case", ["g24a", "c3"])
def test_annealing_matches_oracle(case):
    n, seed, steps = 4, 21, 600
    eng = engine(inp(case), n_replicas=n, seed=seed)
    eng.anneal(350.0, 330.0, 5.0, steps)
    obs = eng.observables()
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r)
        for t in [350.0, 345.0, 340.0, 335.0, 330.0]:
            o.update_temp(t)
            o.run(steps, trace=False)
        ob = o.observables()
        assert obs[r]["temp"] == 330.0
        assert obs[r]["draws"] == ob["draws"]
        for k in ["num_staples", "num_fully_bound", "num_bound", "num_self_bound", "num_stacked", "current_c_i"]:
            assert obs[r][k] == ob[k], (r, k)
        assert abs(obs[r]["energy"] - ob["energy"]) <= 1e-12 * max(1.0, abs(ob["energy"]))
        assert eng.config(r) == o.config()


def test_bad_temperature_interval_is_refused():
    from latticednaorigami_gb300 import LdoError
    eng = engine(inp("g24a"), n_replicas=2, seed=1)
    with pytest.raises(LdoError, match="Bad temperature interval"):
        eng.anneal(350.0, 330.0, 3.0, 100)
