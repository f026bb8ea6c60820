"""Umbrella sampling on the GPU against the CPU restatement in
tests/us_oracle.py: multi-window US with adaptive grid biases, without and
with neighbouring-window exchange.  The biases after every iteration depend on
every visit count and random draw, so exact agreement of the final grid
biases, window assignments and draw counts checks the whole loop."""
import json
import os
import tempfile

import numpy as np
import pytest

import systems

pytestmark = pytest.mark.gpu

WINDOWS = systems.US_WINDOWS


def write_us_case():
    return systems.write_us_case(tempfile.mkdtemp())


@pytest.mark.parametrize("exchange_interval", [0, 50])
def test_us_matches_cpu_restatement(exchange_interval):
    from latticednaorigami_gb300 import Engine
    from us_oracle import USOracle
    inp = write_us_case()
    seed, iters, equil, steps, max_D = 17, 3, 400, 600, 2.0
    eng = Engine(inp, n_replicas=len(WINDOWS), seed=seed)
    eng.us_run("grid", iters, equil, steps, max_D, exchange_interval)
    win, glen = eng.us_windows()
    ora = USOracle(inp, seed, WINDOWS, "grid", "win", glen)
    ora.run(iters, equil, steps, max_D, exchange_interval)
    assert win.tolist() == ora.window_of
    np.testing.assert_array_equal(eng.us_biases(), np.array(ora.E))
    obs = eng.observables()
    for r, rep in enumerate(ora.reps):
        ob = rep.observables()
        assert obs[r]["draws"] == ob["draws"]
        assert obs[r]["num_fully_bound"] == ob["num_fully_bound"]
    # the biases moved: the loop did something
    assert np.abs(eng.us_biases()).max() > 0
