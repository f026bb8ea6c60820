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

WINDOWS = [(0, 8), (4, 14), (10, 20), (16, 24)]


def write_us_case():
    d = tempfile.mkdtemp()
    biases = {"origami": {"bias_functions": [
        {"label": "window", "tag": "win", "type": "SquareWell", "min_op": 0, "max_op": 24, "well_bias": 0,
         "outside_bias": 6.0, "ops": ["numfulldomains"], "level": 0},
        {"label": "grid", "tag": "grid", "type": "Grid", "ops": ["numfulldomains"], "level": 0}]}}
    with open(os.path.join(d, "us_biases.json"), "w") as f:
        json.dump(biases, f)
    with open(os.path.join(d, "us.windows"), "w") as f:
        f.write("win\n" + "".join("%d, %d\n" % w for w in WINDOWS))
    return systems.write_case(d, "g24a", extra=dict(bias_functions_file="us_biases.json",
                                                    windows_file="us.windows", us_grid_bias_tag="grid",
                                                    staple_M=1e-2, temp=330))


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
