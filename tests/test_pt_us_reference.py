"""The parallel-tempering and umbrella-sampling restatements (tests/pt_oracle.py,
tests/us_oracle.py) against golden vectors recorded from the reference's own
exchange code (PTGCMCSimulation / OneD- and TwoDPTGCMCSimulation,
USGCMCSimulation / SimpleUSGCMCSimulation, PTMWUSGCMCSimulation; compiled
from its sources and driven by oracle/ref/ref_exchange.cpp, see
tests/golden/make_golden.py).  CPU only: the MC between exchanges is the
oracle's, which the GPU engine reproduces step for step; the engine's own
exchanges are compared with the same fixtures in test_gpu_pt_us_reference.py.

Pinned exactly: calc_acceptance_p of every pair tried, the permutation, the
number of acceptance draws and every replica's controls after every round,
the attempt and swap counts; the reduced staple chemical potentials."""
import glob
import json
import os

import pytest

from conftest import GOLDEN
import systems

PT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "pt_*.json")))


def pt_case(fx, tmp):
    from pt_oracle import PTOracle
    inp = systems.write_case(str(tmp), fx["case"], extra=fx["extra"])
    return PTOracle(inp, fx["oracle_params"], fx["n_ladders"], fx["seed"], exchange_q=fx["q"] or 1,
                    dim2=fx["dim2"], reference_initial_controls=True)


@pytest.mark.parametrize("path", PT_FIXTURES, ids=[os.path.basename(p)[:-5] for p in PT_FIXTURES])
def test_pt_restatement_matches_reference_exchanges(path, tmp_path):
    with open(path) as f:
        fx = json.load(f)
    ora = pt_case(fx, tmp_path)
    assert ora.red_u == fx["red_u"]
    rounds = iter(fx["rounds"])
    R = ora.n_rungs
    for _ in range(fx["swaps"]):
        ora.swap_i += 1
        deps = ora.run_interval(fx["interval"])
        for l in range(ora.n_ladders):
            rec = next(rounds)
            assert (rec["ladder"], rec["swap_i"]) == (l, ora.swap_i)
            perm = ora.perm[l]
            ps = [ora.acceptance(i, i2, perm[i], perm[i2], deps) for i, i2, _ in ora.pairs()]
            assert ps == rec["p"]
            ora.exchange(l, deps)
            assert ora.perm[l] == rec["perm"]
            assert ora.draws[l] == rec["draws"]
            for k in range(R):
                c = ora.ctrl[l * R + k]
                assert [c["temp"], c["u"], c["bias"], c["stack"]] == rec["ctl"][4 * k:4 * k + 4]
    assert ora.att == fx["att"] and ora.acc == fx["acc"]
    assert sum(fx["acc"]) > 0 and sum(fx["acc"]) < sum(fx["att"])


def us_case(tmp):
    return systems.write_us_case(str(tmp)), systems.US_WINDOWS


def test_us_updates_match_reference(tmp_path):
    """SimpleUSGCMCSimulation::process_iteration of the reference on the
    oracle's visit counts: the restatement's grid biases of every window
    after every iteration, bit for bit."""
    from us_oracle import USOracle
    import numpy as np
    with open(os.path.join(GOLDEN, "us_update_g24a.json")) as f:
        fx = json.load(f)
    inp, windows = us_case(tmp_path)
    assert [list(w) for w in windows] == fx["windows"]
    seen = []

    class Rec(USOracle):
        def process(self, hist, max_D):
            super().process(hist, max_D)
            seen.append(([list(map(int, h)) for h in hist], [e.tolist() for e in self.E]))

    ora = Rec(inp, fx["seed"], windows, "grid", "win", fx["grid_len"])
    ora.run(fx["iters"], fx["equil"], fx["steps"], fx["max_D"], 0)
    assert len(seen) == len(fx["iterations"])
    for (hist, E), it in zip(seen, fx["iterations"]):
        assert hist == it["hist"]
        assert E == it["E"]
    assert ora.window_of == fx["window_of"]
    assert [int(r.observables()["draws"]) for r in ora.reps] == fx["draws"]
    assert np.abs(np.array(fx["iterations"][-1]["E"])).max() > 0


def test_us_window_exchanges_match_reference(tmp_path):
    """PTMWUSGCMCSimulation::attempt_exchange of the reference on seeded
    points and biases: the restatement's window-to-configuration map, draw
    count, attempt and swap counts after every round."""
    from us_oracle import USOracle
    import numpy as np
    with open(os.path.join(GOLDEN, "us_exchange.json")) as f:
        fx = json.load(f)
    inp, windows = us_case(tmp_path)
    ora = USOracle(inp, fx["seed"], windows, "grid", "win", 25)
    for rec in fx["rounds"]:
        ora.E = [np.array(e) for e in rec["E"]]
        ora.exchange_points(rec["points"], rec["swap_i"])
        assert ora.replica_of == rec["configi"], rec["swap_i"]
        assert ora.draws == rec["draws"]
    assert ora.att == fx["att"] and ora.acc == fx["acc"]
    assert 0 < sum(fx["acc"]) < sum(fx["att"])
