"""The engine's in-kernel exchanges against golden vectors recorded from the
reference's own exchange code (see tests/test_pt_us_reference.py and
tests/golden/make_golden.py): the engine's MC between exchanges reproduces the
oracle's step for step, so its permutations and attempt/swap counts must be
the reference's decisions exactly.

The reference's initialize_control_qs gives every replica the staple-u
multiplier 1 (its bias multiplier) until its first exchange; the engine uses
chem_pot_mults from the start.  The fixture whose chem_pot_mults differ from 1
(pt_ut_g24a) therefore pins only the CPU restatement run with the reference's
initial controls, not the engine."""
import glob
import json
import os

import pytest

from conftest import GOLDEN
import systems

pytestmark = pytest.mark.gpu

ENGINE_PT = [p for p in sorted(glob.glob(os.path.join(GOLDEN, "pt_*.json")))
             if not os.path.basename(p).startswith("pt_ut_")]


@pytest.mark.parametrize("path", ENGINE_PT, ids=[os.path.basename(p)[:-5] for p in ENGINE_PT])
def test_engine_pt_matches_reference_exchanges(path, tmp_path):
    from latticednaorigami_gb300 import Engine
    with open(path) as f:
        fx = json.load(f)
    inp = systems.write_case(str(tmp_path), fx["case"], extra=fx["extra"])
    R = len(fx["oracle_params"]["temps"]) * (fx["dim2"] or 1)
    eng = Engine(inp, n_replicas=R * fx["n_ladders"], seed=fx["seed"])
    if fx["dim2"]:
        eng.pt2d_run(len(fx["oracle_params"]["temps"]), fx["dim2"], fx["swaps"], fx["interval"])
    else:
        eng.pt_run(R, fx["swaps"], fx["interval"], fx["q"])
    assert eng.pt_permutation().tolist() == fx["final_perm"]
    att, acc = eng.pt_stats(len(fx["att"]))
    assert att.tolist() == fx["att"] and acc.tolist() == fx["acc"]
    # the ladders' last exchange round, replica controls included
    last = {r["ladder"]: r for r in fx["rounds"] if r["swap_i"] == fx["swaps"]}
    obs = eng.observables()
    for l, rec in last.items():
        for k in range(R):
            assert obs[l * R + k]["temp"] == rec["ctl"][4 * k], (l, k)


def test_engine_us_updates_match_reference():
    """Umbrella iterations without window exchange: the engine's grid biases
    after the last iteration are the reference's SimpleUSGCMCSimulation
    updates (tests/golden/us_update_g24a.json), bit for bit."""
    import tempfile
    import numpy as np
    from latticednaorigami_gb300 import Engine
    with open(os.path.join(GOLDEN, "us_update_g24a.json")) as f:
        fx = json.load(f)
    inp = systems.write_us_case(tempfile.mkdtemp())
    eng = Engine(inp, n_replicas=len(fx["windows"]), seed=fx["seed"])
    eng.us_run("grid", fx["iters"], fx["equil"], fx["steps"], fx["max_D"], 0)
    win, glen = eng.us_windows()
    assert glen >= fx["grid_len"]   # the engine's grid spans every possible value; the fixture 0..24
    assert win.tolist() == fx["window_of"]
    E = eng.us_biases()
    np.testing.assert_array_equal(E[:, :fx["grid_len"]], np.array(fx["iterations"][-1]["E"]))
    assert not E[:, fx["grid_len"]:].any()
    assert [int(o["draws"]) for o in eng.observables()] == fx["draws"]
