"""Umbrella-sampling restart: the reference's .biases files (read_weights /
output_weights, src/us_simulation.cpp:192-244, and the read_biases keys) and
the continuation of iterations across calls and through checkpoints (what the
reference's restart_us_iter archives carry, :272-344)."""
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN
import systems

pytestmark = pytest.mark.gpu

REF_BIASES = os.path.join(GOLDEN, "outputs", "us_update_win1.biases")


def entries(text):
    """The entry blocks of a .biases text, and the text around them."""
    head, _, rest = text.partition('    "biases": [')
    body, _, tail = rest.rpartition("\n    ]\n")
    blocks = [b.strip(",\n") for b in body.split("        }") if b.strip(",\n")]
    return head, sorted(blocks), tail


def test_biases_file_round_trip_matches_reference_layout(tmp_path):
    from latticednaorigami_gb300 import Engine
    inp = systems.write_us_case(str(tmp_path))
    eng = Engine(inp, n_replicas=len(systems.US_WINDOWS), seed=3)
    eng.us_read_biases("grid", 2, REF_BIASES)
    out = str(tmp_path / "w2.biases")
    eng.us_write_biases(2, out)
    with open(REF_BIASES) as f:
        ref = f.read()
    with open(out) as f:
        got = f.read()
    assert entries(got) == entries(ref)
    E = eng.us_biases()
    assert E[2, 1] == -7.328025 and E[2, 2] == 0.0
    assert not E[[0, 1, 3]].any()


def run_us(eng, iters, equil):
    eng.us_run("grid", iters, equil, 400, 2.0, 50)


def state(eng):
    win, _ = eng.us_windows()
    return win.tolist(), eng.us_biases().tolist(), [int(o["draws"]) for o in eng.observables()]


def test_us_iterations_continue_across_calls_and_checkpoints(tmp_path):
    from latticednaorigami_gb300 import Engine
    inp = systems.write_us_case(str(tmp_path))
    nw = len(systems.US_WINDOWS)
    one = Engine(inp, n_replicas=nw, seed=29)
    run_us(one, 4, 300)
    two = Engine(inp, n_replicas=nw, seed=29)
    run_us(two, 2, 300)
    ck = str(tmp_path / "us.ckpt")
    two.save_checkpoint(ck)
    run_us(two, 2, 0)
    assert state(two) == state(one)
    three = Engine(inp, n_replicas=nw, seed=29)
    three.load_checkpoint(ck)
    run_us(three, 2, 0)
    assert state(three) == state(one)
    assert np.abs(np.array(state(one)[1])).max() > 0
    # ldo_us_reset: the next run starts from zero biases again
    two.us_reset()
    run_us(two, 0, 0)
    assert not two.us_biases().any()


def test_read_biases_keys_set_every_window(tmp_path):
    """read_biases with biases_filebase: each window's file is
    <filebase>_win-<min>--<max>.biases (MWUSGCMCSimulation::setup_window_sims)."""
    from latticednaorigami_gb300 import Engine
    d = str(tmp_path)
    inp = systems.write_us_case(d)
    nw = len(systems.US_WINDOWS)
    eng = Engine(inp, n_replicas=nw, seed=31)
    run_us(eng, 2, 300)
    for w, (lo, hi) in enumerate(systems.US_WINDOWS):
        eng.us_write_biases(w, os.path.join(d, "restart_win-%d--%d.biases" % (lo, hi)))
    want = eng.us_biases()
    with open(inp, "a") as f:
        f.write("read_biases=true\nbiases_filebase=restart\n")
    fresh = Engine(inp, n_replicas=nw, seed=31)
    fresh.us_run("grid", 0, 0, 400, 2.0, 0)
    np.testing.assert_allclose(fresh.us_biases(), want, rtol=0, atol=5e-7)   # six decimals in the files
    assert (fresh.us_biases() != 0).sum() == (want != 0).sum()
