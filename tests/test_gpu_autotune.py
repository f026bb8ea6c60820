"""The engine's autotuner (ldo_autotune): it times candidate launch shapes on
the engine's own batch and keeps the fastest, restoring the replicas' state
after every probe.  Tuning must change no result: a tuned engine and an
untuned one with the same seed follow the same trajectories, bit for bit,
through plain runs and a parallel-tempering run."""
import tempfile

import numpy as np
import pytest

import systems

pytestmark = pytest.mark.gpu


def mixed_batch():
    d = tempfile.mkdtemp()
    return [systems.write_case(d, "g24a"), systems.write_case(d, "c1")]


def run_both(tune):
    from latticednaorigami_gb300 import Engine
    files = mixed_batch()
    sys_of = [k % 2 for k in range(96)]
    eng = Engine(files, n_replicas=96, seed=77, sys_of_replica=sys_of)
    eng.set_controls(temps=np.linspace(320.0, 345.0, 96))
    report = eng.autotune(probe_sweeps=3, use_cache=False) if tune else None
    eng.set_sampling(1, 40)
    eng.run_sweeps(40)
    smp, cnt = eng.samples()
    obs = eng.observables()
    cfg = [eng.config(r) for r in range(0, 96, 7)]
    return report, smp, cnt, obs, cfg


def test_autotune_changes_no_trajectory():
    report, smp_t, cnt_t, obs_t, cfg_t = run_both(True)
    _, smp, cnt, obs, cfg = run_both(False)
    assert report["n_candidates"] > 0
    assert report["best_ms"] <= report["default_ms"]
    assert len(report["candidates"]) == report["n_candidates"]
    assert report["warps_per_block"] in (1, 2, 4)
    np.testing.assert_array_equal(cnt_t, cnt)
    np.testing.assert_array_equal(smp_t, smp)
    for a, b in zip(obs_t, obs):
        assert a["draws"] == b["draws"] and a["energy"] == b["energy"] and a["num_staples"] == b["num_staples"]
    assert cfg_t == cfg


def test_autotuned_pt_matches_untuned():
    from latticednaorigami_gb300 import Engine
    temps = [325.0, 330.0, 336.0, 343.0]
    d = tempfile.mkdtemp()
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)), num_reps=4))
    perms = []
    for tune in (True, False):
        eng = Engine(inp, n_replicas=32, seed=19)
        if tune:
            eng.autotune(probe_sweeps=2, use_cache=False)
        eng.pt_run(4, 10, 150, 1)
        perms.append(eng.pt_permutation().tolist())
        obs = eng.observables()
        perms.append([o["draws"] for o in obs])
    assert perms[0] == perms[2] and perms[1] == perms[3]
