"""Batches split by capacity class (ldo_batch_*, csrc/ldo_host.cpp): each
group runs in its own state layout and kernel instantiation, concurrently
with the others, and every replica follows the trajectory it has in one
engine holding the whole batch in the largest class (same Philox stream
key, same moves, same energies)."""
import tempfile

import numpy as np
import pytest

import systems

pytestmark = pytest.mark.gpu


def _cases():
    d = tempfile.mkdtemp()
    # 24-domain staple moves and scaffold regrowth (small class), the
    # 48-domain system (medium class)
    return [systems.write_case(d, "g24e"), systems.write_case(d, "c3"), systems.write_case(d, "s24a")]


def test_batch_groups_by_class_and_matches_one_engine():
    from latticednaorigami_gb300 import Batch, Engine
    inps = _cases()
    sys_of = [0, 1, 2, 1, 0, 2, 1, 0, 2, 0, 1, 1]
    n = len(sys_of)
    temps = np.linspace(320.0, 345.0, n)
    b = Batch(inps, n, seed=11, sys_of_replica=sys_of)
    assert sorted(g["cls"] for g in b.groups) == ["M", "S"]
    for g in b.groups:
        want = {"S": (0, 2), "M": (1,)}[g["cls"]]
        assert all(sys_of[r] in want for r in g["replicas"])
    e = Engine(inps, n, seed=11, sys_of_replica=sys_of)
    for x in (b, e):
        x.set_controls(temps=temps)
        x.set_sampling(5, 200)
    for _ in range(3):
        b.run(300)
        e.run(300)
    sb, cb = b.samples()
    se, ce = e.samples()
    np.testing.assert_array_equal(cb, ce)
    np.testing.assert_array_equal(sb, se)
    obs_e = e.observables()
    for g in b.groups:
        obs_g = g["engine"].observables()
        for k, r in enumerate(g["replicas"]):
            assert obs_g[k]["draws"] == obs_e[r]["draws"]
            assert obs_g[k]["energy"] == obs_e[r]["energy"]
            assert obs_g[k]["num_staples"] == obs_e[r]["num_staples"]
    launches, h2d, d2h = b.counters()
    assert launches >= 3 * len(b.groups)
    b.close()
    e.close()


def test_batch_autotune_keeps_trajectories():
    from latticednaorigami_gb300 import Batch
    inps = _cases()
    sys_of = [0, 1] * 8
    runs = []
    for tune in (False, True):
        b = Batch(inps, len(sys_of), seed=3, sys_of_replica=sys_of)
        if tune:
            reps = b.autotune(probe_sweeps=2, use_cache=False)
            assert len(reps) == len(b.groups)
        b.set_sampling(10, 100)
        b.run_sweeps(20)
        runs.append(b.samples())
        b.close()
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
