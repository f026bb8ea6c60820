"""Configuration import and checkpoint / resume on the GPU.

- ldo_set_config rebuilds a replica from a configuration as the reference's
  constructor does, and the replica then follows the oracle restarted from
  the same configuration (restart_traj_file) step for step;
- a configuration that violates a constraint is refused and leaves the
  replica as it was;
- a checkpoint loaded into a fresh engine (another seed) continues bit for
  bit as the saved engine: plain, scaffold and learned movesets, changed
  temperatures, and a parallel-tempering ladder on its captured graph.
(Restarts of the reference itself from trajectory frames are golden fixtures
run by tests/test_gpu_parity.py.)"""
import os
import tempfile

import numpy as np
import pytest

from conftest import inp
from oracle_lib import OracleReplica
import systems

pytestmark = pytest.mark.gpu

EXACT = [0, 2, 3, 4, 5, 7]


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


def check_trace(tr, ref):
    np.testing.assert_array_equal(tr[:, EXACT], ref[:, EXACT])
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(tr[:, 6], ref[:, 6], rtol=1e-12, atol=1e-12)


def write_trj(path, flat, step=0):
    """A one-frame .trj in the reference's format (OrigamiTrajOutputFile)."""
    lines = [str(step)]
    p = 1
    for _ in range(flat[0]):
        idx, ident, n = flat[p:p + 3]
        doms = flat[p + 3:p + 3 + 7 * n]
        lines.append("%d %d" % (idx, ident))
        lines.append("".join("%d %d %d " % tuple(doms[7 * d:7 * d + 3]) for d in range(n)))
        lines.append("".join("%d %d %d " % tuple(doms[7 * d + 3:7 * d + 6]) for d in range(n)))
        p += 3 + 7 * n
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n\n")
    return path


def restart(trj, frame=0):
    return "restart_traj_file=%s\nrestart_step=%d\n" % (trj, frame)


@pytest.mark.parametrize("case", ["g24a", "c3", "s24a"])
def test_set_config_rebuilds_like_a_restart(case, tmp_path):
    n, seed, steps = 4, 8, 2000
    a = engine(inp(case), n_replicas=n, seed=seed)
    a.run(3000)
    cfg = a.config(1)
    oa = a.observables()[1]
    b = engine(inp(case), n_replicas=n, seed=seed)
    b.set_config(2, cfg)
    assert b.config(2) == cfg
    ob = b.observables()[2]
    for k in ["num_staples", "num_fully_bound", "num_bound", "num_self_bound", "num_stacked", "num_unassigned"]:
        assert ob[k] == oa[k], k
    assert abs(ob["energy"] - oa["energy"]) <= 1e-9 * max(1.0, abs(oa["energy"]))
    assert ob["draws"] == 0
    # the other replicas are untouched
    fresh = engine(inp(case), n_replicas=n, seed=seed)
    for r in [0, 1, 3]:
        assert b.config(r) == fresh.config(r)
    # continuing: the oracle started from the same configuration
    trj = write_trj(str(tmp_path / "cfg.trj"), cfg)
    b.set_trace(n, steps)
    b.run(steps)
    o = OracleReplica(inp(case), seed=seed, replica=2, overrides=restart(trj))
    check_trace(b.trace()[2], o.run(steps))
    assert b.config(2) == o.config()


def test_set_config_refuses_a_violating_configuration():
    from latticednaorigami_gb300 import LdoError
    b = engine(inp("g24a"), n_replicas=2, seed=3)
    b.run(1000)
    before = b.config(1)
    bad = list(before)
    # scaffold domains 1 and 2 on the site of domain 0
    bad[4 + 7:4 + 10] = bad[4:7]
    bad[4 + 14:4 + 17] = bad[4:7]
    with pytest.raises(LdoError, match="Constaints in violation"):
        b.set_config(1, bad)
    assert b.config(1) == before
    with pytest.raises(LdoError, match="ends early"):
        b.set_config(1, before[:-3])
    b.run(500)
    assert b.observables()[1]["status"] == 0


def test_set_configs_batch_equals_one_by_one():
    from latticednaorigami_gb300 import LdoError
    n, seed = 6, 12
    a = engine(inp("c3"), n_replicas=n, seed=seed)
    a.run(2500)
    cfgs = [a.config(r) for r in range(n)][::-1]
    b = engine(inp("c3"), n_replicas=n, seed=seed + 1)
    c = engine(inp("c3"), n_replicas=n, seed=seed + 1)
    b.set_configs(cfgs)
    for r in range(n):
        c.set_config(r, cfgs[r])
    assert [b.config(r) for r in range(n)] == cfgs
    assert b.observables() == c.observables()
    tb, ob, cb = run_traced(b, n, 1500)
    tc, oc, cc = run_traced(c, n, 1500)
    np.testing.assert_array_equal(tb, tc)
    assert cb == cc
    # all or nothing
    before = [b.config(r) for r in range(n)]
    bad = [list(x) for x in before]
    bad[2][4 + 7:4 + 10] = bad[2][4:7]
    bad[2][4 + 14:4 + 17] = bad[2][4:7]
    with pytest.raises(LdoError, match="replica 2: Constaints in violation"):
        b.set_configs(bad)
    assert [b.config(r) for r in range(n)] == before


def run_traced(e, n, steps):
    e.set_trace(n, steps)
    e.run(steps)
    return e.trace(), e.observables(), [e.config(r) for r in range(n)]


@pytest.mark.parametrize("case", ["g24a", "c3", "s24a"])
def test_checkpoint_continues_bit_for_bit(case, tmp_path):
    n, seed = 6, 41
    a = engine(inp(case), n_replicas=n, seed=seed)
    a.run(1500)
    a.set_controls(temps=np.linspace(328.0, 346.0, n))
    a.run(500)
    ck = str(tmp_path / "a.ckpt")
    a.save_checkpoint(ck)
    ta, oa, ca = run_traced(a, n, 2000)
    b = engine(inp(case), n_replicas=n, seed=seed + 1000)
    b.load_checkpoint(ck)
    tb, ob, cb = run_traced(b, n, 2000)
    np.testing.assert_array_equal(ta, tb)
    assert oa == ob
    assert ca == cb


def test_checkpoint_of_learned_moves(tmp_path):
    from test_learned_oracle import learned_moves
    over = "movetype_file = %s" % learned_moves(str(tmp_path), regrowth=True)
    table = np.exp(np.random.default_rng(5).normal(0.0, 2.0, 524544))
    n = 4
    a = engine(inp("g24a"), n_replicas=n, seed=3, overrides=over)
    a.learn_set_table(table)
    a.run(1000)
    ck = str(tmp_path / "l.ckpt")
    a.save_checkpoint(ck)
    ta, oa, ca = run_traced(a, n, 1500)
    b = engine(inp("g24a"), n_replicas=n, seed=4, overrides=over)
    b.load_checkpoint(ck)
    np.testing.assert_array_equal(b.learn_table(), table)
    tb, ob, cb = run_traced(b, n, 1500)
    np.testing.assert_array_equal(ta, tb)
    assert ca == cb


def test_checkpoint_of_a_pt_ladder(tmp_path):
    temps = [325.0, 330.0, 336.0, 343.0]
    umults = [1.0, 1.3, 0.9, 1.1]
    d = tempfile.mkdtemp()
    path = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)),
                                                      chem_pot_mults=" ".join(map(str, umults)),
                                                      num_reps=4, exchange_interval=150))
    a = engine(path, n_replicas=8, seed=31)
    a.pt_run(4, 7, 150, 3)
    ck = str(tmp_path / "pt.ckpt")
    a.save_checkpoint(ck)
    a.pt_run(4, 8, 150, 3)
    b = engine(path, n_replicas=8, seed=77)
    b.load_checkpoint(ck)
    b.pt_run(4, 8, 150, 3)
    np.testing.assert_array_equal(a.pt_permutation(), b.pt_permutation())
    for x, y in zip(a.pt_stats(3), b.pt_stats(3)):
        np.testing.assert_array_equal(x, y)
    assert a.observables() == b.observables()
    assert [a.config(r) for r in range(8)] == [b.config(r) for r in range(8)]


def test_checkpoint_refuses_other_systems(tmp_path):
    from latticednaorigami_gb300 import LdoError
    a = engine(inp("g24a"), n_replicas=4, seed=1)
    ck = str(tmp_path / "x.ckpt")
    a.save_checkpoint(ck)
    with pytest.raises(LdoError, match="other systems or another replica count"):
        engine(inp("g24b"), n_replicas=4, seed=1).load_checkpoint(ck)
    with pytest.raises(LdoError, match="other systems or another replica count"):
        engine(inp("g24a"), n_replicas=5, seed=1).load_checkpoint(ck)
    with open(ck, "rb") as f:
        head = f.read(100)
    with open(str(tmp_path / "t.ckpt"), "wb") as f:
        f.write(head)
    with pytest.raises(LdoError, match="truncated"):
        engine(inp("g24a"), n_replicas=4, seed=1).load_checkpoint(str(tmp_path / "t.ckpt"))
    # one flipped byte in the payload
    data = bytearray(open(ck, "rb").read())
    data[len(data) // 2] ^= 0x40
    with open(str(tmp_path / "c.ckpt"), "wb") as f:
        f.write(bytes(data))
    with pytest.raises(LdoError, match="corrupt"):
        engine(inp("g24a"), n_replicas=4, seed=1).load_checkpoint(str(tmp_path / "c.ckpt"))
