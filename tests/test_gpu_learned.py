"""Learned proposals on the GPU.

- LearnedStapleExchange and LearnedStapleRegrowth trajectories of the engine
  equal those of the CPU restatement (same weight table, same Philox
  streams): lattice state, counts and draws exactly, energies within 1e-12.
- The network's GPU loss and gradient (the training kernels) against the
  numpy reference oracle/learn_ref.py, and the GPU weight table against the
  reference forward pass.
- Trained on counts from the plain sampler, the network reduces its loss, and
  the learned exchange accepts far more often than the plain one (the gain of
  the learned proposal over the method without it), at least as often as with
  untrained weights."""
import os
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT, inp
from oracle_lib import OracleReplica, set_learn_table
from test_gpu_parity import check_trace
from test_learned_oracle import learned_moves

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import learn_ref  # noqa: E402

pytestmark = pytest.mark.gpu


def engine(*a, **k):
    from latticednaorigami_gb300 import Engine
    return Engine(*a, **k)


@pytest.mark.parametrize("case,regrowth", [("c1", False), ("g24a", False), ("c1", True), ("g24a", True),
                                            ("m8", False), ("m8", True)])
def test_learned_moves_match_oracle_per_step(case, regrowth):
    d = tempfile.mkdtemp()
    over = "movetype_file = %s" % learned_moves(d, regrowth)
    table = np.exp(np.random.default_rng(17).normal(0.0, 2.0, learn_ref.TABLE))
    steps, n, seed = 3000, 6, 99
    eng = engine(inp(case), n_replicas=n, seed=seed, overrides=over)
    eng.learn_set_table(table)
    eng.set_trace(n, steps)
    eng.run(steps)
    tr = eng.trace()
    for r in range(n):
        o = OracleReplica(inp(case), seed=seed, replica=r, overrides=over)
        set_learn_table(o, table)
        check_trace(tr[r], o.run(steps))
        assert eng.config(r) == o.config()


def blocks():
    L = learn_ref
    return [("W1", L.OFF_W1, L.OFF_B1), ("b1", L.OFF_B1, L.OFF_W2), ("W2", L.OFF_W2, L.OFF_B2),
            ("b2", L.OFF_B2, L.OFF_W3), ("W3", L.OFF_W3, L.OFF_B3), ("b3", L.OFF_B3, L.OFF_W4),
            ("w4", L.OFF_W4, L.OFF_B4), ("b4", L.OFF_B4, L.NPARAM)]


def test_gradient_matches_cpu_reference():
    from latticednaorigami_gb300.engine import learn_loss_grad
    rng = np.random.default_rng(4)
    params = learn_ref.init_params(5)
    params[learn_ref.OFF_B1:learn_ref.OFF_W2] = rng.normal(0, 0.1, learn_ref.H)
    n = 3000
    idx = rng.choice(learn_ref.TABLE, n, replace=False).astype(np.int32)
    cnt_t = rng.integers(1, 50, n).astype(np.float32)
    cnt_b = np.floor(cnt_t * rng.random(n)).astype(np.float32)
    loss_g, grad_g = learn_loss_grad(params, idx, cnt_b, cnt_t)
    loss_c, grad_c = learn_ref.loss_grad(params, idx, cnt_b, cnt_t, bf16=True)
    assert abs(loss_g - loss_c) <= 1e-4 * abs(loss_c) + 1e-6, (loss_g, loss_c)
    # bf16 operands, fp32 (GPU) vs fp64 (numpy) accumulation: relative error per block
    for name, a, b in blocks():
        c = grad_c[a:b]
        err = np.linalg.norm(grad_g[a:b] - c) / max(np.linalg.norm(c), 1e-12)
        assert err < 2e-2, (name, err)


def test_weight_table_matches_cpu_reference():
    rng = np.random.default_rng(8)
    params = learn_ref.init_params(9)
    eng = engine(inp("c1"), n_replicas=2, seed=1)
    eng.learn_set_params(params)
    np.testing.assert_array_equal(eng.learn_params(), params)
    w = eng.learn_table()
    idx = rng.choice(learn_ref.TABLE, 4000, replace=False)
    ref = learn_ref.table_weights(params, idx)
    np.testing.assert_allclose(np.log(w[idx]), np.log(ref), atol=2e-2)


def test_trained_network_gains_over_plain_and_untrained():
    import bench
    d = tempfile.mkdtemp()
    f = bench.write_c2(d)[1]                      # 12-domain scaffold, 6 staple types
    over = "movetype_file = %s" % learned_moves(d)
    n = 1024
    temps = np.linspace(320.0, 350.0, n)
    # training data from the plain sampler
    eng = engine(f, n_replicas=n, seed=1)
    eng.set_controls(temps=temps)
    eng.run_sweeps(100)
    for _ in range(20):
        eng.run_sweeps(10)
        eng.learn_collect()
    cb, ct = eng.learn_counts()
    assert ct.sum() > 0 and 0 < cb.sum() < ct.sum()
    l0, l1 = eng.learn_train(300, lr=2e-3, seed=0)
    assert l1 < 0.9 * l0, (l0, l1)
    table = eng.learn_table()

    def exchange_acceptance(overrides, tab):
        e = engine(f, n_replicas=n, seed=2, overrides=overrides)
        e.set_controls(temps=temps)
        if tab is not None:
            e.learn_set_table(tab)
        e.run_sweeps(100)
        s0 = e.move_stats(3)
        e.run_sweeps(200)
        s = e.move_stats(3) - s0
        return s[0, 1] / s[0, 0]

    plain = exchange_acceptance("", None)
    untrained = exchange_acceptance(over, None)
    trained = exchange_acceptance(over, table)
    print("exchange acceptance: plain %.4f, learned untrained %.4f, learned trained %.4f"
          % (plain, untrained, trained))
    # the structural part (unbound scaffold targets, complementary staple,
    # binding orientations) carries the gain over the plain exchange; with
    # the deletion choice weighted towards partly bound staples the trained
    # weights move the acceptance by a few per cent either way (they trade
    # accepted insertions for insertions that stay bound) and must not lose
    # more than a tenth of it
    assert trained > 5 * plain
    assert trained >= 0.9 * untrained

    # regrowth: the trained direction weights against the uniform Met regrowth
    over_lr = "movetype_file = %s" % learned_moves(d, regrowth=True)

    def regrowth_acceptance(overrides, tab):
        e = engine(f, n_replicas=n, seed=3, overrides=overrides)
        e.set_controls(temps=temps)
        if tab is not None:
            e.learn_set_table(tab)
        e.run_sweeps(100)
        s0 = e.move_stats(3)
        e.run_sweeps(200)
        s = e.move_stats(3) - s0
        return s[1, 1] / s[1, 0]

    met = regrowth_acceptance(over, table)
    lr_untrained = regrowth_acceptance(over_lr, None)
    lr_trained = regrowth_acceptance(over_lr, table)
    print("regrowth acceptance: Met %.4f, learned untrained %.4f, learned trained %.4f"
          % (met, lr_untrained, lr_trained))
    assert lr_trained > 2 * met
    assert lr_trained > lr_untrained


def test_learned_distribution_matches_plain_on_c2():
    """KL divergence between the bound-domain distributions of plain and
    learned-proposal MC (learned exchange and learned regrowth) on the
    12-domain c2 system (both relaxed from the empty start for 4000 sweeps,
    then 4000 sweeps sampled every 10)."""
    import bench
    d = tempfile.mkdtemp()
    f = bench.write_c2(d)[1]
    over = "movetype_file = %s" % learned_moves(d, regrowth=True)
    n = 1024
    temps = np.linspace(320.0, 350.0, n)
    eng = engine(f, n_replicas=n, seed=5)
    eng.set_controls(temps=temps)
    eng.run_sweeps(200)
    for _ in range(10):
        eng.run_sweeps(10)
        eng.learn_collect()
    eng.learn_train(300, lr=2e-3, seed=0)
    table = eng.learn_table()

    def hist(overrides, tab, seed):
        e = engine(f, n_replicas=n, seed=seed, overrides=overrides)
        e.set_controls(temps=temps)
        if tab is not None:
            e.learn_set_table(tab)
        for _ in range(4):
            e.run_sweeps(1000)
        e.set_sampling(10, 400)
        for _ in range(4):
            e.run_sweeps(1000)
        smp, cnt = e.samples()
        return np.bincount(np.concatenate([smp[r, :cnt[r], 0] for r in range(n)]).astype(np.int64), minlength=25)

    hp = hist("", None, 6).astype(float)
    hl = hist(over, table, 7).astype(float)
    p, q = hp / hp.sum(), (hl + 0.5) / (hl + 0.5).sum()
    m = p > 0
    kl = float(np.sum(p[m] * np.log(p[m] / q[m])))
    print("KL(plain || learned) = %.5f" % kl)
    assert kl < 0.01, kl
