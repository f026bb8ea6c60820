"""Exact staple-only enumeration on the GPU (ldo_enumerate, csrc/ldo_enum.cuh)
against the reference's own enumerator (src/enumerate.cpp, golden weights at
full precision from tests/golden/make_golden.py): the 4-domain system with up
to four staples and the 8-domain system with up to two and up to three
(max_total_staples raised to 3 as in the fixture), where staples bind both
of their domains.  The reference sums its weights in long double, the
engine in FP64: weights agree to 1e-10 relative."""
import json
import os

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,case,max_total,max_type", [("c1_enumeration", "c1", 4, 4),
                                                          ("e8_enumeration", "e8", 2, 1),
                                                          ("e8s3_enumeration", "e8", 3, 1)])
def test_enumeration_matches_reference(name, case, max_total, max_type, data_dir):
    from latticednaorigami_gb300 import Engine
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    eng = Engine(os.path.join(data_dir, case + ".inp"), n_replicas=1, seed=0, overrides=over)
    w, info = eng.enumerate(0, max_total, max_type)
    assert set(w) == set(fx["weights"]), (sorted(w), sorted(fx["weights"]))
    for k, v in fx["weights"].items():
        assert abs(w[k] - v) <= 1e-10 * v, (k, w[k], v)
    assert abs(info["num_configs"] - fx["num_configs"]) <= 1e-9 * fx["num_configs"]


def test_enumeration_units_match_reference(data_dir):
    """Unit by unit: the growth-point sets in the reference's order, each
    with its partition-function sum and number of configurations.

    The reference's per-unit sums are increments of its running partition
    function (long double, 64-bit mantissa): each configuration's weight is
    added to the total so far, so a unit's increment carries an absolute
    error of up to half an ulp of that total per configuration.  The
    tolerance is 1e-10 relative plus that bound (one ulp of the final total
    per configuration); the engine sums each unit from zero in FP64."""
    import numpy as np
    from latticednaorigami_gb300 import Engine
    with open(os.path.join(GOLDEN, "e8_enumeration.json")) as f:
        fx = json.load(f)
    eng = Engine(os.path.join(data_dir, "e8.inp"), n_replicas=1, seed=0)
    eng.enumerate(0, 2, 1)
    units = eng.enumerate_units()
    ref = np.array(fx["units"])
    assert units.shape == ref.shape
    np.testing.assert_array_equal(units[:, 1], ref[:, 1])
    total = ref[:, 0].sum()
    ulp = 2.0 ** -63 * 2.0 ** np.ceil(np.log2(total))
    tol = 1e-10 * np.abs(ref[:, 0]) + np.maximum(ref[:, 1], 1.0) * ulp
    bad = np.abs(units[:, 0] - ref[:, 0]) > tol
    assert not bad.any(), (np.flatnonzero(bad)[:10], units[bad][:5], ref[bad][:5])


@pytest.mark.parametrize("name,max_total,split", [("c1full_enumeration", 2, 0), ("c1full_enumeration", 2, 2),
                                                  ("c1full3_enumeration", 3, 3)])
def test_full_enumeration_matches_reference(name, max_total, split, data_dir):
    """The full conformational enumeration (the scaffold enumerated too,
    ConformationalEnumerator::enumerate) of the 4-domain system with up to
    two and three staples, against the reference's own, whole and split into
    6^split parts per unit.

    The reference adds every configuration's weight to its bin of
    m_state_weights, a running double sum (src/enumerate.cpp:658), over up to
    1e8 configurations per bin; those roundings move a bin by up to (n - 1) u
    relative (n configurations, u = 2^-53; recursive summation's bound,
    Higham, Accuracy and Stability of Numerical Algorithms, 2nd ed., eq.
    4.4), 3e-9 on the ≤3-staple system's smallest bins.  The trace driver
    therefore also sums the reference's own weights, configuration by
    configuration, without that drift (weights_exact: compensated sums,
    oracle/ref/ref_trace.cpp).  The engine's bins (compensated sums of its
    weights) match those at 1e-12, and the reference's printed weights lie
    within the running-sum bound of them.  The reference's running energy
    m_energy (long double) has no drift over a unit (unit_energy_drift)."""
    import numpy as np
    from latticednaorigami_gb300 import Engine
    path = os.path.join(GOLDEN, name + ".json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    with open(path) as f:
        fx = json.load(f)
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    eng = Engine(os.path.join(data_dir, "c1.inp"), n_replicas=1, seed=0, overrides=over)
    w, info = eng.enumerate(0, max_total, 4, full=True, split_levels=split)
    drift = np.array(fx.get("unit_energy_drift", [0.0]))
    offset = np.concatenate([[0.0], np.cumsum(drift)])
    bound = float(np.max(np.abs(offset[:-1]) + np.abs(drift)))
    rtol = 1e-12 + 2 * bound
    exact = fx["weights_exact"]
    assert set(w) == set(fx["weights"]) == set(exact), (sorted(w), sorted(fx["weights"]))
    u = 2.0 ** -53
    for k, v in exact.items():
        assert abs(w[k] - v) <= rtol * v, (k, w[k], v, rtol)
        n = fx["bin_configs"][k]
        # the bin's own running sum, the partition function's (long double,
        # over every configuration), the roundings of the output
        tol = max(n - 1, 1) * u + fx["saved_configs"] * 2.0 ** -64 + 4 * u
        assert abs(fx["weights"][k] - v) <= tol * v, (k, fx["weights"][k], v, n)
    assert abs(info["num_configs"] - fx["num_configs"]) <= 1e-12 * fx["num_configs"]
    if "units" in fx:
        units = eng.enumerate_units()
        ref = np.array(fx["units"])
        assert units.shape == ref.shape
        np.testing.assert_allclose(units[:, 1], ref[:, 1], rtol=1e-12, atol=0)
        total = ref[:, 0].sum()
        ulp = 2.0 ** -63 * 2.0 ** np.ceil(np.log2(total))
        tol = 1e-10 * np.abs(ref[:, 0]) + np.maximum(ref[:, 1], 1.0) * ulp
        bad = np.abs(units[:, 0] - ref[:, 0]) > tol
        assert not bad.any(), (np.flatnonzero(bad)[:10], units[bad][:5], ref[bad][:5])
