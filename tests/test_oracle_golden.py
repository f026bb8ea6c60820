"""The oracle against the reference itself: golden per-step traces recorded
from the reference compiled from its own sources (tests/golden/make_golden.py).
Energies must agree bit for bit at every step, and the random-draw count and
final configuration exactly."""
import glob
import gzip
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, inp
from oracle_lib import OracleReplica

FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.json.gz")))


def load(path):
    with gzip.open(path, "rt") as f:
        return json.load(f)


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-8] for p in FIXTURES])
def test_oracle_matches_reference_trace(path):
    fx = load(path)
    o = OracleReplica(inp(fx["case"]), seed=fx["seed"], replica=0)
    tr = o.run(fx["steps"])
    ref = np.array(fx["trace"], dtype=np.float64)
    assert ref.shape == tr.shape
    # step, staples, fully bound, bound, stacked, draws: exact
    np.testing.assert_array_equal(tr[:, [0, 2, 3, 4, 5, 7]], ref[:, [0, 2, 3, 4, 5, 7]])
    # energy and bias: bit for bit
    np.testing.assert_array_equal(tr[:, 1], ref[:, 1])
    np.testing.assert_array_equal(tr[:, 6], ref[:, 6])
    assert o.config() == fx["final_config"]
    assert o.observables()["draws"] == fx["draws"]


def test_fixtures_cover_the_move_and_potential_variants():
    cases = {load(p)["case"] for p in FIXTURES}
    assert {"c1", "g24a", "g24b", "g24c", "g24d", "g24e"} <= cases
    # the fixtures exercise bound staples and stacking, not just empty lattices
    fx = load(os.path.join(GOLDEN, "g24a_s3.json.gz"))
    t = np.array(fx["trace"])
    assert t[:, 2].max() >= 4 and t[:, 5].max() >= 2
