"""The exact enumerator's work units, listed on the host (no GPU): the
staple sets and growth-point sets without repeats that the reference walks
(StapleEnumerator::enumerate, src/enumerate.cpp:1082; GrowthpointEnumerator
::enumerate, :819), against the number of units the reference's own
enumeration ran (the per-unit sums its trace driver recorded in the golden
files), for both growth-point enumerators (misbinding, no misbinding) and
the staple-only and full enumerations."""
import json
import os

import pytest

from conftest import GOLDEN, inp


@pytest.mark.parametrize("name,case,max_total,max_type", [("e8_enumeration", "e8", 2, 1),
                                                          ("m8_enumeration", "m8", 3, 1),
                                                          ("c1full_enumeration", "c1", 2, 4),
                                                          ("c1full3_enumeration", "c1", 3, 4)])
def test_units_match_the_reference_count(name, case, max_total, max_type):
    from latticednaorigami_gb300.engine import enumeration_plan
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    plan = enumeration_plan(inp(case), 0, max_total, max_type, overrides=over)
    assert len(plan) == len(fx["units"])
    # the empty staple set first, then every unit with one growth point per staple
    assert tuple(plan[0]) == (0, 0)
    assert (plan[1:, 0] >= 1).all() and (plan[1:, 0] <= max_total).all()
    assert (plan[:, 1] == plan[:, 0]).all()
    # units with the same staple count are contiguous, in increasing count
    assert (plan[1:, 0] >= plan[:-1, 0]).all()


@pytest.mark.parametrize("name,case,max_total,max_type", [("c1_enumeration", "c1", 4, 4),
                                                          ("e8s3_enumeration", "e8", 3, 1),
                                                          ("e8s4_enumeration", "e8", 4, 1)])
def test_unit_count_matches_the_reference(name, case, max_total, max_type):
    """The larger staple-only enumerations (the reference's unit count only):
    up to 151 553 growth-point sets, each checked against those enumerated
    before it."""
    from latticednaorigami_gb300.engine import enumeration_plan
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    if "n_units" not in fx:
        pytest.skip("fixture without a unit count")
    over = "\n".join("%s = %s" % kv for kv in sorted(fx["options"].items()))
    plan = enumeration_plan(inp(case), 0, max_total, max_type, overrides=over)
    assert len(plan) == fx["n_units"]


def test_plan_refuses_a_system_without_an_enumerator(tmp_path):
    from latticednaorigami_gb300.engine import LdoError, enumeration_plan
    with pytest.raises(LdoError, match="No enumerator"):
        enumeration_plan(inp("c4"), 0, 1, 1)
