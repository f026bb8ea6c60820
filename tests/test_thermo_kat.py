"""Energy tables: the reference's own unit-test values for the
nearest-neighbour model (tests/src/test_nearest_neighbour.cpp:63-141 of the
reference), and the engine's host table builder against the oracle's, entry
for entry, bit for bit."""
import numpy as np
import pytest

from conftest import inp
from oracle_lib import OracleReplica

# (sequence, temperature, [cation], reduced free energy) from the reference tests
KAT = [("AT", 300, 1, 2.5328725104506113), ("TA", 300, 1, 2.9857702441073424),
       ("TGCA", 300, 1, -5.4850947742870915), ("CT", 300, 1, 0.9057954673134645),
       ("CG", 300, 1, -0.18451389148978148), ("AATTACAGTCTGACGGCC", 300, 1, -43.193024598743925),
       ("AT", 300, 0.5, 2.7895932252887095)]


def lib_or_skip():
    from latticednaorigami_gb300.engine import LIB_PATH
    import os
    if not os.path.exists(LIB_PATH):
        pytest.skip("engine library not built here")


@pytest.mark.parametrize("seq,temp,cation,energy", KAT)
def test_nn_duplex_energy_matches_reference_unit_tests(seq, temp, cation, energy):
    lib_or_skip()
    from latticednaorigami_gb300.engine import nn_duplex_thermo
    h, s = nn_duplex_thermo(seq, temp, cation)
    assert h - s == pytest.approx(energy, rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("case,temp,mult", [("c1", 330, 1.0), ("g24a", 341.5, 1.0), ("g24c", 320, 1.0),
                                            ("g24d", 300, 1.0), ("g24b", 355, 0.8)])
def test_engine_tables_equal_oracle_tables(case, temp, mult):
    lib_or_skip()
    from latticednaorigami_gb300.engine import energy_tables
    o = OracleReplica(inp(case))
    o.update_temp(temp, mult)
    oi, oe, oh, os_, ost, oinit = o.tables()
    imax, (e, h, s, st), init = energy_tables(inp(case), temp, mult)
    assert imax == oi
    # compare only identity pairs present in the system (other entries are unused)
    mask = (oe != 0) | (oh != 0) | (os_ != 0)
    np.testing.assert_array_equal(e[mask], oe[mask])
    np.testing.assert_array_equal(h[mask], oh[mask])
    np.testing.assert_array_equal(s[mask], os_[mask])
    np.testing.assert_array_equal(st[mask], ost[mask])
    np.testing.assert_array_equal(init, oinit)
