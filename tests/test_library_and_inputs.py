"""CPU-side checks: the engine library loads and exports every entry point of
include/ldo.h; input files are read with the reference's option names,
defaults and error behaviour (no GPU call is made)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, inp
from oracle_lib import OracleError, OracleReplica

HEADER = os.path.join(ROOT, "include", "ldo.h")


def declared():
    return sorted(set(re.findall(r"\b(ldo_\w+)\s*\(", open(HEADER).read())))


def test_library_exports_every_declared_symbol():
    from latticednaorigami_gb300.engine import EXPORTS, LIB_PATH
    if not os.path.exists(LIB_PATH):
        pytest.skip("engine library not built here")
    lib = ctypes.CDLL(LIB_PATH)
    missing = [s for s in declared() if not hasattr(lib, s)]
    assert not missing
    assert sorted(EXPORTS) == declared()


def test_create_fails_cleanly_on_bad_input(tmp_path):
    from latticednaorigami_gb300 import Engine, LdoError
    from latticednaorigami_gb300.engine import LIB_PATH
    if not os.path.exists(LIB_PATH):
        pytest.skip("engine library not built here")
    with pytest.raises(LdoError) as e:
        Engine(str(tmp_path / "missing.inp"), n_replicas=1)
    assert "does not exist" in str(e.value)
    bad = tmp_path / "bad.inp"
    bad.write_text(open(inp("c1")).read().replace("domain_type=HalfTurn", "domain_type=Halfturn"))
    os.symlink(os.path.join(ROOT, "tests", "data", "four.json"), tmp_path / "four.json")
    os.symlink(os.path.join(ROOT, "tests", "data", "moves_met3.json"), tmp_path / "moves_met3.json")
    os.symlink(os.path.join(ROOT, "tests", "data", "ops.json"), tmp_path / "ops.json")
    with pytest.raises(LdoError) as e:
        Engine(str(bad), n_replicas=1)
    assert "Halfturn: No such domain type" in str(e.value)


def test_oracle_rejects_like_the_reference(tmp_path):
    # default domain_type "Halfturn" (sic, src/parser.cpp:40) is not a domain type
    text = open(inp("c1")).read().replace("domain_type=HalfTurn\n", "")
    p = tmp_path / "x.inp"
    p.write_text(text.replace("four.json", os.path.join(ROOT, "tests", "data", "four.json"))
                 .replace("moves_met3.json", os.path.join(ROOT, "tests", "data", "moves_met3.json"))
                 .replace("ops.json", os.path.join(ROOT, "tests", "data", "ops.json")))
    with pytest.raises(OracleError, match="Halfturn: No such domain type"):
        OracleReplica(str(p))


def test_misbinding_sequences_are_checked(tmp_path):
    import json
    d = json.load(open(os.path.join(ROOT, "tests", "data", "four.json")))
    # make a staple domain not complementary to its scaffold partner
    d["origami"]["sequences"][1][0] = "A" * 16
    p = tmp_path / "four.json"
    p.write_text(json.dumps(d))
    for f in ["moves_met3.json", "ops.json"]:
        os.symlink(os.path.join(ROOT, "tests", "data", f), tmp_path / f)
    q = tmp_path / "c1.inp"
    q.write_text(open(inp("c1")).read())
    with pytest.raises(OracleError, match="should be complementary"):
        OracleReplica(str(q))


def test_reference_biases_file_reads(tmp_path):
    """USGCMCSimulation::read_weights' format: the .biases file the
    reference's output_weights wrote (golden), read without an engine."""
    from latticednaorigami_gb300.engine import LIB_PATH, read_biases
    if not os.path.exists(LIB_PATH):
        pytest.skip("engine library not built here")
    import json
    from conftest import GOLDEN
    pts, b = read_biases(os.path.join(GOLDEN, "outputs", "us_update_win1.biases"))
    with open(os.path.join(GOLDEN, "us_update_g24a.json")) as f:
        fx = json.load(f)
    E = fx["iterations"][-1]["E"][1]
    assert pts.shape[1] == 1
    got = dict(zip(pts[:, 0].tolist(), b.tolist()))
    want = {x: round(E[x], 6) for x in range(len(E)) if E[x] != 0 or x in got}
    assert set(got) == set(want)
    for x in got:
        assert abs(got[x] - E[x]) <= 5e-7
    bad = tmp_path / "bad.biases"
    bad.write_text('{"biases": [{"bias": 1.0}]}')
    with pytest.raises(Exception):
        read_biases(str(bad))
