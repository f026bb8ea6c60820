"""ldo_replica_status_noalloc: the status read-out for callers that may not
allocate device memory (a program whose own pool allocator owns all device
memory, or a step loop that must not stall the device on cudaMalloc/cudaFree).
It keeps its scratch in a fixed device array of the library instead of
engine buffers.  Its output must equal what ldo_get_observables reports for
the same replicas, call after call, and it must refuse more replicas than its
array holds.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import inp

pytestmark = pytest.mark.gpu

LDO_EINVAL, LDO_EINVARIANT = 1, 4
LIMIT = 65536


def moves_with_exchange_mult(tmp_path, mult):
    """Met exchange with an exchange multiplier above 1 on staple type 1: the
    reference throws "Nonsensical exchange probability detected" on the first
    such move whose multiplied probability exceeds 1, so replicas fail at
    different steps and the status words are a mix of zero and nonzero."""
    mv = {"origami": {"movetypes": [
        {"label": "Met staple exchange", "type": "MetStapleExchange", "freq": "1/3", "adaptive_exchange": False,
         "exchange_mults": [mult, 1.0]},
        {"label": "Met staple regrowth", "type": "MetStapleRegrowth", "freq": "1/3"},
        {"label": "CB staple regrowth", "type": "CBStapleRegrowth", "freq": "1/3"}]}}
    p = os.path.join(str(tmp_path), "moves_mult.json")
    with open(p, "w") as f:
        json.dump(mv, f)
    return p


def status_noalloc(eng, n=None):
    n = eng.n if n is None else n
    per = np.full(max(n, 1), -1, np.int32)
    worst, bad = ctypes.c_int32(-1), ctypes.c_int32(-1)
    i32p = ctypes.POINTER(ctypes.c_int32)
    st = eng.lib.ldo_replica_status_noalloc(eng.h, per.ctypes.data_as(i32p), n, ctypes.byref(worst),
                                            ctypes.byref(bad))
    return st, per[:n], worst.value, bad.value


def test_noalloc_status_matches_observables(tmp_path):
    from latticednaorigami_gb300 import Engine
    from latticednaorigami_gb300.engine import LdoError
    mv = moves_with_exchange_mult(tmp_path, 1.5)
    eng = Engine(inp("c1"), n_replicas=64, seed=7, overrides="movetype_file = %s" % mv)
    saw_mix = False
    for call in range(2):                      # two calls in a row share the scratch array
        try:
            eng.run(20)
        except LdoError as x:
            assert x.code == LDO_EINVARIANT
        ref = np.array([o["status"] for o in eng.observables()], np.int32)
        st, per, worst, bad = status_noalloc(eng)
        assert st == 0, eng.lib.ldo_last_error(eng.h)
        np.testing.assert_array_equal(per, ref)
        assert worst == ref.max()
        assert bad == int(np.count_nonzero(ref))
        saw_mix |= 0 < bad < eng.n
    assert saw_mix


def test_noalloc_status_rejects_sizes_beyond_limit():
    from latticednaorigami_gb300 import Engine
    eng = Engine(inp("c1"), n_replicas=8, seed=1)
    st, _, _, _ = status_noalloc(eng, n=7)
    assert st == LDO_EINVAL
    big = Engine(inp("c1"), n_replicas=LIMIT + 1, seed=1)
    st, _, worst, bad = status_noalloc(big)
    assert st == LDO_EINVAL
    assert b"65536" in big.lib.ldo_last_error(big.h)
    assert (worst, bad) == (-1, -1)
    # the engine's own calls are unaffected, and the array still serves a small engine
    st, per, worst, bad = status_noalloc(eng)
    assert (st, worst, bad) == (0, 0, 0)
    np.testing.assert_array_equal(per, np.zeros(8, np.int32))
