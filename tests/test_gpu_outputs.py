"""Output files against the reference's own writers.

tests/golden/outputs holds the files the reference wrote (its
setup_output_files, src/simulation.cpp:47, driven by oracle/ref/ref_trace)
every 400 steps of 2000 on three systems; the engine replays the same
trajectories (same Philox streams) and writes its replica with ldo_writer_*.
Every file must be identical, except .ene whose energies (printed to 10
significant digits) are compared numerically."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import systems

pytestmark = pytest.mark.gpu

RUNS = [("g24a", 3, 2000, 400), ("g24b", 4, 2000, 400), ("c3", 8, 2000, 400)]
EXTS = [".vsf", ".trj", ".vcf", ".states", ".ores", ".counts", ".staples", ".staplestates", ".ops"]


@pytest.mark.parametrize("case,seed,steps,freq", RUNS)
def test_writer_reproduces_reference_output_files(case, seed, steps, freq, tmp_path):
    from latticednaorigami_gb300 import Engine
    d = str(tmp_path)
    inp = systems.write_case(d, case, extra=dict(ops_to_output="numstaples numfulldomains"))
    eng = Engine(inp, n_replicas=1, seed=seed)
    base = os.path.join(d, "out")
    w = eng.open_writer(0, base, 31)
    for step in range(freq, steps + 1, freq):
        eng.run(freq)
        w.write(step)
    w.close()
    ref = os.path.join(GOLDEN, "outputs", "%s_s%d" % (case, seed))
    for ext in EXTS:
        with open(base + ext) as f, open(ref + ext) as g:
            assert f.read() == g.read(), ext
    with open(base + ".ene") as f, open(ref + ".ene") as g:
        got, exp = f.read().splitlines(), g.read().splitlines()
    assert got[0] == exp[0] and len(got) == len(exp)
    a = np.array([[float(x) for x in line.split()] for line in got[1:]])
    b = np.array([[float(x) for x in line.split()] for line in exp[1:]])
    np.testing.assert_array_equal(a[:, 0], b[:, 0])
    np.testing.assert_allclose(a[:, 1:], b[:, 1:], rtol=1e-9, atol=1e-9)
