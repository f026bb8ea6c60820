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


@pytest.mark.parametrize("freq", [150, 300])
def test_swap_file_follows_pt_permutations(freq, tmp_path):
    """.swp of ladder 1 (PTGCMCSimulation::initialize_swap_file /
    write_swap_entry): header of the exchanged controls per slot, then before
    every exchange whose step is a multiple of freq the slot -> replica row,
    and the end-of-run row; permutations from the CPU restatement."""
    from latticednaorigami_gb300 import Engine
    from pt_oracle import PTOracle
    temps = [325.0, 330.0, 336.0, 343.0]
    umults = [1.0, 1.3, 0.9, 1.1]
    d = str(tmp_path)
    inp = systems.write_case(d, "g24a", extra=dict(temps=" ".join(map(str, temps)),
                                                   chem_pot_mults=" ".join(map(str, umults)), num_reps=4))
    n_ladders, swaps, interval, seed, q, lad = 2, 12, 150, 31, 3, 1
    eng = Engine(inp, n_replicas=4 * n_ladders, seed=seed)
    base = os.path.join(d, "pt")
    w = eng.open_swap_writer(4, q, lad, base, freq)
    eng.pt_run(4, swaps, interval, q)
    w.write(swaps * interval)
    w.close()
    ora = PTOracle(inp, dict(temps=temps, chem_pot_mults=umults, temp=335.0, staple_M=1e-3,
                             staple_lengths=[2] * 12), n_ladders, seed, exchange_q=q)
    expect = ["".join("%g/%g/ " % (t, u) for t, u in zip(temps, umults))]
    for k in range(1, swaps + 1):
        row = [x - lad * 4 for x in ora.perm[lad]]
        if (k * interval) % freq == 0:
            expect.append("".join("%d " % x for x in row))
        ora.round(interval)
    expect.append("".join("%d " % (x - lad * 4) for x in ora.perm[lad]))
    with open(base + ".swp") as f:
        got = f.read().split("\n")
    assert got[-1] == ""
    assert got[:-1] == expect


def test_times_file_format(tmp_path):
    from latticednaorigami_gb300 import Engine
    d = str(tmp_path)
    inp = systems.write_case(d, "g24a")
    eng = Engine(inp, n_replicas=1, seed=1)
    base = os.path.join(d, "t")
    w = eng.open_writer(0, base, 32)
    for step in (100, 200, 300):
        eng.run(100)
        w.write(step)
    w.close()
    with open(base + ".times") as f:
        lines = f.read().splitlines()
    assert lines[0] == "step time"
    rows = [line.split() for line in lines[1:]]
    assert [int(r[0]) for r in rows] == [100, 200, 300]
    t = [float(r[1]) for r in rows]
    assert 0 <= t[0] <= t[1] <= t[2]
