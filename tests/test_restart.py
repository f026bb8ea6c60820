"""Restart from a trajectory, on the CPU: the engine library's .trj reader
(ldo_read_trj_frame, host only) against an independent parse of
reference-written trajectories, its error behaviour, and the oracle started
from a trajectory frame.  The traces of the reference itself restarted from
those frames are pinned in tests/test_oracle_golden.py (fixtures *_r*_s*)."""
import glob
import os

import pytest

from conftest import GOLDEN, inp
from oracle_lib import OracleReplica

TRJ = sorted(glob.glob(os.path.join(GOLDEN, "outputs", "*.trj")))


def frames(path):
    """Independent parse: frames split at empty lines; per chain a line
    'index identity', a line of positions, a line of orientations."""
    out = []
    for block in open(path).read().split("\n\n"):
        lines = block.split("\n")
        if not lines or not lines[0].strip():
            continue
        chains = []
        for k in range(1, len(lines) - 2, 3):
            idx, ident = map(int, lines[k].split())
            pos = list(map(int, lines[k + 1].split()))
            ore = list(map(int, lines[k + 2].split()))
            chains.append((idx, ident, pos, ore))
        out.append((int(lines[0]), chains))
    return out


def flat(chains, states=None):
    f = [len(chains)]
    for c, (idx, ident, pos, ore) in enumerate(chains):
        n = len(pos) // 3
        f += [idx, ident, n]
        for d in range(n):
            f += pos[3 * d:3 * d + 3] + ore[3 * d:3 * d + 3] + [0 if states is None else states[c][d]]
    return f


def lib_or_skip():
    from latticednaorigami_gb300.engine import LIB_PATH
    if not os.path.exists(LIB_PATH):
        pytest.skip("engine library not built here")


@pytest.mark.parametrize("path", TRJ, ids=[os.path.basename(p) for p in TRJ])
def test_library_reads_every_frame(path):
    lib_or_skip()
    from latticednaorigami_gb300.engine import read_trj_frame
    fr = frames(path)
    assert len(fr) >= 3
    for k, (_, chains) in enumerate(fr):
        assert read_trj_frame(path, k) == flat(chains)


def test_missing_frame_fails_like_the_reference():
    lib_or_skip()
    from latticednaorigami_gb300 import LdoError
    from latticednaorigami_gb300.engine import read_trj_frame
    path = TRJ[0]
    n = len(frames(path))
    # OrigamiTrajInputFile::go_to_step (src/files.cpp:191)
    with pytest.raises(LdoError, match="Step %d not found in trajectory input file" % n):
        read_trj_frame(path, n)
    with pytest.raises(LdoError, match="does not exist"):
        read_trj_frame(path + ".missing", 0)


def test_oracle_starts_from_the_frame():
    path = os.path.join(GOLDEN, "outputs", "g24a_s3.trj")
    for k, (_, chains) in enumerate(frames(path)):
        o = OracleReplica(inp("g24a"), seed=1, overrides="restart_traj_file=%s\nrestart_step=%d\n" % (path, k))
        got = o.config()
        # positions and orientations as written; states recomputed by set_all_domains
        assert got[0] == len(chains)
        p = 1
        for idx, ident, pos, ore in chains:
            assert got[p:p + 2] == [idx, ident]
            n = got[p + 2]
            assert n == len(pos) // 3
            doms = got[p + 3:p + 3 + 7 * n]
            for d in range(n):
                assert doms[7 * d:7 * d + 3] == pos[3 * d:3 * d + 3]
                assert doms[7 * d + 3:7 * d + 6] == ore[3 * d:3 * d + 3]
            p += 3 + 7 * n
