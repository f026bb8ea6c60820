"""Algorithmic bytes per move attempt of the c2 and c3 workloads (test
infrastructure: the oracle build with state-touch counters).

The engine's hot path is bound by neither HBM nor tensor cores: each replica's
lattice state lives in shared memory for a whole launch.  Its roofline is
shared-memory traffic, counted on the reference's algorithm as restated by the
oracle (liboracle_touch.so, built by oracle/Makefile): every access to a
domain record (16 bytes: position, orientation, state, partner) and every
operation on the occupancy map (an 8-byte entry), per move attempt, after
burn-in, for the scaffold sizes and temperatures of the workload and both
movesets (the learned one with a uniform proposal table: the moves' own work,
not the quality of a trained network).

    B_attempt = (16 * domain-record accesses + 8 * occupancy operations) / attempts

Run from the repository root: python oracle/touch_counts.py [c2|c3]  (prints
JSON)."""
import ctypes
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

DOM_BYTES, SITE_BYTES = 16, 8


def load():
    so = os.path.join(ROOT, "oracle", "liboracle_touch.so")
    if not os.path.exists(so):
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    L = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    L.oracle_create.restype = vp
    L.oracle_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32]
    L.oracle_destroy.argtypes = [vp]
    L.oracle_run.argtypes = [vp, ctypes.c_longlong, ctypes.c_longlong, vp]
    L.oracle_update_temp.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.oracle_touch_counts.argtypes = [vp, vp, ctypes.c_int]
    L.oracle_set_learn_table.argtypes = [vp, vp, ctypes.c_int]
    L.oracle_last_error.restype = ctypes.c_char_p
    return L


def counts(L, h):
    out = np.zeros(3 * 16, np.int64)
    n = L.oracle_touch_counts(h, out.ctypes.data, len(out))
    if n < 0:
        raise RuntimeError("oracle built without touch counters")
    return out[:3 * n].reshape(n, 3)


def measure(chains, moves_override, burn_sweeps=1500, rec_sweeps=1500, table=None):
    """chains: (system file, scaffold domains, temperature, group, seed)
    per replica; counts are summed per group and over all."""
    L = load()
    by_group, tot = {}, None
    for f, n, temp, group, seed in chains:
        h = L.oracle_create(os.fsencode(f), moves_override.encode(), 0, seed)
        if not h:
            raise RuntimeError(L.oracle_last_error().decode())
        if table is not None:
            L.oracle_set_learn_table(h, table.ctypes.data, len(table))
        L.oracle_update_temp(h, float(temp), 1.0)
        if L.oracle_run(h, burn_sweeps * n, 0, None) != 0:
            raise RuntimeError(L.oracle_last_error().decode())
        c0 = counts(L, h)
        if L.oracle_run(h, rec_sweeps * n, burn_sweeps * n, None) != 0:
            raise RuntimeError(L.oracle_last_error().decode())
        c = counts(L, h) - c0
        L.oracle_destroy(h)
        by_group[group] = c if group not in by_group else by_group[group] + c
        tot = c if tot is None else tot + c

    def bytes_per_attempt(c):
        att = c[:, 0].sum()
        return float((DOM_BYTES * c[:, 1].sum() + SITE_BYTES * c[:, 2].sum()) / att)

    per_move = [float((DOM_BYTES * tot[m, 1] + SITE_BYTES * tot[m, 2]) / max(tot[m, 0], 1)) for m in range(len(tot))]
    return {"bytes_per_attempt": bytes_per_attempt(tot),
            "bytes_per_attempt_by_group": {str(g): bytes_per_attempt(c) for g, c in by_group.items()},
            "bytes_per_attempt_by_movetype": per_move,
            "dom_accesses_per_attempt": float(tot[:, 1].sum() / tot[:, 0].sum()),
            "site_ops_per_attempt": float(tot[:, 2].sum() / tot[:, 0].sum())}


def c2_chains(files):
    """6 replicas per scaffold size of the c2 workload at its temperatures."""
    import bench
    temps = bench.replica_temps()
    per = bench.N_REP // len(bench.SIZES)
    return [(f, bench.SIZES[i], temps[i * per + k], bench.SIZES[i], i * per + k)
            for i, f in enumerate(files) for k in range(6)]


def c3_chains(f):
    """The 48-domain PT system at every eighth of its 64 temperatures, two
    replicas each (constant temperature: the counts per attempt, not the
    exchange)."""
    import bench
    return [(f, 48, bench.C3_TEMPS[q], "%.1f" % bench.C3_TEMPS[q], 2 * q + k) for q in range(0, 64, 9) for k in range(2)]


def main():
    import bench
    workload = sys.argv[1] if len(sys.argv) > 1 else "c2"
    tmp = tempfile.mkdtemp()
    if workload == "c3":
        chains = c3_chains(bench.write_c3(tmp))
        sample = "2 replicas at each of 8 of the 64 temperatures, 1500 sweeps after 1500 burn-in"
    else:
        chains = c2_chains(bench.write_c2(tmp))
        sample = "6 replicas per scaffold size at the workload's temperatures, 1500 sweeps after 1500 burn-in"
    learned = "movetype_file = %s" % bench.write_learned_moves(tmp)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import learn_ref
    table = np.ones(learn_ref.TABLE)
    out = {"workload": workload, "plain": measure(chains, ""), "learned": measure(chains, learned, table=table),
           "dom_bytes": DOM_BYTES, "site_bytes": SITE_BYTES, "sample": sample}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
