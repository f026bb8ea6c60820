"""Algorithmic bytes per move attempt of the c2 workload (test
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

Run from the repository root: python oracle/touch_counts.py  (prints JSON)."""
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


def measure(files, moves_override, reps_per_size=6, burn_sweeps=1500, rec_sweeps=1500, table=None):
    import bench
    L = load()
    temps = bench.replica_temps()
    per = bench.N_REP // len(bench.SIZES)
    by_size, tot = {}, None
    for i, f in enumerate(files):
        n = bench.SIZES[i]
        acc = None
        for k in range(reps_per_size):
            h = L.oracle_create(os.fsencode(f), moves_override.encode(), 0, i * per + k)
            if not h:
                raise RuntimeError(L.oracle_last_error().decode())
            if table is not None:
                L.oracle_set_learn_table(h, table.ctypes.data, len(table))
            L.oracle_update_temp(h, float(temps[i * per + k]), 1.0)
            if L.oracle_run(h, burn_sweeps * n, 0, None) != 0:
                raise RuntimeError(L.oracle_last_error().decode())
            c0 = counts(L, h)
            if L.oracle_run(h, rec_sweeps * n, burn_sweeps * n, None) != 0:
                raise RuntimeError(L.oracle_last_error().decode())
            c = counts(L, h) - c0
            acc = c if acc is None else acc + c
            L.oracle_destroy(h)
        by_size[n] = acc
        tot = acc if tot is None else tot + acc

    def bytes_per_attempt(c):
        att = c[:, 0].sum()
        return float((DOM_BYTES * c[:, 1].sum() + SITE_BYTES * c[:, 2].sum()) / att)

    per_move = [float((DOM_BYTES * tot[m, 1] + SITE_BYTES * tot[m, 2]) / max(tot[m, 0], 1)) for m in range(len(tot))]
    return {"bytes_per_attempt": bytes_per_attempt(tot),
            "bytes_per_attempt_by_size": {str(n): bytes_per_attempt(c) for n, c in by_size.items()},
            "bytes_per_attempt_by_movetype": per_move,
            "dom_accesses_per_attempt": float(tot[:, 1].sum() / tot[:, 0].sum()),
            "site_ops_per_attempt": float(tot[:, 2].sum() / tot[:, 0].sum())}


def main():
    import bench
    tmp = tempfile.mkdtemp()
    files = bench.write_c2(tmp)
    learned = "movetype_file = %s" % bench.write_learned_moves(tmp)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import learn_ref
    table = np.ones(learn_ref.TABLE)
    out = {"plain": measure(files, ""), "learned": measure(files, learned, table=table),
           "dom_bytes": DOM_BYTES, "site_bytes": SITE_BYTES,
           "sample": "6 replicas per scaffold size at the workload's temperatures, 1500 sweeps after 1500 burn-in"}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
