"""ctypes wrapper of the CPU oracle (oracle/liboracle.so), the checker the
GPU engine is compared with.  Test infrastructure only."""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            import subprocess
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        L = ctypes.CDLL(ORACLE_SO)
        vp = ctypes.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_run.argtypes = [vp, ctypes.c_longlong, ctypes.c_longlong, vp]
        L.oracle_get_config.argtypes = [vp, vp, ctypes.c_int]
        L.oracle_observables.argtypes = [vp, vp]
        L.oracle_move_stats.argtypes = [vp, vp, ctypes.c_int]
        L.oracle_tables.argtypes = [vp, vp, vp, vp, vp, vp]
        L.oracle_update_temp.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.oracle_dependent_qs.argtypes = [vp, vp]
        L.oracle_set_grid.argtypes = [vp, ctypes.c_char_p, vp, ctypes.c_int]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_run_batch.restype = ctypes.c_double
        L.oracle_run_batch.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int,
                                       ctypes.c_longlong, ctypes.c_int]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


class OracleReplica:
    """One replica of the CPU restatement, same Philox stream as the engine's
    replica `replica` under `seed`."""

    def __init__(self, inp, seed=0, replica=0, overrides=""):
        self.L = lib()
        self.h = self.L.oracle_create(os.fsencode(inp), overrides.encode(), seed, replica)
        if not self.h:
            raise OracleError(self.L.oracle_last_error().decode())
        self.step = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def set_reference_arithmetic(self, on=True):
        """The reference's own arithmetic: long double Rosenbluth weights and
        the C library's exp (default: the engine's FP64 weights and its own
        exp, ldo_math.h, which the GPU computes bit for bit alike)."""
        self.L.oracle_set_reference_arithmetic.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.oracle_set_reference_arithmetic(self.h, 1 if on else 0)

    def run(self, steps, trace=True):
        tr = np.zeros((steps, 8)) if trace else None
        rc = self.L.oracle_run(self.h, steps, self.step, tr.ctypes.data if trace else None)
        if rc != 0:
            raise OracleError(self.L.oracle_last_error().decode())
        self.step += steps
        return tr

    def config(self):
        buf = np.zeros(1 << 16, np.int32)
        n = self.L.oracle_get_config(self.h, buf.ctypes.data, len(buf))
        return buf[:n].tolist()

    def observables(self):
        o = np.zeros(10)
        self.L.oracle_observables(self.h, o.ctypes.data)
        keys = ["energy", "num_staples", "num_fully_bound", "num_bound", "num_self_bound", "num_stacked",
                "num_unassigned", "total_bias", "draws", "current_c_i"]
        return dict(zip(keys, o.tolist()))

    def move_stats(self, n):
        o = np.zeros(2 * n, np.int64)
        self.L.oracle_move_stats(self.h, o.ctypes.data, 2 * n)
        return o.reshape(n, 2)

    def tables(self):
        imax = self.L.oracle_tables(self.h, None, None, None, None, None)
        d = 2 * imax + 1
        e, h, s, st = (np.zeros(d * d) for _ in range(4))
        init = np.zeros(3)
        self.L.oracle_tables(self.h, e.ctypes.data, h.ctypes.data, s.ctypes.data, st.ctypes.data, init.ctypes.data)
        return imax, e.reshape(d, d), h.reshape(d, d), s.reshape(d, d), st.reshape(d, d), init

    def update_temp(self, temp, stacking_mult=1.0):
        if self.L.oracle_update_temp(self.h, temp, stacking_mult) != 0:
            raise OracleError(self.L.oracle_last_error().decode())

    def dependent_qs(self):
        o = np.zeros(4)
        self.L.oracle_dependent_qs(self.h, o.ctypes.data)
        return o

    def set_grid(self, tag, values):
        v = np.ascontiguousarray(values, np.float64)
        if self.L.oracle_set_grid(self.h, tag.encode(), v.ctypes.data, len(v)) != 0:
            raise OracleError(self.L.oracle_last_error().decode())


def run_batch(inp, seed, n_rep, steps, threads, overrides=""):
    """CPU baseline: wall seconds for n_rep replicas x steps on `threads` threads."""
    t = lib().oracle_run_batch(os.fsencode(inp), overrides.encode(), seed, n_rep, steps, threads)
    if t < 0:
        raise OracleError(lib().oracle_last_error().decode() or "oracle batch failed")
    return t


def staple_counts(rep):
    L = lib()
    L.oracle_staple_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    out = np.zeros(256, np.int32)
    n = L.oracle_staple_counts(rep.h, out.ctypes.data, 256)
    return out[:n]


def swap_uniform(seed, ladder, index):
    L = lib()
    L.oracle_swap_uniforms.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_ulonglong, ctypes.c_int,
                                       ctypes.c_void_p]
    out = np.zeros(1)
    L.oracle_swap_uniforms(seed, ladder, index, 1, out.ctypes.data)
    return float(out[0])


def run_golden(o, fx):
    """The run a golden fixture records: fx["steps"] steps, or, for a fixture
    of the reference's annealing loop (AnnealingGCMCSimulation::run), the
    temperatures max_temp, max_temp - interval, ... down to min_temp with
    update_temp before steps_per_temp steps at each (the systems of these
    fixtures have no biases, so the staple chemical potentials that
    update_staple_us changes do not enter)."""
    if "anneal" not in fx:
        return o.run(fx["steps"])
    tmax, tmin, dt, steps, _ = fx["anneal"]
    steps = int(steps)
    parts = []
    t = tmax
    step = 0
    while t >= tmin:
        o.update_temp(t)
        # the reference's step counter: step += simulate(steps, step), and
        # simulate returns its last step + 1 (src/annealing_simulation.cpp:47,
        # src/simulation.cpp:568), so every temperature after the first starts
        # at a step number that jumps ahead
        o.step = step
        parts.append(o.run(steps))
        step += step + steps + 1
        t -= dt
    return np.concatenate(parts)


def run_batch_sampled(inp, seed, n_rep, sweeps, sweep_len, threads, overrides="", temps=None):
    """CPU baseline with one numfulldomains sample per replica per sweep:
    returns (wall seconds, samples[n_rep, sweeps]).  temps[n_rep], if given,
    sets each replica's temperature before the timed run."""
    L = lib()
    L.oracle_run_batch_sampled.restype = ctypes.c_double
    L.oracle_run_batch_sampled.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int,
                                           ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p]
    out = np.zeros((n_rep, sweeps), np.int16)
    tp = None
    if temps is not None:
        temps = np.ascontiguousarray(temps, np.float64)
        assert len(temps) == n_rep
        tp = temps.ctypes.data
    t = L.oracle_run_batch_sampled(os.fsencode(inp), overrides.encode(), seed, n_rep, sweeps, sweep_len, threads,
                                   tp, out.ctypes.data)
    if t < 0:
        raise OracleError(L.oracle_last_error().decode() or "oracle batch failed")
    return t, out


def run_batch_sampled_centres(inp, seed, n_rep, sweeps, sweep_len, threads, temps, centre_tag, centres,
                              overrides=""):
    """run_batch_sampled with one Harmonic bias centre per replica."""
    L = lib()
    L.oracle_run_batch_sampled_centres.restype = ctypes.c_double
    L.oracle_run_batch_sampled_centres.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int,
                                                   ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros((n_rep, sweeps), np.int16)
    temps = np.ascontiguousarray(temps, np.float64)
    centres = np.ascontiguousarray(centres, np.float64)
    assert len(temps) == n_rep and len(centres) == n_rep
    t = L.oracle_run_batch_sampled_centres(os.fsencode(inp), overrides.encode(), seed, n_rep, sweeps, sweep_len,
                                           threads, temps.ctypes.data, centre_tag.encode(), centres.ctypes.data,
                                           out.ctypes.data)
    if t < 0:
        raise OracleError(L.oracle_last_error().decode() or "oracle batch failed")
    return t, out


def set_bias_centre(rep, tag, centre):
    L = rep.L
    L.oracle_set_bias_centre.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double]
    if L.oracle_set_bias_centre(rep.h, tag.encode(), float(centre)) != 0:
        raise OracleError(L.oracle_last_error().decode())


def uniform(seed, key1, stream, index):
    L = lib()
    L.oracle_uniforms.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_ulonglong,
                                  ctypes.c_int, ctypes.c_void_p]
    out = np.zeros(1)
    L.oracle_uniforms(seed, key1, stream, index, 1, out.ctypes.data)
    return float(out[0])


def set_window(rep, tag, min_op, max_op):
    L = lib()
    L.oracle_set_window.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    if L.oracle_set_window(rep.h, tag.encode(), min_op, max_op) != 0:
        raise OracleError(L.oracle_last_error().decode())


def run_batch_states(inp, seed, n_rep, burn, gap, n_snaps, threads, overrides="", learn_w=None):
    """Independent replicas; (staples, fully bound) at n_snaps snapshots after
    burn steps, gap steps apart: int32[n_rep, n_snaps, 2]."""
    L = lib()
    L.oracle_run_batch_states.restype = ctypes.c_int
    L.oracle_run_batch_states.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros((n_rep, n_snaps, 2), np.int32)
    w = None
    if learn_w is not None:
        w = np.ascontiguousarray(learn_w, np.float64)
    rc = L.oracle_run_batch_states(os.fsencode(inp), overrides.encode(), seed, n_rep, burn, gap, n_snaps, threads,
                                   w.ctypes.data if w is not None else None, out.ctypes.data)
    if rc != 0:
        raise OracleError(L.oracle_last_error().decode() or "oracle batch failed")
    return out


def set_learn_table(rep, w):
    L = rep.L
    L.oracle_set_learn_table.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    w = np.ascontiguousarray(w, np.float64)
    rep._learn_w = w
    if L.oracle_set_learn_table(rep.h, w.ctypes.data, len(w)) != 0:
        raise OracleError(L.oracle_last_error().decode())


def engine_exp(x):
    """ldo_math::exp evaluated on the host."""
    L = lib()
    L.oracle_engine_exp.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    L.oracle_engine_exp(x.ctypes.data, y.ctypes.data, len(x))
    return y
