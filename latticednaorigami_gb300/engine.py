"""ctypes binding of the engine's C ABI (include/ldo.h).

The engine itself is CUDA; this module only marshals arguments.  Loading fails
loudly if the compiled library is missing: there is no CPU fallback."""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libldo_gb300.so")

STATUS = {0: "LDO_OK", 1: "LDO_EINVAL", 2: "LDO_ENOMEM", 3: "LDO_ECUDA",
          4: "LDO_EINVARIANT", 5: "LDO_EITERCAP", 6: "LDO_ECAPACITY"}

# Names and order of every entry point declared in include/ldo.h.
EXPORTS = [
    "ldo_create_from_inp", "ldo_create_multi", "ldo_destroy", "ldo_last_error", "ldo_num_replicas",
    "ldo_set_controls", "ldo_run", "ldo_run_sweeps", "ldo_state_bytes", "ldo_get_observables", "ldo_get_config", "ldo_set_sampling",
    "ldo_get_samples", "ldo_get_counters", "ldo_set_trace", "ldo_get_trace", "ldo_get_move_stats", "ldo_set_grid_bias",
    "ldo_set_window", "ldo_pt_run", "ldo_pt_get_permutation", "ldo_pt_get_stats", "ldo_nn_duplex_thermo",
    "ldo_energy_tables", "ldo_us_run", "ldo_us_get_biases", "ldo_us_get_windows", "ldo_replica_status_noalloc",
    "ldo_learn_collect", "ldo_learn_reset_counts", "ldo_learn_get_counts", "ldo_learn_train", "ldo_learn_set_params",
    "ldo_learn_get_params", "ldo_learn_get_table", "ldo_learn_set_table", "ldo_learn_loss_grad",
    "ldo_writer_open", "ldo_writer_write", "ldo_writer_close", "ldo_pt2d_run", "ldo_engine_exp",
    "ldo_set_bias_centre", "ldo_swap_writer_open", "ldo_set_config", "ldo_set_configs", "ldo_anneal_run", "ldo_read_trj_frame", "ldo_checkpoint_save",
    "ldo_checkpoint_load", "ldo_autotune", "ldo_autotune_candidates", "ldo_us_write_biases",
    "ldo_us_read_biases", "ldo_us_reset", "ldo_read_biases", "ldo_enumerate", "ldo_enumerate_full", "ldo_enumerate_units",
    "ldo_enumerate_unit_weights", "ldo_enumeration_plan",
    "ldo_batch_create", "ldo_batch_destroy", "ldo_batch_last_error", "ldo_batch_num_groups", "ldo_batch_group",
    "ldo_batch_set_controls", "ldo_batch_run", "ldo_batch_run_sweeps", "ldo_batch_set_sampling",
    "ldo_batch_get_samples", "ldo_batch_get_counters", "ldo_batch_autotune",
]

LEARN_TABLE = 524544      # network inputs: 524288 insertion + 256 regrowth-direction (ldo_learn.h)
LEARN_NPARAM = 148481     # network parameters


class LdoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class TuneReport(ctypes.Structure):
    _fields_ = [("warps_per_block", ctypes.c_int32), ("smem_pad_bytes", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("interleaved", ctypes.c_int32), ("best_ms", ctypes.c_double),
                ("default_ms", ctypes.c_double), ("n_candidates", ctypes.c_int32)]


class Observables(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("total_bias", ctypes.c_double), ("temp", ctypes.c_double),
                ("enthalpy", ctypes.c_double), ("entropy", ctypes.c_double), ("stacking", ctypes.c_double),
                ("draws", ctypes.c_int64), ("num_staples", ctypes.c_int32),
                ("num_fully_bound", ctypes.c_int32), ("num_bound", ctypes.c_int32),
                ("num_self_bound", ctypes.c_int32), ("num_stacked", ctypes.c_int32),
                ("num_unassigned", ctypes.c_int32), ("current_c_i", ctypes.c_int32),
                ("status", ctypes.c_int32)]


_lib = None


def load_library(path=None):
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("engine library %s is missing: run __graft_entry__.build() "
                           "(the engine has no CPU fallback)" % p)
    lib = ctypes.CDLL(p)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    lib.ldo_create_from_inp.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ip, ctypes.c_uint32,
                                        ctypes.POINTER(vp)]
    lib.ldo_create_multi.argtypes = [ctypes.POINTER(ctypes.c_char_p), ip, ctypes.c_char_p,
                                     ctypes.POINTER(ctypes.c_int), ip, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.ldo_destroy.argtypes = [vp]
    lib.ldo_last_error.argtypes = [vp]
    lib.ldo_last_error.restype = ctypes.c_char_p
    lib.ldo_num_replicas.argtypes = [vp]
    lib.ldo_set_controls.argtypes = [vp, dp, dp, dp, ip]
    lib.ldo_run.argtypes = [vp, ctypes.c_int64, dp]
    lib.ldo_run_sweeps.argtypes = [vp, ctypes.c_int64, dp]
    lib.ldo_state_bytes.argtypes = [vp]
    lib.ldo_us_write_biases.argtypes = [vp, ip, ctypes.c_char_p]
    lib.ldo_us_read_biases.argtypes = [vp, ctypes.c_char_p, ip, ctypes.c_char_p]
    lib.ldo_us_reset.argtypes = [vp]
    lib.ldo_read_biases.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32), dp, ip,
                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.ldo_enumerate.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                  ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, dp, dp,
                                  ctypes.POINTER(ctypes.c_int32), dp]
    lib.ldo_enumerate_units.argtypes = [vp, dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    lib.ldo_enumerate_unit_weights.argtypes = [vp, dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    lib.ldo_enumerate_full.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                       ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp,
                                       dp, ctypes.POINTER(ctypes.c_int32), dp]
    lib.ldo_autotune.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(TuneReport)]
    lib.ldo_autotune_candidates.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), dp, ctypes.c_int32]
    lib.ldo_get_observables.argtypes = [vp, ctypes.POINTER(Observables), ip]
    lib.ldo_get_config.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int32), ip, ctypes.POINTER(ctypes.c_int)]
    lib.ldo_set_config.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int32), ip]
    lib.ldo_anneal_run.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ip, dp]
    lib.ldo_set_configs.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ip]
    lib.ldo_read_trj_frame.argtypes = [ctypes.c_char_p, ip, ctypes.POINTER(ctypes.c_int32), ip,
                                       ctypes.POINTER(ctypes.c_int)]
    lib.ldo_checkpoint_save.argtypes = [vp, ctypes.c_char_p]
    lib.ldo_checkpoint_load.argtypes = [vp, ctypes.c_char_p]
    lib.ldo_set_sampling.argtypes = [vp, ip, ip]
    lib.ldo_get_samples.argtypes = [vp, ctypes.POINTER(ctypes.c_int16), ip, ctypes.POINTER(ctypes.c_int)]
    lib.ldo_set_trace.argtypes = [vp, ip, ip]
    lib.ldo_get_trace.argtypes = [vp, dp, ip, ip]
    lib.ldo_get_move_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ip]
    i64p = ctypes.POINTER(ctypes.c_int64)
    lib.ldo_get_counters.argtypes = [vp, i64p, i64p, i64p]
    lib.ldo_batch_create.argtypes = [ctypes.POINTER(ctypes.c_char_p), ip, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                     ip, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.ldo_batch_destroy.argtypes = [vp]
    lib.ldo_batch_destroy.restype = None
    lib.ldo_batch_last_error.argtypes = [vp]
    lib.ldo_batch_last_error.restype = ctypes.c_char_p
    lib.ldo_batch_num_groups.argtypes = [vp]
    lib.ldo_batch_group.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(vp)]
    lib.ldo_batch_set_controls.argtypes = [vp, dp, dp, dp, ip]
    lib.ldo_batch_run.argtypes = [vp, ctypes.c_int64, dp]
    lib.ldo_batch_run_sweeps.argtypes = [vp, ctypes.c_int64, dp]
    lib.ldo_batch_set_sampling.argtypes = [vp, ip, ip]
    lib.ldo_batch_get_samples.argtypes = [vp, ctypes.POINTER(ctypes.c_int16), ip, ctypes.POINTER(ctypes.c_int)]
    lib.ldo_batch_get_counters.argtypes = [vp, i64p, i64p, i64p]
    lib.ldo_set_grid_bias.argtypes = [vp, ctypes.c_char_p, ip, dp, ip]
    lib.ldo_set_window.argtypes = [vp, ctypes.c_char_p, ip, ip, ip]
    lib.ldo_set_bias_centre.argtypes = [vp, ctypes.c_char_p, ip, ctypes.c_double]
    lib.ldo_swap_writer_open.argtypes = [vp, ip, ip, ip, ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(vp)]
    lib.ldo_pt_run.argtypes = [vp, ip, ctypes.c_int64, ip, ip, dp]
    lib.ldo_pt2d_run.argtypes = [vp, ip, ip, ctypes.c_int64, ip, dp]
    lib.ldo_pt_get_permutation.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ip]
    lib.ldo_pt_get_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ip]
    lib.ldo_us_run.argtypes = [vp, ctypes.c_char_p, ip, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ip, dp]
    lib.ldo_us_get_biases.argtypes = [vp, dp, ip, ip]
    lib.ldo_us_get_windows.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ip, ctypes.POINTER(ctypes.c_int)]
    i32p = ctypes.POINTER(ctypes.c_int32)
    lib.ldo_replica_status_noalloc.argtypes = [vp, i32p, ip, i32p, i32p]
    lib.ldo_engine_exp.restype = ctypes.c_int
    lib.ldo_engine_exp.argtypes = [vp, vp, ctypes.c_int]
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ldo_learn_collect.argtypes = [vp]
    lib.ldo_learn_reset_counts.argtypes = [vp]
    lib.ldo_learn_get_counts.argtypes = [vp, fp, fp, ip]
    lib.ldo_learn_train.argtypes = [vp, ip, ctypes.c_double, ctypes.c_uint32, dp, dp]
    lib.ldo_learn_set_params.argtypes = [vp, fp, ip]
    lib.ldo_learn_get_params.argtypes = [vp, fp, ip]
    lib.ldo_learn_get_table.argtypes = [vp, dp, ip]
    lib.ldo_learn_set_table.argtypes = [vp, dp, ip]
    lib.ldo_learn_loss_grad.argtypes = [fp, i32p, fp, fp, ip, dp, fp]
    lib.ldo_writer_open.argtypes = [vp, ip, ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.ldo_writer_write.argtypes = [vp, ctypes.c_int64]
    lib.ldo_writer_close.argtypes = [vp]
    lib.ldo_nn_duplex_thermo.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, dp, dp]
    lib.ldo_energy_tables.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                                      dp, dp, dp, dp, dp, ip]
    lib.ldo_enumeration_plan.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32, i32p, ctypes.c_int32, i32p]
    if path is None:
        _lib = lib
    return lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


class Engine:
    """A batch of replicas of one or more origami systems on the GPU."""

    def __init__(self, inp, n_replicas, seed=0, overrides="", sys_of_replica=None):
        self.lib = load_library()
        h = ctypes.c_void_p()
        if isinstance(inp, (list, tuple)):
            arr = (ctypes.c_char_p * len(inp))(*[os.fsencode(p) for p in inp])
            so = None
            if sys_of_replica is not None:
                so = (ctypes.c_int * n_replicas)(*[int(x) for x in sys_of_replica])
            rc = self.lib.ldo_create_multi(arr, len(inp), overrides.encode(), so, n_replicas, seed,
                                           ctypes.byref(h))
        else:
            rc = self.lib.ldo_create_from_inp(os.fsencode(inp), overrides.encode(), n_replicas, seed,
                                              ctypes.byref(h))
        if rc != 0:
            raise LdoError(rc, self.lib.ldo_last_error(None).decode())
        self.h = h
        self.n = n_replicas
        self._trace = None
        self._samples = None

    @classmethod
    def _borrowed(cls, lib, handle, n_replicas):
        """An Engine over a handle owned by someone else (a Batch group)."""
        e = cls.__new__(cls)
        e.lib, e.h, e.n, e._trace, e._samples, e._owned = lib, handle, n_replicas, None, None, False
        return e

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                self.lib.ldo_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc):
        if rc != 0:
            raise LdoError(rc, self.lib.ldo_last_error(self.h).decode())

    def run(self, steps):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_run(self.h, int(steps), ctypes.byref(ms)))
        return ms.value

    def run_sweeps(self, sweeps):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_run_sweeps(self.h, int(sweeps), ctypes.byref(ms)))
        return ms.value

    def state_bytes(self):
        return self.lib.ldo_state_bytes(self.h)

    def enumerate(self, min_total, max_total, max_type, ops=("numstaples", "numfulldomains"), shape=(9, 49),
                  full=False, split_levels=0):
        """Exact enumeration on the GPU: staple-only (ldo_enumerate) or, with
        full, the scaffold enumerated too (ldo_enumerate_full, each unit split
        into 6^split_levels parallel parts): dict "k1 k2" -> normalised
        weight, and a dict of counts and timing."""
        w = np.zeros(shape[0] * shape[1])
        nconf = ctypes.c_double(0)
        nu = ctypes.c_int32(0)
        ms = ctypes.c_double(0)
        if full:
            self._check(self.lib.ldo_enumerate_full(self.h, int(min_total), int(max_total), int(max_type),
                                                    ops[0].encode(), ops[1].encode(), shape[0], shape[1],
                                                    int(split_levels), _dptr(w), ctypes.byref(nconf),
                                                    ctypes.byref(nu), ctypes.byref(ms)))
        else:
            self._check(self.lib.ldo_enumerate(self.h, int(min_total), int(max_total), int(max_type),
                                               ops[0].encode(), ops[1].encode(), shape[0], shape[1], _dptr(w),
                                               ctypes.byref(nconf), ctypes.byref(nu), ctypes.byref(ms)))
        w = w.reshape(shape)
        out = {"%d %d" % (a, b): float(w[a, b]) for a in range(shape[0]) for b in range(shape[1]) if w[a, b] != 0}
        return out, {"num_configs": nconf.value, "units": nu.value, "ms": ms.value}

    def enumerate_units(self):
        """(partition sum, configurations) of every unit of the last
        enumeration, in the reference's growth-point-set order."""
        n = ctypes.c_int32(0)
        self._check(self.lib.ldo_enumerate_units(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(2 * n.value)
        self._check(self.lib.ldo_enumerate_units(self.h, _dptr(out), n.value, ctypes.byref(n)))
        return out.reshape(-1, 2)

    def enumerate_unit_weights(self, shape=(9, 49)):
        """Unnormalised (op1, op2) weights of every unit of the last
        enumeration (shape: the histogram shape it was called with)."""
        n = ctypes.c_int32(0)
        self._check(self.lib.ldo_enumerate_unit_weights(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value * shape[0] * shape[1])
        self._check(self.lib.ldo_enumerate_unit_weights(self.h, _dptr(out), out.size, ctypes.byref(n)))
        return out.reshape(n.value, shape[0], shape[1])

    def autotune(self, probe_sweeps=4, use_cache=True):
        """The engine's autotuner (ldo_autotune): the fastest launch shape for
        this batch, kept for the following runs; returns its report and the
        candidate table (warps per block, padding, blocks per SM,
        interleaved, probe ms)."""
        rep = TuneReport()
        self._check(self.lib.ldo_autotune(self.h, int(probe_sweeps), 1 if use_cache else 0, ctypes.byref(rep)))
        out = {f[0]: getattr(rep, f[0]) for f in TuneReport._fields_}
        n = rep.n_candidates
        cands = []
        if n > 0:
            shape = (ctypes.c_int32 * (4 * n))()
            ms = (ctypes.c_double * n)()
            self._check(self.lib.ldo_autotune_candidates(self.h, shape, ms, n))
            cands = [[shape[4 * k], shape[4 * k + 1], shape[4 * k + 2], shape[4 * k + 3], ms[k]] for k in range(n)]
        out["candidates"] = cands
        return out

    def set_controls(self, temps=None, stacking_mults=None, staple_u_mults=None):
        def arr(x):
            return None if x is None else np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (self.n,)))
        t, s, u = arr(temps), arr(stacking_mults), arr(staple_u_mults)
        self._check(self.lib.ldo_set_controls(self.h, _dptr(t), _dptr(s), _dptr(u), self.n))

    def observables(self):
        out = (Observables * self.n)()
        self._check(self.lib.ldo_get_observables(self.h, out, self.n))
        return [dict((f, getattr(o, f)) for f, _ in Observables._fields_) for o in out]

    def config(self, replica):
        cap = 1 << 16
        buf = (ctypes.c_int32 * cap)()
        n = ctypes.c_int(0)
        self._check(self.lib.ldo_get_config(self.h, replica, buf, cap, ctypes.byref(n)))
        return list(buf[:n.value])

    def set_config(self, replica, flat):
        """Replaces a replica's configuration (ldo_get_config's flat format)."""
        buf = (ctypes.c_int32 * len(flat))(*flat)
        self._check(self.lib.ldo_set_config(self.h, replica, buf, len(flat)))

    def anneal(self, max_temp, min_temp, temp_interval, steps_per_temp, constant_staple_M=True):
        """AnnealingGCMCSimulation::run over every replica (ldo_anneal_run)."""
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_anneal_run(self.h, float(max_temp), float(min_temp), float(temp_interval),
                                            int(steps_per_temp), 1 if constant_staple_M else 0, ctypes.byref(ms)))
        return ms.value

    def set_configs(self, flats):
        """Replaces every replica's configuration (one flat list per replica)."""
        off = np.zeros(len(flats) + 1, np.int32)
        off[1:] = np.cumsum([len(f) for f in flats])
        buf = np.ascontiguousarray(np.concatenate([np.asarray(f, np.int32) for f in flats]), np.int32)
        i32 = ctypes.POINTER(ctypes.c_int32)
        self._check(self.lib.ldo_set_configs(self.h, buf.ctypes.data_as(i32), off.ctypes.data_as(i32), len(flats)))

    def save_checkpoint(self, path):
        self._check(self.lib.ldo_checkpoint_save(self.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        self._check(self.lib.ldo_checkpoint_load(self.h, os.fsencode(path)))

    def set_trace(self, n_trace, max_steps):
        self._check(self.lib.ldo_set_trace(self.h, n_trace, max_steps))
        self._trace = (min(n_trace, self.n), max_steps)

    def trace(self):
        nt, ms = self._trace
        out = np.zeros((nt, ms, 8))
        self._check(self.lib.ldo_get_trace(self.h, _dptr(out), nt, ms))
        return out

    def set_sampling(self, interval, capacity):
        self._check(self.lib.ldo_set_sampling(self.h, interval, capacity))
        self._samples = capacity

    def samples(self):
        cap = self._samples
        out = np.zeros((self.n, cap, 2), np.int16)
        cnt = np.zeros(self.n, np.int32)
        self._check(self.lib.ldo_get_samples(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), cap,
                                             cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out, cnt

    def counters(self):
        """(kernel launches, host-to-device bytes, device-to-host bytes) of
        this engine so far (ldo_get_counters)."""
        v = [ctypes.c_int64(0) for _ in range(3)]
        self._check(self.lib.ldo_get_counters(self.h, *[ctypes.byref(x) for x in v]))
        return tuple(int(x.value) for x in v)

    def move_stats(self, n_moves):
        out = np.zeros(2 * n_moves, np.int64)
        self._check(self.lib.ldo_get_move_stats(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n_moves))
        return out.reshape(n_moves, 2)

    def set_grid_bias(self, tag, values, replica=-1):
        v = np.ascontiguousarray(values, np.float64)
        self._check(self.lib.ldo_set_grid_bias(self.h, tag.encode(), replica, _dptr(v), len(v)))

    def set_window(self, tag, replica, min_op, max_op):
        self._check(self.lib.ldo_set_window(self.h, tag.encode(), replica, min_op, max_op))

    def set_bias_centre(self, tag, replica, centre):
        self._check(self.lib.ldo_set_bias_centre(self.h, tag.encode(), replica, float(centre)))

    def pt_run(self, n_rungs, swaps, exchange_interval, exchange_q=1):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_pt_run(self.h, n_rungs, int(swaps), exchange_interval, exchange_q,
                                        ctypes.byref(ms)))
        return ms.value

    def pt2d_run(self, n_temps, n_stacking, swaps, exchange_interval):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_pt2d_run(self.h, n_temps, n_stacking, int(swaps), exchange_interval,
                                          ctypes.byref(ms)))
        return ms.value

    def us_run(self, grid_tag, n_iters, equil_steps, iter_steps, max_D_bias, exchange_interval=0):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_us_run(self.h, grid_tag.encode(), n_iters, int(equil_steps), int(iter_steps),
                                        float(max_D_bias), exchange_interval, ctypes.byref(ms)))
        return ms.value

    def us_windows(self):
        w = np.zeros(self.n, np.int32)
        gl = ctypes.c_int(0)
        self._check(self.lib.ldo_us_get_windows(self.h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), self.n,
                                                ctypes.byref(gl)))
        return w, gl.value

    def us_biases(self):
        w, gl = self.us_windows()
        out = np.zeros((self.n, gl))
        self._check(self.lib.ldo_us_get_biases(self.h, _dptr(out), self.n, gl))
        return out

    def us_write_biases(self, window, path):
        """The window's grid biases as a .biases file (output_weights)."""
        self._check(self.lib.ldo_us_write_biases(self.h, int(window), os.fsencode(path)))

    def us_read_biases(self, grid_tag, window, path):
        """Grid biases of a window from a .biases file (read_weights)."""
        self._check(self.lib.ldo_us_read_biases(self.h, grid_tag.encode(), int(window), os.fsencode(path)))

    def us_reset(self):
        self._check(self.lib.ldo_us_reset(self.h))

    def open_swap_writer(self, n_rungs, exchange_q, ladder, filebase, freq):
        """The .swp file of one parallel-tempering ladder (ldo_swap_writer_open);
        Writer.write(step) appends the rows recorded by pt_run (step >= 0 adds
        the end-of-run row)."""
        w = ctypes.c_void_p()
        self._check(self.lib.ldo_swap_writer_open(self.h, n_rungs, exchange_q, ladder, os.fsencode(filebase),
                                                  int(freq), ctypes.byref(w)))
        return Writer(self, w)

    def open_writer(self, replica, filebase, kinds=31):
        """Output files of one replica in the reference's formats
        (1 .trj, 2 .vcf/.states/.ores, 4 .counts/.staples/.staplestates,
        8 .ene, 16 .ops, 32 .times); returns a Writer."""
        w = ctypes.c_void_p()
        self._check(self.lib.ldo_writer_open(self.h, replica, os.fsencode(filebase), kinds, ctypes.byref(w)))
        return Writer(self, w)

    # learned insertion proposal
    def learn_collect(self):
        self._check(self.lib.ldo_learn_collect(self.h))

    def learn_reset_counts(self):
        self._check(self.lib.ldo_learn_reset_counts(self.h))

    def learn_counts(self):
        b = np.zeros(LEARN_TABLE, np.float32)
        t = np.zeros(LEARN_TABLE, np.float32)
        self._check(self.lib.ldo_learn_get_counts(self.h, _fptr(b), _fptr(t), LEARN_TABLE))
        return b, t

    def learn_train(self, iters, lr=1e-3, seed=0):
        l0, l1 = ctypes.c_double(0), ctypes.c_double(0)
        self._check(self.lib.ldo_learn_train(self.h, int(iters), float(lr), seed, ctypes.byref(l0), ctypes.byref(l1)))
        return l0.value, l1.value

    def learn_params(self):
        p = np.zeros(LEARN_NPARAM, np.float32)
        self._check(self.lib.ldo_learn_get_params(self.h, _fptr(p), LEARN_NPARAM))
        return p

    def learn_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        self._check(self.lib.ldo_learn_set_params(self.h, _fptr(p), len(p)))

    def learn_table(self):
        w = np.zeros(LEARN_TABLE)
        self._check(self.lib.ldo_learn_get_table(self.h, _dptr(w), LEARN_TABLE))
        return w

    def learn_set_table(self, w):
        w = np.ascontiguousarray(w, np.float64)
        self._check(self.lib.ldo_learn_set_table(self.h, _dptr(w), len(w)))

    def pt_permutation(self):
        out = np.zeros(self.n, np.int32)
        self._check(self.lib.ldo_pt_get_permutation(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                    self.n))
        return out

    def pt_stats(self, n_pairs):
        a = np.zeros(n_pairs, np.int64)
        b = np.zeros(n_pairs, np.int64)
        self._check(self.lib.ldo_pt_get_stats(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              b.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n_pairs))
        return a, b


class Writer:
    """Appends one replica's state to its output files (ldo_writer_*)."""

    def __init__(self, eng, handle):
        self.eng = eng
        self.h = handle

    def write(self, step):
        self.eng._check(self.eng.lib.ldo_writer_write(self.h, int(step)))

    def close(self):
        if getattr(self, "h", None):
            self.eng.lib.ldo_writer_close(self.h)
            self.h = None

    __del__ = close


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def learn_loss_grad(params, idx, cnt_bound, cnt_total):
    """Loss and gradient of the proposal network on the GPU (ldo_learn_loss_grad)."""
    lib = load_library()
    p = np.ascontiguousarray(params, np.float32)
    i = np.ascontiguousarray(idx, np.int32)
    b = np.ascontiguousarray(cnt_bound, np.float32)
    t = np.ascontiguousarray(cnt_total, np.float32)
    loss = ctypes.c_double(0)
    grad = np.zeros(LEARN_NPARAM, np.float32)
    rc = lib.ldo_learn_loss_grad(_fptr(p), i.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _fptr(b), _fptr(t),
                                 len(i), ctypes.byref(loss), _fptr(grad))
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    return loss.value, grad


def read_biases(path):
    """A .biases file (USGCMCSimulation::read_weights) without an engine:
    (points int32[n, dim], biases float64[n])."""
    lib = load_library()
    n, dim = ctypes.c_int(0), ctypes.c_int(0)
    rc = lib.ldo_read_biases(os.fsencode(path), None, None, 0, ctypes.byref(n), ctypes.byref(dim))
    if rc != 0:
        raise LdoError(rc, "cannot read %s" % path)
    pts = np.zeros((n.value, max(dim.value, 1)), np.int32)
    b = np.zeros(n.value)
    rc = lib.ldo_read_biases(os.fsencode(path), pts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dptr(b),
                             n.value, ctypes.byref(n), ctypes.byref(dim))
    if rc != 0:
        raise LdoError(rc, "cannot read %s" % path)
    return pts[:, :dim.value], b


def read_trj_frame(path, frame):
    """Frame `frame` of a .trj file in ldo_get_config's flat format (host only)."""
    lib = load_library()
    cap = 1 << 20
    buf = (ctypes.c_int32 * cap)()
    n = ctypes.c_int(0)
    rc = lib.ldo_read_trj_frame(os.fsencode(path), frame, buf, cap, ctypes.byref(n))
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    return list(buf[:n.value])


def engine_exp(x):
    """The engine's exponential evaluated on the GPU (ldo_engine_exp)."""
    lib = load_library()
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    rc = lib.ldo_engine_exp(x.ctypes.data, y.ctypes.data, len(x))
    if rc != 0:
        raise LdoError(rc, "ldo_engine_exp failed")
    return y


def nn_duplex_thermo(seq, temp, cation_M):
    """Reduced (H/RT, S/R) of a fully paired duplex (host-side helper)."""
    lib = load_library()
    h, s = ctypes.c_double(), ctypes.c_double()
    rc = lib.ldo_nn_duplex_thermo(seq.encode(), temp, cation_M, ctypes.byref(h), ctypes.byref(s))
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    return h.value, s.value


def energy_tables(inp, temp, stacking_mult=1.0):
    """Dense energy tables of an .inp system at one temperature (host-side helper)."""
    lib = load_library()
    imax = ctypes.c_int()
    rc = lib.ldo_energy_tables(os.fsencode(inp), temp, stacking_mult, ctypes.byref(imax), None, None, None, None,
                               None, 0)
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    d = 2 * imax.value + 1
    arrs = [np.zeros(d * d) for _ in range(4)]
    init = np.zeros(3)
    rc = lib.ldo_energy_tables(os.fsencode(inp), temp, stacking_mult, ctypes.byref(imax), *[_dptr(a) for a in arrs],
                               _dptr(init), d * d)
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    return imax.value, [a.reshape(d, d) for a in arrs], init


def enumeration_plan(inp, min_total, max_total, max_type, overrides=""):
    """(staples, growth points) of every work unit an exact enumeration of
    the .inp system runs, in the reference's order (ldo_enumeration_plan;
    host only, no GPU)."""
    lib = load_library()
    n = ctypes.c_int32(0)
    rc = lib.ldo_enumeration_plan(os.fsencode(inp), overrides.encode(), min_total, max_total, max_type, None, 0,
                                  ctypes.byref(n))
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    out = np.zeros(2 * n.value, np.int32)
    rc = lib.ldo_enumeration_plan(os.fsencode(inp), overrides.encode(), min_total, max_total, max_type,
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), out.size, ctypes.byref(n))
    if rc != 0:
        raise LdoError(rc, lib.ldo_last_error(None).decode())
    return out.reshape(-1, 2)


class Batch:
    """Replicas of several systems split by capacity class (ldo_batch_*): one
    engine per class with its own layout and kernel, launched together.
    Replica r follows the trajectory it has in Engine(inps, n_replicas, seed,
    overrides, sys_of_replica)."""

    def __init__(self, inps, n_replicas, seed=0, overrides="", sys_of_replica=None):
        self.lib = load_library()
        h = ctypes.c_void_p()
        arr = (ctypes.c_char_p * len(inps))(*[os.fsencode(p) for p in inps])
        so = None
        if sys_of_replica is not None:
            so = (ctypes.c_int * n_replicas)(*[int(x) for x in sys_of_replica])
        rc = self.lib.ldo_batch_create(arr, len(inps), overrides.encode(), so, n_replicas, seed, ctypes.byref(h))
        if rc != 0:
            raise LdoError(rc, self.lib.ldo_batch_last_error(None).decode())
        self.h = h
        self.n = n_replicas
        self._samples = None
        self.groups = []
        for g in range(self.lib.ldo_batch_num_groups(self.h)):
            cls, n = ctypes.c_int(0), ctypes.c_int(0)
            self._check(self.lib.ldo_batch_group(self.h, g, ctypes.byref(cls), ctypes.byref(n), None, None))
            reps = np.zeros(n.value, np.int32)
            eh = ctypes.c_void_p()
            self._check(self.lib.ldo_batch_group(self.h, g, None, None,
                                                 reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(eh)))
            self.groups.append({"cls": "SML"[cls.value], "replicas": reps,
                                "engine": Engine._borrowed(self.lib, eh, n.value)})

    def close(self):
        if getattr(self, "h", None):
            for g in self.groups:
                g["engine"].h = None
            self.lib.ldo_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc):
        if rc != 0:
            raise LdoError(rc, self.lib.ldo_batch_last_error(self.h).decode())

    def set_controls(self, temps=None, stacking_mults=None, staple_u_mults=None):
        def arr(x):
            return None if x is None else np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (self.n,)))
        t, s, u = arr(temps), arr(stacking_mults), arr(staple_u_mults)
        self._check(self.lib.ldo_batch_set_controls(self.h, _dptr(t), _dptr(s), _dptr(u), self.n))

    def run(self, steps):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_batch_run(self.h, int(steps), ctypes.byref(ms)))
        return ms.value

    def run_sweeps(self, sweeps):
        ms = ctypes.c_double(0)
        self._check(self.lib.ldo_batch_run_sweeps(self.h, int(sweeps), ctypes.byref(ms)))
        return ms.value

    def set_sampling(self, interval, capacity):
        self._check(self.lib.ldo_batch_set_sampling(self.h, interval, capacity))
        self._samples = capacity
        for g in self.groups:
            g["engine"]._samples = capacity

    def samples(self):
        cap = self._samples
        out = np.zeros((self.n, cap, 2), np.int16)
        cnt = np.zeros(self.n, np.int32)
        self._check(self.lib.ldo_batch_get_samples(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), cap,
                                                   cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out, cnt

    def counters(self):
        v = [ctypes.c_int64(0) for _ in range(3)]
        self._check(self.lib.ldo_batch_get_counters(self.h, *[ctypes.byref(x) for x in v]))
        return tuple(int(x.value) for x in v)

    def autotune(self, probe_sweeps=4, use_cache=True):
        """Each group's autotuner on its own replicas: one report per group."""
        return [g["engine"].autotune(probe_sweeps, use_cache) for g in self.groups]
