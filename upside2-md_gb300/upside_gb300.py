"""Python host side of the GB300 Upside engine.

`Upside` mirrors the reference's ctypes wrapper (py/upside_engine.py:186-276:
energy / deriv / set_param / get_param / get_param_deriv / get_output /
get_sens / get_value_by_name) over the drop-in C ABI of libupside.so.
`Batch` drives many systems at once through the batch API (upside_gb300.h).
`upside_main` runs the upside command line (trajectories logged to /output).

The CUDA library is required: importing this module on a host without the
built libupside.so raises immediately; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libupside.so")
_lib = None

c_float_p = ctypes.POINTER(ctypes.c_float)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libupside.so is not built (run __graft_entry__.build()); "
                               "the engine has no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p
        L.construct_deriv_engine.restype = vp
        L.construct_deriv_engine.argtypes = [ip, cp, ctypes.c_bool]
        L.free_deriv_engine.argtypes = [vp]
        for nm in ["evaluate_energy", "evaluate_deriv"]:
            getattr(L, nm).argtypes = [vp, vp, vp]
        for nm in ["set_param", "get_param", "get_param_deriv", "get_output", "get_sens"]:
            getattr(L, nm).argtypes = [ip, vp, vp, cp]
        L.get_output_dims.argtypes = [vp, vp, vp, cp]
        L.get_value_by_name.argtypes = [ip, vp, vp, cp, cp]
        L.ug_last_error.restype = cp
        L.ug_create.restype = vp
        L.ug_create.argtypes = [ip, ctypes.POINTER(cp), vp]
        L.ug_free.argtypes = [vp]
        L.ug_atom_total.argtypes = [vp]
        for nm in ["ug_set_pos", "ug_get_pos", "ug_set_mom", "ug_get_mom"]:
            getattr(L, nm).argtypes = [vp, vp]
        L.ug_evaluate.argtypes = [vp, vp, vp]
        L.ug_set_thermostat.argtypes = [vp, vp, vp]
        L.ug_set_round.argtypes = [vp, vp]
        L.ug_set_integrator.argtypes = [vp, ip, ip]
        L.ug_level_forces.argtypes = [vp, ip, vp]
        L.ug_monte_carlo.argtypes = [vp, ctypes.c_uint64, vp]
        L.ug_run.argtypes = [vp, ip, ctypes.c_float, ctypes.c_float, ip, ip]
        L.ug_node_dims.argtypes = [vp, cp, vp, vp]
        L.ug_node_output.argtypes = [vp, cp, vp, ip]
        L.ug_node_sens.argtypes = [vp, cp, vp, ip]
        L.ug_node_edges.argtypes = [vp, cp, vp, ip]
        L.ug_value_by_name.argtypes = [vp, cp, cp, vp, ip]
        L.ug_node_potential.argtypes = [vp, cp, vp]
        L.ug_replica_exchange.argtypes = [vp, ip, vp, ctypes.c_uint32, ctypes.c_uint64, vp]
        L.ug_set_replica_exchange.argtypes = [vp, ip, vp, vp, ctypes.c_uint32, ip, ip]
        L.ug_replica_state.argtypes = [vp, vp, vp, vp, ip, vp, vp, vp]
        L.ug_timed_rounds.argtypes = [vp]
        L.ug_exchange_now.argtypes = [vp]
        L.ug_set_box.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.ug_status.argtypes = [vp, ip]
        L.ug_info.argtypes = [vp, vp, vp]
        L.ug_profile.argtypes = [vp, ip, ctypes.c_char_p, ip, vp, ip]
        L.ug_bench.argtypes = [vp, ip, ctypes.c_float, ctypes.c_float, ip, ip, vp]
        L.ug_set_device.argtypes = [ip]
        L.ug_bench_kernel.argtypes = [vp, vp]
        L.ug_autotune.argtypes = [vp, ip, ctypes.c_float, ctypes.c_float, ctypes.c_char_p, ip]
        L.ug_set_tuning.argtypes = [vp, ctypes.c_float, ip, ip]
        for nm in ["ug_set_param", "ug_get_param", "ug_param_deriv"]:
            getattr(L, nm).argtypes = [vp, cp, vp, ip]
        i64, f = ctypes.c_int64, ctypes.c_float
        L.ug_set_warm_start.argtypes = [vp, vp, vp, vp, vp, vp, vp, ip]
        L.ug_mlp_gemm.argtypes = [vp, i64, i64, vp, i64, i64, vp, ip, ip, ip, ip, ip, vp]
        L.ug_mlp_bias_act.argtypes = [vp, vp, vp, vp, ip, ip, ip, vp]
        L.ug_mlp_to_bf16.argtypes = [vp, vp, vp, i64, vp]
        L.ug_mlp_softmax_xent.argtypes = [vp, vp, vp, vp, vp, ip, f, vp]
        L.ug_mlp_colsum.argtypes = [vp, vp, ip, ip, vp]
        L.ug_mlp_adam.argtypes = [vp, vp, vp, vp, vp, ip, f, f, f, f, ip, vp]
        L.ug_pair_list.argtypes = [vp, ip, ctypes.c_float, vp, ip, vp, vp]
        L.ug_pair_list_noalloc.argtypes = [vp, ip, ctypes.c_float, vp, ip, vp, vp]
        L.upside_main.restype = ip
        L.upside_main.argtypes = [ip, ctypes.POINTER(ctypes.c_char_p), ip]
        _lib = L
    return _lib


def pair_list(pos_ptr, n, cutoff, pairs_ptr, cap, n_pairs_ptr, stream=0):
    """ug_pair_list on device pointers (ints): pairs (i, j), i < j, closer than cutoff."""
    if lib().ug_pair_list(pos_ptr, n, cutoff, pairs_ptr, cap, n_pairs_ptr, stream):
        raise RuntimeError(lib().ug_last_error().decode())


def pair_list_noalloc(pos_ptr, n, cutoff, pairs_ptr, cap, n_pairs_ptr, stream=0):
    """ug_pair_list_noalloc: as pair_list, scratch in a fixed device array
    (n <= 262144), asynchronous on `stream`."""
    if lib().ug_pair_list_noalloc(pos_ptr, n, cutoff, pairs_ptr, cap, n_pairs_ptr, stream):
        raise RuntimeError(lib().ug_last_error().decode())


def upside_main(args, verbose=True):
    """Run the upside command line in this process on the GPU (the
    reference's in_process_upside, py/upside_engine.py:94-118): `args` are
    the arguments after the program name.  Raises RuntimeError on a non-zero
    return code."""
    argv = ["python_library", "--re-raise-signal"] + [str(a) for a in args]
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    rc = lib().upside_main(len(argv), arr, int(bool(verbose)))
    if rc:
        raise RuntimeError("In process Upside returned %i" % rc)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Upside:
    """Single-system engine over the drop-in ABI (same methods as the reference wrapper)."""

    def __init__(self, config, n_atom=None):
        from h5lite import H5File
        if n_atom is None:
            with H5File(config) as f:
                n_atom = f.read("/input/pos").shape[0]
        self.config = config
        self.n_atom = int(n_atom)
        self.engine = lib().construct_deriv_engine(self.n_atom, config.encode(), True)
        if not self.engine:
            raise RuntimeError("Unable to initialize the engine from " + config)

    def __del__(self):
        try:
            if self.engine:
                lib().free_deriv_engine(self.engine)
        except Exception:
            pass

    def _pos(self, pos):
        pos = _f32(pos)
        assert pos.shape == (self.n_atom, 3)
        return pos

    def energy(self, pos):
        pos = self._pos(pos)
        e = np.zeros(1, np.float32)
        if lib().evaluate_energy(e.ctypes.data, self.engine, pos.ctypes.data):
            raise RuntimeError("evaluate_energy failed")
        return float(e[0])

    def deriv(self, pos):
        pos = self._pos(pos)
        d = np.zeros_like(pos)
        if lib().evaluate_deriv(d.ctypes.data, self.engine, pos.ctypes.data):
            raise RuntimeError("evaluate_deriv failed")
        return d

    def set_param(self, param, node_name):
        param = _f32(param)
        if lib().set_param(param.size, param.ctypes.data, self.engine, node_name.encode()):
            raise RuntimeError("set_param failed")

    def get_param(self, shape, node_name):
        p = np.zeros(shape, np.float32)
        if lib().get_param(p.size, p.ctypes.data, self.engine, node_name.encode()):
            raise RuntimeError("get_param failed")
        return p

    def get_param_deriv(self, shape, node_name):
        p = np.zeros(shape, np.float32)
        if lib().get_param_deriv(p.size, p.ctypes.data, self.engine, node_name.encode()):
            raise RuntimeError("get_param_deriv failed")
        return p

    def get_output_dims(self, node_name):
        n, w = ctypes.c_int(), ctypes.c_int()
        if lib().get_output_dims(ctypes.byref(n), ctypes.byref(w), self.engine, node_name.encode()):
            raise RuntimeError("get_output_dims failed")
        return n.value, w.value

    def get_output(self, node_name):
        n, w = self.get_output_dims(node_name)
        o = np.zeros((n, w), np.float32)
        if lib().get_output(o.size, o.ctypes.data, self.engine, node_name.encode()):
            raise RuntimeError("get_output failed")
        return o

    def get_sens(self, node_name):
        n, w = self.get_output_dims(node_name)
        o = np.zeros((n, w), np.float32)
        if lib().get_sens(o.size, o.ctypes.data, self.engine, node_name.encode()):
            raise RuntimeError("get_sens failed")
        return o

    def get_value_by_name(self, shape, node_name, log_name):
        o = np.zeros(shape, np.float32)
        if lib().get_value_by_name(o.size, o.ctypes.data, self.engine, node_name.encode(), log_name.encode()):
            raise RuntimeError("get_value_by_name failed")
        return o


class Batch:
    """Many systems (identical node graphs) advanced by one set of kernels."""

    def __init__(self, configs, n_atoms=None):
        from h5lite import H5File
        if n_atoms is None:
            n_atoms = []
            for c in configs:
                with H5File(c) as f:
                    n_atoms.append(f.read("/input/pos").shape[0])
        self.configs = list(configs)
        self.n_atoms = np.asarray(n_atoms, dtype=np.int32)
        self.n_sys = len(self.configs)
        arr = (ctypes.c_char_p * self.n_sys)(*[c.encode() for c in self.configs])
        self.h = lib().ug_create(self.n_sys, arr, self.n_atoms.ctypes.data)
        if not self.h:
            raise RuntimeError(lib().ug_last_error().decode())
        self.atom_total = int(self.n_atoms.sum())
        self.atom_off = np.concatenate([[0], np.cumsum(self.n_atoms)])

    def __del__(self):
        try:
            if self.h:
                lib().ug_free(self.h)
        except Exception:
            pass

    def _chk(self, r):
        if r:
            raise RuntimeError(lib().ug_last_error().decode())

    def set_pos(self, pos):
        pos = _f32(pos).reshape(self.atom_total, 3)
        self._chk(lib().ug_set_pos(self.h, pos.ctypes.data))

    def get_pos(self):
        p = np.zeros((self.atom_total, 3), np.float32)
        self._chk(lib().ug_get_pos(self.h, p.ctypes.data))
        return p

    def set_mom(self, mom):
        mom = _f32(mom).reshape(self.atom_total, 3)
        self._chk(lib().ug_set_mom(self.h, mom.ctypes.data))

    def get_mom(self):
        p = np.zeros((self.atom_total, 3), np.float32)
        self._chk(lib().ug_get_mom(self.h, p.ctypes.data))
        return p

    def evaluate(self, want_deriv=True):
        e = np.zeros(self.n_sys, np.float64)
        d = np.zeros((self.atom_total, 3), np.float32) if want_deriv else None
        self._chk(lib().ug_evaluate(self.h, e.ctypes.data, d.ctypes.data if want_deriv else None))
        return e, d

    def set_thermostat(self, temperature, seed):
        t = _f32(temperature)
        s = np.ascontiguousarray(seed, dtype=np.uint32)
        self._chk(lib().ug_set_thermostat(self.h, t.ctypes.data, s.ctypes.data))

    def set_round(self, rounds):
        r = np.ascontiguousarray(rounds, dtype=np.uint64)
        self._chk(lib().ug_set_round(self.h, r.ctypes.data))

    def set_integrator(self, multistep=False, inner_step=3):
        """The three-stage cycle, or the multistep integrator: per round a
        slow-force kick of inner_step dt, then inner_step fast stages."""
        self._chk(lib().ug_set_integrator(self.h, int(bool(multistep)), int(inner_step)))

    def monte_carlo(self, round):
        """One pivot and one jump move per system (where the config has them);
        returns (n_sys, 2) accepted flags: 1, 0, or -1 without that sampler."""
        acc = np.zeros((self.n_sys, 2), np.int32)
        self._chk(lib().ug_monte_carlo(self.h, int(round), acc.ctypes.data))
        return acc

    def level_forces(self, level):
        """dE/dx of the integrator level's nodes (0 fast, 1 slow)."""
        d = np.zeros((self.atom_total, 3), np.float32)
        self._chk(lib().ug_level_forces(self.h, int(level), d.ctypes.data))
        return d

    def run(self, n_round, dt=0.009, timescale=5.0, use_graph=True, graph_rounds=1):
        self._chk(lib().ug_run(self.h, int(n_round), float(dt), float(timescale), int(use_graph), int(graph_rounds)))

    def node_dims(self, name):
        n, w = ctypes.c_int(), ctypes.c_int()
        self._chk(lib().ug_node_dims(self.h, name.encode(), ctypes.byref(n), ctypes.byref(w)))
        return n.value, w.value

    def node_output(self, name, sens=False):
        n, w = self.node_dims(name)
        o = np.zeros((n, w), np.float32)
        fn = lib().ug_node_sens if sens else lib().ug_node_output
        self._chk(fn(self.h, name.encode(), o.ctypes.data, o.size))
        return o

    def node_potential(self, name):
        o = np.zeros(self.n_sys, np.float64)
        self._chk(lib().ug_node_potential(self.h, name.encode(), o.ctypes.data))
        return o

    def set_param(self, name, param):
        p = _f32(param).ravel()
        self._chk(lib().ug_set_param(self.h, name.encode(), p.ctypes.data, p.size))

    def get_param(self, name, shape):
        p = np.zeros(shape, np.float32)
        self._chk(lib().ug_get_param(self.h, name.encode(), p.ctypes.data, p.size))
        return p

    def param_deriv(self, name, shape):
        """dE/d(param) of the last evaluate(), summed over the batch's systems."""
        p = np.zeros(shape, np.float32)
        self._chk(lib().ug_param_deriv(self.h, name.encode(), p.ctypes.data, p.size))
        return p

    def node_edges(self, name, cap=1 << 22):
        buf = np.zeros((cap, 2), np.int32)
        n = lib().ug_node_edges(self.h, name.encode(), buf.ctypes.data, cap)
        if n < 0:
            raise RuntimeError(lib().ug_last_error().decode())
        return buf[:min(n, cap)].copy()

    def value_by_name(self, name, what, n):
        o = np.zeros(n, np.float32)
        self._chk(lib().ug_value_by_name(self.h, name.encode(), what.encode(), o.ctypes.data, n))
        return o

    def set_warm_start(self, weights=None, enable=1):
        """Load learned BP warm-start weights (dict W1, b1, W2, b2, W3, b3) and/or
        select the BP start: 0 uniform, 1 learned, 2 previous marginals,
        3 previous messages and marginals."""
        if weights is None:
            ptrs = [None] * 6
            keep = []
        else:
            keep = [_f32(weights[k]) for k in ("W1", "b1", "W2", "b2", "W3", "b3")]
            ptrs = [a.ctypes.data for a in keep]
        self._chk(lib().ug_set_warm_start(self.h, *ptrs, int(enable)))

    def replica_exchange(self, pairs, seed, round_):
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        acc = np.zeros(len(pairs), np.int32)
        self._chk(lib().ug_replica_exchange(self.h, len(pairs), pairs.ctypes.data, int(seed), int(round_),
                                            acc.ctypes.data))
        return acc

    def set_replica_exchange(self, sets, seed, interval, criterion=0):
        """Periodic replica exchange on the device: after every interval-th
        round, one exchange with the next swap set in turn (sets: lists of
        (s1, s2) pairs).  sets=[] removes the plan."""
        sizes = np.array([len(s) for s in sets], np.int32)
        pairs = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int32).reshape(-1, 2) for s in sets])
                                     if sets else np.zeros((0, 2), np.int32), dtype=np.int32)
        self._chk(lib().ug_set_replica_exchange(self.h, len(sets), sizes.ctypes.data, pairs.ctypes.data,
                                                int(seed), int(interval), int(criterion)))
        self._remd_pairs = sum(len(s) for s in sets)
        self._remd_max = max([len(s) for s in sets] or [0])

    def replica_state(self):
        """(replica index per system, attempts per pair, successes per pair,
        exchanges made, last exchange's accept flags, last set)."""
        n = max(1, self._remd_pairs)
        rep = np.zeros(self.n_sys, np.int32)
        na = np.zeros(n, np.uint32)
        ns = np.zeros(n, np.uint32)
        acc = np.zeros(max(1, self._remd_max), np.int32)
        ne = ctypes.c_ulonglong()
        last = ctypes.c_int()
        self._chk(lib().ug_replica_state(self.h, rep.ctypes.data, na.ctypes.data, ns.ctypes.data, n,
                                         ctypes.byref(ne), acc.ctypes.data, ctypes.byref(last)))
        return rep, na[:self._remd_pairs], ns[:self._remd_pairs], ne.value, acc, last.value

    def set_box(self, lx, ly, lz):
        """periodic box edge lengths (0: open direction); minimum image in
        the pair terms"""
        self._chk(lib().ug_set_box(self.h, float(lx), float(ly), float(lz)))

    def exchange_now(self):
        """one exchange of the periodic plan now (next set, its round key)"""
        self._chk(lib().ug_exchange_now(self.h))

    def timed_rounds(self):
        return lib().ug_timed_rounds(self.h)

    def status(self, clear=True):
        return lib().ug_status(self.h, int(clear))

    def info(self):
        l, b = ctypes.c_int(), ctypes.c_int64()
        self._chk(lib().ug_info(self.h, ctypes.byref(l), ctypes.byref(b)))
        return l.value, b.value

    def bench(self, n_round, dt=0.009, timescale=5.0, flush_l2=True, e2e=False):
        """Device time (ms) of each of n_round timed integration rounds."""
        ms = np.zeros(n_round, np.float32)
        self._chk(lib().ug_bench(self.h, int(n_round), float(dt), float(timescale), int(flush_l2), int(e2e),
                                 ms.ctypes.data))
        return ms

    def autotune(self, n_round=5, dt=0.009, timescale=5.0):
        """Tune cache buffer and BP launch variant from the current state;
        returns ({setting: ms per round}, chosen setting)."""
        buf = ctypes.create_string_buffer(1 << 14)
        n = lib().ug_autotune(self.h, int(n_round), float(dt), float(timescale), buf, 1 << 14)
        if n < 0:
            raise RuntimeError(lib().ug_last_error().decode())
        trials, chosen = {}, None
        for line in buf.value.decode().splitlines():
            k, v = line.split("\t")
            if k == "chosen":
                chosen = v
            else:
                trials[k] = float(v)
        return trials, chosen

    def set_tuning(self, cache_buffer_scale=1.0, bp_variant=0, node_streams=4):
        self._chk(lib().ug_set_tuning(self.h, float(cache_buffer_scale), int(bp_variant), int(node_streams)))

    def bench_kernel(self):
        """The BP solve kernel over the last bench(): summed device ms, launches,
        summed algorithmic bytes."""
        s = np.zeros(3, np.float64)
        self._chk(lib().ug_bench_kernel(self.h, s.ctypes.data))
        return {"ms": float(s[0]), "launches": int(s[1]), "bytes": float(s[2])}

    def profile(self, n_eval=5):
        names = ctypes.create_string_buffer(1 << 16)
        ms = np.zeros(256, np.float32)
        n = lib().ug_profile(self.h, n_eval, names, 1 << 16, ms.ctypes.data, 256)
        if n < 0:
            raise RuntimeError(lib().ug_last_error().decode())
        return list(zip(names.value.decode().split("\n")[:n], ms[:n].tolist()))
