"""ctypes access to the CPU oracle (test infrastructure only).

Oracle: the CPU restatement (libupside_oracle.so, float or FP64).
RefEngine: the reference engine built here (oracle/_ref/libupside_ref.so),
available only on the x86-64 build host.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_L = None


def _lib():
    global _L
    if _L is None:
        import build as oracle_build
        path = oracle_build.build_oracle()
        L = ctypes.CDLL(path)
        vp, ip, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p
        L.ocpu_create.restype = vp
        L.ocpu_create.argtypes = [cp, ip, ip]
        L.ocpu_free.argtypes = [vp]
        L.ocpu_last_error.restype = cp
        L.ocpu_evaluate.argtypes = [vp, vp, vp, vp]
        L.ocpu_output_dims.argtypes = [vp, cp, vp, vp]
        L.ocpu_get_output.argtypes = [vp, cp, vp, ip]
        L.ocpu_get_sens.argtypes = [vp, cp, vp, ip]
        L.ocpu_value_by_name.argtypes = [vp, cp, cp, vp, ip]
        L.ocpu_param_size.argtypes = [vp, cp]
        L.ocpu_get_param_deriv.argtypes = [vp, cp, vp, ip]
        L.ocpu_set_param.argtypes = [vp, cp, vp, ip]
        L.ocpu_edges.argtypes = [vp, cp, vp, ip]
        L.ocpu_run.argtypes = [vp, vp, vp, ip, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32,
                               ctypes.c_uint64]
        L.ocpu_thermostat_normals.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ip, vp]
        _L = L
    return _L


class Oracle:
    def __init__(self, path, n_atom, fp64=False):
        L = _lib()
        self.n = n_atom
        self.h = L.ocpu_create(path.encode(), n_atom, 1 if fp64 else 0)
        if not self.h:
            raise RuntimeError(L.ocpu_last_error().decode())

    def __del__(self):
        try:
            _lib().ocpu_free(self.h)
        except Exception:
            pass

    def evaluate(self, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        e = ctypes.c_double()
        d = np.zeros_like(pos)
        if _lib().ocpu_evaluate(self.h, pos.ctypes.data, ctypes.byref(e), d.ctypes.data):
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return e.value, d

    def dims(self, node):
        n, w = ctypes.c_int(), ctypes.c_int()
        if _lib().ocpu_output_dims(self.h, node.encode(), ctypes.byref(n), ctypes.byref(w)):
            raise KeyError(node)
        return n.value, w.value

    def node(self, node, sens=False):
        n, w = self.dims(node)
        o = np.zeros((n, w), np.float32)
        fn = _lib().ocpu_get_sens if sens else _lib().ocpu_get_output
        if fn(self.h, node.encode(), o.ctypes.data, o.size):
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return o

    def value(self, node, what, n):
        o = np.zeros(n, np.float32)
        if _lib().ocpu_value_by_name(self.h, node.encode(), what.encode(), o.ctypes.data, n):
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return o

    def edges(self, node, cap=1 << 22):
        buf = np.zeros((cap, 2), np.int32)
        n = _lib().ocpu_edges(self.h, node.encode(), buf.ctypes.data, cap)
        if n < 0:
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return buf[:n].copy()

    def param_deriv(self, node):
        n = _lib().ocpu_param_size(self.h, node.encode())
        o = np.zeros(n, np.float32)
        if _lib().ocpu_get_param_deriv(self.h, node.encode(), o.ctypes.data, n):
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return o

    def set_param(self, node, p):
        p = np.ascontiguousarray(p, np.float32)
        if _lib().ocpu_set_param(self.h, node.encode(), p.ctypes.data, p.size):
            raise RuntimeError(_lib().ocpu_last_error().decode())

    def run(self, pos, mom, n_round, dt=0.009, temperature=0.85, timescale=5.0, seed=1, round_start=0):
        pos = np.ascontiguousarray(pos, np.float32).copy()
        mom = np.ascontiguousarray(mom, np.float32).copy()
        if _lib().ocpu_run(self.h, pos.ctypes.data, mom.ctypes.data, n_round, dt, temperature, timescale, seed,
                           round_start):
            raise RuntimeError(_lib().ocpu_last_error().decode())
        return pos, mom


def thermostat_normals(seed, invocation, n_atom):
    out = np.zeros((n_atom, 3), np.float32)
    _lib().ocpu_thermostat_normals(seed, invocation, n_atom, out.ctypes.data)
    return out
