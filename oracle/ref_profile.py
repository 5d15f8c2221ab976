"""Where the reference engine's CPU time goes, by its own per-node timers
(test infrastructure; runs where the reference engine is built, oracle/_ref).

The reference engine is compiled once more with COLLECT_PROFILE
(`make -C oracle/ref_build prof`), which runs every node's compute and
derivative pass under a Timer (src/timing.h:33-57); after the timed
evaluations, its own report (TimeKeeper::print_report, src/timing.cpp:11-55)
prints each timer's share, here in microseconds per force evaluation summed
over the systems.  The systems are the first ones of the bench's C4 batch,
each relaxed first by the FP32 restatement's dynamics (the random initial
coils are not what dynamics evaluates), then evaluated by the reference for a
few seconds on one core.

    OMP_NUM_THREADS=1 python oracle/ref_profile.py [--systems 6] [--seconds 3] [--relax 100]
"""
import argparse
import ctypes
import os
import platform
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "upside2-md_gb300"), HERE]


def build_prof():
    import build as oracle_build
    if oracle_build.build_reference() is None:
        raise SystemExit("the reference engine is not built on this host (needs the reference checkout, x86-64)")
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref_build"), "prof", "REF=" + oracle_build.REF],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode:
        raise SystemExit("profiling build failed:\n" + r.stdout[-4000:])
    return os.path.join(HERE, "_ref", "prof", "libupside_ref_prof.so")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=6)
    ap.add_argument("--seconds", type=float, default=3.0)
    ap.add_argument("--relax", type=int, default=100, help="integration rounds of the restatement before timing")
    a = ap.parse_args()
    import oracle_py
    import workloads
    L = ctypes.CDLL(build_prof())
    L.construct_deriv_engine.restype = ctypes.c_void_p
    L.construct_deriv_engine.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_bool]
    L.evaluate_deriv.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.ref_time_report.argtypes = [ctypes.c_int]
    W = workloads.workload("C4", seed=1)
    n_eval, res_evals, t_all = 0, 0, 0.0
    sizes = []
    for i in range(a.systems):
        path = W["configs"][i]
        x0 = workloads.initial_positions([path])
        o = oracle_py.Oracle(path, x0.shape[0])
        x, _ = o.run(x0, np.zeros_like(x0), a.relax, dt=0.009, temperature=float(W["temps"][i]), timescale=5.0,
                     seed=1 + i)
        xs = np.ascontiguousarray(x, np.float32)
        d = np.zeros_like(xs)
        e = L.construct_deriv_engine(xs.shape[0], path.encode(), True)
        assert e
        assert L.evaluate_deriv(d.ctypes.data, e, xs.ctypes.data) == 0  # caches and pair lists
        k, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < a.seconds:
            assert L.evaluate_deriv(d.ctypes.data, e, xs.ctypes.data) == 0
            k += 1
        t_all += time.perf_counter() - t0
        n_eval += k
        res_evals += k * (xs.shape[0] // 3)
        sizes.append(xs.shape[0] // 3)
    print("host: %s, one core; systems of %s residues, relaxed by %d rounds; %d evaluations, %.4g residue-evaluations/s"
          % (platform.machine(), ",".join(map(str, sizes)), a.relax, n_eval, res_evals / t_all), flush=True)
    print("per-node timers (microseconds per evaluation, share):", flush=True)
    sys.stdout.flush()
    L.ref_time_report(n_eval)


if __name__ == "__main__":
    main()
