"""Speed of the reference engine against the CPU restatement (test
infrastructure; runs where the reference engine is built, oracle/_ref).

The GPU host has no reference checkout and no way to build one, so the CPU
baseline timed there is the restatement (oracle/cpu_engine.cpp).  This script
measures, on one host and one core, how the two compare on whole force
evaluations (one compute of energy and derivatives: the reference's
evaluate_deriv, src/engine_c_library.cpp:48-65) of the same seeded proteins
at the same coordinates, so that the restatement's timing can be read against the
reference's.

    OMP_NUM_THREADS=1 python oracle/ref_speed.py [--systems 6] [--seconds 3]
"""
import argparse
import importlib.util
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "upside2-md_gb300"), HERE]


def rate(fn, seconds):
    fn()  # first call builds caches and pair lists
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        fn()
        n += 1
    return n / (time.perf_counter() - t0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=6)
    ap.add_argument("--seconds", type=float, default=3.0)
    a = ap.parse_args()
    import oracle_py
    import workloads
    spec = importlib.util.spec_from_file_location("mf", os.path.join(ROOT, "tests", "golden", "make_fixtures.py"))
    mf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mf)
    L = mf.load_ref()
    W = workloads.workload("C4", seed=1)
    rows = []
    for i in range(a.systems):
        path = W["configs"][i]
        x = workloads.initial_positions([path])
        n_res = x.shape[0] // 3
        ref = mf.RefEngine(L, path, x.shape[0])
        port = oracle_py.Oracle(path, x.shape[0])
        xs = np.ascontiguousarray(x, np.float32)
        d = np.zeros_like(xs)
        # one compute(PotentialAndDerivMode): energy and forces, as one
        # evaluate of the restatement
        r_ref = rate(lambda: L.evaluate_deriv(d.ctypes.data, ref.e, xs.ctypes.data), a.seconds)
        r_port = rate(lambda: port.evaluate(x), a.seconds)
        rows.append((n_res, r_ref, r_port))
        print("system %d (%d residues): reference %.1f evaluations/s, restatement %.1f, ratio %.2f"
              % (i, n_res, r_ref, r_port, r_ref / r_port), flush=True)
    ref_rate = sum(n * r for n, r, _ in rows) / len(rows)
    port_rate = sum(n * p for n, _, p in rows) / len(rows)
    print("host: %s, %s, one core" % (platform.machine(), platform.processor() or "cpu"))
    print("residue-evaluations/s: reference %.4g restatement %.4g" % (ref_rate, port_rate))
    print("ratio: %.3f" % (ref_rate / port_rate))


if __name__ == "__main__":
    main()
