"""Benchmark: residue-steps/s of the batched GB300 Upside engine.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload C4] [--impl gpu|reference]

A step is the reference's unit: the time per step it reports divides by the
number of integration rounds (src/main.cpp:1009-1012), one round being the
thermostat and one integration_cycle, 3 x {force, p -= dt F, x += dt p}
(src/deriv_engine.cpp:317-331).  A timed iteration is one round of the whole
batch (with replica exchange: one exchange interval of rounds and its
exchange).  residue-steps/s = sum over systems of residues x rounds / time.
The default workload is C4 (64 chains, lengths uniform in [40,400]).

Multi-GPU: one process per GPU (torchrun); each rank advances its own batch of
independently seeded systems ("replicas only", weak scaling); ranks only meet
for a barrier and the max-over-ranks timing reduction.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "upside2-md_gb300"))

METRIC = "residue-steps/s on 1 GB300: batched+learned-BP vs plain GPU at same force error"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="C4")
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain single-system GPU comparison")
    ap.add_argument("--bp-start", default="learned", choices=["uniform", "learned", "previous", "reuse"],
                    help="BP initial state of the batched run")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="", help="SCALE,VARIANT: set the tuned quantities instead of tuning")
    ap.add_argument("--equilibrate", type=int, default=300,
                    help="untimed integration rounds from the initial coils before the warm-up")
    ap.add_argument("--profile", action="store_true", help="print per-node device times to stderr")
    ap.add_argument("--pbc", action="store_true",
                    help="periodic box (the workload's box, 200 A for C5; a mode of this engine only)")
    return ap.parse_args()


class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------ CPU oracle ---
def _cpu_worker(args):
    path, n_atom, seconds, seed, pos, mom = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "upside2-md_gb300"))
    import numpy as np
    import oracle_py
    from h5lite import H5File
    if pos is None:
        with H5File(path) as f:
            pos = f.read("/input/pos")[:, :, 0].astype(np.float32)
        mom = np.zeros_like(pos)
    o = oracle_py.Oracle(path, n_atom)
    t0 = time.perf_counter()
    rounds = 0
    while time.perf_counter() - t0 < seconds:
        pos, mom = o.run(pos, mom, 1, seed=seed, round_start=rounds)
        rounds += 1
    return rounds, time.perf_counter() - t0, n_atom // 3


def cpu_port_rate(configs, seconds, max_procs=None, states=None):
    """Oracle port (the CPU restatement) timed on the host cores: one process
    per system (the reference parallelises across systems only), each running
    whole integration rounds for `seconds` from the given (positions, momenta)
    of each system, or from the config's coordinates at rest.  Returns
    (residue-steps/s, cores, sample)."""
    import multiprocessing as mp
    from workloads import n_res_of
    procs = min(len(configs), max_procs or os.cpu_count() or 1)
    jobs = [(configs[i], 3 * n_res_of(configs[i]), seconds, 1 + i) + (states[i] if states else (None, None))
            for i in range(procs)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_worker, jobs)
    rate = sum(r * n / t for r, t, n in res)
    sample = "%d systems (%s residues), %.0f s of whole integration rounds each, %d rounds total" % (
        procs, ",".join(str(n) for _, _, n in res[:8]) + ("..." if procs > 8 else ""), seconds,
        sum(r for r, _, _ in res))
    return rate, procs, sample


# ----------------------------------------------------------------- main ---
def main():
    a = parse()
    d = Dist()
    if a.gpus != d.world and d.world > 1:
        print("warning: --gpus %d but WORLD_SIZE %d" % (a.gpus, d.world), file=sys.stderr)
    import numpy as np
    import workloads

    W = workloads.workload(a.workload, seed=1 + d.rank)
    n_res_total = sum(W["n_res"])

    if a.impl == "reference":
        if d.rank != 0:
            return
        rate, cores, sample = cpu_port_rate(W["configs"], a.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "residue-steps/s",
                "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
                "ms_per_step": 1e3 * n_res_total / rate, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ff_2.1 proteins)",
                "config": {"workload": a.workload, "systems": len(W["configs"]), "residues": n_res_total},
                "cpu_baseline": dict({"value": rate, "unit": "residue-steps/s", "cores": cores, "kind": "port",
                                      "sample": sample}, **cpu_fields(rate)),
                "e2e": {"value": rate, "unit": "residue-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import upside_gb300 as U
    U.lib().ug_set_device(d.local)
    b = U.Batch(W["configs"])
    b.set_pos(workloads.initial_positions(W["configs"]))
    b.set_thermostat(W["temps"], np.array(W["seeds"], np.uint32))
    if a.pbc:
        if not W.get("box"):
            raise SystemExit("--pbc: workload %s has no box" % a.workload)
        b.set_box(*W["box"])
    if W["swap_sets"]:  # replica exchange every 20 rounds, alternating sets, on the device
        b.set_replica_exchange(W["swap_sets"], 1 + d.rank, W["exchange_interval"], 0)
    bp_start = set_bp_start(b, a.bp_start)
    # equilibrate: the random initial coils relax for a few hundred rounds
    # before the dynamics reach their steady state (untimed)
    if a.equilibrate:
        b.run(a.equilibrate, use_graph=True, graph_rounds=10)
    tuned = None
    if a.tuning:  # fixed setting (profiling runs)
        parts = a.tuning.split(",")
        streams = int(parts[2]) if len(parts) > 2 else 4
        b.set_tuning(float(parts[0]), int(parts[1]), streams)
        tuned = {"chosen": "cache_buffer_scale=%s,bp_variant=%s,node_streams=%d (given)" % (parts[0], parts[1], streams)}
    elif not a.no_autotune:  # untimed; the state is restored after the trials
        trials, chosen = b.autotune(8)
        tuned = {"chosen": chosen, "trial_ms_per_round": trials}
    pos_eq, mom_eq = b.get_pos(), b.get_mom()
    states = [(pos_eq[b.atom_off[i]:b.atom_off[i + 1]].copy(), mom_eq[b.atom_off[i]:b.atom_off[i + 1]].copy())
              for i in range(b.n_sys)]
    b.run(a.warmup, use_graph=True, graph_rounds=1)
    launches, dev_bytes = b.info()
    if a.profile:
        for nm, ms in sorted(b.profile(5), key=lambda x: -x[1])[:25]:
            print("%-48s %8.3f ms" % (nm, ms), file=sys.stderr)
    rounds_per_iter = b.timed_rounds()
    # one untimed pass of the timing loop itself (graph with its event nodes,
    # L2 flush buffer, event reads), so that the timed rounds start warm
    b.bench(max(3, a.warmup), flush_l2=True)
    d.barrier()
    with Clocks(d.local) as clk:
        ms = b.bench(a.steps, flush_l2=True)
    d.barrier()
    peak, peak_kind = measured_peaks()
    roof = roofline(b, W, a, peak, peak_kind)
    t_dev = d.max(float(ms.sum()) / 1e3)
    units = d.sum(n_res_total * rounds_per_iter * a.steps)
    value = units / t_dev
    # end to end: the same rounds with the state round-tripped through pinned host memory
    ms_e2e = b.bench(a.steps, flush_l2=True, e2e=True)
    t_e2e = d.max(float(ms_e2e.sum()) / 1e3)
    e2e_value = units / t_e2e
    st = b.status()
    plain = plain_single_rate(W, a, states) if not a.no_plain else None
    cpu = None
    if d.rank == 0 and d.world == 1 and not a.no_cpu_baseline:
        rate, cores, sample = cpu_port_rate(W["configs"], a.cpu_seconds, states=states)
        sample += ", from the same equilibrated state as the GPU run"
        cpu = dict({"value": rate, "unit": "residue-steps/s", "cores": cores, "kind": "port", "sample": sample},
                   **cpu_fields(rate))
    if d.rank != 0:
        return
    state_bytes = 2 * 12 * b.atom_total
    line = {
        "metric": METRIC, "value": value, "unit": "residue-steps/s", "n_gpus": d.world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * t_dev / (a.steps * rounds_per_iter), "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ff_2.1 proteins, random initial chains)",
        "config": {"workload": a.workload, "systems": len(W["configs"]), "residues": n_res_total,
                   "step": "one integration round per system (thermostat + integration_cycle: 3 force "
                           "evaluations and integrator stages), the reference's step (src/main.cpp:1009-1012)",
                   "force_evaluations_per_step": 3,
                   "rounds_per_timed_iteration": rounds_per_iter,
                   "periodic_box": W.get("box") if a.pbc else None,
                   "replica_exchange": (None if not W["swap_sets"] else
                                        "every %d rounds on the device, alternating even/odd sets, criterion 0"
                                        % W["exchange_interval"]),
                   "equilibration_rounds": a.equilibrate, "autotune": tuned,
                   "l2": "256 MiB buffer rewritten before every timed round", "bp_init": warm_outcome(b, bp_start),
                   "bp_sweeps_per_solve": bp_sweeps(b)},
        "e2e": {"value": e2e_value, "unit": "residue-steps/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes},
        "gpu_launches": int(a.steps * (rounds_per_iter * (3 * launches + 5) +
                                       (2 * launches + 4 if W["swap_sets"] else 0))),
        "clocks": clk.summary(),
        "roofline": roof,
        "cpu_baseline": cpu,
        "plain_single_replica": plain,
        "status_bits": st,
        "device_bytes": dev_bytes,
    }
    print(json.dumps(line))


def set_bp_start(b, mode):
    """BP initial state of the batched run: the learned warm start (with its
    per-system fallback to the uniform start), the previous solve's marginals,
    or the reference's uniform start."""
    if mode == "uniform":
        return "uniform messages (reference)"
    if mode == "previous":
        b.set_warm_start(None, 2)
        return "previous solve's marginals"
    if mode == "reuse":
        b.set_warm_start(None, 3)
        return "previous solve's messages and marginals"
    import warm_start
    if not os.path.exists(warm_start.WEIGHTS):
        return "uniform messages (no trained warm-start weights)"
    b.set_warm_start(warm_start.load(), 1)
    return "learned warm start (bf16 MLP), per-system fallback to uniform"


def warm_outcome(b, bp_start):
    """The learned start's per-system fallback at the end of the run: on how
    many systems the next solve starts from the network's prediction, and the
    measured mean sweeps of the two starts (warm_stat: mean warm, mean
    uniform, solves, known bits; the learned start is kept only while it
    saves 8 sweeps, the price of its kernels)."""
    import numpy as np
    if not bp_start.startswith("learned"):
        return bp_start
    try:
        ws = np.asarray(b.value_by_name("rotamer", "warm_stat", 4 * b.n_sys)).reshape(-1, 4)
    except Exception:
        return bp_start
    known = ws[:, 3].astype(int)
    both = (known & 3) == 3
    used = both & (ws[:, 0] + 8.0 <= ws[:, 1])
    mw = float(ws[both, 0].mean()) if both.any() else float("nan")
    mu = float(ws[both, 1].mean()) if both.any() else float("nan")
    if not used.any():
        return ("uniform messages: the learned warm start fell back on all %d systems (measured %.1f sweeps "
                "from the learned start vs %.1f from uniform)" % (b.n_sys, mw, mu))
    return ("learned warm start on %d of %d systems, uniform on the rest (measured %.1f vs %.1f sweeps)"
            % (int(used.sum()), b.n_sys, mw, mu))


def bp_sweeps(b):
    """BP sweeps of each system's last solve, averaged (first sweep included)."""
    import numpy as np
    try:
        return float(np.mean(b.value_by_name("rotamer", "n_iter", b.n_sys))) + 1.0
    except Exception:
        return None


def plain_single_rate(W, a, states, n_sample=6, rounds=8):
    """The plain single-replica GPU path on a sample of the same workload:
    each sampled system in an engine of its own (one system per launch, the
    same kernels and one-round CUDA graph, the reference's uniform BP start),
    from the same equilibrated state as the batch, timed like the batch.
    Returns residue-steps/s of running the sample one system after another."""
    import numpy as np
    import upside_gb300 as U
    idx = list(range(min(n_sample, len(W["configs"]))))
    units = t = 0.0
    for i in idx:
        c = W["configs"][i]
        s = U.Batch([c])
        s.set_pos(states[i][0])
        s.set_mom(states[i][1])
        s.set_thermostat([W["temps"][i]], np.array([W["seeds"][i]], np.uint32))
        s.run(3, use_graph=True, graph_rounds=1)
        ms = s.bench(rounds, flush_l2=True)
        units += W["n_res"][i] * rounds
        t += float(ms.sum()) / 1e3
        del s
    return {"value": units / t, "unit": "residue-steps/s",
            "sample": "systems %s of the workload (%s residues), %d rounds each, one system per engine" % (
                ",".join(map(str, idx)), ",".join(str(W["n_res"][i]) for i in idx), rounds)}


def reference_over_port():
    """Measured speed ratio of the reference engine to the restatement on one
    x86 core (profiles/cpu_reference_vs_port.md, line 'ratio: R'), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "cpu_reference_vs_port.md")) as f:
            for line in f:
                if line.startswith("ratio:"):
                    return float(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return None


def cpu_fields(rate):
    """Estimate of the reference engine's rate on the same cores from the
    restatement's measured rate and the measured x86 ratio between them."""
    r = reference_over_port()
    if not r:
        return {}
    return {"reference_over_port_x86": r, "reference_estimate": rate * r,
            "reference_estimate_note": "restatement rate x the reference/restatement speed ratio measured on one "
                                       "x86 core (profiles/cpu_reference_vs_port.md); the reference cannot be "
                                       "built on the GPU host"}


def ncu_traffic(workload):
    """DRAM bytes per launch of the BP solve kernel from the committed ncu
    summary of this workload (profiles/bp_solve_kernel_<workload>.md, line
    'dram_bytes_per_launch: N'), or None when no capture was summarised."""
    path = os.path.join(ROOT, "profiles", "bp_solve_kernel_%s.md" % workload)
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("dram_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def roofline(b, W, a, peak, peak_kind):
    """The dominant kernel (the rotamer BP solve, bp_solve_kernel) against the
    HBM roofline: algorithmic bytes per launch (tallied by the kernel) over its
    mean launch time, both from the timed rounds (CUDA events recorded around
    every launch inside the replayed graph on the engine stream)."""
    k = b.bench_kernel()
    if not k["launches"] or k["ms"] <= 0:
        return {"error": "no timed launches of the BP solve kernel"}
    per_launch_s = k["ms"] / 1e3 / k["launches"]
    bytes_per_launch = k["bytes"] / k["launches"]
    achieved = bytes_per_launch / per_launch_s / 1e9
    return {"kernel": "bp_solve_kernel", "bound": "hbm", "achieved": achieved, "peak": peak,
            "peak_kind": "of " + peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": ncu_traffic(a.workload), "algorithmic_bytes_per_launch": bytes_per_launch,
            "ms_per_launch": 1e3 * per_launch_s, "launches": k["launches"]}


if __name__ == "__main__":
    main()
