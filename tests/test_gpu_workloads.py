"""The benchmark configurations other than the bench's own (C4) as parity
cases: the 300-residue chain (C2), the 2000-residue eight-chain system with
chain breaks (C5), and the 48-replica exchange batch (C3).

Tolerances as in test_gpu_parity.py: energy 1e-5 of sum |E_node| and max force
1e-4 of max |F| against the FP32 and FP64 oracles.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_ORC, F_ORC = 1e-5, 1e-4


def _scale(path, eng):
    from h5lite import H5File
    tot = 0.0
    for nm in H5File(path).list("/input/potential"):
        n, w = eng.get_output_dims(nm)
        if n == 1 and w == 1:
            tot += abs(float(eng.get_output(nm)[0, 0]))
    return max(tot, 1.0)


def _check_vs_oracle(path, x, bp_slack=False):
    """GPU against both oracles.  The force bound is 1e-4 of max |F|, or 2.5
    times the FP32 oracle's own distance from FP64 when that is larger.  At
    the steep steric walls of relaxed random coils (backbone pairs,
    src/backbone_steric.cpp:18-30) FP32 coordinates of ~50 A carry ~1e-4
    relative force noise in any FP32 evaluation order (the reference shows
    8e-5 on its own fixture); the largest-atom figure of that noise varies
    with the order, observed 0.7-1.4e-4 for the GPU where the FP32 oracle
    shows 0.7-0.8e-4 on frames of one trajectory.  In a 2000-residue system
    an FP32 force component also sums thousands of terms.  bp_slack: 5e-4 in
    place of 1e-4 (BP stopped at the recipe's tolerance)."""
    f_tol = 5e-4 if bp_slack else F_ORC
    import oracle_py
    import upside_gb300 as U
    eng = U.Upside(path, x.shape[0])
    e, d = eng.energy(x), eng.deriv(x)
    sc = _scale(path, eng)
    e32, d32 = oracle_py.Oracle(path, x.shape[0]).evaluate(x)
    e64, d64 = oracle_py.Oracle(path, x.shape[0], fp64=True).evaluate(x)
    fmax = np.abs(d64).max()
    fp32_gap = np.abs(d32 - d64).max() / fmax
    bound = max(f_tol, 2.5 * fp32_gap)
    assert abs(e - e32) < E_ORC * sc, (e, e32)
    assert abs(e - e64) < E_ORC * sc, (e, e64)
    gpu_gap = np.abs(d - d64).max() / fmax
    gpu_32 = np.abs(d - d32).max() / fmax
    print("%s: GPU-FP64 %.2e FP32 oracle-FP64 %.2e GPU-FP32 oracle %.2e (bound %.2e)" %
          (os.path.basename(path), gpu_gap, fp32_gap, gpu_32, bound))
    # the FP64 instantiation is the yardstick; two FP32 evaluation orders
    # (GPU, FP32 oracle) differ by up to the sum of their distances from it
    assert gpu_gap < bound, (gpu_gap, fp32_gap)
    assert gpu_32 < max(f_tol, gpu_gap + fp32_gap) * 1.001, (gpu_32, gpu_gap, fp32_gap)


@pytest.mark.parametrize("name", ["C2", "C5"])
def test_workload_energy_forces_vs_oracle(built, name, tmp_path):
    """Initial coil and, after 20 integration rounds (of the FP32 oracle), a
    relaxed frame.

    The relaxed frame is also evaluated from a copy of the config with the BP
    tolerance tightened to 1e-7: at the recipe's 1e-3 two solves that iterate
    in different float orders may stop at marginals up to ~1e-3 apart on
    near-degenerate residues, and in the 2000-residue system that alone moves
    some forces by ~2e-4 of max |F| (observed; 1.25e-4 on a relaxed
    300-residue frame).  The bound is 5e-4 at the recipe's tolerance (the
    2000-residue coil and both relaxed frames) and 1e-4 (or the FP32 rule of _check_vs_oracle) at the
    tight one.  FP32 cannot resolve 1e-7, so the GPU and FP32-oracle solves of
    the tight copy run to the 1000-iteration cap while FP64 converges in
    ~60 sweeps; on the 2000-residue frame the FP32 oracle then sits
    1.2e-4..2.0e-4 of max |F| from FP64 and the GPU 0.5e-4..1.4e-4 from the
    FP32 oracle (observed over independent trajectories)."""
    import config_gen
    import workloads
    from h5lite import H5File
    W = workloads.workload(name, seed=3)
    path = W["configs"][0]
    x0 = workloads.initial_positions([path])
    _check_vs_oracle(path, x0, bp_slack=name == "C5")
    # a relaxed frame after 20 integration rounds of the FP32 oracle (its
    # trajectory is deterministic, so the frame and the margins below are the
    # same in every run; GPU dynamics are checked in test_gpu_dynamics.py)
    import oracle_py
    x1, _ = oracle_py.Oracle(path, x0.shape[0]).run(x0, np.zeros_like(x0), 20, dt=0.009,
                                                    temperature=float(W["temps"][0]), timescale=5.0,
                                                    seed=int(W["seeds"][0]))
    # at the recipe's tolerance: both chains' solves may stop
    # at marginals ~1e-3 apart (C2 observed at 1.25e-4 of max |F|); the
    # tight copy below holds the 1e-4 bound
    _check_vs_oracle(path, x1, bp_slack=True)
    with H5File(path) as f:
        seq = [s.decode() for s in f.read("/input/sequence")]
        starts = list(f.read("/input/chain_break/chain_first_residue")) if f.exists("/input/chain_break") else []
    tight = str(tmp_path / "tight.up")
    config_gen.write_config(tight, seq, 3, chain_first_residue=starts, pos=x1.reshape(-1, 3), bp_tol=1e-7)
    _check_vs_oracle(tight, x1)


def test_c5_bonded_terms_stop_at_chain_breaks(built):
    """C5's eight chains are bonded only within themselves: 3N - 1 bonds and
    3N - 2 angles per chain of N residues, so 8 fewer bonds and 16 fewer
    angles than one 2000-residue chain."""
    import upside_gb300 as U
    import workloads
    W = workloads.workload("C5", seed=3)
    path = W["configs"][0]
    x = workloads.initial_positions([path])
    eng = U.Upside(path, x.shape[0])
    assert np.isfinite(eng.energy(x))
    assert eng.get_output_dims("Distance3D")[0] == 8 * (3 * 250 - 1)
    assert eng.get_output_dims("Angle")[0] == 8 * (3 * 250 - 2)


def test_c3_replica_exchange_batch(built):
    """48 replicas of one chain with the alternating even/odd swap sets every
    20 rounds (the reference's --replica-interval in its step unit), the
    exchanges made on the device inside the captured graphs: after 60 rounds
    three exchanges were made (sets 0, 1, 0), the replica indices are a
    permutation, every pair was attempted as often as its set came up, some
    swaps were accepted, and a plain single exchange through
    ug_replica_exchange agrees with the energies it saw (decisions are
    checked draw for draw in test_gpu_remd.py)."""
    import upside_gb300 as U
    import workloads
    W = workloads.workload("C3", seed=3)
    assert W["exchange_interval"] == 20
    b = U.Batch(W["configs"])
    b.set_pos(workloads.initial_positions(W["configs"]))
    b.set_thermostat(np.asarray(W["temps"]), np.array(W["seeds"], np.uint32))
    b.set_replica_exchange(W["swap_sets"], 11, W["exchange_interval"], 0)
    b.run(60, use_graph=True, graph_rounds=20)
    rep, na, ns, n_ex, _, _ = b.replica_state()
    assert n_ex == 3
    assert sorted(rep.tolist()) == list(range(48))
    n0 = len(W["swap_sets"][0])
    assert np.all(na[:n0] == 2) and np.all(na[n0:] == 1)
    assert np.all(ns <= na) and ns.sum() > 0
    assert b.status() & 3 == 0
