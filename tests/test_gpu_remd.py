"""Replica exchange on the device (ReplicaExchange::attempt_swaps,
src/main.cpp:243-316) against a restatement, decision for decision and draw
for draw.

The restatement takes the engine's own energies at the coordinates before the
exchange (identical Hamiltonians, so a swapped system's new energy is its
partner's old one), the temperatures, and the replica-exchange stream of the
oracle's Threefry-4x32-20 (pinned to the reference's Random123 by the
known-answer test): key (seed, 1, 0, 0), counter (round lo, round hi, 0, k)
for the k-th draw, u = r123::u01<float> of the first word; a draw is made only
for a negative change of log Boltzmann factors.  Criterion 0 undoes a swap
when exp(diff) < u; criterion 1 swaps when diff >= 0 or exp(diff) >= u.  The
cases cover accepted swaps with and without a draw and rejected ones.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_REP = 8


def uniform(seed, round_, k):
    import oracle_py
    L = oracle_py._lib()
    L.ocpu_threefry4x32.argtypes = [ctypes.c_void_p] * 3
    c = np.array([round_ & 0xffffffff, round_ >> 32, 0, k], np.uint32)
    key = np.array([seed, 1, 0, 0], np.uint32)
    out = np.zeros(4, np.uint32)
    L.ocpu_threefry4x32(c.ctypes.data, key.ctypes.data, out.ctypes.data)
    return float(np.float32(out[0]) * np.float32(1.0 / 4294967296.0) + np.float32(0.5 / 4294967296.0))


def restate(energy, temps, pairs, seed, round_, criterion):
    """expected accept flags and the kinds of decision (nodraw, accept, reject)"""
    lb = -np.asarray(energy, np.float64) / np.asarray(temps, np.float64)
    acc, kinds, k = [], [], 0
    for s1, s2 in pairs:
        if criterion == 0:  # after the swap system s1 holds s2's coordinates and vice versa
            diff = (-energy[s2] / temps[s1] - energy[s1] / temps[s2]) - (lb[s1] + lb[s2])
        else:
            diff = lb[s2] - lb[s1]
        if diff >= 0:
            acc.append(1)
            kinds.append("nodraw")
            continue
        u = uniform(seed, round_, k)
        k += 1
        a = math.exp(diff) >= u
        acc.append(int(a))
        kinds.append("accept" if a else "reject")
    return np.array(acc), kinds


def _batch(syn_configs, temps, seed=0):
    import upside_gb300 as U
    path, z = syn_configs[60]
    rng = np.random.RandomState(seed)
    xs = [z["pos"][k % 3] + rng.normal(0, 0.03, z["pos"][0].shape).astype(np.float32) for k in range(N_REP)]
    b = U.Batch([path] * N_REP)
    b.set_pos(np.concatenate(xs))
    b.set_thermostat(temps, np.arange(N_REP, dtype=np.uint32))
    return b, xs


SETS = [[(0, 1), (2, 3), (4, 5), (6, 7)], [(1, 2), (3, 4), (5, 6)]]
TEMPS = [list(0.80 * (1.25 ** (np.arange(N_REP) / (N_REP - 1)))), [0.85 + 0.004 * k for k in range(N_REP)]]


def test_single_exchange_draw_for_draw(syn_configs):
    """ug_replica_exchange (criterion 0) at given seeds and rounds."""
    seen = set()
    for ti, temps in enumerate(TEMPS):
        for seed, round_ in ((5, 10), (7, 1 << 33), (11, 3)):
            b, xs = _batch(syn_configs, temps, seed=seed + ti)
            e_old, _ = b.evaluate(want_deriv=False)
            for pairs in SETS:
                want, kinds = restate(e_old, temps, pairs, seed, round_, 0)
                x0 = b.get_pos().reshape(N_REP, -1, 3)
                got = b.replica_exchange(pairs, seed=seed, round_=round_)
                assert np.array_equal(got, want), (ti, seed, round_, pairs, got, want, kinds)
                x1 = b.get_pos().reshape(N_REP, -1, 3)
                for (i, j), a in zip(pairs, got):
                    if a:
                        assert np.array_equal(x1[i], x0[j]) and np.array_equal(x1[j], x0[i])
                    else:
                        assert np.array_equal(x1[i], x0[i]) and np.array_equal(x1[j], x0[j])
                seen.update(kinds)
                e_old, _ = b.evaluate(want_deriv=False)
    assert seen == {"nodraw", "accept", "reject"}, seen


@pytest.mark.parametrize("criterion", [0, 1])
def test_plan_exchanges_draw_for_draw(syn_configs, criterion):
    """The periodic plan's exchanges, made one at a time: the set alternates,
    the draws are keyed by round (k + 1) * interval, replica indices and
    per-pair counters follow the decisions."""
    interval, seed = 20, 9
    seen = set()
    for ti, temps in enumerate(TEMPS):
        b, _ = _batch(syn_configs, temps, seed=3 + ti)
        b.set_replica_exchange(SETS, seed, interval, criterion)
        replica = np.arange(N_REP)
        att = np.zeros(sum(len(s) for s in SETS), int)
        suc = np.zeros_like(att)
        for k in range(4):
            e_old, _ = b.evaluate(want_deriv=False)
            pairs = SETS[k % 2]
            want, kinds = restate(e_old, temps, pairs, seed, (k + 1) * interval, criterion)
            b.exchange_now()
            rep, na, ns, n_ex, last, last_set = b.replica_state()
            assert n_ex == k + 1 and last_set == k % 2
            assert np.array_equal(last[:len(pairs)], want), (ti, k, last, want, kinds)
            off = 0 if k % 2 == 0 else len(SETS[0])
            for q, ((i, j), a) in enumerate(zip(pairs, want)):
                att[off + q] += 1
                suc[off + q] += a
                if a:
                    replica[i], replica[j] = replica[j], replica[i]
            assert np.array_equal(rep, replica) and np.array_equal(na, att) and np.array_equal(ns, suc)
            seen.update(kinds)
    assert "nodraw" in seen and ("accept" in seen or "reject" in seen), seen


def test_exchanges_inside_graph_equal_eager(syn_configs):
    """Periodic exchanges every 5 rounds: 20 rounds as captured graphs (each
    replay one interval and its exchange) and the same 20 rounds eagerly give
    the same replica permutation and counters, and nearby coordinates."""
    temps = TEMPS[1]
    out = []
    for use_graph in (True, False):
        b, _ = _batch(syn_configs, temps, seed=1)
        b.set_replica_exchange(SETS, 4, 5, 0)
        b.run(20, use_graph=use_graph, graph_rounds=5)
        rep, na, ns, n_ex, _, _ = b.replica_state()
        assert n_ex == 4
        out.append((rep, na, ns, b.get_pos()))
        assert b.status() & 3 == 0
    (r0, a0, s0, x0), (r1, a1, s1, x1) = out
    assert np.array_equal(r0, r1) and np.array_equal(a0, a1) and np.array_equal(s0, s1)
    # FP32 trajectories of 20 rounds whose force sums differ in atomic order
    assert np.abs(x0 - x1).max() < 0.1


def test_plan_rejects_bad_sets(syn_configs):
    import upside_gb300 as U
    b, _ = _batch(syn_configs, TEMPS[0])
    with pytest.raises(RuntimeError, match="Overlapping"):
        b.set_replica_exchange([[(0, 1), (1, 2)]], 1, 5, 0)
    with pytest.raises(RuntimeError):
        b.set_replica_exchange([[(0, 8)]], 1, 5, 0)
    path60 = syn_configs[60][0]
    path150 = syn_configs[150][0]
    m = U.Batch([path60, path150])
    with pytest.raises(RuntimeError, match="same number of atoms"):
        m.set_replica_exchange([[(0, 1)]], 1, 5, 0)
