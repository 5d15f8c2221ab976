"""Standalone device pair list (ug_pair_list) against a numpy brute force.

The distance test is the engine's: d2 = (dx*dx + dy*dy) + dz*dz with every
operation rounded to float32, hit when d2 < cutoff*cutoff (float32).  Pairs
come in the reference's pair-list order, (i // 4, j, i % 4)
(src/interaction_graph.h:122-157).  Integer output: compared bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def brute_pairs(x, cutoff):
    x = x.astype(np.float32)
    n = len(x)
    c2 = np.float32(cutoff) * np.float32(cutoff)
    ii, jj = np.triu_indices(n, 1)
    d = x[ii] - x[jj]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    hit = d2 < c2
    i, j = ii[hit], jj[hit]
    order = np.lexsort((i % 4, j, i // 4))
    return np.stack([i[order], j[order]], 1).astype(np.int32)


def run_pair_list(x, cutoff, cap):
    import torch
    import upside_gb300 as U
    pos = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    pairs = torch.full((max(cap, 1), 2), -1, dtype=torch.int32, device="cuda")
    n_pairs = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    U.pair_list(pos.data_ptr() if len(x) else 0, len(x), cutoff, pairs.data_ptr(), cap, n_pairs.data_ptr())
    return pairs.cpu().numpy()[:cap], int(n_pairs.item())


def cloud(n, seed, density=0.02):
    rng = np.random.RandomState(seed)
    side = (n / density) ** (1 / 3)
    return (rng.rand(n, 3) * side).astype(np.float32)


@pytest.mark.parametrize("n", [0, 1, 5, 131, 3001])
def test_pair_list_matches_brute_force(built, n):
    x = cloud(n, 11 + n)
    ref = brute_pairs(x, 6.0) if n > 1 else np.zeros((0, 2), np.int32)
    got, total = run_pair_list(x, 6.0, max(len(ref), 1))
    assert total == len(ref)
    assert np.array_equal(got[:total], ref)


def test_pair_list_truncates_at_cap(built):
    x = cloud(700, 3)
    ref = brute_pairs(x, 6.0)
    cap = len(ref) // 3
    got, total = run_pair_list(x, 6.0, cap)
    assert total == len(ref)
    assert np.array_equal(got, ref[:cap])


def test_pair_list_cutoff_is_strict(built):
    # points on a line 2.0 apart: 2.0 is exactly representable, so the pair at
    # distance exactly 2.0 is excluded and 1.5 is included
    x = np.array([[0, 0, 0], [2, 0, 0], [3.5, 0, 0], [10, 0, 0]], np.float32)
    got, total = run_pair_list(x, 2.0, 8)
    assert total == 1 and got[0].tolist() == [1, 2]


def test_pair_list_rejects_bad_arguments(built):
    import upside_gb300 as U
    with pytest.raises(RuntimeError):
        U.pair_list(0, -1, 2.0, 0, 0, 0)
    with pytest.raises(RuntimeError):
        U.pair_list(0, 4, 2.0, 0, 0, 0)
    with pytest.raises(RuntimeError, match="finite"):
        U.pair_list(0, 4, float("inf"), 0, 0, 0)


def test_pair_list_rejects_unaligned_output(built):
    import torch
    import upside_gb300 as U
    pos = torch.zeros((8, 3), dtype=torch.float32, device="cuda")
    buf = torch.zeros(64, dtype=torch.int32, device="cuda")
    n_pairs = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError, match="aligned"):
        U.pair_list(pos.data_ptr(), 8, 2.0, buf.data_ptr() + 4, 8, n_pairs.data_ptr())


def test_pair_list_total_beyond_int32(built):
    """70000 points within a small ball and a cutoff that covers them all:
    n (n - 1) / 2 = 2.45e9 pairs, beyond int32.  The total saturates at
    INT32_MAX, the first cap pairs come in order, and nothing outside the
    caller's [0, cap) pairs is written (guard words on both sides)."""
    import torch
    import upside_gb300 as U
    n, cap, guard = 70000, 1000, 64
    rng = np.random.RandomState(5)
    pos = torch.from_numpy(rng.rand(n, 3).astype(np.float32)).cuda()
    buf = torch.full((cap + 2 * guard, 2), -1, dtype=torch.int32, device="cuda")
    n_pairs = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    U.pair_list(pos.data_ptr(), n, 1e6, buf[guard].data_ptr(), cap, n_pairs.data_ptr())
    out = buf.cpu().numpy()
    assert int(n_pairs.item()) == 2 ** 31 - 1
    assert np.all(out[:guard] == -1) and np.all(out[guard + cap:] == -1)
    ii, jj = np.triu_indices(64, 1)
    order = np.lexsort((ii % 4, jj, ii // 4))
    first = np.stack([ii[order], jj[order]], 1)
    first = first[first[:, 0] < 4]  # row 0 (points 0-3) comes first, j ascending
    got = out[guard:guard + cap]
    assert np.array_equal(got[:len(first)], first)
    assert np.all(got[:, 0] < 4) and np.all(np.diff(got[:, 1]) >= 0)
