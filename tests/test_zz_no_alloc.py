"""ug_pair_list_noalloc (fixed device scratch, no allocation) against the
allocating ug_pair_list, through the C ABI.

Integer output, so the comparison is exact.  Two consecutive calls must both
agree: the second finds the scratch holding the first call's values, which
must not leak into its result.  This file is collected last so that it also
runs after everything else has used the device.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CUTOFF = 6.0


def _cloud(n, seed):
    rng = np.random.RandomState(seed)
    side = (n / 0.02) ** (1 / 3)
    return (rng.rand(n, 3) * side).astype(np.float32)


def _call(fn, pos, n, cap, cutoff=CUTOFF):
    import torch
    pairs = torch.full((max(cap, 1), 2), -1, dtype=torch.int32, device="cuda")
    n_pairs = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fn(pos.data_ptr() if n else 0, n, cutoff, pairs.data_ptr(), cap, n_pairs.data_ptr(), 0)
    torch.cuda.synchronize()
    return pairs.cpu().numpy()[:cap], int(n_pairs.item())


@pytest.mark.parametrize("n", [20000, 5])
def test_noalloc_matches_allocating(built, n):
    import torch
    import upside_gb300 as U
    pos = torch.from_numpy(_cloud(n, 17)).cuda()
    ref, total = _call(U.pair_list, pos, n, 400000)
    assert 0 < total <= 400000 or n == 5
    for _ in range(2):
        got, got_total = _call(U.pair_list_noalloc, pos, n, 400000)
        assert got_total == total
        assert np.array_equal(got[:total], ref[:total])


@pytest.mark.parametrize("n", [262144, 262141])
def test_noalloc_at_the_limit(built, n):
    """The largest accepted sizes: every row of the fixed scratch in use (the
    total lands in its last word), and a size that is not a multiple of 4."""
    import torch
    import upside_gb300 as U
    pos = torch.from_numpy(_cloud(n, 23)).cuda()
    ref, total = _call(U.pair_list, pos, n, 400000, cutoff=2.0)
    assert 0 < total <= 400000
    for _ in range(2):
        got, got_total = _call(U.pair_list_noalloc, pos, n, 400000, cutoff=2.0)
        assert got_total == total
        assert np.array_equal(got[:total], ref[:total])


def test_noalloc_rejects_oversize(built):
    import upside_gb300 as U
    with pytest.raises(RuntimeError, match="262144"):
        U.pair_list_noalloc(0, 262145, CUTOFF, 0, 0, 0)
