"""Periodic box mode (a mode of this engine only: the reference has open
boundaries, so there is no reference output to compare with; it is checked
against the open-boundary engine on images of the same configuration).

  * a box much larger than the system changes nothing: the same pair lists
    in the same order, energies and forces up to the run-to-run order of their
    atomic sums;
  * two chains that touch only across a face of the box give the energy and
    forces of the same two chains made adjacent by moving one of them by a box
    vector, with open boundaries (energy 1e-5 relative, forces 5e-4 of max
    |F|; the two differ only in FP32 rounding of the shifted coordinates),
    and the same number of pairs in every interaction graph (up to one pair
    at a cutoff that this rounding moves);
  * moving a chain by a box vector leaves energy and forces unchanged;
  * a box edge under twice a graph's reach is rejected.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAPHS = ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond", "environment_coverage_sc",
          "environment_coverage_hb", "hb_environment_coverage_hn", "hb_environment_coverage_oc", "backbone_pairs"]
N1 = 40
L = 90.0


@pytest.fixture(scope="module")
def two_chains(tmp_path_factory, built):
    """Two 40-residue chains, the second starting at residue 40; coordinates
    from the generator's random chains, chain A centred at x = 35 and chain B
    at x = 55 - 90: their centres are 20 A apart across the x face of a box
    of side 90 A, and 70 A apart with open boundaries."""
    import config_gen
    from h5lite import H5File
    path = str(tmp_path_factory.mktemp("pbc") / "two_chains.up")
    rng = np.random.RandomState(4)
    seq = config_gen.random_sequence(2 * N1, rng)
    config_gen.write_config(path, seq, 4, chain_first_residue=[N1])
    with H5File(path) as f:
        x = f.read("/input/pos")[:, :, 0].astype(np.float64)
    a, b = x[:3 * N1] - x[:3 * N1].mean(0), x[3 * N1:] - x[3 * N1:].mean(0)
    a[:, 0] += 35.0
    b[:, 0] += 55.0 - L
    return path, np.concatenate([a, b]).astype(np.float32)


def _eval(path, x, box=None):
    import upside_gb300 as U
    bt = U.Batch([path])
    if box is not None:
        bt.set_box(*box)
    bt.set_pos(x)
    e, d = bt.evaluate()
    edges = {g: bt.node_edges(g) for g in GRAPHS}
    return bt, e[0], d, edges


def test_large_box_changes_nothing(two_chains):
    path, x = two_chains
    _, e0, d0, ed0 = _eval(path, x)
    _, e1, d1, ed1 = _eval(path, x, box=(1000.0, 1000.0, 1000.0))
    for g in GRAPHS:
        assert np.array_equal(ed0[g], ed1[g]), g
    # energies and forces are sums whose atomic-add order varies from run to run
    assert abs(e0 - e1) <= 1e-7 * max(1.0, abs(e0))
    assert np.abs(d0 - d1).max() <= 1e-5 * np.abs(d0).max()


def test_contact_across_the_face_equals_its_image(two_chains):
    path, x = two_chains
    shift = np.zeros_like(x)
    shift[3 * N1:, 0] = L
    # open boundaries, B moved next to A: the physical contact
    _, e_open, d_open, ed_open = _eval(path, x + shift)
    # periodic, B at the far face: the same contact through the boundary
    _, e_box, d_box, ed_box = _eval(path, x, box=(L, L, L))
    # open boundaries, B at the far face: no contact
    _, e_far, _, ed_far = _eval(path, x)
    contact = sum(len(ed_open[g]) for g in GRAPHS) - sum(len(ed_far[g]) for g in GRAPHS)
    assert contact > 20  # inter-chain pairs exist only through the face
    for g in GRAPHS:  # equal up to a pair at the cutoff that rounding of the shifted coordinates moves
        assert abs(len(ed_box[g]) - len(ed_open[g])) <= 1, g
    scale = max(1.0, abs(e_open), abs(e_far))
    assert abs(e_box - e_open) <= 1e-5 * scale, (e_box, e_open)
    assert abs(e_open - e_far) > 1e-3 * scale  # the contact matters
    # the two configurations' FP32 coordinates of chain B differ by rounding
    # (~4e-6 A at 55 A), which steep steric walls turn into ~1e-4 of max |F|
    assert np.abs(d_box - d_open).max() <= 5e-4 * np.abs(d_open).max()


def test_box_vector_shift_is_invisible(two_chains):
    path, x = two_chains
    _, e0, d0, _ = _eval(path, x, box=(L, L, L))
    for axis in range(3):
        y = x.copy()
        y[:3 * N1, axis] -= L  # chain A by a box vector
        _, e1, d1, _ = _eval(path, y, box=(L, L, L))
        assert abs(e1 - e0) <= 1e-5 * max(1.0, abs(e0)), axis
        assert np.abs(d1 - d0).max() <= 1e-4 * np.abs(d0).max(), axis


def test_box_too_small_is_rejected(two_chains):
    import upside_gb300 as U
    path, _ = two_chains
    bt = U.Batch([path])
    with pytest.raises(RuntimeError, match="twice the reach"):
        bt.set_box(8.0, 8.0, 8.0)
    with pytest.raises(RuntimeError):
        bt.set_box(-1.0, 0.0, 0.0)


def test_periodic_dynamics_run(two_chains):
    """Rounds in the periodic box run through the captured graph without
    status bits, and the energy stays finite."""
    import upside_gb300 as U
    path, x = two_chains
    bt = U.Batch([path])
    bt.set_box(L, L, L)
    bt.set_pos(x)
    bt.set_thermostat([0.85], np.array([3], np.uint32))
    bt.run(20, use_graph=True, graph_rounds=5)
    e, _ = bt.evaluate()
    assert np.isfinite(e).all() and bt.status() & 3 == 0
