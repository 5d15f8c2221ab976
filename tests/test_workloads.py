"""The bench workloads (upside2-md_gb300/workloads.py) as bench.py and the GPU
tests use them, generated on the CPU: system counts and sizes, temperatures,
replica-exchange sets, the periodic box, and the node graph written into
their configurations.  A small system of the plain and of the membrane kind
is evaluated by the FP32 oracle to a finite energy and forces, so that a
change of the configuration writer that breaks them shows here rather than
on the GPU."""
import numpy as np
import pytest

FF21 = {"affine_alignment", "rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond",
        "environment_coverage_sc", "environment_coverage_hb", "hb_environment_coverage_hn",
        "hb_environment_coverage_oc", "sigmoid_coupling_environment", "backbone_pairs", "rama_map_pot"}
MEMBRANE = {"surface", "cb_surf_membrane_potential", "hb_surf_membrane_potential", "membranelateral_potential"}


def nodes(path):
    from h5lite import H5File
    return set(H5File(path).list("/input/potential"))


def test_c4_batch():
    """64 chains, lengths uniform in [40, 400] (14,918 residues with seed 1),
    temperatures in [0.80, 0.95], the ff_2.1 node graph."""
    import workloads
    W = workloads.workload("C4", seed=1)
    n = np.array(W["n_res"])
    assert len(W["configs"]) == 64 and n.min() >= 40 and n.max() <= 400
    assert int(n.sum()) == 14918
    t = np.array(W["temps"])
    assert t.min() >= 0.80 and t.max() <= 0.95
    assert W["swap_sets"] is None and W["box"] is None
    assert FF21 <= nodes(W["configs"][0])
    assert not (MEMBRANE & nodes(W["configs"][0]))
    # the same seed gives the same batch
    assert workloads.workload("C4", seed=1)["n_res"] == W["n_res"]


def test_c3_replicas():
    """48 replicas of one 150-residue chain on a geometric temperature ladder
    from 0.80 to 1.00, exchanges between even and odd neighbours every 20
    rounds."""
    import workloads
    W = workloads.workload("C3", seed=1)
    assert len(W["configs"]) == 48 and len(set(W["configs"])) == 1 and W["n_res"] == [150] * 48
    t = np.array(W["temps"])
    assert abs(t[0] - 0.80) < 1e-12 and abs(t[-1] - 1.00) < 1e-12
    assert np.allclose(t[1:] / t[:-1], (1.0 / 0.8) ** (1 / 47.))
    even, odd = W["swap_sets"]
    assert even == [(i, i + 1) for i in range(0, 47, 2)] and odd == [(i, i + 1) for i in range(1, 47, 2)]
    assert W["exchange_interval"] == 20


def test_c5_system():
    """One 2000-residue system of eight chains in a 200 A box."""
    import workloads
    from h5lite import H5File
    W = workloads.workload("C5", seed=1)
    assert W["n_res"] == [2000] and W["box"] == (200.0, 200.0, 200.0)
    f = H5File(W["configs"][0])
    assert f.read("/input/pos").shape[0] == 3 * 2000
    assert FF21 <= nodes(W["configs"][0])


def test_m1_membrane_batch():
    """64 membrane chains, lengths uniform in [40, 200] (7,813 residues with
    seed 1), with the surface node and the surface-dependent terms."""
    import workloads
    W = workloads.workload("M1", seed=1)
    n = np.array(W["n_res"])
    assert len(W["configs"]) == 64 and n.min() >= 40 and n.max() <= 200 and int(n.sum()) == 7813
    assert (FF21 | MEMBRANE) <= nodes(W["configs"][0])


@pytest.mark.parametrize("name", ["C1", "M1"])
def test_oracle_evaluates_workload_system(built, name):
    """The first system of the workload evaluates in the FP32 oracle to a
    finite, non-zero energy and finite forces."""
    import oracle_py
    import workloads
    W = workloads.workload(name, seed=1)
    path = W["configs"][0]
    x = workloads.initial_positions([path])
    e, f = oracle_py.Oracle(path, len(x)).evaluate(x)
    assert np.isfinite(e) and e != 0.0
    assert f.shape == x.shape and np.all(np.isfinite(f)) and np.abs(f).max() > 0
