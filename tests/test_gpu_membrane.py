"""Membrane potential on the GPU: cb_membrane_potential and
hb_membrane_potential (src/membrane_potential.cpp:221-672) and Const3D
(src/coord_const.cpp:107-179), flat and on a curved bilayer, in the fixture
of golden/membrane_spec.py.

Tolerances as in test_gpu_parity.py: energy 1e-5 of sum |E_node| and max
force 1e-4 of max |F| against the FP32 and FP64 oracle; 1e-5 and 1e-4
against the reference engine (conftest.ref_force_bound).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import E_REF_TOL as E_REF, ref_force_bound  # noqa: E402

E_ORC, F_ORC = 1e-5, 1e-4
MEMB = ("cb_membrane_potential", "hb_membrane_potential")


def energy_scale(eng, path):
    from h5lite import H5File
    tot = 0.0
    for nm in H5File(path).list("/input/potential"):
        n, w = eng.get_output_dims(nm)
        if n == 1 and w == 1:
            tot += abs(float(eng.get_output(nm)[0, 0]))
    return max(tot, 1.0)


def rel_f(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("variant", ["flat", "curved"])
def test_membrane_frames(membrane_configs, variant):
    """Frames in order on one engine (the position-captured Const3D keeps
    frame 0's atoms): energy and forces against the reference and both
    oracles, and the membrane nodes' outputs and sensitivities against the
    reference's."""
    import oracle_py
    import upside_gb300 as U
    paths, z = membrane_configs
    path = paths[variant]
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o32, o64 = oracle_py.Oracle(path, na), oracle_py.Oracle(path, na, fp64=True)
    for k in range(len(z["pos"])):
        x = z["pos"][k]
        e, d = eng.energy(x), eng.deriv(x)
        sc = energy_scale(eng, path)
        assert abs(e - z[variant + "/ref_energy"][k]) < E_REF * sc, k
        assert rel_f(d, z[variant + "/ref_deriv"][k]) < ref_force_bound(z[variant + "/ref_deriv"][k],
                                                                         o64.evaluate(x)[1]), k
        for o in (o32, o64):
            eo, do = o.evaluate(x)
            assert abs(e - eo) < E_ORC * sc, k
            assert rel_f(d, do) < F_ORC, k
        for nm in MEMB + ("Const3D_probe", "Const3D_curvature_center", "Const1D_probe", "Const2D_fixed"):
            ref = z["%s/out/%s" % (variant, nm)][k]
            assert np.abs(eng.get_output(nm) - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1.0), (k, nm)
        for nm in ("placement_fixed_point_only_CB",):
            ref = z["%s/sens/%s" % (variant, nm)][k]
            assert np.abs(eng.get_sens(nm) - ref).max() <= 1e-4 * max(np.abs(ref).max(), 1.0), (k, nm)
            assert np.abs(eng.get_sens(nm) - o32.node(nm, sens=True)).max() <= 1e-4 * max(np.abs(ref).max(), 1.0)


def test_membrane_batch(membrane_configs, tmp_path):
    """Flat bilayers of two lengths in one batch equal single evaluations;
    flat and curved systems do not share a batch (different attributes)."""
    import membrane_spec
    import upside_gb300 as U
    paths, z = membrane_configs
    p62 = str(tmp_path / "m62.up")
    membrane_spec.write(p62, "flat", n_res=62, seed=21)
    x62 = membrane_spec.frames(seed=5, n_res=62)
    sets = [(p62, x62[1]), (paths["flat"], z["pos"][2]), (p62, x62[2])]
    b = U.Batch([p for p, _ in sets])
    b.set_pos(np.concatenate([x for _, x in sets]))
    e, d = b.evaluate()
    lo = 0
    for k, (p, x) in enumerate(sets):
        s = U.Upside(p, len(x))
        es, ds = s.energy(x), s.deriv(x)
        assert abs(e[k] - es) < 1e-5 * energy_scale(s, p), k
        assert rel_f(d[lo:lo + len(x)], ds) < 1e-5, k
        lo += len(x)
    with pytest.raises(RuntimeError):
        U.Batch([paths["flat"], paths["curved"]])


def test_membrane_dynamics_and_const_capture(membrane_configs):
    """Graph replays keep the captured Const3D rows at the first
    evaluation's positions; graph and eager trajectories agree."""
    import upside_gb300 as U
    paths, z = membrane_configs
    res = []
    for graph in (False, True):
        b = U.Batch([paths["curved"], paths["curved"]])
        x0 = np.concatenate([z["pos"][0], z["pos"][2]])
        b.set_pos(x0)
        b.set_thermostat([0.8, 0.9], np.array([5, 6], np.uint32))
        b.run(6, use_graph=graph, graph_rounds=3)
        res.append(b.get_pos())
        probe = b.node_output("Const3D_probe")
        assert np.array_equal(probe[:2], z["pos"][0][[5, 17]])
        assert np.array_equal(probe[2:], z["pos"][2][[5, 17]])
        assert b.status() & 3 == 0
    assert np.all(np.isfinite(res[0]))
    assert np.abs(res[0] - res[1]).max() < 1e-3


def test_membrane_params(membrane_configs):
    """get_param / set_param of the spline tables: doubling them doubles
    each membrane node's energy."""
    import upside_gb300 as U
    paths, z = membrane_configs
    b = U.Batch([paths["flat"]])
    b.set_pos(z["pos"][1])
    b.evaluate()
    shapes = {"cb_membrane_potential": (20, 2, 18), "hb_membrane_potential": (2, 2, 18)}
    e0 = {nm: b.node_potential(nm)[0] for nm in MEMB}
    for nm in MEMB:
        p = b.get_param(nm, shapes[nm])
        b.set_param(nm, 2 * p)
    b.evaluate()
    for nm in MEMB:
        assert abs(b.node_potential(nm)[0] - 2 * e0[nm]) < 1e-5 * max(abs(e0[nm]), 1.0), nm


def test_membrane_driver_run(membrane_configs, tmp_path):
    """The upside driver runs the curved-membrane configuration: frame 0
    holds the potential of the initial coordinates, later frames stay
    finite."""
    import shutil
    import upside_gb300 as U
    from h5lite import H5File
    paths, _ = membrane_configs
    cfg = str(tmp_path / "memb.up")
    shutil.copyfile(paths["curved"], cfg)
    rt = float(np.float32(3) * np.float32(0.009))
    U.upside_main(["--duration", repr(30 * rt), "--frame-interval", repr(10 * rt), "--temperature", "0.85",
                   "--seed", "3", cfg], verbose=False)
    f = H5File(cfg)
    pos, pot = f.read("/output/pos"), f.read("/output/potential")
    assert pos.shape[0] == 3 and np.all(np.isfinite(pos)) and np.all(np.isfinite(pot))
    eng = U.Upside(paths["curved"], pos.shape[2])
    x0 = f.read("/input/pos")[:, :, 0]
    assert abs(eng.energy(x0) - pot[0, 0]) < 1e-4 * max(abs(pot[0, 0]), 1.0)
