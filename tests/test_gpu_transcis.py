"""Trans-cis proline nodes on the GPU: RamaMap2 (src/rama_map_pot.cpp:96-175),
SigmoidCoord (src/coord_map.cpp:609-675), Add / Mean / Multiply
(src/coord_operator.cpp:15-351) and SigmoidEnergy / SigmoidLEnergy
(src/sigmoid_energy.cpp), in the fixture of golden/transcis_spec.py (which
also fixes rotamers and holds a cis proline).

Tolerances as in test_gpu_parity.py: energy 1e-5 of sum |E_node| and max
force 1e-4 of max |F| against the FP32 and FP64 oracle; against the reference
engine's frames energy 1e-5 and force 1e-4 (conftest.ref_force_bound).
"""
import numpy as np
import pytest

from conftest import E_REF_TOL as E_REF, quat_align, ref_force_bound

pytestmark = pytest.mark.gpu

E_ORC, F_ORC = 1e-5, 1e-4


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


def test_trans_cis_frames(transcis_config):
    import oracle_py
    import upside_gb300 as U
    path, z = transcis_config
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o32, o64 = oracle_py.Oracle(path, na), oracle_py.Oracle(path, na, fp64=True)
    for k in range(len(z["pos"])):
        x = z["pos"][k]
        e, d = eng.energy(x), eng.deriv(x)
        sc = energy_scale(eng, path)
        assert abs(e - z["ref_energy"][k]) < E_REF * sc, k
        assert rel_f(d, z["ref_deriv"][k]) < ref_force_bound(z["ref_deriv"][k], o64.evaluate(x)[1]), k
        for o in (o32, o64):
            eo, do = o.evaluate(x)
            assert abs(e - eo) < E_ORC * sc, k
            assert rel_f(d, do) < F_ORC, k


def test_trans_cis_nodes(transcis_config):
    """Every node's output and sensitivity against the FP32 oracle, and the
    trans-cis nodes against the reference engine's, at every frame."""
    import oracle_py
    import upside_gb300 as U
    from h5lite import H5File
    path, z = transcis_config
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o = oracle_py.Oracle(path, na)
    names = H5File(path).list("/input/potential")
    for k in range(len(z["pos"])):
        eng.energy(z["pos"][k])
        o.evaluate(z["pos"][k])
        for nm in names:
            a, b = eng.get_output(nm), o.node(nm)
            if nm == "affine_alignment":
                a = quat_align(a, b)
            assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1.0), (k, nm)
            sa, sb = eng.get_sens(nm), o.node(nm, sens=True)
            if nm == "protein_hbond":
                # scores of ~0 take the hbond energy's sensitivity in one FP32
                # order and not another; it multiplies d(score)/dx ~ 0
                tiny = b[:, 6] < 1e-6
                sa, sb = sa.copy(), sb.copy()
                sa[tiny, 6] = sb[tiny, 6] = 0.0
            assert np.abs(sa - sb).max() <= 1e-3 * max(np.abs(sb).max(), 1.0), (k, nm)
            if "out/" + nm in z.files and nm != "rama_coord":
                assert np.abs(eng.get_output(nm) - z["out/" + nm][k]).max() <= 1e-5 * max(
                    np.abs(z["out/" + nm][k]).max(), 1.0), (k, nm)
                assert np.abs(eng.get_sens(nm) - z["sens/" + nm][k]).max() <= 1e-4 * max(
                    np.abs(z["sens/" + nm][k]).max(), 1.0), (k, nm)


def test_trans_cis_batch(transcis_config, tmp_path):
    """Systems of different lengths with the same trans-cis graph in one
    batch: per-system switch rows and combine rows."""
    import transcis_spec
    import upside_gb300 as U
    path, z = transcis_config
    p48 = str(tmp_path / "tc48.up")
    transcis_spec.write(p48, n_res=48, seed=9)
    x48 = transcis_spec.frames(seed=77, n_res=48)
    b = U.Batch([p48, path, p48])
    xs = [x48[1], z["pos"][2], x48[3]]
    b.set_pos(np.concatenate(xs))
    e, d = b.evaluate()
    lo = 0
    for k, (p, x) in enumerate(zip([p48, path, p48], xs)):
        s = U.Upside(p, len(x))
        es, ds = s.energy(x), s.deriv(x)
        assert abs(e[k] - es) < 1e-5 * energy_scale(s, p), k
        assert rel_f(d[lo:lo + len(x)], ds) < 1e-5, k
        lo += len(x)


def test_trans_cis_dynamics_graph_matches_eager(transcis_config):
    import upside_gb300 as U
    path, z = transcis_config
    res = []
    for graph in (False, True):
        b = U.Batch([path, path])
        b.set_pos(np.concatenate([z["pos"][0], z["pos"][3]]))
        b.set_thermostat([0.8, 0.9], np.array([3, 4], np.uint32))
        b.run(6, use_graph=graph, graph_rounds=3)
        res.append(b.get_pos())
        assert b.status() & 3 == 0
    assert np.all(np.isfinite(res[0]))
    assert np.abs(res[0] - res[1]).max() < 1e-3


def test_trans_cis_driver_run(transcis_config, tmp_path):
    """The upside driver runs the trans-cis configuration with its frames
    finite and frame 0 at the initial coordinates' potential."""
    import shutil
    import upside_gb300 as U
    from h5lite import H5File
    path, _ = transcis_config
    cfg = str(tmp_path / "tc.up")
    shutil.copyfile(path, cfg)
    rt = float(np.float32(3) * np.float32(0.009))
    U.upside_main(["--duration", repr(30 * rt), "--frame-interval", repr(10 * rt), "--temperature", "0.85",
                   "--seed", "4", cfg], verbose=False)
    f = H5File(cfg)
    pos, pot = f.read("/output/pos"), f.read("/output/potential")
    assert pos.shape[0] == 3 and np.all(np.isfinite(pos)) and np.all(np.isfinite(pot))
    eng = U.Upside(path, pos.shape[2])
    x0 = f.read("/input/pos")[:, :, 0]
    assert abs(eng.energy(x0) - pot[0, 0]) < 1e-4 * max(abs(pot[0, 0]), 1.0)
