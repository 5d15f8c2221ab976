"""GPU engine parity: the sm_103a kernels through the C ABI against the golden
fixtures (reference engine), the FP32 oracle and the FP64 oracle.

Tolerances (see test_oracle.py for why the reference-facing ones are looser):
  vs FP32 / FP64 oracle : energy 1e-5 of sum |E_node|, max force 1e-4 of max |F|
  vs reference engine   : energy 1e-5 of sum |E_node|, max force 1e-4 of max |F|
                          (or twice the reference's own distance from FP64
                          where that is larger; conftest.ref_force_bound)
  pair lists            : bit-exact (same pairs, same order) vs the oracle, and
                          per-type pair counts equal to the reference's
"""
import os

import numpy as np
import pytest

from conftest import E_REF_TOL as E_REF, GOLDEN, quat_align, ref_force_bound

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


def test_chig_reference_frames(built):
    import oracle_py
    import upside_gb300 as U
    z = np.load(os.path.join(GOLDEN, "chig_frames.npz"))
    path = os.path.join(GOLDEN, "chig.up")
    eng = U.Upside(path, 30)
    o32 = oracle_py.Oracle(path, 30)
    o64 = oracle_py.Oracle(path, 30, fp64=True)
    for k in range(len(z["pos"])):
        x = z["pos"][k]
        e, d = eng.energy(x), eng.deriv(x)
        sc = energy_scale(eng, path)
        e32, d32 = o32.evaluate(x)
        e64, d64 = o64.evaluate(x)
        assert abs(e - z["ref_energy"][k]) < E_REF * sc, k
        assert abs(e - z["logged_potential"][k]) < E_REF * sc, k
        assert rel_f(d, z["ref_deriv"][k]) < ref_force_bound(z["ref_deriv"][k], d64), k
        assert abs(e - e32) < E_ORC * sc, k
        assert rel_f(d, d32) < F_ORC, k
        assert abs(e - e64) < E_ORC * sc, k
        assert rel_f(d, d64) < F_ORC, k


@pytest.mark.parametrize("n", [60, 150])
def test_synthetic_energy_forces(syn_configs, n):
    import oracle_py
    import upside_gb300 as U
    path, z = syn_configs[n]
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o32 = oracle_py.Oracle(path, na)
    o64 = oracle_py.Oracle(path, na, fp64=True)
    for k in range(len(z["pos"])):
        x = z["pos"][k]
        e, d = eng.energy(x), eng.deriv(x)
        sc = energy_scale(eng, path)
        e32, d32 = o32.evaluate(x)
        e64, d64 = o64.evaluate(x)
        assert abs(e - z["ref_energy"][k]) < E_REF * sc
        assert rel_f(d, z["ref_deriv"][k]) < ref_force_bound(z["ref_deriv"][k], d64), k
        assert abs(e - e32) < E_ORC * sc
        assert rel_f(d, d32) < F_ORC
        assert abs(e - e64) < E_ORC * sc
        assert rel_f(d, d64) < F_ORC


def test_nodes_vs_oracle(syn_configs):
    import oracle_py
    import upside_gb300 as U
    from h5lite import H5File
    path, z = syn_configs[150]
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o = oracle_py.Oracle(path, na)
    eng.energy(z["pos"][1])
    o.evaluate(z["pos"][1])
    for nm in H5File(path).list("/input/potential"):
        a, b = eng.get_output(nm), o.node(nm)
        if nm == "affine_alignment":
            a = quat_align(a, b)
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1.0), nm
        sa, sb = eng.get_sens(nm), o.node(nm, sens=True)
        if nm == "protein_hbond":
            # the hbond energy adds to the sensitivity of a score only when the
            # residue's score sum is non-zero (src/hbond.cpp:624-626); scores of
            # ~1e-9 are zero in one FP32 evaluation order and not in another.
            # That sensitivity multiplies d(score)/dx ~ 0, so forces agree.
            tiny = b[:, 6] < 1e-6
            sa, sb = sa.copy(), sb.copy()
            sa[tiny, 6] = sb[tiny, 6] = 0.0
        assert np.abs(sa - sb).max() <= 1e-3 * max(np.abs(sb).max(), 1.0), nm


def test_nodes_vs_reference(syn_configs):
    """Every node's output and sensitivity on the GPU against the reference
    engine's own (syn60 frame 0 fixture): outputs 1e-5 and sensitivities 1e-4
    of the node's largest entry."""
    import upside_gb300 as U
    path, z = syn_configs[60]
    eng = U.Upside(path, z["pos"].shape[1])
    eng.energy(z["pos"][0])
    for key in z.files:
        if not key.startswith("out/"):
            continue
        nm = key[4:]
        ref, got = z[key], eng.get_output(nm)
        if nm == "affine_alignment":
            got = quat_align(got, ref)
        assert np.abs(got - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1e-6) + 1e-6, nm
        if nm == "protein_hbond":  # zero-score sensitivity, see test_nodes_vs_oracle
            continue
        sref, sgot = z["sens/" + nm], eng.get_sens(nm)
        assert np.abs(sgot - sref).max() <= 1e-4 * max(np.abs(sref).max(), 1e-6) + 1e-6, nm


def _set_sizes(path, node):
    from h5lite import H5File
    f = H5File(path)
    g = "/input/potential/" + node
    if node == "rotamer":
        n = f.read(g + "/pair_interaction/index").shape[0]
        return n, n
    return f.read(g + "/index1").shape[0], f.read(g + "/index2").shape[0]


def test_pair_lists_bit_exact(syn_configs):
    """Batched pair search reproduces the oracle's edge lists exactly, per system."""
    import oracle_py
    import upside_gb300 as U
    (p60, z60), (p150, z150) = syn_configs[60], syn_configs[150]
    b = U.Batch([p60, p150])
    b.set_pos(np.concatenate([z60["pos"][0], z150["pos"][0]]))
    b.evaluate()
    o60 = oracle_py.Oracle(p60, z60["pos"].shape[1])
    o150 = oracle_py.Oracle(p150, z150["pos"].shape[1])
    o60.evaluate(z60["pos"][0])
    o150.evaluate(z150["pos"][0])
    for node in ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond",
                 "environment_coverage_sc", "environment_coverage_hb", "hb_environment_coverage_hn",
                 "hb_environment_coverage_oc"]:
        ge = b.node_edges(node)
        e0, e1 = o60.edges(node), o150.edges(node)
        n1, n2 = _set_sizes(p60, node)
        assert len(ge) == len(e0) + len(e1), node
        assert np.array_equal(ge[:len(e0)], e0), node
        assert np.array_equal(ge[len(e0):] - np.array([n1, n2]), e1), node


GRAPH_NODES = ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond",
               "environment_coverage_sc", "environment_coverage_hb", "hb_environment_coverage_hn",
               "hb_environment_coverage_oc"]


def test_pair_lists_bit_exact_vs_reference(syn_configs):
    """Every interaction graph's edge list on the GPU equals the reference
    engine's own, pair for pair and in order (syn_graph_ref.npz: read out of
    the reference's InteractionGraph, src/interaction_graph.h:51-258), with
    the fixture's frames evaluated in order on one engine so that the pair
    caches carry over as they do in the reference."""
    import upside_gb300 as U
    g = np.load(os.path.join(GOLDEN, "syn_graph_ref.npz"))
    for n in (60, 150):
        path, z = syn_configs[n]
        b = U.Batch([path])
        for k in range(len(z["pos"])):
            b.set_pos(z["pos"][k])
            b.evaluate()
            for nm in GRAPH_NODES:
                ref = g["edges%d/%d/%s" % (n, k, nm)].astype(np.int32)
                got = b.node_edges(nm)
                assert got.shape == ref.shape and np.array_equal(got, ref), (n, k, nm)


def test_param_derivs_vs_reference(syn_configs, tmp_path):
    """dE/d(parameters) of the GPU adjoint against the reference's own
    get_param_deriv (src/engine_c_library.cpp:94-110): rotamer pair splines,
    both hbond coverage graphs and the nonlinear environment coupling, at two
    frames: 1e-3 of the largest component."""
    import config_gen
    import upside_gb300 as U
    g = np.load(os.path.join(GOLDEN, "syn_graph_ref.npz"))
    _, z = syn_configs[60]
    path = str(tmp_path / "syn60_env0.up")
    config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0],
                            environment_potential_type=0)
    b = U.Batch([path])
    for k in (0, 1):
        b.set_pos(z["pos"][k])
        b.evaluate()
        for nm in ("rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "nonlinear_coupling_environment"):
            ref = g["pd/%d/%s" % (k, nm)]
            got = b.param_deriv(nm, ref.shape)
            err = np.abs(got - ref).max() / np.abs(ref).max()
            print("param deriv %s frame %d: %.2e of max" % (nm, k, err))
            assert err <= 1e-3, (k, nm, err)


def test_pair_counts_vs_reference(syn_configs):
    import upside_gb300 as U
    for n in (60, 150):
        path, z = syn_configs[n]
        eng = U.Upside(path, z["pos"].shape[1])
        eng.energy(z["pos"][0])
        for key in z.files:
            if key.startswith("count/"):
                nm = key[6:]
                got = eng.get_value_by_name(z[key].size, nm, "count_edges_by_type")
                assert np.array_equal(got, z[key]), nm


def test_batch_equals_single(syn_configs):
    import upside_gb300 as U
    (p60, z60), (p150, z150) = syn_configs[60], syn_configs[150]
    b = U.Batch([p150, p60, p150])
    x = np.concatenate([z150["pos"][1], z60["pos"][1], z150["pos"][0]])
    b.set_pos(x)
    e, d = b.evaluate()
    s150 = U.Upside(p150, 450)
    s60 = U.Upside(p60, 180)
    for k, (eng, xx, lo) in enumerate([(s150, z150["pos"][1], 0), (s60, z60["pos"][1], 450),
                                       (s150, z150["pos"][0], 630)]):
        es, ds = eng.energy(xx), eng.deriv(xx)
        assert abs(e[k] - es) < 1e-5 * energy_scale(eng, eng.config)
        assert rel_f(d[lo:lo + len(xx)], ds) < 1e-5


def test_param_derivatives_vs_oracle(syn_configs):
    import oracle_py
    import upside_gb300 as U
    path, z = syn_configs[60]
    eng = U.Upside(path, 180)
    o = oracle_py.Oracle(path, 180)
    eng.energy(z["pos"][0])
    o.evaluate(z["pos"][0])
    for nm, shape in [("rotamer", (20, 20, 54)), ("hbond_coverage", (8, 20, 50)),
                      ("hbond_coverage_hydrophobe", (12, 20, 50))]:
        g = eng.get_param_deriv(shape, nm).ravel()
        c = o.param_deriv(nm)
        assert np.abs(g - c).max() <= 1e-3 * max(np.abs(c).max(), 1.0), nm


def test_error_codes(built, tmp_path):
    import upside_gb300 as U
    with pytest.raises(RuntimeError):
        U.Upside(str(tmp_path / "missing.up"), 30)
    eng = U.Upside(os.path.join(GOLDEN, "chig.up"), 30)
    with pytest.raises(RuntimeError):
        eng.get_output("no_such_node")
    with pytest.raises(RuntimeError):
        eng.set_param(np.zeros(3), "rotamer")
    with pytest.raises(RuntimeError):
        eng.get_value_by_name(5, "rotamer", "count_edges_by_type")
    # the engine stays usable after the errors
    z = np.load(os.path.join(GOLDEN, "chig_frames.npz"))
    assert abs(eng.energy(z["pos"][0]) - z["ref_energy"][0]) < 1e-3


def test_pair_cache_transparent(syn_configs):
    """After many integration rounds (candidate caches reused and partly
    rebuilt), every edge list equals the one a fresh engine finds from scratch
    at the same coordinates, and so do energies and forces."""
    import upside_gb300 as U
    (p60, z60), (p150, z150) = syn_configs[60], syn_configs[150]
    b = U.Batch([p60, p150])
    b.set_pos(np.concatenate([z60["pos"][0], z150["pos"][0]]))
    b.set_thermostat([0.85, 0.9], np.array([3, 4], np.uint32))
    b.run(60, use_graph=True, graph_rounds=10)
    x = b.get_pos()
    e_run, d_run = b.evaluate()
    fresh = U.Batch([p60, p150])
    fresh.set_pos(x)
    e_new, d_new = fresh.evaluate()
    for node in ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond",
                 "environment_coverage_sc", "environment_coverage_hb", "hb_environment_coverage_hn",
                 "hb_environment_coverage_oc"]:
        assert np.array_equal(b.node_edges(node), fresh.node_edges(node)), node
    assert np.abs(e_run - e_new).max() < 1e-4 * max(1.0, np.abs(e_new).max())
    assert rel_f(d_run, d_new) < 1e-4


def test_bp_shared_layout_fallback(syn_configs):
    """The BP solve's compact shared layout falls back to global-memory
    messages and beliefs for a cluster whose entries overflow the reserved
    message slots: with the slots capped at 16 (every cluster overflows) the
    energy and forces still match the oracle, and match the shared-memory
    solve of the same coordinates."""
    import json
    import subprocess
    import sys
    import oracle_py
    import upside_gb300 as U
    from conftest import ROOT
    path, z = syn_configs[150]
    x = z["pos"][1]
    na = x.shape[0]
    np.save(os.path.join(os.path.dirname(path), "x150.npy"), x)
    code = ("import sys, json, numpy as np; sys.path.insert(0, %r); import upside_gb300 as U; "
            "e = U.Upside(%r, %d); x = np.load(%r); "
            "print(json.dumps([e.energy(x), e.deriv(x).tolist()]))"
            % (os.path.join(ROOT, "upside2-md_gb300"), path, na, os.path.join(os.path.dirname(path), "x150.npy")))
    env = dict(os.environ, UPSIDE_GB300_BP_MSG_SLOTS="16")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    e_fb, d_fb = json.loads(out.stdout.strip().splitlines()[-1])
    d_fb = np.array(d_fb, np.float32)
    eng = U.Upside(path, na)
    e_sh, d_sh = eng.energy(x), eng.deriv(x)
    e64, d64 = oracle_py.Oracle(path, na, fp64=True).evaluate(x)
    sc = energy_scale(eng, path)
    assert abs(e_fb - e64) < E_ORC * sc and abs(e_sh - e64) < E_ORC * sc
    assert rel_f(d_fb, d64) < F_ORC and rel_f(d_sh, d64) < F_ORC
    assert abs(e_fb - e_sh) < E_ORC * sc and rel_f(d_fb, d_sh) < F_ORC
