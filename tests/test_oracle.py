"""The CPU oracle pinned against the reference's golden vectors.

Golden data (tests/golden, made by make_fixtures.py from the reference):
  * chig_frames.npz: the 20 frames logged by the reference's own example run
    (potential written by the reference binary at run time) and the reference
    engine's energy / derivative at each frame, recomputed here;
  * syn60/syn150: seeded synthetic ff_2.1 proteins, reference energy,
    derivative, per-node outputs and pair counts by type;
  * threefry_kat.txt: the reference's vendored Random123 Threefry outputs.

Tolerances.  The oracle restates the reference's affine eigen-solve (its
Householder + implicit QR with the 1e-5 relative off-diagonal stop and the
four-residue SIMD grouping, src/eig.cpp:57-275), so the truncation error of
the frames is the reference's own.  What remains is FP32 rounding: the
reference evaluates in FP32 with SSE approximate reciprocals (one Newton
step, src/Float4.h:201-238).  Energy: 1e-5 of the energy scale
sum_nodes |E_node| (the total is a sum of large, partly cancelling terms, so
|E| itself can be near zero).  Force: 1e-4 of max |F|, or twice the
reference's own distance from the FP64 instantiation where that is larger:
at steep steric walls (src/backbone_steric.cpp:18-30) FP32 positions of ~50 A
magnitude carry ~1e-4 relative force noise, and the reference shows it too
(8e-5 from FP64 on the 150-residue fixture's second frame).
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, quat_align

E_REF_TOL = 1e-5
F_REF_TOL = 1e-4


def f_ref_bound(ref_vs_fp64):
    """force bound against the reference given the reference's own relative
    max-force distance from the FP64 instantiation"""
    return max(F_REF_TOL, 2.0 * ref_vs_fp64)


def rel_e(a, b, scale=None):
    return abs(a - b) / max(1.0, abs(b) if scale is None else scale)


def energy_scale(o, path):
    """sum over potential nodes of |E_node| after an evaluation"""
    from h5lite import H5File
    tot = 0.0
    for nm in H5File(path).list("/input/potential"):
        n, w = o.dims(nm)
        if n == 1 and w == 1:
            tot += abs(float(o.node(nm)[0, 0]))
    return tot


def rel_f(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("fp64", [False, True])
def test_chig_golden_frames(built, fp64):
    import oracle_py
    z = np.load(os.path.join(GOLDEN, "chig_frames.npz"))
    path = os.path.join(GOLDEN, "chig.up")
    o = oracle_py.Oracle(path, 30, fp64=fp64)
    o64 = oracle_py.Oracle(path, 30, fp64=True)
    for k in range(len(z["pos"])):
        e, d = o.evaluate(z["pos"][k])
        sc = energy_scale(o, path)
        assert rel_e(e, z["logged_potential"][k], sc) < E_REF_TOL, k
        assert rel_e(e, z["ref_energy"][k], sc) < E_REF_TOL, k
        bound = f_ref_bound(rel_f(z["ref_deriv"][k], o64.evaluate(z["pos"][k])[1]))
        assert rel_f(d, z["ref_deriv"][k]) < bound, k


@pytest.mark.parametrize("n", [60, 150])
def test_synthetic_energy_forces(syn_configs, n):
    import oracle_py
    path, z = syn_configs[n]
    o64 = oracle_py.Oracle(path, z["pos"].shape[1], fp64=True)
    bounds = [f_ref_bound(rel_f(z["ref_deriv"][k], o64.evaluate(z["pos"][k])[1])) for k in range(len(z["pos"]))]
    for fp64 in (False, True):
        o = oracle_py.Oracle(path, z["pos"].shape[1], fp64=fp64)
        for k in range(len(z["pos"])):
            e, d = o.evaluate(z["pos"][k])
            assert rel_e(e, z["ref_energy"][k], energy_scale(o, path)) < E_REF_TOL
            assert rel_f(d, z["ref_deriv"][k]) < bounds[k], k


def test_synthetic_nodes(syn_configs):
    import oracle_py
    path, z = syn_configs[60]
    o = oracle_py.Oracle(path, z["pos"].shape[1])
    o.evaluate(z["pos"][0])
    for key in z.files:
        if not key.startswith("out/"):
            continue
        nm = key[4:]
        ref, got = z[key], o.node(nm)
        if nm == "affine_alignment":
            got = quat_align(got, ref)
        scale = max(np.abs(ref).max(), 1e-6)
        assert np.abs(got - ref).max() <= 1e-5 * scale + 1e-6, nm
        sref, sgot = z["sens/" + nm], o.node(nm, sens=True)
        # protein_hbond: at a score of exactly zero the reference adds no
        # sensitivity (src/hbond.cpp:624-626), a discontinuity that rounding
        # decides; it multiplies d(score)/dx ~ 0, so forces are unaffected
        if nm != "protein_hbond":
            assert np.abs(sgot - sref).max() <= 1e-4 * max(np.abs(sref).max(), 1e-6) + 1e-6, nm


def test_pair_counts_match_reference(syn_configs):
    import oracle_py
    for n in (60, 150):
        path, z = syn_configs[n]
        o = oracle_py.Oracle(path, z["pos"].shape[1])
        o.evaluate(z["pos"][0])
        for key in z.files:
            if key.startswith("count/"):
                nm = key[6:]
                got = o.value(nm, "count_edges_by_type", z[key].size)
                assert np.array_equal(got, z[key]), nm


GRAPH_NODES = ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond",
               "environment_coverage_sc", "environment_coverage_hb", "hb_environment_coverage_hn",
               "hb_environment_coverage_oc"]


def test_pair_lists_match_reference_lists(syn_configs):
    """The oracle's edge lists of every interaction graph equal the
    reference's own, pair for pair and in order (syn_graph_ref.npz: read out
    of the reference engine's InteractionGraph after each frame, frames
    evaluated in order on one engine so that pair caches carry over)."""
    import oracle_py
    g = np.load(os.path.join(GOLDEN, "syn_graph_ref.npz"))
    for n in (60, 150):
        path, z = syn_configs[n]
        o = oracle_py.Oracle(path, z["pos"].shape[1])
        for k in range(len(z["pos"])):
            o.evaluate(z["pos"][k])
            for nm in GRAPH_NODES:
                ref = g["edges%d/%d/%s" % (n, k, nm)].astype(np.int32)
                got = o.edges(nm)
                assert got.shape == ref.shape and np.array_equal(got, ref), (n, k, nm)


PARAM_DERIV_NODES = ("rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "nonlinear_coupling_environment")


@pytest.fixture(scope="module")
def env0_config(syn_configs, tmp_path_factory):
    """syn60 written with the nonlinear environment coupling (type 0)."""
    import config_gen
    _, z = syn_configs[60]
    path = str(tmp_path_factory.mktemp("env0") / "syn60_env0.up")
    config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0],
                            environment_potential_type=0)
    return path, z


def test_param_derivs_match_reference(env0_config):
    """The oracle's dE/d(parameters) against the reference's get_param_deriv
    (src/engine_c_library.cpp:94-110; src/interaction_graph.h:406-416 for
    the rotamer and coverage graphs, src/environment.cpp:788-833 for the
    nonlinear coupling): 1e-4 of the largest component (observed ~1e-5)."""
    import oracle_py
    g = np.load(os.path.join(GOLDEN, "syn_graph_ref.npz"))
    path, z = env0_config
    o = oracle_py.Oracle(path, z["pos"].shape[1])
    for k in (0, 1):
        o.evaluate(z["pos"][k])
        for nm in PARAM_DERIV_NODES:
            ref = g["pd/%d/%s" % (k, nm)]
            got = o.param_deriv(nm)
            assert got.shape == ref.shape, nm
            assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max(), (k, nm)


def test_threefry_known_answers(built):
    import oracle_py
    L = oracle_py._lib()
    L.ocpu_threefry4x32.argtypes = [ctypes.c_void_p] * 3
    n = 0
    for line in open(os.path.join(GOLDEN, "threefry_kat.txt")):
        if line.startswith("#"):
            continue
        seed, stream, step, atom, *want = map(int, line.split())
        c = np.array([step & 0xffffffff, step >> 32, atom, 0], np.uint32)
        k = np.array([seed, stream, 0, 0], np.uint32)
        out = np.zeros(4, np.uint32)
        L.ocpu_threefry4x32(c.ctypes.data, k.ctypes.data, out.ctypes.data)
        assert list(out) == want
        n += 1
    assert n >= 24


def test_fp32_matches_fp64(syn_configs):
    import oracle_py
    path, z = syn_configs[150]
    a = oracle_py.Oracle(path, z["pos"].shape[1])
    b = oracle_py.Oracle(path, z["pos"].shape[1], fp64=True)
    e1, d1 = a.evaluate(z["pos"][1])
    e2, d2 = b.evaluate(z["pos"][1])
    assert rel_e(e1, e2) < 1e-5
    assert rel_f(d1, d2) < 1e-4


def test_reference_engine_if_built(syn_configs):
    """Cross-check against the reference engine itself when it is built here."""
    ref = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libupside_ref.so")
    if not os.path.exists(ref):
        pytest.skip("reference engine not built on this host")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mf", os.path.join(GOLDEN, "make_fixtures.py"))
    mf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mf)
    L = mf.load_ref()
    path, z = syn_configs[60]
    r = mf.RefEngine(L, path, z["pos"].shape[1])
    e, d = r.eval(z["pos"][2])
    assert rel_e(e, z["ref_energy"][2]) < 1e-6
    assert rel_f(d, z["ref_deriv"][2]) < 1e-5


def test_reference_profile_if_built():
    """oracle/ref_profile.py, where the reference engine is built here: its
    profiling build and its own per-node timer report, which names the
    rotamer node's two timers."""
    import subprocess
    import sys
    ref = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libupside_ref.so")
    if not os.path.exists(ref):
        pytest.skip("reference engine not built on this host")
    script = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "ref_profile.py")
    out = subprocess.run([sys.executable, script, "--systems", "1", "--seconds", "0.2", "--relax", "2"],
                         capture_output=True, text=True, timeout=900, env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert out.returncode == 0, out.stderr[-2000:]
    assert "rotamer_solve" in out.stdout and "rotamer_fill" in out.stdout and "(total)" in out.stdout



@pytest.mark.parametrize("fp64", [False, True])
def test_trans_cis_golden_frames(transcis_config, fp64):
    """RamaMap2, SigmoidCoord, Add/Mean/Multiply and SigmoidEnergy/LEnergy
    (src/rama_map_pot.cpp:96-175, src/coord_map.cpp:609-675,
    src/coord_operator.cpp:15-351, src/sigmoid_energy.cpp) against the
    reference engine: energy, forces, and every trans-cis node's output and
    sensitivity at frames whose proline omegas sweep the barrier and switch
    segments."""
    import oracle_py
    path, z = transcis_config
    o = oracle_py.Oracle(path, z["pos"].shape[1], fp64=fp64)
    o64 = oracle_py.Oracle(path, z["pos"].shape[1], fp64=True)
    for k in range(len(z["pos"])):
        bound = f_ref_bound(rel_f(z["ref_deriv"][k], o64.evaluate(z["pos"][k])[1]))
        e, d = o.evaluate(z["pos"][k])
        assert rel_e(e, z["ref_energy"][k], energy_scale(o, path)) < E_REF_TOL, k
        assert rel_f(d, z["ref_deriv"][k]) < bound, k
        for key in z.files:
            if not key.startswith("out/"):
                continue
            nm = key[4:]
            for got, ref, tol in ((o.node(nm), z[key][k], 1e-5),
                                  # rama_coord's sensitivity also collects the
                                  # hbond energy's Rama derivative, where the
                                  # reference's FP32 rounding enters
                                  (o.node(nm, sens=True), z["sens/" + nm][k], 1e-4 if nm == "rama_coord" else 1e-5)):
                assert got.shape == ref.shape, nm
                assert np.abs(got - ref).max() <= tol * max(np.abs(ref).max(), 1.0), (k, nm)


def test_trans_cis_frames_cover_switches(transcis_config):
    """The fixture frames visit every barrier segment and both ramps of every
    switch, so each branch of the nodes is compared somewhere."""
    _, z = transcis_config
    om = z["out/Dihedral_OmegaTransCis"][..., 0]
    seg = np.floor((om + np.pi) / (np.pi / 2)).astype(int).clip(0, 3)
    assert set(seg.ravel().tolist()) == {0, 1, 2, 3}
    for nm in ("SigmoidCoord_trans1", "SigmoidCoord_trans2", "SigmoidCoord_cis1", "SigmoidCoord_cis2"):
        v = z["out/" + nm].ravel()
        assert ((v > 0) & (v < 1)).any(), nm
        assert (v == 0).any() and (v == 1).any(), nm
    # the empty row of the repeated-output Multiply is zero, and its repeated
    # row carries the reference's own-factor sensitivity
    assert np.all(z["out/Multiply_dup"][:, 2] == 0)


def test_config_trans_cis_and_fixed_rotamers(transcis_config):
    """Structure of the trans-cis writer (py/upside_config.py:571-673,
    848-993) and of fixed rotamers (:1077-1190)."""
    import config_gen
    import transcis_spec
    from h5lite import H5File
    path, _ = transcis_config
    f = H5File(path)
    seq = [s.decode() for s in f.read("/input/sequence")]
    assert seq[transcis_spec.CPR] == "CPR"
    pot = "/input/potential/"
    names = f.list("/input/potential")
    for nm in ("Dihedral_OmegaTransCis", "Add_lambda_trans", "Multiply_lambda_cis", "RamaMap2_trans",
               "RamaMap2_cis") + tuple("SigmoidEnergy_" + x for x in ("trans1", "cis0", "cis1", "trans0")):
        assert nm in names, nm
    om = f.read(pot + "Dihedral_OmegaTransCis/id")
    assert sorted(((om[:, 3] - 1) // 3).tolist()) == sorted(transcis_spec.PRO_TC)
    sp = f.read(pot + "Dihedral_omega/id")
    rid = (sp[:, 3] - 1) // 3
    assert not set(rid.tolist()) & set(transcis_spec.PRO_TC)
    eq = f.read(pot + "Spring_omega/equil_dist")
    assert np.all(eq[rid == transcis_spec.CPR] == 0.0) and np.all(eq[rid != transcis_spec.CPR] == np.pi)
    assert list(f.read(pot + "RamaMap2_cis/residue_id")) == list(transcis_spec.PRO_TC)
    assert not set(f.read(pot + "rama_map_pot/residue_id").tolist()) & set(transcis_spec.PRO_TC)
    # GLU 3 at chi1 -60 (class 2), chi2 170: the state with the most negative
    # wrapped chi2 offset; CYS 7 has one state at chi1 65; residue 12 (chi1
    # NaN) stays free
    fix = dict(f.read(pot + "placement_fixed_point_vector_only/fix_rotamer").tolist())
    assert fix == {3: 3, 7: 0}
    assert config_gen.fix_rotamer_states([(3, seq[3], 'A', 3, -60.0, 170.0)], seq) == {3: 3}
    ids = f.read(pot + "placement_fixed_point_vector_only/id_seq")
    res = f.read(pot + "placement_fixed_point_vector_only/affine_residue")
    n_rot = (ids >> config_gen.N_BIT_ROTAMER) & ((1 << config_gen.N_BIT_ROTAMER) - 1)
    for r in (3, 7):
        assert np.all(n_rot[res == r] == 1) and (res == r).sum() == 1
    assert (res == 12).sum() > 1
    with pytest.raises(ValueError):
        config_gen.read_trans_cis([(4, 0, 1.0, 0.5, 45.0)], seq)  # not a proline


@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("variant", ["flat", "curved"])
def test_membrane_golden_frames(membrane_configs, variant, fp64):
    """cb_membrane_potential, hb_membrane_potential and Const3D
    (src/membrane_potential.cpp:221-672, src/coord_const.cpp:107-179) against
    the reference engine, frames evaluated in order so the position-captured
    Const3D keeps the first frame's atoms."""
    import oracle_py
    paths, z = membrane_configs
    path = paths[variant]
    o = oracle_py.Oracle(path, z["pos"].shape[1], fp64=fp64)
    o64 = oracle_py.Oracle(path, z["pos"].shape[1], fp64=True)
    for k in range(len(z["pos"])):
        bound = f_ref_bound(rel_f(z[variant + "/ref_deriv"][k], o64.evaluate(z["pos"][k])[1]))
        e, d = o.evaluate(z["pos"][k])
        assert rel_e(e, z[variant + "/ref_energy"][k], energy_scale(o, path)) < E_REF_TOL, k
        assert rel_f(d, z[variant + "/ref_deriv"][k]) < bound, k
        for key in z.files:
            if not key.startswith(variant + "/out/"):
                continue
            nm = key.split("/", 2)[2]
            ref, sref = z[key][k], z[variant + "/sens/" + nm][k]
            assert np.abs(o.node(nm) - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1.0), (k, nm)
            # the CB placement's sensitivity sums the membrane force with the
            # reference's other consumers of the point (approximate rsqrt)
            tol = 1e-4 if nm == "placement_fixed_point_only_CB" else 1e-5
            assert np.abs(o.node(nm, sens=True) - sref).max() <= tol * max(np.abs(sref).max(), 1.0), (k, nm)


def test_membrane_frames_cover_slab(membrane_configs):
    """The frames put CB atoms inside the slab, in both head-group regions
    and outside, and the probe keeps frame 0's coordinates."""
    _, z = membrane_configs
    cbz = z["flat/out/placement_fixed_point_only_CB"][..., 2].ravel()
    for lo, hi in ((-np.inf, -20), (-20, -10), (-5, 5), (10, 20), (20, np.inf)):
        assert ((cbz > lo) & (cbz < hi)).any(), (lo, hi)
    assert np.array_equal(z["flat/out/Const3D_probe"][3], z["pos"][0][[5, 17]])


def test_config_membrane(membrane_configs):
    """Structure of the membrane writer (py/upside_config.py:1727-1835)."""
    import membrane_spec
    from h5lite import H5File
    paths, _ = membrane_configs
    f = H5File(paths["curved"])
    g = "/input/potential/cb_membrane_potential"
    assert [a.decode() for a in f.attr(g, "arguments")] == [
        "placement_fixed_point_only_CB", "environment_coverage_sc", "Const3D_curvature_center"]
    assert f.attr(g, "z_start") == -17.0 - 15.0 and f.attr(g, "z_scale") == 0.5
    cb = f.read(g + "/cb_index")
    assert len(cb) == membrane_spec.N_RES - 3 and not set(cb) & set(membrane_spec.EXCLUDE)
    h = "/input/potential/hb_membrane_potential"
    assert f.attr(h, "z_start") == -33.0 - 15.0 and f.attr(h, "use_curvature") == 1
    assert np.array_equal(f.read("/input/potential/Const3D_curvature_center/value"), [[0., 0., 60.]])


@pytest.mark.parametrize("variant", ["diffusion", "fast_curved", "included"])
@pytest.mark.parametrize("fp64", [False, True])
def test_surface_golden_frames(surface_configs, variant, fp64):
    """The surface node and the surface-dependent membrane terms
    (src/surface.cpp:54-696; cb_surf_membrane_potential,
    hb_surf_membrane_potential, membranelateral_potential,
    src/membrane_potential.cpp:674-1354) against the reference engine, the
    frames evaluated in order on one engine as the surface node keeps state.
    The surface fraction is a count of discrete decisions and matches
    exactly; the surface force columns are sums of per-turn forces and match
    to rounding."""
    import oracle_py
    paths, z = surface_configs
    path = paths[variant]
    o = oracle_py.Oracle(path, z["pos"].shape[1], fp64=fp64)
    o64 = oracle_py.Oracle(path, z["pos"].shape[1], fp64=True)
    for k in range(len(z["pos"])):
        bound = f_ref_bound(rel_f(z[variant + "/ref_deriv"][k], o64.evaluate(z["pos"][k])[1]))
        e, d = o.evaluate(z["pos"][k])
        assert rel_e(e, z[variant + "/ref_energy"][k], energy_scale(o, path)) < E_REF_TOL, k
        assert rel_f(d, z[variant + "/ref_deriv"][k]) < bound, k
        ref = z[variant + "/out/surface"][k]
        s = o.node("surface")
        assert np.array_equal(s[:, 0], ref[:, 0]), k
        assert np.abs(s[:, 1:] - ref[:, 1:]).max() <= 1e-5 * np.abs(ref[:, 1:]).max(), k
        cat = z[variant + "/out/cat_pos_bb_cb"][k]
        assert np.abs(o.node("cat_pos_bb_cb") - cat).max() <= 1e-5 * np.abs(cat).max(), k
        for nm in ("placement_fixed_point_only_CB", "protein_hbond", "environment_coverage_sc"):
            sref, got = z[variant + "/sens/" + nm][k], o.node(nm, sens=True)
            if nm == "protein_hbond":
                # the probability column also holds hbond_energy's residue
                # energy wherever the residue's summed hbond probability is
                # not exactly 0 (src/hbond.cpp:618-619); for these unbonded
                # coils that sum is 0 or a rounding residue of 1 - exp(-x)
                # (1e-14 in FP64), so only the geometric columns are compared
                sref, got = sref[:, :6], got[:, :6]
            assert np.abs(got - sref).max() <= 1e-4 * max(np.abs(sref).max(), 1.0), (k, nm)


def test_surface_fixture_exercises_terms(surface_configs):
    """The frames give surface residues and residues inside and outside the
    slab, both surface methods, and lateral forces of the order of the CB
    membrane forces."""
    _, z = surface_configs
    for var in ("diffusion", "fast_curved", "included"):
        frac = z[var + "/out/surface"][..., 0]
        assert (frac > 0).sum() > 100 and (frac == 0).sum() > 20 and ((frac > 0) & (frac < 1)).any(), var
        assert (np.abs(z[var + "/out/surface"][..., 1:]) > 0).mean() > 0.3, var
    cbz = z["diffusion/out/cat_pos_bb_cb"][:, 180:, 2].ravel()
    assert (np.abs(cbz) < 15).any() and (np.abs(cbz) > 15).any()
    inc = z["included/out/surface"][..., 0]
    assert (inc[:, :5] == 0).all() and (inc[:, 50:] == 0).all()


def test_config_surface(surface_configs):
    """Structure of the surface, channel and lateral writers
    (py/upside_config.py:1544-1602, 1837-2021)."""
    import config_gen
    from h5lite import H5File
    paths, _ = surface_configs
    f = H5File(paths["included"])
    g = "/input/potential/surface"
    assert f.attr(g, "method_type") == 1 and f.attr(g, "n_rotation") == 20 and f.attr(g, "exclusion") == 1
    assert f.attr(g, "n_smallgridz") == 2 and f.attr(g, "atom_radius") == np.float64(1.6)
    assert np.array_equal(f.read(g + "/index_cb"), np.arange(60) + 180)
    aux = f.read(g + "/auxiliary_point")
    assert aux.shape == (18, 2) and np.allclose(np.hypot(aux[:, 0], aux[:, 1])[:12:2], 1.0, atol=1e-3)
    assert np.array_equal(f.read(g + "/included_list"), np.arange(5, 50))
    cb = "/input/potential/cb_surf_membrane_potential"
    assert [a.decode() for a in f.attr(cb, "arguments")] == [
        "placement_fixed_point_only_CB", "environment_coverage_sc", "surface", "Const3D_curvature_center"]
    assert f.read(cb + "/coeff_inner").shape == (20, 18)
    hb = "/input/potential/hb_surf_membrane_potential"
    n = len(f.read(hb + "/hb_index"))
    assert len(f.read(hb + "/hb_type")) == n and len(f.read(hb + "/hb_res")) == n
    lat = "/input/potential/membranelateral_potential"
    pp = f.read(lat + "/params")
    assert f.attr(lat, "n_knot") == len(pp) == 63 + 2 and f.attr(lat, "min_z") == -32.0
    # the clamped spline through the sampled profile reproduces its samples
    vals = config_gen.clamped_spline_solve(np.linspace(0., 5., 7) ** 2)
    b = (vals[:-2] + 4 * vals[1:-1] + vals[2:]) / 6
    assert np.allclose(b, np.linspace(0., 5., 7) ** 2, atol=1e-4)
    assert vals[0] == vals[2] and vals[-1] == vals[-3]
