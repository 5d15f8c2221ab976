"""The surface node and the surface-dependent membrane terms on the GPU:
surface (src/surface.cpp:54-696), cb_surf_membrane_potential,
hb_surf_membrane_potential and membranelateral_potential
(src/membrane_potential.cpp:674-1354), in the fixture of
golden/surface_spec.py (lipid-diffusion surface, fast surface on a curved
bilayer, surface over an included residue list).

The surface fraction is a count of discrete voxel decisions: it must equal
the reference's exactly.  The surface force columns are float sums of
per-turn forces: 1e-5 of their largest magnitude.  Energies and forces as
in test_gpu_membrane.py: 1e-5 of sum |E_node| and 1e-4 of max |F| against
the oracles, the reference-facing bounds of conftest against the reference.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from conftest import E_REF_TOL as E_REF, ref_force_bound  # noqa: E402

E_ORC, F_ORC = 1e-5, 1e-4
SENS = ("placement_fixed_point_only_CB", "protein_hbond", "environment_coverage_sc")


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


def check_surface(s, ref, what):
    assert np.array_equal(s[:, 0], ref[:, 0]), (what, np.nonzero(s[:, 0] != ref[:, 0]))
    scale = max(np.abs(ref[:, 1:]).max(), 1e-12)
    assert np.abs(s[:, 1:] - ref[:, 1:]).max() <= 1e-5 * scale, what


@pytest.mark.parametrize("variant", ["diffusion", "fast_curved", "included"])
def test_surface_frames(surface_configs, variant):
    """Frames in order on one engine (the surface node keeps state between
    evaluations): energy and forces against the reference and both oracles,
    the surface output and the sensitivities the membrane terms write against
    the reference's."""
    import oracle_py
    import upside_gb300 as U
    paths, z = surface_configs
    path = paths[variant]
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o32, o64 = oracle_py.Oracle(path, na), oracle_py.Oracle(path, na, fp64=True)
    for k in range(len(z["pos"])):
        x = z["pos"][k]
        e, d = eng.energy(x), eng.deriv(x)
        sc = energy_scale(eng, path)
        ref_d = z[variant + "/ref_deriv"][k]
        assert abs(e - z[variant + "/ref_energy"][k]) < E_REF * sc, k
        assert rel_f(d, ref_d) < ref_force_bound(ref_d, o64.evaluate(x)[1]), k
        for o in (o32, o64):
            eo, do = o.evaluate(x)
            assert abs(e - eo) < E_ORC * sc, k
            assert rel_f(d, do) < F_ORC, k
        s = eng.get_output("surface")
        check_surface(s, z[variant + "/out/surface"][k], (variant, k, "reference"))
        check_surface(s, o32.node("surface"), (variant, k, "oracle"))
        for nm in SENS:
            ref = z["%s/sens/%s" % (variant, nm)][k]
            tol = 1e-4 * max(np.abs(ref).max(), 1.0)
            got, orc = eng.get_sens(nm), o32.node(nm, sens=True)
            if nm == "protein_hbond":
                # the probability column also holds hbond_energy's residue
                # energy wherever the residue's summed hbond probability is
                # not exactly 0 (src/hbond.cpp:618-619); for these unbonded
                # coils that sum is 0 or a rounding residue of 1 - exp(-x),
                # so only the geometric columns are compared
                got, ref, orc = got[:, :6], ref[:, :6], orc[:, :6]
            assert np.abs(got - ref).max() <= tol, (k, nm)
            assert np.abs(got - orc).max() <= tol, (k, nm)


def test_surface_history(surface_configs):
    """The node's output depends on the evaluations before it as the
    reference's does: a residue that leaves the slab keeps its last force,
    and TM list entries left from earlier evaluations repeat the final
    division.  Frame 3 evaluated first on a fresh engine equals the oracle's
    fresh evaluation, and differs from frame 3 after frames 0-2."""
    import oracle_py
    import upside_gb300 as U
    paths, z = surface_configs
    path = paths["diffusion"]
    na = z["pos"].shape[1]
    eng = U.Upside(path, na)
    o = oracle_py.Oracle(path, na)
    eng.deriv(z["pos"][3])
    o.evaluate(z["pos"][3])
    fresh = eng.get_output("surface")
    check_surface(fresh, o.node("surface"), "fresh")
    after = z["diffusion/out/surface"][3]
    assert np.array_equal(fresh[:, 0], after[:, 0])
    assert np.abs(fresh[:, 1:] - after[:, 1:]).max() > 1e-3 * np.abs(after[:, 1:]).max()


def test_surface_batch(surface_configs, tmp_path):
    """Systems of two lengths in one batch equal single-system engines,
    surface outputs included; different surface methods do not share a
    batch (different attributes)."""
    import surface_spec
    import upside_gb300 as U
    paths, z = surface_configs
    p64 = str(tmp_path / "s64.up")
    surface_spec.write(p64, "diffusion", n_res=64, seed=31)
    x64 = surface_spec.frames(seed=9, n_res=64)
    sets = [(p64, x64[1]), (paths["diffusion"], z["pos"][2]), (p64, x64[4])]
    b = U.Batch([p for p, _ in sets])
    b.set_pos(np.concatenate([x for _, x in sets]))
    e, d = b.evaluate()
    surf = b.node_output("surface")
    lo = rlo = 0
    for k, (p, x) in enumerate(sets):
        s = U.Upside(p, len(x))
        es, ds = s.energy(x), s.deriv(x)
        assert abs(e[k] - es) < 1e-5 * energy_scale(s, p), k
        assert rel_f(d[lo:lo + len(x)], ds) < 1e-5, k
        n_res = len(x) // 3
        check_surface(surf[rlo:rlo + n_res], s.get_output("surface"), ("batch", k))
        lo += len(x)
        rlo += n_res
    with pytest.raises(RuntimeError):
        U.Batch([paths["diffusion"], paths["fast_curved"]])


def test_surface_dynamics(surface_configs):
    """Integration rounds with the surface terms: graph replays and eager
    rounds agree, and the trajectory stays finite."""
    import upside_gb300 as U
    paths, z = surface_configs
    res = []
    for graph in (False, True):
        b = U.Batch([paths["diffusion"], paths["diffusion"]])
        b.set_pos(np.concatenate([z["pos"][0], z["pos"][4]]))
        b.set_thermostat([0.8, 0.9], np.array([5, 6], np.uint32))
        b.run(6, use_graph=graph, graph_rounds=3)
        res.append(b.get_pos())
        assert b.status() & 3 == 0
        assert np.all(np.isfinite(b.node_output("surface")))
    assert np.all(np.isfinite(res[0]))
    assert np.abs(res[0] - res[1]).max() < 1e-3


def test_surface_large_grid(surface_configs):
    """A frame spread over more voxels than the small tier's grid (64 per
    axis) goes through the large tier: the surface output still equals the
    oracle's, and turns of both tiers mix in one evaluation."""
    import oracle_py
    import upside_gb300 as U
    paths, z = surface_configs
    path = paths["diffusion"]
    for f in (4.0, 7.0, 12.0):
        x = z["pos"][0].copy()
        x[:, :2] *= f
        eng = U.Upside(path, len(x))
        o = oracle_py.Oracle(path, len(x))
        eng.deriv(x)
        o.evaluate(x)
        check_surface(eng.get_output("surface"), o.node("surface"), ("stretched", f))
        assert (eng.get_output("surface")[:, 0] > 0).sum() > 10


def test_surface_grid_capacity_error(surface_configs, capfd):
    """TM residues spread over more voxels than the kernel's grid holds end
    the evaluation with an error naming the surface node (the kernel skips
    the turn and sets a status bit; no out-of-grid access).  The C ABI
    reports the failure by its return code and prints the reason, as the
    reference's library does."""
    import upside_gb300 as U
    paths, z = surface_configs
    x = z["pos"][0].copy()
    x[:, 0] *= 60.0
    eng = U.Upside(paths["diffusion"], len(x))
    with pytest.raises(RuntimeError):
        eng.deriv(x)
    assert "surface" in capfd.readouterr().err
    # the engine stays usable
    eng.deriv(z["pos"][0])
    assert np.isfinite(eng.get_output("surface")).all()
