"""Multistep integrator (the reference's integration_cycle with inner_step,
src/deriv_engine.cpp:180-237, 262-292, 333-351).

The forces of each integrator level are pinned against the oracle evaluated
on a copy of the configuration that keeps only that level's potentials: the
gradient of the slow (level 1) potentials is what the reference's
compute(DerivMode, 1) leaves in the position sensitivity, and likewise for
level 0.  One multistep round is then checked against those oracle forces
applied in the reference's order: a slow kick of inner_step dt, then
inner_step fast stages.
"""
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = np.float32(0.009)


def _level_config(src, dst, keep_level):
    """Copy of src without the potential nodes of the other level (the nodes
    no other node takes as an argument)."""
    import h5lite
    from h5lite import H5File
    f = H5File(src)
    names = f.list("/input/potential")
    used = set()
    for nm in names:
        used |= {a.decode() for a in f.attr("/input/potential/" + nm, "arguments")}
    skip = []
    for nm in names:
        if nm in used:
            continue
        # a potential without the attribute, or out of range, is fast (0)
        lvl = int(f.attrs("/input/potential/" + nm).get("integrator_level", 2))
        lvl = 0 if lvl not in (0, 1) else lvl
        if lvl != keep_level:
            skip.append("/input/potential/" + nm)
    h5lite.copy_file(src, dst, skip)
    return skip


@pytest.fixture(scope="module")
def level_setup(syn_configs, tmp_path_factory):
    import oracle_py
    src, z = syn_configs[60]
    d = tmp_path_factory.mktemp("levels")
    cfgs = {}
    for lvl in (0, 1):
        p = str(d / ("level%d.up" % lvl))
        skipped = _level_config(src, p, lvl)
        assert skipped, lvl  # the ff_2.1 config has potentials on both levels
        cfgs[lvl] = oracle_py.Oracle(p, 180)
    return src, z, cfgs


def test_level_forces_match_oracle(built, level_setup):
    import upside_gb300 as U
    src, z, orc = level_setup
    x = z["pos"][1].astype(np.float32)
    b = U.Batch([src])
    b.set_pos(x)
    _, total = b.evaluate()
    f = {lvl: b.level_forces(lvl) for lvl in (0, 1)}
    scale = np.abs(total).max()
    assert np.abs(f[0] + f[1] - total).max() < 1e-4 * scale
    for lvl in (0, 1):
        _, ref = orc[lvl].evaluate(x)
        assert np.abs(f[lvl] - ref).max() < 1e-4 * max(np.abs(ref).max(), 1.0), lvl
        assert np.abs(ref).max() > 0.0, lvl


@pytest.mark.parametrize("inner", [3, 5])
def test_multistep_round_matches_oracle_forces(built, level_setup, inner):
    """Temperature 0 makes the thermostat a deterministic scaling of the
    momenta by exp(-inner dt / timescale)."""
    import upside_gb300 as U
    src, z, orc = level_setup
    x0 = z["pos"][1].astype(np.float32)
    rng = np.random.RandomState(4)
    p0 = (0.3 * rng.randn(*x0.shape)).astype(np.float32)
    b = U.Batch([src])
    b.set_integrator(True, inner)
    b.set_pos(x0)
    b.set_mom(p0)
    b.set_thermostat([0.0], np.array([3], np.uint32))
    b.run(1, dt=float(DT), timescale=5.0, use_graph=False)
    xg, pg = b.get_pos(), b.get_mom()
    ms = np.float32(np.exp(np.float32(-(np.float32(inner) * DT)) / np.float32(5.0)))
    x, p = x0.copy(), (ms * p0).astype(np.float32)
    _, f1 = orc[1].evaluate(x)
    p = (p - np.float32(inner) * DT * f1).astype(np.float32)
    for _ in range(inner):
        _, f0 = orc[0].evaluate(x)
        p = (p - DT * f0).astype(np.float32)
        x = (x + DT * p).astype(np.float32)
    assert np.abs(pg - p).max() < 2e-4 * np.abs(p).max(), np.abs(pg - p).max()
    assert np.abs(xg - x).max() < 3e-5, np.abs(xg - x).max()


def test_multistep_graph_replay_matches_eager(built, syn_configs):
    import upside_gb300 as U
    (p60, z60), (p150, z150) = syn_configs[60], syn_configs[150]
    x = np.concatenate([z60["pos"][0], z150["pos"][0]])
    res = []
    for graph in (False, True):
        b = U.Batch([p60, p150])
        b.set_integrator(True, 4)
        b.set_pos(x)
        b.set_thermostat([0.85, 0.9], np.array([1, 2], np.uint32))
        b.run(4, use_graph=graph, graph_rounds=2)
        res.append(b.get_pos())
        assert b.status() & 3 == 0
    assert np.abs(res[0] - res[1]).max() < 1e-3


def test_driver_multistep(built, syn_configs, tmp_path):
    """--integrator mv --inner-step 4: a round is 4 dt of simulation time, so
    the frames, the logged times and the thermostat follow it."""
    import upside_gb300 as U
    from h5lite import H5File
    src, _ = syn_configs[60]
    cfg = str(tmp_path / "a.up")
    shutil.copyfile(src, cfg)
    rt = float(np.float32(4) * DT)
    out = str(tmp_path / "mv.h5")
    U.upside_main(["--duration", repr(40 * rt), "--frame-interval", repr(10 * rt), "--temperature", "0.9",
                   "--integrator", "mv", "--inner-step", "4", "--output", out, cfg], verbose=False)
    f = H5File(out)
    t = f.read("/output/time")
    assert t.shape == (4,)
    assert np.array_equal(t, [np.float32(np.float32(4) * DT) * np.float32(10 * k) for k in range(4)])
    kin = f.read("/output/kinetic")[:, 0]
    assert np.all(np.isfinite(f.read("/output/pos"))) and np.all(kin > 0) and kin.max() < 10.0
    assert os.path.exists(out)
