"""The upside driver (upside_main) on the GPU.

Pins, in order of strength:
  * the reference's own logged run of its example (outputs/simple_test/
    chig.run.up, committed as tests/golden/chig_run_output.npz): frame 0 is
    logged before any integration step, so the same command line must give
    the same positions, potential, kinetic energy (the thermostat's first
    draw from zero momenta), time, temperature, hbond and node-level arrays
    (rotamer free energy, average energy, entropy and one-body energies per
    residue, Rama and sigmoid-coupling energies per residue, bad BP solves),
    and the arrays must have the reference's names, shapes and types;
  * the oracle integrating the same schedule (recentre + log every round,
    thermalise once at the start, thermostat each round) for the first frames;
  * replica exchange bookkeeping, restarts from logged momenta, annealing.
"""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

DT = np.float32(0.009)
RT = float(np.float32(3) * DT)  # one round of simulation time, as the driver forms it


def _out(path):
    from h5lite import H5File
    f = H5File(path)
    return {k: f.read("/output/" + k) for k in f.list("/output")}, f


def test_chig_frame0_matches_reference_run(built, tmp_path):
    import upside_gb300 as U
    ref = np.load(os.path.join(GOLDEN, "chig_run_output.npz"))
    # the reference ran --duration 1000 --frame-interval 50 --temperature 0.8
    # --seed 1 --disable-recentering; a shorter duration keeps two frames
    assert b"--frame-interval 50 --temperature 0.8 --seed 1 --disable-recentering" in bytes(ref["invocation"])
    cfg = str(tmp_path / "chig.up")
    shutil.copyfile(os.path.join(GOLDEN, "chig.up"), cfg)
    U.upside_main(["--duration", "60", "--frame-interval", "50", "--temperature", "0.8", "--seed", "1",
                   "--disable-recentering", cfg], verbose=False)
    out, f = _out(cfg)
    assert f.exists("/input/potential/rotamer")  # written in place, input kept
    assert "--seed 1" in f.attr("/output", "invocation").decode()
    for k in ("pos", "kinetic", "potential", "time", "temperature", "hbond"):
        assert out[k].dtype == ref[k].dtype, k
        assert out[k].shape[1:] == ref[k].shape[1:], k
        assert out[k].shape[0] == 2, k
    assert np.array_equal(out["pos"][0], ref["pos"][0])
    # the logged values come from the reference's own build on another host
    # (-ffast-math; BP stopped at its 1e-3 tolerance): 1e-4 relative, the
    # bound the engine's parity tests hold against the same log
    assert abs(out["potential"][0, 0] - ref["potential"][0, 0]) < 1e-4 * max(1., abs(ref["potential"][0, 0]))
    assert abs(out["kinetic"][0, 0] - ref["kinetic"][0, 0]) < 1e-6 * ref["kinetic"][0, 0]
    assert np.array_equal(out["time"], ref["time"][:2])  # (3 dt) * round in FP32, as logged
    assert np.array_equal(out["temperature"][:, 0], ref["temperature"][:2, 0])
    assert np.abs(out["hbond"][0] - ref["hbond"][0]).max() < 1e-4
    # the node-level arrays of the default (detailed) log level: the same set,
    # shapes and types, and frame 0's values.  The rotamer decomposition
    # follows the marginals, which two builds stop at the BP tolerance (1e-3)
    # in different float orders: 1e-3 of the array's scale (observed <= 2.3e-4)
    assert set(out) == set(ref.files) - {"invocation"}
    for k in set(out) - {"pos", "kinetic", "potential", "time", "temperature", "hbond"}:
        assert out[k].dtype == ref[k].dtype and out[k].shape[1:] == ref[k].shape[1:], k
        diff = np.abs(out[k][0].astype(np.float64) - ref[k][0]).max()
        assert diff < 1e-3 * max(1., np.abs(ref[k][0]).max()), (k, out[k][0], ref[k][0])
    # frame 1 lies 1852 rounds later on a chaotic trajectory: only its scale
    assert 0.2 < out["kinetic"][1, 0] / (1.5 * 0.8) < 3.0


def _thermal_mom(seed, n_atom, T, timescale=5.0):
    import oracle_py
    z = oracle_py.thermostat_normals(seed, 0, n_atom)
    ms = np.float32(np.exp(np.float32(-3 * DT) / np.float32(timescale)))
    ns = np.float32(np.sqrt(np.float32(T) * (np.float32(1) - ms * ms)))
    return (ns * z).astype(np.float32)


def test_trajectory_matches_oracle(built, syn_configs, tmp_path):
    """Frames every round for 4 rounds with recentring, against the oracle run
    through the same schedule from the same thermalised start."""
    import oracle_py
    import upside_gb300 as U
    from h5lite import H5File
    src, _ = syn_configs[60]
    cfg = str(tmp_path / "syn60.up")
    shutil.copyfile(src, cfg)
    T, seed = 0.85, 7
    U.upside_main(["--duration", repr(4 * RT), "--frame-interval", repr(RT), "--temperature", str(T),
                   "--seed", str(seed), "--record-momentum", "--log-level", "basic", "--output",
                   str(tmp_path / "out.h5"), cfg], verbose=False)
    out, _ = _out(str(tmp_path / "out.h5"))
    assert out["pos"].shape == (4, 1, 180, 3) and "hbond" not in out
    o = oracle_py.Oracle(cfg, 180)
    x = H5File(cfg).read("/input/pos")[:, :, 0].astype(np.float32)
    m = _thermal_mom(seed, 180, T)
    for r in range(4):
        x = (x - x.mean(0, dtype=np.float32)).astype(np.float32)
        e, _ = o.evaluate(x)
        tol = 2e-5 * 4 ** r  # FP32 differences grow over the 3 force evaluations of a round
        assert np.abs(out["pos"][r, 0] - x).max() < tol, (r, np.abs(out["pos"][r, 0] - x).max())
        assert np.abs(out["mom"][r, 0] - m).max() < 10 * tol * max(1., np.abs(m).max()), r
        assert abs(out["potential"][r, 0] - e) < max(1e-5, tol) * max(1., abs(e)), (r, out["potential"][r, 0], e)
        kin = 0.5 / 180 * np.sum((m * m).sum(1).astype(np.float64))
        assert abs(out["kinetic"][r, 0] - kin) < max(1e-6, tol) * kin, r
        x, m = o.run(x, m, 1, dt=float(DT), temperature=T, timescale=5.0, seed=seed, round_start=r + 1)


def test_replica_exchange_bookkeeping(built, syn_configs, tmp_path):
    import upside_gb300 as U
    src, _ = syn_configs[60]
    cfgs = []
    for k in range(4):
        cfgs.append(str(tmp_path / ("r%d.up" % k)))
        shutil.copyfile(src, cfgs[-1])
    base = str(tmp_path / "rex")
    U.upside_main(["--duration", repr(20 * RT), "--frame-interval", repr(2 * RT), "--replica-interval",
                   repr(2 * RT), "--swap-set", "0-1,2-3", "--swap-set", "1-2", "--temperature",
                   "0.80,0.85,0.90,0.95", "--output-base", base] + cfgs, verbose=False)
    outs = [_out("%s_%d.h5" % (base, k))[0] for k in range(4)]
    partners = [list(o["replica_swap_partner"]) for o in outs]
    assert partners == [[1], [0, 2], [3, 1], [2]]
    idx = np.stack([o["replica_index"][:, 0] for o in outs], 1)
    assert idx.shape == (10, 4)
    for row in idx:
        assert sorted(row) == [0, 1, 2, 3]
    assert list(idx[0]) == [0, 1, 2, 3]
    cum = [o["replica_cumulative_swaps"] for o in outs]
    for c in cum:
        assert np.all(np.diff(c[:, :, 1], axis=0) >= 0) and np.all(c[:, :, 0] <= c[:, :, 1])
    # exchanges after rounds 2, 4, ...: set 0 at the 1st, 3rd, ... attempt;
    # the frame at round 2k has seen k attempts
    assert list(cum[0][:, 0, 1]) == [(k + 1) // 2 for k in range(10)]
    assert list(cum[1][:, 1, 1]) == [k // 2 for k in range(10)]
    # both members of a pair count the same swaps
    assert np.array_equal(cum[0][:, 0], cum[1][:, 0]) and np.array_equal(cum[2][:, 0], cum[3][:, 0])
    assert np.array_equal(cum[1][:, 1], cum[2][:, 1])
    assert cum[0][-1, 0, 0] + cum[2][-1, 0, 0] + cum[1][-1, 1, 0] > 0  # some swaps accepted
    assert all(o["temperature"][0, 0] == np.float32(t) for o, t in zip(outs, (0.80, 0.85, 0.90, 0.95)))


def test_restart_from_logged_momenta(built, syn_configs, tmp_path):
    import upside_gb300 as U
    from h5lite import H5File, H5Writer
    src, _ = syn_configs[60]
    cfg = str(tmp_path / "a.up")
    shutil.copyfile(src, cfg)
    U.upside_main(["--duration", repr(6 * RT), "--frame-interval", repr(2 * RT), "--temperature", "0.9",
                   "--record-momentum", "--disable-recentering", cfg], verbose=False)
    a, f = _out(cfg)
    # the config keeps its input next to the new output
    orig = H5File(src)
    for nm in orig.list("/input/potential/rotamer"):
        if orig.kind("/input/potential/rotamer/" + nm) == 0:
            assert np.array_equal(orig.read("/input/potential/rotamer/" + nm),
                                  f.read("/input/potential/rotamer/" + nm))
    w = H5Writer()
    w.dataset("/input/pos", a["pos"][-1, 0][:, :, None])
    w.dataset("/input/mom", a["mom"][-1, 0][:, :, None])
    rst = str(tmp_path / "restart.h5")
    w.save(rst)
    out2 = str(tmp_path / "b.h5")
    U.upside_main(["--duration", repr(2 * RT), "--frame-interval", repr(2 * RT), "--temperature", "0.9",
                   "--record-momentum", "--disable-recentering", "--restart-using-momentum", "-i", rst,
                   "--output", out2, cfg], verbose=False)
    b, _ = _out(out2)
    assert b["pos"].shape[0] == 1
    assert np.array_equal(b["pos"][0], a["pos"][-1]) and np.array_equal(b["mom"][0], a["mom"][-1])
    assert b["kinetic"][0, 0] == a["kinetic"][-1, 0]
    # without /input/mom a restart is refused
    w2 = H5Writer()
    w2.dataset("/input/pos", a["pos"][-1, 0][:, :, None])
    w2.save(str(tmp_path / "nomom.h5"))
    with pytest.raises(RuntimeError):
        U.upside_main(["--duration", repr(RT), "--frame-interval", repr(RT), "--restart-using-momentum", "-i",
                       str(tmp_path / "nomom.h5"), "--output", str(tmp_path / "c.h5"), cfg], verbose=False)


def test_annealing_and_thermostat_interval(built, syn_configs, tmp_path):
    """--anneal-factor with the default end time drops to the final
    temperature at the first thermostat step (src/main.cpp:606-618); the
    logged temperature of frame 0 is the initial one.  A thermostat interval
    of 3 rounds runs the same schedule without graphs."""
    import upside_gb300 as U
    src, _ = syn_configs[60]
    cfg = str(tmp_path / "a.up")
    shutil.copyfile(src, cfg)
    out = str(tmp_path / "ann.h5")
    U.upside_main(["--duration", repr(6 * RT), "--frame-interval", repr(RT), "--temperature", "0.9",
                   "--anneal-factor", "0.5", "--output", out, cfg], verbose=False)
    o, _ = _out(out)
    assert o["temperature"][0, 0] == np.float32(0.9)
    assert np.all(o["temperature"][1:, 0] == np.float32(np.float32(0.9) * 0.5))
    out3 = str(tmp_path / "ti.h5")
    U.upside_main(["--duration", repr(9 * RT), "--frame-interval", repr(3 * RT), "--temperature", "0.9",
                   "--thermostat-interval", repr(3 * RT), "--output", out3, cfg], verbose=False)
    o3, _ = _out(out3)
    assert o3["pos"].shape[0] == 3 and np.all(np.isfinite(o3["pos"]))
    assert np.all(o3["kinetic"] > 0)
