"""Monte Carlo pivot and jump moves (the reference's
src/monte_carlo_sampler.cpp) on the GPU batch, against a NumPy restatement
of the proposals driven by the oracle's Threefry (pinned against the
reference's own Random123) and the oracle's energies: the same random draws,
the same moved atoms, the same Metropolis decisions.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F = np.float32
PI = F(3.14159265358979)


def _threefry(seed, stream, round_, k):
    import oracle_py
    L = oracle_py._lib()
    ctr = (ctypes.c_uint32 * 4)(round_ & 0xffffffff, round_ >> 32, 0, k)
    key = (ctypes.c_uint32 * 4)(seed, stream, 0, 0)
    out = (ctypes.c_uint32 * 4)()
    L.ocpu_threefry4x32(ctr, key, out)
    return [int(x) for x in out]


def _u01(b):
    return F(F(np.uint32(b)) * F(1. / 4294967296.) + F(0.5 / 4294967296.))


def _box_muller(b0, b1):
    a = PI * (F(F(np.int32(np.uint32(b0).view(np.int32))) * F(1. / 2147483648.)) + F(0.5 / 2147483648.))
    r = np.sqrt(F(-2.) * np.log(_u01(b1)))
    return F(np.sin(a) * r), F(np.cos(a) * r)


def _axis_angle(angle, a):
    c, s = np.cos(F(angle)), np.sin(F(angle))
    C = F(1) - c
    x, y, z = a
    return np.array([[x * x * C + c, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, y * y * C + c, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, z * z * C + c]], dtype=F)


def _dihedral(r1, r2, r3, r4):
    Fv, G, H = r1 - r2, r2 - r3, r4 - r3
    A, B = np.cross(Fv, G), np.cross(H, G)
    C = np.cross(B, A)
    return F(np.arctan2(F(np.dot(C, G)), F(np.dot(A, B) * np.sqrt(F(np.dot(G, G))))))


def _pivot_tables(path):
    from h5lite import H5File
    f = H5File(path)
    pot = f.read("/input/pivot_moves/proposal_pot").astype(F)
    nl, nb = pot.shape[0], pot.shape[1]
    pot = pot.reshape(nl, nb * nb).copy()
    cdf = np.zeros_like(pot)
    for layer in range(nl):
        s = np.cumsum(np.exp(-pot[layer].astype(np.float64)))
        cdf[layer] = (s.astype(F).astype(np.float64) / s[-1]).astype(F)
        pot[layer] = (pot[layer].astype(np.float64) + np.log(s[-1])).astype(F)
        cdf[layer, -1] = 1.
    return (pot, cdf, nb, f.read("/input/pivot_moves/pivot_atom"), f.read("/input/pivot_moves/pivot_range"),
            f.read("/input/pivot_moves/pivot_restype"))


def _pivot_propose(x, tables, seed, round_):
    pot, cdf, nb, atoms, ranges, layers = tables
    b = _threefry(seed, 2, round_, 0)
    ux, uy, uz, uw = (_u01(v) for v in b)
    n = len(atoms)
    loc = min(int(F(n) * uz), n - 1)
    layer = layers[loc]
    binx = min(int(np.searchsorted(cdf[layer], uw, side="left")), nb * nb - 1)
    new_lp = pot[layer, binx]
    w = F(2) * PI / F(nb)
    nphi = F(w * (F(binx // nb) + ux - F(0.5)) - PI)
    npsi = F(w * (F(binx % nb) + uy - F(0.5)) - PI)
    at = atoms[loc]
    prevC, N, CA, C, nN = (x[a] for a in at)
    ophi, opsi = _dihedral(prevC, N, CA, C), _dihedral(N, CA, C, nN)
    obp = int(F(F(ophi + PI) * F(0.5 / PI) * F(nb) + F(0.5)))
    obs = int(F(F(opsi + PI) * F(0.5 / PI) * F(nb) + F(0.5)))
    obp, obs = (0 if obp >= nb else obp), (0 if obs >= nb else obs)
    old_lp = pot[layer, obp * nb + obs]
    u1 = (CA - N) / np.sqrt(F(np.dot(CA - N, CA - N)))
    u2 = (C - CA) / np.sqrt(F(np.dot(C - CA, C - CA)))
    U1, U2 = _axis_angle(nphi - ophi, u1), _axis_angle(npsi - opsi, u2)
    y = x.copy()
    moved = [at[3], at[4]] + list(range(ranges[loc][0], ranges[loc][1]))
    for a in moved:
        t = C + U2 @ (x[a] - C)
        y[a] = CA + U1 @ (t - CA)
    return y, F(new_lp - old_lp), _u01(_threefry(seed, 2, round_, 1)[0])


def _jump_propose(x, ranges, sig_t, sig_r, seed, round_):
    b = _threefry(seed, 3, round_, 0)
    kind = int(F(2) * _u01(b[0]))
    ch = min(int(F(len(ranges)) * _u01(b[3])), len(ranges) - 1)
    a0, a1 = ranges[ch]
    b2 = _threefry(seed, 3, round_, 1)
    n0, n1 = _box_muller(b2[0], b2[1])
    n2, n3 = _box_muller(b2[2], b2[3])
    y = x.copy()
    if kind == 0:
        y[a0:a1] += F(sig_t[ch] / np.sqrt(F(3))) * np.array([n0, n1, n2], dtype=F)
    else:
        ax = np.array([n1, n2, n3], dtype=F)
        ax = ax / (np.sqrt(F(np.dot(ax, ax))) + F(1e-16))
        U = _axis_angle(F(sig_r[ch]) * n0, ax)
        com = x[a0:a1].mean(0, dtype=F)
        y[a0:a1] = com + (x[a0:a1] - com) @ U.T
    return y, F(0), _u01(_threefry(seed, 3, round_, 2)[0])


def _run(built_cfg, n_atom, temps, seeds, x0, propose, rounds, k):
    """GPU steps against the restatement; returns the accept counts."""
    import oracle_py
    import upside_gb300 as U
    S = len(seeds)
    b = U.Batch([built_cfg] * S)
    b.set_pos(np.concatenate([x0] * S))
    b.set_thermostat(temps, np.array(seeds, np.uint32))
    orc = oracle_py.Oracle(built_cfg, n_atom)
    xs = [x0.copy() for _ in range(S)]
    n_acc = 0
    for r in rounds:
        acc = b.monte_carlo(r)
        got = b.get_pos().reshape(S, n_atom, 3)
        for s in range(S):
            e_old, _ = orc.evaluate(xs[s])
            y, dl, u = propose(xs[s], seeds[s], r)
            e_new, _ = orc.evaluate(y)
            lb = F(dl - F(1. / F(temps[s])) * (F(e_new) - F(e_old)))
            ok = lb >= 0 or np.exp(lb) >= u
            assert acc[s, k] == int(ok), (r, s, lb, u)
            assert acc[s, 1 - k] == -1
            xs[s] = y if ok else xs[s]
            assert np.abs(got[s] - xs[s]).max() < 2e-4, (r, s, np.abs(got[s] - xs[s]).max())
            n_acc += ok
    return n_acc


def test_pivot_moves_match_restatement(built, syn_configs, tmp_path):
    import config_gen
    _, z = syn_configs[60]
    cfg = str(tmp_path / "piv.up")
    config_gen.write_config(cfg, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][1], moves=True)
    tables = _pivot_tables(cfg)
    n = _run(cfg, 180, [0.9, 2.0, 5.0, 10.0], [5, 6, 7, 8], z["pos"][1].astype(F),
             lambda x, seed, r: _pivot_propose(x, tables, seed, r), [1, 2, 3], 0)
    assert n > 0  # some proposals accepted


def test_jump_moves_match_restatement(built, tmp_path):
    import config_gen
    from h5lite import H5File
    rng = np.random.RandomState(11)
    seq = config_gen.random_sequence(40, rng)
    cfg = str(tmp_path / "jump.up")
    x0 = config_gen.write_config(cfg, seq, 11, chain_first_residue=[20], moves=True,
                                 chain_offsets=np.array([[0., 0., 0.], [30., 0., 0.]]))
    f = H5File(cfg)
    ranges = f.read("/input/jump_moves/atom_range")
    st, sr = f.read("/input/jump_moves/sigma_trans"), f.read("/input/jump_moves/sigma_rot")
    assert not f.exists("/input/pivot_moves")
    n = _run(cfg, 120, [1.0, 1.0, 3.0, 3.0], [21, 22, 23, 24], x0.astype(F),
             lambda x, seed, r: _jump_propose(x, ranges, st, sr, seed, r), [1, 2, 3, 4], 1)
    assert n > 0


def test_driver_monte_carlo_stats(built, syn_configs, tmp_path):
    """--monte-carlo-interval: moves at every nonzero multiple of the interval
    (in rounds), pivot_stats per frame = [successes, attempts] since the
    previous frame."""
    import config_gen
    import upside_gb300 as U
    _, z = syn_configs[60]
    cfg = str(tmp_path / "piv.up")
    config_gen.write_config(cfg, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][1], moves=True)
    rt = float(F(3) * F(0.009))
    out = str(tmp_path / "mc.h5")
    U.upside_main(["--duration", repr(12 * rt), "--frame-interval", repr(4 * rt), "--monte-carlo-interval",
                   repr(2 * rt), "--temperature", "0.9", "--output", out, cfg], verbose=False)
    from h5lite import H5File
    st = H5File(out).read("/output/pivot_stats")
    # frames at rounds 0, 4, 8; moves at rounds 2, 4, 6, 8, 10 (before the frame of the same round)
    assert st.shape == (3, 2)
    assert list(st[:, 1]) == [0, 2, 2]
    assert np.all(st[:, 0] <= st[:, 1])
