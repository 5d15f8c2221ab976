"""The membrane fixture (syn_membrane_ref.npz): a 50-residue chain written by
config_gen with the ff_2.1 membrane potential (thickness 30 angstrom, three
residues excluded from the CB term), once flat and once on a curved bilayer
(radius 60, sign -1), plus a Const3D node that takes two atoms' positions at
the first evaluation, a Const1D that takes three atoms' z and a fixed
Const2D.  Shared by make_fixtures.py and the tests, which
regenerate the configurations from it.
"""
import numpy as np

N_RES = 50
SEED = 8
EXCLUDE = (4, 5, 30)
VARIANTS = {"flat": {}, "curved": {"use_curvature": True, "curvature_radius": 60., "curvature_sign": -1}}
PROBE = ("Const3D_probe", ["pos"], {"dim1": 0, "dim2": 1, "dim3": 2, "initialized_by_coord": 1},
         {"id": np.array([5, 17])})
PROBES_12 = [("Const1D_probe", ["pos"], {"dim": 2, "initialized_by_coord": 1}, {"id": np.array([3, 9, 40])}),
             ("Const2D_fixed", ["pos"], {"dim1": 0, "dim2": 1, "initialized_by_coord": 0},
              {"id": np.arange(2), "value": np.array([[1.5, -2.0], [0.25, 4.0]])})]


def write(path, variant, pos=None, n_res=N_RES, seed=SEED):
    """Write one variant; returns its initial coordinates."""
    import config_gen
    seq = config_gen.random_sequence(n_res, np.random.RandomState(seed))
    return config_gen.write_config(path, seq, seed, pos=pos, membrane_thickness=30.,
                                   membrane_exclude_residues=EXCLUDE, extra_nodes=[PROBE] + PROBES_12,
                                   **VARIANTS[variant])


# z shift of each frame: through the slab and out of it on either side
SHIFTS = [0.0, 9.0, -14.0, 25.0]


def frames(seed=SEED + 3000, n_res=N_RES):
    """Random coils, each turned by a random rotation and moved along z."""
    import config_gen
    rng = np.random.RandomState(seed)
    out = []
    for dz in SHIFTS:
        x = config_gen.random_initial_config(n_res, rng)
        q, _ = np.linalg.qr(rng.randn(3, 3))
        x = (x - x.mean(0)) @ q.T + np.array([0., 0., dz])
        out.append((x + 0.02 * rng.randn(*x.shape)).astype(np.float32))
    return np.array(out)
