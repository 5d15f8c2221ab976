"""The surface fixture (syn_surface_ref.npz): a 60-residue chain written by
config_gen with the surface node and the surface-dependent membrane terms
(--surface, --channel-membrane-potential, --membrane-lateral-potential;
thickness 30 angstrom), once with the lipid-diffusion surface (method 1),
once with the fast surface (method 0) on a curved bilayer, and once with the
surface restricted to an included residue list.  Shared by make_fixtures.py
and the tests, which regenerate the configurations from it.  The frames are
evaluated in order on one engine: the surface node keeps state between
evaluations.
"""
import numpy as np

N_RES = 60
SEED = 12
VARIANTS = {
    "diffusion": {"surface": 1},
    "fast_curved": {"surface": 0, "use_curvature": True, "curvature_radius": 80., "curvature_sign": 1},
    "included": {"surface": 1, "surface_included_residues": tuple(range(5, 50))},
}


def lateral_table():
    """A synthetic lateral pressure profile (z, bar) over [-32, 30], large
    and nonzero at its lower end (where the reference's spline coordinate
    reads it inside the profile's range), so that the lateral forces are of
    the order of the other membrane forces (the M1 workload's profile)."""
    import workloads
    return workloads.lateral_pressure_profile()


def write(path, variant, pos=None, n_res=N_RES, seed=SEED):
    """Write one variant; returns its initial coordinates."""
    import config_gen
    seq = config_gen.random_sequence(n_res, np.random.RandomState(seed))
    return config_gen.write_config(path, seq, seed, pos=pos, membrane_thickness=30., channel_membrane=True,
                                   lateral_pressure=lateral_table(), **VARIANTS[variant])


# z shift of each frame: centred in the slab, partly out of it, back in
SHIFTS = [0.0, 3.0, -6.0, 14.0, 0.5, -1.0]


def frames(seed=SEED + 4000, n_res=N_RES):
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
