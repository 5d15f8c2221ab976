"""The trans-cis proline fixture (syn_transcis_ref.npz): one 40-residue
chain written by config_gen with two trans-cis prolines (listed out of
residue order), a cis proline (CPR), two fixed rotamers, and extra switch
nodes that no config script writes (Mean, a Multiply with a repeated and an
empty output row, a Sum whose entries are out of order, SigmoidLEnergy with
and without cutoffs).  Shared by
make_fixtures.py and the tests, which regenerate the configuration from it.
"""
import numpy as np

N_RES = 40
SEED = 5
PRO_TC = (25, 10)   # trans-cis prolines, in table order
CPR = 31


def sequence(n_res=N_RES, seed=SEED):
    import config_gen
    seq = config_gen.random_sequence(n_res, np.random.RandomState(seed))
    for r in PRO_TC:
        seq[r] = 'PRO'
    seq[CPR] = 'CPR'
    return seq


def write(path, pos=None, n_res=N_RES, seed=SEED):
    """Write the configuration (another length or seed gives a system with
    the same node graph for batches); returns its initial coordinates."""
    import config_gen
    seq = sequence(n_res, seed)
    tc = [(25, 0, 4.0, 0.5, 45.0), (10, 1, 3.0, 0.8, 40.0)]
    fix = [(3, seq[3], 'A', 3, -60.0, 170.0), (7, seq[7], 'A', 7, 65.0, -80.0), (12, seq[12], 'A', 12, 'nan', 0)]
    n = len(PRO_TC)
    ar = np.arange(n)
    extra = [
        ("Mean_lambda_mix", ["SigmoidCoord_trans1", "SigmoidCoord_cis2"], {"n_dim": 1, "n_size": n},
         {"dim1": [0], "dim2": [0], "id_pos1": ar, "id_pos2": ar[::-1], "id1_out": ar, "id2_out": ar}),
        ("Multiply_dup", ["SigmoidCoord_trans2", "SigmoidCoord_cis1"], {"n_dim": 1, "n_size": n + 1},
         {"dim1": [0], "dim2": [0], "id_pos1": [0, 1, 0], "id1_out": [0, 1, 1], "id_pos2": [1, 0],
          "id2_out": [0, 1]}),
        ("SigmoidLEnergy_mix", ["Dihedral_OmegaTransCis", "Mean_lambda_mix"],
         {"integrator_level": 0, "use_cutoff": 0, "dim1": 0},
         {"id1": ar, "id2": ar, "a": [0.7, -0.4], "b": [1.5, 2.0], "c": [0.3, -2.0], "s": [1.0, 0.8],
          "min": [0., 0.], "max": [0., 0.]}),
        ("Sum_lambda", ["SigmoidCoord_trans1"], {"n_dim": 1},
         {"id_pos": [1, 0], "dim": [0], "weight": [0.7, 1.3]}),
        ("SigmoidLEnergy_sum", ["Dihedral_OmegaTransCis", "Sum_lambda"],
         {"integrator_level": 0, "use_cutoff": 0, "dim1": 0},
         {"id1": [1], "id2": [0], "a": [0.3], "b": [1.2], "c": [-2.2], "s": [0.9], "min": [0.], "max": [0.]}),
        ("SigmoidLEnergy_dup", ["Dihedral_OmegaTransCis", "Multiply_dup"],
         {"integrator_level": 0, "use_cutoff": 1, "dim1": 0},
         {"id1": [0, 1, 0], "id2": [0, 1, 2], "a": [0.5, 1.0, 2.0], "b": [-1.0, 0.6, 1.0],
          "c": [2.0, -1.0, 0.0], "s": [0.7, 1.2, 0.5], "min": [1.0, -2.5, -3.0], "max": [3.0, 0.5, 3.0]}),
    ]
    return config_gen.write_config(path, seq, seed, pos=pos, trans_cis=tc, fix_rotamer=fix, extra_nodes=extra)


# omega (radians) preceding each trans-cis proline, per frame: across the
# barrier segments and switch ramps (the cis proline's omega stays near 0)
OMEGAS = [(-2.4, 0.35), (-1.0, 2.0), (0.6, -2.9), (2.7, -0.3), (np.pi, 1.2)]


def frames(seed=SEED + 2000, n_res=N_RES):
    """Chains built from random (phi, psi) with the omegas above, plus noise."""
    import config_gen
    rng = np.random.RandomState(seed)
    out = []
    for om in OMEGAS:
        rama = rng.random_sample((n_res, 3)) * 2 * np.pi - np.pi
        rama[:, 2] = np.pi
        rama[CPR - 1, 2] = 0.1
        for r, w in zip(PRO_TC, om):
            rama[r - 1, 2] = w
        ang = np.zeros_like(rama)
        ang[:, 0], ang[:, 1], ang[:, 2] = 120.0 * config_gen.DEG, 120.0 * config_gen.DEG, 109.5 * config_gen.DEG
        ln = np.zeros_like(rama)
        ln[:, 0], ln[:, 1], ln[:, 2] = 1.453, 1.526, 1.300
        x = config_gen.chain_from_rama(rama, ang, ln)
        out.append((x - x.mean(0) + 0.02 * rng.randn(*x.shape)).astype(np.float32))
    return np.array(out)
