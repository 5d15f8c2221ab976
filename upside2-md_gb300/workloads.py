"""Seeded synthetic workloads (the five benchmark configurations).

  C1  1 chain of 60 residues, T=0.85
  C2  1 chain of 300 residues, T=0.85
  C3  48 replicas of one 150-residue chain, T geometric 0.80 -> 1.00, replica
      exchange between alternating even/odd neighbour pairs every 20 steps
      (rounds, the reference's step)
  C4  64 independent chains, lengths uniform in [40, 400], T uniform in [0.80, 0.95]
  C5  8 chains of 250 residues in one system (2000 residues), spaced apart,
      in a periodic box of side 200 A when the box mode is asked for
  M1  64 chains, lengths uniform in [40, 200], T uniform in [0.80, 0.95], in a
      30 A membrane with the surface node (lipid-diffusion method) and the
      surface-dependent CB, H/O and lateral-pressure terms (not one of the
      five; it measures the membrane path)

Sequences are drawn uniformly over the 20 amino acids from the seed; initial
structures are random (phi, psi) chains (py/upside_config.py:186-201).  Files
are cached under a work directory keyed by the configuration, the seed and a
hash of the generator.
"""
import os

import numpy as np

import config_gen

WORK = os.environ.get("UPSIDE_GB300_WORK", "/tmp/upside_gb300_work")


def _generator_key():
    """Short hash of the config generator and its parameter bundle, so that
    cached files are regenerated whenever either changes."""
    import hashlib
    h = hashlib.sha1()
    for f in (config_gen.__file__, config_gen.DEFAULT_PARAMS):
        if f and os.path.exists(f):
            with open(f, "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()[:10]


def _cfg(name, seed, n_res, **kw):
    os.makedirs(WORK, exist_ok=True)
    path = os.path.join(WORK, "%s_s%d_n%d_%s.up" % (name, seed, n_res if isinstance(n_res, int) else sum(n_res),
                                                     _generator_key()))
    if not os.path.exists(path):
        rng = np.random.RandomState(seed)
        seq = config_gen.random_sequence(int(n_res) if isinstance(n_res, int) else int(sum(n_res)), rng)
        tmp = path + ".tmp%d" % os.getpid()
        config_gen.write_config(tmp, seq, seed, **kw)
        os.replace(tmp, path)
    return path


def lateral_pressure_profile():
    """A synthetic lateral pressure profile (z, bar) over [-32, 30] A."""
    z = np.arange(-32., 31., 2.)
    p = 4000. * np.cos(z / 6.) * np.exp(-(z / 25.) ** 2) + 1500.
    return np.column_stack((z, p))


def n_res_of(path):
    from h5lite import H5File
    with H5File(path) as f:
        return f.read("/input/pos").shape[0] // 3


def workload(name, seed=1):
    """Returns dict(configs=[...], n_res=[...], temps=[...], seeds=[...], swap_sets=None|[...])."""
    if name == "C1":
        cfgs = [_cfg("C1", seed, 60)]
        temps = [0.85]
    elif name == "C2":
        cfgs = [_cfg("C2", seed, 300)]
        temps = [0.85]
    elif name == "C3":
        c = _cfg("C3", seed, 150)
        cfgs = [c] * 48
        temps = list(0.80 * (1.00 / 0.80) ** (np.arange(48) / 47.))
    elif name == "C4":
        rng = np.random.RandomState(1000 + seed)
        lengths = rng.randint(40, 401, size=64)
        cfgs = [_cfg("C4c%02d" % i, seed * 100 + i, int(n)) for i, n in enumerate(lengths)]
        temps = list(rng.uniform(0.80, 0.95, size=64))
    elif name == "C5":
        starts = [250 * k for k in range(1, 8)]
        offsets = np.array([[60.0 * (k % 4) - 90.0, 60.0 * (k // 4) - 30.0, 0.0] for k in range(8)])
        cfgs = [_cfg("C5", seed, 2000, chain_first_residue=starts, chain_offsets=offsets)]
        temps = [0.85]
    elif name == "M1":
        rng = np.random.RandomState(2000 + seed)
        lengths = rng.randint(40, 201, size=64)
        cfgs = [_cfg("M1c%02d" % i, seed * 100 + i, int(n), membrane_thickness=30., surface=1, channel_membrane=True,
                     lateral_pressure=lateral_pressure_profile()) for i, n in enumerate(lengths)]
        temps = list(rng.uniform(0.80, 0.95, size=64))
    else:
        raise ValueError("unknown workload " + name)
    n_res = [n_res_of(c) for c in cfgs]
    swap_sets = None
    if name == "C3":
        even = [(i, i + 1) for i in range(0, 47, 2)]
        odd = [(i, i + 1) for i in range(1, 47, 2)]
        swap_sets = [even, odd]
    return dict(configs=cfgs, n_res=n_res, temps=temps, seeds=[seed + i for i in range(len(cfgs))],
                swap_sets=swap_sets, exchange_interval=20 if swap_sets else 0,
                box=(200.0, 200.0, 200.0) if name == "C5" else None)


def initial_positions(configs):
    from h5lite import H5File
    out = []
    for c in configs:
        with H5File(c) as f:
            out.append(f.read("/input/pos")[:, :, 0].astype(np.float32))
    return np.concatenate(out)
