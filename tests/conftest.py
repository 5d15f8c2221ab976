import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (os.path.join(ROOT, "upside2-md_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Compile the in-tree libraries once per session."""
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def syn_configs(tmp_path_factory, built):
    """The synthetic fixture configs regenerated from their sequence and seed."""
    import config_gen
    d = tmp_path_factory.mktemp("cfg")
    out = {}
    for n in (60, 150):
        z = np.load(os.path.join(GOLDEN, "syn%d_ref.npz" % n))
        path = str(d / ("syn%d.up" % n))
        config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0])
        out[n] = (path, z)
    return out


@pytest.fixture(scope="session")
def transcis_config(tmp_path_factory, built):
    """The trans-cis proline fixture config (golden/transcis_spec.py) and its
    reference data."""
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import transcis_spec
    path = str(tmp_path_factory.mktemp("tc") / "syn_transcis.up")
    transcis_spec.write(path)
    return path, np.load(os.path.join(GOLDEN, "syn_transcis_ref.npz"))


@pytest.fixture(scope="session")
def membrane_configs(tmp_path_factory, built):
    """The membrane fixture configs (golden/membrane_spec.py), by variant,
    and their reference data."""
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import membrane_spec
    d = tmp_path_factory.mktemp("memb")
    paths = {}
    for var in membrane_spec.VARIANTS:
        paths[var] = str(d / ("syn_membrane_%s.up" % var))
        membrane_spec.write(paths[var], var)
    return paths, np.load(os.path.join(GOLDEN, "syn_membrane_ref.npz"))


@pytest.fixture(scope="session")
def surface_configs(tmp_path_factory, built):
    """The surface fixture configs (golden/surface_spec.py), by variant, and
    their reference data."""
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import surface_spec
    d = tmp_path_factory.mktemp("surf")
    paths = {}
    for var in surface_spec.VARIANTS:
        paths[var] = str(d / ("syn_surface_%s.up" % var))
        surface_spec.write(paths[var], var)
    return paths, np.load(os.path.join(GOLDEN, "syn_surface_ref.npz"))


# Reference-facing bounds (energy: of sum_nodes |E_node|; force: of max |F|).
# The frames' eigen-solve restates the reference's truncated QR, so what is
# left is FP32 rounding; where the reference's own distance from the FP64
# instantiation is larger than half the force bound (steep steric walls at
# ~50 A coordinates), the bound is twice that distance.
E_REF_TOL = 1e-5
F_REF_TOL = 1e-4


def ref_force_bound(ref_deriv, d64):
    """relative max-force bound against the reference's derivative, given the
    FP64 oracle's derivative at the same coordinates"""
    dist = np.abs(ref_deriv - d64).max() / np.abs(ref_deriv).max()
    return max(F_REF_TOL, 2.0 * dist)


def quat_align(a, ref):
    """Flip the quaternion columns (3:7) of affine outputs to the sign of ref
    (q and -q are the same rotation)."""
    a = np.array(a, copy=True)
    s = np.sign((a[:, 3:] * ref[:, 3:]).sum(1))
    s[s == 0] = 1
    a[:, 3:] *= s[:, None]
    return a
