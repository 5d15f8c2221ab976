"""Generate the golden fixtures the parity tests compare against.

Run here, where the reference checkout exists; writes small files next to
this script, which are committed (the GPU host has no reference checkout):

  chig.up            the reference's own ff_2.1 example config
                     (example/15.SpatialTransformation/inputs/chig.up)
  chig_run_output.npz  every /output array of that run and its invocation
                     (python make_fixtures.py chig_run writes only this file)
  chig_frames.npz    the 20 logged frames of the reference's example run
                     (outputs/simple_test/chig.run.up /output/pos, /output/potential)
                     plus the locally built reference engine's energy and
                     derivative at each frame
  syn<N>_ref.npz     seeded synthetic ff_2.1 proteins (config_gen): sequence,
                     seed, coordinates (initial + perturbed frames), and the
                     reference engine's energy, derivative, per-node outputs,
                     sensitivities, potentials and pair-list counts by type
  syn_transcis_ref.npz the trans-cis proline fixture (transcis_spec.py):
                     frames, reference energy and derivative, and the
                     trans-cis nodes' outputs and sensitivities per frame
                     (python make_fixtures.py trans_cis writes only this file)
  syn_membrane_ref.npz the membrane fixture (membrane_spec.py), flat and
                     curved: frames, reference energy and derivative, and the
                     membrane nodes' outputs and sensitivities per frame
                     (python make_fixtures.py membrane writes only this file)
  syn_surface_ref.npz the surface fixture (surface_spec.py): per variant
                     the frames' reference energy and derivative, the surface
                     node's output and the sensitivities the surface-dependent
                     membrane terms write (python make_fixtures.py surface
                     writes only this file)
  syn_graph_ref.npz  the reference's own edge lists of every interaction
                     graph of syn60/syn150 per frame, and its parameter
                     derivatives (get_param_deriv) of the rotamer, coverage
                     and nonlinear-coupling nodes (python make_fixtures.py
                     graph writes only this file)

The reference engine is oracle/_ref/libupside_ref.so (oracle/build.py).
"""
import ctypes
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "upside2-md_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import config_gen  # noqa: E402
from h5lite import H5File  # noqa: E402
import build as oracle_build  # noqa: E402

# the reference checkout: $UPSIDE_REFERENCE, else a "reference" directory beside the repository
REF = os.environ.get("UPSIDE_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
EX = os.path.join(REF, "example", "15.SpatialTransformation")


class RefEngine:
    def __init__(self, lib, path, n_atom):
        self.L = lib
        self.e = lib.construct_deriv_engine(n_atom, path.encode(), True)
        assert self.e
        self.n = n_atom

    def eval(self, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        en = ctypes.c_float()
        assert self.L.evaluate_energy(ctypes.byref(en), self.e, pos.ctypes.data) == 0
        d = np.zeros_like(pos)
        assert self.L.evaluate_deriv(d.ctypes.data, self.e, pos.ctypes.data) == 0
        return en.value, d

    def dims(self, nm):
        n, w = ctypes.c_int(), ctypes.c_int()
        assert self.L.get_output_dims(ctypes.byref(n), ctypes.byref(w), self.e, nm.encode()) == 0
        return n.value, w.value

    def node(self, nm, sens=False):
        n, w = self.dims(nm)
        o = np.zeros((n, w), np.float32)
        fn = self.L.get_sens if sens else self.L.get_output
        assert fn(o.size, o.ctypes.data, self.e, nm.encode()) == 0
        return o

    def value(self, nm, what, n):
        o = np.zeros(n, np.float32)
        r = self.L.get_value_by_name(n, o.ctypes.data, self.e, nm.encode(), what.encode())
        return o if r == 0 else None


def load_ref():
    path = oracle_build.build_reference()
    L = ctypes.CDLL(path)
    L.construct_deriv_engine.restype = ctypes.c_void_p
    L.construct_deriv_engine.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_bool]
    L.evaluate_energy.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
    L.evaluate_deriv.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.get_output.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    L.get_sens.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    L.get_output_dims.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    L.get_value_by_name.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]
    return L


GRAPH_NODES = ["rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "protein_hbond"]


def chig(L):
    shutil.copyfile(os.path.join(EX, "inputs", "chig.up"), os.path.join(HERE, "chig.up"))
    run = H5File(os.path.join(EX, "outputs", "simple_test", "chig.run.up"))
    pos = run.read("/output/pos")[:, 0].astype(np.float32)
    pot = run.read("/output/potential")[:, 0]
    eng = RefEngine(L, os.path.join(HERE, "chig.up"), pos.shape[1])
    E, D = [], []
    for x in pos:
        e, d = eng.eval(x)
        E.append(e)
        D.append(d)
    np.savez_compressed(os.path.join(HERE, "chig_frames.npz"), pos=pos, logged_potential=pot,
                        ref_energy=np.array(E), ref_deriv=np.array(D))


def chig_run_output():
    """Every /output array of the reference's logged example run and its
    command line, for the driver tests: frame 0 is logged before any
    integration, so the driver must reproduce it from the same invocation."""
    run = H5File(os.path.join(EX, "outputs", "simple_test", "chig.run.up"))
    out = {k: run.read("/output/" + k) for k in run.list("/output")}
    out["invocation"] = np.array(run.attr("/output", "invocation"))
    np.savez_compressed(os.path.join(HERE, "chig_run_output.npz"), **out)


def synthetic(L, n_res, seed, n_frames=3, tmpdir="/tmp"):
    rng = np.random.RandomState(seed)
    seq = config_gen.random_sequence(n_res, rng)
    path = os.path.join(tmpdir, "syn%d_%d.up" % (n_res, seed))
    pos0 = config_gen.write_config(path, seq, seed)
    # every frame carries coordinate noise: the initial structure of a random
    # chain has residue 0's N, CA, C exactly coplanar with the reference frame
    # geometry, a degenerate case in which the reference eigen-solver returns
    # a non-maximal eigenvector: its Householder step meets an exactly zero
    # column and the QR iteration converges to the wrong eigenpair
    frames = []
    prng = np.random.RandomState(seed + 1000)
    for k in range(n_frames):
        frames.append((pos0 + (0.02 if k == 0 else 0.05) * prng.randn(*pos0.shape)).astype(np.float32))
    eng = RefEngine(L, path, pos0.shape[0])
    out = {"seq": np.array([s.encode() for s in seq]), "seed": np.int64(seed), "pos": np.array(frames)}
    E, D = [], []
    names = H5File(path).list("/input/potential")
    for k, x in enumerate(frames):
        e, d = eng.eval(x)
        E.append(e)
        D.append(d)
        if k == 0:
            for nm in names:
                out["out/" + nm] = eng.node(nm)
                out["sens/" + nm] = eng.node(nm, sens=True)
            for nm in GRAPH_NODES:
                n_t = {"rotamer": 400, "hbond_coverage": 8 * 20, "hbond_coverage_hydrophobe": 12 * 20}.get(nm)
                if n_t:
                    v = eng.value(nm, "count_edges_by_type", n_t)
                    if v is not None:
                        out["count/" + nm] = v
    out["ref_energy"] = np.array(E)
    out["ref_deriv"] = np.array(D)
    np.savez_compressed(os.path.join(HERE, "syn%d_ref.npz" % n_res), **out)


TRANS_CIS_NODES = ["Dihedral_OmegaTransCis", "SigmoidCoord_trans1", "SigmoidCoord_trans2", "SigmoidCoord_cis1",
                   "SigmoidCoord_cis2", "Add_lambda_trans", "Multiply_lambda_cis", "Mean_lambda_mix", "Multiply_dup",
                   "SigmoidEnergy_trans1", "SigmoidEnergy_cis0", "SigmoidEnergy_cis1", "SigmoidEnergy_trans0",
                   "RamaMap2_trans", "RamaMap2_cis", "SigmoidLEnergy_mix", "SigmoidLEnergy_dup", "Sum_lambda",
                   "SigmoidLEnergy_sum", "rama_coord",
                   "rama_map_pot", "Spring_omega"]


def trans_cis(L, tmpdir="/tmp"):
    """syn_transcis_ref.npz: the trans-cis fixture of transcis_spec.py, the
    reference engine's energy and derivative at each frame, and the outputs
    and sensitivities of the trans-cis nodes at each frame."""
    import transcis_spec as T
    path = os.path.join(tmpdir, "syn_transcis.up")
    T.write(path)
    frames = T.frames()
    eng = RefEngine(L, path, frames.shape[1])
    out = {"pos": frames}
    E, D = [], []
    for k, x in enumerate(frames):
        e, d = eng.eval(x)
        E.append(e)
        D.append(d)
        for nm in TRANS_CIS_NODES:
            out.setdefault("out/" + nm, []).append(eng.node(nm))
            out.setdefault("sens/" + nm, []).append(eng.node(nm, sens=True))
    out = {k: np.array(v) for k, v in out.items()}
    out["ref_energy"] = np.array(E)
    out["ref_deriv"] = np.array(D)
    np.savez_compressed(os.path.join(HERE, "syn_transcis_ref.npz"), **out)


MEMBRANE_NODES = ["cb_membrane_potential", "hb_membrane_potential", "Const3D_curvature_center", "Const3D_probe",
                  "Const1D_probe", "Const2D_fixed", "placement_fixed_point_only_CB"]


def membrane(L, tmpdir="/tmp"):
    """syn_membrane_ref.npz: both variants of membrane_spec.py at the same
    frames (evaluated in order, so the probe keeps frame 0's positions): the
    reference engine's energy, derivative, and the membrane nodes' outputs
    and sensitivities."""
    import membrane_spec as M
    frames = M.frames()
    out = {"pos": frames}
    for var in M.VARIANTS:
        path = os.path.join(tmpdir, "syn_membrane_%s.up" % var)
        M.write(path, var)
        eng = RefEngine(L, path, frames.shape[1])
        E, D = [], []
        for x in frames:
            e, d = eng.eval(x)
            E.append(e)
            D.append(d)
            for nm in MEMBRANE_NODES:
                out.setdefault("%s/out/%s" % (var, nm), []).append(eng.node(nm))
                out.setdefault("%s/sens/%s" % (var, nm), []).append(eng.node(nm, sens=True))
        out[var + "/ref_energy"] = E
        out[var + "/ref_deriv"] = D
    out = {k: np.array(v) for k, v in out.items()}
    np.savez_compressed(os.path.join(HERE, "syn_membrane_ref.npz"), **out)


SURFACE_OUT = ["surface", "cat_pos_bb_cb"]
SURFACE_SENS = ["placement_fixed_point_only_CB", "protein_hbond", "environment_coverage_sc"]


def surface(L, tmpdir="/tmp"):
    """syn_surface_ref.npz: every variant of surface_spec.py at the same
    frames, evaluated in order on one engine (the surface node keeps state):
    the reference engine's energy, derivative, the surface node's output and
    the sensitivities of the nodes the membrane terms read."""
    import surface_spec as S
    frames = S.frames()
    out = {"pos": frames}
    for var in S.VARIANTS:
        path = os.path.join(tmpdir, "syn_surface_%s.up" % var)
        S.write(path, var)
        eng = RefEngine(L, path, frames.shape[1])
        E, D = [], []
        for x in frames:
            e, d = eng.eval(x)
            E.append(e)
            D.append(d)
            for nm in SURFACE_OUT:
                out.setdefault("%s/out/%s" % (var, nm), []).append(eng.node(nm))
            for nm in SURFACE_SENS:
                out.setdefault("%s/sens/%s" % (var, nm), []).append(eng.node(nm, sens=True))
        out[var + "/ref_energy"] = E
        out[var + "/ref_deriv"] = D
    out = {k: np.array(v) for k, v in out.items()}
    np.savez_compressed(os.path.join(HERE, "syn_surface_ref.npz"), **out)


KAT_SRC = r"""
#include <cstdio>
#include <cstdint>
#include <Random123/threefry.h>
int main() {
  for (uint32_t seed : {1u, 12345u, 4294967290u}) for (unsigned long long step : {0ull, 1ull, 4294967298ull})
  for (uint32_t stream : {0u, 1u}) for (uint32_t atom : {0u, 7u}) {
    threefry4x32_key_t k = {{seed, stream, 0u, 0u}};
    threefry4x32_ctr_t c = {{uint32_t(step & 0xffffffffu), uint32_t(step >> 32), atom, 0u}};
    threefry4x32_ctr_t r = threefry4x32(c, k);
    printf("%u %u %llu %u %u %u %u %u\n", seed, stream, step, atom, r.v[0], r.v[1], r.v[2], r.v[3]);
  }
}
"""


def threefry_kat():
    """Known answers of the reference's vendored Threefry-4x32-20 (src/include/Random123)."""
    import subprocess
    import tempfile
    d = tempfile.mkdtemp()
    src, exe = os.path.join(d, "kat.cpp"), os.path.join(d, "kat")
    open(src, "w").write(KAT_SRC)
    subprocess.check_call(["g++", "-O1", "-I", os.path.join(REF, "src", "include"), src, "-o", exe])
    out = subprocess.check_output([exe], text=True)
    with open(os.path.join(HERE, "threefry_kat.txt"), "w") as f:
        f.write("# seed stream counter_lo_hi(step) atom out0 out1 out2 out3\n" + out)


# interaction-graph nodes whose edge lists the reference build exposes
# (oracle/ref_build/dump), by accessor
EDGE_ACCESSORS = (("hb_environment_coverage", "hb_environment_coverage"),
                  ("environment_coverage", "environment_coverage"),
                  ("hbond_coverage", "hbond_coverage"), ("protein_hbond", "protein_hbond"),
                  ("rotamer", "rotamer"))
PARAM_DERIV_NODES = ("rotamer", "hbond_coverage", "hbond_coverage_hydrophobe", "nonlinear_coupling_environment")


def ref_edges(L, eng, node):
    """The reference's own edge list of an interaction-graph node, (index1,
    index2) in its order, or None for other nodes."""
    for prefix, acc in EDGE_ACCESSORS:
        if node.startswith(prefix):
            f = getattr(L, "ref_edges_" + acc)
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int]
            n = f(eng.e, node.encode(), None, 0)
            assert n >= 0, node
            a = np.zeros((max(n, 1), 2), np.int32)
            f(eng.e, node.encode(), a.ctypes.data, n)
            return a[:n]
    return None


def edges_and_param_derivs(L, tmpdir="/tmp"):
    """syn_graph_ref.npz: the reference's own pair lists and parameter
    derivatives.

      edges<N>/<k>/<node>  int16 (n_edge, 2): the edge list of every
                           interaction-graph node of the syn<N> fixture after
                           evaluating its frames 0..k in order on one engine
                           (the pair caches carry over between frames, as in
                           the reference)
      pd/<k>/<node>        get_param_deriv of the syn60 fixture written with
                           the nonlinear environment coupling (environment
                           potential type 0) after evaluate_deriv at frame k
    """
    L.get_param_deriv.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    out = {}
    for n in (60, 150):
        z = np.load(os.path.join(HERE, "syn%d_ref.npz" % n))
        path = os.path.join(tmpdir, "syn%d_graph.up" % n)
        config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0])
        eng = RefEngine(L, path, z["pos"].shape[1])
        for k, x in enumerate(z["pos"]):
            eng.eval(x)
            for nm in H5File(path).list("/input/potential"):
                e = ref_edges(L, eng, nm)
                if e is not None:
                    assert e.size == 0 or e.max() < 32767
                    out["edges%d/%d/%s" % (n, k, nm)] = e.astype(np.int16)
    z = np.load(os.path.join(HERE, "syn60_ref.npz"))
    path = os.path.join(tmpdir, "syn60_env0.up")
    config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0],
                            environment_potential_type=0)
    eng = RefEngine(L, path, z["pos"].shape[1])
    for k in (0, 1):
        eng.eval(z["pos"][k])
        for nm in PARAM_DERIV_NODES:
            size = {"rotamer": 20 * 20 * 54, "hbond_coverage": 8 * 20 * 50,
                    "hbond_coverage_hydrophobe": 12 * 20 * 50}.get(nm)
            if size is None:
                size = H5File(path).read("/input/potential/%s/coeff" % nm).size + 20 * 20
            d = np.zeros(size, np.float32)
            assert L.get_param_deriv(size, d.ctypes.data, eng.e, nm.encode()) == 0, nm
            out["pd/%d/%s" % (k, nm)] = d
    np.savez_compressed(os.path.join(HERE, "syn_graph_ref.npz"), **out)


def main():
    if sys.argv[1:] == ["graph"]:
        edges_and_param_derivs(load_ref())
        return
    if sys.argv[1:] == ["chig_run"]:
        chig_run_output()
        return
    if sys.argv[1:] == ["trans_cis"]:
        trans_cis(load_ref())
        return
    if sys.argv[1:] == ["membrane"]:
        membrane(load_ref())
        return
    if sys.argv[1:] == ["surface"]:
        surface(load_ref())
        return
    threefry_kat()
    L = load_ref()
    chig(L)
    chig_run_output()
    synthetic(L, 60, 1)
    synthetic(L, 150, 2, n_frames=2)
    trans_cis(L)
    membrane(L)
    surface(L)
    edges_and_param_derivs(L)


if __name__ == "__main__":
    main()
