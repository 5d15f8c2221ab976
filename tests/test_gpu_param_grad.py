"""dE/d(parameters) through torch.autograd (param_grad.FrameEnergy) on the GPU.

The gradient of the frame-averaged potential with respect to the rotamer
pair-spline coefficients and the nonlinear environment-coupling coefficients
(environment potential type 0) is checked two ways:

  * against the FP32 oracle's own parameter derivatives at every frame
    (same adjoint, restated on the CPU): 1e-3 of the largest component;
  * against central finite differences of the GPU energy, h = 1e-3, on the
    largest components: |fd - g| <= 2e-2 |g| + 2e-3 (the energy is an FP64
    sum of FP32 terms and BP is converged to its tolerance, which bounds how
    well a difference quotient resolves the derivative).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_FRAMES = 8
NODES = [("rotamer", (20, 20, 54)), ("nonlinear_coupling_environment", None)]


@pytest.fixture(scope="module")
def env0_config(syn_configs, tmp_path_factory):
    import config_gen
    path0, z = syn_configs[60]
    path = str(tmp_path_factory.mktemp("env0") / "syn60_env0.up")
    config_gen.write_config(path, [s.decode() for s in z["seq"]], int(z["seed"]), pos=z["pos"][0],
                            environment_potential_type=0)
    rng = np.random.RandomState(11)
    frames = [z["pos"][k % len(z["pos"])] + rng.normal(0, 0.05, z["pos"][0].shape).astype(np.float32)
              for k in range(N_FRAMES)]
    return path, frames


def _n_param(path, frames, node):
    import oracle_py
    o = oracle_py.Oracle(path, frames[0].shape[0])
    o.evaluate(frames[0])
    return o.param_deriv(node).size


def _batch(path, frames):
    import upside_gb300 as U
    b = U.Batch([path] * len(frames))
    b.set_pos(np.concatenate(frames))
    return b


@pytest.mark.parametrize("node,shape", NODES)
def test_autograd_matches_oracle_adjoint(env0_config, node, shape):
    import oracle_py
    import torch
    from param_grad import mean_energy
    path, frames = env0_config
    o = oracle_py.Oracle(path, frames[0].shape[0])
    n_par = _n_param(path, frames, node) if shape is None else int(np.prod(shape))
    shape = shape or (n_par,)
    b = _batch(path, frames)
    p0 = b.get_param(node, shape)
    p = torch.tensor(p0, requires_grad=True)
    e = mean_energy(p, b, node)
    e.backward()
    g = p.grad.numpy().ravel()
    ref = np.zeros(n_par)
    e_ref = 0.0
    for x in frames:
        ei, _ = o.evaluate(x)
        e_ref += ei / len(frames)
        ref += o.param_deriv(node) / len(frames)
    assert abs(e.item() - e_ref) < 1e-3 * max(1.0, abs(e_ref))
    assert np.abs(ref).max() > 0
    assert np.abs(g - ref).max() <= 1e-3 * np.abs(ref).max(), node


@pytest.mark.parametrize("node,shape", NODES)
def test_autograd_matches_central_differences(env0_config, node, shape):
    import torch
    from param_grad import mean_energy
    path, frames = env0_config
    b = _batch(path, frames)
    if shape is None:
        shape = (_n_param(path, frames, node),)
    p0 = b.get_param(node, shape).astype(np.float32)
    p = torch.tensor(p0, requires_grad=True)
    mean_energy(p, b, node).backward()
    g = p.grad.numpy().ravel()
    n_coeff = g.size
    if node == "nonlinear_coupling_environment":
        from h5lite import H5File
        with H5File(path) as f:
            n_coeff = f.read("/input/potential/%s/coeff" % node).size
    h = 1e-3
    for i in np.argsort(-np.abs(g))[:6]:
        # a symmetric pair interaction reports, for entry (t1, t2, c), the
        # derivative along moving (t1, t2, c) and (t2, t1, c) together (the
        # diagonal t1 == t2 counts its single entry twice), as the
        # reference's get_param_deriv does
        step = np.zeros(p0.size, np.float32)
        scale = 1.0
        if len(shape) == 3 and shape[0] == shape[1]:
            t1, t2, c = np.unravel_index(i, shape)
            step[np.ravel_multi_index((t1, t2, c), shape)] = h
            step[np.ravel_multi_index((t2, t1, c), shape)] = h
            scale = 2.0 if t1 == t2 else 1.0
        elif i >= n_coeff:
            # 20 independent weights: the weight of residue type aa is shared
            # by every coupling type, and the reported derivative is the one
            # along that shared weight (src/environment.cpp:822-833)
            aa = (i - n_coeff) % 20
            step[n_coeff + aa + 20 * np.arange(20)] = h
        else:
            step[i] = h
        plus = (p0.ravel() + step).reshape(shape)
        minus = (p0.ravel() - step).reshape(shape)
        ep = mean_energy(torch.tensor(plus), b, node).item()
        em = mean_energy(torch.tensor(minus), b, node).item()
        fd = scale * (ep - em) / (2 * h)
        assert abs(fd - g[i]) <= 2e-2 * abs(g[i]) + 2e-3, (node, int(i), fd, float(g[i]))
    b.set_param(node, p0)


@pytest.fixture(scope="module")
def c5_frames(built):
    """Config 5's system (8 chains x 250 residues) written with the nonlinear
    environment coupling (environment potential type 0) and 256 frames of
    one trajectory of it, 2 rounds apart after 50 rounds of relaxation."""
    import config_gen
    import upside_gb300 as U
    import workloads
    from h5lite import H5File
    W = workloads.workload("C5", seed=3)
    src = W["configs"][0]
    with H5File(src) as f:
        seq = [s.decode() for s in f.read("/input/sequence")]
        starts = list(f.read("/input/chain_break/chain_first_residue"))
        x0 = f.read("/input/pos")[:, :, 0].astype(np.float32)
    path = os.path.join(os.path.dirname(src), "C5_env0_test.up")
    config_gen.write_config(path, seq, 3, chain_first_residue=starts, pos=x0, environment_potential_type=0)
    b = U.Batch([path])
    b.set_pos(x0)
    b.set_thermostat([0.85], np.array([5], np.uint32))
    b.run(50, use_graph=True, graph_rounds=10)
    frames = []
    for _ in range(256):
        b.run(2, use_graph=True, graph_rounds=2)
        frames.append(b.get_pos())
    return path, frames


@pytest.mark.parametrize("node", ["rotamer", "nonlinear_coupling_environment"])
def test_c5_gradient_over_256_frames(c5_frames, node):
    """Config 5's parameter gradient: dE/d(theta) of the mean over 256 frames
    of the 2000-residue system, from batched evaluations of the frames (the
    adjoint kernels summed over each batch, behind torch.autograd),
    against central differences of the same mean (h = 1e-3) on its largest
    components, and on two of the frames against the FP32 oracle's adjoint
    (which matches the reference's get_param_deriv to 1e-5 on the syn60
    fixture, test_oracle.test_param_derivs_match_reference)."""
    import oracle_py
    import torch
    import upside_gb300 as U
    from param_grad import mean_energy
    path, frames = c5_frames
    # 8 batches of 32 frames (one batch of 256 copies of the system would hold
    # the pair lists of 512,000 residues); the autograd sum over the batches'
    # means, each weighted by its share of the frames, is the 256-frame mean
    chunks = []
    for k in range(0, len(frames), 32):
        bk = U.Batch([path] * 32)
        bk.set_pos(np.concatenate(frames[k:k + 32]))
        chunks.append(bk)

    def mean_256(param):
        return sum(mean_energy(param, bk, node) * (bk.n_sys / len(frames)) for bk in chunks)

    b = chunks[0]
    o = oracle_py.Oracle(path, frames[0].shape[0])
    o.evaluate(frames[0])
    n_par = o.param_deriv(node).size
    shape = (20, 20, 54) if node == "rotamer" else (n_par,)
    p0 = b.get_param(node, shape).astype(np.float32)
    p = torch.tensor(p0, requires_grad=True)
    mean_256(p).backward()
    g = p.grad.numpy().ravel()
    # the FP32 oracle on two frames: their mean derivative from a batch of the two
    two = U.Batch([path] * 2)
    two.set_pos(np.concatenate([frames[0], frames[255]]))
    two.evaluate(want_deriv=False)
    g2 = two.param_deriv(node, shape).ravel() / 2.0
    ref = np.zeros(n_par)
    for x in (frames[0], frames[255]):
        o.evaluate(x)
        ref += o.param_deriv(node) / 2.0
    assert np.abs(g2 - ref).max() <= 1e-3 * np.abs(ref).max(), node
    # central differences of the 256-frame mean on the largest components
    n_coeff = g.size
    if node == "nonlinear_coupling_environment":
        from h5lite import H5File
        with H5File(path) as f:
            n_coeff = f.read("/input/potential/%s/coeff" % node).size
    def central(i, h):
        step = np.zeros(p0.size, np.float32)
        scale = 1.0
        if len(shape) == 3:
            t1, t2, c = np.unravel_index(i, shape)
            step[np.ravel_multi_index((t1, t2, c), shape)] = h
            step[np.ravel_multi_index((t2, t1, c), shape)] = h
            scale = 2.0 if t1 == t2 else 1.0
        elif i >= n_coeff:
            aa = (i - n_coeff) % 20
            step[n_coeff + aa + 20 * np.arange(20)] = h
        else:
            step[i] = h
        ep = mean_256(torch.tensor((p0.ravel() + step).reshape(shape))).item()
        em = mean_256(torch.tensor((p0.ravel() - step).reshape(shape))).item()
        return scale * (ep - em) / (2 * h)

    for i in np.argsort(-np.abs(g))[:4]:
        tol = 2e-2 * abs(g[i]) + 2e-3
        fd = central(i, 1e-3)
        if abs(fd - g[i]) > tol:
            # a BP solve that stops after a different number of sweeps at +h
            # and -h moves the energy by up to its convergence tolerance,
            # which a 1e-3 step magnifies; a wider step has to agree then
            fd3 = central(i, 3e-3)
            assert abs(fd3 - g[i]) <= tol, (node, int(i), fd, fd3, float(g[i]))
