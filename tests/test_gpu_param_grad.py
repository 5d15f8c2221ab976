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
