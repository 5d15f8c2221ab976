"""The CPU restatement of the warm-start network (oracle/warm_mlp_ref.py)
pinned by central finite differences: with the bf16 rounding switched off,
its analytic weight gradients match (L(w + h) - L(w - h)) / 2h in float64."""
import numpy as np


def test_reference_gradients_match_finite_differences(monkeypatch):
    import warm_mlp_ref as R
    monkeypatch.setattr(R, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.RandomState(4)
    M = 40
    X = rng.normal(size=(M, 64))
    nrot = rng.choice([1, 3, 6], size=M).astype(np.int32)
    T = np.zeros((M, 8))
    for i in range(M):
        T[i, :nrot[i]] = rng.dirichlet(np.ones(nrot[i]))
    w = {"W1": rng.normal(0, 0.3, (64, 128)), "b1": rng.normal(0, 0.1, 128), "W2": rng.normal(0, 0.1, (128, 128)),
         "b2": rng.normal(0, 0.1, 128), "W3": rng.normal(0, 0.2, (128, 8)), "b3": rng.normal(0, 0.1, 8)}
    _, g = R.loss_and_grads(X, T, nrot, w)
    h = 1e-6
    for k in w:
        flat = w[k].reshape(-1)
        for i in rng.choice(flat.size, 5, replace=False):
            old = flat[i]
            flat[i] = old + h
            lp, _ = R.loss_and_grads(X, T, nrot, w)
            flat[i] = old - h
            lm, _ = R.loss_and_grads(X, T, nrot, w)
            flat[i] = old
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k].reshape(-1)[i]) <= 1e-5 + 1e-4 * abs(fd), (k, i)
