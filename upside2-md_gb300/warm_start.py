"""Learned warm start for the rotamer BP solve: data, training, deployment.

The network (64 features -> 128 -> 128 -> 8 logits, ReLU, bf16 weights with
FP32 accumulation) predicts each residue's converged rotamer marginal from
its local backbone geometry, residue type and one-body rotamer energies.  It
is trained on marginals the engine itself produces: seeded synthetic proteins
are advanced with the integrator, and at sampled frames the converged BP
marginals and the features are read back from the rotamer node.

Every arithmetic step of training runs in the library's own kernels
(ug_mlp_*: mma.sync bf16 GEMMs, epilogues, softmax cross-entropy, Adam);
PyTorch only holds the device buffers.  The engine uses the weights through
ug_set_warm_start.

    python warm_start.py --out weights.npz [--frames 8] [--epochs 12]
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_IN, N_HID, N_OUT = 64, 128, 8
ROTAMER = "rotamer"
WEIGHTS = os.path.join(HERE, "warm_start_ff21.npz")


def _lib():
    import upside_gb300 as U
    return U.lib()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _chk(r):
    if r:
        raise RuntimeError(_lib().ug_last_error().decode())


# ----------------------------------------------------------- bf16 (host) ---
def to_bf16_bits(x):
    """FP32 -> bf16 bit patterns (round to nearest even), as int16."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16).view(np.int16)


def from_bf16_bits(h):
    return (np.asarray(h).view(np.uint16).astype(np.uint32) << 16).view(np.float32)


# ------------------------------------------------------------------ data ---
def collect(configs, temps, seeds, frames, rounds_between, warmup_rounds):
    """Features, converged marginals and rotamer counts of every multi-rotamer
    BP node at `frames` frames of a trajectory of the given systems."""
    import upside_gb300 as U
    import workloads
    b = U.Batch(configs)
    b.set_pos(workloads.initial_positions(configs))
    b.set_thermostat(temps, np.asarray(seeds, np.uint32))
    b.run(warmup_rounds, use_graph=True, graph_rounds=1)
    n_node = int(b.value_by_name(ROTAMER, "bp_n_node", 1)[0])
    X, T, R = [], [], []
    for _ in range(frames):
        b.run(rounds_between, use_graph=True, graph_rounds=1)
        b.evaluate(want_deriv=False)
        nrot = b.value_by_name(ROTAMER, "bp_nrot", n_node).astype(np.int32)
        x = b.value_by_name(ROTAMER, "warm_features", n_node * N_IN).reshape(n_node, N_IN)
        t = b.value_by_name(ROTAMER, "bp_marginal", n_node * 8).reshape(n_node, 8)
        keep = nrot > 1
        X.append(x[keep])
        T.append(t[keep])
        R.append(nrot[keep])
    return np.concatenate(X), np.concatenate(T), np.concatenate(R)


# --------------------------------------------------------------- network ---
class WarmNet:
    """FP32 master weights, bf16 copies and Adam moments on the device."""

    def __init__(self, seed=0, weights=None):
        import torch
        self.torch = torch
        dev = "cuda"
        if weights is None:
            rng = np.random.RandomState(seed)
            weights = {
                "W1": rng.normal(0, np.sqrt(2.0 / N_IN), (N_IN, N_HID)),
                "b1": np.zeros(N_HID),
                "W2": rng.normal(0, np.sqrt(2.0 / N_HID), (N_HID, N_HID)),
                "b2": np.zeros(N_HID),
                "W3": rng.normal(0, np.sqrt(1.0 / N_HID), (N_HID, N_OUT)),
                "b3": np.zeros(N_OUT),
            }
        self.w = {k: torch.tensor(np.asarray(v, np.float32), device=dev) for k, v in weights.items()}
        self.wb = {k: torch.tensor(to_bf16_bits(weights[k]), device=dev) for k in ("W1", "W2", "W3")}
        self.m = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.step_no = 0

    def numpy(self):
        return {k: v.detach().cpu().numpy().copy() for k, v in self.w.items()}

    def _buf(self, shape, dtype=None):
        t = self.torch
        return t.empty(shape, dtype=dtype or t.float32, device="cuda")

    def forward(self, X):
        """X: (M, 64) int16 bf16 bits on the device -> H1, H2 (bf16), Z (FP32 logits)."""
        t, L, st = self.torch, _lib(), _stream()
        M = X.shape[0]
        Zh = self._buf((M, N_HID))
        H1 = self._buf((M, N_HID), t.int16)
        H2 = self._buf((M, N_HID), t.int16)
        Z = self._buf((M, N_OUT))
        _chk(L.ug_mlp_gemm(_p(X), N_IN, 1, _p(self.wb["W1"]), N_HID, 1, _p(Zh), N_HID, M, N_HID, N_IN, 0, st))
        _chk(L.ug_mlp_bias_act(_p(Zh), _p(self.w["b1"]), _p(H1), None, M, N_HID, 1, st))
        _chk(L.ug_mlp_gemm(_p(H1), N_HID, 1, _p(self.wb["W2"]), N_HID, 1, _p(Zh), N_HID, M, N_HID, N_HID, 0, st))
        _chk(L.ug_mlp_bias_act(_p(Zh), _p(self.w["b2"]), _p(H2), None, M, N_HID, 1, st))
        _chk(L.ug_mlp_gemm(_p(H2), N_HID, 1, _p(self.wb["W3"]), N_OUT, 1, _p(Z), N_OUT, M, N_OUT, N_HID, 0, st))
        _chk(L.ug_mlp_bias_act(_p(Z), _p(self.w["b3"]), None, _p(Z), M, N_OUT, 0, st))
        return H1, H2, Z

    def grads(self, X, T, R):
        """Mean soft-target cross-entropy over rows with n_rot > 1 and its
        gradients with respect to every weight."""
        t, L, st = self.torch, _lib(), _stream()
        M = X.shape[0]
        H1, H2, Z = self.forward(X)
        n_valid = max(1, int((R > 1).sum().item()))
        dZ = self._buf((M, N_OUT))
        loss = t.zeros(1, device="cuda")
        _chk(L.ug_mlp_softmax_xent(_p(Z), _p(T), _p(R), _p(dZ), _p(loss), M, ctypes.c_float(1.0 / n_valid), st))
        g = {k: t.zeros_like(v) for k, v in self.w.items()}
        dZb = self._buf((M, N_OUT), t.int16)
        _chk(L.ug_mlp_to_bf16(_p(dZ), None, _p(dZb), M * N_OUT, st))
        # layer 3: dW3 = H2^T dZ, db3 = sum dZ, dH2 = dZ W3^T
        _chk(L.ug_mlp_gemm(_p(H2), 1, N_HID, _p(dZb), N_OUT, 1, _p(g["W3"]), N_OUT, N_HID, N_OUT, M, 0, st))
        _chk(L.ug_mlp_colsum(_p(dZ), _p(g["b3"]), M, N_OUT, st))
        dH = self._buf((M, N_HID))
        _chk(L.ug_mlp_gemm(_p(dZb), N_OUT, 1, _p(self.wb["W3"]), 1, N_OUT, _p(dH), N_HID, M, N_HID, N_OUT, 0, st))
        dHb = self._buf((M, N_HID), t.int16)
        _chk(L.ug_mlp_to_bf16(_p(dH), _p(H2), _p(dHb), M * N_HID, st))
        # layer 2
        _chk(L.ug_mlp_gemm(_p(H1), 1, N_HID, _p(dHb), N_HID, 1, _p(g["W2"]), N_HID, N_HID, N_HID, M, 0, st))
        _chk(L.ug_mlp_colsum(_p(dH), _p(g["b2"]), M, N_HID, st))
        dH1 = self._buf((M, N_HID))
        _chk(L.ug_mlp_gemm(_p(dHb), N_HID, 1, _p(self.wb["W2"]), 1, N_HID, _p(dH1), N_HID, M, N_HID, N_HID, 0, st))
        dH1b = self._buf((M, N_HID), t.int16)
        _chk(L.ug_mlp_to_bf16(_p(dH1), _p(H1), _p(dH1b), M * N_HID, st))
        # layer 1
        _chk(L.ug_mlp_gemm(_p(X), 1, N_IN, _p(dH1b), N_HID, 1, _p(g["W1"]), N_HID, N_IN, N_HID, M, 0, st))
        _chk(L.ug_mlp_colsum(_p(dH1), _p(g["b1"]), M, N_HID, st))
        return float(loss.item()), g

    def step(self, g, lr):
        L, st = _lib(), _stream()
        self.step_no += 1
        for k, w in self.w.items():
            wb = self.wb.get(k)
            _chk(L.ug_mlp_adam(_p(w), _p(g[k]), _p(self.m[k]), _p(self.v[k]), _p(wb) if wb is not None else None,
                               w.numel(), ctypes.c_float(lr), ctypes.c_float(0.9), ctypes.c_float(0.999),
                               ctypes.c_float(1e-8), self.step_no, st))

    def loss(self, X, T, R, batch=16384):
        tot, n = 0.0, 0
        for i in range(0, X.shape[0], batch):
            l, _ = self.grads(X[i:i + batch], T[i:i + batch], R[i:i + batch])
            k = int((R[i:i + batch] > 1).sum().item())
            tot += l * k
            n += k
        return tot / max(n, 1)


def to_device(X, T, R):
    import torch
    return (torch.tensor(to_bf16_bits(X), device="cuda"), torch.tensor(np.asarray(T, np.float32), device="cuda"),
            torch.tensor(np.asarray(R, np.int32), device="cuda"))


def train(net, data, val, epochs, batch, lr, seed=0):
    import torch
    X, T, R = data
    n = X.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to("cuda")
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch]
            _, gr = net.grads(X[idx].contiguous(), T[idx].contiguous(), R[idx].contiguous())
            net.step(gr, lr_ep)
        hist.append((ep, net.loss(*data), net.loss(*val)))
    return hist


def sweeps_per_solve(batch, n_eval):
    """mean BP sweeps per system over n_eval force evaluations at the
    batch's current coordinates (first sweep included)."""
    its = []
    for _ in range(n_eval):
        batch.evaluate(want_deriv=False)
        its.append(batch.value_by_name(ROTAMER, "n_iter", batch.n_sys))
    return float(np.mean(its)) + 1.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--workload", default="C4")
    ap.add_argument("--train-seeds", default="101,102,103")
    ap.add_argument("--val-seed", type=int, default=104)
    ap.add_argument("--frames", type=int, default=8)
    ap.add_argument("--rounds-between", type=int, default=15)
    ap.add_argument("--warmup-rounds", type=int, default=30)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    a = ap.parse_args()
    import workloads
    t0 = time.time()
    parts = []
    for s in [int(x) for x in a.train_seeds.split(",")]:
        W = workloads.workload(a.workload, seed=s)
        parts.append(collect(W["configs"], W["temps"], W["seeds"], a.frames, a.rounds_between, a.warmup_rounds))
    Xtr = np.concatenate([p[0] for p in parts])
    Ttr = np.concatenate([p[1] for p in parts])
    Rtr = np.concatenate([p[2] for p in parts])
    Wv = workloads.workload(a.workload, seed=a.val_seed)
    Xv, Tv, Rv = collect(Wv["configs"], Wv["temps"], Wv["seeds"], 2, a.rounds_between, a.warmup_rounds)
    t_data = time.time() - t0
    net = WarmNet(seed=0)
    hist = train(net, to_device(Xtr, Ttr, Rtr), to_device(Xv, Tv, Rv), a.epochs, a.batch, a.lr)
    w = net.numpy()
    np.savez(a.out, **w)
    print(json.dumps({"samples": int(Xtr.shape[0]), "val_samples": int(Xv.shape[0]), "data_s": t_data,
                      "train_s": time.time() - t0 - t_data, "loss": [[e, lt, lv] for e, lt, lv in hist],
                      "out": a.out}))


def load(path=WEIGHTS):
    z = np.load(path)
    return {k: z[k] for k in ("W1", "b1", "W2", "b2", "W3", "b3")}


if __name__ == "__main__":
    main()
