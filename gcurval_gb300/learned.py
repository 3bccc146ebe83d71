"""Learned form: training data from the plain adaptive method, training of
the MLP on the GPU with the library's own FP32 kernels, and the shipped
network (include/gcurval_gb300_learned.h).

    python -m gcurval_gb300.learned --train            # writes MODEL_PATH
    w = load_model()                                   # packed FP32 weights
    calc = ArclengthCalculateGpu.from_batch(b, precision=GCV_MIXED, learned=True)
    calc.set_learned_model(w)

Training pairs: every B-spline knot interval of seeded uneven batches
(the generator of the uneven-batch workload, its own seed), features as the
library computes them, labels from the table the plain FP64 walk builds at
the same tolerance.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _lib
from ._lib import GCV_PLAIN_FP64, check

MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "mlp_uneven.npz")
N_PARAM = 39328  # gcv_mlp_param_count()


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _mcheck(status):
    if status != 0:
        lib = _lib.load()
        raise _lib.GcvError(status, lib.gcv_mlp_last_error().decode() or lib.gcv_last_error().decode())


def load_model(path: str = MODEL_PATH) -> np.ndarray:
    """The packed FP32 weights of a trained network."""
    with np.load(path) as z:
        w = np.ascontiguousarray(z["weights"], np.float32)
    if w.size != N_PARAM:
        raise ValueError(f"{path}: {w.size} weights, {N_PARAM} expected")
    return w


def training_set(n_intervals: int, seed: int, rtol: float = 5e-9, chunk_curves: int = 4000):
    """(X, depth, share, tguess) CUDA tensors of n_intervals B-spline knot
    intervals of positive width, labelled by the plain FP64 walk at rtol."""
    import torch

    import gcurval_gb300 as g
    from . import datasets as ds
    xs, ds_, ss, ts = [], [], [], []
    have, k = 0, 0
    while have < n_intervals:
        b = ds.uneven_batch(chunk_curves, seed=seed * 1000 + k)
        k += 1
        calc = g.ArclengthCalculateGpu.from_batch(b, precision=GCV_PLAIN_FP64, rtol=rtol)
        try:
            calc.createArclengthTable()
            n = calc.n_segments
            X = torch.empty((n, 16), dtype=torch.float32, device="cuda")
            D = torch.empty(n, dtype=torch.int32, device="cuda")
            S = torch.empty((n, 4), dtype=torch.float32, device="cuda")
            T = torch.empty((n, 8), dtype=torch.float32, device="cuda")
            calc.learned_features(X)
            calc.learned_labels(D, S, T)
        finally:
            calc.close()
        keep = X[:, 0] > 0  # B-spline intervals (degree / 5 > 0) ...
        keep &= X[:, 11] > 0  # ... of positive width
        xs.append(X[keep])
        ds_.append(D[keep])
        ss.append(S[keep])
        ts.append(T[keep])
        have += int(keep.sum().item())
    X, D, S, T = (torch.cat(a)[:n_intervals].contiguous() for a in (xs, ds_, ss, ts))
    return X, D, S, T


class Trainer:
    """gcv_mlp_trainer: FP32 forward / backward / Adam on the GPU."""

    def __init__(self, max_batch: int, seed: int = 0, weights: np.ndarray | None = None):
        self.lib = _lib.load()
        self.h = ctypes.c_void_p()
        _mcheck(self.lib.gcv_mlp_trainer_create(ctypes.byref(self.h), int(max_batch), int(seed)))
        self.max_batch = max_batch
        if weights is not None:
            self.set_weights(weights)

    def close(self):
        if self.h:
            self.lib.gcv_mlp_trainer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _mcheck(self.lib.gcv_mlp_trainer_set_weights(self.h, w.ctypes.data_as(ctypes.c_void_p)))

    def weights(self) -> np.ndarray:
        w = np.empty(N_PARAM, np.float32)
        _mcheck(self.lib.gcv_mlp_trainer_get_weights(self.h, w.ctypes.data_as(ctypes.c_void_p)))
        return w

    def forward(self, X):
        import torch
        out = torch.empty((X.shape[0], 32), dtype=torch.float32, device=X.device)
        _mcheck(self.lib.gcv_mlp_trainer_forward(self.h, _ptr(X), int(X.shape[0]), _ptr(out)))
        return out

    def gradients(self, X, D, S, T):
        g = np.empty(N_PARAM, np.float32)
        loss = np.empty(3, np.float32)
        _mcheck(self.lib.gcv_mlp_trainer_gradients(self.h, _ptr(X), _ptr(D), _ptr(S), _ptr(T), int(X.shape[0]),
                                                   g.ctypes.data_as(ctypes.c_void_p),
                                                   loss.ctypes.data_as(ctypes.c_void_p)))
        return g, loss

    def step(self, X, D, S, T, lr: float):
        loss = np.empty(3, np.float32)
        _mcheck(self.lib.gcv_mlp_trainer_step(self.h, _ptr(X), _ptr(D), _ptr(S), _ptr(T), int(X.shape[0]),
                                              ctypes.c_float(lr), loss.ctypes.data_as(ctypes.c_void_p)))
        return loss


def infer(weights: np.ndarray, X):
    """Outputs of the BF16 tensor-core network (gcv_mlp_infer) for CUDA features X."""
    import torch
    lib = _lib.load()
    w = np.ascontiguousarray(weights, np.float32)
    out = torch.empty((X.shape[0], 32), dtype=torch.float32, device=X.device)
    _mcheck(lib.gcv_mlp_infer(w.ctypes.data_as(ctypes.c_void_p), _ptr(X), int(X.shape[0]), _ptr(out)))
    return out


def train(X, D, S, T, epochs: int = 6, batch: int = 8192, lr: float = 2e-3, seed: int = 0, log=print) -> np.ndarray:
    import torch
    tr = Trainer(batch, seed)
    gen = torch.Generator(device=X.device)
    gen.manual_seed(seed)
    n = X.shape[0]
    steps = 0
    total = epochs * ((n + batch - 1) // batch)
    try:
        for ep in range(epochs):
            perm = torch.randperm(n, device=X.device, generator=gen)
            acc = np.zeros(3)
            nb = 0
            for i in range(0, n - batch + 1, batch):
                idx = perm[i:i + batch]
                # cosine decay of the step size
                cur = lr * 0.5 * (1.0 + np.cos(np.pi * steps / total))
                acc += tr.step(X[idx], D[idx], S[idx], T[idx], cur)
                nb += 1
                steps += 1
            log(f"epoch {ep}: loss depth {acc[0] / nb:.4f} split {acc[1] / nb:.4f} t {acc[2] / nb:.5f}")
        return tr.weights()
    finally:
        tr.close()


def evaluate(weights, X, D, S, T) -> dict:
    """Accuracy of the tensor-core network on labelled intervals."""
    import torch
    out = infer(weights, X)
    pred = out[:, :13].argmax(dim=1).to(torch.int32)
    t_err = (out[:, 17:25] - T).abs()
    return {"intervals": int(X.shape[0]),
            "depth_exact": float((pred == D).float().mean().item()),
            "depth_within_1": float(((pred - D).abs() <= 1).float().mean().item()),
            "depth_over": float((pred > D).float().mean().item()),
            "t_mean_abs_err": float(t_err.mean().item())}


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--intervals", type=int, default=5_000_000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--rtol", type=float, default=5e-9, help="the uneven batch's per-interval tolerance")
    ap.add_argument("--out", default=MODEL_PATH)
    a = ap.parse_args(argv)
    if not a.train:
        ap.print_help()
        return
    t0 = time.perf_counter()
    X, D, S, T = training_set(a.intervals, seed=1, rtol=a.rtol)
    t1 = time.perf_counter()
    w = train(X, D, S, T, epochs=a.epochs)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    Xv, Dv, Sv, Tv = training_set(500_000, seed=2, rtol=a.rtol)
    ev = evaluate(w, Xv, Dv, Sv, Tv)
    meta = {"rtol": a.rtol, "intervals": a.intervals, "epochs": a.epochs, "train_seed": 1, "eval_seed": 2,
            "data_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2), "eval": ev}
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    np.savez(a.out, weights=w, meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
