"""The learned surrogate of the simulator for delayed-acceptance MCMC.

``MLP`` wraps the tensor-core network of the native library (arbo_mlp_*, BF16 operands, FP32
accumulation, Adam). ``Surrogate`` maps a parameter vector of the prior box to the simulator's
monthly incidence per serotype (the network predicts log(1 + cases)) and turns the prediction into
the negative-binomial log-likelihood of the observed reported cases; ``training_set`` draws
parameter vectors uniformly from the prior box and runs the simulator on them in batches.
"""
from __future__ import annotations

import ctypes
import math
from ctypes import POINTER, byref, c_float, c_uint32, c_void_p
from typing import Optional

import numpy as np

from . import configs
from ._native import check, load
from .mcmc import chain_batch, month_rows, monthly, sim_seed

_F = POINTER(c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_F)


class MLP:
    """hidden_layers SiLU layers of `hidden` units and a linear output, trained on the GPU."""

    def __init__(self, n_in: int, hidden: int, hidden_layers: int, n_out: int, max_batch: int = 512, seed: int = 1):
        self._lib = load()
        h = c_void_p()
        check(self._lib.arbo_mlp_create(n_in, hidden, hidden_layers, n_out, max_batch, seed, byref(h)))
        self._h = h
        self.n_in, self.n_out, self.max_batch = n_in, n_out, max_batch
        L = c_uint32()
        dims = (c_uint32 * (hidden_layers + 2))()
        check(self._lib.arbo_mlp_dims(h, byref(L), dims))
        self.layers = L.value
        self.dims = list(dims[: self.layers + 1])

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.arbo_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        pad = (-n) % 16
        if pad:
            x = np.concatenate([x, np.zeros((pad, x.shape[1]), np.float32)])
        out = np.zeros((x.shape[0], self.n_out), np.float32)
        for i in range(0, x.shape[0], self.max_batch):
            xb = np.ascontiguousarray(x[i:i + self.max_batch])
            yb = np.zeros((xb.shape[0], self.n_out), np.float32)
            check(self._lib.arbo_mlp_forward(self._h, _fp(xb), xb.shape[0], _fp(yb), None))
            out[i:i + xb.shape[0]] = yb
        return out[:n]

    def gradients(self, x: np.ndarray, t: np.ndarray) -> float:
        x, t = np.ascontiguousarray(x, np.float32), np.ascontiguousarray(t, np.float32)
        loss = c_float()
        check(self._lib.arbo_mlp_gradients(self._h, _fp(x), _fp(t), x.shape[0], byref(loss), None))
        return loss.value

    def train_step(self, x: np.ndarray, t: np.ndarray, lr: float) -> float:
        x, t = np.ascontiguousarray(x, np.float32), np.ascontiguousarray(t, np.float32)
        loss = c_float()
        check(self._lib.arbo_mlp_train_step(self._h, _fp(x), _fp(t), x.shape[0], float(lr), byref(loss), None))
        return loss.value

    def layer(self, l: int):
        i, o = self.dims[l], self.dims[l + 1]
        w, dw = np.zeros((o, i), np.float32), np.zeros((o, i), np.float32)
        b, db = np.zeros(o, np.float32), np.zeros(o, np.float32)
        check(self._lib.arbo_mlp_get_layer(self._h, l, _fp(w), _fp(b), _fp(dw), _fp(db)))
        return w, b, dw, db

    def set_layer(self, l: int, w: np.ndarray, b: np.ndarray) -> None:
        w, b = np.ascontiguousarray(w, np.float32), np.ascontiguousarray(b, np.float32)
        check(self._lib.arbo_mlp_set_layer(self._h, l, _fp(w), _fp(b)))


def tc_gemm(a: np.ndarray, b: np.ndarray, reps: int = 0):
    """c = bf16(a) @ bf16(b).T on the tensor cores (FP32 result), with the mean ms per launch."""
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    M, K = a.shape
    N = b.shape[0]
    c = np.zeros((M, N), np.float32)
    ms = c_float()
    check(load().arbo_tc_gemm(_fp(a), _fp(b), M, N, K, _fp(c), reps, byref(ms)))
    return c, ms.value


def normalize(theta: np.ndarray, box=None) -> np.ndarray:
    box = box if box is not None else configs.PRIOR_BOX
    lo = np.array([b[1] for b in box])
    hi = np.array([b[2] for b in box])
    return (2.0 * (np.asarray(theta) - lo) / (hi - lo) - 1.0).astype(np.float32)


def nb_loglik(observed: np.ndarray, mean: np.ndarray, size: float = 10.0) -> np.ndarray:
    """Negative-binomial log-likelihood of observed [months, S] under means [n, months, S], in FP64,
    floored at -250 per cell like the simulator-based likelihood. Returns [n]."""
    k = observed.astype(np.float64)[None]
    mu = np.maximum(np.asarray(mean, np.float64), 0.0)
    lg = np.vectorize(math.lgamma)
    const = lg(k + size) - math.lgamma(size) - lg(k + 1.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = const - size * np.log1p(mu / size) + k * (np.log(mu) - np.log(size + mu))
    v = np.where(mu > 0, v, np.where(k == 0, 0.0, -np.inf))
    return np.maximum(v, -250.0).sum(axis=(1, 2))


class Surrogate:
    """theta (prior box) -> monthly incidence per serotype, and the surrogate log-likelihood."""

    def __init__(self, months: int, serotypes: int, hidden: int = 512, hidden_layers: int = 4, seed: int = 1,
                 max_batch: int = 512, report_param: int = 5, box=None):
        self.months, self.S = months, serotypes
        self.box = box if box is not None else configs.PRIOR_BOX
        self.report = report_param
        self.net = MLP(len(self.box), hidden, hidden_layers, months * serotypes, max_batch, seed)

    def fit(self, theta: np.ndarray, incidence: np.ndarray, epochs: int, batch: int = 256, lr: float = 1e-3,
            seed: int = 0, decay: float = 0.0):
        """Trains on (theta [n, D], monthly incidence [n, months, S]); returns the loss per epoch."""
        x = normalize(theta, self.box)
        y = np.log1p(np.asarray(incidence, np.float64)).reshape(len(x), -1).astype(np.float32)
        rng = np.random.default_rng(seed)
        losses = []
        n = len(x) - len(x) % batch
        for ep in range(epochs):
            order = rng.permutation(len(x))[:n]
            rate = lr / (1.0 + decay * ep)
            acc = 0.0
            for i in range(0, n, batch):
                idx = order[i:i + batch]
                acc += self.net.train_step(x[idx], y[idx], rate)
            losses.append(acc / max(1, n // batch))
        return np.array(losses)

    def predict(self, theta: np.ndarray) -> np.ndarray:
        out = self.net.forward(normalize(np.atleast_2d(theta), self.box))
        return np.expm1(np.maximum(out, 0.0)).reshape(-1, self.months, self.S)

    def loglik(self, theta: np.ndarray, observed: np.ndarray, size: float = 10.0) -> np.ndarray:
        theta = np.atleast_2d(theta)
        return nb_loglik(observed, theta[:, self.report][:, None, None] * self.predict(theta), size)


def training_set(workload: configs.Workload, n: int, months: int, seed: int = 0, batch_size: int = 64,
                 box=None, on_batch=None):
    """n parameter vectors uniform in the prior box and the simulator's monthly incidence for each,
    simulated in batches of batch_size instances (arbo_batch_*)."""
    from .simulation import Simulation

    box = box if box is not None else configs.PRIOR_BOX
    lo = np.array([b[1] for b in box])
    hi = np.array([b[2] for b in box])
    rng = np.random.default_rng(seed)
    theta = lo + (hi - lo) * rng.uniform(size=(n, len(box)))
    rows = month_rows(workload.max_time, months)
    w = workload
    sims = [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
            for _ in range(min(batch_size, n))]
    inc = np.zeros((n, months, int(w.parameter.simulation.nStrains)), np.int64)
    try:
        with chain_batch(sims) as b:
            for i0 in range(0, n, len(sims)):
                k = min(len(sims), n - i0)
                b.set_params([configs.apply_theta(w.parameter.simulation, theta[min(i0 + j, n - 1)])
                              for j in range(len(sims))],
                             [sim_seed(w.seed ^ 0x5A5A, i0 + j, 0, 0) for j in range(len(sims))])
                b.init()
                b.run()
                for j in range(k):
                    inc[i0 + j] = monthly(sims[j].series("n_incidence"), rows)
                if on_batch:
                    on_batch(i0 + k)
    finally:
        for s in sims:
            s.close()
    return theta, inc


def main(argv=None):
    """python -m arbo_gpu_fit_gb300.surrogate gemm M N K [reps]: one tensor-core product of
    standard-normal inputs (rounded to BF16), timed over reps launches; prints M N K ms TFLOP/s."""
    import sys

    from . import _native

    args = list(sys.argv[1:] if argv is None else argv)
    if len(args) < 4 or args[0] != "gemm":
        raise SystemExit(main.__doc__)
    M, N, K = (int(x) for x in args[1:4])
    reps = int(args[4]) if len(args) > 4 else 20
    _native.check(_native.load().arbo_set_device(0))
    rng = np.random.default_rng(1)
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((N, K)).astype(np.float32)
    _, ms = tc_gemm(a, b, reps=reps)
    print(M, N, K, ms, 2.0 * M * N * K / (ms * 1e-3) / 1e12 if ms else 0.0)


if __name__ == "__main__":
    main()
