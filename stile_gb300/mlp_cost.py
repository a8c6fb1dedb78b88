"""Learned cost model for ELL (row-bucket) tiles.

The reference scores ELL tiles with an 18-feature MLP (get_MLP_features_in_batch
and PyTorchMLP, my_cost_model.py:925-1029; training MLP_train_cost_model.py)
trained on its own A100 kernel timings, with the analytic model as the
alternative.  Here a 12-feature network of the same hidden widths is trained
on timings of this package's own GB300 ELL kernel (stile_gb300.calibrate_mlp)
with hand-written CUDA kernels (csrc/mlp.cu: forward, backward, weight
gradients, Adam), and scores all candidate tiles of a search step in one
launch of the fused inference kernel.  Owned and atomic tiles have separate
networks, as in the reference.  Predictions are the log of the cost in ms
per wave of sm_num tiles, the unit of CostModel.

Features of a tile with I rows and K slots, over the uncovered entries of its
rows (row_nnz, I values) and the distinct columns they read:
  log2 I, log2 K, nnz / (I K), mean / max / min row nnz / K,
  distinct / nnz, log2(nnz + 1), log2(distinct + 1), N / 128,
  fraction of non-empty rows, row-nnz standard deviation / K.
"""
from __future__ import annotations

import ctypes
import json
from dataclasses import dataclass, field

import numpy as np

from . import _lib

FEATURES = 12
H1, H2 = 64, 32
N_PARAMS = FEATURES * H1 + H1 + H1 * H2 + H2 + H2 + 1
WORK = 2 * H1 + 2 * H2


def ell_tile_features(I, K, row_nnz, distinct, N):
    """[n, FEATURES] float32 features of n tiles of shape (I, K); row_nnz is
    [n, I] (rows past the operator's end count as empty), distinct [n]."""
    r = np.asarray(row_nnz, dtype=np.float64).reshape(-1, I)
    d = np.asarray(distinct, dtype=np.float64).reshape(-1)
    nnz = r.sum(1)
    f = np.empty((len(r), FEATURES), dtype=np.float64)
    f[:, 0] = np.log2(I)
    f[:, 1] = np.log2(K)
    f[:, 2] = nnz / (I * K)
    f[:, 3] = r.mean(1) / K
    f[:, 4] = r.max(1) / K
    f[:, 5] = r.min(1) / K
    f[:, 6] = d / np.maximum(nnz, 1.0)
    f[:, 7] = np.log2(nnz + 1.0)
    f[:, 8] = np.log2(d + 1.0)
    f[:, 9] = N / 128.0
    f[:, 10] = (r > 0).mean(1)
    f[:, 11] = r.std(1) / K
    return f.astype(np.float32)


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class MlpNet:
    """One network: flat parameters and the feature standardisation."""
    params: np.ndarray
    mean: np.ndarray
    std: np.ndarray

    def standardise(self, x):
        return ((np.asarray(x, dtype=np.float32) - self.mean) / self.std).astype(np.float32)

    def predict(self, x):
        """Network outputs for raw features x [n, FEATURES], computed by the
        fused inference kernel on the current CUDA device."""
        import torch
        x = self.standardise(x)
        n = len(x)
        if n == 0:
            return np.zeros(0, dtype=np.float32)
        lib = _lib.load()
        p = torch.as_tensor(self.params, device="cuda")
        xt = torch.as_tensor(x, device="cuda")
        y = torch.empty(n, device="cuda")
        _lib.check(lib.stile_mlp_forward(p.data_ptr(), xt.data_ptr(), n, y.data_ptr(), _stream()), "stile_mlp_forward")
        return y.cpu().numpy()

    def to_dict(self):
        return {"params": self.params.tolist(), "mean": self.mean.tolist(), "std": self.std.tolist()}

    @staticmethod
    def from_dict(d):
        return MlpNet(np.asarray(d["params"], np.float32), np.asarray(d["mean"], np.float32),
                      np.asarray(d["std"], np.float32))


def init_params(seed, target_mean=0.0):
    """He-initialised weights, zero biases, output bias at the target mean."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((FEATURES, H1)) * np.sqrt(2.0 / FEATURES)
    W2 = rng.standard_normal((H1, H2)) * np.sqrt(2.0 / H1)
    W3 = rng.standard_normal(H2) * np.sqrt(1.0 / H2) * 0.1
    p = np.concatenate([W1.ravel(), np.zeros(H1), W2.ravel(), np.zeros(H2), W3, [target_mean]])
    return p.astype(np.float32)


def train_net(x, t, epochs=3000, lr=3e-3, seed=0, log_every=0):
    """Fit a network to targets t from raw features x with full-batch Adam,
    every step on the GPU (stile_mlp_gradient, stile_mlp_adam)."""
    import torch
    x = np.asarray(x, dtype=np.float32)
    t = np.asarray(t, dtype=np.float32)
    mean = x.mean(0)
    std = x.std(0)
    std[std < 1e-6] = 1.0
    net = MlpNet(init_params(seed, float(t.mean())), mean.astype(np.float32), std.astype(np.float32))
    lib = _lib.load()
    n = len(x)
    p = torch.as_tensor(net.params, device="cuda").contiguous()
    xs = torch.as_tensor(net.standardise(x), device="cuda")
    ts = torch.as_tensor(t, device="cuda")
    work = torch.empty(n * WORK, device="cuda")
    dy = torch.empty(n, device="cuda")
    grad = torch.empty(N_PARAMS, device="cuda")
    loss = torch.empty(1, device="cuda")
    m = torch.zeros(N_PARAMS, device="cuda")
    v = torch.zeros(N_PARAMS, device="cuda")
    st = _stream()
    history = []
    for step in range(1, epochs + 1):
        _lib.check(lib.stile_mlp_gradient(p.data_ptr(), xs.data_ptr(), ts.data_ptr(), n, work.data_ptr(),
                                          dy.data_ptr(), grad.data_ptr(), loss.data_ptr(), st), "stile_mlp_gradient")
        step_lr = lr * (0.1 ** (step / epochs))  # exponential decay to lr / 10
        _lib.check(lib.stile_mlp_adam(p.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(), N_PARAMS,
                                      ctypes.c_float(step_lr), ctypes.c_float(0.9), ctypes.c_float(0.999),
                                      ctypes.c_float(1e-8), step, st), "stile_mlp_adam")
        if log_every and (step % log_every == 0 or step == 1):
            history.append((step, float(loss.item())))
    net.params = p.cpu().numpy()
    return net, history


@dataclass
class MlpCostModel:
    """Owned and atomic ELL-tile networks; costs in ms per wave."""
    owned: MlpNet
    atomic: MlpNet
    name: str = "gb300_mlp"
    meta: dict = field(default_factory=dict)

    def ell_costs(self, I, K, row_nnz, distinct, N, atomic):
        x = ell_tile_features(I, K, row_nnz, distinct, N)
        net = self.atomic if atomic else self.owned
        return np.exp(net.predict(x).astype(np.float64))

    def to_json(self):
        return json.dumps({"name": self.name, "meta": self.meta, "owned": self.owned.to_dict(),
                           "atomic": self.atomic.to_dict()})

    @staticmethod
    def from_json(s):
        d = json.loads(s)
        return MlpCostModel(MlpNet.from_dict(d["owned"]), MlpNet.from_dict(d["atomic"]), d.get("name", "gb300_mlp"),
                            d.get("meta", {}))
