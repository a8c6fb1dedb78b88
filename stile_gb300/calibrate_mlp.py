"""Measure ELL-tile timings of this package's kernel on the GPU and train
the learned cost model on them (the reference's MLP_train_cost_model.py
trains on A100 timings of its own kernels the same way).

Each sample is a random ELL tile kind: a shape (I, 32, K) with I*K = 8*mbs,
per-row fills, a column footprint and owned / atomic rows.  A fake operator
holding sm_num * R / 4 tiles of that kind is timed and the time per wave of
sm_num tiles is the label, as in calibrate.py.  Every sample also records
the analytic model's prediction, so the two methods are compared on the same
held-out samples.

Usage on a GPU:
  python -m stile_gb300.calibrate_mlp --samples 480 \\
      --data stile_gb300/gb300_ell_timings.npz --model stile_gb300/gb300_mlp_cost_model.json
"""
from __future__ import annotations

import argparse
import math

import numpy as np

from .calibrate import R, _empty_tc, _time
from .cost_model import gb300_model
from .device import TC_BF16, SpmmDevice
from .mlp_cost import MlpCostModel, ell_tile_features, train_net


def fake_ell_rows(n_tiles, I, K, lens, footprint, atomic, n_cols, rng):
    """n_tiles ELL tiles of I rows x K slots; row r of every tile holds
    lens[r] live slots with columns drawn from a per-tile pool of
    `footprint` columns.  Returns the layout and the distinct columns of
    the first tile."""
    n_rows = n_tiles * I
    kidx = np.zeros((n_tiles, I, K), np.int32)
    first_distinct = 0
    for t in range(n_tiles):
        pool = rng.choice(n_cols, size=max(footprint, 1), replace=False)
        kidx[t] = rng.choice(pool, size=(I, K))
        if t == 0:
            live = np.concatenate([kidx[0, r, :lens[r]] for r in range(I)]) if lens.sum() else np.zeros(0)
            first_distinct = len(np.unique(live))
    row_len = np.tile(lens.astype(np.int32), n_tiles)
    if atomic:
        orow = (np.arange(n_rows) % max(1, n_rows // 4)).astype(np.int32)
    else:
        orow = np.arange(n_rows, dtype=np.int32)
    d = dict(M=int(orow.max()) + 1, K=n_cols, nnz=0, tc_mode=TC_BF16, zero_rows=np.zeros(0, np.int32),
             ell_item_row0=(np.arange(n_tiles + 1) * I).astype(np.int32), ell_item_K=np.full(n_tiles, K, np.int32),
             ell_item_slot0=(np.arange(n_tiles) * I * K).astype(np.int32),
             ell_item_flags=np.full(n_tiles, 1 if atomic else 0, np.int32), ell_out_row=orow, ell_row_len=row_len,
             ell_vals=rng.uniform(-1, 1, n_rows * K).astype(np.float32), ell_kidx=kidx.reshape(-1),
             ell_nnz_id=np.full(n_rows * K, -1, np.int32))
    d.update(_empty_tc())
    return SpmmDevice(**d), first_distinct


def measure(samples, N=128, mbs=32, seed=0, verbose=True):
    import torch
    from .ops import DeviceSpmmPlan
    rng = np.random.default_rng(seed)
    sm_num = torch.cuda.get_device_properties(0).multi_processor_count
    n_cols = 1 << 20
    B = torch.randn(n_cols, N, device="cuda")
    model = gb300_model()
    shapes = [(8 * mbs // K, K) for K in [2 ** t for t in range(int(math.log2(mbs)) + 1)] if 8 * mbs // K >= 8]
    rows = []
    for s in range(samples):
        I, K = shapes[rng.integers(len(shapes))]
        lo = int(rng.integers(0, K + 1))
        lens = rng.integers(lo, K + 1, size=I)
        lens[rng.random(I) < rng.uniform(0.0, 0.5)] = 0
        if lens.sum() == 0:
            lens[0] = 1
        nnz = int(lens.sum())
        footprint = int(np.clip(np.exp(rng.uniform(0, math.log(nnz + 1))), 1, nnz))
        atomic = bool(rng.integers(2))
        dev, distinct = fake_ell_rows(sm_num * R // 4, I, K, lens, footprint, atomic, n_cols, rng)
        p = DeviceSpmmPlan(dev)
        out = torch.empty((dev.M, N), device="cuda")
        ms = _time(lambda: p.run(B, out=out), reps=10) * 4 / R
        p.close()
        k_is = distinct + (1 if nnz < I * K else 0)
        analytic = float(model.ell_costs(I, 32, K, np.array([k_is]), atomic)[0])
        f = ell_tile_features(I, K, lens[None, :], np.array([distinct]), N)[0]
        rows.append((f, atomic, math.log(ms), math.log(max(analytic, 1e-9)), I, K, nnz, distinct))
        if verbose and s % 40 == 0:
            print(f"sample {s}: I={I} K={K} nnz={nnz} distinct={distinct} atomic={atomic} "
                  f"ms/wave={ms:.5f} analytic={analytic:.5f}", flush=True)
    return {"features": np.stack([r[0] for r in rows]).astype(np.float32),
            "atomic": np.array([r[1] for r in rows]),
            "log_ms": np.array([r[2] for r in rows]),
            "analytic_log_ms": np.array([r[3] for r in rows]),
            "shape": np.array([[r[4], r[5], r[6], r[7]] for r in rows], dtype=np.int64)}


def split(n, seed=1, test_frac=0.2):
    """Held-out mask (deterministic in seed)."""
    rng = np.random.default_rng(seed)
    return rng.random(n) < test_frac


def train(data, epochs=3000, verbose=True):
    test = split(len(data["log_ms"]))
    nets, meta = {}, {}
    for kind, atomic in (("owned", False), ("atomic", True)):
        sel = (data["atomic"] == atomic) & ~test
        net, hist = train_net(data["features"][sel], data["log_ms"][sel], epochs=epochs, log_every=500)
        nets[kind] = net
        te = (data["atomic"] == atomic) & test
        pred = net.predict(data["features"][te])
        mlp_err = float(np.mean(np.abs(pred - data["log_ms"][te])))
        ana_err = float(np.mean(np.abs(data["analytic_log_ms"][te] - data["log_ms"][te])))
        meta[kind] = {"train": int(sel.sum()), "test": int(te.sum()), "test_mean_abs_log_err_mlp": mlp_err,
                      "test_mean_abs_log_err_analytic": ana_err, "loss_history": hist}
        if verbose:
            print(kind, meta[kind], flush=True)
    return MlpCostModel(nets["owned"], nets["atomic"], meta=meta)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=480)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--data", required=True)
    ap.add_argument("--model", required=True)
    args = ap.parse_args()
    data = measure(args.samples)
    np.savez_compressed(args.data, **data)
    m = train(data, epochs=args.epochs)
    with open(args.model, "w") as f:
        f.write(m.to_json())
    print("wrote", args.data, args.model)


if __name__ == "__main__":
    main()
