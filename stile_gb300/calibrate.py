"""Recalibrate the tile cost model on the GB300 from timings of this
package's own kernels.

Method (the reference's, MY_sparse/SPMM_get_cost_model_TC.py:15-28,
:205-217 and SPMM_get_cost_model_ELL.py:36-95): build a fake operator that
holds SM_num x R copies of one tile kind, time the fused kernel, and take
time / R as the tile's cost "per wave of SM_num tiles".

* tensor-core tiles (16, 32, K), K = 16..160: owned and atomic tables;
* ELL tiles (I, 32, K) with I*K = 8*mbs: sampled fills and column
  footprints, refit of cost = a1*x + b1 (owned) and the atomic factor
  (a2*x_atomic/x + b2), x = FLOPs / roofline throughput as in the analytic
  model;
* 1D SDDMM chunks: refit of cost = a*x + b.

Usage on a GPU:  python -m stile_gb300.calibrate [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import math
import os

import numpy as np

from .cost_model import A100_FP16, GB300_CALIBRATION, CostModel
from .device import TC_BF16, SddmmDevice, SpmmDevice, _to_bf16_bits, operand_image_16bit

R = 100


def _time(fn, reps=20):
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    return float(np.median(ts))


def _empty_ell():
    z = np.zeros(0, np.int32)
    return dict(ell_item_row0=np.zeros(1, np.int32), ell_item_K=z, ell_item_slot0=z, ell_item_flags=z,
                ell_out_row=z, ell_row_len=z, ell_vals=np.zeros(0, np.float32), ell_kidx=z, ell_nnz_id=z)


def _empty_tc():
    z = np.zeros(0, np.int32)
    return dict(tc_item_kbeg=np.zeros(1, np.int32), tc_item_flags=z, tc_out_rows=z, tc_cols=z,
                tc_vals=np.zeros(0, np.uint8), tc_kstep_bytes=512, tc_nnz_id=z,
                tc_values_f32=np.zeros((0, 16, 16), np.float32))


def fake_tc_layout(n_tiles, K, atomic, n_cols, rng):
    """n_tiles dense 16 x K blocks; owned tiles write distinct row blocks,
    atomic tiles pile 8 tiles onto every row block."""
    nsub = K // 16
    n_ks = n_tiles * nsub
    cols = rng.integers(0, n_cols, size=(n_ks, 16)).astype(np.int32)
    vals = rng.uniform(-1, 1, size=(n_ks, 16, 16)).astype(np.float32)
    img = operand_image_16bit(_to_bf16_bits(vals).reshape(n_ks, 16, 16))
    if atomic:
        blk = np.arange(n_tiles) // 8
    else:
        blk = np.arange(n_tiles)
    rows = (blk[:, None] * 16 + np.arange(16)[None, :]).astype(np.int32)
    M = int(rows.max()) + 1
    zero = np.unique(rows).astype(np.int32) if atomic else np.zeros(0, np.int32)
    d = dict(M=M, K=n_cols, nnz=0, tc_mode=TC_BF16,
             tc_item_kbeg=(np.arange(n_tiles + 1) * nsub).astype(np.int32),
             tc_item_flags=np.full(n_tiles, 1 if atomic else 0, np.int32), tc_out_rows=rows.reshape(-1),
             tc_cols=cols.reshape(-1), tc_vals=np.ascontiguousarray(img).view(np.uint8).reshape(-1),
             tc_kstep_bytes=512, tc_nnz_id=np.full(n_ks * 256, -1, np.int32), tc_values_f32=vals,
             zero_rows=zero)
    d.update(_empty_ell())
    return SpmmDevice(**d)


def fake_ell_layout(n_tiles, I, K, fill, footprint, atomic, n_cols, rng):
    """n_tiles ELL tiles of I rows x K slots; each row holds ``fill`` live
    slots whose columns come from a per-tile pool of ``footprint`` columns."""
    n_rows = n_tiles * I
    kidx = np.empty((n_tiles, I, K), np.int32)
    for t in range(n_tiles):
        pool = rng.choice(n_cols, size=max(footprint, 1), replace=False)
        kidx[t] = rng.choice(pool, size=(I, K))
    lens = np.full(n_rows, fill, np.int32)
    if atomic:
        orow = (np.arange(n_rows) % max(1, n_rows // 4)).astype(np.int32)
        zero = np.unique(orow).astype(np.int32)
    else:
        orow = np.arange(n_rows, dtype=np.int32)
        zero = np.zeros(0, np.int32)
    d = dict(M=int(orow.max()) + 1, K=n_cols, nnz=0, tc_mode=TC_BF16, zero_rows=zero,
             ell_item_row0=(np.arange(n_tiles + 1) * I).astype(np.int32), ell_item_K=np.full(n_tiles, K, np.int32),
             ell_item_slot0=(np.arange(n_tiles) * I * K).astype(np.int32),
             ell_item_flags=np.full(n_tiles, 1 if atomic else 0, np.int32), ell_out_row=orow, ell_row_len=lens,
             ell_vals=rng.uniform(-1, 1, n_rows * K).astype(np.float32), ell_kidx=kidx.reshape(-1),
             ell_nnz_id=np.full(n_rows * K, -1, np.int32))
    d.update(_empty_tc())
    return SpmmDevice(**d)


def calibrate(N=32, mbs=32, sm_num=None, seed=0, verbose=True):
    import torch
    from .ops import DeviceSddmmPlan, DeviceSpmmPlan
    rng = np.random.default_rng(seed)
    if sm_num is None:
        sm_num = torch.cuda.get_device_properties(0).multi_processor_count
    n_cols = 1 << 20
    B = torch.randn(n_cols, N, device="cuda")
    model = CostModel(name=f"gb300_measured_N{N}", dsize=16, sm_num=sm_num, tp_cap=A100_FP16.tp_cap)
    n_tiles = sm_num * R
    # tensor-core tables
    for atomic in (False, True):
        table = {}
        for K in range(16, 161, 16):
            dev = fake_tc_layout(n_tiles, K, atomic, n_cols, rng)
            p = DeviceSpmmPlan(dev)
            out = torch.empty((dev.M, N), device="cuda")
            ms = _time(lambda: p.run(B, out=out))
            table[K] = ms / R
            p.close()
        if atomic:
            model.tc_atomic = table
        else:
            model.tc_owned = table
        if verbose:
            print("tc", "atomic" if atomic else "owned", table, flush=True)
    # ELL fit
    samples = {False: [], True: []}
    shapes = [(8 * mbs // K, 32, K) for K in [2 ** t for t in range(int(math.log2(mbs)) + 1)]
              if (8 * mbs // K) >= 8]
    for (I, J, K) in shapes:
        for fill in sorted({max(1, K // 2), K}):
            for footprint in sorted({max(1, fill), I * fill // 4 + 1, I * fill}):
                kis = min(footprint, I * fill)
                cls = 32 * 8 / model.dsize
                compute = I * J * K * 2
                mem = math.ceil(I * K / cls) + math.ceil(J / cls) * kis + math.ceil(J * model.dsize / 256) * I
                mem_at = mem + math.ceil(J * model.dsize / 256) * I
                x = compute / min(compute / (mem * 32), model.tp_cap)
                xa = compute / min(compute / (mem_at * 32), model.tp_cap)
                for atomic in (False, True):
                    dev = fake_ell_layout(n_tiles // 4, I, K, fill, footprint, atomic, n_cols, rng)
                    p = DeviceSpmmPlan(dev)
                    out = torch.empty((dev.M, N), device="cuda")
                    ms = _time(lambda: p.run(B, out=out)) * 4 / R
                    samples[atomic].append((x, xa, ms))
                    p.close()
    xs = np.array([s[0] for s in samples[False]])
    ys = np.array([s[2] for s in samples[False]])
    a1, b1 = np.polyfit(xs, ys, 1)
    own = {round(s[0], 3): s[2] for s in samples[False]}
    ratio_x, ratio_y = [], []
    for (x, xa, ms) in samples[True]:
        base = a1 * x + b1
        ratio_x.append(xa / x)
        ratio_y.append(ms / base)
    a2, b2 = np.polyfit(np.array(ratio_x), np.array(ratio_y), 1)
    model.ell_owned = (float(a1), float(b1))
    model.ell_atomic = (float(a2), float(b2))
    if verbose:
        print("ell owned fit", model.ell_owned, "atomic factor fit", model.ell_atomic, flush=True)
    del own
    # 1D SDDMM fit
    X = torch.randn(n_cols, N, device="cuda")
    pts = []
    for rows_per in (1, 4, 16, 32):
        for cols_per in (1, 8, 32):
            n_chunks = n_tiles
            mid = np.repeat(rng.integers(0, n_cols, size=(n_chunks, rows_per)), math.ceil(32 / rows_per), axis=1)[:, :32]
            jj = np.repeat(rng.integers(0, n_cols, size=(n_chunks, cols_per)), math.ceil(32 / cols_per), axis=1)[:, :32]
            nnz = n_chunks * 32
            dev = SddmmDevice(M=n_cols, K=n_cols, nnz=nnz, mid_idx=mid.reshape(-1).astype(np.int32),
                              j_idx=jj.reshape(-1).astype(np.int32), remap=np.arange(nnz, dtype=np.int32),
                              bm=16, bn=16, blk_i=np.zeros(0, np.int32), blk_j=np.zeros(0, np.int32),
                              blk_indptr=np.zeros(1, np.int32), blk_dense_pos=np.zeros(0, np.int32),
                              blk_out=np.zeros(0, np.int32))
            p = DeviceSddmmPlan(dev)
            out = torch.empty(nnz, device="cuda")
            ms = _time(lambda: p.run(X, B, out=out)) / R
            compute = N * 32 * 2
            mem = ((rows_per + cols_per) * N + 32) * model.dsize / 8
            x = compute / min(compute / mem, model.tp_cap)
            pts.append((x, ms))
            p.close()
    a, b = np.polyfit([p_[0] for p_ in pts], [p_[1] for p_ in pts], 1)
    model.one_d = (float(a), float(b))
    if verbose:
        print("1d fit", model.one_d, flush=True)
    calibrate_tc_sddmm(model, rng, verbose=verbose)
    return model


def fake_tc_sddmm_layout(n_tiles, n_cols, rng):
    """n_tiles full 16 x 16 SDDMM blocks on random rows and columns."""
    bi = rng.integers(0, n_cols, size=(n_tiles, 16)).astype(np.int32)
    bj = rng.integers(0, n_cols, size=(n_tiles, 16)).astype(np.int32)
    nnz = n_tiles * 256
    z = np.zeros(0, np.int32)
    return SddmmDevice(M=n_cols, K=n_cols, nnz=nnz, mid_idx=z, j_idx=z, remap=z, bm=16, bn=16,
                       blk_i=bi.reshape(-1), blk_j=bj.reshape(-1),
                       blk_indptr=(np.arange(n_tiles + 1) * 256).astype(np.int32),
                       blk_dense_pos=np.tile(np.arange(256, dtype=np.int32), n_tiles),
                       blk_out=np.arange(nnz, dtype=np.int32))


def calibrate_tc_sddmm(model, rng, verbose=True):
    """Tensor-core SDDMM block table: the per-wave cost of 16 x 16 blocks
    with J features (the entry (J, 16) the search reads), measured with this
    package's block kernel; the reference's A100 entries for other block
    widths are kept, scaled by the measured (J, 16) ratio."""
    import torch
    from .ops import DeviceSddmmPlan
    n_cols = 1 << 20
    n_tiles = model.sm_num * R
    table = dict(A100_FP16.tc_sddmm)
    for J in (16, 32, 64):
        X = torch.randn(n_cols, J, device="cuda")
        Y = torch.randn(n_cols, J, device="cuda")
        dev = fake_tc_sddmm_layout(n_tiles, n_cols, rng)
        p = DeviceSddmmPlan(dev)
        out = torch.empty(dev.nnz, device="cuda")
        ms = _time(lambda: p.run(X, Y, out=out)) / R
        p.close()
        ratio = ms / A100_FP16.tc_sddmm[(J, 16)]
        for (j, k), v in A100_FP16.tc_sddmm.items():
            if j == J:
                table[(j, k)] = v * ratio
        table[(J, 16)] = ms
    model.tc_sddmm = table
    if verbose:
        print("tc sddmm", {k: v for k, v in table.items() if k[1] == 16}, flush=True)
    return model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=GB300_CALIBRATION)
    ap.add_argument("--N", type=int, default=32)
    ap.add_argument("--only-tc-sddmm", action="store_true",
                    help="re-measure only the SDDMM block table of the installed calibration")
    args = ap.parse_args()
    if args.only_tc_sddmm:
        with open(GB300_CALIBRATION) as f:
            m = CostModel.from_json(f.read())
        calibrate_tc_sddmm(m, np.random.default_rng(0))
    else:
        m = calibrate(N=args.N)
    with open(args.out, "w") as f:
        f.write(m.to_json())
    print("wrote", args.out)


if __name__ == "__main__":
    main()
