"""Benchmark: hybrid-tile SpMM / SDDMM forward + backward of the two-layer
GCN workload.

Workload (one step): a 232,965-node symmetric power-law graph (degree
exponent 1.9, ~11.4M nonzeros, planted 16x16 communities, values 1/deg) and
the sparse products of a two-layer graph convolution, 602 -> 128 -> 41, with
the dense operands synthetic N(0,1):
    layer 1  C1 = A @ B1 (N = 128)          layer 2  C2 = A @ B2 (N = 41)
    backward dB_l = A^T @ dC_l (transposed plan) and, from the same dC rows,
             dvals_l = <dC_l[row], B_l[col]>           for l = 2, 1
FLOPs per step = 3 * 2 * nnz * (128 + 41).  The dense GEMMs of the GCN
(X W1, Z1 W2) are cuBLAS work outside the metric; the line times the whole
training step of the model for context (``gcn_training_step``).  The
169,343-node graph (one layer, N = 128) is reported in ``secondary``.

Output: one JSON line (metric / value / e2e / roofline / cpu_baseline / ...).
`--impl reference` times the CPU restatement of the same step on the host
cores instead (the reference has no runnable GPU path here).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMM/SDDMM GFLOP/s and %HBM roofline: hybrid-TC vs plain CSR, fwd+bwd, GB300"
WORKLOAD = "gcn2_232965_nnz11.4M_602-128-41_fwd_bwd"
WIDTHS = (128, 41)
GRAPH_WORKLOAD = "hybrid_graph_169343_nnz1.17M_N128_fwd_bwd"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def errors(name, x, ref):
    """Relative Frobenius and max-abs error of x against its float64
    reference."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.linalg.norm(ref)
    return {f"{name}_rel_fro": float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0)),
            f"{name}_max_abs": float(np.abs(x - ref).max()) if x.size else 0.0}


def make_gcn_workload(seed=0):
    """(A, [(B_l, dC_l) for the two layer widths]): the GCN graph and
    synthetic N(0, 1) layer operands (float32, C-contiguous)."""
    from stile_gb300 import synthetic as syn
    from stile_gb300 import workloads as W
    w = W.gcn(WIDTHS[0], seed=seed)
    A = w.A
    layers = [(w.dense["B"], w.dense["dC"])]
    for j, N in enumerate(WIDTHS[1:]):
        layers.append((syn.dense_operand(A.shape[1], N, seed=3 + 2 * j),
                       syn.dense_operand(A.shape[0], N, seed=4 + 2 * j)))
    return A, layers


def make_graph_workload(seed=0):
    from stile_gb300 import workloads as W
    w = W.graph(seed)
    return w.A, [(w.dense["B"], w.dense["dC"])]


def step_flops(A, layers):
    return sum(3 * 2 * A.nnz * B.shape[1] for B, _ in layers)


def algorithmic_bytes_spmm(A, N, s_a=4, s_b=4, s_c=4):
    """Format-independent lower bound on the bytes of one SpMM: row pointers,
    (index, value) per nonzero, every touched B row once, C written once."""
    M = A.shape[0]
    k_touched = int(np.count_nonzero(np.bincount(A.indices, minlength=A.shape[1])))
    return (M + 1) * 4 + A.nnz * (4 + s_a) + k_touched * N * s_b + M * N * s_c


# Random 512-byte fp32 row gathers from L2 measured on this GPU (16-lane
# groups of 128-bit loads, two rows in flight per group, 8 blocks of 256
# threads per SM, 119 MB matrix): the rate the row gathers of a SpMM can
# reach, whatever the HBM roofline says.
GATHER_PEAK_GBS = 16340.0


def gathered_bytes_spmm(op, N, s_b=4):
    """Bytes of B rows one forward of ``op`` gathers: one row per live ELL
    entry and 16 rows per tensor-core k-step (a row of N elements each)."""
    dev = op.device_layout
    n_ell = int((dev.ell_nnz_id >= 0).sum()) if len(dev.ell_nnz_id) else int(np.count_nonzero(dev.ell_row_len))
    return (n_ell + len(dev.tc_cols)) * N * s_b


def algorithmic_bytes_sddmm(A, F, s=4):
    m_t = int(np.count_nonzero(np.diff(A.indptr)))
    n_t = int(np.count_nonzero(np.bincount(A.indices, minlength=A.shape[1])))
    return (A.shape[0] + 1) * 4 + A.nnz * 4 + (m_t + n_t) * F * s + A.nnz * s


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture (profiles/)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class _Nvml:
    """Minimal NVML through ctypes (SM clock, max SM clock, throttle reasons)."""

    HW_SLOWDOWN, SW_THERMAL, HW_THERMAL, SW_POWER_CAP = 0x8, 0x20, 0x40, 0x4

    def __init__(self, index):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise RuntimeError("nvml handle")
        self._reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(self.lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        self.sm_clock()
        self.reasons()

    def sm_clock(self):
        v = self.ct.c_uint()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, self.ct.byref(v))
        return int(v.value)

    def max_sm_clock(self):
        v = self.ct.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, self.ct.byref(v))
        return int(v.value)

    def reasons(self):
        v = self.ct.c_ulonglong()
        self._reasons_fn(self.h, self.ct.byref(v))
        return int(v.value)


class ClockSampler:
    """Samples the SM clock and clock-event reasons during the timed region:
    NVML at ~1 kHz (read-only queries), nvidia-smi as the fallback."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.samples = []
        self.reason_bits = 0
        self.nvml = None
        self.max_mhz = None
        self._stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.gpu)
            self.max_mhz = self.nvml.max_sm_clock()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
        except Exception:
            self.nvml = None
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
                self.thread = threading.Thread(target=self._read, daemon=True)
                self.thread.start()
            except Exception:
                self.proc = None
        return self

    def _poll(self):
        while not self._stop.is_set():
            self.samples.append(self.nvml.sm_clock())
            self.reason_bits |= self.nvml.reasons()
            time.sleep(0.001)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self._stop.set()
        if self.nvml is not None:
            self.thread.join(timeout=2)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None and self.samples:
            names = []
            for bit, nm in ((_Nvml.HW_SLOWDOWN, "hw_slowdown"), (_Nvml.HW_THERMAL, "hw_thermal_slowdown"),
                            (_Nvml.SW_THERMAL, "sw_thermal_slowdown"), (_Nvml.SW_POWER_CAP, "sw_power_cap")):
                if self.reason_bits & bit:
                    names.append(nm)
            return {"sm_mhz": float(np.median(self.samples)), "sm_max_mhz": float(self.max_mhz),
                    "reasons": names, "samples": len(self.samples), "source": "nvml"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi"}


# ---------------------------------------------------------------------------
# CPU (oracle) step
# ---------------------------------------------------------------------------
def cpu_step_fn(A, AT, layers, threads):
    """The step's sparse products on the host: per layer CSR SpMM for A and
    A^T and the gather-dot SDDMM (the C restatement of the reference's CPU
    path)."""
    from oracle import cpu as ocpu
    rows = np.repeat(np.arange(A.shape[0], dtype=np.int32), np.diff(A.indptr))
    ip, ix, vv = A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float32)
    ipt, ixt, vvt = AT.indptr.astype(np.int32), AT.indices.astype(np.int32), AT.data.astype(np.float32)
    cols = A.indices.astype(np.int32)
    bufs = [(np.ascontiguousarray(B, np.float32), np.ascontiguousarray(dC, np.float32),
             np.empty((A.shape[0], B.shape[1]), np.float32), np.empty((A.shape[1], B.shape[1]), np.float32),
             np.empty(A.nnz, np.float32)) for B, dC in layers]

    def step():
        out = []
        for B, dC, C, dB, dv in bufs:
            ocpu.csr_spmm(ip, ix, vv, B, threads=threads, out=C)
            ocpu.sddmm(rows, cols, dC, B, threads=threads, out=dv)
            ocpu.csr_spmm(ipt, ixt, vvt, dC, threads=threads, out=dB)
            out.append((C, dv, dB))
        return out
    return step


def run_cpu_baseline(A, layers, flops_per_step, budget_s=12.0):
    from oracle import cpu as ocpu
    ocpu.build()
    AT = A.T.tocsr()
    AT.sort_indices()
    threads = os.cpu_count() or 1
    step = cpu_step_fn(A, AT, layers, threads)
    step()
    n, t0 = 0, time.perf_counter()
    while True:
        step()
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 50:
            break
    dt = (time.perf_counter() - t0) / n
    return {"value": flops_per_step / dt / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": f"{n} full fwd+bwd steps of the workload (both layers; C restatement of CSR SpMM x2 + "
                      f"gather-dot SDDMM per layer, fp32, pthreads)"}


def base_config(A, layers, workload):
    return {"workload": workload, "M": int(A.shape[0]), "K": int(A.shape[1]), "nnz": int(A.nnz),
            "N": [int(B.shape[1]) for B, _ in layers]}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import cpu as ocpu
    ocpu.build()
    A, layers = make_gcn_workload()
    AT = A.T.tocsr()
    AT.sort_indices()
    threads = os.cpu_count() or 1
    step = cpu_step_fn(A, AT, layers, threads)
    flops = step_flops(A, layers)
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    val = flops / dt / 1e9
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": "GFLOP/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {**base_config(A, layers, WORKLOAD),
                      "l2": "not applicable (host CPU path; each step reads its operands from host memory)",
                      "parallelism": f"{threads} host threads"},
           "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                            "sample": "the whole fwd+bwd step of both layers per iteration (C restatement of "
                                      "the reference's CPU path: CSR SpMM x2 + gather-dot SDDMM per layer)"},
           "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def max_over_ranks(x, dev=None):
    """The largest of every rank's x (replicas: the slowest rank's time is the
    job's); x itself without a process group or with one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aligned_device(x, dev):
    """A float32 device copy of x [rows, n] whose row stride is n rounded up
    to 4 (a view of a padded buffer): what the SpMM kernels read without a
    copy."""
    import torch
    rows, n = x.shape
    ld = (n + 3) // 4 * 4
    buf = torch.zeros((rows, ld), dtype=torch.float32, device=dev)
    buf[:, :n] = torch.as_tensor(np.ascontiguousarray(x, np.float32), device=dev)
    return buf[:, :n]


def aligned_empty(rows, n, dev, pin=False):
    import torch
    ld = (n + 3) // 4 * 4
    if pin:
        return torch.empty((rows, ld), dtype=torch.float32, pin_memory=True)[:, :n]
    return torch.empty((rows, ld), dtype=torch.float32, device=dev)[:, :n]


def padded(t):
    """The row-padded buffer under a [rows, n] view whose row stride exceeds
    n (a contiguous [rows, stride] tensor on the same storage), else t: a
    copy between host and device of that buffer is one contiguous
    asynchronous transfer, where a strided view would go through a
    synchronous staging copy."""
    import torch
    if t.dim() == 2 and t.stride(1) == 1 and t.stride(0) > t.shape[1]:
        return torch.as_strided(t, (t.shape[0], t.stride(0)), (t.stride(0), 1))
    return t


def xfer(dst, src):
    """dst <- src across host and device: the padded buffers when both have
    the same padding (one contiguous asynchronous copy), else the views."""
    pd, ps = padded(dst), padded(src)
    if pd.shape == ps.shape:
        pd.copy_(ps, non_blocking=True)
    else:
        dst.copy_(src, non_blocking=True)


class SparseStep:
    """The step's sparse products on the GPU for one adjacency and a list of
    layer widths: operators (one plan per width; the transposed operator of
    a symmetric pattern reuses the forward plan), device-resident operands
    and outputs, the plain CSR comparator."""

    def __init__(self, A, layers, dev, tc_mode, cache_dir=None):
        from stile_gb300.api import PlanConfig, SpmmOperator
        self.A, self.dev = A, dev
        t0 = time.time()
        self.ops = []
        for B, _ in layers:
            op = SpmmOperator(A, B.shape[1], PlanConfig(tc_mode=tc_mode, cache_dir=cache_dir))
            op.transposed
            self.ops.append(op)
        self.plan_s = time.time() - t0
        self.B = [aligned_device(B, dev) for B, _ in layers]
        self.dC = [aligned_device(dC, dev) for _, dC in layers]
        self.C = [aligned_empty(A.shape[0], B.shape[1], dev) for B, _ in layers]
        self.dB = [aligned_empty(A.shape[1], B.shape[1], dev) for B, _ in layers]
        self.dv = [None] * len(layers)
        self.flops = step_flops(A, layers)

    def forward(self, ev=None):
        # ev: events at the boundaries of the step's operations (forward of
        # every layer, then backward of every layer in reverse)
        for i, op in enumerate(self.ops):
            if ev is not None and i == 0:
                ev[0].record()
            op(self.B[i], out=self.C[i])
            if ev is not None:
                ev[1 + i].record()

    def backward(self, ev=None):
        # dB_l and dvals_l (fused or separate, as each operator chose)
        L = len(self.ops)
        for j, i in enumerate(reversed(range(L))):
            _, self.dv[i] = self.ops[i].backward(self.dC[i], self.B[i], self.dB[i])
            if ev is not None:
                ev[1 + L + j].record()

    def n_events(self):
        return 1 + 2 * len(self.ops)

    def op_names(self):
        L = len(self.ops)
        return ([f"forward_N{self.B[i].shape[1]}" for i in range(L)]
                + [f"backward_N{self.B[i].shape[1]}" for i in reversed(range(L))])

    def step(self, ev=None):
        self.forward(ev)
        self.backward(ev)

    def breakdown(self, timed, steps):
        """Median ms of every operation of the step on its own (L2 flushed
        before each) and the backward variant each width runs."""
        out = {}
        for i, op in enumerate(self.ops):
            N = self.B[i].shape[1]
            t, _ = timed(lambda: op(self.B[i], out=self.C[i]), steps)
            out[f"forward_N{N}_ms"] = float(np.median(t))
            t, _ = timed(lambda: op.backward(self.dC[i], self.B[i], self.dB[i]), steps)
            out[f"backward_N{N}_ms"] = float(np.median(t))
            out[f"backward_N{N}_variant"] = op._bwd_choice.get(N, op.cfg.backward)
        return out

    def graph_step_ms(self, timed, steps):
        """Median ms of the step replayed as one CUDA graph (the same kernels
        and arguments, captured once; L2 flushed before each replay): the
        step without the host's per-launch work.  None (with the reason) if
        the capture fails."""
        import torch
        try:
            side = torch.cuda.Stream(self.dev)
            side.wait_stream(torch.cuda.current_stream(self.dev))
            with torch.cuda.stream(side):
                self.step()
            torch.cuda.current_stream(self.dev).wait_stream(side)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.step()
            torch.cuda.synchronize()
            g.replay()
            torch.cuda.synchronize()
            t, _ = timed(g.replay, steps)
            return float(np.median(t)), None
        except Exception as e:  # noqa: BLE001 -- reported, the eager numbers stand
            torch.cuda.synchronize()
            return None, f"{type(e).__name__}: {e}"[:200]

    def accuracy(self, layers):
        import oracle.semantics as S
        from stile_gb300 import workloads as W
        AT = self.ops[0].transposed[0].A
        acc = {}
        for i, (B, dC) in enumerate(layers):
            tag = f"N{B.shape[1]}_"
            acc.update(errors(tag + "C", self.C[i].cpu().numpy(), S.spmm_fp64(self.A, B)))
            acc.update(errors(tag + "dB", self.dB[i].cpu().numpy(), S.spmm_fp64(AT, dC)))
            ids, ref = W.sddmm_fp64_sample(self.A, dC, B)
            acc.update(errors(tag + "dvals_sampled", self.dv[i].cpu().numpy()[ids], ref))
        return acc

    def plain(self):
        """The plain CSR path on the same GPU: CSR-row SpMM for A and A^T and
        the gather-dot SDDMM per layer."""
        from stile_gb300 import device as D
        from stile_gb300.ops import CsrMatrix, DeviceSddmmPlan
        A = self.A
        csrA, csrAT = CsrMatrix(A), CsrMatrix(self.ops[0].transposed[0].A)
        plain_dev = D.SddmmDevice(M=A.shape[0], K=A.shape[1], nnz=A.nnz,
                                  mid_idx=np.repeat(np.arange(A.shape[0]), np.diff(A.indptr)).astype(np.int32),
                                  j_idx=A.indices.astype(np.int32), remap=np.arange(A.nnz, dtype=np.int32),
                                  bm=16, bn=16, blk_i=np.zeros(0, np.int32), blk_j=np.zeros(0, np.int32),
                                  blk_indptr=np.zeros(1, np.int32), blk_dense_pos=np.zeros(0, np.int32),
                                  blk_out=np.zeros(0, np.int32))
        sd = DeviceSddmmPlan(plain_dev)

        def step():
            for i in range(len(self.ops)):
                csrA.spmm(self.B[i], out=self.C[i])
            for i in reversed(range(len(self.ops))):
                sd.run(self.dC[i], self.B[i])
                csrAT.spmm(self.dC[i], out=self.dB[i])
        return step

    def plan_summary(self):
        return [{f"{k[0]}{'/atomic' if k[1] else ''}": v for k, v in op.plan.summary().items()} for op in self.ops]


def make_timer(flush):
    import torch

    def timed(fn, steps, per_step_events=False, host_sync=False):
        """Per-step device times between CUDA events, L2 flushed before each
        step outside the events.  The host enqueues every step before the
        first has ended (one synchronize after the last), so the events see
        the GPU's time for the step, not the host's launch latency after a
        synchronize; host_sync=True waits for each step (an end-to-end step
        whose result the host reads)."""
        rec = []
        for _ in range(steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(int(per_step_events))] \
                if per_step_events else None
            s.record()
            if per_step_events:
                fn(ev)
            else:
                fn()
            e.record()
            if host_sync:
                e.synchronize()
            rec.append((s, e, ev))
        torch.cuda.synchronize()
        times = [s.elapsed_time(e) for s, e, _ in rec]
        # per step: the times between consecutive events
        fwd = [[ev[k].elapsed_time(ev[k + 1]) for k in range(len(ev) - 1)] for _, _, ev in rec] \
            if per_step_events else []
        return times, fwd
    return timed


def run_secondary_graph(dev, tc_mode, steps, timed, peak, cache_dir=None):
    """The 169,343-node graph (one layer, N = 128): step, forward and the
    plain CSR step, accuracy, forward roofline, and the plan of the learned
    cost model against the analytic one."""
    import oracle.semantics as S
    from stile_gb300.api import PlanConfig, SpmmOperator
    A, layers = make_graph_workload()
    st = SparseStep(A, layers, dev, tc_mode, cache_dir)
    st.step()
    import torch
    torch.cuda.synchronize()
    acc = st.accuracy(layers)
    for _ in range(3):
        st.step()
    t, ops_t = timed(st.step, steps, per_step_events=st.n_events())
    ms = float(np.mean(t))
    fwd_ms = float(np.mean([o[0] for o in ops_t]))
    plain = st.plain()
    for _ in range(3):
        plain()
    tp, _ = timed(plain, steps)
    plain_ms = float(np.mean(tp))
    alg = algorithmic_bytes_spmm(A, layers[0][0].shape[1])
    out = {"workload": GRAPH_WORKLOAD, "config": base_config(A, layers, GRAPH_WORKLOAD), "plan": st.plan_summary(),
           "plan_search_s": round(st.plan_s, 2), "value": st.flops / (ms * 1e-3) / 1e9, "unit": "GFLOP/s",
           "ms_per_step": ms, "forward_ms": fwd_ms, "csr_step_ms": plain_ms,
           "speedup_hybrid_over_csr": plain_ms / ms,
           "roofline_forward": {"algorithmic_bytes": int(alg), "achieved_gbs": alg / (fwd_ms * 1e-3) / 1e9,
                                "frac": alg / (fwd_ms * 1e-3) / 1e9 / peak},
           "accuracy": acc}
    # the learned cost model, measured by the forward time of the plan it chooses
    try:
        t0 = time.time()
        op_l = SpmmOperator(A, layers[0][0].shape[1], PlanConfig(tc_mode=tc_mode, learned=True, cache_dir=cache_dir))
        t_l = time.time() - t0
        Cl = torch.empty_like(st.C[0])
        op = st.ops[0]
        for _ in range(3):
            op_l(st.B[0], out=Cl)
            op(st.B[0], out=st.C[0])
        tl, _ = timed(lambda: op_l(st.B[0], out=Cl), max(steps, 5))
        ta, _ = timed(lambda: op(st.B[0], out=st.C[0]), max(steps, 5))
        from stile_gb300.cost_model import gb300_mlp_model
        mm = gb300_mlp_model().meta
        out["learned_cost_model"] = {
            "plan_forward_ms": float(np.median(tl)), "analytic_plan_forward_ms": float(np.median(ta)),
            "plan": {f"{k[0]}{'/atomic' if k[1] else ''}": v for k, v in op_l.plan.summary().items()},
            "plan_search_s": round(t_l, 2),
            "held_out_mean_abs_log_err": {k: {"mlp": v["test_mean_abs_log_err_mlp"],
                                              "analytic": v["test_mean_abs_log_err_analytic"]} for k, v in mm.items()},
            "C_rel_fro": S.rel_fro(Cl.cpu().numpy(), S.spmm_fp64(A, layers[0][0]))}
        op_l.handle.close()
    except FileNotFoundError as exc:
        out["learned_cost_model"] = {"unavailable": str(exc)}
    return out


def gcn_training_step_ms(st, dev, timed, steps):
    """The whole two-layer GCN training step (dense GEMMs, ReLU, the sparse
    products and their backward; X resident on the device) for context."""
    import torch
    from stile_gb300.gcn import TwoLayerGCN
    n = st.A.shape[0]
    g = torch.Generator(device=dev).manual_seed(7)
    X = torch.randn((n, 602), device=dev, generator=g)
    W1 = torch.randn((602, WIDTHS[0]), device=dev, generator=g) / 602 ** 0.5
    W2 = torch.randn((WIDTHS[0], WIDTHS[1]), device=dev, generator=g) / WIDTHS[0] ** 0.5
    G = torch.randn((n, WIDTHS[1]), device=dev, generator=g)
    model = TwoLayerGCN(st.A, W1, W2, ops=tuple(st.ops))
    params = [model.lin1.weight, model.lin2.weight, model.vals]

    def train_step():
        H2 = model(X)
        torch.autograd.grad(H2, params, grad_outputs=G)

    for _ in range(3):
        train_step()
    t, _ = timed(train_step, steps)
    del X
    return float(np.mean(t))


def run_gpu(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from stile_gb300 import device as D
    from stile_gb300.api import HybridSpMMFunction
    from stile_gb300.ops import launch_count

    t0 = time.time()
    A, layers = make_gcn_workload()
    log(f"[bench] workload {A.shape} nnz={A.nnz} ({time.time() - t0:.1f}s)")
    tc_mode = D.TC_BF16
    st = SparseStep(A, layers, dev, tc_mode, args.plan_cache)
    log(f"[bench] plans {st.plan_summary()} ({st.plan_s:.1f}s)")
    flops = st.flops
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    timed = make_timer(flush)
    peak, peak_kind = measured_peaks()

    # accuracy against the FP64 oracle (outside the timed region)
    st.step()
    torch.cuda.synchronize()
    acc = st.accuracy(layers)
    log(f"[bench] accuracy {acc}")

    plain = st.plain()
    for _ in range(max(args.warmup, 3)):
        st.step()
        plain()
    torch.cuda.synchronize()

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = launch_count()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        # an NVTX range around the timed steps (a profiler's launch list can
        # be limited to it)
        torch.cuda.nvtx.range_push("timed_steps")
        times, ops_t = timed(st.step, args.steps, per_step_events=st.n_events())
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = launch_count() - launches0
    ms = max_over_ranks(float(np.sum(times)) / args.steps, dev)
    value = world * flops / (ms * 1e-3) / 1e9

    plain_times, _ = timed(plain, args.steps)
    plain_ms = float(np.sum(plain_times)) / args.steps
    plain_value = flops / (plain_ms * 1e-3) / 1e9
    breakdown = st.breakdown(timed, args.steps)
    breakdown["step_ms_first_median_min_max"] = [float(times[0]), float(np.median(times)), float(np.min(times)),
                                                 float(np.max(times))]
    # every operation's median time inside the timed steps (events between them)
    breakdown["in_step_ms"] = {name: float(np.median([o[k] for o in ops_t]))
                               for k, name in enumerate(st.op_names())}

    # roofline of the dominant kernel: the layer-1 forward SpMM (N = 128)
    fwd_ms = float(np.mean([o[0] for o in ops_t]))
    alg = algorithmic_bytes_spmm(A, WIDTHS[0])
    achieved = alg / (fwd_ms * 1e-3) / 1e9
    gathered = gathered_bytes_spmm(st.ops[0], WIDTHS[0])
    traffic = profile_traffic("fused_spmm_gcn.md")
    step_bytes = sum(2 * algorithmic_bytes_spmm(A, B.shape[1]) + algorithmic_bytes_sddmm(A, B.shape[1])
                     for B, _ in layers)

    # end to end through the public autograd API with host buffers: each
    # layer's operand and output gradient go up from pinned memory, every
    # product comes back (C_l, dB_l, and the shared value gradient)
    vals = torch.as_tensor(A.data.astype(np.float32), device=dev)
    hB = [aligned_empty(A.shape[1], B.shape[1], dev, pin=True) for B, _ in layers]
    hdC = [aligned_empty(A.shape[0], B.shape[1], dev, pin=True) for B, _ in layers]
    for i, (B, dC) in enumerate(layers):
        hB[i].copy_(torch.as_tensor(B))
        hdC[i].copy_(torch.as_tensor(dC))
    # every transfer moves the row-padded buffers (contiguous, asynchronous)
    hC = [aligned_empty(A.shape[0], B.shape[1], dev, pin=True) for B, _ in layers]
    hdB = [aligned_empty(A.shape[1], B.shape[1], dev, pin=True) for B, _ in layers]
    hdv = torch.empty(A.nnz, dtype=torch.float32, pin_memory=True)
    Bd = [aligned_empty(A.shape[1], B.shape[1], dev) for B, _ in layers]
    dCd = [aligned_empty(A.shape[0], B.shape[1], dev) for B, _ in layers]
    main = torch.cuda.current_stream(dev)
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    L = len(layers)
    # the edge values are a parameter resident on the device (one leaf for
    # every step, as a training loop holds it): the operators reload them
    # only when they change
    v = vals.detach().requires_grad_(True)

    def e2e_step():
        # up: every layer's operand in forward order, then the output
        # gradients in the order the backward needs them (last layer first),
        # so each layer's backward starts as soon as its own dC has landed
        ev_b = [torch.cuda.Event() for _ in range(L)]
        ev_dc = [torch.cuda.Event() for _ in range(L)]
        up.wait_stream(main)
        with torch.cuda.stream(up):
            for i in range(L):
                xfer(Bd[i], hB[i])
                ev_b[i].record(up)
            for i in reversed(range(L)):
                xfer(dCd[i], hdC[i])
                ev_dc[i].record(up)
        Bin, Cs = [], []
        for i in range(L):
            main.wait_event(ev_b[i])
            b = Bd[i].detach().requires_grad_(True)
            Bin.append(b)
            Cs.append(HybridSpMMFunction.apply(v, b, st.ops[i]))
            ev_c = torch.cuda.Event()
            ev_c.record(main)
            down.wait_event(ev_c)
            with torch.cuda.stream(down):
                xfer(hC[i], Cs[i].detach())
            Cs[i].record_stream(down)
        # backward layer by layer (last first): each dB_l goes down while the
        # next layer's backward runs; the value gradient (shared by the
        # layers) is summed on the device and goes down last
        dv = None
        for i in reversed(range(L)):
            main.wait_event(ev_dc[i])
            g_v, g_b = torch.autograd.grad(Cs[i], [v, Bin[i]], grad_outputs=dCd[i])
            dv = g_v if dv is None else dv.add_(g_v)
            ev_bw = torch.cuda.Event()
            ev_bw.record(main)
            down.wait_event(ev_bw)
            with torch.cuda.stream(down):
                xfer(hdB[i], g_b)
            g_b.record_stream(down)
        ev_dv = torch.cuda.Event()
        ev_dv.record(main)
        down.wait_event(ev_dv)
        with torch.cuda.stream(down):
            hdv.copy_(dv, non_blocking=True)
        dv.record_stream(down)
        main.wait_stream(down)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_times, _ = timed(e2e_step, args.steps, host_sync=True)
    e2e_ms = max_over_ranks(float(np.sum(e2e_times)) / args.steps, dev)
    e2e_val = world * flops / (e2e_ms * 1e-3) / 1e9
    h2d = sum(padded(hB[i]).numel() * 4 + padded(hdC[i]).numel() * 4 for i in range(L))
    d2h = sum(padded(hC[i]).numel() * 4 + padded(hdB[i]).numel() * 4 for i in range(L)) + A.nnz * 4

    train_ms = gcn_training_step_ms(st, dev, timed, args.steps)
    secondary = run_secondary_graph(dev, tc_mode, args.steps, timed, peak, args.plan_cache) if rank == 0 else None

    cpu = run_cpu_baseline(A, layers, flops) if (rank == 0 and world == 1) else None
    # last: the step as one CUDA graph (a failed capture leaves nothing after it to disturb)
    breakdown["graph_step_ms"], graph_err = st.graph_step_ms(timed, args.steps)
    if graph_err:
        breakdown["graph_error"] = graph_err

    if rank == 0:
        cfg = base_config(A, layers, WORKLOAD)
        cfg.update({"l2": "flushed between steps (256 MiB write, untimed)",
                    "parallelism": "replicas" if world > 1 else "single GPU"})
        plan_info = {"tc_tiles": "bf16 operands, fp32 accumulate (tcgen05, TMEM)", "row_tiles": "fp32 (CUDA cores)",
                     "plans": st.plan_summary(), "plan_search_s": round(st.plan_s, 2),
                     "cost_model": st.ops[0].plan.meta.get("cost_model")}
        out = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+bf16", "data": "synthetic", "config": cfg, "plan": plan_info,
            "e2e": {"value": e2e_val, "unit": "GFLOP/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                    "path": "HybridSpMMFunction forward of both layers, torch.autograd.grad per layer (last "
                            "first), pinned host buffers; copies on two side streams (up: B_l, then dC_l last "
                            "layer first; down: C_l during the rest, dB_l after its layer's backward, the "
                            "summed value gradient last)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "layer-1 forward SpMM (N = 128)",
                         "algorithmic_bytes_per_launch": int(alg), "ms_per_launch": fwd_ms,
                         "peak_source": peak_kind,
                         "gather": {"bytes_per_launch": int(gathered),
                                    "achieved_gbs": gathered / (fwd_ms * 1e-3) / 1e9,
                                    "peak_gbs": GATHER_PEAK_GBS,
                                    "frac": gathered / (fwd_ms * 1e-3) / 1e9 / GATHER_PEAK_GBS,
                                    "what": "B rows gathered from L2 (one per row-tile entry, 16 per tensor-core "
                                            "k-step) against the measured random-row gather rate"}},
            "step_roofline": {"algorithmic_bytes_per_step": int(step_bytes),
                              "achieved_gbs": step_bytes / (ms * 1e-3) / 1e9,
                              "frac": step_bytes / (ms * 1e-3) / 1e9 / peak},
            "csr_baseline": {"value": plain_value, "unit": "GFLOP/s", "ms_per_step": plain_ms,
                             "speedup_hybrid_over_csr": value / plain_value},
            "accuracy": acc,
            "breakdown": breakdown,
            "gcn_training_step": {"ms": train_ms, "what": "whole two-layer GCN step (X W1, Z1 W2 and their "
                                                          "gradients in torch fp32 GEMMs, ReLU, the sparse "
                                                          "products), X resident"},
            "secondary": secondary,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "wall_s_timed_region": wall,
            "device_mem_peak_gb": torch.cuda.max_memory_allocated() / 1e9,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# the other configurations (one JSON line each; the headline is "gcn2")
# ---------------------------------------------------------------------------
def run_attention(args):
    """Sparse attention on the reference's LogSparse and Strided patterns
    (n = 4096, 8 heads, F = Fv = 64): the fused one-pass kernel against the
    three-launch path (hybrid SDDMM, row softmax, batched hybrid SpMM), both
    against float64 on the first two heads."""
    import torch
    import oracle.attention as OA
    import oracle.semantics as S
    from stile_gb300 import synthetic as syn
    from stile_gb300.api import SparseAttention

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    n, H, F = 4096, 8, 64

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        rec = []
        for _ in range(args.steps):  # enqueued ahead, one synchronize (as make_timer)
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            rec.append((s, e))
        torch.cuda.synchronize()
        return float(np.median([s.elapsed_time(e) for s, e in rec]))

    out = {"workload": "sparse_attention", "n": n, "heads": H, "F": F, "Fv": F, "steps": args.steps,
           "l2": "flushed between iterations (256 MiB write)"}
    rng = np.random.default_rng(0)
    Q, K, V = (torch.as_tensor(rng.standard_normal((H, n, F)).astype(np.float32), device=dev) for _ in range(3))
    for kind in ("logsparse", "strided"):
        A = syn.logsparse_pattern(n) if kind == "logsparse" else syn.strided_pattern(n)
        fused = SparseAttention(A, F)
        three = SparseAttention(A, F, fused=False)
        ref = OA.attention_fp64(A, Q[:2].cpu().numpy(), K[:2].cpu().numpy(), V[:2].cpu().numpy(), 1.0 / np.sqrt(F))
        r = {"nnz": int(A.nnz)}
        for name, att in (("fused", fused), ("three_launches", three)):
            o = att(Q, K, V)
            torch.cuda.synchronize()
            r[name] = {"ms": timed(lambda: att(Q, K, V)),
                       "rel_fro_first_two_heads": S.rel_fro(o[:2].cpu().numpy(), ref)}
        r["speedup_fused"] = r["three_launches"]["ms"] / r["fused"]["ms"]
        out[kind] = r
    print(json.dumps(out), flush=True)


def run_config(args):
    import torch
    import oracle.semantics as S
    from stile_gb300 import device as D
    from stile_gb300 import workloads as W
    from stile_gb300.api import PlanConfig, SddmmOperator, SpmmOperator
    from stile_gb300.ops import CsrMatrix, DeviceSddmmPlan

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    w = W.BY_NAME[args.workload]()
    A = w.A
    log(f"[bench] {w.name} {A.shape} nnz={A.nnz} ({time.time() - t0:.1f}s)")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed(fn, steps):
        for _ in range(max(args.warmup, 3)):
            fn()
        rec = []
        for _ in range(steps):  # enqueued ahead, one synchronize (as make_timer)
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            rec.append((s, e))
        torch.cuda.synchronize()
        return float(np.median([s.elapsed_time(e) for s, e in rec]))

    def plan_summary(plan):
        return {f"{k[0]}{'/atomic' if k[1] else ''}": v for k, v in plan.summary().items()}

    peak, peak_kind = measured_peaks()
    out = {"workload": w.name, "note": w.note, "M": int(A.shape[0]), "K": int(A.shape[1]), "nnz": int(A.nnz),
           "width": int(w.width), "steps": args.steps, "l2": "flushed between iterations (256 MiB write)"}
    if w.kind == "spmm":
        N = w.width
        tc_mode = D.TC_SPLIT_BF16 if w.fp32 else D.TC_BF16
        t0 = time.time()
        op = SpmmOperator(A, N, PlanConfig(tc_mode=tc_mode))
        opT, _ = op.transposed
        out["plan_search_s"] = round(time.time() - t0, 2)
        out["plan"] = plan_summary(op.plan)
        out["tc_mode"] = {D.TC_BF16: "bf16", D.TC_SPLIT_BF16: "split-bf16 (fp32 path)"}[tc_mode]
        B_np, dC_np = w.dense["B"], w.dense["dC"]
        B = torch.as_tensor(B_np, device=dev)
        dC = torch.as_tensor(dC_np, device=dev)
        C = aligned_empty(A.shape[0], N, dev)
        dB = aligned_empty(A.shape[1], N, dev)
        AT = opT.A

        def step():
            op(B, out=C)
            op.backward(dC, B, dB)   # dB and dvals from one pass over A^T's tiles

        op(B, out=C)
        _, dv = op.backward(dC, B, dB)
        torch.cuda.synchronize()
        ids, ref = W.sddmm_fp64_sample(A, dC_np, B_np)
        out["accuracy"] = {**errors("C", C.cpu().numpy(), S.spmm_fp64(A, B_np)),
                           **errors("dB", dB.cpu().numpy(), S.spmm_fp64(AT, dC_np)),
                           **errors("dvals_sampled", dv.cpu().numpy()[ids], ref),
                           "dvals_sample": int(len(ids))}
        ms_step = timed(step, args.steps)
        ms_fwd = timed(lambda: op(B, out=C), args.steps)
        csrA, csrAT = CsrMatrix(A), CsrMatrix(AT)
        plain_dev = D.SddmmDevice(M=A.shape[0], K=A.shape[1], nnz=A.nnz,
                                  mid_idx=np.repeat(np.arange(A.shape[0]), np.diff(A.indptr)).astype(np.int32),
                                  j_idx=A.indices.astype(np.int32), remap=np.arange(A.nnz, dtype=np.int32), bm=16,
                                  bn=16, blk_i=np.zeros(0, np.int32), blk_j=np.zeros(0, np.int32),
                                  blk_indptr=np.zeros(1, np.int32), blk_dense_pos=np.zeros(0, np.int32),
                                  blk_out=np.zeros(0, np.int32))
        plain_sddmm = DeviceSddmmPlan(plain_dev)

        def plain_step():
            csrA.spmm(B, out=C)
            plain_sddmm.run(dC, B)
            csrAT.spmm(dC, out=dB)

        ms_plain = timed(plain_step, args.steps)
        ms_plain_fwd = timed(lambda: csrA.spmm(B, out=C), args.steps)
        flops = 3 * 2 * A.nnz * N
        alg = algorithmic_bytes_spmm(A, N)
        out.update({"metric": "fwd+bwd GFLOP/s", "value": flops / (ms_step * 1e-3) / 1e9, "ms_per_step": ms_step,
                    "forward_ms": ms_fwd, "csr_step_ms": ms_plain, "csr_forward_ms": ms_plain_fwd,
                    "speedup_step_over_csr": ms_plain / ms_step, "speedup_forward_over_csr": ms_plain_fwd / ms_fwd,
                    "roofline_forward": {"algorithmic_bytes": int(alg), "achieved_gbs": alg / (ms_fwd * 1e-3) / 1e9,
                                         "peak_gbs": peak, "frac": alg / (ms_fwd * 1e-3) / 1e9 / peak,
                                         "peak_source": peak_kind}})
        # the operator left to choose its path (hybrid plan or plain CSR
        # kernels, timed on these operands at the first call of each width)
        op_a = SpmmOperator(A, N, PlanConfig(tc_mode=tc_mode, path="auto"), plan=op.plan)
        Ca, dBa = aligned_empty(C.shape[0], C.shape[1], dev), aligned_empty(dB.shape[0], dB.shape[1], dev)

        def auto_step():
            op_a(B, out=Ca)
            op_a.backward(dC, B, dBa)
        auto_step()
        torch.cuda.synchronize()
        out["auto_path"] = {"forward": op_a._fwd_choice.get(N), "backward": op_a._bwd_choice.get(N),
                            "ms_per_step": timed(auto_step, args.steps),
                            "forward_ms": timed(lambda: op_a(B, out=Ca), args.steps),
                            "C_rel_fro": S.rel_fro(Ca.cpu().numpy(), S.spmm_fp64(A, B_np))}
        op_a.handle.close()
        if args.workload.startswith("pruned"):
            # activations in bf16, as the configuration has them: read as is
            B16 = B.to(torch.bfloat16)
            C16 = aligned_empty(C.shape[0], C.shape[1], dev)
            op(B16, out=C16)
            torch.cuda.synchronize()
            out["bf16_B"] = {"forward_ms": timed(lambda: op(B16, out=C16), args.steps),
                             "C_rel_fro": S.rel_fro(C16.cpu().numpy(),
                                                    S.spmm_fp64(A, B16.float().cpu().numpy()))}
            # tensor-core tiles as 16x16 blocks on the column grid
            # (TC_k_notsorted): the block-pruned blocks go to the tensor
            # cores as they are, the scattered rest to row tiles
            t0 = time.time()
            op_b = SpmmOperator(A, N, PlanConfig(tc_mode=tc_mode, tc_k_notsorted=True))
            t_b = time.time() - t0
            Cb = aligned_empty(C.shape[0], C.shape[1], dev)
            op_b(B, out=Cb)
            torch.cuda.synchronize()
            out["column_blocks"] = {"plan": plan_summary(op_b.plan), "plan_search_s": round(t_b, 2),
                                    "tc_ksteps": op_b.device_layout.stats()["tc_ksteps"],
                                    "forward_ms": timed(lambda: op_b(B, out=Cb), args.steps),
                                    "bf16_B_forward_ms": timed(lambda: op_b(B16, out=C16), args.steps),
                                    "C_rel_fro": S.rel_fro(Cb.cpu().numpy(), S.spmm_fp64(A, B_np))}
            op_b.handle.close()
            # fp8 e4m3 tensor tiles (per tile-row weight scales, per-tensor
            # activation scale), the same plan, fp32 activations
            op_f8 = SpmmOperator(A, N, PlanConfig(tc_mode=D.TC_FP8), plan=op.plan)
            C8 = aligned_empty(C.shape[0], C.shape[1], dev)
            op_f8(B, out=C8)
            torch.cuda.synchronize()
            out["fp8_tiles"] = {"forward_ms": timed(lambda: op_f8(B, out=C8), args.steps),
                                **errors("C", C8.cpu().numpy(), S.spmm_fp64(A, B_np))}
            op_f8.handle.close()
            # context: the zero-filled weight as a dense bf16 GEMM (cuBLAS
            # through torch.matmul, bf16 output) on the same activations
            Wd = torch.as_tensor(A.toarray(), device=dev).to(torch.bfloat16)
            Cd = torch.empty((A.shape[0], N), device=dev, dtype=torch.bfloat16)
            torch.matmul(Wd, B16, out=Cd)
            torch.cuda.synchronize()
            out["dense_bf16_gemm"] = {"forward_ms": timed(lambda: torch.matmul(Wd, B16, out=Cd), args.steps),
                                      "flop": 2 * A.shape[0] * A.shape[1] * N,
                                      "C_rel_fro": S.rel_fro(Cd.float().cpu().numpy(),
                                                             S.spmm_fp64(A, B16.float().cpu().numpy()))}
            del Wd, Cd
            # the plan chosen by the learned cost model against the analytic one
            try:
                t0 = time.time()
                op_l = SpmmOperator(A, N, PlanConfig(tc_mode=tc_mode, learned=True))
                t_l = time.time() - t0
                Cl = aligned_empty(C.shape[0], C.shape[1], dev)
                ms_l = timed(lambda: op_l(B, out=Cl), args.steps)
                out["learned_cost_model"] = {"plan": plan_summary(op_l.plan), "plan_search_s": round(t_l, 2),
                                             "forward_ms": ms_l, "analytic_forward_ms": ms_fwd,
                                             "C_rel_fro": S.rel_fro(Cl.cpu().numpy(), S.spmm_fp64(A, B_np))}
                op_l.handle.close()
            except FileNotFoundError as exc:
                out["learned_cost_model"] = {"unavailable": str(exc)}
    else:
        F = w.width
        t0 = time.time()
        op = SddmmOperator(A, F)
        out["plan_search_s"] = round(time.time() - t0, 2)
        out["plan"] = plan_summary(op.plan)
        X_np, Y_np = w.dense["X"], w.dense["Y"]
        X = torch.as_tensor(X_np, device=dev)
        Y = torch.as_tensor(Y_np, device=dev)
        res = op(X, Y)
        torch.cuda.synchronize()
        ids, ref = W.sddmm_fp64_sample(A, X_np, Y_np)
        out["accuracy"] = {**errors("out_sampled", res.cpu().numpy()[ids], ref), "sample": int(len(ids))}
        ms = timed(lambda: op(X, Y), args.steps)
        plain_dev = D.SddmmDevice(M=A.shape[0], K=A.shape[1], nnz=A.nnz,
                                  mid_idx=np.repeat(np.arange(A.shape[0]), np.diff(A.indptr)).astype(np.int32),
                                  j_idx=A.indices.astype(np.int32), remap=np.arange(A.nnz, dtype=np.int32), bm=16,
                                  bn=16, blk_i=np.zeros(0, np.int32), blk_j=np.zeros(0, np.int32),
                                  blk_indptr=np.zeros(1, np.int32), blk_dense_pos=np.zeros(0, np.int32),
                                  blk_out=np.zeros(0, np.int32))
        plain = DeviceSddmmPlan(plain_dev)
        ms_plain = timed(lambda: plain.run(X, Y), args.steps)
        flops = 2 * A.nnz * F
        op_a = SddmmOperator(A, F, PlanConfig(max_bucket_size=32, path="auto"), plan=op.plan)
        op_a(X, Y)
        torch.cuda.synchronize()
        out["auto_path"] = {"choice": next(iter(op_a._choice.values())), "ms": timed(lambda: op_a(X, Y), args.steps)}
        alg = algorithmic_bytes_sddmm(A, F)
        out.update({"metric": "SDDMM GFLOP/s", "value": flops / (ms * 1e-3) / 1e9, "ms": ms,
                    "plain_list_ms": ms_plain, "speedup_over_plain_list": ms_plain / ms,
                    "roofline": {"algorithmic_bytes": int(alg), "achieved_gbs": alg / (ms * 1e-3) / 1e9,
                                 "peak_gbs": peak, "frac": alg / (ms * 1e-3) / 1e9 / peak,
                                 "peak_source": peak_kind}})
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="stile", choices=["stile", "reference"])
    ap.add_argument("--workload", default="gcn2",
                    help="gcn2 (the headline line: the two-layer GCN step) or one of the configurations: "
                         "plain, plain_min10, graph, pruned, pruned_t, sddmm, gcn, gcn_41, attention (one JSON "
                         "line of measurements each)")
    ap.add_argument("--plan-cache", default=None,
                    help="directory of the on-disk plan cache (searched plans are stored and reloaded); "
                         "default: search every run")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "attention":
        run_attention(args)
    elif args.workload != "gcn2":
        run_config(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
