"""Build and load ``libstile_gb300.so`` (the C ABI declared in
include/stile_gb300.h) with ctypes.

The library is compiled in-tree for sm_103a only.  There is no CPU fallback:
every operator raises if the library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libstile_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["spmm.cu", "sddmm.cu", "attention.cu", "probe.cu", "capi.cu", "noalloc.cu", "mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    """Compile every translation unit in parallel and link the shared
    library.  Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "stile_gb300.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([_nvcc(), *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or not _newer(LIB_PATH, objs):
        run([_nvcc(), *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcudart"])
    return LIB_PATH


# ---------------------------------------------------------------------------
# ctypes mirror of the header
# ---------------------------------------------------------------------------
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_f32p = ctypes.POINTER(ctypes.c_float)


class SpmmPlanHost(ctypes.Structure):
    _fields_ = [
        ("M", ctypes.c_int32), ("K", ctypes.c_int32),
        ("tc_mode", ctypes.c_int32),
        ("tc_n_items", ctypes.c_int32), ("tc_n_ksteps", ctypes.c_int32),
        ("tc_item_kbeg", c_i32p), ("tc_item_flags", c_i32p), ("tc_out_rows", c_i32p),
        ("tc_cols", c_i32p), ("tc_vals", ctypes.c_void_p), ("tc_kstep_bytes", ctypes.c_int32),
        ("tc_nnz_id", c_i32p),
        ("ell_n_items", ctypes.c_int32), ("ell_n_rows", ctypes.c_int32), ("ell_n_slots", ctypes.c_int32),
        ("ell_item_row0", c_i32p), ("ell_item_K", c_i32p), ("ell_item_slot0", c_i32p),
        ("ell_item_flags", c_i32p), ("ell_out_row", c_i32p), ("ell_row_len", c_i32p),
        ("ell_vals", c_f32p), ("ell_kidx", c_i32p), ("ell_nnz_id", c_i32p),
        ("n_zero_rows", ctypes.c_int32), ("zero_rows", c_i32p),
        ("nnz", ctypes.c_int64),
        ("tc_row_scale", c_f32p),
    ]


class SddmmPlanHost(ctypes.Structure):
    _fields_ = [
        ("M", ctypes.c_int32), ("K", ctypes.c_int32), ("nnz", ctypes.c_int64),
        ("n_1d", ctypes.c_int32), ("mid_idx", c_i32p), ("j_idx", c_i32p), ("remap", c_i32p),
        ("n_blk", ctypes.c_int32), ("bm", ctypes.c_int32), ("bn", ctypes.c_int32),
        ("n_blk_nnz", ctypes.c_int32),
        ("blk_i", c_i32p), ("blk_j", c_i32p), ("blk_indptr", c_i32p),
        ("blk_dense_pos", c_i32p), ("blk_out", c_i32p),
    ]


EXPORTS = {
    "stile_spmm_plan_upload": (ctypes.c_int, [ctypes.POINTER(SpmmPlanHost), ctypes.POINTER(ctypes.c_void_p)]),
    "stile_sddmm_plan_upload": (ctypes.c_int, [ctypes.POINTER(SddmmPlanHost), ctypes.POINTER(ctypes.c_void_p)]),
    "stile_spmm_plan_free": (ctypes.c_int, [ctypes.c_void_p]),
    "stile_sddmm_plan_free": (ctypes.c_int, [ctypes.c_void_p]),
    "stile_spmm_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                      ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_values_bytes": (ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int32]),
    "stile_spmm_values_pack": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    "stile_spmm_run_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_run_bf16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_dvals": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "stile_sddmm_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "stile_sddmm_run_bf16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                            ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_dvals_bf16": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "stile_csr_spmm_run": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "stile_csr_group_nnz": (ctypes.c_int32, []),
    "stile_sparse_attention": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p]),
    "stile_csr_row_softmax": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p]),
    "stile_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "stile_mlp_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "stile_mlp_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, ctypes.c_int32, ctypes.c_void_p]),
    "stile_csr_spmm_run_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                                  ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_plan_set_values": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "stile_spmm_plan_set_transpose_ids": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                         ctypes.c_void_p]),
    "stile_spmm_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                           ctypes.c_int32, ctypes.c_void_p]),
    "stile_spmm_plan_set_wait_policy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "stile_spmm_plan_set_dvals_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "stile_spmm_plan_error_flag": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_i32p]),
    "stile_sddmm_plan_error_flag": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_i32p]),
    "stile_debug_umma_probe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                              ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "stile_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "stile_launch_count": (ctypes.c_int64, []),
}

_lib = None
_lock = threading.Lock()


def load(path=None):
    """Load the shared library (building it first if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.stile_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc}): {last_error()}")
