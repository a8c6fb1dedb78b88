"""ctypes wrapper of oracle/cpu_kernels.c (TEST INFRASTRUCTURE: tests,
smoke() and bench.py's CPU-baseline leg only)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle_cpu.so")
SRC = os.path.join(HERE, "cpu_kernels.c")


def build():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    subprocess.run(["gcc", "-O3", "-shared", "-fPIC", "-pthread", SRC, "-o", LIB], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.oracle_csr_spmm.argtypes = [ctypes.c_int32] + [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p,
                                                                                 ctypes.c_int64, ctypes.c_int32,
                                                                                 ctypes.c_int32]
        L.oracle_sddmm.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 3 + [ctypes.c_int64, ctypes.c_void_p,
                                                                              ctypes.c_int64, ctypes.c_void_p,
                                                                              ctypes.c_int32, ctypes.c_int32]
        _lib = L
    return _lib


def csr_spmm(indptr, indices, vals, B, threads=1, out=None):
    indptr = np.ascontiguousarray(indptr, np.int32)
    indices = np.ascontiguousarray(indices, np.int32)
    vals = np.ascontiguousarray(vals, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M = len(indptr) - 1
    if out is None:
        out = np.empty((M, B.shape[1]), np.float32)
    lib().oracle_csr_spmm(M, indptr.ctypes.data, indices.ctypes.data, vals.ctypes.data, B.ctypes.data,
                          B.shape[1], out.ctypes.data, out.shape[1], B.shape[1], threads)
    return out


def sddmm(rows, cols, X, Y, threads=1, out=None):
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    if out is None:
        out = np.empty(len(rows), np.float32)
    lib().oracle_sddmm(len(rows), rows.ctypes.data, cols.ctypes.data, X.ctypes.data, X.shape[1],
                       Y.ctypes.data, Y.shape[1], out.ctypes.data, X.shape[1], threads)
    return out
