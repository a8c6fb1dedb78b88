"""Numpy execution of the device layout (test helper): what the fused kernel
computes from the arrays it is given, with exact fp32 tile values."""
import numpy as np


def spmm_device_exec(dev, B):
    B = np.asarray(B, dtype=np.float64)
    C = np.full((dev.M, B.shape[1]), np.nan)
    C[dev.zero_rows] = 0.0
    kb = dev.tc_item_kbeg
    cols = dev.tc_cols.reshape(-1, 16)
    vals = dev.tc_values_f32.astype(np.float64)
    rows = dev.tc_out_rows.reshape(-1, 16)
    for it in range(len(dev.tc_item_flags)):
        acc = np.zeros((16, B.shape[1]))
        for ks in range(kb[it], kb[it + 1]):
            acc += vals[ks] @ B[cols[ks]]
        for n in range(16):
            r = rows[it, n]
            if r < 0:
                continue
            if dev.tc_item_flags[it] & 1:
                C[r] += acc[n]
            else:
                C[r] = acc[n]
    r0 = dev.ell_item_row0
    for it in range(len(dev.ell_item_K)):
        K = dev.ell_item_K[it]
        for r in range(r0[it], r0[it + 1]):
            o = dev.ell_out_row[r]
            if o < 0:
                continue
            s0 = dev.ell_item_slot0[it] + (r - r0[it]) * K
            n = dev.ell_row_len[r]
            acc = dev.ell_vals[s0:s0 + n].astype(np.float64) @ B[dev.ell_kidx[s0:s0 + n]]
            if dev.ell_item_flags[it] & 1:
                C[o] += acc
            else:
                C[o] = acc
    return C
