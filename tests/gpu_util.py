"""Helpers shared by the GPU tests."""
import ctypes
import functools

import numpy as np
import scipy.sparse as sp

# layout the fused kernel uses (see stile_gb300/csrc/spmm.cu):
# A operand MN-major 128B-swizzle, LBO = 2048 (between 64-wide MN atoms),
# SBO = 1024 (between 8-row K groups); B operand K-major no-swizzle,
# LBO = 128 (K direction), SBO = 256 (row direction)
KERNEL_DESC = (2048, 1024, 2, 128, 256, 0)


def bf16_round(x):
    from stile_gb300.device import _to_bf16_bits, _bf16_bits_to_f32
    return _bf16_bits_to_f32(_to_bf16_bits(np.asarray(x, np.float32)))


def a_image(A, lbo=2048, sbo=1024):
    """A [128 (m) x 16 (k)] -> 8 KB MN-major 128B-swizzled image (bf16)."""
    from stile_gb300.device import _to_bf16_bits
    img = np.zeros(4096, dtype=np.uint16)
    bits = _to_bf16_bits(A.astype(np.float32))
    for m in range(128):
        for k in range(16):
            off = (m // 64) * lbo + (k // 8) * sbo + (k % 8) * 128 + ((((m % 64) // 8) ^ (k % 8)) << 4) + (m % 8) * 2
            img[off // 2] = bits[m, k]
    return img


def b_image(Bm):
    """B [16 (n) x 16 (k)] -> K-major no-swizzle image (bf16), as the plan stores it."""
    from stile_gb300.device import _to_bf16_bits, operand_image_16bit
    img = np.zeros(4096, dtype=np.uint16)
    img[:256] = operand_image_16bit(_to_bf16_bits(Bm.astype(np.float32)).reshape(1, 16, 16))[0]
    return img


PROBE_IMAGE_BYTES = 16384   # the probe copies this many bytes of each image


def probe_image(img):
    """A device copy of an operand image, zero-padded to the probe's image
    size."""
    import torch
    raw = np.frombuffer(np.ascontiguousarray(img).tobytes(), dtype=np.uint8)
    assert raw.size <= PROBE_IMAGE_BYTES
    buf = np.zeros(PROBE_IMAGE_BYTES, dtype=np.uint8)
    buf[:raw.size] = raw
    return torch.as_tensor(buf, device="cuda")


def run_probe(A, Bm, desc6):
    import torch
    from stile_gb300 import _lib
    lib = _lib.load()
    ai = probe_image(a_image(A, desc6[0], desc6[1]))
    bi = probe_image(b_image(Bm))
    out = torch.zeros(128 * 16, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_uint32 * 6)(*desc6)
    idesc = (1 << 4) | (1 << 7) | (1 << 10) | (1 << 15) | (0 << 16) | ((16 >> 3) << 17) | ((128 >> 4) << 24)
    rc = lib.stile_debug_umma_probe(ai.data_ptr(), bi.data_ptr(), d, idesc, 0, out.data_ptr(), err.data_ptr(),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "probe")
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 16), int(err.item())


@functools.lru_cache(maxsize=None)
def umma_layout_ok():
    rng = np.random.default_rng(5)
    A = bf16_round(rng.standard_normal((128, 16)))
    Bm = bf16_round(rng.standard_normal((16, 16)))
    D, err = run_probe(A, Bm, KERNEL_DESC)
    ref = A.astype(np.float64) @ Bm.astype(np.float64).T
    return err == 0 and np.allclose(D, ref, rtol=1e-5, atol=1e-4)


def random_values(A, seed=0, dist="uniform"):
    A = sp.csr_matrix(A, dtype=np.float64).copy()
    rng = np.random.default_rng(seed)
    A.data = rng.uniform(-1, 1, size=A.nnz) if dist == "uniform" else rng.standard_normal(A.nnz)
    return A


# kind::tf32 probe images: A [128 (m) x 8 (k)] and B [16 (n) x 8 (k)] fp32,
# both K-major without swizzle (core matrices 8 rows x 16 B, LBO 128 B along
# k, SBO 256 B between 8-row groups).


def b_image_tf32(Bm, lbo=128, sbo=256):
    img = np.zeros(2048, dtype=np.uint32)
    bits = np.ascontiguousarray(Bm, dtype=np.float32).view(np.uint32)
    for n in range(16):
        for k in range(8):
            off = (n // 8) * sbo + (k // 4) * lbo + (n % 8) * 16 + (k % 4) * 4
            img[off // 4] = bits[n, k]
    return img


def a_image_tf32_kmajor(A, lbo=128, sbo=256):
    """A [128 (m) x 8 (k)] fp32, K-major no swizzle: core matrices 8 rows x
    4 elements, LBO between the two k cores, SBO between 8-row groups."""
    img = np.zeros(2048, dtype=np.uint32)
    bits = np.ascontiguousarray(A, dtype=np.float32).view(np.uint32)
    for m in range(128):
        for k in range(8):
            off = (m // 8) * sbo + (k // 4) * lbo + (m % 8) * 16 + (k % 4) * 4
            img[off // 4] = bits[m, k]
    return img


def run_probe_tf32(A, Bm, desc6=(128, 256, 0, 128, 256, 0), a_kmajor=True):
    import torch
    from stile_gb300 import _lib
    lib = _lib.load()
    assert a_kmajor, "the kernels use K-major tf32 operands only"
    aimg = a_image_tf32_kmajor(A, desc6[0], desc6[1])
    ai = probe_image(aimg)
    bi = probe_image(b_image_tf32(Bm, desc6[3], desc6[4]))
    out = torch.zeros(128 * 16, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_uint32 * 6)(*desc6)
    idesc = (1 << 4) | (2 << 7) | (2 << 10) | (0 << 15) | (0 << 16) | ((16 >> 3) << 17) | ((128 >> 4) << 24)
    rc = lib.stile_debug_umma_probe(ai.data_ptr(), bi.data_ptr(), d, idesc, 1, out.data_ptr(), err.data_ptr(),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "probe")
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 16), int(err.item())


def tf32_trunc(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def e4m3_round(x):
    """float32 values rounded to the nearest e4m3 value (saturated to
    +-448), kept as float32, and their e4m3 bytes."""
    import torch
    t = torch.as_tensor(np.asarray(x, np.float32)).clamp(-448.0, 448.0).to(torch.float8_e4m3fn)
    return t.to(torch.float32).numpy(), t.view(torch.uint8).numpy()


def kmajor_image_8bit(bytes_rk):
    """[rows, 32 (k)] bytes -> K-major, no-swizzle tcgen05 operand image:
    core matrices of 8 rows x 16 bytes, the two k halves 128 B apart (LBO),
    8-row groups 256 B apart (SBO)."""
    rows = bytes_rk.shape[0]
    img = np.zeros(8192, dtype=np.uint8)
    for r in range(rows):
        for k in range(32):
            img[(r // 8) * 256 + (k // 16) * 128 + (r % 8) * 16 + k % 16] = bytes_rk[r, k]
    return img


def run_probe_f8(Abytes, Bbytes):
    """One kind::f8f6f4 MMA (e4m3 x e4m3, K = 32) on K-major images."""
    import torch
    from stile_gb300 import _lib
    lib = _lib.load()
    ai = probe_image(kmajor_image_8bit(Abytes))
    bi = probe_image(kmajor_image_8bit(Bbytes))
    out = torch.zeros(128 * 16, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_uint32 * 6)(128, 256, 0, 128, 256, 0)
    idesc = (1 << 4) | (0 << 7) | (0 << 10) | (0 << 15) | (0 << 16) | ((16 >> 3) << 17) | ((128 >> 4) << 24)
    rc = lib.stile_debug_umma_probe(ai.data_ptr(), bi.data_ptr(), d, idesc, 2, out.data_ptr(), err.data_ptr(),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "probe")
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 16), int(err.item())


def kmajor_image_16bit(vals_rk):
    """[rows, 16 (k)] bf16 values -> K-major, no-swizzle image: core
    matrices of 8 rows x 16 bytes (8 k), the two k halves 128 B apart
    (LBO), 8-row groups 256 B apart (SBO)."""
    from stile_gb300.device import _to_bf16_bits
    rows = vals_rk.shape[0]
    bits = _to_bf16_bits(np.asarray(vals_rk, np.float32))
    img = np.zeros(4096, dtype=np.uint16)
    for r in range(rows):
        for k in range(16):
            img[((r // 8) * 256 + (k // 8) * 128 + (r % 8) * 16 + (k % 8) * 2) // 2] = bits[r, k]
    return img


def run_probe_bf16_kmajor(A, Bm):
    """One kind::f16 MMA (bf16, K = 16) with both operands K-major without
    swizzle (the SDDMM block kernel's layout)."""
    import torch
    from stile_gb300 import _lib
    lib = _lib.load()
    ai = probe_image(kmajor_image_16bit(A))
    bi = probe_image(kmajor_image_16bit(Bm))
    out = torch.zeros(128 * 16, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_uint32 * 6)(128, 256, 0, 128, 256, 0)
    idesc = (1 << 4) | (1 << 7) | (1 << 10) | (0 << 15) | (0 << 16) | ((16 >> 3) << 17) | ((128 >> 4) << 24)
    rc = lib.stile_debug_umma_probe(ai.data_ptr(), bi.data_ptr(), d, idesc, 0, out.data_ptr(), err.data_ptr(),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "probe")
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 16), int(err.item())


def kmajor_sw128_image_16bit(vals_rk):
    """[rows, K <= 64] bf16 values -> K-major image with the 128-byte
    swizzle: 128-byte rows of 64 k, 8-row atoms of 1 KB (SBO), the 16-byte
    chunk c of row r stored at chunk c ^ (r % 8)."""
    from stile_gb300.device import _to_bf16_bits
    rows, K = vals_rk.shape
    bits = _to_bf16_bits(np.asarray(vals_rk, np.float32))
    img = np.zeros(rows * 64, dtype=np.uint16)
    for r in range(rows):
        for k in range(K):
            off = (r // 8) * 1024 + (r % 8) * 128 + (((k // 8) ^ (r % 8)) << 4) + (k % 8) * 2
            img[off // 2] = bits[r, k]
    return img


def run_probe_bf16_kmajor_sw128(A, Bm):
    """One kind::f16 MMA (bf16, K = 16) with both operands K-major and the
    128-byte swizzle (SBO 1024 B; LBO unused by this layout)."""
    import torch
    from stile_gb300 import _lib
    lib = _lib.load()
    ai = probe_image(kmajor_sw128_image_16bit(A))
    bi = probe_image(kmajor_sw128_image_16bit(Bm))
    out = torch.zeros(128 * 16, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_uint32 * 6)(16, 1024, 2, 16, 1024, 2)
    idesc = (1 << 4) | (1 << 7) | (1 << 10) | (0 << 15) | (0 << 16) | ((16 >> 3) << 17) | ((128 >> 4) << 24)
    rc = lib.stile_debug_umma_probe(ai.data_ptr(), bi.data_ptr(), d, idesc, 0, out.data_ptr(), err.data_ptr(),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "probe")
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 16), int(err.item())
