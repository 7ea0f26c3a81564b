"""ctypes binding of libfhgb300.so (the C ABI declared in include/fhgb300.h).

The library is the only compute path: importing works anywhere, but every call raises
``FHError`` when the shared object is missing or no CUDA device is usable.  There is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfhgb300.so")

FH_OK = 0
STATUS_NAMES = {0: "FH_OK", 1: "FH_ERR_ARG", 2: "FH_ERR_UNSUPPORTED", 3: "FH_ERR_NONFINITE",
                4: "FH_ERR_ILLCOND", 5: "FH_ERR_LAUNCH", 6: "FH_ERR_INDEX", 7: "FH_ERR_TIMEOUT"}


class FHError(RuntimeError):
    def __init__(self, func, status, msg=""):
        self.status = status
        super().__init__("%s failed: %s (%d)%s" % (func, STATUS_NAMES.get(status, "?"), status,
                                                   (": " + msg) if msg else ""))


class fh_tile(C.Structure):
    _fields_ = [("chrom", C.c_int32), ("row0", C.c_int32), ("rows", C.c_int32),
                ("width", C.c_int32), ("shift", C.c_int32), ("s0", C.c_int32),
                ("rank", C.c_int32), ("n_rwr", C.c_int32), ("xoff", C.c_int64),
                ("brow0", C.c_int64), ("uoff", C.c_int64)]


TILE_DTYPE = np.dtype([("chrom", "<i4"), ("row0", "<i4"), ("rows", "<i4"), ("width", "<i4"),
                       ("shift", "<i4"), ("s0", "<i4"), ("rank", "<i4"), ("n_rwr", "<i4"),
                       ("xoff", "<i8"), ("brow0", "<i8"), ("uoff", "<i8")])
assert TILE_DTYPE.itemsize == C.sizeof(fh_tile) == 56

P, I32, I64, SZ, D = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t, C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "fh_status_string": (C.c_char_p, [C.c_int]),
    "fh_version": (C.c_int, []),
    "fh_contacts_count": (C.c_int, [P, P, P, I64, I32, P, I32, I32, I32, P, P, P]),
    "fh_scan_workspace": (SZ, [I64]),
    "fh_scan_add_base": (C.c_int, [P, I64, P, P]),
    "fh_exclusive_scan": (C.c_int, [P, I64, P, P, SZ, P]),
    "fh_exclusive_scan_noalloc": (C.c_int, [P, I64, P, P]),
    "fh_contacts_scatter": (C.c_int, [P, P, P, P, I64, I32, P, I32, I32, I32, P, P, P, P]),
    "fh_densify_tile": (C.c_int, [P, I32, I32, I32, I32, P, P, P, P]),
    "fh_rwr_tiles_f32": (C.c_int, [P, I32, I32, I32, I32, P, P, P, I64, P, P, P]),
    "fh_rwr_tiles_rp_f32": (C.c_int, [P, I32, I32, I32, I32, P, P, C.c_float, P, I64, P, P, P]),
    "fh_rwr_grad_f32": (C.c_int, [P, I32, I32, I32, I32, P, P, C.c_float, P, P, I64, P, P]),
    "fh_recon_workspace": (SZ, [I32, I64, I32]),
    "fh_recon_loss_f32": (C.c_int, [P, I64, I32, I64, P, P, I32, P, P, SZ, P]),
    "fh_recon_loss_bwd_f32": (C.c_int, [P, P, I64, I32, I64, P, P, I32, P, P, P, P, P, P, SZ,
                                        P]),
    "fh_factor_grad_workspace": (SZ, [I32, I32, I32]),
    "fh_factor_grad_f32": (C.c_int, [I32, I32, P, P, I32, P, P, P, I32, I32, I32, P, P, P, P,
                                     SZ, P]),
    "fh_conv_tiles_f32": (C.c_int, [P, I32, I32, I32, I32, P, P, P, I64, P, P]),
    "fh_conv_dense_f32": (C.c_int, [P, I32, I32, I32, P, P]),
    "fh_rwr_tiles_dense_f32": (C.c_int, [P, I32, I32, I32, I32, P, P, I64, P, P, P]),
    "fh_rwr_tiles_dense_bf16": (C.c_int, [P, I32, I32, I32, I32, P, P, I64, I64, P, P, P]),
    "fh_rwr_tiles_dense_deltas": (C.c_int, [P, I32, I32, I32, I32, P, I64, I32, P, P, P]),
    "fh_rwr_dense_f32": (C.c_int, [P, I32, I32, I32, I32, I32, P, P, P]),
    "fh_rwr_col_tiles": (C.c_int, [P, I32, I32, I32, I32, P, P, P, P, I64, P, P, P, I64, I64,
                                   P, P, P, P]),
    "fh_rwr_col_dense": (C.c_int, [P, I32, I32, I32, I32, I32, P, P, P, P]),
    "fh_col_coverage": (C.c_int, [P, I32, I32, P, I32, P, I64, I64, P, P]),
    "fh_col_coverage_finalize": (C.c_int, [P, I64, P]),
    "fh_rwr_dense_deltas": (C.c_int, [P, I32, I32, I32, I32, I32, P, P, P]),
    "fh_rwr_tiles_deltas": (C.c_int, [P, I32, I32, I32, I32, P, P, I32, P, P, P]),
    "fh_xe_f32": (C.c_int, [P, I64, I32, I64, P, I32, P, P]),
    "fh_xg_splits": (C.c_int, [I32, I64]),
    "fh_xg_f32": (C.c_int, [P, I64, I32, I64, P, I32, I32, P, P, I32, P]),
    "fh_project_y_f32": (C.c_int, [P, P, I64, P, P, I32, P, I32, P]),
    "fh_rwr_tiles_bf16": (C.c_int, [P, I32, I32, I32, I32, P, P, P, I64, I64, P, P, P]),
    "fh_rwr_tiles_tc": (C.c_int, [P, I32, I32, I32, I32, P, P, P, I64, I64, P, I32, P, P]),
    "fh_split_bf16": (C.c_int, [P, I64, I32, I64, P, P]),
    "fh_xe_bf16": (C.c_int, [P, I64, I32, I32, I32, I64, P, I32, I32, P, P, P]),
    "fh_xg_bf16_splits": (C.c_int, [I32, I64]),
    "fh_xg_bf16": (C.c_int, [P, I64, I32, I32, I32, I64, P, I32, I32, I32, P, P, I32, P, P]),
    "fh_procrustes_f32": (C.c_int, [P, P, I64, I32, I32, P, P, I32, P, P, I32, I32, I32, P, P,
                                    P, P, P]),
    "fh_projection_g_f32": (C.c_int, [P, P, I64, I32, I32, P, I32, P, P, I32, I32, I32, P, P,
                                      P]),
    "fh_polar_smem": (SZ, [I32, I32]),
    "fh_polar_f32": (C.c_int, [P, I64, I32, I32, P, P, P, P]),
    "fh_polar_svals_f32": (C.c_int, [P, P, I64, I32, I32, P, P]),
    "fh_meta_polar_workspace": (SZ, [I32, I32]),
    "fh_meta_polar": (C.c_int, [P, I32, I32, I32, P, P, P, SZ, P, P]),
    "fh_cp_workspace": (SZ, [I32, I32, I32, I32]),
    "fh_cp_als": (C.c_int, [I32, I32, P, P, P, P, P, I32, I32, I32, I32, I32, P, P, P, SZ, P,
                            P]),
    "fh_core_norm": (C.c_int, [I32, I32, P, P, P, P, P, I32, I32, I32, I32, P, P, SZ, P, P]),
    "fh_selftest_wait": (C.c_int, [P, I64, P]),
    "fh_pack_workspace": (SZ, [I32, I32, I32, I64]),
    "fh_embed_assemble": (C.c_int, [P, I32, I32, I64, P, I32, I64, P, P, I64, P]),
    "fh_gemm_scale_f32": (C.c_int, [P, I64, P, I64, P, I32, I32, I32, P, I64, P]),
    "fh_quantile_workspace": (SZ, [I32, I32]),
    "fh_quantile_uniform": (C.c_int, [P, I32, I32, P, P, SZ, P]),
    "fh_lstsq_workspace": (SZ, [I32, I32]),
    "fh_lstsq_residual": (C.c_int, [P, I32, I32, P, I64, I32, I32, P, I64, P, SZ, P, P]),
    "fh_range_svd_workspace": (SZ, [I32, I32, I32]),
    "fh_range_svd": (C.c_int, [P, I64, I32, I32, P, I64, I32, I32, P, I64, P, P, SZ, P, P]),
    "fh_l2_rows": (C.c_int, [P, I64, I32, I32, P, I64, P]),
    "fh_impute_maps": (C.c_int, [P, P, I64, I32, P, I64, I32, I32, P, P, P]),
    "fh_cross_f32": (C.c_int, [P, I64, I32, P, I64, I32, I32, P, I64, P]),
    "fh_pool_rows": (C.c_int, [P, I32, P, P, I64, P, I64, I32, P, I64, P]),
    "fh_unpool_rows": (C.c_int, [P, I32, P, P, I64, I64, P, I64, I32, P, I64, P]),
    "fh_pack_chromosome": (C.c_int, [P, P, P, P, I32, P, I32, I32, I32, I32, P, P, I64, P, P,
                                     SZ, P, P]),
    "fh_host_alloc": (C.c_int, [I64, P]),
    "fh_host_free": (C.c_int, [P]),
    "fh_memcpy_async": (C.c_int, [P, P, I64, P]),
}

# kernels each entry point launches (the count the benchmark reports as gpu_launches)
_KERNELS = {"fh_contacts_count": 1, "fh_exclusive_scan": 3, "fh_scan_add_base": 1, "fh_exclusive_scan_noalloc": 3, "fh_contacts_scatter": 1,
            "fh_densify_tile": 1, "fh_rwr_tiles_f32": 1, "fh_rwr_dense_f32": 1,
            "fh_rwr_dense_deltas": 1, "fh_rwr_tiles_deltas": 1, "fh_xe_f32": 1, "fh_xg_f32": 2,
            "fh_project_y_f32": 1, "fh_procrustes_f32": 1, "fh_projection_g_f32": 1,
            "fh_rwr_tiles_bf16": 1, "fh_rwr_tiles_tc": 1, "fh_split_bf16": 1, "fh_xe_bf16": 1, "fh_xg_bf16": 2,
            "fh_conv_tiles_f32": 1, "fh_conv_dense_f32": 1, "fh_rwr_tiles_dense_f32": 1,
            "fh_rwr_tiles_dense_bf16": 1, "fh_rwr_tiles_dense_deltas": 1,
            "fh_rwr_tiles_rp_f32": 1, "fh_rwr_grad_f32": 1, "fh_recon_loss_f32": 2,
            "fh_recon_loss_bwd_f32": 4, "fh_factor_grad_f32": 2, "fh_rwr_col_tiles": 1,
            "fh_rwr_col_dense": 1, "fh_col_coverage": 1, "fh_col_coverage_finalize": 1,
            "fh_polar_f32": 1, "fh_polar_svals_f32": 1, "fh_meta_polar": 5, "fh_core_norm": 2,
            "fh_selftest_wait": 1, "fh_pack_chromosome": 18,
            "fh_embed_assemble": 2, "fh_gemm_scale_f32": 1, "fh_quantile_uniform": 3,
            "fh_lstsq_residual": 7, "fh_range_svd": 13, "fh_l2_rows": 1,
            "fh_impute_maps": 1, "fh_cross_f32": 1, "fh_pool_rows": 1,
            "fh_unpool_rows": 1}
launches = 0


def _kernel_count(name, args):
    if name == "fh_cp_als":
        n_iter = args[11]
        return 2 if n_iter == 0 else 3 + 4 * n_iter
    if name == "fh_range_svd":
        return 14 if args[10] else 13
    return _KERNELS.get(name, 0)


_lib = None


def load():
    """Loads the shared library (building nothing).  Raises FHError if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FHError("load", 5, "%s is missing; run fh_gb300.build.build()" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def exported_symbols():
    return sorted(SIGNATURES)


def call(name, *args):
    """Calls an fh_status-returning entry point and raises FHError on failure."""
    global launches
    f = getattr(load(), name)
    st = f(*args)
    launches += _kernel_count(name, args)
    if st != FH_OK:
        raise FHError(name, st, load().fh_status_string(st).decode())
    return st


def value(name, *args):
    """Calls an entry point that returns a plain value (a size or a count)."""
    return getattr(load(), name)(*args)


_HOST_BUFFERS = {}     # address -> bytes of the live HostBuffers


class HostBuffer:
    """Page-locked host memory from the library (fh_host_alloc: cudaHostAlloc, exactly the
    bytes asked for), freed when the last reference to it (or to an array over it) goes."""

    def __init__(self, nbytes, zero=True):
        p = C.c_void_p()
        call("fh_host_alloc", int(nbytes), C.byref(p))
        self.ptr = int(p.value)
        self.nbytes = int(nbytes)
        _HOST_BUFFERS[self.ptr] = self.nbytes
        if zero:
            C.memset(self.ptr, 0, self.nbytes)

    def array(self, dtype, shape):
        """A numpy array over the buffer; it keeps the buffer alive."""
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        if n > self.nbytes:
            raise FHError("HostBuffer", 1, "array larger than the buffer")
        raw = (C.c_uint8 * max(n, 1)).from_address(self.ptr)
        raw._owner = self
        return np.frombuffer(raw, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.ptr:
            _HOST_BUFFERS.pop(self.ptr, None)
            call("fh_host_free", self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def host_pinned(addr, nbytes):
    """True if [addr, addr + nbytes) lies in a live HostBuffer (page-locked already)."""
    for p, n in _HOST_BUFFERS.items():
        if p <= addr and addr + nbytes <= p + n:
            return True
    return False


def pinned_copy(a):
    """A copy of numpy array a in page-locked memory (a HostBuffer)."""
    a = np.ascontiguousarray(a)
    out = HostBuffer(max(a.nbytes, 1), zero=False).array(a.dtype, a.shape)
    np.copyto(out, a)
    return out


def ptr(t):
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
