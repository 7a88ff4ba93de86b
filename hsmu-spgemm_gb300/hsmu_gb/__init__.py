"""Python host layer over the C ABI of the GB300 HSMU SpGEMM engine.

This mirrors the reference's operator interface for the C = A*B path
(``NHC_spgemm(compressed_bin*, NHC_bin*, NHC_CSR *A, NHC_CSR *B, NHC_CSR *C,
NHC_mask_matrix*)``, src/NHC_spgemm.cuh:7, with the device copies made by
``HtD_value_col_ptr``, src/loading.cuh:86-94, and the release by
``free_C_matrix``, src/loading.cuh:151-165): a caller uploads A and B to the
device, calls :meth:`Engine.spgemm`, and gets a device CSR ``C`` with sorted
columns and FP64 values, freed when the Python object is released.

PyTorch is used only for device memory and streams.  All compute runs in the
hand-written sm_103a kernels of ``libhsmu_gb.so``; there is no CPU fallback:
if the library is missing or no GB300-class device is present, constructing
an :class:`Engine` raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import gen  # noqa: F401  (re-exported: seeded workload generators)
from .gen import CSR

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libhsmu_gb.so")

HSMU_OK = 0
STATUS = {0: "HSMU_OK", 1: "HSMU_ERR_INVALID", 2: "HSMU_ERR_ALLOC", 3: "HSMU_ERR_CUDA",
          4: "HSMU_ERR_OVERFLOW", 5: "HSMU_ERR_UNSORTED", 6: "HSMU_ERR_INTERNAL",
          7: "HSMU_ERR_TIMEOUT", 8: "HSMU_ERR_NO_DEVICE", 9: "HSMU_ERR_UNSUPPORTED",
          10: "HSMU_ERR_CAPACITY"}
HSMU_ERR_CAPACITY = 10
BATCH_PRODUCT, BATCH_GALERKIN = 0, 1
ARITH_RN, ARITH_FMA, ARITH_IMUL = 0, 1, 2  # hsmu_opts.arith

# every symbol include/hsmu_gb.h declares (checked by the CPU test suite)
EXPORTS = ["hsmu_strerror", "hsmu_abi_version", "hsmu_handle_create", "hsmu_handle_destroy",
           "hsmu_spgemm", "hsmu_spgemm_tiled", "hsmu_spgemm_host", "hsmu_csr_transpose", "hsmu_btiles_build", "hsmu_btiles_free",
           "hsmu_csr_free", "hsmu_csr_download", "hsmu_selftest_dmul", "hsmu_btiles_build_noalloc",
           "hsmu_batch_create", "hsmu_batch_execute", "hsmu_batch_graph_launch", "hsmu_batch_status",
           "hsmu_batch_result", "hsmu_batch_set_params", "hsmu_batch_autotune", "hsmu_batch_destroy",
           "hsmu_gen_poisson7", "hsmu_gen_aggregation", "hsmu_spgemm_learned", "hsmu_row_features",
           "hsmu_row_nnz", "hsmu_mlp_forward", "hsmu_mlp_grad", "hsmu_mlp_adam", "hsmu_spgemm64",
           "hsmu_csr64_free", "hsmu_csr64_download", "hsmu_probe_fp64_rate", "hsmu_debug_fail_alloc",
           "hsmu_debug_plan_panels"]
MLP_FLOATS = 1259


class HsmuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class c_csr(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int32), ("N", ctypes.c_int32), ("nnz", ctypes.c_int32),
                ("owned", ctypes.c_int32), ("row_ptr", ctypes.c_void_p), ("col", ctypes.c_void_p),
                ("val", ctypes.c_void_p)]


class c_csr64(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int32), ("N", ctypes.c_int32), ("nnz", ctypes.c_int64),
                ("owned", ctypes.c_int32), ("reserved", ctypes.c_int32), ("row_ptr", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("val", ctypes.c_void_p)]


class c_btiles(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int32), ("N", ctypes.c_int32), ("ntiles", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("tile_ptr", ctypes.c_void_p),
                ("tile_col", ctypes.c_void_p), ("mask", ctypes.c_void_p),
                ("tile_off", ctypes.c_void_p)]


class c_opts(ctypes.Structure):
    _fields_ = [("validate", ctypes.c_int32), ("arith", ctypes.c_int32),
                ("window_cap", ctypes.c_int32), ("panels", ctypes.c_int32), ("wait_polls", ctypes.c_int32),
                ("no_tile_store", ctypes.c_int32), ("learned_always", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class c_mlp(ctypes.Structure):
    _fields_ = [("params", ctypes.c_void_p), ("margin", ctypes.c_float), ("reserved", ctypes.c_int32)]


class c_stats(ctypes.Structure):
    _fields_ = [("products", ctypes.c_uint64), ("nnz_c", ctypes.c_int64),
                ("ntiles_b", ctypes.c_int64), ("windows", ctypes.c_int64),
                ("ms_convert", ctypes.c_float), ("ms_symbolic", ctypes.c_float),
                ("ms_alloc", ctypes.c_float), ("ms_structure", ctypes.c_float),
                ("ms_numeric", ctypes.c_float), ("ms_total", ctypes.c_float),
                ("launches", ctypes.c_int32), ("routed", ctypes.c_int32),
                ("spec_capacity", ctypes.c_int64), ("fallback_rows", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libhsmu_gb.so (raises OSError if it was not built).  HSMU_LIB in the
    environment names an alternative build of the same library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("HSMU_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise OSError("libhsmu_gb.so not built: run __graft_entry__.build() (missing %s)" % path)
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.hsmu_strerror.restype = ctypes.c_char_p
    L.hsmu_strerror.argtypes = [ctypes.c_int]
    L.hsmu_abi_version.restype = ctypes.c_int
    L.hsmu_handle_create.argtypes = [ctypes.POINTER(P)]
    L.hsmu_handle_destroy.argtypes = [P]
    L.hsmu_spgemm.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), ctypes.POINTER(c_csr),
                              ctypes.POINTER(c_opts), P, ctypes.POINTER(c_stats)]
    L.hsmu_spgemm_tiled.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr),
                                    ctypes.POINTER(c_btiles), ctypes.POINTER(c_csr),
                                    ctypes.POINTER(c_opts), P, ctypes.POINTER(c_stats)]
    L.hsmu_spgemm_host.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), ctypes.POINTER(c_csr),
                                   ctypes.POINTER(c_opts), P, ctypes.POINTER(c_stats)]
    L.hsmu_btiles_build.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_btiles), P]
    L.hsmu_csr_transpose.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), P]
    L.hsmu_btiles_free.argtypes = [ctypes.POINTER(c_btiles)]
    L.hsmu_csr_free.argtypes = [ctypes.POINTER(c_csr)]
    L.hsmu_csr_download.argtypes = [ctypes.POINTER(c_csr), P, P, P, P]
    L.hsmu_btiles_build_noalloc.argtypes = [ctypes.POINTER(c_csr), P, P, P, P, P]
    L.hsmu_batch_create.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr),
                                    ctypes.POINTER(c_csr), ctypes.POINTER(c_opts), ctypes.POINTER(P), P]
    L.hsmu_batch_execute.argtypes = [P, P]
    L.hsmu_batch_graph_launch.argtypes = [P, P]
    L.hsmu_batch_status.argtypes = [P, P]
    L.hsmu_batch_result.argtypes = [P, ctypes.c_int, ctypes.POINTER(c_csr)]
    L.hsmu_batch_set_params.argtypes = [P, ctypes.c_int, ctypes.c_int]
    L.hsmu_batch_autotune.argtypes = [P, P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_float)]
    L.hsmu_batch_destroy.argtypes = [P]
    L.hsmu_gen_poisson7.argtypes = [ctypes.c_int, ctypes.POINTER(c_csr), P]
    L.hsmu_gen_aggregation.argtypes = [ctypes.c_int, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), P]
    L.hsmu_spgemm_learned.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), ctypes.POINTER(c_csr),
                                      ctypes.POINTER(c_mlp), ctypes.POINTER(c_opts), P, ctypes.POINTER(c_stats)]
    L.hsmu_row_features.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), P, P, P]
    L.hsmu_row_nnz.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), P, P]
    L.hsmu_mlp_forward.argtypes = [P, P, ctypes.c_int, P, P]
    L.hsmu_mlp_grad.argtypes = [P, P, P, ctypes.c_int, P, P, P]
    L.hsmu_mlp_adam.argtypes = [P, P, P, P, ctypes.c_float, ctypes.c_float, ctypes.c_int, P]
    L.hsmu_selftest_dmul.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), P]
    L.hsmu_probe_fp64_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), P]
    L.hsmu_debug_fail_alloc.argtypes = [ctypes.c_int64]
    L.hsmu_debug_plan_panels.argtypes = [ctypes.c_int32, P, ctypes.c_int64, P, ctypes.c_int32, P, P, P]
    L.hsmu_spgemm64.argtypes = [P, ctypes.POINTER(c_csr), ctypes.POINTER(c_csr), ctypes.POINTER(c_csr64),
                                ctypes.c_int64, ctypes.POINTER(c_opts), P]
    L.hsmu_csr64_free.argtypes = [ctypes.POINTER(c_csr64)]
    L.hsmu_csr64_download.argtypes = [ctypes.POINTER(c_csr64), P, P, P, P]
    _lib = L
    return L


def _check(rc: int, what: str):
    if rc != HSMU_OK:
        msg = load_library().hsmu_strerror(rc).decode()
        raise HsmuError(rc, "%s: %s" % (what, msg))


def _torch():
    import torch

    return torch


class DeviceCSR:
    """A CSR matrix in device memory.

    Inputs keep torch tensors alive (``from_host``); outputs of the engine hold
    library-owned arrays that are released with ``hsmu_csr_free`` on
    :meth:`free` or garbage collection."""

    def __init__(self, desc: c_csr, keep=None):
        self.desc = desc
        self._keep = keep

    @property
    def M(self):
        return self.desc.M

    @property
    def N(self):
        return self.desc.N

    @property
    def nnz(self):
        return self.desc.nnz

    @staticmethod
    def from_host(A: CSR, device="cuda", pinned_stream=None) -> "DeviceCSR":
        torch = _torch()
        rp = torch.from_numpy(np.ascontiguousarray(A.row_ptr, dtype=np.int32)).to(device)
        col = torch.from_numpy(np.ascontiguousarray(A.col, dtype=np.int32)).to(device)
        val = torch.from_numpy(np.ascontiguousarray(A.val, dtype=np.float64)).to(device)
        return DeviceCSR.from_tensors(A.M, A.N, rp, col, val)

    @staticmethod
    def from_tensors(M: int, N: int, rp, col, val) -> "DeviceCSR":
        torch = _torch()
        assert rp.dtype == torch.int32 and col.dtype == torch.int32 and val.dtype == torch.float64
        assert rp.is_contiguous() and col.is_contiguous() and val.is_contiguous()
        d = c_csr(M, N, int(col.numel()), 0, rp.data_ptr(), col.data_ptr() if col.numel() else 0,
                  val.data_ptr() if val.numel() else 0)
        return DeviceCSR(d, keep=(rp, col, val))

    def to_host(self, stream=None) -> CSR:
        L = load_library()
        rp = np.empty(self.M + 1, dtype=np.int32)
        col = np.empty(self.nnz, dtype=np.int32)
        val = np.empty(self.nnz, dtype=np.float64)
        _check(L.hsmu_csr_download(ctypes.byref(self.desc), rp.ctypes.data, col.ctypes.data,
                                   val.ctypes.data, _stream_ptr(stream)), "hsmu_csr_download")
        return CSR(self.M, self.N, rp, col, val)

    def row_ptr_host(self) -> np.ndarray:
        """C's row pointers (int32[M+1]) copied to the host."""
        rp = np.empty(self.M + 1, dtype=np.int32)
        _memcpy_d2h(rp.ctypes.data, self.desc.row_ptr, rp.nbytes)
        return rp

    def rows_to_host(self, rows, row_ptr=None):
        """Only the listed rows, copied to the host: (local row_ptr int64[k+1],
        col, val) in the order of `rows`.  Runs of consecutive rows are copied
        as one slice each, so a sample of a huge product costs a few copies."""
        rp = self.row_ptr_host() if row_ptr is None else row_ptr
        return _rows_from_device(rp, self.desc.col, self.desc.val, rows)

    def free(self):
        if self.desc.owned:
            load_library().hsmu_csr_free(ctypes.byref(self.desc))
        self._keep = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class BTiles:
    """B converted once to 64-column bit tiles, reusable across products."""

    def __init__(self, engine: "Engine", B: DeviceCSR, stream=None):
        self.desc = c_btiles()
        self.B = B
        _check(load_library().hsmu_btiles_build(engine.handle, ctypes.byref(B.desc),
                                                ctypes.byref(self.desc), _stream_ptr(stream)),
               "hsmu_btiles_build")

    @property
    def ntiles(self):
        return self.desc.ntiles

    def arrays(self):
        """(tile_ptr, tile_col, mask, tile_off) copied to host numpy arrays."""
        T = self.desc.ntiles
        out = []
        for ptr, n, dt in ((self.desc.tile_ptr, self.desc.M + 1, np.int32),
                           (self.desc.tile_col, T, np.int32), (self.desc.mask, T, np.uint64),
                           (self.desc.tile_off, T, np.int32)):
            a = np.empty(n, dtype=dt)
            if n:
                _memcpy_d2h(a.ctypes.data, ptr, a.nbytes)
            out.append(a)
        return tuple(out)

    def free(self):
        if self.desc.tile_ptr:
            load_library().hsmu_btiles_free(ctypes.byref(self.desc))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


_cudart = None


def _memcpy_d2h(dst: int, src: int, nbytes: int) -> None:
    """Synchronous device-to-host copy through the CUDA runtime the engine links."""
    global _cudart
    if _cudart is None:
        load_library()
        _cudart = ctypes.CDLL("libcudart.so.13")
        _cudart.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _cudart.cudaMemcpy.restype = ctypes.c_int
    rc = _cudart.cudaMemcpy(dst, src, nbytes, 2)  # cudaMemcpyDeviceToHost
    if rc != 0:
        raise HsmuError(3, "cudaMemcpy failed (%d)" % rc)


def _rows_from_device(rp: np.ndarray, col_ptr: int, val_ptr: int, rows):
    """(local row_ptr, col, val) of the listed rows of a device CSR whose row
    pointers (int32 or int64) are already on the host."""
    rows = np.asarray(rows, dtype=np.int64)
    lens = (rp[rows + 1] - rp[rows]).astype(np.int64)
    lrp = np.zeros(rows.size + 1, dtype=np.int64)
    np.cumsum(lens, out=lrp[1:])
    col = np.empty(int(lrp[-1]), dtype=np.int32)
    val = np.empty(int(lrp[-1]), dtype=np.float64)
    i = 0
    while i < rows.size:
        j = i + 1
        while j < rows.size and rows[j] == rows[j - 1] + 1:
            j += 1
        e0, e1 = int(rp[rows[i]]), int(rp[rows[j - 1] + 1])
        o = int(lrp[i])
        if e1 > e0:
            _memcpy_d2h(col.ctypes.data + 4 * o, col_ptr + 4 * e0, 4 * (e1 - e0))
            _memcpy_d2h(val.ctypes.data + 8 * o, val_ptr + 8 * e0, 8 * (e1 - e0))
        i = j
    return lrp, col, val


def _stream_ptr(stream):
    if stream is None:
        torch = _torch()
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


class DeviceCSR64:
    """A library-owned CSR with int64 row pointers (output of hsmu_spgemm64)."""

    def __init__(self, desc: c_csr64):
        self.desc = desc

    @property
    def M(self):
        return self.desc.M

    @property
    def N(self):
        return self.desc.N

    @property
    def nnz(self):
        return self.desc.nnz

    def row_ptr_host(self) -> np.ndarray:
        """C's row pointers (int64[M+1]) copied to the host."""
        rp = np.empty(self.M + 1, dtype=np.int64)
        _memcpy_d2h(rp.ctypes.data, self.desc.row_ptr, rp.nbytes)
        return rp

    def rows_to_host(self, rows, row_ptr=None):
        """Only the listed rows on the host: (local row_ptr int64[k+1], col, val)."""
        rp = self.row_ptr_host() if row_ptr is None else row_ptr
        return _rows_from_device(rp, self.desc.col, self.desc.val, rows)

    def to_host(self, stream=None):
        """(row_ptr int64, col int32, val float64) numpy arrays"""
        rp = np.empty(self.M + 1, dtype=np.int64)
        col = np.empty(self.nnz, dtype=np.int32)
        val = np.empty(self.nnz, dtype=np.float64)
        _check(load_library().hsmu_csr64_download(ctypes.byref(self.desc), rp.ctypes.data, col.ctypes.data,
                                                  val.ctypes.data, _stream_ptr(stream)), "hsmu_csr64_download")
        return rp, col, val

    def free(self):
        if self.desc.owned:
            load_library().hsmu_csr64_free(ctypes.byref(self.desc))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Engine:
    """One library handle on the current CUDA device (hsmu_handle_create)."""

    def __init__(self):
        torch = _torch()
        if not torch.cuda.is_available():
            raise HsmuError(8, "no CUDA device: the engine has no CPU path")
        torch.cuda.init()
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.hsmu_handle_create(ctypes.byref(h)), "hsmu_handle_create")
        self.handle = h
        self.last_stats: dict | None = None

    def close(self):
        if getattr(self, "handle", None):
            load_library().hsmu_handle_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spgemm_learned(self, A: DeviceCSR, B: DeviceCSR, params, margin: float, *, arith: int = 0,
                       validate: bool = False, stream=None, stats: bool = False, wait_polls: int = 0,
                       always: bool = False) -> DeviceCSR:
        """C = A * B with predicted row slots (hsmu_spgemm_learned); params: device float tensor.
        always (a test hook): use the prediction even where the plain path would be chosen."""
        L = load_library()
        C = c_csr()
        o = c_opts(int(validate), int(arith), 0, 0, int(wait_polls), 0, int(always))
        m = c_mlp(params.data_ptr(), float(margin), 0)
        st = c_stats()
        rc = L.hsmu_spgemm_learned(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc), ctypes.byref(C),
                                   ctypes.byref(m), ctypes.byref(o), _stream_ptr(stream),
                                   ctypes.byref(st) if stats else None)
        _check(rc, "hsmu_spgemm_learned")
        self.last_stats = st.as_dict() if stats else None
        return DeviceCSR(C)

    def row_features(self, A: DeviceCSR, B: DeviceCSR, stream=None):
        """(features [M,4] float32, products [M] int64) as device tensors."""
        torch = _torch()
        f = torch.empty((A.M, 4), dtype=torch.float32, device="cuda")
        p = torch.empty(A.M, dtype=torch.int64, device="cuda")
        _check(load_library().hsmu_row_features(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc),
                                                f.data_ptr(), p.data_ptr(), _stream_ptr(stream)),
               "hsmu_row_features")
        return f, p

    def row_nnz(self, A: DeviceCSR, B: DeviceCSR, stream=None):
        """exact nnz of every row of A*B (device int32 tensor) from the symbolic pass."""
        torch = _torch()
        n = torch.empty(A.M + 1, dtype=torch.int32, device="cuda")
        _check(load_library().hsmu_row_nnz(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc), n.data_ptr(),
                                           _stream_ptr(stream)), "hsmu_row_nnz")
        return n[:A.M]

    def spgemm(self, A: DeviceCSR, B: DeviceCSR, *, validate: bool = False, arith: int = 0,
               tiles: BTiles | None = None, stream=None, stats: bool = False, wait_polls: int = 0,
               tile_store: bool = True) -> DeviceCSR:
        """C = A * B on the device (hsmu_spgemm / hsmu_spgemm_tiled).  wait_polls: the
        test hook of hsmu_opts (bounded device waits give up after that many polls);
        tile_store=False: the structure pass repeats the large rows' OR walk."""
        L = load_library()
        C = c_csr()
        o = c_opts(int(validate), int(arith), 0, 0, int(wait_polls), int(not tile_store))
        st = c_stats()
        sp = ctypes.byref(st) if stats else None
        if tiles is None:
            rc = L.hsmu_spgemm(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc), ctypes.byref(C),
                               ctypes.byref(o), _stream_ptr(stream), sp)
        else:
            rc = L.hsmu_spgemm_tiled(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc),
                                     ctypes.byref(tiles.desc), ctypes.byref(C), ctypes.byref(o),
                                     _stream_ptr(stream), sp)
        _check(rc, "hsmu_spgemm")
        self.last_stats = st.as_dict() if stats else None
        return DeviceCSR(C)

    def spgemm64(self, A: DeviceCSR, B: DeviceCSR, *, max_panel_nnz: int = 0, validate: bool = False,
                 arith: int = 0, stream=None) -> "DeviceCSR64":
        """C = A * B with int64 row pointers (hsmu_spgemm64): rows processed in panels of
        at most max_panel_nnz entries (0: INT32_MAX), written into one C."""
        L = load_library()
        C = c_csr64()
        o = c_opts(int(validate), int(arith), 0)
        _check(L.hsmu_spgemm64(self.handle, ctypes.byref(A.desc), ctypes.byref(B.desc), ctypes.byref(C),
                               int(max_panel_nnz), ctypes.byref(o), _stream_ptr(stream)), "hsmu_spgemm64")
        return DeviceCSR64(C)


    def transpose(self, A: DeviceCSR, stream=None) -> DeviceCSR:
        """A^T on the device, rows in ascending column order (hsmu_csr_transpose)."""
        C = c_csr()
        _check(load_library().hsmu_csr_transpose(self.handle, ctypes.byref(A.desc), ctypes.byref(C),
                                                 _stream_ptr(stream)), "hsmu_csr_transpose")
        return DeviceCSR(C)

    def spgemm_host(self, A, B, out=None, *, arith: int = 0, panels: int = 0, validate: bool = False,
                    stream=None, stats: bool = False):
        """C = A * B with host operands and a host result (hsmu_spgemm_host).

        A, B: objects with M, N and host arrays row_ptr (int32), col (int32),
        val (float64) -- numpy arrays or CPU torch tensors (page-locked ones let
        the copies overlap the compute).  out: (row_ptr, col, val) host arrays
        to fill, col/val of any capacity; None allocates numpy arrays of the
        exact size (one extra symbolic pass).  Returns (row_ptr, col, val) of
        length M+1, nnz, nnz as views of the output arrays."""
        L = load_library()
        a = _host_desc(A)
        b = a if B is A else _host_desc(B)
        o = c_opts(int(validate), int(arith), 0, int(panels))
        st = c_stats()
        sp = ctypes.byref(st) if stats else None
        if out is None:
            probe = np.empty(A.M + 1, np.int32)
            c = c_csr(A.M, B.N, 0, 0, _host_ptr(probe), None, None)
            rc = L.hsmu_spgemm_host(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                    ctypes.byref(o), _stream_ptr(stream), None)
            if rc not in (HSMU_OK, HSMU_ERR_CAPACITY):
                _check(rc, "hsmu_spgemm_host")
            out = (probe, np.empty(c.nnz, np.int32), np.empty(c.nnz, np.float64))
        rp, col, val = out
        cap = min(_host_len(col), _host_len(val))
        c = c_csr(A.M, B.N, cap, 0, _host_ptr(rp), _host_ptr(col), _host_ptr(val))
        rc = L.hsmu_spgemm_host(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(o),
                                _stream_ptr(stream), sp)
        _check(rc, "hsmu_spgemm_host")
        self.last_stats = st.as_dict() if stats else None
        return rp[:A.M + 1], col[:c.nnz], val[:c.nnz]


def _host_ptr(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        if x.is_cuda or not x.is_contiguous():
            raise ValueError("host arrays must be contiguous CPU tensors")
        return x.data_ptr()
    if not x.flags["C_CONTIGUOUS"]:
        raise ValueError("host arrays must be contiguous")
    return x.ctypes.data


def _host_len(x) -> int:
    return int(x.numel()) if hasattr(x, "numel") else int(x.size)


def _host_desc(X) -> c_csr:
    for arr, dt in ((X.row_ptr, "int32"), (X.col, "int32"), (X.val, "float64")):
        name = str(arr.dtype).replace("torch.", "")
        if name != dt:
            raise ValueError("host CSR arrays must be int32/int32/float64, got %s" % name)
    nnz = _host_len(X.col)
    return c_csr(X.M, X.N, nnz, 0, _host_ptr(X.row_ptr), _host_ptr(X.col) if nnz else None,
                 _host_ptr(X.val) if nnz else None)


class Batch:
    """Many products in one persistent launch (hsmu_batch_*).

    kind BATCH_PRODUCT: C_p = A[p] * B[p]; BATCH_GALERKIN: C_p = Pt[p] * (A[p] * B[p]).
    Results are views into the batch's output pool (valid while the batch lives)."""

    def __init__(self, engine: "Engine", kind: int, A, B, Pt=None, arith: int = 0, stream=None,
                 wait_polls: int = 0):
        n = len(A)
        self._keep = (list(A), list(B), list(Pt) if Pt is not None else None)
        arrA = (c_csr * n)(*[x.desc for x in A])
        arrB = (c_csr * n)(*[x.desc for x in B])
        arrP = (c_csr * n)(*[x.desc for x in Pt]) if Pt is not None else None
        o = c_opts(0, int(arith), 0, 0, int(wait_polls))
        h = ctypes.c_void_p()
        _check(load_library().hsmu_batch_create(engine.handle, kind, n, arrA, arrB, arrP, ctypes.byref(o),
                                                ctypes.byref(h), _stream_ptr(stream)), "hsmu_batch_create")
        self.handle = h
        self.n = n

    def execute(self, stream=None):
        _check(load_library().hsmu_batch_execute(self.handle, _stream_ptr(stream)), "hsmu_batch_execute")

    def graph_launch(self, stream=None):
        _check(load_library().hsmu_batch_graph_launch(self.handle, _stream_ptr(stream)), "hsmu_batch_graph_launch")

    def status(self, stream=None):
        _check(load_library().hsmu_batch_status(self.handle, _stream_ptr(stream)), "hsmu_batch_status")

    def set_params(self, tiny: int, grid: int = 0):
        _check(load_library().hsmu_batch_set_params(self.handle, tiny, grid), "hsmu_batch_set_params")

    def autotune(self, stream=None):
        t, g, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(load_library().hsmu_batch_autotune(self.handle, _stream_ptr(stream), ctypes.byref(t),
                                                  ctypes.byref(g), ctypes.byref(ms)), "hsmu_batch_autotune")
        return t.value, g.value, ms.value

    def result(self, p: int) -> "DeviceCSR":
        C = c_csr()
        _check(load_library().hsmu_batch_result(self.handle, p, ctypes.byref(C)), "hsmu_batch_result")
        return DeviceCSR(C, keep=self)

    def close(self):
        if getattr(self, "handle", None):
            load_library().hsmu_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gen_poisson7(side: int, stream=None) -> "DeviceCSR":
    """7-point Poisson matrix of a side^3 grid generated on the device (owned)."""
    C = c_csr()
    _check(load_library().hsmu_gen_poisson7(side, ctypes.byref(C), _stream_ptr(stream)), "hsmu_gen_poisson7")
    return DeviceCSR(C)


def gen_aggregation(side: int, stream=None):
    """(P, P^T) of the 2x2x2 aggregation of a side^3 grid, generated on the device (owned)."""
    P, Pt = c_csr(), c_csr()
    _check(load_library().hsmu_gen_aggregation(side, ctypes.byref(P), ctypes.byref(Pt), _stream_ptr(stream)),
           "hsmu_gen_aggregation")
    return DeviceCSR(P), DeviceCSR(Pt)


def selftest_dmul(n: int = 1 << 24, seed: int = 1) -> int:
    """Mismatches of the integer-pipe multiply vs the FP64 pipe on n pairs (0 expected)."""
    out = ctypes.c_uint64(0)
    _check(load_library().hsmu_selftest_dmul(n, seed, ctypes.byref(out), _stream_ptr(None)),
           "hsmu_selftest_dmul")
    return int(out.value)


def debug_fail_alloc(nth: int) -> None:
    """Test hook: the nth device allocation from now on fails (0 disarms)."""
    _check(load_library().hsmu_debug_fail_alloc(int(nth)), "hsmu_debug_fail_alloc")


def probe_fp64_rate(iters: int = 8192, stream=None) -> float:
    """FP64 lane operations per second of the device's FP64 pipe (rounded
    multiply and add chains over a full grid; hsmu_probe_fp64_rate)."""
    out = ctypes.c_double(0.0)
    _check(load_library().hsmu_probe_fp64_rate(iters, ctypes.byref(out), _stream_ptr(stream)),
           "hsmu_probe_fp64_rate")
    return float(out.value)


def spgemm_host(A: CSR, B: CSR, engine: Engine | None = None, **kw) -> CSR:
    """Convenience: upload A and B, multiply on the GPU, download C."""
    eng = engine or Engine()
    dA = DeviceCSR.from_host(A)
    dB = dA if B is A else DeviceCSR.from_host(B)
    C = eng.spgemm(dA, dB, **kw)
    out = C.to_host()
    C.free()
    return out
