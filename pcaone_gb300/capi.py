"""ctypes binding of the C-ABI in include/pcaone_gpu.h.

The library is the in-tree build pcaone_gb300/lib/libpcaone_gb300.so (see
pcaone_gb300/build.py).  There is no fallback: if the library is missing or a
call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "lib", "libpcaone_gb300.so")

PCAONE_OK = 0
ERRORS = {-1: "PCAONE_E_ARG", -2: "PCAONE_E_CUDA", -3: "PCAONE_E_NOMEM", -4: "PCAONE_E_FORMAT",
          -5: "PCAONE_E_NUMERIC", -6: "PCAONE_E_LIMIT"}
PREC_FP32, PREC_BF16, PREC_FP8, PREC_BF16X3, PREC_FP64 = 0, 1, 2, 3, 4
SVD_SINGLE, SVD_WINDOW = 1, 2
MAX_L = 112

# every symbol include/pcaone_gpu.h declares
EXPORTS = [
    "pcaone_gpu_default_params", "pcaone_gpu_open", "pcaone_gpu_close", "pcaone_gpu_last_error",
    "pcaone_gpu_abi_version", "pcaone_gpu_timings", "pcaone_gpu_load_bed", "pcaone_gpu_load_bed_file_image",
    "pcaone_gpu_load_bed_device", "pcaone_gpu_counts", "pcaone_gpu_op_init", "pcaone_gpu_set_omega",
    "pcaone_gpu_set_flags", "pcaone_gpu_compute_g_and_h", "pcaone_gpu_compute_usv", "pcaone_gpu_run_halko",
    "pcaone_gpu_get_perm", "pcaone_gpu_matvec", "pcaone_gpu_load_synthetic", "pcaone_gpu_get_bed",
    "pcaone_gpu_set_profiling", "pcaone_gpu_kernel_stats", "pcaone_gpu_launch_count",
    "pcaone_gpu_matvec_static", "pcaone_gpu_mlp_default_params", "pcaone_gpu_set_warm_start",
    "pcaone_gpu_mlp_stats", "pcaone_gpu_mlp_forward_backward", "pcaone_gpu_load_dense",
    "pcaone_gpu_load_binary_file_image", "pcaone_gpu_load_synthetic_dense", "pcaone_gpu_project",
    "pcaone_gpu_random_omega", "pcaone_gpu_shuffle_order", "pcaone_gpu_set_wait_limit",
    "pcaone_gpu_set_product_form",
    "pcaone_gpu_load_bed_stream", "pcaone_gpu_load_bed_file_image_stream", "pcaone_gpu_stream_plan",
    "pcaone_gpu_stream_info", "pcaone_gpu_ooc_order", "pcaone_gpu_load_pgen_genovecs",
    "pcaone_gpu_load_pgen_file_image", "pcaone_gpu_pgen_layout", "pcaone_gpu_filter_maf",
    "pcaone_gpu_kept_snps",
]
MLP_PARAMS, MLP_INPUTS = 82689, 64


class Params(ctypes.Structure):
    _fields_ = [("svd", c_int), ("k", c_int), ("oversamples", c_int), ("maxp", c_int), ("bands", c_int),
                ("seed", c_int), ("rand", c_int), ("perm", c_int), ("emu", c_int), ("maxiter", c_int),
                ("tol", c_double), ("tolem", c_double), ("ploidy", c_int), ("standardize", c_int),
                ("precision", c_int)]


class MlpParams(ctypes.Structure):
    _fields_ = [("enable", c_int), ("train_entries", c_int), ("holdout_entries", c_int), ("epochs", c_int),
                ("batch", c_int), ("lr", ctypes.c_float), ("seed", c_uint64)]


class Desc(ctypes.Structure):
    _fields_ = [("device", c_int), ("verbose", c_int)]


class PcaoneError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIBPATH) -> ctypes.CDLL:
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run pcaone_gb300/build.py)")
    lib = ctypes.CDLL(path)
    P = POINTER
    lib.pcaone_gpu_default_params.argtypes = [P(Params)]
    lib.pcaone_gpu_default_params.restype = None
    lib.pcaone_gpu_open.argtypes = [P(Desc), P(c_void_p)]
    lib.pcaone_gpu_close.argtypes = [c_void_p]
    lib.pcaone_gpu_last_error.argtypes = [c_void_p]
    lib.pcaone_gpu_last_error.restype = c_char_p
    lib.pcaone_gpu_abi_version.argtypes = []
    lib.pcaone_gpu_timings.argtypes = [c_void_p, c_void_p]
    lib.pcaone_gpu_load_bed.argtypes = [c_void_p, c_void_p, c_uint64, c_uint32]
    lib.pcaone_gpu_load_bed_file_image.argtypes = [c_void_p, c_void_p, c_uint64, c_uint64, c_uint32]
    lib.pcaone_gpu_load_bed_device.argtypes = [c_void_p, c_void_p, c_uint64, c_uint64, c_uint32]
    lib.pcaone_gpu_counts.argtypes = [c_void_p, c_void_p, c_void_p]
    lib.pcaone_gpu_op_init.argtypes = [c_void_p, P(Params)]
    lib.pcaone_gpu_set_omega.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32]
    lib.pcaone_gpu_set_flags.argtypes = [c_void_p, c_int, c_int]
    lib.pcaone_gpu_compute_g_and_h.argtypes = [c_void_p, c_int, c_void_p, c_void_p]
    lib.pcaone_gpu_compute_usv.argtypes = [c_void_p, c_int, c_double, c_void_p, c_void_p, c_void_p, P(c_int)]
    lib.pcaone_gpu_run_halko.argtypes = [c_void_p, P(Params), c_void_p, c_void_p, c_void_p, P(c_int)]
    lib.pcaone_gpu_get_perm.argtypes = [c_void_p, c_void_p]
    lib.pcaone_gpu_matvec.argtypes = [c_void_p, c_void_p, c_void_p, c_int]
    lib.pcaone_gpu_load_synthetic.argtypes = [c_void_p, c_uint64, c_uint32, c_int, c_void_p, c_void_p, c_void_p,
                                              c_void_p, c_uint64]
    lib.pcaone_gpu_get_bed.argtypes = [c_void_p, c_void_p]
    lib.pcaone_gpu_filter_maf.argtypes = [c_void_p, ctypes.c_double, c_void_p]
    lib.pcaone_gpu_kept_snps.argtypes = [c_void_p, c_void_p]
    lib.pcaone_gpu_set_profiling.argtypes = [c_void_p, c_int]
    lib.pcaone_gpu_kernel_stats.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lib.pcaone_gpu_launch_count.argtypes = []
    lib.pcaone_gpu_matvec_static.argtypes = [c_void_p, c_uint64, c_uint64, c_uint32, c_void_p, c_int, c_void_p,
                                             c_void_p, c_void_p]
    lib.pcaone_gpu_load_dense.argtypes = [c_void_p, c_void_p, c_uint64, c_uint32]
    lib.pcaone_gpu_load_binary_file_image.argtypes = [c_void_p, c_void_p, c_uint64]
    lib.pcaone_gpu_project.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]
    lib.pcaone_gpu_load_synthetic_dense.argtypes = [c_void_p, c_uint64, c_uint32, c_int, c_void_p, c_void_p,
                                                    c_double, c_uint64]
    lib.pcaone_gpu_mlp_default_params.argtypes = [P(MlpParams)]
    lib.pcaone_gpu_mlp_default_params.restype = None
    lib.pcaone_gpu_set_warm_start.argtypes = [c_void_p, P(MlpParams)]
    lib.pcaone_gpu_mlp_stats.argtypes = [c_void_p, c_void_p]
    lib.pcaone_gpu_mlp_forward_backward.argtypes = [c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                                    c_void_p]
    lib.pcaone_gpu_random_omega.argtypes = [c_int, c_int, c_uint64, c_uint32, c_void_p]
    lib.pcaone_gpu_shuffle_order.argtypes = [c_uint64, c_void_p]
    lib.pcaone_gpu_set_wait_limit.argtypes = [c_void_p, ctypes.c_longlong]
    lib.pcaone_gpu_set_product_form.argtypes = [c_void_p, c_int]
    lib.pcaone_gpu_load_bed_stream.argtypes = [c_void_p, c_void_p, c_uint64, c_uint32, c_uint64, c_uint32]
    lib.pcaone_gpu_load_bed_file_image_stream.argtypes = [c_void_p, c_void_p, c_uint64, c_uint64, c_uint32,
                                                          c_uint64, c_uint32]
    lib.pcaone_gpu_ooc_order.argtypes = [c_uint64, c_uint32, c_int, c_uint32, c_void_p]
    lib.pcaone_gpu_load_pgen_genovecs.argtypes = [c_void_p, c_void_p, c_uint64, c_uint64, c_uint32]
    lib.pcaone_gpu_load_pgen_file_image.argtypes = [c_void_p, c_void_p, c_uint64, c_uint32]
    lib.pcaone_gpu_pgen_layout.argtypes = [c_void_p, c_uint64, c_uint32, P(c_int), P(c_uint64), P(c_uint32),
                                           P(c_uint64), P(c_uint64)]
    lib.pcaone_gpu_stream_plan.argtypes = [c_uint64, c_uint32, c_int, c_int, c_uint64, P(c_uint64), P(c_uint64)]
    lib.pcaone_gpu_stream_info.argtypes = [c_void_p, P(c_int), P(c_double)]
    for name in EXPORTS:
        if name not in ("pcaone_gpu_default_params", "pcaone_gpu_last_error", "pcaone_gpu_mlp_default_params"):
            getattr(lib, name).restype = c_int
    lib.pcaone_gpu_launch_count.restype = ctypes.c_ulonglong
    _lib = lib
    return lib


def random_omega(seed: int, rows: int, cols: int, gaussian: bool = True) -> np.ndarray:
    """The library's initial test matrix (pcaone_gpu_random_omega): host only."""
    out = np.empty((rows, cols), dtype=np.float64, order="F")
    rc = load().pcaone_gpu_random_omega(seed, int(gaussian), rows, cols, out.ctypes.data)
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_random_omega failed")
    return out


def shuffle_order(n: int) -> np.ndarray:
    """The library's in-core SNP order (pcaone_gpu_shuffle_order): host only."""
    out = np.empty(n, dtype=np.int32)
    rc = load().pcaone_gpu_shuffle_order(n, out.ctypes.data)
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_shuffle_order failed")
    return out


def stream_plan(nsnps: int, nsamples: int, svd: int, bands: int, device_budget: int):
    """The out-of-core block plan (pcaone_gpu_stream_plan): (SNPs per block,
    blocks).  Host only; PcaoneError(PCAONE_E_LIMIT) when the budget holds
    fewer than two blocks."""
    b, nb = c_uint64(0), c_uint64(0)
    rc = load().pcaone_gpu_stream_plan(nsnps, nsamples, svd, bands, device_budget, ctypes.byref(b), ctypes.byref(nb))
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_stream_plan failed")
    return int(b.value), int(nb.value)


def pgen_layout(image: bytes, nsamples: int = 0) -> dict:
    """The storage layout of a .pgen image (pcaone_gpu_pgen_layout): host only."""
    buf = np.frombuffer(image, dtype=np.uint8)
    mode, m, n, off, rec = c_int(0), c_uint64(0), c_uint32(0), c_uint64(0), c_uint64(0)
    rc = load().pcaone_gpu_pgen_layout(_ptr(buf), buf.size, nsamples, ctypes.byref(mode), ctypes.byref(m),
                                       ctypes.byref(n), ctypes.byref(off), ctypes.byref(rec))
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_pgen_layout failed")
    return {"mode": mode.value, "nsnps": m.value, "nsamples": n.value, "offset": off.value, "record_bytes": rec.value}


def ooc_order(nsnps: int, nsamples: int, bands: int, buffer_gb: int = 2) -> np.ndarray:
    """The out-of-core SNP order (pcaone_gpu_ooc_order): host only."""
    out = np.empty(nsnps, dtype=np.int32)
    rc = load().pcaone_gpu_ooc_order(nsnps, nsamples, bands, buffer_gb, out.ctypes.data)
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_ooc_order failed")
    return out


def default_params(**kw) -> Params:
    p = Params()
    load().pcaone_gpu_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def mlp_default_params(**kw) -> MlpParams:
    p = MlpParams()
    load().pcaone_gpu_mlp_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def mlp_forward_backward(X: np.ndarray, y: np.ndarray, params: np.ndarray, device: int = 0):
    """One forward + backward pass of the warm-start network on the GPU:
    returns (out, loss, grads)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    params = np.ascontiguousarray(params, dtype=np.float32)
    B = X.shape[0]
    if X.shape != (B, MLP_INPUTS) or y.shape != (B,) or params.shape != (MLP_PARAMS,):
        raise ValueError("shapes: X (B, 64), y (B,), params (82689,)")
    out = np.empty(B, np.float32)
    grads = np.empty(MLP_PARAMS, np.float32)
    loss = ctypes.c_float(0)
    rc = load().pcaone_gpu_mlp_forward_backward(device, X.ctypes.data, y.ctypes.data, B, params.ctypes.data,
                                                out.ctypes.data, ctypes.byref(loss), grads.ctypes.data)
    if rc != PCAONE_OK:
        raise PcaoneError(rc, "pcaone_gpu_mlp_forward_backward failed")
    return out, float(loss.value), grads


def _ptr(a):
    return None if a is None else a.ctypes.data


class Context:
    """One GPU context (pcaone_gpu_open / pcaone_gpu_close)."""

    def __init__(self, device: int = 0, verbose: int = 0):
        self.lib = load()
        self.h = c_void_p()
        d = Desc(device, verbose)
        rc = self.lib.pcaone_gpu_open(ctypes.byref(d), ctypes.byref(self.h))
        if rc != PCAONE_OK:
            raise PcaoneError(rc, "pcaone_gpu_open failed (no usable CUDA device?)")
        self.nsamples = 0
        self.nsnps = 0
        self.L = 0
        self.k = 0

    def close(self):
        if self.h:
            self.lib.pcaone_gpu_close(self.h)
            self.h = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != PCAONE_OK:
            msg = self.lib.pcaone_gpu_last_error(self.h)
            raise PcaoneError(rc, msg.decode() if msg else "")

    # ---- data ----
    def load_bed(self, packed: np.ndarray, nsamples: int):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_load_bed(self.h, _ptr(packed), packed.shape[0], nsamples))
        self.nsamples, self.nsnps = int(nsamples), int(packed.shape[0])

    def load_bed_file_image(self, image: bytes, nsnps: int, nsamples: int):
        buf = np.frombuffer(image, dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_load_bed_file_image(self.h, _ptr(buf), buf.size, nsnps, nsamples))
        self.nsamples, self.nsnps = int(nsamples), int(nsnps)

    def load_bed_stream(self, packed, nsamples: int, device_budget: int = 0, nsnps: int | None = None,
                        buffer_gb: int = 2):
        """Out-of-core load (pcaone_gpu_load_bed_stream): ``packed`` is a
        numpy array of rows or an address of host memory (then give nsnps)."""
        if isinstance(packed, np.ndarray):
            packed = np.ascontiguousarray(packed, dtype=np.uint8)
            ptr, nsnps = _ptr(packed), packed.shape[0]
        else:
            ptr = c_void_p(int(packed))
        self._check(self.lib.pcaone_gpu_load_bed_stream(self.h, ptr, int(nsnps), nsamples, int(device_budget),
                                                        int(buffer_gb)))
        self.nsamples, self.nsnps = int(nsamples), int(nsnps)

    def load_bed_file_image_stream(self, image: bytes, nsnps: int, nsamples: int, device_budget: int = 0,
                                   buffer_gb: int = 2):
        buf = np.frombuffer(image, dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_load_bed_file_image_stream(self.h, _ptr(buf), buf.size, nsnps, nsamples,
                                                                   int(device_budget), int(buffer_gb)))
        self.nsamples, self.nsnps = int(nsamples), int(nsnps)

    def load_pgen_genovecs(self, genovecs: np.ndarray, nsamples: int):
        """PLINK 2 hard calls (pcaone_gpu_load_pgen_genovecs): rows of 2-bit ALT
        counts, 3 = missing."""
        g = np.ascontiguousarray(genovecs, dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_load_pgen_genovecs(self.h, _ptr(g), g.shape[1], g.shape[0], nsamples))
        self.nsamples, self.nsnps = int(nsamples), int(g.shape[0])

    def load_pgen_file_image(self, image: bytes, nsamples: int = 0):
        buf = np.frombuffer(image, dtype=np.uint8)
        lay = pgen_layout(image, nsamples)
        self._check(self.lib.pcaone_gpu_load_pgen_file_image(self.h, _ptr(buf), buf.size, nsamples))
        self.nsamples, self.nsnps = int(lay["nsamples"]), int(lay["nsnps"])

    def stream_info(self):
        """(streamed, bytes copied into the device slots since the last call)."""
        on, nbytes = c_int(0), c_double(0)
        self._check(self.lib.pcaone_gpu_stream_info(self.h, ctypes.byref(on), ctypes.byref(nbytes)))
        return bool(on.value), float(nbytes.value)

    def load_bed_device(self, dev_ptr: int, pitch: int, nsnps: int, nsamples: int):
        self._check(self.lib.pcaone_gpu_load_bed_device(self.h, c_void_p(dev_ptr), pitch, nsnps, nsamples))
        self.nsamples, self.nsnps = int(nsamples), int(nsnps)

    def load_synthetic(self, model):
        """Generate ``model`` (synthetic.PopulationModel) on the device."""
        fr = np.ascontiguousarray(model.freq, dtype=np.float64)
        w = np.ascontiguousarray(model.weights, dtype=np.float64)
        ms = np.ascontiguousarray(model.miss_sample, dtype=np.float64)
        mj = np.ascontiguousarray(model.miss_snp, dtype=np.float64)
        self._check(self.lib.pcaone_gpu_load_synthetic(self.h, model.nsnps, model.nsamples, model.npop, _ptr(fr),
                                                       _ptr(w), _ptr(ms), _ptr(mj), model.seed))
        self.nsamples, self.nsnps = int(model.nsamples), int(model.nsnps)

    def get_bed(self, out_ptr: int = 0):
        """Packed genotypes back to the host: a new array, or into the host
        buffer at ``out_ptr`` (nsnps * ceil(N/4) bytes, e.g. pinned memory)."""
        if out_ptr:
            self._check(self.lib.pcaone_gpu_get_bed(self.h, c_void_p(out_ptr)))
            return None
        out = np.empty((self.nsnps, (self.nsamples + 3) // 4), dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_get_bed(self.h, _ptr(out)))
        return out

    def load_bed_ptr(self, host_ptr: int, nsnps: int, nsamples: int):
        """pcaone_gpu_load_bed from a raw host pointer (e.g. pinned memory)."""
        self._check(self.lib.pcaone_gpu_load_bed(self.h, c_void_p(host_ptr), nsnps, nsamples))
        self.nsamples, self.nsnps = int(nsamples), int(nsnps)

    def filter_maf(self, maf: float) -> int:
        """--maf: keep the SNPs with min(F, 1-F) > maf (Data::filter_snps_resize_F);
        returns the new SNP count."""
        n = ctypes.c_uint64(0)
        self._check(self.lib.pcaone_gpu_filter_maf(self.h, float(maf), ctypes.byref(n)))
        self.nsnps = int(n.value)
        return self.nsnps

    def kept_snps(self) -> np.ndarray:
        """File row of each resident SNP (Data::keepSNPs)."""
        out = np.empty(self.nsnps, dtype=np.int64)
        self._check(self.lib.pcaone_gpu_kept_snps(self.h, _ptr(out)))
        return out

    def counts(self):
        cnt = np.empty((self.nsnps, 4), dtype=np.int32)
        F = np.empty(self.nsnps, dtype=np.float64)
        self._check(self.lib.pcaone_gpu_counts(self.h, _ptr(cnt), _ptr(F)))
        return cnt, F

    # ---- operator ----
    def op_init(self, params: Params):
        self._check(self.lib.pcaone_gpu_op_init(self.h, ctypes.byref(params)))
        self.k, self.L = params.k, params.k + params.oversamples

    def set_omega(self, omega):
        if omega is None:
            self._check(self.lib.pcaone_gpu_set_omega(self.h, None, 0, 0))
            return
        om = np.asfortranarray(omega, dtype=np.float64)
        self._check(self.lib.pcaone_gpu_set_omega(self.h, _ptr(om), om.shape[0], om.shape[1]))

    def set_flags(self, update: bool, standardize: bool):
        self._check(self.lib.pcaone_gpu_set_flags(self.h, int(update), int(standardize)))

    def compute_g_and_h(self, pi: int):
        G = np.empty((self.nsnps, self.L), dtype=np.float64, order="F")
        H = np.empty((self.nsamples, self.L), dtype=np.float64, order="F")
        self._check(self.lib.pcaone_gpu_compute_g_and_h(self.h, pi, _ptr(G), _ptr(H)))
        return G, H

    def _outs(self):
        U = np.empty((self.nsamples, self.k), dtype=np.float64, order="F")
        S = np.empty(self.k, dtype=np.float64)
        V = np.empty((self.nsnps, self.k), dtype=np.float64, order="F")
        return U, S, V

    def compute_usv(self, p: int, tol: float):
        U, S, V = self._outs()
        ep = c_int(0)
        self._check(self.lib.pcaone_gpu_compute_usv(self.h, p, tol, _ptr(U), _ptr(S), _ptr(V), ctypes.byref(ep)))
        return U, S, V, ep.value

    def run_halko(self, params: Params, want_v: bool = True):
        self.k, self.L = params.k, params.k + params.oversamples
        U, S, V = self._outs()
        it = c_int(0)
        self._check(self.lib.pcaone_gpu_run_halko(self.h, ctypes.byref(params), _ptr(U), _ptr(S),
                                                  _ptr(V) if want_v else None, ctypes.byref(it)))
        return U, S, (V if want_v else None), it.value

    def load_dense(self, values: np.ndarray):
        """FileBinary matrix (SNPs x samples), held as FP16 on the device."""
        v = np.ascontiguousarray(values, dtype=np.float32)
        self._check(self.lib.pcaone_gpu_load_dense(self.h, v.ctypes.data, v.shape[0], v.shape[1]))
        self.nsnps, self.nsamples = v.shape

    def project(self, F: np.ndarray, V: np.ndarray, S: np.ndarray, mode: int = 1) -> np.ndarray:
        """Scores of the loaded samples on a fit (F, V in file order, S)."""
        F = np.ascontiguousarray(F, dtype=np.float64)
        Vc = np.asfortranarray(V, dtype=np.float64)
        S = np.ascontiguousarray(S, dtype=np.float64)
        k = Vc.shape[1]
        U = np.empty((self.nsamples, k), dtype=np.float64, order="F")
        self._check(self.lib.pcaone_gpu_project(self.h, _ptr(F), Vc.ctypes.data, _ptr(S), k, mode, U.ctypes.data))
        return U

    def load_synthetic_dense(self, model, sd: float = 0.1):
        """Continuous dosages of ``model`` generated on the device (FP16)."""
        fr = np.ascontiguousarray(model.freq, dtype=np.float64)
        w = np.ascontiguousarray(model.weights, dtype=np.float64)
        self._check(self.lib.pcaone_gpu_load_synthetic_dense(self.h, model.nsnps, model.nsamples, model.npop,
                                                             _ptr(fr), _ptr(w), float(sd), model.seed))
        self.nsnps, self.nsamples = model.nsnps, model.nsamples

    def load_binary_file_image(self, image: bytes):
        buf = np.frombuffer(image, dtype=np.uint8)
        self._check(self.lib.pcaone_gpu_load_binary_file_image(self.h, buf.ctypes.data, buf.size))
        m, n = np.frombuffer(image[:8], dtype=np.uint32)
        self.nsnps, self.nsamples = int(m), int(n)

    def set_warm_start(self, p):
        """Learned EM warm start for the next run_halko calls (None disables)."""
        self._check(self.lib.pcaone_gpu_set_warm_start(self.h, ctypes.byref(p) if p is not None else None))

    def mlp_stats(self):
        out = np.zeros(6)
        self._check(self.lib.pcaone_gpu_mlp_stats(self.h, _ptr(out)))
        return {"train_mse": out[0], "holdout_mse": out[1], "holdout_mse_mean_fill": out[2], "train_s": out[3],
                "fill_s": out[4], "filled": int(out[5])}

    def perm(self):
        out = np.empty(self.nsnps, dtype=np.int32)
        self._check(self.lib.pcaone_gpu_get_perm(self.h, _ptr(out)))
        return out

    def matvec(self, x: np.ndarray, standardize: bool = True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self._check(self.lib.pcaone_gpu_matvec(self.h, _ptr(x), _ptr(y), int(standardize)))
        return y

    def set_wait_limit(self, cycles: int):
        self._check(self.lib.pcaone_gpu_set_wait_limit(self.h, int(cycles)))

    def set_product_form(self, form: int):
        """G-shaped product launches: 0 one CTA per (tile, chunk) item, 1 resident CTAs
        taking items in turn, 2 (default) resident CTAs except in the E4M3 epochs."""
        self._check(self.lib.pcaone_gpu_set_product_form(self.h, int(form)))

    def set_profiling(self, on: bool):
        self._check(self.lib.pcaone_gpu_set_profiling(self.h, int(on)))

    def kernel_stats(self):
        """Per window-product class: device ms, algorithmic flops, launches
        (g/h_product: exact forms; g/h_product_e4m3: the FP8 form's E4M3 epochs)."""
        ms = np.zeros(4)
        fl = np.zeros(4)
        n = np.zeros(4, dtype=np.int64)
        self._check(self.lib.pcaone_gpu_kernel_stats(self.h, _ptr(ms), _ptr(fl), _ptr(n)))
        names = ("g_product", "h_product", "g_product_e4m3", "h_product_e4m3")
        return {names[i]: dict(ms=float(ms[i]), flops=float(fl[i]), launches=int(n[i])) for i in range(4)
                if i < 2 or n[i] > 0}

    def launch_count(self) -> int:
        return int(self.lib.pcaone_gpu_launch_count())

    def timings(self):
        t = np.zeros(4, dtype=np.float64)
        self._check(self.lib.pcaone_gpu_timings(self.h, _ptr(t)))
        return dict(total=t[0], products=t[1], qr_svd=t[2], em_fill=t[3])
