"""ctypes binding of libnsg.so (the C ABI declared in include/nsg.h).

The product path has no fallback: if the library is missing or no CUDA device is
usable, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import threading
import os
from pathlib import Path

_LIB = None

OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_NONFINITE, ERR_NOT_CONVERGED, ERR_TIMEOUT, ERR_UNSUPPORTED = range(8)
F64, C128 = 0, 1
PREC_FP64, PREC_TF32X3, PREC_OZAKI = 0, 1, 2
PREC_OZAKI8 = 3
PRECISIONS = {"fp64": PREC_FP64, "tf32x3": PREC_TF32X3, "ozaki": PREC_OZAKI, "ozaki8": PREC_OZAKI8}


class NsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nsg error {code}: {msg}")
        self.code = code


p = C.c_void_p
i32 = C.c_int
i64 = C.c_int64
u64 = C.c_uint64
dbl = C.c_double
P_i64 = C.POINTER(C.c_int64)
P_i32 = C.POINTER(C.c_int32)
P_int = C.POINTER(C.c_int)
P_dbl = C.POINTER(C.c_double)
P_p = C.POINTER(C.c_void_p)

_SIGS = {
    "nsg_ctx_create": (i32, [i32, u64, P_p]),
    "nsg_ctx_destroy": (i32, [p]),
    "nsg_last_error": (C.c_char_p, [p]),
    "nsg_ctx_set_precision": (i32, [p, i32]),
    "nsg_ctx_synchronize": (i32, [p]),
    "nsg_ctx_memory": (i32, [p, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "nsg_device_memory": (i32, [i32, C.POINTER(u64), C.POINTER(u64)]),
    "nsg_region_step": (i32, [p, p, p, p, p, p, p, i32, i32, i32, dbl, dbl, i64, i64, P_p, P_p, P_dbl, C.POINTER(i64),
                              P_dbl]),
    "nsg_ctx_counters": (i32, [p, C.POINTER(u64), i32]),
    "nsg_ctx_event_record": (i32, [p, i32]),
    "nsg_ctx_event_elapsed": (i32, [p, i32, i32, C.POINTER(C.c_float)]),
    "nsg_ctx_profile": (i32, [p, i32]),
    "nsg_ctx_profile_read": (i32, [p, i32, C.POINTER(u64), P_dbl, P_dbl]),
    "nsg_ctx_wait_probe": (i32, [p, i64]),
    "nsg_ctx_set_tuning": (i32, [p, i32, i32]),
    "nsg_ctx_timers": (i32, [p, i32]),
    "nsg_ctx_phase": (i32, [p, i32, i32]),
    "nsg_get_timers": (i32, [p, C.POINTER(u64), P_dbl]),
    "nsg_tensor_create": (i32, [p, i32, i32, P_i64, P_p]),
    "nsg_tensor_upload": (i32, [p, i32, i32, P_i64, p, P_p]),
    "nsg_tensor_download": (i32, [p, p, p]),
    "nsg_tensor_release": (i32, [p, p]),
    "nsg_tensor_shape": (i32, [p, P_int, P_int, P_i64]),
    "nsg_tensor_copy": (i32, [p, p, P_p]),
    "nsg_tensor_device_ptr": (i32, [p, P_p]),
    "nsg_axpby": (i32, [p, dbl, dbl, p, dbl, dbl, p]),
    "nsg_dot": (i32, [p, p, p, P_dbl, P_dbl]),
    "nsg_norm": (i32, [p, p, P_dbl]),
    "nsg_permute": (i32, [p, p, P_int, i32, P_p]),
    "nsg_concat": (i32, [p, p, p, i32, P_p]),
    "nsg_contract": (i32, [p, i32, P_p, P_i32, P_int, i32, P_i32, P_p]),
    "nsg_linmap_create": (i32, [p, i32, P_p, P_i32, P_int, i32, P_i32, P_i32, P_p]),
    "nsg_linmap_apply": (i32, [p, p, p, p]),
    "nsg_linmap_release": (i32, [p, p]),
    "nsg_linmap_flops": (i32, [p, P_dbl]),
    "nsg_eigsolve": (i32, [p, p, p, i32, i32, dbl, P_dbl, P_int]),
    "nsg_exponentiate": (i32, [p, p, dbl, dbl, p, i32, i32, dbl, P_int, P_int]),
    "nsg_runge_kutta": (i32, [p, p, dbl, dbl, p, i32]),
    "nsg_factorize": (i32, [p, p, P_int, i32, dbl, i64, i64, P_p, P_p, P_i64, P_dbl, P_dbl, i64]),
    "nsg_factorize_complement": (i32, [p, p, P_int, i32, dbl, i64, i64, P_p, P_p, P_p, P_i64, P_dbl]),
    "nsg_qr": (i32, [p, p, P_int, i32, P_p, P_p]),
    "nsg_copy_submatrix": (i32, [p, p, i64, i64, i64, p, i64, i64, i64, i64, i64, i32]),
    "nsg_eigh": (i32, [p, p, P_int, i32, dbl, i64, i64, P_p, P_dbl, i64, P_i64, P_dbl]),
    "nsg_gemm_tf32x3_noalloc": (i32, [p, i64, i32, p, i64, i32, p, i64, i64, i64, i64, dbl, dbl, p,
                                      C.c_char_p, i32]),
}


def lib_path() -> Path:
    return Path(os.environ.get("NSG_LIB", Path(__file__).resolve().parent / "libnsg.so"))


def lib():
    """Load libnsg.so; raises if it was not built."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it with `python -m networksolvers_gb300.build`")
        L = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def exported_symbols():
    return list(_SIGS)


# the region step's phases, in the order of NSG_PHASE_* (include/nsg.h)
PHASES = ["extract", "subspace", "krylov", "heff", "factorize"]


class Context:
    """Owns an nsg_ctx (one CUDA stream + memory pool on one device)."""

    def __init__(self, device=0, hbm_budget=0, precision="fp64"):
        self.L = lib()
        self.timing = False
        h = C.c_void_p()
        self._check_raw(self.L.nsg_ctx_create(device, hbm_budget, C.byref(h)), None)
        self.h = h
        self.set_precision(precision)

    def _check_raw(self, rc, h):
        if rc != OK:
            msg = self.L.nsg_last_error(h).decode() if h else "context creation failed"
            raise NsgError(rc, msg)

    def check(self, rc):
        if rc != OK:
            raise NsgError(rc, self.L.nsg_last_error(self.h).decode())

    def set_precision(self, precision):
        code = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.check(self.L.nsg_ctx_set_precision(self.h, code))
        self.precision = precision

    def synchronize(self):
        self.check(self.L.nsg_ctx_synchronize(self.h))

    def memory(self):
        a, b, c = u64(), u64(), u64()
        self.check(self.L.nsg_ctx_memory(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def counters(self, reset=False):
        arr = (u64 * 4)()
        self.check(self.L.nsg_ctx_counters(self.h, arr, int(reset)))
        return {"launches": arr[0], "flops": arr[1], "contractions": arr[2], "applies": arr[3]}

    def record(self, slot):
        self.check(self.L.nsg_ctx_event_record(self.h, slot))

    def elapsed_ms(self, a, b):
        f = C.c_float()
        self.check(self.L.nsg_ctx_event_elapsed(self.h, a, b, C.byref(f)))
        return f.value

    def set_tuning(self, param, value):
        """Launch-choice override (0 restores the compiled-in tuning table): param
        "splitk" (FP64 GEMM K slices, 1..64), "tridiag" (-1 grid kernel, 2..16 cluster)
        or "dc_leaf" (divide and conquer leaf order, 4..32)."""
        code = {"splitk": 0, "tridiag": 1, "dc_leaf": 2}[param]
        self.check(self.L.nsg_ctx_set_tuning(self.h, code, int(value)))

    def profile(self, enable):
        self.check(self.L.nsg_ctx_profile(self.h, int(enable)))

    def profile_read(self):
        names = ["tc_gemm", "split", "simt_gemm", "tridiag", "dc"]
        out = {}
        for k, nm in enumerate(names):
            n, ms, fl = u64(), dbl(), dbl()
            self.check(self.L.nsg_ctx_profile_read(self.h, k, C.byref(n), C.byref(ms), C.byref(fl)))
            out[nm] = dict(launches=n.value, ms=ms.value, flops=fl.value)
        return out

    def timers(self, enable):
        """Per-phase device timers of the region step (nsg_ctx_timers); enabling resets."""
        self.check(self.L.nsg_ctx_timers(self.h, int(enable)))
        self.timing = bool(enable)

    def phase(self, name, begin):
        """Open (begin=True) or close a phase interval on the context's stream; a no-op
        unless the timers run."""
        if self.timing:
            self.check(self.L.nsg_ctx_phase(self.h, PHASES.index(name), int(bool(begin))))

    def read_timers(self):
        """{phase: {"count": closed intervals, "ms": summed device milliseconds}}."""
        n = (u64 * len(PHASES))()
        ms = (dbl * len(PHASES))()
        self.check(self.L.nsg_get_timers(self.h, n, ms))
        return {nm: dict(count=n[k], ms=ms[k]) for k, nm in enumerate(PHASES)}

    def close(self):
        if getattr(self, "h", None):
            self.L.nsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None
_local = threading.local()


def default_context():
    """The calling thread's context if it set one (worker threads of a solve pool each
    own a context and stream), else the process-wide one."""
    global _default
    ctx = getattr(_local, "ctx", None)
    if ctx is not None:
        return ctx
    if _default is None:
        _default = Context()
    return _default


def current_context():
    """The context default_context() would return, or None when none exists yet (creates
    nothing)."""
    return getattr(_local, "ctx", None) or _default


def set_default_context(ctx):
    """Process-wide default context (the main thread's)."""
    global _default
    _default = ctx


def device_free_bytes(device=0):
    """Free device memory in bytes (cudaMemGetInfo)."""
    L = lib()
    f, t = u64(), u64()
    rc = L.nsg_device_memory(int(device), C.byref(f), C.byref(t))
    if rc != 0:
        raise RuntimeError(f"nsg_device_memory failed ({rc})")
    return int(f.value)


def set_thread_context(ctx):
    """Default context of the calling thread only (None clears it)."""
    _local.ctx = ctx
