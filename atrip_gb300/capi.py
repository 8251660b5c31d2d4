"""ctypes binding of the C ABI declared in include/atrip_gb300.h.

The shared library is built in-tree (``atrip_gb300/_lib``).  Loading fails
loudly when it is missing: there is no CPU fallback anywhere in the product.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

# enum atrip_status
OK, ERR_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_STATE, ERR_TIMEOUT, ERR_UNSUPPORTED, \
    ERR_NO_DEVICE = range(8)
# enum atrip_tensor
EPSI, EPSA, TAI, TABIJ, VABIJ, VIJKA, VABCI, JIJKA, JABCI = range(9)
TENSOR_IDS = {"epsi": EPSI, "epsa": EPSA, "Tai": TAI, "Tabij": TABIJ, "Vabij": VABIJ,
              "Vijka": VIJKA, "Vabci": VABCI, "Jijka": JIJKA, "Jabci": JABCI}
# enum atrip_form
FORM_FP64, FORM_SPLIT_BF16, FORM_AUTO, FORM_SPLIT_F16 = range(4)
FORMS = {"fp64": FORM_FP64, "split_bf16": FORM_SPLIT_BF16, "auto": FORM_AUTO,
         "split_f16": FORM_SPLIT_F16}

EXPORTED = [
    "atrip_gpu_create", "atrip_gpu_upload", "atrip_gpu_upload_device", "atrip_gpu_release",
    "atrip_gpu_run", "atrip_gpu_tuple_energies", "atrip_gpu_n_tuples", "atrip_gpu_tuple_at",
    "atrip_gpu_destroy", "atrip_gpu_last_error", "atrip_gpu_version", "atrip_gpu_measure_peaks",
    "atrip_gpu_run_fp64_noalloc", "atrip_gpu_batch_create", "atrip_gpu_batch_run",
    "atrip_gpu_batch_destroy", "atrip_gpu_batch_plan", "atrip_gpu_set_tuning",
    "atrip_gpu_get_tuning", "atrip_gpu_batch_set_tuning", "atrip_gpu_last_sums",
    "atrip_gpu_device_count", "atrip_gpu_split_profile",
]

# counters of atrip_gpu_split_profile, by index
SPLIT_PROFILE = ("producer_total", "producer_wait_stage", "producer_wait_tuple_slot",
                 "mma_total", "mma_wait_tuple", "mma_wait_accumulator", "mma_wait_stage",
                 "epilogue_total", "epilogue_wait_tuple", "epilogue_wait_w_buffer",
                 "epilogue_wait_accumulator", "energy_total", "energy_wait_tuple",
                 "energy_wait_w", "energy_w_convert", None, "stages", "tuples", "ctas")
SPLIT_PROFILE_COUNTERS = 20


class AtripError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"atrip_gb300 status {status}: {message}")
        self.status = status


# enum atrip_field
FIELD_REAL, FIELD_COMPLEX = range(2)


class Dims(ctypes.Structure):
    _fields_ = [("no", ctypes.c_int32), ("nv", ctypes.c_int32), ("device", ctypes.c_int32),
                ("field", ctypes.c_int32)]


class RunOptions(ctypes.Structure):
    _fields_ = [("form", ctypes.c_int32), ("slices", ctypes.c_int32), ("ijkabc", ctypes.c_int32),
                ("use_j", ctypes.c_int32), ("first_iteration", ctypes.c_int64),
                ("max_iterations", ctypes.c_int64), ("start_energy", ctypes.c_double),
                ("stream", ctypes.c_void_p)]


class DeviceInputs(ctypes.Structure):
    """atrip_device_inputs: device pointers to column-major FP64 tensors."""
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("epsi", "epsa", "tai", "tabij", "vabij", "vijka", "vabci", "jijka", "jabci")]


class Tuning(ctypes.Structure):
    """atrip_tuning: launch parameters (zero = built-in choice)."""
    _fields_ = [("fp64_ctas_per_sm", ctypes.c_int32), ("fp64_tile_rows", ctypes.c_int32),
                ("tuples_per_claim", ctypes.c_int32), ("split_stages", ctypes.c_int32),
                ("split_ctas", ctypes.c_int32), ("fp64_min_blocks", ctypes.c_int32),
                ("split_w_global", ctypes.c_int32), ("tuple_block", ctypes.c_int32),
                ("split_variant", ctypes.c_int32), ("split_prefetch", ctypes.c_int32),
                ("split_wait_kcycles", ctypes.c_int32),
                ("split_test_unpublished", ctypes.c_int32), ("split_profile", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Result(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("ct_energy", ctypes.c_double),
                ("tuples_done", ctypes.c_int64), ("next_iteration", ctypes.c_int64),
                ("device_ms", ctypes.c_double), ("form_used", ctypes.c_int32),
                ("slices_used", ctypes.c_int32), ("kernel_launches", ctypes.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libatrip_gb300.so (building it first if allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and _build.needs_build():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise ImportError("libatrip_gb300.so is not built; run atrip_gb300._build.build()")
    lib = ctypes.CDLL(_build.LIB)
    P = ctypes.c_void_p
    lib.atrip_gpu_create.argtypes = [ctypes.POINTER(Dims), ctypes.POINTER(P)]
    lib.atrip_gpu_upload.argtypes = [P, ctypes.c_int32, P, ctypes.c_int64]
    lib.atrip_gpu_upload_device.argtypes = [P, ctypes.c_int32, P, ctypes.c_int64]
    lib.atrip_gpu_release.argtypes = [P, ctypes.c_int32]
    lib.atrip_gpu_run.argtypes = [P, ctypes.POINTER(RunOptions), ctypes.POINTER(Result)]
    lib.atrip_gpu_tuple_energies.argtypes = [P, ctypes.c_int64, ctypes.c_int64, P, P]
    lib.atrip_gpu_n_tuples.argtypes = [ctypes.c_int32]
    lib.atrip_gpu_n_tuples.restype = ctypes.c_int64
    lib.atrip_gpu_tuple_at.argtypes = [ctypes.c_int32, ctypes.c_int64] + [
        ctypes.POINTER(ctypes.c_int32)] * 3
    lib.atrip_gpu_destroy.argtypes = [P]
    lib.atrip_gpu_last_error.restype = ctypes.c_char_p
    lib.atrip_gpu_version.restype = ctypes.c_char_p
    lib.atrip_gpu_measure_peaks.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_double)]
    lib.atrip_gpu_run_fp64_noalloc.argtypes = [
        ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(DeviceInputs), ctypes.c_int64,
        ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]
    lib.atrip_gpu_batch_create.argtypes = [P, ctypes.c_int32, ctypes.POINTER(P)]
    lib.atrip_gpu_batch_run.argtypes = [P, ctypes.POINTER(RunOptions), P]
    lib.atrip_gpu_batch_destroy.argtypes = [P]
    lib.atrip_gpu_batch_plan.argtypes = [P, P, ctypes.c_int32, P]
    lib.atrip_gpu_set_tuning.argtypes = [P, ctypes.POINTER(Tuning)]
    lib.atrip_gpu_get_tuning.argtypes = [P, ctypes.POINTER(Tuning)]
    lib.atrip_gpu_batch_set_tuning.argtypes = [P, ctypes.POINTER(Tuning)]
    lib.atrip_gpu_last_sums.argtypes = [P, ctypes.POINTER(ctypes.c_double)]
    lib.atrip_gpu_device_count.argtypes = [ctypes.POINTER(ctypes.c_int32)]
    lib.atrip_gpu_split_profile.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int32]
    for name in EXPORTED:
        if name not in ("atrip_gpu_n_tuples", "atrip_gpu_last_error", "atrip_gpu_version"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().atrip_gpu_last_error().decode(errors="replace")
        raise AtripError(status, msg)


def n_tuples(nv: int) -> int:
    return int(load().atrip_gpu_n_tuples(nv))


def tuple_at(nv: int, t: int):
    a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    check(load().atrip_gpu_tuple_at(nv, t, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return a.value, b.value, c.value


def measure_peaks(device: int = 0):
    f64, f32 = ctypes.c_double(), ctypes.c_double()
    check(load().atrip_gpu_measure_peaks(device, ctypes.byref(f64), ctypes.byref(f32)))
    return f64.value, f32.value


class Context:
    """One GPU's engine state (wraps atrip_gpu_context)."""

    def __init__(self, No: int, Nv: int, device: int = 0, field: str = "real"):
        self.lib = load()
        self.No, self.Nv, self.device, self.field = No, Nv, device, field
        f = {"real": FIELD_REAL, "complex": FIELD_COMPLEX}[field]
        h = ctypes.c_void_p()
        check(self.lib.atrip_gpu_create(ctypes.byref(Dims(No, Nv, device, f)), ctypes.byref(h)))
        self.h = h

    def upload(self, name: str, array) -> None:
        """Upload a tensor: a numpy array (column-major data, any memory
        order of the logical array) or a CUDA torch tensor holding the
        column-major data as one contiguous buffer (complex128 for a complex
        context)."""
        tid = TENSOR_IDS[name]
        mod = type(array).__module__
        if mod.startswith("torch") and array.is_cuda:
            t = array.contiguous()
            check(self.lib.atrip_gpu_upload_device(self.h, tid, ctypes.c_void_p(t.data_ptr()),
                                                   t.numel()))
            return
        import numpy as np
        dtype = np.complex128 if self.field == "complex" else np.float64
        a = np.asarray(array, dtype=dtype)
        flat = np.ascontiguousarray(a.ravel(order="F"))
        check(self.lib.atrip_gpu_upload(self.h, tid, flat.ctypes.data, flat.size))

    def upload_ptr(self, name: str, ptr: int, n: int, on_device: bool) -> None:
        fn = self.lib.atrip_gpu_upload_device if on_device else self.lib.atrip_gpu_upload
        check(fn(self.h, TENSOR_IDS[name], ctypes.c_void_p(ptr), n))

    def release(self, name: str) -> None:
        check(self.lib.atrip_gpu_release(self.h, TENSOR_IDS[name]))

    def run(self, form: str = "fp64", slices: int = 0, ijkabc: bool = False, use_j: bool = True,
            first_iteration: int = 0, max_iterations: int = 0, start_energy: float = 0.0,
            stream: int = 0) -> Result:
        opts = RunOptions(FORMS[form], slices, int(ijkabc), int(use_j), first_iteration,
                          max_iterations, start_energy, ctypes.c_void_p(stream or None))
        res = Result()
        check(self.lib.atrip_gpu_run(self.h, ctypes.byref(opts), ctypes.byref(res)))
        return res

    def set_tuning(self, **kw) -> None:
        """Launch parameters (fields of atrip_tuning; unnamed fields are 0)."""
        t = Tuning()
        for k, v in kw.items():
            setattr(t, k, int(v))
        check(self.lib.atrip_gpu_set_tuning(self.h, ctypes.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning()
        check(self.lib.atrip_gpu_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def last_sums(self):
        """(sum, compensation) of the last run's per-tuple energies and of
        its (cT) energies: (s_e, c_e, s_ct, c_ct), no sign applied."""
        out = (ctypes.c_double * 4)()
        check(self.lib.atrip_gpu_last_sums(self.h, out))
        return tuple(out)

    def split_profile(self) -> dict:
        """Role profile of the last split run made with tuning
        split_profile=1: SM cycles per role and wait, summed over CTAs,
        and the stage / tuple / CTA counts (atrip_gpu_split_profile)."""
        out = (ctypes.c_uint64 * SPLIT_PROFILE_COUNTERS)()
        check(self.lib.atrip_gpu_split_profile(self.h, out, SPLIT_PROFILE_COUNTERS))
        return {name: int(out[k]) for k, name in enumerate(SPLIT_PROFILE) if name}

    def tuple_energies(self, t0: int, n: int):
        import numpy as np
        e = np.zeros(max(n, 1))
        ect = np.zeros(max(n, 1))
        check(self.lib.atrip_gpu_tuple_energies(self.h, t0, n, e.ctypes.data, ect.ctypes.data))
        return e[:n], ect[:n]

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.atrip_gpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def batch_plan(no, nv):
    """Launch order (cost-descending, stable) the batch gives these sizes."""
    import numpy as np
    no = np.ascontiguousarray(no, dtype=np.int32)
    nv = np.ascontiguousarray(nv, dtype=np.int32)
    order = np.zeros(max(no.size, 1), dtype=np.int32)
    check(load().atrip_gpu_batch_plan(no.ctypes.data, nv.ctypes.data, no.size, order.ctypes.data))
    return order[:no.size]


class Batch:
    """Several contexts run together (wraps atrip_gpu_batch)."""

    def __init__(self, contexts):
        self.lib = load()
        self.contexts = list(contexts)
        arr = (ctypes.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        h = ctypes.c_void_p()
        check(self.lib.atrip_gpu_batch_create(arr, len(self.contexts), ctypes.byref(h)))
        self.h = h

    def run(self, form: str = "fp64", slices: int = 0, ijkabc: bool = False, use_j: bool = True,
            first_iteration: int = 0, max_iterations: int = 0, stream: int = 0):
        opts = RunOptions(FORMS[form], slices, int(ijkabc), int(use_j), first_iteration,
                          max_iterations, 0.0, ctypes.c_void_p(stream or None))
        res = (Result * len(self.contexts))()
        check(self.lib.atrip_gpu_batch_run(self.h, ctypes.byref(opts), res))
        return list(res)

    def set_tuning(self, **kw) -> None:
        """Batch launch parameters: FP64 batch kernel (fp64_ctas_per_sm,
        fp64_min_blocks, tuples_per_claim); split_variant=1 runs the split
        form as one launch per system instead of one launch for all."""
        t = Tuning()
        for k, v in kw.items():
            setattr(t, k, int(v))
        check(self.lib.atrip_gpu_batch_set_tuning(self.h, ctypes.byref(t)))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.atrip_gpu_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
