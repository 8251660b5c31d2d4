"""CPU oracle for the CCSD(T) triples hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may use this package, and only as the checker / the timed CPU baseline.
The product (``atrip_gb300``) never imports it.

* ``triples_oracle.c`` restates atrip's per-tuple kernels in plain C
  (doubles: src/atrip/Equations.cxx:455-728, singles :387-426, energy
  :101-238, driver semantics src/atrip/Atrip.cxx:623-684, 899-963,
  1094-1111).  ``build()`` compiles it to ``liboracle.so``.
* ``Makefile`` / ``ref_harness.cxx`` / ``ref_shims/`` compile the atrip
  reference's own sources, unmodified, into ``_ref/`` (only where the
  reference tree is present).  ``tests/golden/make_golden.py`` ran that build
  to produce the committed fixtures the restatement is pinned against.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, seconds)."""
    srcs = [os.path.join(HERE, f) for f in ("triples_oracle.c", "triples_oracle_z.c")]
    stale = not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(LIB_PATH) < os.path.getmtime(s) for s in srcs)
    if force or stale:
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-o", tmp, *srcs,
                               "-lpthread", "-ldl", "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_reference(reference: str | None = None) -> bool:
    """Compile the reference's own sources with the shims into ``_ref/``.
    ``reference`` (default: the ``ATRIP_REFERENCE`` environment variable)
    is the root of an atrip source tree.  Returns False when it is not
    given or not present."""
    reference = reference or os.environ.get("ATRIP_REFERENCE", "")
    if not reference or not os.path.isdir(os.path.join(reference, "src", "atrip")):
        return False
    subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference}"])
    return True


class _Inputs(ctypes.Structure):
    _fields_ = [("No", ctypes.c_int), ("Nv", ctypes.c_int)] + [
        (n, ctypes.c_void_p) for n in
        ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci")]


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        lib.oracle_n_tuples.restype = ctypes.c_int64
        lib.oracle_n_tuples.argtypes = [ctypes.c_int]
        lib.oracle_tuple_list.argtypes = [ctypes.c_int, ctypes.c_void_p]
        lib.oracle_tuple_energies.restype = ctypes.c_int
        lib.oracle_tuple_energies.argtypes = [ctypes.POINTER(_Inputs), ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p]
        lib.oracle_tuple_arrays.restype = ctypes.c_int
        lib.oracle_tuple_arrays.argtypes = [ctypes.POINTER(_Inputs), ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]
        lib.oracle_total.restype = ctypes.c_double
        lib.oracle_total.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]
        lib.oracle_set_blas.restype = ctypes.c_int
        lib.oracle_set_blas.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        lib.oracle_energy_distinct.restype = ctypes.c_double
        lib.oracle_energy_distinct.argtypes = [ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 3
        lib.oracle_energy_same.restype = ctypes.c_double
        lib.oracle_energy_same.argtypes = [ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 3
        lib.oracle_port_prepare.restype = ctypes.c_void_p
        lib.oracle_port_prepare.argtypes = [ctypes.POINTER(_Inputs)]
        lib.oracle_port_run.restype = ctypes.c_int
        lib.oracle_port_run.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_port_free.argtypes = [ctypes.c_void_p]
        lib.oracle_z_tuple_energies.restype = ctypes.c_int
        lib.oracle_z_tuple_energies.argtypes = [ctypes.POINTER(_Inputs), ctypes.c_void_p,
                                                ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_void_p]
        lib.oracle_z_tuple_arrays.restype = ctypes.c_int
        lib.oracle_z_tuple_arrays.argtypes = [ctypes.POINTER(_Inputs), ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p]
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class Problem:
    """Keeps the column-major arrays alive and hands them to the C oracle.
    Complex inputs (any complex array) make a complex problem: every array
    is then held as complex128, i.e. interleaved (re, im) FP64."""

    def __init__(self, d: dict):
        self.No, self.Nv = int(d["No"]), int(d["Nv"])
        self.arrays = {}
        names = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci")
        self.complex = any(d.get(n) is not None and np.iscomplexobj(d[n]) for n in names)
        dtype = np.complex128 if self.complex else np.float64
        for n in names:
            a = d.get(n)
            if a is not None:
                a = np.asfortranarray(a, dtype=dtype)
            self.arrays[n] = a
        self.c = _Inputs(self.No, self.Nv, *[_ptr(self.arrays[n]) for n in
                                             ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka",
                                              "Vabci", "Jijka", "Jabci")])

    @property
    def has_j(self) -> bool:
        return self.arrays["Jijka"] is not None and self.arrays["Jabci"] is not None


def n_tuples(Nv: int) -> int:
    return int(_load().oracle_n_tuples(Nv))


def tuple_list(Nv: int) -> np.ndarray:
    n = n_tuples(Nv)
    out = np.zeros((max(n, 1), 3), dtype=np.int32)
    _load().oracle_tuple_list(Nv, out.ctypes.data)
    return out[:n]


def tuple_energies(p: Problem, t0: int = 0, t1: int | None = None, ijkabc: bool = False,
                   use_j: bool = True, route: str = "naive", threads: int = 1):
    """Per-tuple (e, e_ct) for lexicographic tuples t0..t1-1 (a complex
    problem always takes the complex restatement)."""
    n = n_tuples(p.Nv)
    t1 = n if t1 is None else t1
    e = np.zeros(max(t1 - t0, 1))
    ect = np.zeros(max(t1 - t0, 1))
    if p.complex:
        lst = np.ascontiguousarray(tuple_list(p.Nv))
        _load().oracle_z_tuple_energies(ctypes.byref(p.c), lst.ctypes.data, t0, t1, int(ijkabc),
                                        int(use_j), max(1, threads), e.ctypes.data,
                                        ect.ctypes.data)
        return e[:t1 - t0], ect[:t1 - t0]
    rc = _load().oracle_tuple_energies(ctypes.byref(p.c), t0, t1, int(ijkabc), int(use_j),
                                       {"naive": 0, "port": 1}[route], threads,
                                       e.ctypes.data, ect.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_tuple_energies rejected its arguments")
    return e[:t1 - t0], ect[:t1 - t0]


def total(e: np.ndarray, ijkabc: bool = False) -> float:
    e = np.ascontiguousarray(e, dtype=np.float64)
    return float(_load().oracle_total(e.ctypes.data, len(e), int(ijkabc)))


def run(p: Problem, ijkabc: bool = False, use_j: bool = True, threads: int = 1,
        route: str = "naive", max_iterations: int = 0, first_iteration: int = 0,
        start_energy: float = 0.0):
    """(energy, ct_energy) with the driver semantics of Atrip::run:
    tuples first_iteration .. max_iterations (inclusive) when max_iterations
    != 0 (src/atrip/Atrip.cxx:1052-1056), a checkpointed physical energy
    added back (src/atrip/Atrip.cxx:612-616), final sign unless ijkabc."""
    n = n_tuples(p.Nv)
    t1 = n if max_iterations == 0 else min(n, max_iterations + 1)
    t0 = min(first_iteration, t1)
    e, ect = tuple_energies(p, t0, t1, ijkabc, use_j, route, threads)
    sign = 1.0 if ijkabc else -1.0
    local = -start_energy  # src/atrip/Atrip.cxx:612-616 negates unconditionally
    return sign * (local + float(np.sum(e))), sign * (float(np.sum(ect)))


class PreparedPort:
    """The DGEMM-route port with its operand slices cut once, so that tuple
    ranges can be timed without the set-up (bench.py's CPU baseline)."""

    def __init__(self, p: Problem):
        self.p = p
        self.h = _load().oracle_port_prepare(ctypes.byref(p.c))

    def run(self, t0: int, t1: int, threads: int, ijkabc: bool = False, use_j: bool = True):
        n = t1 - t0
        e = np.zeros(max(n, 1))
        ect = np.zeros(max(n, 1))
        rc = _load().oracle_port_run(self.h, t0, t1, int(ijkabc), int(use_j), threads,
                                     e.ctypes.data, ect.ctypes.data)
        if rc != 0:
            raise ValueError("oracle_port_run rejected its arguments")
        return e[:n], ect[:n]

    def close(self):
        if self.h:
            _load().oracle_port_free(self.h)
            self.h = None


def tuple_arrays(p: Problem, a: int, b: int, c: int, ijkabc: bool = False):
    No = p.No
    if p.complex:
        T = np.zeros(No ** 3, dtype=np.complex128)
        Z = np.zeros(No ** 3, dtype=np.complex128)
        _load().oracle_z_tuple_arrays(ctypes.byref(p.c), a, b, c, int(ijkabc), T.ctypes.data,
                                      Z.ctypes.data)
        return T, Z
    T = np.zeros(No ** 3)
    Z = np.zeros(No ** 3)
    _load().oracle_tuple_arrays(ctypes.byref(p.c), a, b, c, int(ijkabc), T.ctypes.data, Z.ctypes.data)
    return T, Z


def register_numpy_openblas() -> str | None:
    """Point the port's dgemm at numpy's bundled ILP64 OpenBLAS (single
    threaded per worker), if numpy ships one.  Returns its path or None."""
    import glob
    base = os.path.dirname(np.__file__)
    cands = sorted(glob.glob(os.path.join(base, "..", "numpy.libs", "libscipy_openblas64_*.so*")))
    cands += sorted(glob.glob(os.path.join(base, ".libs", "libscipy_openblas64_*.so*")))
    for c in cands:
        if _load().oracle_set_blas(c.encode(), b"scipy_dgemm_64_",
                                   b"scipy_openblas_set_num_threads64_"):
            return c
    return None


def reference_binary(variant: str = "dgemm") -> str | None:
    p = os.path.join(REF_DIR, f"atrip_ref_{variant}")
    return p if os.path.exists(p) else None


def run_reference(bin_dir: str, variant: str = "dgemm", max_iterations: int = 0,
                  ijkabc: bool = False, use_j: bool = True):
    """Atrip::run of the one-rank reference build (GROUP_AND_SORT, see
    DESIGN notes on NAIVE).  Returns (energy, ct_energy, seconds)."""
    exe = reference_binary(variant)
    if exe is None:
        raise FileNotFoundError("reference build missing; run oracle.build_reference()")
    out = subprocess.run([exe, bin_dir, "run", str(max_iterations), str(int(ijkabc)),
                          str(int(use_j)), "1"], check=True, capture_output=True, text=True).stdout
    for line in out.splitlines():
        if line.startswith("RESULT"):
            _, e, ect, secs = line.split()
            return float(e), float(ect), float(secs)
    raise RuntimeError("reference printed no RESULT line:\n" + out)


def reference_tuples(bin_dir: str, n: int, ijkabc: bool = False, use_j: bool = True,
                     variant: str = "dgemm"):
    exe = reference_binary(variant)
    out = subprocess.run([exe, bin_dir, "tuples", str(n), str(int(ijkabc)), str(int(use_j))],
                         check=True, capture_output=True, text=True).stdout
    rows = [line.split() for line in out.splitlines() if line.startswith("TUPLE")]
    abc = np.array([[int(r[2]), int(r[3]), int(r[4])] for r in rows], dtype=np.int32)
    e = np.array([float(r[5]) for r in rows])
    ect = np.array([float(r[6]) for r in rows])
    return abc, e, ect


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))
