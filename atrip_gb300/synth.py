"""Seeded synthetic CCSD(T) inputs with the value distributions of the
benchmark workloads (all FP64, column-major / first index fastest, which is
the element order atrip's CTF tensors hand to ``read_all``;
src/atrip/Atrip.cxx:176-187, src/atrip/Unions.hpp:97-277).

Distributions (sigma is a standard deviation):

* t1 ``Tai[a,i]``            ~ N(0, 0.01)
* t2 ``Tabij[a,b,i,j]``      = (X + X^P)/2 with X ~ N(0, 0.05) and
  X^P[a,b,i,j] = X[b,a,j,i], so ``T[a,b,i,j] == T[b,a,j,i]`` exactly
* ``Vabij``                  same pair symmetrisation, X ~ N(0, 0.1)
* ``Vijka`` (No,No,No,Nv), ``Vabci`` (Nv,Nv,Nv,No) ~ N(0, 0.1)
* optional (cT) intermediates ``Jijka``, ``Jabci`` ~ N(0, 0.1)
* eps_occ ~ U[-2, -0.3], eps_virt ~ U[0.1, 3]

The stream is counter based (splitmix64 of seed, tensor id and element
index) so any element can be regenerated independently and in chunks; the
Gaussian is Box-Muller over the two 32-bit halves of one 64-bit draw.  Results only depend on IEEE
arithmetic and the platform's ``log``/``cos``/``sqrt`` (ulp-level
differences across libms are far below every tolerance used here).
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_TENSOR_IDS = {
    "epsi": 1, "epsa": 2, "Tai": 3, "Tabij": 4, "Vabij": 5,
    "Vijka": 6, "Vabci": 7, "Jijka": 8, "Jabci": 9, "sizes": 10,
}
_CHUNK = 1 << 21
_IMAG_SEED_OFFSET = 1 << 40  # imaginary parts of complex inputs: seed + this


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def _key(seed: int, tensor: str) -> np.uint64:
    with np.errstate(over="ignore"):
        k = np.array([(seed * 0x9E3779B97F4A7C15 + _TENSOR_IDS[tensor] * 0xD1B54A32D192ED69)
                      & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64)
        return _mix(k)[0]


def _uniform(key: np.uint64, start: int, n: int) -> np.ndarray:
    """Uniform doubles in [0, 1) (53-bit) for counters start .. start+n-1."""
    with np.errstate(over="ignore"):
        ctr = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = _mix(key + ctr * _GOLDEN)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _normal_chunk(key: np.uint64, start: int, n: int) -> np.ndarray:
    """Box-Muller from one 64-bit draw per element: the high and low 32 bits
    give the two uniforms (u1 in (0, 1], u2 in [0, 1))."""
    with np.errstate(over="ignore"):
        ctr = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = _mix(key + ctr * _GOLDEN)
    u1 = ((z >> np.uint64(32)).astype(np.float64) + 1.0) * (1.0 / 4294967296.0)
    u2 = (z & np.uint64(0xFFFFFFFF)).astype(np.float64) * (1.0 / 4294967296.0)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos((2.0 * np.pi) * u2)


def _normal_flat(key: np.uint64, n: int, sigma: float) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    starts = list(range(0, n, _CHUNK))

    def work(s):
        m = min(_CHUNK, n - s)
        out[s:s + m] = _normal_chunk(key, s, m) * sigma

    if len(starts) > 1:
        # numpy releases the GIL inside these ufuncs, so chunks run in parallel
        from concurrent.futures import ThreadPoolExecutor
        import os
        with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            list(ex.map(work, starts))
    else:
        for s in starts:
            work(s)
    return out


def _uniform_flat(key: np.uint64, n: int, lo: float, hi: float) -> np.ndarray:
    return lo + (hi - lo) * _uniform(key, 0, n)


def _colmajor(flat: np.ndarray, shape) -> np.ndarray:
    return flat.reshape(shape, order="F")


def _pair_symmetrise(x: np.ndarray) -> np.ndarray:
    # X^P[a,b,i,j] = X[b,a,j,i]
    return 0.5 * (x + x.transpose(1, 0, 3, 2))


def make_inputs(No: int, Nv: int, seed: int = 0, with_j: bool = False,
                scale: float = 1.0, field: str = "real", eps_imag: float = 0.0) -> dict:
    """All atrip inputs as Fortran-ordered FP64 arrays.

    ``scale`` multiplies t1, t2 and every integral tensor; a power of two
    keeps the relative structure bit-for-bit and scales E(T) by scale**4
    (used for the small-magnitude twin of a workload).

    ``field="complex"`` gives complex128 arrays (atrip's run<Complex>): the
    real parts are the real workload's arrays, the imaginary parts come from
    their own streams with the same distributions (and the same pair
    symmetry for t2 and V_pphh); orbital energies get an imaginary part
    ~ N(0, eps_imag) (0: real orbital energies, as in CCSD(T)).
    """
    if field == "complex":
        re = make_inputs(No, Nv, seed, with_j, scale)
        im = make_inputs(No, Nv, seed + _IMAG_SEED_OFFSET, with_j, scale)
        d = {"No": No, "Nv": Nv, "seed": seed}
        for n in ("Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci"):
            if n in re:
                d[n] = np.asfortranarray(re[n] + 1j * im[n])
        for n, m in (("epsi", No), ("epsa", Nv)):
            d[n] = re[n] + 1j * (eps_imag * _normal_flat(_key(seed + 2 * _IMAG_SEED_OFFSET, n), m, 1.0) if eps_imag
                                 else np.zeros(m))
        return d
    key = lambda name: _key(seed, name)  # noqa: E731
    d = {
        "No": No, "Nv": Nv, "seed": seed,
        "epsi": _uniform_flat(key("epsi"), No, -2.0, -0.3),
        "epsa": _uniform_flat(key("epsa"), Nv, 0.1, 3.0),
        "Tai": _colmajor(_normal_flat(key("Tai"), Nv * No, 0.01), (Nv, No)),
    }
    x = _colmajor(_normal_flat(key("Tabij"), Nv * Nv * No * No, 0.05), (Nv, Nv, No, No))
    d["Tabij"] = np.asfortranarray(_pair_symmetrise(x))
    x = _colmajor(_normal_flat(key("Vabij"), Nv * Nv * No * No, 0.1), (Nv, Nv, No, No))
    d["Vabij"] = np.asfortranarray(_pair_symmetrise(x))
    del x
    d["Vijka"] = _colmajor(_normal_flat(key("Vijka"), No * No * No * Nv, 0.1), (No, No, No, Nv))
    d["Vabci"] = _colmajor(_normal_flat(key("Vabci"), Nv * Nv * Nv * No, 0.1), (Nv, Nv, Nv, No))
    if with_j:
        d["Jijka"] = _colmajor(_normal_flat(key("Jijka"), No * No * No * Nv, 0.1), (No, No, No, Nv))
        d["Jabci"] = _colmajor(_normal_flat(key("Jabci"), Nv * Nv * Nv * No, 0.1), (Nv, Nv, Nv, No))
    if scale != 1.0:
        for name in ("Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci"):
            if name in d:
                d[name] = d[name] * scale
    return d


def write_bin_dir(d: dict, path: str) -> None:
    """Write the layout the one-rank reference harness reads (meta.txt + .bin)."""
    import os
    os.makedirs(path, exist_ok=True)
    has_j = int("Jijka" in d)
    cplx = int(np.iscomplexobj(d["Tabij"]))
    with open(os.path.join(path, "meta.txt"), "w") as f:
        f.write(f"{d['No']} {d['Nv']} {has_j} {cplx}\n")
    dtype = np.complex128 if cplx else np.float64
    for name in ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci"):
        if name in d:
            np.asarray(d[name], dtype=dtype).ravel(order="F").tofile(
                os.path.join(path, name + ".bin"))


def multi_system_sizes(n: int = 96, no_range=(4, 20), nv_range=(30, 200)):
    """(No, Nv, seed) of the multi-system workload: system s has seed s and
    No, Nv drawn uniformly (inclusive ranges) from its own counter stream."""
    out = []
    for s in range(n):
        u = _uniform(_key(s, "sizes"), 0, 2)
        No = no_range[0] + min(int(u[0] * (no_range[1] - no_range[0] + 1)),
                               no_range[1] - no_range[0])
        Nv = nv_range[0] + min(int(u[1] * (nv_range[1] - nv_range[0] + 1)),
                               nv_range[1] - nv_range[0])
        out.append((No, Nv, s))
    return out


def n_tuples(Nv: int) -> int:
    """a <= b <= c without a == b == c (src/atrip/Tuples.cxx:89-93)."""
    return Nv * (Nv + 1) * (Nv + 2) // 6 - Nv


def flops_per_tuple(No: int, Nv: int) -> float:
    """The reference's own count, 12 No^3 (No + Nv) (src/atrip/Atrip.cxx:578-580)."""
    return 12.0 * No ** 3 * (No + Nv)
