"""Python mirror of atrip's public interface (src/atrip/Atrip.hpp:41-140).

Under torch.distributed (one process per GPU, ``Atrip.init(group)``) the
tuple list is split into contiguous shares and the energies merged at the
end (``atrip_gb300.shard``).

``Atrip.init``, the ``Input`` builder with every ``with_*`` attribute and
its default, ``Output(energy, ct_energy)`` and ``Atrip.run`` behave as in the
reference, but the tuple loop runs on one GB300 through the C ABI
(include/atrip_gb300.h).  Tensors are numpy arrays (logical shape, any memory
order; their column-major flattening is the data, as CTF's read_all gives
it), CUDA torch tensors holding column-major data, or any object with
``lens`` and ``read_all()`` like a CTF tensor.

Checkpoints keep atrip's flat YAML format and resume semantics
(src/atrip/Checkpoint.hpp:27-79, src/atrip/Atrip.cxx:584-621, 713-731).
"""
from __future__ import annotations

import enum
import os
import time
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import capi, shard


@dataclass
class Output:
    """src/atrip/Atrip.hpp:134-137."""
    energy: float = 0.0
    ct_energy: float = 0.0


@dataclass
class IterationDescription:
    """src/atrip/Debug.hpp:96-109."""
    current_iteration: int
    total_iterations: int
    current_elapsed_time: float


_descriptor: Optional[Callable[[IterationDescription], None]] = None


def register_iteration_descriptor(fn: Callable[[IterationDescription], None]) -> None:
    """src/atrip/Debug.hpp:107, src/atrip/Atrip.cxx:49-52."""
    global _descriptor
    _descriptor = fn


# ------------------------------------------------------------ checkpoints

@dataclass
class Checkpoint:
    """src/atrip/Checkpoint.hpp:27-37."""
    no: int = 0
    nv: int = 0
    nranks: int = 1
    nnodes: int = 1
    energy: float = 0.0
    iteration: int = 0
    rank_round_robin: bool = False


def _atoi(s: str) -> int:
    s = s.strip()
    n = 0
    sign = 1
    i = 0
    if i < len(s) and s[i] in "+-":
        sign = -1 if s[i] == "-" else 1
        i += 1
    while i < len(s) and s[i].isdigit():
        n = n * 10 + int(s[i])
        i += 1
    return sign * n


def _atof(s: str) -> float:
    import re
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|nan)", s, re.I)
    return float(m.group(0)) if m else 0.0


def write_checkpoint(c: Checkpoint, path: str) -> None:
    """src/atrip/Checkpoint.hpp:40-49 (energy with 19 significant digits)."""
    with open(path, "w") as f:
        f.write(f"No: {c.no}\nNv: {c.nv}\nNranks: {c.nranks}\nNnodes: {c.nnodes}\n"
                f"Energy: {format(c.energy, '.19g')}\nIteration: {c.iteration}\n"
                f"RankRoundRobin: {'true' if c.rank_round_robin else 'false'}\n")


def read_checkpoint(path: str) -> Checkpoint:
    """src/atrip/Checkpoint.hpp:51-75: 'header: value' lines, unknown keys
    ignored, values parsed like atoi / atof."""
    c = Checkpoint()
    with open(path) as f:
        text = f.read()
    pos = 0
    while True:
        colon = text.find(":", pos)
        if colon < 0:
            break
        header = text[pos:colon].strip(" \t")
        nl = text.find("\n", colon + 1)
        value = text[colon + 1:] if nl < 0 else text[colon + 1:nl]
        value = value.strip(" \t")
        pos = len(text) if nl < 0 else nl + 1
        if header == "No":
            c.no = _atoi(value)
        elif header == "Nv":
            c.nv = _atoi(value)
        elif header == "Nranks":
            c.nranks = _atoi(value)
        elif header == "Nnodes":
            c.nnodes = _atoi(value)
        elif header == "Energy":
            c.energy = _atof(value)
        elif header == "Iteration":
            c.iteration = _atoi(value)
        elif header == "RankRoundRobin":
            c.rank_round_robin = value[:1] == "t"
    return c


# ------------------------------------------------------------------ input

class TuplesDistribution(enum.IntEnum):
    """src/atrip/Atrip.hpp:108-111.  On one GPU both map to the same
    on-device work queue over the lexicographic tuple list."""
    NAIVE = 0
    GROUP_AND_SORT = 1


_ATTRIBUTES = {  # src/atrip/Atrip.hpp:113-131, with the reference defaults
    "delete_Vppph": False,
    "rank_round_robin": False,
    "chrono": False,
    "barrier": False,
    "blocking": False,
    "max_iterations": 0,
    "iteration_mod": -1,
    "percentage_mod": -1,
    "tuples_distribution": TuplesDistribution.NAIVE,
    "checkpoint_path": "atrip-checkpoint.yaml",
    "read_checkpoint_if_exists": True,
    "writeCheckpoint": True,
    "checkpoint_at_percentage": 10.0,
    "checkpoint_at_every_iteration": 0,
    "ijkabc": False,
    "ooo_threads": 0,
    "ooo_blocks": 0,
    # GPU attributes (no counterpart in the reference)
    "form": "fp64",          # "fp64" | "split_bf16" | "split_f16" | "auto"
    "slices": 0,             # split forms: slices per operand (0 = 3 BF16 / 2 FP16)
    "device": 0,
    "checkpoint_chunks": 100,  # tuple chunks per run when checkpoints are written
}

_TENSORS = {  # builder name -> (attribute, C-ABI tensor name)
    "epsilon_i": ("ei", "epsi"), "epsilon_a": ("ea", "epsa"), "Tai": ("Tph", "Tai"),
    "Tabij": ("Tpphh", "Tabij"), "Vabij": ("Vpphh", "Vabij"), "Vijka": ("Vhhhp", "Vijka"),
    "Vabci": ("Vppph", "Vabci"), "Jijka": ("Jhhhp", "Jijka"), "Jabci": ("Jppph", "Jabci"),
}


class Input:
    """src/atrip/Atrip.hpp:67-132: tensor slots plus ADD_ATTRIBUTE options,
    each settable through a chaining ``with_<name>``."""

    TuplesDistribution = TuplesDistribution

    def __init__(self):
        for attr, _ in _TENSORS.values():
            setattr(self, attr, None)
        for k, v in _ATTRIBUTES.items():
            setattr(self, k, v)

    def __getattr__(self, name):
        if name.startswith("with_"):
            key = name[5:]
            if key in _TENSORS:
                attr = _TENSORS[key][0]
            elif key in _ATTRIBUTES:
                attr = key
            else:
                raise AttributeError(name)

            def setter(value):
                setattr(self, attr, value)
                return self
            return setter
        raise AttributeError(name)


def _lens(t):
    if hasattr(t, "lens"):
        return [int(x) for x in t.lens]
    return list(t.shape)


def _payload(t, complex_field: bool = False):
    """numpy/torch arrays pass through; CTF-like objects are read_all'ed."""
    if hasattr(t, "read_all") and not hasattr(t, "shape"):
        n = int(np.prod(_lens(t)))
        buf = np.empty(n, dtype=np.complex128 if complex_field else np.float64)
        t.read_all(buf)
        return buf
    return t


def _is_complex(t) -> bool:
    """Field of an input: complex dtype (numpy/torch) or a CTF-like object
    that says so through ``is_complex`` / ``dtype``."""
    if getattr(t, "is_complex", None) is True:
        return True
    dt = getattr(t, "dtype", None)
    if dt is None:
        return False
    try:
        return bool(np.issubdtype(np.dtype(dt), np.complexfloating))
    except TypeError:
        return "complex" in str(dt)


class Atrip:
    """src/atrip/Atrip.hpp:41-63.  One process drives one GPU; several
    processes (torch.distributed ranks, one GPU each) split the tuple list
    into contiguous shares and merge their compensated sums at the end."""

    rank = 0
    np = 1
    group = None
    chrono: dict = {}
    Input = Input
    Output = Output

    @staticmethod
    def init(comm=None) -> None:
        """src/atrip/Atrip.cxx:54-63.  ``comm``: None (one process), or a
        torch.distributed process group; with None and an initialised
        default group, that group is used."""
        Atrip.rank, Atrip.np, Atrip.group = 0, 1, None
        try:
            import torch.distributed as dist
            if dist.is_available() and dist.is_initialized():
                Atrip.group = comm
                Atrip.rank = dist.get_rank(comm)
                Atrip.np = dist.get_world_size(comm)
        except ImportError:  # pragma: no cover
            pass
        Atrip.chrono = {}

    @staticmethod
    def run(inp: Input) -> Output:
        """src/atrip/Atrip.cxx:66-1133 on one GPU per process."""
        if inp.ei is None or inp.ea is None:
            raise ValueError("epsilon_i and epsilon_a are required")
        No, Nv = _lens(inp.ei)[0], _lens(inp.ea)[0]
        t_start = time.perf_counter()
        # run<Complex> (src/atrip/Atrip.cxx:1136) when the inputs are complex
        cplx = any(_is_complex(getattr(inp, attr)) for attr, _ in _TENSORS.values()
                   if getattr(inp, attr) is not None)
        device = inp.device
        if Atrip.np > 1 and "LOCAL_RANK" in os.environ:
            device = int(os.environ["LOCAL_RANK"])
        with capi.Context(No, Nv, device, field="complex" if cplx else "real") as ctx:
            for key, (attr, cname) in _TENSORS.items():
                t = getattr(inp, attr)
                if t is None:
                    continue
                ctx.upload(cname, _payload(t, cplx))
            if inp.delete_Vppph:
                inp.Vppph = None  # the caller's V_pphp is dropped as in src/atrip/Atrip.cxx:310
            n = capi.n_tuples(Nv)
            first, start_energy = 0, 0.0
            if inp.read_checkpoint_if_exists and os.path.exists(inp.checkpoint_path):
                c = read_checkpoint(inp.checkpoint_path)
                first, start_energy = int(c.iteration), float(c.energy)
            end = n if inp.max_iterations == 0 else min(n, inp.max_iterations + 1)
            opts = dict(form=inp.form, slices=inp.slices, ijkabc=inp.ijkabc, use_j=True)
            if Atrip.np > 1:
                energy, ct = Atrip._run_shard(ctx, first, end, start_energy, opts, inp.ijkabc)
                Atrip.chrono["run"] = time.perf_counter() - t_start
                return Output(energy, ct)
            # write condition of src/atrip/Atrip.cxx:588-591, 713:
            # only a zero modulus writes (at every iteration in the reference;
            # here at chunk boundaries of the device queue)
            mod = (inp.checkpoint_at_every_iteration if inp.checkpoint_at_every_iteration != 0
                   else int(n * inp.checkpoint_at_percentage / 100))
            write = mod == 0
            if not write:
                r = ctx.run(first_iteration=first, max_iterations=inp.max_iterations,
                            start_energy=start_energy, **opts)
                energy, ct = r.energy, r.ct_energy
                Atrip.chrono["iterations"] = r.device_ms / 1e3
            else:
                chunk = max(1, -(-(end - first) // max(1, int(inp.checkpoint_chunks))))
                energy_phys, ct_acc = start_energy, 0.0
                sign = 1.0 if inp.ijkabc else -1.0
                pos = first
                while pos < end:
                    write_checkpoint(Checkpoint(No, Nv, 1, 1, energy_phys, pos,
                                                inp.rank_round_robin), inp.checkpoint_path)
                    stop = min(end, pos + chunk)
                    r = ctx.run(first_iteration=pos, max_iterations=stop - 1,
                                start_energy=energy_phys, **opts)
                    energy_phys = r.energy if not inp.ijkabc else -r.energy
                    ct_acc += sign * r.ct_energy
                    pos = stop
                    if _descriptor:
                        _descriptor(IterationDescription(pos, n, time.perf_counter() - t_start))
                energy = energy_phys if not inp.ijkabc else -energy_phys
                ct = sign * ct_acc
        Atrip.chrono["run"] = time.perf_counter() - t_start
        return Output(energy, ct)

    @staticmethod
    def _run_shard(ctx, first, end, start_energy, opts, ijkabc):
        """This rank's contiguous share of tuples first .. end-1, then the
        merge of every rank's compensated sums (the role of atrip's
        MPI_Reduce, src/atrip/Atrip.cxx:1094-1107).  Checkpoints are read
        (resume point and energy) but not written across processes."""
        t0, t1 = shard.tuple_range(first, end, Atrip.rank, Atrip.np)
        local = (0.0, 0.0, 0.0, 0.0)
        if t1 > t0:
            if t1 - 1 == 0 and end > 1:
                # max_iterations = 0 would mean "every tuple": run two and
                # keep the first one's energies
                ctx.run(first_iteration=0, max_iterations=1, **opts)
                e, ect = ctx.tuple_energies(0, 1)
                local = (float(e[0]), 0.0, float(ect[0]), 0.0)
            else:
                r = ctx.run(first_iteration=t0, max_iterations=t1 - 1, **opts)
                Atrip.chrono["iterations"] = r.device_ms / 1e3
                local = ctx.last_sums()
        return shard.reduce_energies(local, ijkabc, start_energy, Atrip.group)


def run(inp: Input) -> Output:
        """src/atrip/Atrip.cxx:66-1133 on one GPU."""
        if inp.ei is None or inp.ea is None:
            raise ValueError("epsilon_i and epsilon_a are required")
        No, Nv = _lens(inp.ei)[0], _lens(inp.ea)[0]
        t_start = time.perf_counter()
        # run<Complex> (src/atrip/Atrip.cxx:1136) when the inputs are complex
        cplx = any(_is_complex(getattr(inp, attr)) for attr, _ in _TENSORS.values()
                   if getattr(inp, attr) is not None)
        with capi.Context(No, Nv, inp.device, field="complex" if cplx else "real") as ctx:
            for key, (attr, cname) in _TENSORS.items():
                t = getattr(inp, attr)
                if t is None:
                    continue
                ctx.upload(cname, _payload(t, cplx))
            if inp.delete_Vppph:
                inp.Vppph = None  # the caller's V_pphp is dropped as in src/atrip/Atrip.cxx:310
            n = capi.n_tuples(Nv)
            first, start_energy = 0, 0.0
            if inp.read_checkpoint_if_exists and os.path.exists(inp.checkpoint_path):
                c = read_checkpoint(inp.checkpoint_path)
                first, start_energy = int(c.iteration), float(c.energy)
            # write condition of src/atrip/Atrip.cxx:588-591, 713:
            # only a zero modulus writes (at every iteration in the reference;
            # here at chunk boundaries of the device queue)
            mod = (inp.checkpoint_at_every_iteration if inp.checkpoint_at_every_iteration != 0
                   else int(n * inp.checkpoint_at_percentage / 100))
            write = mod == 0
            end = n if inp.max_iterations == 0 else min(n, inp.max_iterations + 1)
            opts = dict(form=inp.form, slices=inp.slices, ijkabc=inp.ijkabc, use_j=True)
            if not write:
                r = ctx.run(first_iteration=first, max_iterations=inp.max_iterations,
                            start_energy=start_energy, **opts)
                energy, ct = r.energy, r.ct_energy
                Atrip.chrono["iterations"] = r.device_ms / 1e3
            else:
                chunk = max(1, -(-(end - first) // max(1, int(inp.checkpoint_chunks))))
                energy_phys, ct_acc = start_energy, 0.0
                sign = 1.0 if inp.ijkabc else -1.0
                pos = first
                while pos < end:
                    write_checkpoint(Checkpoint(No, Nv, 1, 1, energy_phys, pos,
                                                inp.rank_round_robin), inp.checkpoint_path)
                    stop = min(end, pos + chunk)
                    r = ctx.run(first_iteration=pos, max_iterations=stop - 1,
                                start_energy=energy_phys, **opts)
                    energy_phys = r.energy if not inp.ijkabc else -r.energy
                    ct_acc += sign * r.ct_energy
                    pos = stop
                    if _descriptor:
                        _descriptor(IterationDescription(pos, n, time.perf_counter() - t_start))
                energy = energy_phys if not inp.ijkabc else -energy_phys
                ct = sign * ct_acc
        Atrip.chrono["run"] = time.perf_counter() - t_start
        return Output(energy, ct)


def run(inp: Input) -> Output:
    return Atrip.run(inp)
