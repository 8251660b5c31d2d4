"""The no-allocation entry point (atrip_gpu_run_fp64_noalloc) against the
regular one (atrip_gpu_run), through the C ABI.

atrip_gpu_run_fp64_noalloc serves hosts that cannot allocate device memory
themselves -- their pool allocator owns all of HBM, or cudaMalloc is off
limits on their threads because it synchronises the device.  They pass
device pointers to their column-major inputs and outputs, and the library
uses a fixed scratch array of its own.  This test runs it twice in a row
(the second call reuses the scratch the first one left behind) and checks
both against the regular entry point at the FP64 tolerance of the other
GPU tests (1e-10 relative).  It lives in its own file, named to be collected
last, and passes both alone and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

from atrip_gb300 import capi, synth

pytestmark = pytest.mark.gpu
REL = 1e-10
NAMES = ("epsi", "epsa", "Tai", "Tabij", "Vabij", "Vijka", "Vabci", "Jijka", "Jabci")


def _device_columns(d):
    import torch
    out = {}
    for n in NAMES:
        flat = np.ascontiguousarray(np.asarray(d[n], dtype=np.float64).ravel(order="F"))
        out[n] = torch.from_numpy(flat).to("cuda:0")
    return out


def _noalloc(lib, No, Nv, dev, first, maxit, use_j, ijkabc=0, drop_j=False):
    import torch
    n_all = capi.n_tuples(Nv)
    end = n_all if maxit == 0 else min(n_all, maxit + 1)
    n = end - min(first, end)
    e = torch.full((max(n, 1),), float("nan"), dtype=torch.float64, device="cuda:0")
    ect = torch.full((max(n, 1),), float("nan"), dtype=torch.float64, device="cuda:0")
    energies = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")
    ptrs = capi.DeviceInputs(*[None if drop_j and k in ("Jijka", "Jabci") else dev[k].data_ptr()
                               for k in NAMES])
    torch.cuda.synchronize()
    capi.check(lib.atrip_gpu_run_fp64_noalloc(No, Nv, ctypes.byref(ptrs), first, maxit, ijkabc,
                                              int(use_j), e.data_ptr(), ect.data_ptr(),
                                              energies.data_ptr(), None))
    torch.cuda.synchronize()
    return e[:n].cpu().numpy(), ect[:n].cpu().numpy(), energies.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    No, Nv = 10, 14
    d = synth.make_inputs(No, Nv, 21, with_j=True)
    dev = _device_columns(d)
    lib = capi.load()
    with capi.Context(No, Nv, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        for first, maxit in ((0, 0), (100, 300)):
            ref = ctx.run(form="fp64", first_iteration=first, max_iterations=maxit)
            ref_e, ref_ect = ctx.tuple_energies(first, ref.tuples_done)
            e, ect, energies = _noalloc(lib, No, Nv, dev, first, maxit, True)
            assert len(e) == ref.tuples_done
            scale = np.max(np.abs(ref_e))
            assert np.max(np.abs(e - ref_e)) <= REL * scale
            assert np.max(np.abs(ect - ref_ect)) <= REL * scale
            assert abs(energies[0] - ref.energy) <= REL * abs(ref.energy)
            assert abs(energies[1] - ref.ct_energy) <= REL * abs(ref.energy)


def _compare(ctx, lib, No, Nv, dev, first, maxit, ijkabc=False, drop_j=False):
    ref = ctx.run(form="fp64", first_iteration=first, max_iterations=maxit, ijkabc=ijkabc,
                  use_j=not drop_j)
    ref_e, ref_ect = ctx.tuple_energies(first, ref.tuples_done)
    e, ect, energies = _noalloc(lib, No, Nv, dev, first, maxit, True, int(ijkabc), drop_j)
    assert len(e) == ref.tuples_done
    scale = np.max(np.abs(ref_e))
    assert np.max(np.abs(e - ref_e)) <= REL * scale
    assert np.max(np.abs(ect - ref_ect)) <= REL * scale
    assert abs(energies[0] - ref.energy) <= REL * abs(ref.energy)
    assert abs(energies[1] - ref.ct_energy) <= REL * abs(ref.energy)
    return energies


def test_noalloc_ijkabc_and_without_j():
    """ijkabc (negated T1, no final negation) and NULL J pointers (then
    ct_energy == energy), each against the regular entry point."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    No, Nv = 9, 13
    d = synth.make_inputs(No, Nv, 22, with_j=True)
    dev = _device_columns(d)
    lib = capi.load()
    with capi.Context(No, Nv, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        _compare(ctx, lib, No, Nv, dev, 0, 0, ijkabc=True)
        energies = _compare(ctx, lib, No, Nv, dev, 3, 200, drop_j=True)
        assert energies[1] == energies[0]


def test_noalloc_large_no_grid_capped_by_scratch():
    """At No=56 the 32 MiB array holds W for only 11 CTAs (2 No^3 doubles
    each): fewer CTAs than the occupancy grid, every tuple still run."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    No, Nv = 56, 8
    d = synth.make_inputs(No, Nv, 23, with_j=True)
    dev = _device_columns(d)
    lib = capi.load()
    with capi.Context(No, Nv, 0) as ctx:
        for n in NAMES:
            ctx.upload(n, d[n])
        _compare(ctx, lib, No, Nv, dev, 0, 60)


def test_noalloc_rejects_out_of_range_sizes():
    pytest.importorskip("torch")
    lib = capi.load()
    ptrs = capi.DeviceInputs(*([None] * 9))
    rc = lib.atrip_gpu_run_fp64_noalloc(65, 10, ctypes.byref(ptrs), 0, 0, 0, 0, 1, 1, 1, None)
    assert rc == capi.ERR_UNSUPPORTED
    assert b"No must be" in lib.atrip_gpu_last_error()
