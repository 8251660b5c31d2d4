"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares (no compute calls are made)."""
import ctypes
import glob
import os
import re

from atrip_gb300 import _build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(atrip_gpu_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    _build.build()
    lib = ctypes.CDLL(_build.LIB)
    names = declared_symbols()
    assert len(names) >= 12
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(capi.EXPORTED) <= names


def test_pure_host_entry_points():
    lib = capi.load()
    assert lib.atrip_gpu_version().startswith(b"atrip_gb300")
    assert capi.n_tuples(1) == 0 and capi.n_tuples(2) == 2 and capi.n_tuples(40) == 11440
    import oracle
    for nv in (2, 3, 9, 40):
        lst = oracle.tuple_list(nv)
        for t in range(len(lst)):
            assert tuple(lst[t]) == capi.tuple_at(nv, t)


def test_errors_without_gpu_are_status_codes():
    lib = capi.load()
    ctx = ctypes.c_void_p()
    rc = lib.atrip_gpu_create(ctypes.byref(capi.Dims(0, 10, 0, 0)), ctypes.byref(ctx))
    assert rc == capi.ERR_UNSUPPORTED
    assert b"No must be" in lib.atrip_gpu_last_error()
    rc = lib.atrip_gpu_tuple_at(10, 10 ** 6, *(ctypes.byref(ctypes.c_int32()) for _ in range(3)))
    assert rc == capi.ERR_ARGUMENT


def test_batch_plan_orders_by_cost():
    """Host logic of the batching form: systems in descending per-tuple
    cost, ties kept in caller order; empty input is fine."""
    import numpy as np
    no = [4, 20, 7, 20, 13, 4]
    nv = [30, 33, 12, 33, 41, 30]
    order = capi.batch_plan(no, nv)
    assert sorted(order.tolist()) == list(range(len(no)))

    def cost(i):
        return ((no[i] ** 2 + 63) // 64) * ((no[i] + 7) // 8) * (nv[i] + no[i])
    costs = [cost(i) for i in order]
    assert costs == sorted(costs, reverse=True)
    assert order.tolist().index(1) < order.tolist().index(3)  # stable
    assert order.tolist().index(0) < order.tolist().index(5)
    assert capi.batch_plan([], []).size == 0
    lib = capi.load()
    assert lib.atrip_gpu_batch_plan(None, None, 3, None) == capi.ERR_ARGUMENT
    h = ctypes.c_void_p()
    assert lib.atrip_gpu_batch_create(None, 0, ctypes.byref(h)) == capi.ERR_ARGUMENT


def test_split_profile_counter_layout_matches_kernel_and_header():
    """capi.SPLIT_PROFILE (the Python names of atrip_gpu_split_profile's
    counters) follows the kernel's slot enum and the header's count."""
    src = open(os.path.join(ROOT, "atrip_gb300", "csrc", "split_bf16.cu")).read()
    body = re.search(r"enum ProfSlot \{(.*?)\};", src, re.S).group(1)
    slots, nxt = {}, 0
    for item in (x.strip() for x in body.split(",")):
        if not item:
            continue
        name, _, val = (p.strip() for p in item.partition("="))
        nxt = int(val) if val else nxt
        slots[name] = nxt
        nxt += 1
    hdr = open(os.path.join(ROOT, "include", "atrip_gb300.h")).read()
    count = int(re.search(r"#define ATRIP_SPLIT_PROFILE_COUNTERS (\d+)", hdr).group(1))
    assert slots["kProfSlots"] == count == capi.SPLIT_PROFILE_COUNTERS
    kernel_names = {
        "kProfProdTotal": "producer_total", "kProfProdEmpty": "producer_wait_stage",
        "kProfProdTupleEmpty": "producer_wait_tuple_slot", "kProfMmaTotal": "mma_total",
        "kProfMmaTupleFull": "mma_wait_tuple", "kProfMmaAccEmpty": "mma_wait_accumulator",
        "kProfMmaFull": "mma_wait_stage", "kProfEpiTotal": "epilogue_total",
        "kProfEpiTupleFull": "epilogue_wait_tuple", "kProfEpiWFree": "epilogue_wait_w_buffer",
        "kProfEpiAccFull": "epilogue_wait_accumulator", "kProfEnTotal": "energy_total",
        "kProfEnTupleFull": "energy_wait_tuple", "kProfEnWFull": "energy_wait_w",
        "kProfEnWConvert": "energy_w_convert", "kProfUnits": "stages",
        "kProfTuples": "tuples", "kProfCtas": "ctas"}
    for k, py in kernel_names.items():
        assert capi.SPLIT_PROFILE[slots[k]] == py, (k, slots[k])
    assert len(kernel_names) == len([n for n in capi.SPLIT_PROFILE if n])
