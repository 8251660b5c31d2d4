"""atrip_gb300 -- CCSD(T) triples energy on one NVIDIA GB300 (sm_103a).

A drop-in for the hot path of atrip: the Atrip / Input / Output interface
(``atrip_gb300.atrip``), backed by hand-written CUDA kernels behind the C ABI
in include/atrip_gb300.h (``atrip_gb300.capi``).
"""
from .atrip import (Atrip, Checkpoint, Input, IterationDescription, Output,  # noqa: F401
                    TuplesDistribution, read_checkpoint, register_iteration_descriptor, run,
                    write_checkpoint)

__all__ = ["Atrip", "Input", "Output", "Checkpoint", "IterationDescription",
           "TuplesDistribution", "read_checkpoint", "write_checkpoint",
           "register_iteration_descriptor", "run"]
