"""atrip's C++ API through the drop-in header (include/atrip.hpp): compiles
against the MPI/CTF stand-ins without a GPU; runs on the GPU and matches
the oracle (FP64 form at 1e-10, split forms within their bounds, the
complex field's FP64 form at 1e-10)."""
import os
import subprocess

import pytest

import oracle
from atrip_gb300 import _build, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_main.cxx")


def build_driver(tmpdir):
    _build.build()
    exe = os.path.join(tmpdir, "dropin")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ref_shims"), "-I", "/usr/local/cuda/include",
           SRC, "-o", exe, "-L", os.path.dirname(_build.LIB), "-latrip_gb300",
           "-Wl,-rpath," + os.path.dirname(_build.LIB)]
    subprocess.check_call(cmd)
    return exe


def test_dropin_header_compiles(tmp_path):
    assert os.path.exists(build_driver(str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("form,tol,field", [(0, 1e-10, "real"), (1, 1e-6, "real"),
                                            (3, 5e-6, "real"), (0, 1e-10, "complex")])
def test_dropin_runs_and_matches_oracle(tmp_path, form, tol, field):
    """run<double> in the FP64 form and the two split forms (BF16, 3 slices;
    FP16, 2 slices) and run<Complex> (FP64 form)."""
    exe = build_driver(str(tmp_path))
    d = synth.make_inputs(6, 11, 2, with_j=True, field=field)
    data = str(tmp_path / "in")
    synth.write_bin_dir(d, data)
    out = subprocess.run([exe, data, str(form)], capture_output=True, text=True, check=True)
    line = [l for l in out.stdout.splitlines() if l.startswith("RESULT")][0]
    e, ect = (float(x) for x in line.split()[1:])
    ref_e, ref_ect = oracle.run(oracle.Problem(d))
    assert abs(e - ref_e) <= tol * abs(ref_e)
    assert abs(ect - ref_ect) <= tol * abs(ref_e)
