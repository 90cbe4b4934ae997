"""The C ABI library (libhbtu.so) on the CPU: it builds, loads without a GPU,
exports every entry point include/hbtu.h declares, and its structures have
the layout the header gives them.  No compute call is made here."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from hbtplus_gb300 import _lib
from hbtplus_gb300 import build as B

HEADER = os.path.join(os.path.dirname(B.HERE), "include", "hbtu.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(hbtu_\w+)\s*\(", text, re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert "hbtu_unbind" in names and "hbtu_unbind_batch" in names
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures out of date"
    assert lib.hbtu_version() >= 10000


def test_struct_layouts_match_header():
    src = r"""
#include <stddef.h>
#include <stdio.h>
#include "hbtu.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("params %zu\nstate %zu\nresult %zu\nparticles %zu\nstats %zu\n", sizeof(hbtu_params),
         sizeof(hbtu_state), sizeof(hbtu_result), sizeof(hbtu_particles), sizeof(hbtu_stats));
  P(hbtu_stats, small_ms) P(hbtu_stats, small_subhaloes)
  P(hbtu_result, nbound_type) P(hbtu_result, iterations) P(hbtu_result, evaluations)
  P(hbtu_result, status) P(hbtu_params, precision) P(hbtu_params, device)
  P(hbtu_state, mostbound_id) P(hbtu_particles, location)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    assert int(got["params"]) == C.sizeof(_lib.hbtu_params)
    assert int(got["state"]) == C.sizeof(_lib.hbtu_state)
    assert int(got["result"]) == C.sizeof(_lib.hbtu_result)
    assert int(got["particles"]) == C.sizeof(_lib.hbtu_particles)
    assert int(got["stats"]) == C.sizeof(_lib.hbtu_stats)
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            assert int(val) == getattr(getattr(_lib, t), f).offset, key


def test_invalid_parameters_rejected_before_any_device_use():
    lib = _lib.load()
    p = _lib.hbtu_params(softening=0.0, open_angle=0.45, bound_mass_precision=0.995,
                         min_num_part=20, periodic=1, box_size=100.0, G=43.0071, hubble=100.0,
                         scale_factor=1.0)
    h = C.c_void_p()
    assert lib.hbtu_create(C.byref(p), C.byref(h)) == _lib.HBTU_ERR_INVALID_ARGUMENT
    assert b"softening" in lib.hbtu_last_error(None)
    p.softening = 0.002
    p.bound_mass_precision = 1.5
    assert lib.hbtu_create(C.byref(p), C.byref(h)) == _lib.HBTU_ERR_INVALID_ARGUMENT


def test_create_without_gpu_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    p = _lib.hbtu_params(softening=0.002, open_angle=0.45, bound_mass_precision=0.995,
                         min_num_part=20, periodic=1, box_size=100.0, G=43.0071, hubble=100.0,
                         scale_factor=1.0)
    h = C.c_void_p()
    assert lib.hbtu_create(C.byref(p), C.byref(h)) == _lib.HBTU_ERR_NO_DEVICE
