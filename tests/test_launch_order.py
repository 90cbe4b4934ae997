"""Every kernel the library launches with programmatic stream serialisation
(launch_k in hbtplus_gb300/csrc/hbtu_internal.h) may be scheduled while its
predecessor in the stream still runs, so its first statement must be
HBTU_KERNEL_PROLOGUE() (griddepcontrol.wait: nothing is read or written before
the predecessor has completed).  This test reads the sources: each kernel
named in a launch_k call is found and its body's first statement checked."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hbtplus_gb300", "csrc")


def _sources():
    out = {}
    for f in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh"))):
        with open(f) as fh:
            out[os.path.basename(f)] = fh.read()
    return out


def _kernel_bodies(src):
    """name -> first statement of each __global__ function's body."""
    bodies = {}
    sig = r"__global__\s+(?:void\s+)?(?:__launch_bounds__\([^)]*\)\s+)?(?:void\s+)?([A-Za-z_]\w*)\s*\("
    for m in re.finditer(sig, src):
        brace = src.index("{", m.end())
        rest = src[brace + 1:].lstrip()
        first = rest.split(";", 1)[0].strip() + ";"
        bodies.setdefault(m.group(1), []).append(first)
    return bodies


def test_launch_k_kernels_open_with_the_dependency_wait():
    srcs = _sources()
    bodies = {}
    for src in srcs.values():
        for k, v in _kernel_bodies(src).items():
            bodies.setdefault(k, []).extend(v)
    launched = set()
    for name, src in srcs.items():
        for m in re.finditer(r"\blaunch_k\(\s*([A-Za-z_]\w*)", src):
            launched.add(m.group(1))
    launched.discard("kernel")  # the wrapper's own parameter
    assert len(launched) >= 40, sorted(launched)
    for k in sorted(launched):
        assert k in bodies, f"kernel {k} launched by launch_k but not found"
        for first in bodies[k]:
            assert first == "HBTU_KERNEL_PROLOGUE();", f"{k} opens with {first!r}"


def test_no_plain_launch_of_a_serialised_kernel():
    """A kernel launched both ways would be fine, but the hot path uses one:
    no <<< >>> launch remains in the files that use launch_k."""
    for name, src in _sources().items():
        if "launch_k(" in src and name not in ("hbtu_internal.h",):
            assert "<<<" not in src, f"{name} mixes launch_k and <<< >>> launches"
