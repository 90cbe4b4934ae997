"""The C++ drop-in (include/hbtu_subhalo.hpp) used the way HBT+ would use it.

CPU: the shim compiles against stand-ins with the reference's member names
(tests/shim/shim_lib.cpp) and, where the reference sources are present,
against the reference's own headers.  GPU: the compiled harness unbinds golden
subhaloes through hbtu::UnbindGPU and leaves them as the reference's Unbind
does (FP64 mode: bit-exact Nbound, Mbound, order and Energies), and computes
their profile and shape through hbtu::PropertiesGPU as the reference's
CalculateProfileProperties and CalculateShape do (tests/golden/props_10.npz),
and finds the reference's sinks through hbtu::DetectTrapsGPU
(tests/golden/merge_10.npz)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import load_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "shim")
SO = os.path.join(SHIM, "_build", "libshim.so")
from oracle import REFERENCE_DIR  # noqa: E402

REF_SRC = os.path.join(REFERENCE_DIR, "src") if REFERENCE_DIR else ""


def build_shim():
    from hbtplus_gb300 import build as B
    lib = B.build()
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    subprocess.run(["g++", "-std=c++11", "-O2", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "include"), os.path.join(SHIM, "shim_lib.cpp"), lib,
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", SO], check=True)
    return SO


def test_shim_compiles():
    assert os.path.exists(build_shim())


@pytest.mark.skipif(not REF_SRC or not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_shim_compiles_against_reference_types(tmp_path):
    src = tmp_path / "use_ref.cpp"
    src.write_text('#include "subhalo.h"\n#include "hbtu_subhalo.hpp"\n'
                   "void f(hbtu_handle *h, const hbtu_params &p, Subhalo_t &s, const Snapshot_t &e)"
                   "{ std::vector<float> E; hbtu::UnbindGPU(h, p, s, e, &E); "
                   "std::vector<Subhalo_t> v(1); hbtu::UnbindBatchGPU(h, p, v, {0}, e); "
                   "hbtu::PropertiesGPU(h, v, {0}, e); std::vector<char> m; "
                   "hbtu::DetectTrapsGPU(h, v, e, m); }\n")
    subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-DHBT_INT8", "-w",
                    "-I", os.path.join(ROOT, "oracle", "ref", "stubs"), "-I", REF_SRC,
                    "-I", os.path.join(ROOT, "include"), str(src)], check=True)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["nfw_2200_bulk", "nfw_3300_corner", "disrupt_220"])
def test_shim_unbind_matches_reference(case):
    from hbtplus_gb300 import _lib
    from hbtplus_gb300.unbind import Unbinder, _state, params_from_dict
    so = C.CDLL(build_shim())
    par, inp, ref = load_case(case)
    n = len(inp["mass"])
    cp = params_from_dict(par, precision=1)
    st = _state(inp["ref_pos"], inp["ref_vel"], inp["mostbound_pos"], inp["mostbound_vel"],
                inp["id"][0])
    arr = {k: np.ascontiguousarray(inp[k]) for k in ("id", "pos", "vel", "mass", "type")}
    out_id = np.zeros(n, np.int64)
    out_e = np.zeros(n, np.float32)
    res = _lib.hbtu_result()
    death = C.c_int32(0)
    with Unbinder(par, precision=1) as ub:
        rc = so.shim_unbind(ub.handle, C.byref(cp), C.c_int64(n),
                            *[C.c_void_p(arr[k].ctypes.data)
                              for k in ("id", "pos", "vel", "mass", "type")],
                            C.byref(st), C.c_void_p(out_id.ctypes.data),
                            C.c_void_p(out_e.ctypes.data), C.byref(res), C.byref(death))
    assert rc == 0
    nb = int(ref["nbound"])
    assert res.nbound == nb and res.mbound == float(ref["mbound"])
    np.testing.assert_array_equal(np.array(list(res.ref_pos), np.float32), ref["ref_pos"])
    ref_ids = inp["id"][ref["order"]]
    if int(ref["disrupted"]):
        np.testing.assert_array_equal(out_id, ref_ids)
        assert death.value == 7  # SnapshotIndexOfDeath set by the disruption branch
    else:
        np.testing.assert_array_equal(out_e[:nb], ref["energy"][:nb])
        assert set(out_id[:nb].tolist()) == set(ref_ids[:nb].tolist())
        assert death.value == -1


@pytest.mark.gpu
def test_shim_properties_match_reference():
    """The profile and shape of the reference's unbound subhaloes (props_10:
    the reference's order, Nbound, Mbound and most-bound position), computed
    through hbtu::PropertiesGPU with the member names of Subhalo_t."""
    from hbtplus_gb300 import _lib
    from hbtplus_gb300.unbind import Unbinder
    from test_props import SCALARS, TENSORS, compare, fixture_props, load
    so = C.CDLL(build_shim())
    par, b, ref, props, snap = load("props_10")  # the fixture's epoch is snapshot 1
    with Unbinder(par) as ub:
        for s in range(len(b["offsets"]) - 1):
            o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
            idx = o0 + ref["order"][o0:o1]  # the particles as Unbind leaves them
            pos = np.ascontiguousarray(b["pos"][idx], np.float32)
            mass = np.ascontiguousarray(b["mass"][idx], np.float32)
            ids = np.ascontiguousarray(b["id"][idx], np.int64)
            mbp = np.ascontiguousarray(ref["mostbound_pos"][s], np.float32)
            out = _lib.hbtu_props()
            rc = so.shim_properties(ub.handle, C.c_int64(o1 - o0), C.c_void_p(ids.ctypes.data),
                                    C.c_void_p(pos.ctypes.data), C.c_void_p(mass.ctypes.data),
                                    C.c_int64(int(ref["nbound"][s])),
                                    C.c_float(float(ref["mbound"][s])),
                                    C.c_void_p(mbp.ctypes.data),
                                    C.c_float(float(b["last_max_vmax"][s])),
                                    C.c_int32(int(b["last_snap"][s])), C.byref(out))
            assert rc == 0
            got = {k: getattr(out, k) for k in SCALARS + TENSORS}
            got = {k: (np.array(list(v), np.float32) if hasattr(v, "__len__") else v)
                   for k, v in got.items()}
            want = fixture_props(props, s)
            if int(ref["nbound"][s]) > 1:
                # the harness's epoch is snapshot 7 and the fixture's 1: the index of the
                # last maximum follows the epoch, everything else the particles
                if want["snapshot_of_last_max_vmax"] == snap:
                    want["snapshot_of_last_max_vmax"] = 7
                compare(got, want, ("shim", s))


@pytest.mark.gpu
def test_shim_detect_traps_match_reference():
    """hbtu::DetectTrapsGPU on the subhaloes of merge_10 (nests glued as
    MergeSubhalos glues them) gives the reference's sinks and merged hosts."""
    from hbtplus_gb300.merge import glued_nests
    from hbtplus_gb300.unbind import Unbinder
    from test_merge import load
    so = C.CDLL(build_shim())
    par, st, ref, isnap, relax = load()
    nests, _ = glued_nests(st)
    nest_off = np.concatenate([[0], np.cumsum([len(x) for x in nests])]).astype(np.int64)
    nest_idx = np.array([c for x in nests for c in x], np.int64)
    nsub = len(st["list_off"]) - 1
    a = {k: np.ascontiguousarray(st[k]) for k in ("list_off", "id", "pos", "vel", "mass",
                                                   "nbound", "mostbound_pos", "mostbound_vel",
                                                   "sink")}
    sink = np.zeros(nsub, np.int64)
    snap = np.zeros(nsub, np.int32)
    merged = np.zeros(nsub, np.int32)
    ptr = lambda x: C.c_void_p(x.ctypes.data)  # noqa: E731
    with Unbinder(par) as ub:
        rc = so.shim_detect_traps(ub.handle, C.c_int64(nsub), ptr(a["list_off"]), ptr(a["id"]),
                                  ptr(a["pos"]), ptr(a["vel"]), ptr(a["mass"]), ptr(a["nbound"]),
                                  ptr(a["mostbound_pos"]), ptr(a["mostbound_vel"]),
                                  ptr(nest_off), ptr(nest_idx), ptr(a["sink"]), ptr(sink),
                                  ptr(snap), ptr(merged))
    assert rc == 0
    assert list(sink) == list(ref["sink"])
    newly = ref["sink_snap"] == isnap  # trapped at this snapshot (the harness's epoch is 7)
    assert list(np.nonzero(snap == 7)[0]) == list(np.nonzero(newly)[0])
    want = {int(ref["sink"][s]) for s in np.nonzero(newly)[0] if st["nbound"][s] > 1}
    assert set(np.nonzero(merged)[0].tolist()) == want
