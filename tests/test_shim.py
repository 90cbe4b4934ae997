"""The C++ drop-in (include/hbtu_subhalo.hpp) used the way HBT+ would use it.

Also, on the GPU: the nested caller (hbtu::RecursiveUnbindGPU + TruncateSource,
and hbtu::RefineParticlesGPU with a member table) reproduces the reference's
RecursiveUnbind forest (tests/golden/forest_10.npz), the merge caller
(hbtu::MergeSubhalosGPU) the reference's MergeSubhalos (merge_10.npz), and a
pass cap leaves a subhalo alike through UnbindGPU and UnbindBatchGPU.

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
                            C.c_void_p(out_e.ctypes.data), C.byref(res), C.byref(death),
                            C.c_int32(0))
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


def _ptr(x):
    return C.c_void_p(np.ascontiguousarray(x).ctypes.data)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_shim_forest_matches_reference(mode):
    """forest_10 (two haloes with satellites three deep, an orphan with a
    satellite, a satellite that disrupts, a field subhalo) through
    hbtu::RecursiveUnbindGPU + TruncateSource (mode 0) and through
    hbtu::RefineParticlesGPU with the haloes' member table (mode 1): the
    reference's final lists and Nbound, FP64 mode, bit for bit."""
    from hbtplus_gb300.unbind import Unbinder, params_from_dict
    from test_refine import golden_forest
    so = C.CDLL(build_shim())
    forest, params, z = golden_forest()
    nsub = len(forest["list_off"]) - 1
    f = {k: np.ascontiguousarray(v) for k, v in forest.items()}
    # the member table of mode 1: halo 0 is the tree of subhalo 0, halo 1 that of 7, and
    # subhalo 9 (no nests, not an orphan) is a field subhalo
    group_off = np.array([0, 7, 9], np.int64)
    group_idx = np.array([0, 1, 2, 3, 4, 5, 6, 7, 8], np.int64)
    heads_off = np.array([0, 1, 2], np.int64)
    heads_idx = np.array([0, 7], np.int64)
    field = np.array([9], np.int64)
    cap = 4 * len(f["id"])
    out_off = np.zeros(nsub + 1, np.int64)
    out_row = np.zeros(cap, np.int64)
    out_nb = np.zeros(nsub, np.int64)
    cp = params_from_dict(params, precision=1)
    keep = [out_off, out_row, out_nb, group_off, group_idx, heads_off, heads_idx, field]
    with Unbinder(params, precision=1) as ub:
        rc = so.shim_recursive_unbind(
            ub.handle, C.byref(cp), C.c_int32(mode), C.c_int64(nsub), _ptr(f["list_off"]),
            _ptr(f["id"]), _ptr(f["pos"]), _ptr(f["vel"]), _ptr(f["mass"]), _ptr(f["type"]),
            _ptr(f["nbound_prev"]), _ptr(f["ref_pos"]), _ptr(f["ref_vel"]),
            _ptr(f["mostbound_pos"]), _ptr(f["mostbound_vel"]), _ptr(f["nest_off"]),
            _ptr(f["nest_idx"]), C.c_int64(len(f["roots"])), _ptr(f["roots"]),
            C.c_int64(2), _ptr(group_off), _ptr(group_idx), _ptr(heads_off), _ptr(heads_idx),
            C.c_int64(1), _ptr(field), C.c_float(float(z["relax"])), C.c_int64(cap),
            _ptr(out_off), _ptr(out_row), _ptr(out_nb))
    del keep
    assert rc == 0, rc
    assert list(out_nb) == list(z["ref_nbound"])
    assert np.array_equal(out_off, z["ref_off"])
    assert np.array_equal(out_row[:out_off[-1]], z["ref_pos_out"])


@pytest.mark.gpu
def test_shim_merge_matches_reference():
    """merge_10 through hbtu::MergeSubhalosGPU (glued head nests, traps found
    on the GPU, MergeTo depth first on the host, the merged hosts unbound again
    in one batch and truncated), FP64 mode: the reference's lists, Nbound,
    sinks and deaths."""
    from hbtplus_gb300.unbind import Unbinder, params_from_dict
    from helpers import tie_groups_equal
    from test_merge import load
    so = C.CDLL(build_shim())
    par, st, ref, isnap, relax = load()
    nsub = len(st["list_off"]) - 1
    a = {k: np.ascontiguousarray(v) for k, v in st.items()}
    a["sink"] = np.ascontiguousarray(a["sink"], np.int64)
    a["death"] = np.ascontiguousarray(a["death"], np.int32)
    cap = 4 * len(a["id"])
    out_off = np.zeros(nsub + 1, np.int64)
    out_id = np.zeros(cap, np.int64)
    out_e = np.zeros(cap, np.float32)
    nb = np.zeros(nsub, np.int64)
    sink = np.zeros(nsub, np.int64)
    sink_snap = np.zeros(nsub, np.int32)
    death = np.zeros(nsub, np.int32)
    cp = params_from_dict(par, precision=1)
    nhalo = len(a["group_off"]) - 1
    with Unbinder(par, precision=1) as ub:
        rc = so.shim_merge_subhalos(
            ub.handle, C.byref(cp), C.c_int64(nsub), _ptr(a["list_off"]), _ptr(a["id"]),
            _ptr(a["pos"]), _ptr(a["vel"]), _ptr(a["mass"]), _ptr(a["type"]), _ptr(a["nbound"]),
            _ptr(a["ref_pos"]), _ptr(a["ref_vel"]), _ptr(a["mostbound_pos"]),
            _ptr(a["mostbound_vel"]), _ptr(a["nest_off"]), _ptr(a["nest_idx"]), C.c_int64(nhalo),
            _ptr(a["group_off"]), _ptr(a["group_idx"]), _ptr(a["heads_off"]), _ptr(a["heads_idx"]),
            _ptr(a["sink"]), _ptr(a["death"]), C.c_int32(isnap), C.c_float(relax),
            C.c_int64(cap), _ptr(out_off), _ptr(out_id), _ptr(out_e), _ptr(nb), _ptr(sink),
            _ptr(sink_snap), _ptr(death))
    assert rc == 0, rc
    assert list(nb) == list(ref["nbound"])
    assert list(sink) == list(ref["sink"])
    assert list(death) == list(ref["death"])
    newly = ref["sink_snap"] >= 0
    assert list(sink_snap[newly]) == list(ref["sink_snap"][newly])
    for s in range(nsub):
        got = out_id[out_off[s]:out_off[s + 1]]
        want = ref["id"][ref["off"][s]:ref["off"][s + 1]]
        e = out_e[out_off[s]:out_off[s + 1]]
        if np.isnan(e).all():
            assert np.array_equal(got, want), s
        else:  # unbound again: bound part up to runs of equal energy, tail exact
            k = int(np.sum(~np.isnan(e)))
            assert tie_groups_equal(got[:k], want[:k], e[:k]), s
            assert np.array_equal(got[k:], want[k:]), s


@pytest.mark.gpu
def test_shim_pass_cap_leaves_single_and_batch_forms_alike():
    """With max_passes reached, hbtu::UnbindGPU and hbtu::UnbindBatchGPU both
    return HBTU_ERR_NOT_CONVERGED and leave the subhalo in the same state (the
    last pass's order, Nbound and frame)."""
    from hbtplus_gb300 import _lib
    from hbtplus_gb300.unbind import Unbinder, _state, params_from_dict
    so = C.CDLL(build_shim())
    par, inp, _ = load_case("nfw_1100")
    n = len(inp["mass"])
    cp = params_from_dict(par, precision=1, max_passes=1)
    st = _state(inp["ref_pos"], inp["ref_vel"], inp["mostbound_pos"], inp["mostbound_vel"],
                inp["id"][0])
    arr = {k: np.ascontiguousarray(inp[k]) for k in ("id", "pos", "vel", "mass", "type")}
    outs = []
    with Unbinder(par, precision=1, max_passes=1) as ub:
        for via_batch in (0, 1):
            out_id = np.zeros(n, np.int64)
            out_e = np.zeros(n, np.float32)
            res = _lib.hbtu_result()
            death = C.c_int32(0)
            rc = so.shim_unbind(ub.handle, C.byref(cp), C.c_int64(n),
                                *[_ptr(arr[k]) for k in ("id", "pos", "vel", "mass", "type")],
                                C.byref(st), _ptr(out_id), _ptr(out_e), C.byref(res),
                                C.byref(death), C.c_int32(via_batch))
            assert rc == _lib.HBTU_ERR_NOT_CONVERGED
            outs.append((out_id.copy(), res.nbound, res.mbound, list(res.ref_pos)))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert outs[0][1:] == outs[1][1:]
    assert not np.array_equal(outs[0][0], arr["id"])  # the last pass's order was applied
