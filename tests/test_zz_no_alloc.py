"""hbtu_unbind_noalloc, the entry point that allocates nothing, against hbtu_unbind.

Some callers cannot allocate GPU memory at the moment they unbind: code that
runs inside another framework's memory pool, a process that reserves all
device memory at start-up, or a pipeline that forbids allocation after it has
started.  hbtu_unbind_noalloc serves them.  It takes device-resident inputs
and outputs from the caller and does its work in a fixed scratch array
compiled into the library.

This file is collected last, so a run that stops at the first failure has
already run every other test.  The checks call the entry point through the C
ABI twice in a row on different subhaloes.  The second call runs on the
scratch contents the first one left behind.  Each call must give exactly
hbtu_unbind's output for the same subhalo; both paths run the same kernels in
the same order.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_case

pytestmark = pytest.mark.gpu


def _noalloc(lib, _lib, par, inp, torch, precision=0):
    """Run hbtu_unbind_noalloc on device copies of a subhalo; return host results."""
    from hbtplus_gb300.unbind import _state, params_from_dict
    n = len(inp["mass"])
    dev = {k: torch.from_numpy(np.ascontiguousarray(inp[k])).cuda()
           for k in ("id", "pos", "vel", "mass", "type")}
    order = torch.full((max(n, 1),), -7, dtype=torch.int64, device="cuda")
    energy = torch.full((max(n, 1),), float("nan"), dtype=torch.float32, device="cuda")
    res = torch.zeros(C.sizeof(_lib.hbtu_result), dtype=torch.uint8, device="cuda")
    p = _lib.hbtu_particles(id=dev["id"].data_ptr(), pos=dev["pos"].data_ptr(),
                            vel=dev["vel"].data_ptr(), mass=dev["mass"].data_ptr(),
                            type=dev["type"].data_ptr(), location=_lib.HBTU_DEVICE, reserved=0)
    st = _state(inp["ref_pos"], inp["ref_vel"], inp["mostbound_pos"], inp["mostbound_vel"],
                inp.get("mostbound_id", inp["id"][0]))
    cp = params_from_dict(par, precision=precision)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.hbtu_unbind_noalloc(C.byref(cp), C.byref(p), n, C.byref(st), order.data_ptr(),
                                 energy.data_ptr(), res.data_ptr(), C.c_void_p(stream))
    torch.cuda.synchronize()
    _lib.check(rc, None)
    r = _lib.hbtu_result.from_buffer_copy(res.cpu().numpy().tobytes())
    return order.cpu().numpy()[:n], energy.cpu().numpy()[:n], r


def test_noalloc_matches_unbind_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import _lib
    from hbtplus_gb300.unbind import Unbinder, result_to_dict
    lib = _lib.load()
    for case in ("nfw_3300_corner", "nfw_1100"):
        par, inp, _ = load_case(case)
        assert len(inp["mass"]) <= _lib.HBTU_NOALLOC_MAX_PARTICLES
        with Unbinder(par) as ub:
            o_ref, e_ref, r_ref = ub.unbind(inp)
        order, energy, r = _noalloc(lib, _lib, par, inp, torch)
        assert np.array_equal(order, o_ref), case
        assert np.array_equal(energy, e_ref, equal_nan=True), case
        got = result_to_dict(r)
        for k, v in r_ref.items():
            np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(v), err_msg=f"{case}: {k}")


def _nfw(n, seed):
    """An NFW subhalo with contaminants, cut to exactly n particles."""
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(seed))
    sub = S.nfw_subhalo(rng, n, 0.2 * (n / 1e5) ** (1 / 3), 10.0, contaminant_frac=0.2,
                        center=rng.uniform(0, 100, 3))
    S._assign_ids(rng, [sub])
    for k in ("id", "pos", "vel", "mass", "type"):
        sub[k] = np.ascontiguousarray(sub[k][:n])
    assert len(sub["mass"]) == n
    return sub


@pytest.mark.parametrize("precision,max_sample", [(0, 0), (1, 0), (0, 1000), (1, 1000)])
def test_noalloc_multiblock_sizes_match_unbind(precision, max_sample):
    """Subhaloes large enough for the multi-block sort (more than 4096 records:
    its per-tile status words, tile counter and scan levels live in the scratch
    array too), up to the stated capacity, in both walk precisions and with the
    reference's sampled potentials; two calls in a row, each bit for bit equal
    to hbtu_unbind."""
    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import _lib
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder, result_to_dict
    lib = _lib.load()
    par = S.default_params(max_sample_size=max_sample)
    for n, seed in ((_lib.HBTU_NOALLOC_MAX_PARTICLES, 1), (9_000, 2)):
        inp = _nfw(n, seed)
        with Unbinder(par, precision=precision) as ub:
            o_ref, e_ref, r_ref = ub.unbind(inp)
        cp_par = dict(par)
        order, energy, r = _noalloc(lib, _lib, cp_par, inp, torch, precision=precision)
        tag = f"n={n} precision={precision} max_sample={max_sample}"
        assert np.array_equal(order, o_ref), tag
        assert np.array_equal(energy, e_ref, equal_nan=True), tag
        got = result_to_dict(r)
        for k, v in r_ref.items():
            np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(v), err_msg=f"{tag}: {k}")


def test_noalloc_rejects_oversized_and_host_inputs():
    pytest.importorskip("torch")
    from hbtplus_gb300 import _lib
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import _state, params_from_dict
    lib = _lib.load()
    cp = params_from_dict(S.default_params())
    st = _state([0, 0, 0], [0, 0, 0], [0, 0, 0], [0, 0, 0], 0)
    p = _lib.hbtu_particles(id=1, pos=1, vel=1, mass=1, type=0, location=_lib.HBTU_DEVICE,
                            reserved=0)
    res = _lib.hbtu_result()
    big = _lib.HBTU_NOALLOC_MAX_PARTICLES + 1
    rc = lib.hbtu_unbind_noalloc(C.byref(cp), C.byref(p), big, C.byref(st), 1, 1,
                                 C.addressof(res), None)
    assert rc == _lib.HBTU_ERR_TOO_LARGE
    assert b"capacity" in lib.hbtu_last_error(None)
    p.location = _lib.HBTU_HOST
    rc = lib.hbtu_unbind_noalloc(C.byref(cp), C.byref(p), 10, C.byref(st), 1, 1,
                                 C.addressof(res), None)
    assert rc == _lib.HBTU_ERR_INVALID_ARGUMENT
