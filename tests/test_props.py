"""Post-unbinding properties (hbtu_subhalo_properties): the members
Subhalo_t::CalculateProfileProperties and ::CalculateShape write
(src/subhalo.cpp:242-398) after each subhalo's Unbind.

CPU: the C restatement (oracle) reproduces the reference's own properties in
tests/golden/props_*.npz (made by tests/golden/make_golden.py from the
reference build: Unbind, then the two property routines), field for field and
bit for bit, on the reference's bound particles.
GPU: the library's unbinding (with the FP64 walk, which reproduces the
reference's bound sets) followed by its properties call gives, against the
same fixtures, and against the oracle on random batches (with mixed-mass
species, distance ties, box faces and subhaloes too small to have a profile):
every profile field bit for bit (Rmax, Vmax, RHalf, R2Sigma, M200Crit,
R200Crit, the last-maximum update), and the inertia tensors within one float
unit in the last place -- the tolerance of a double sum taken in another order
than the reference's sequential loop; nearly all of them agree exactly.  The
batch call, one call per subhalo and the device-resident call agree; both ways
of summing the cumulative mass (exact fixed point and the sequential double
fallback for masses of too wide a binary range) are exercised.
"""
import os
import sys

import numpy as np
import pytest

from helpers import GOLDEN, tie_groups_equal

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))

SCALARS = ("rmax_comoving", "vmax_physical", "last_max_vmax_physical",
           "snapshot_of_last_max_vmax", "r2sigma_comoving", "rhalf_comoving",
           "r200crit_comoving", "m200crit")
TENSORS = ("inertial_tensor", "inertial_tensor_weighted")
TENSOR_ULPS = 1  # double sums in another order, cast to float
CASES = ("props_10", "props_a05")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    par = {k[4:]: z[k].item() for k in z.files if k.startswith("par_")}
    b = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    props = {k[6:]: z[k] for k in z.files if k.startswith("props_")}
    return par, b, ref, props, int(z["snapshot_index"])


def ulp_diff(a, b):
    """Distance in float32 units in the last place (same-sign values)."""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7fffffff), ia)
    ib = np.where(ib < 0, -(ib & 0x7fffffff), ib)
    return np.abs(ia - ib)


def same_bits(g, w):
    """float32 values equal bit for bit, or both NaN (NaN payloads differ
    between CPUs and GPUs)."""
    g = np.asarray(g, np.float32)
    w = np.asarray(w, np.float32)
    both_nan = np.isnan(g) & np.isnan(w)
    return bool(np.all(both_nan | (g.view(np.uint32) == w.view(np.uint32))))


def compare(got, want, tag=""):
    """Scalars bit for bit, tensors within TENSOR_ULPS; returns the number of
    tensor components that differ at all."""
    for k in SCALARS:
        if k == "snapshot_of_last_max_vmax":
            assert int(got[k]) == int(want[k]), (tag, k, got[k], want[k])
        else:
            assert same_bits(got[k], want[k]), (tag, k, got[k], want[k])
    ndiff = 0
    for k in TENSORS:
        g = np.asarray(got[k], np.float32)
        w = np.asarray(want[k], np.float32)
        nan = np.isnan(g) & np.isnan(w)
        d = np.where(nan, 0, ulp_diff(np.where(nan, 0, g), np.where(nan, 0, w)))
        assert d.max() <= TENSOR_ULPS, (tag, k, got[k], want[k])
        ndiff += int((d > 0).sum())
    return ndiff


def fixture_props(props, s):
    return {k: props[k][s] for k in SCALARS + TENSORS}


def bound_part(b, order, nbound, s):
    o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
    idx = o0 + np.asarray(order[o0:o1], np.int64)[:max(int(nbound), 0)]
    return b["pos"][idx], b["mass"][idx]


def oracle_props(orc, par, b, order, results, last_max, last_snap, snap):
    out = []
    for s, r in enumerate(results):
        pos, mass = bound_part(b, order, r["nbound"], s)
        out.append(orc.subhalo_properties(par, pos, mass, r["mostbound_pos"], r["mbound"],
                                          float(last_max[s]), int(last_snap[s]), snap))
    return out


def mass_paths(b, nbounds, order):
    """How the library sums each subhalo's cumulative mass in one batch call:
    'fixed' (exact 64-bit fixed point) or 'seq' (sequential double), by the
    rule of the CUDA code (units of the batch's lowest mass bit, every prefix
    inside an int64, the subhalo's total below 2^53 units)."""
    segs = []
    for s, nb in enumerate(nbounds):
        nb = int(nb) if nb > 1 else 0
        segs.append(bound_part(b, order, nb, s)[1].astype(np.float64))
    allm = np.concatenate(segs) if segs else np.zeros(0)
    T = len(allm)
    if (allm < 0).any() or not np.isfinite(allm).all():
        return ["seq"] * len(segs)
    nz = allm[allm != 0]
    if len(nz) == 0:
        return ["fixed"] * len(segs)
    f, e = np.frexp(nz)
    M = (f * 2.0 ** 24).astype(np.int64)
    tz = np.array([(int(x) & -int(x)).bit_length() - 1 for x in M])
    lo, hi = int((e - 24 + tz).min()), int((e - 1).max())
    if hi - lo + 1 + int(T).bit_length() > 62:
        return ["seq"] * len(segs)
    return ["fixed" if sum(int(np.ldexp(m, -lo)) for m in sg) < 2 ** 53 else "seq"
            for sg in segs]


@pytest.fixture(scope="module")
def oracle():
    from oracle import Oracle
    return Oracle()


# ------------------------------------------------------------------- CPU
@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_props(oracle, name):
    par, b, ref, props, snap = load(name)
    nsub = len(b["offsets"]) - 1
    for s in range(nsub):
        pos, mass = bound_part(b, ref["order"], ref["nbound"][s], s)
        got = oracle.subhalo_properties(par, pos, mass, ref["mostbound_pos"][s],
                                        float(ref["mbound"][s]), float(b["last_max_vmax"][s]),
                                        int(b["last_snap"][s]), snap)
        want = fixture_props(props, s)
        for k in SCALARS + TENSORS:  # the oracle sums in the reference's order: all exact
            assert same_bits(got[k], want[k]), (name, s, k)


def test_fixture_covers_edges():
    par, b, ref, props, snap = load("props_10")
    nb = ref["nbound"]
    assert (nb <= 1).sum() >= 2                                 # no profile at all
    upd = props["snapshot_of_last_max_vmax"] == snap
    assert upd.any() and (~upd & (nb > 1)).any()                # last maximum moved and kept
    assert (props["r200crit_comoving"][nb > 1] > 0).all()
    # cumulative-mass paths: batch-wide sequential (the 2^60 mass range) ...
    assert set(mass_paths(b, nb, ref["order"])) == {"seq"}
    # ... and per subhalo both ways
    paths = []
    for s in range(len(nb)):
        one = {k: b[k] for k in ("pos", "mass")}
        o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
        one = {k: v[o0:o1] for k, v in one.items()}
        one["offsets"] = np.array([0, o1 - o0])
        paths += mass_paths(one, [nb[s]], ref["order"][o0:o1])
    assert "fixed" in paths and "seq" in paths


def test_mass_path_rule():
    b = dict(offsets=np.array([0, 4, 8]), mass=np.array([1, 1, 1, 1, 1, 2, 3, 4], np.float32),
             pos=np.zeros((8, 3), np.float32))
    order = np.array([0, 1, 2, 3, 0, 1, 2, 3])
    assert mass_paths(b, [4, 4], order) == ["fixed", "fixed"]
    # lowest bit 2^-23, highest 2^30: the batch keeps a scale (54 + 4 bits), but
    # the second subhalo's total exceeds 2^53 units
    b["mass"][5] = np.float32(2.0 ** 30)
    b["mass"][6] = np.float32(1.0 + 2.0 ** -23)
    assert mass_paths(b, [4, 4], order) == ["fixed", "seq"]
    b["mass"][5] = np.float32(2.0 ** 40)  # 68 bits: no scale for the batch
    assert mass_paths(b, [4, 4], order) == ["seq", "seq"]
    b["mass"][5] = np.float32(2.0)
    b["mass"][0] = np.float32(-1.0)
    assert mass_paths(b, [4, 4], order) == ["seq", "seq"]


# ------------------------------------------------------------------- GPU
def gpu_unbinder(par, precision=0):
    from hbtplus_gb300.unbind import Unbinder
    return Unbinder(par, precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_props(name):
    par, b, ref, props, snap = load(name)
    nsub = len(b["offsets"]) - 1
    ub = gpu_unbinder(par, precision=1)  # the FP64 walk: the reference's bound sets exactly
    order, energy, res = ub.unbind_batch(b)
    for s in range(nsub):  # the reference's order up to runs of equal energy
        o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
        assert tie_groups_equal(order[o0:o1], ref["order"][o0:o1], energy[o0:o1]), s
        nb = int(ref["nbound"][s])
        assert np.array_equal(energy[o0:o0 + nb], ref["energy"][o0:o0 + nb]), s
    assert [r["nbound"] for r in res] == list(ref["nbound"])
    got = ub.subhalo_properties(b, order, res, b["last_max_vmax"], b["last_snap"], snap)
    ndiff = sum(compare(got[s], fixture_props(props, s), (name, s)) for s in range(nsub))
    assert ndiff <= 2 * nsub, ndiff
    # one call per subhalo: the same values
    for s in range(nsub):
        o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
        one = dict(id=b["id"][o0:o1], pos=b["pos"][o0:o1], vel=b["vel"][o0:o1],
                   mass=b["mass"][o0:o1], offsets=np.array([0, o1 - o0], np.int64))
        g1 = ub.subhalo_properties(one, order[o0:o1], [res[s]], b["last_max_vmax"][s:s + 1],
                                   b["last_snap"][s:s + 1], snap)[0]
        compare(g1, fixture_props(props, s), (name, "single", s))
    ub.close()


def random_batch(seed, nsub=160):
    from hbtplus_gb300 import synthetic as S
    b = S.subhalo_batch(nsub=nsub, seed=seed, nmax=6000)
    rng = np.random.default_rng(seed)
    off = b["offsets"]
    for s in range(nsub):
        o0, o1 = int(off[s]), int(off[s + 1])
        u = rng.uniform()
        if u < 0.15:  # mixed species: masses over 2^-6 .. 2^6 of the base
            f = np.exp2(rng.uniform(-6, 6, o1 - o0))
            b["mass"][o0:o1] = (b["mass"][o0:o1] * f).astype(np.float32)
        elif u < 0.3:  # coincident particles: distance ties
            k = np.arange(o0 + 1, o1, 5)
            b["pos"][k] = b["pos"][k - 1]
    last_max = rng.uniform(0.0, 400.0, nsub).astype(np.float32)
    last_max[rng.uniform(size=nsub) < 0.3] = 0.0
    last_snap = rng.integers(-1, 30, nsub).astype(np.int32)
    return b, last_max, last_snap


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [41, 42])
def test_gpu_matches_oracle_random(oracle, seed):
    from hbtplus_gb300 import synthetic as S
    par = S.default_params()
    b, last_max, last_snap = random_batch(seed)
    ub = gpu_unbinder(par)
    order, energy, res = ub.unbind_batch(b, check_status=False)
    got = ub.subhalo_properties(b, order, res, last_max, last_snap, 31)
    want = oracle_props(oracle, par, b, order, res, last_max, last_snap, 31)
    nsub = len(res)
    ndiff = sum(compare(got[s], want[s], (seed, s)) for s in range(nsub))
    assert ndiff <= 0.02 * 12 * nsub, ndiff
    paths = mass_paths(b, [r["nbound"] for r in res], order)
    assert set(paths) == {"fixed"} or "seq" in paths
    # every subhalo alone: covers both cumulative-mass paths
    seen = set()
    for s in range(0, nsub, 7):
        o0, o1 = int(b["offsets"][s]), int(b["offsets"][s + 1])
        one = dict(pos=b["pos"][o0:o1], mass=b["mass"][o0:o1],
                   offsets=np.array([0, o1 - o0], np.int64))
        g1 = ub.subhalo_properties(one, order[o0:o1], [res[s]], last_max[s:s + 1],
                                   last_snap[s:s + 1], 31)[0]
        compare(g1, want[s], (seed, "single", s))
        seen.update(mass_paths(one, [res[s]["nbound"]], order[o0:o1]))
    assert "fixed" in seen
    ub.close()


@pytest.mark.gpu
def test_gpu_sequential_fallback_matches_oracle(oracle):
    """Masses over 2^-30 .. 2^30 of the base: no fixed-point scale for the
    batch, every subhalo summed sequentially in double."""
    from hbtplus_gb300 import synthetic as S
    par = S.default_params()
    b, last_max, last_snap = random_batch(43, nsub=40)
    rng = np.random.default_rng(5)
    b["mass"] = (b["mass"] * np.exp2(rng.uniform(-30, 30, len(b["mass"])))).astype(np.float32)
    ub = gpu_unbinder(par)
    order, energy, res = ub.unbind_batch(b, check_status=False)
    assert set(mass_paths(b, [r["nbound"] for r in res], order)) == {"seq"}
    got = ub.subhalo_properties(b, order, res, last_max, last_snap, 2)
    want = oracle_props(oracle, par, b, order, res, last_max, last_snap, 2)
    for s in range(len(res)):
        compare(got[s], want[s], ("seq", s))
    ub.close()


@pytest.mark.gpu
def test_gpu_device_resident_and_empty(oracle):
    """The device-resident call (torch tensors from unbind_batch_device) equals
    the host call; an empty subhalo and NULL last-maximum arrays give zeros and
    the defaults (0, -1)."""
    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import synthetic as S
    par = S.default_params()
    b, last_max, last_snap = random_batch(44, nsub=60)
    # an empty subhalo in the middle
    off = b["offsets"]
    b["offsets"] = np.concatenate([off[:31], off[30:]]).astype(np.int64)
    for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
        b[k] = np.concatenate([b[k][:30], b[k][30:31], b[k][30:]])
    b["mostbound_id"] = np.concatenate([b["mostbound_id"][:30], [-1], b["mostbound_id"][30:]])
    nsub = len(b["offsets"]) - 1
    ub = gpu_unbinder(par)
    order, energy, res = ub.unbind_batch(b, check_status=False)
    host = ub.subhalo_properties(b, order, res)
    z = host[30]
    assert z["vmax_physical"] == 0 and z["last_max_vmax_physical"] == 0
    assert z["snapshot_of_last_max_vmax"] == -1
    dev = {k: torch.from_numpy(np.ascontiguousarray(b[k])).cuda()
           for k in ("id", "pos", "vel", "mass", "type")}
    n = int(b["offsets"][-1])
    out = dict(order=torch.empty(n, dtype=torch.int64, device="cuda"),
               energy=torch.empty(n, dtype=torch.float32, device="cuda"),
               res=torch.empty(nsub * C_sizeof_result(), dtype=torch.uint8, device="cuda"))
    ub.set_stream(torch.cuda.current_stream().cuda_stream)
    ub.unbind_batch_device(dev, b["offsets"], ub.make_states(b), out)
    arr = ub.subhalo_properties_device(dev, b["offsets"], out["order"], out["res"])
    torch.cuda.synchronize()
    from hbtplus_gb300.unbind import props_to_dict
    for s in range(nsub):
        g = props_to_dict(arr[s])
        for k in SCALARS + TENSORS:  # the same code path: identical
            assert same_bits(g[k], host[s][k]), (s, k)
    ub.close()


def C_sizeof_result():
    import ctypes
    from hbtplus_gb300 import _lib
    return ctypes.sizeof(_lib.hbtu_result)


@pytest.mark.gpu
def test_gpu_large_subhalo(oracle):
    """One subhalo of 2e6 particles (about 2000 shape chunks): against the oracle."""
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(77))
    sub = S.nfw_subhalo(rng, 2_000_000, 0.6, 8.0, contaminant_frac=0.05)
    S._assign_ids(rng, [sub])
    b = S.concat([sub])
    par = S.default_params()
    ub = gpu_unbinder(par)
    order, energy, res = ub.unbind_batch(b)
    got = ub.subhalo_properties(b, order, res, [100.0], [3], 4)[0]
    want = oracle_props(oracle, par, b, order, res, [100.0], [3], 4)[0]
    compare(got, want, "2e6")
    ub.close()


@pytest.mark.gpu
def test_gpu_rejects_bad_order():
    """An order entry outside its subhalo is refused (the kernels read the
    subhalo's first particle instead, so nothing is read out of bounds)."""
    from hbtplus_gb300 import _lib
    par, b, ref, props, snap = load("props_a05")
    ub = gpu_unbinder(par, precision=1)
    order, energy, res = ub.unbind_batch(b)
    bad = order.copy()
    bad[3] = int(b["offsets"][1]) + 5
    with pytest.raises(_lib.HBTUError):
        ub.subhalo_properties(b, bad, res)
    got = ub.subhalo_properties(b, order, res, b["last_max_vmax"], b["last_snap"], snap)
    compare(got[0], fixture_props(props, 0))  # the handle still works
    ub.close()
