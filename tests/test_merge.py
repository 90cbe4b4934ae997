"""Merging of trapped subhaloes (hbtplus_gb300.merge, hbtu_merge_detect):
SubhaloSnapshot_t::MergeSubhalos, src/subhalo_merge.cpp:187-262.

tests/golden/merge_10.npz holds the reference's own MergeSubhalos (built from
its sources by oracle/Makefile, driven by oracle/ref/ref_driver.cpp) over ten
subhaloes after their unbinding: a satellite sinking into its central's core,
a sub-satellite sinking into its satellite host, a second top-level subhalo
sinking into its halo's central (through the glued nest), an orphan that is
trapped but gives no particles, a subhalo trapped earlier that merges now,
and subhaloes that stay; the central also lists particles of the sinking
satellite, so the union drops duplicate Ids.

CPU: the C restatement of the cores and trap detection gives the reference's
sinks and merged hosts; the merge orchestration, run on the oracle, gives the
reference's lists, Nbound, sinks, deaths and re-unbinding results.
GPU: the cores and traps of hbtu_merge_detect equal the restatement's bit for
bit on random forests (periodic faces, chains several hosts deep, orphans,
subhaloes trapped before); the whole merge with the GPU unbinding (FP64 walk)
gives the reference's result; a host chain with a cycle is refused.
"""
import os
import sys

import numpy as np
import pytest

from helpers import GOLDEN, OracleUnbinder, tie_groups_equal

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))


def load():
    z = np.load(os.path.join(GOLDEN, "merge_10.npz"))
    par = {k[4:]: z[k].item() for k in z.files if k.startswith("par_")}
    st = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    return par, st, ref, int(z["isnap"]), float(z["relax"])


@pytest.fixture(scope="module")
def oracle():
    from oracle import Oracle
    return Oracle()


def check_against_reference(out, st, ref, energy_of):
    nsub = len(st["list_off"]) - 1
    ids = st["id"]
    assert list(out["nbound"]) == list(ref["nbound"])
    assert list(out["sink"]) == list(ref["sink"])
    assert list(out["death"]) == list(ref["death"])
    newly = out["sink_snap"] >= 0
    assert list(out["sink_snap"][newly]) == list(ref["sink_snap"][newly])
    for s in range(nsub):
        got = ids[out["lists"][s]]
        want = ref["id"][ref["off"][s]:ref["off"][s + 1]]
        if out["merged"][s]:  # unbound again: the order up to runs of equal energy
            e = energy_of(s)
            assert tie_groups_equal(got, want, e[:len(got)]), s
            r = out["results"][s]
            for k in ("nbound", "mbound", "mostbound_pos", "mostbound_vel", "ref_pos", "ref_vel"):
                assert np.array_equal(np.asarray(r[k]), ref[k][s]), (s, k)
        else:
            assert np.array_equal(got, want), s


# ------------------------------------------------------------------- CPU
def test_fixture_covers_the_cases():
    par, st, ref, isnap, relax = load()
    from hbtplus_gb300.merge import glued_nests, host_track_ids
    nests, groups = glued_nests(st)
    host = host_track_ids(len(st["list_off"]) - 1, nests)
    sunk = np.nonzero(ref["death"] == isnap)[0]
    assert len(sunk) >= 4
    assert (ref["sink"][sunk] >= 0).all()
    assert any(host[s] >= 0 and st["heads_idx"].tolist().count(s) for s in sunk)  # glued head
    assert (st["nbound"][sunk] <= 1).any()                 # an orphan
    assert (st["sink"] >= 0).any()                          # trapped before
    ids = ref["id"]
    for s in range(len(ref["nbound"])):
        lst = ids[ref["off"][s]:ref["off"][s + 1]]
        assert len(np.unique(lst)) == len(lst)             # the union kept Ids unique


def test_oracle_detect_matches_reference(oracle):
    par, st, ref, isnap, relax = load()
    from hbtplus_gb300.merge import glued_nests, host_track_ids
    nests, groups = glued_nests(st)
    nsub = len(st["list_off"]) - 1
    host = host_track_ids(nsub, nests)
    sink, snap, merged, cores = oracle.merge_detect(
        par, st["list_off"], st["pos"], st["vel"], st["mass"], st["nbound"], host,
        st["mostbound_pos"], st["mostbound_vel"], isnap, st["sink"])
    assert list(sink) == list(ref["sink"])
    newly = snap >= 0
    assert list(snap[newly]) == list(ref["sink_snap"][newly])
    assert set(np.nonzero(newly)[0]) == set(np.nonzero(ref["sink_snap"] == isnap)[0])
    want_merged = {int(sink[s]) for s in np.nonzero(newly)[0] if st["nbound"][s] > 1}
    assert set(np.nonzero(merged)[0].tolist()) == want_merged


def test_merge_on_oracle_matches_reference(oracle):
    par, st, ref, isnap, relax = load()
    from hbtplus_gb300.merge import merge_subhalos
    out = merge_subhalos(OracleUnbinder(oracle, par), st, isnap, relax)
    check_against_reference(out, st, ref, lambda s: out["energy"][s])


def test_host_track_ids_rule():
    from hbtplus_gb300.merge import glued_nests, host_track_ids
    st = dict(nest_off=np.array([0, 2, 3, 3, 3, 3]), nest_idx=np.array([1, 2, 2]),
              group_off=np.array([0, 3, 5]), group_idx=np.array([0, 1, 2, 3, 4]),
              heads_off=np.array([0, 1, 3]), heads_idx=np.array([0, 3, 4]))
    nests, groups = glued_nests(st)
    assert nests[3] == [4]                            # head 4 glued to central 3
    assert list(host_track_ids(5, nests)) == [-1, 0, 1, -1, 3]  # 2: the last nest wins


# ------------------------------------------------------------------- GPU
def random_state(seed, nsub=3000):
    """Subhaloes of 1-60 particles in a periodic box; a random forest of
    hosts (chains several deep); most-bound particles placed near a host's
    core for some, so traps happen at every depth."""
    rng = np.random.default_rng(seed)
    box = 100.0
    n = rng.integers(0, 61, nsub)
    n[rng.uniform(size=nsub) < 0.05] = 1
    lo = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
    host = np.full(nsub, -1, np.int64)
    for s in range(1, nsub):
        if rng.uniform() < 0.8:
            host[s] = rng.integers(max(0, s - 50), s)
    centre = rng.uniform(0, box, (nsub, 3))
    centre[rng.uniform(size=nsub) < 0.1, 0] = rng.uniform(-0.01, 0.01) % box  # box face
    vcen = rng.normal(0, 200, (nsub, 3))
    for s in range(nsub):  # satellites near their host, some in its core
        if host[s] >= 0:
            near = rng.uniform() < 0.5
            centre[s] = (centre[host[s]] + rng.normal(0, 0.002 if near else 0.2, 3)) % box
            vcen[s] = vcen[host[s]] + rng.normal(0, 3 if near else 200, 3)
    N = int(lo[-1])
    seg = np.repeat(np.arange(nsub), n)
    pos = ((centre[seg] + rng.normal(0, 0.004, (N, 3))) % box).astype(np.float32)
    vel = (vcen[seg] + rng.normal(0, 5, (N, 3))).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, N).astype(np.float32)
    nbound = np.minimum(n, rng.integers(0, 61, nsub)).astype(np.int64)
    mbp = np.array([pos[lo[s]] if n[s] else centre[s] for s in range(nsub)], np.float32)
    mbv = np.array([vel[lo[s]] if n[s] else vcen[s] for s in range(nsub)], np.float32)
    sink = np.full(nsub, -1, np.int64)
    sink[rng.uniform(size=nsub) < 0.05] = 0
    return dict(list_off=lo, pos=pos, vel=vel, mass=mass, nbound=nbound, host=host,
                mostbound_pos=mbp, mostbound_vel=mbv, sink=sink)


@pytest.mark.gpu
@pytest.mark.parametrize("seed,periodic", [(61, 1), (62, 1), (63, 0)])
def test_gpu_detect_matches_oracle(oracle, seed, periodic):
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder
    par = S.default_params(periodic=periodic)
    r = random_state(seed)
    want = oracle.merge_detect(par, r["list_off"], r["pos"], r["vel"], r["mass"], r["nbound"],
                               r["host"], r["mostbound_pos"], r["mostbound_vel"], 9, r["sink"])
    with Unbinder(par) as ub:
        got = ub.merge_detect(r, r["list_off"], r["nbound"], r["host"], r["mostbound_pos"],
                              r["mostbound_vel"], 9, r["sink"])
    for a, b in zip(got[:3], want[:3]):
        assert np.array_equal(a, b)
    for cg, cw in zip(got[3], want[3]):
        for k in ("pos", "vel", "sigma_r", "sigma_v"):
            assert np.array_equal(np.float32(cg[k]).view(np.uint32),
                                  np.float32(cw[k]).view(np.uint32)), k
    newly = int((want[1] >= 0).sum())
    assert newly > 50 and want[2].sum() > 20  # traps and merged hosts did occur


@pytest.mark.gpu
def test_gpu_merge_matches_reference():
    par, st, ref, isnap, relax = load()
    from hbtplus_gb300.merge import merge_subhalos
    from hbtplus_gb300.unbind import Unbinder
    with Unbinder(par, precision=1) as ub:  # the FP64 walk: the reference's bound sets
        out = merge_subhalos(ub, st, isnap, relax)
    check_against_reference(out, st, ref, lambda s: out["energy"][s])


@pytest.mark.gpu
def test_gpu_detect_refuses_a_cycle():
    from hbtplus_gb300 import _lib
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder
    r = random_state(64, nsub=50)
    r["host"][:] = -1
    r["host"][10], r["host"][11], r["host"][12] = 11, 12, 10
    r["sink"][:] = -1
    r["mostbound_pos"][10:13] += 50.0  # far from every core: the walk goes round
    with Unbinder(S.default_params()) as ub:
        with pytest.raises(_lib.HBTUError):
            ub.merge_detect(r, r["list_off"], r["nbound"], r["host"], r["mostbound_pos"],
                            r["mostbound_vel"], 9, r["sink"])
