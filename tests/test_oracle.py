"""The CPU oracle (C restatement of Subhalo_t::Unbind) against the golden
vectors produced by the reference itself, and its partition against the
closed form used on the GPU.  CPU only."""
import os

import numpy as np
import pytest

from helpers import FIRST_PASS_CASES, SINGLE_CASES, load_case, partition_emulation, tie_groups_equal
from oracle import REF_SO, Oracle

RESULT_EXACT = ("nbound", "mbound", "ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel",
                "specific_potential", "specific_kinetic", "specific_angmom", "nbound_type",
                "mbound_type", "disrupted", "converged", "too_few")


@pytest.fixture(scope="module")
def orc():
    return Oracle()


@pytest.mark.parametrize("case", SINGLE_CASES)
def test_oracle_matches_reference_golden(orc, case):
    par, inp, ref = load_case(case)
    order, energy, res = orc.unbind(par, inp, nthreads=1, drand_seed=int(ref["drand_seed"]))
    nb = int(ref["nbound"])
    for k in RESULT_EXACT:
        if len(inp["mass"]) <= 1 and k.startswith("specific"):
            continue  # the reference returns before writing these (subhalo_unbind.cpp:284-293)
        np.testing.assert_array_equal(np.asarray(res[k]), ref[k], err_msg=f"{case}: {k}")
    np.testing.assert_array_equal(energy[:nb], ref["energy"][:nb])
    assert tie_groups_equal(order, ref["order"], energy if res["converged"] else np.arange(len(order)))


@pytest.mark.parametrize("case", FIRST_PASS_CASES)
def test_oracle_first_pass_golden(orc, case):
    par, inp, ref = load_case(case)
    E, pot, nint = orc.binding_energies(par, inp["pos"], inp["vel"], inp["mass"], inp["ref_pos"],
                                        inp["ref_vel"], nthreads=1)
    np.testing.assert_array_equal(E, ref["energy"])
    np.testing.assert_array_equal(pot, ref["potential"])
    assert nint > len(E)


@pytest.mark.parametrize("case", FIRST_PASS_CASES)
def test_oracle_tree_potentials_golden(orc, case):
    """The targeted form (one tree, chosen targets, several opening angles) gives
    the reference's first-pass potentials at the fixture's angle, and the full
    first-pass walk's potentials at the others."""
    par, inp, ref = load_case(case)
    rng = np.random.default_rng(3)
    t = np.sort(rng.choice(len(inp["mass"]), 300, replace=False))
    thetas = (0.3, par["open_angle"], 0.7)
    pot, cnt = orc.tree_potentials(par, inp["pos"], inp["mass"], t, thetas, nthreads=2)
    np.testing.assert_array_equal(pot[1], ref["potential"][t])
    for k in (0, 2):
        _, full, _ = orc.binding_energies(dict(par, open_angle=thetas[k]), inp["pos"], inp["vel"],
                                          inp["mass"], inp["ref_pos"], inp["ref_vel"], nthreads=1)
        np.testing.assert_array_equal(pot[k], full[t])
    assert cnt[0] > cnt[1] > cnt[2] > 0


def test_oracle_batch_golden(orc):
    par, inp, ref = load_case("batch_48")
    order, energy, res = orc.unbind_batch(par, inp, nthreads=4)
    off = inp["offsets"]
    for s in range(len(off) - 1):
        a, b = off[s], off[s + 1]
        for k in ("nbound", "mbound", "ref_pos", "ref_vel", "disrupted"):
            np.testing.assert_array_equal(np.asarray(res[s][k]), ref[k][s], err_msg=f"sub {s} {k}")
        nb = res[s]["nbound"]
        np.testing.assert_array_equal(energy[a:a + nb], ref["energy"][a:a + nb])
        if res[s]["converged"]:
            assert tie_groups_equal(order[a:b], ref["order"][a:b], energy[a:b])


def test_partition_closed_form_matches_reference_algorithm(orc):
    rng = np.random.default_rng(5)
    for trial in range(3000):
        n = int(rng.integers(0, 40))
        E = rng.choice(np.array([-1.0, 1.0, 0.0], np.float32), size=n,
                       p=[0.55, 0.4, 0.05]).astype(np.float32) * rng.uniform(0.5, 2, n).astype(np.float32)
        nb, Eo, idx = orc.partition(E)
        nb2, src = partition_emulation(E)
        assert nb == nb2, (E, nb, nb2)
        np.testing.assert_array_equal(idx, src)


def test_shuffle_helper_is_a_permutation(orc):
    perm = orc.reference_shuffle(1000, 7)
    assert sorted(perm.tolist()) == list(range(1000))
    assert not np.array_equal(perm, np.arange(1000))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference build (oracle/_ref) not present")
def test_oracle_matches_reference_random_inputs(orc):
    from hbtplus_gb300 import synthetic as S
    ref = Oracle(reference=True)
    for seed in range(3):
        rng = np.random.Generator(np.random.PCG64(900 + seed))
        n = int(rng.integers(50, 1500))
        sub = S.nfw_subhalo(rng, n, 0.2 * (n / 1e5) ** (1 / 3), rng.uniform(5, 20),
                            contaminant_frac=0.2)
        S._assign_ids(rng, [sub])
        p = S.default_params(open_angle=float(rng.choice([0.3, 0.45, 0.7])))
        o1, e1, r1 = orc.unbind(p, sub, nthreads=1)
        o2, e2, r2 = ref.unbind(p, sub, nthreads=1)
        nb = r1["nbound"]
        assert nb == r2["nbound"]
        np.testing.assert_array_equal(e1[:nb], e2[:nb])
        assert r1["mbound"] == r2["mbound"]
        if r1["converged"]:
            assert tie_groups_equal(o1, o2, e1)


def test_oracle_counts_random_octant_draws(orc):
    """random_splits counts the drand48 draws of a subhalo's unbinding: none for
    a cloud with no pair closer than the tree resolution (0.1 softening), some
    for every seed when particles sit closer than it (src/oct_tree.tpp:112-123;
    how many depends on where the earlier draws put the particles)."""
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(91))
    p = S.default_params()
    n = 400
    sub = dict(pos=(50.0 + rng.uniform(-0.5, 0.5, (n, 3))).astype(np.float32),
               vel=rng.normal(0.0, 5.0, (n, 3)).astype(np.float32),
               mass=np.full(n, 1e-3, np.float32), id=np.arange(n, dtype=np.int64),
               type=np.ones(n, np.int32), ref_pos=np.full(3, 50.0, np.float32),
               ref_vel=np.zeros(3, np.float32), mostbound_pos=np.full(3, 50.0, np.float32),
               mostbound_vel=np.zeros(3, np.float32), mostbound_id=0)
    d = np.linalg.norm(sub["pos"][:, None, :].astype(np.float64) - sub["pos"][None, :, :], axis=2)
    assert np.min(d + np.eye(n)) > 1e-3
    _, _, res = orc.unbind(p, sub, nthreads=1)
    assert res["random_splits"] == 0
    close = dict(sub)
    close["pos"] = sub["pos"].copy()
    close["pos"][1:6] = close["pos"][0] + np.float32(1e-5) * np.arange(1, 6, dtype=np.float32)[:, None]
    for seed in (1, 2, 3):
        assert orc.unbind(p, close, nthreads=1, drand_seed=seed)[2]["random_splits"] > 0
