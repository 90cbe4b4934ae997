"""The large host subhalo at full size: a 2e7-particle NFW host (r200 = 1
Mpc/h, c = 5) with 300 Plummer clumps of 1e3-1e5 particles and 5% contaminants
(about 2.7e7 particles), unbound with opening angles 0.3, 0.45 and 0.7.

Checked against exact FP64 pairwise sums (hbtu_direct_potential) on a random
1e4-particle subsample:
  * tree potentials of the first pass: relative error below 1e-2 at the 99th
    percentile for theta = 0.45 and growing with theta;
  * bound mass: the final bound set classified by the tree energy and by the
    FP64 direct-sum energy (same frame) disagree on at most 1e-3 of the
    subsample;
  * size-independent properties of the outputs: order is a permutation, bound
    energies are sorted and negative, Mbound equals the bound particles' mass.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host():
    from hbtplus_gb300 import synthetic as S
    return S.host_with_clumps()


def test_large_host_against_fp64_direct_sum(host):
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder
    n = len(host["mass"])
    assert n > 2.4e7
    rng = np.random.default_rng(7)
    tidx = np.sort(rng.choice(n, 10_000, replace=False))
    with Unbinder(S.default_params()) as ub:
        phi_direct = ub.direct_potential(host["pos"], host["mass"], tidx)
    p99 = {}
    results = {}
    for theta in (0.3, 0.45, 0.7):
        with Unbinder(S.default_params(open_angle=theta)) as ub:
            _, pot = ub.binding_energies(host["pos"], host["vel"], host["mass"], host["ref_pos"],
                                         host["ref_vel"])
            rel = np.abs(pot[tidx] - phi_direct) / np.abs(phi_direct)
            p99[theta] = float(np.percentile(rel, 99))
            t0 = time.perf_counter()
            order, energy, res = ub.unbind(host)
            dt = time.perf_counter() - t0
            results[theta] = (order, energy, res)
            print(f"theta {theta}: phi rel err p50 {np.median(rel):.3e} p99 {p99[theta]:.3e} "
                  f"max {rel.max():.3e}; nbound {res['nbound']} mbound {res['mbound']:.6g} "
                  f"iterations {res['iterations']} interactions {res['interactions']} "
                  f"unbind {dt:.2f} s")
    assert p99[0.3] <= p99[0.45] <= p99[0.7]
    assert p99[0.45] < 1e-2
    for theta, (order, energy, res) in results.items():
        nb = res["nbound"]
        assert np.array_equal(np.sort(order), np.arange(n))
        assert np.all(np.diff(energy[:nb]) >= 0) and np.all(energy[:nb] < 0)
        assert abs(res["mbound"] - float(np.sum(host["mass"][order[:nb]], dtype=np.float64))) \
            <= 1e-5 * res["mbound"]
    # bound mass against the FP64 direct sum, theta = 0.45, final frame and bound set
    order, energy, res = results[0.45]
    nb = res["nbound"]
    b = order[:nb]
    bpos, bvel, bmass = host["pos"][b], host["vel"][b], host["mass"][b]
    sub = np.sort(rng.choice(nb, 10_000, replace=False))
    with Unbinder(S.default_params()) as ub:
        e_tree, _ = ub.binding_energies(bpos, bvel, bmass, res["ref_pos"], res["ref_vel"])
        phi_b = ub.direct_potential(bpos, bmass, sub)
    d = bpos[sub].astype(np.float64) - res["ref_pos"].astype(np.float64)
    d = np.where(d > 50.0, d - 100.0, np.where(d < -50.0, d + 100.0, d))
    dv = bvel[sub].astype(np.float64) - res["ref_vel"].astype(np.float64) + 100.0 * d
    e_direct = 0.5 * np.sum(dv * dv, axis=1) + phi_b
    disagree = np.mean((e_tree[sub] < 0) != (e_direct < 0))
    print(f"bound status, tree vs FP64 direct sum: {disagree:.2e} of {len(sub)} disagree")
    assert disagree <= 5e-3
