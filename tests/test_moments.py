"""The tree's cell moments at the sizes where their work is split differently:
a subtree of at most 256 particles is computed in a batch of such subtrees,
one of 257..2048 alone, and cells holding more than 2048 particles climb by
countdown above them (csrc/tree.cu).  First-pass potentials of single
subhaloes on both sides of each boundary, in FP64 mode, equal the C oracle's
(the reference's OctTree_t::Build + ProcessNode + the walk,
src/oct_tree.tpp:16-144, src/gravity_tree.cpp:18-161) bit for bit; FP32 mode
within 1e-6 of the largest term summed: |phi| + G m / (a eps), since the FP32
walk sums each particle's own softened term in float and cancels it in double,
which dominates the error of a few-particle subhalo whose potential is much
smaller than that term.  The particles are a uniform cloud plus a concentrated core, with
no pair closer than the tree resolution (so the reference draws no random
octant)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [2, 3, 20, 255, 256, 257, 2047, 2048, 2049, 4096, 5000, 70_000]


def cloud(n, seed):
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(seed))
    core = n // 3
    pos = np.concatenate([rng.uniform(-1.0, 1.0, (n - core, 3)),
                          rng.normal(0.0, 0.08, (core, 3))]) + 50.0
    vel = rng.normal(0.0, 100.0, (n, 3))
    mass = np.full(n, 1e-4)
    mass[rng.choice(n, n // 10, replace=False)] = 3e-4
    # keep only points farther than 1e-3 from every other (the resolution is 2e-4)
    if n > 1:
        from scipy.spatial import cKDTree
        tree = cKDTree(pos)
        pairs = tree.query_pairs(1e-3, output_type="ndarray")
        drop = np.unique(pairs[:, 1]) if len(pairs) else np.zeros(0, int)
        for k in drop:  # move each close point somewhere empty
            pos[k] = 50.0 + rng.uniform(-1.0, 1.0, 3)
        assert len(cKDTree(pos).query_pairs(1e-3)) == 0
    p = S.default_params()
    return p, pos.astype(np.float32), vel.astype(np.float32), mass.astype(np.float32)


@pytest.mark.parametrize("n", SIZES)
def test_first_pass_potentials_across_chunk_sizes(n):
    pytest.importorskip("scipy")
    from hbtplus_gb300.unbind import Unbinder
    from oracle import Oracle
    p, pos, vel, mass = cloud(n, 500 + n)
    rp = pos.mean(axis=0)
    rv = vel.mean(axis=0)
    E_ref, pot_ref, _ = Oracle().binding_energies(p, pos, vel, mass, rp, rv)
    with Unbinder(p, precision=1) as ub:
        E, pot = ub.binding_energies(pos, vel, mass, rp, rv)
    np.testing.assert_array_equal(pot, pot_ref)
    np.testing.assert_array_equal(E, E_ref)
    with Unbinder(p, precision=0) as ub:
        E, pot = ub.binding_energies(pos, vel, mass, rp, rv)
    self_term = p["G"] / p["scale_factor"] * mass.astype(np.float64) / p["softening"]
    scale = np.abs(pot_ref) + self_term
    assert np.max(np.abs(pot - pot_ref) / scale) < 1e-6
