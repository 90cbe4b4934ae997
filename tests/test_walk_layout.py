"""The FP32 walk over the sibling-block node records (walk_layout 1, the
default; used for passes whose trees hold at least 2^16 particles in all)
visits the same nodes in the same order as the walk over the preorder
records (walk_layout 0), so every output of the unbinding is the same bit
for bit: orders, energies, results, interaction counts.  Batches with
subhaloes on box faces, a large single subhalo at two opening angles, and
the energies-only entry (hbtu_binding_energies) with potentials."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(params, batch, layout, precision=0):
    from hbtplus_gb300.unbind import Unbinder
    with Unbinder(params, precision=precision) as ub:
        ub.set_option("walk_layout", layout)
        assert ub.get_option("walk_layout") == layout
        return ub.unbind_batch(batch, check_status=False)


def same(a, b):
    oa, ea, ra = a
    ob, eb, rb = b
    assert np.array_equal(oa, ob)
    assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32))
    for x, y in zip(ra, rb):
        for k in x:
            assert np.array_equal(np.asarray(x[k]), np.asarray(y[k])), k


@pytest.mark.parametrize("seed", [71, 72])
def test_batch_layouts_agree(seed):
    from hbtplus_gb300 import synthetic as S
    b = S.subhalo_batch(nsub=1200, seed=seed)  # above 2^17 particles in all
    assert b["offsets"][-1] >= 1 << 17
    p = S.default_params()
    same(run(p, b, 1), run(p, b, 0))


def test_single_subhalo_and_theta_layouts_agree():
    from hbtplus_gb300 import synthetic as S
    b = S.concat([S.single_subhalo(n=200_000, seed=73)])
    for theta in (0.45, 0.7):
        p = S.default_params(open_angle=theta)
        same(run(p, b, 1), run(p, b, 0))


def test_binding_energies_layouts_agree():
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder
    sub = S.single_subhalo(n=200_000, seed=74)
    p = S.default_params()
    out = []
    for layout in (1, 0):
        with Unbinder(p) as ub:
            ub.set_option("walk_layout", layout)
            out.append(ub.binding_energies(sub["pos"], sub["vel"], sub["mass"], sub["ref_pos"],
                                           sub["ref_vel"]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
