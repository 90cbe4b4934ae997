"""Nested unbinding (hbtplus_gb300.refine): RecursiveUnbind + TruncateSource
over a forest of subhaloes, one GPU batch per nesting depth.

CPU: a literal depth-first restatement on the C oracle's Unbind
(helpers.recursive_unbind_oracle) reproduces the reference's own
RecursiveUnbind (tests/golden/forest_10.npz: two haloes with satellites three
deep, an orphan with a satellite, a satellite that disrupts, a field
subhalo): the final lists and Nbound.
GPU: the depth-batched GPU version gives the same lists and Nbound (FP64 mode
bit for bit; FP32 mode too on this forest), and matches the restatement on
random forests."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, recursive_unbind_oracle


def golden_forest():
    z = dict(np.load(os.path.join(GOLDEN, "forest_10.npz")))
    forest = {k[3:]: v for k, v in z.items() if k.startswith("in_")}
    params = {k[4:]: v.item() for k, v in z.items() if k.startswith("par_")}
    return forest, params, z


def test_oracle_restatement_matches_reference_forest():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "oracle"))
    from oracle import Oracle
    forest, params, z = golden_forest()
    off, pos, nbound = recursive_unbind_oracle(Oracle(), params, forest, float(z["relax"]))
    assert np.array_equal(nbound, z["ref_nbound"])
    assert np.array_equal(off, z["ref_off"])
    assert np.array_equal(pos, z["ref_pos_out"])


def test_depth_and_source_size():
    from hbtplus_gb300.refine import nesting_depth, source_size
    forest, _, _ = golden_forest()
    d = nesting_depth(len(forest["list_off"]) - 1, forest["nest_off"], forest["nest_idx"],
                      forest["roots"])
    assert list(d) == [0, 1, 2, 3, 1, 2, 1, 0, 1, 0]
    assert source_size(1, 10, 3.0) == 1 and source_size(0, 10, 3.0) == 0
    assert source_size(5, 100, 3.0) == 15 and source_size(5, 12, 3.0) == 12
    assert source_size(16777217, 10**9, 1.0) == 16777216  # float product, as the reference


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [1, 0])
def test_gpu_forest_matches_reference(precision):
    from hbtplus_gb300.refine import recursive_unbind
    from hbtplus_gb300.unbind import Unbinder
    forest, params, z = golden_forest()
    with Unbinder(params, precision=precision) as ub:
        out = recursive_unbind(ub, forest, forest["list_off"], forest["nbound_prev"],
                               forest["nest_off"], forest["nest_idx"], forest["roots"], forest,
                               relax=float(z["relax"]))
    assert [r["nbound"] for r in out["results"]] == list(z["ref_nbound"])
    assert np.array_equal(out["off"], z["ref_off"])
    assert np.array_equal(out["pos"], z["ref_pos_out"])


@pytest.mark.gpu
def test_gpu_random_forests_match_restatement():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "oracle"))
    from oracle import Oracle
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.refine import recursive_unbind
    from hbtplus_gb300.unbind import Unbinder
    sys.path.insert(0, GOLDEN)
    from make_golden import forest_case
    orc = Oracle()
    p = S.default_params()
    for seed in (201, 202, 203):
        forest = forest_case(seed=seed, n_scale=0.5)
        off, pos, nbound = recursive_unbind_oracle(orc, p, forest)
        with Unbinder(p, precision=1) as ub:
            out = recursive_unbind(ub, forest, forest["list_off"], forest["nbound_prev"],
                                   forest["nest_off"], forest["nest_idx"], forest["roots"],
                                   forest)
        assert [r["nbound"] for r in out["results"]] == list(nbound)
        assert np.array_equal(out["off"], off) and np.array_equal(out["pos"], pos)
