"""The per-subhalo loop (small.cu): once every active subhalo of a call has
at most small_cutoff particles in its energy list, one persistent launch
finishes them all, one thread block running a subhalo's remaining passes.

It runs the batch kernels' own per-element steps, so its outputs must equal
the batch path's bit for bit (option small_cutoff = 0 turns it off): order,
energies and every result field, in both walk precisions, with disruptions,
correction passes, a pass cap, a non-periodic box and sampled potentials.  It
is also checked directly against the reference: every golden fixture in FP64
mode, bit for bit, with the hand-over at its earliest (a subhalo of up to 2048
particles runs every pass in it).
"""
import numpy as np
import pytest

from helpers import SINGLE_CASES, load_case

pytestmark = pytest.mark.gpu


def _run(par, batch, cutoff, precision=0, max_passes=0):
    from hbtplus_gb300.unbind import Unbinder
    with Unbinder(par, precision=precision, max_passes=max_passes) as ub:
        ub.set_option("small_cutoff", cutoff)
        ub.reset_stats()
        out = ub.unbind_batch(batch, check_status=False)
        st = ub.stats()
    return out, st


def _same(a, b, tag, offsets=None):
    oa, ea, ra = a
    ob, eb, rb = b
    bad = []
    for s, (x, y) in enumerate(zip(ra, rb)):
        fields = [k for k in x if not np.array_equal(np.asarray(x[k]), np.asarray(y[k]))]
        if offsets is not None:
            o0, o1 = int(offsets[s]), int(offsets[s + 1])
            if not np.array_equal(oa[o0:o1], ob[o0:o1]):
                fields.append("order")
            if not np.array_equal(ea[o0:o1], eb[o0:o1], equal_nan=True):
                fields.append("energy")
        if fields:
            n = None if offsets is None else int(offsets[s + 1] - offsets[s])
            bad.append((s, n, int(x["iterations"]), int(y["iterations"]), fields))
    assert not bad, f"{tag}: {len(bad)} subhaloes differ (index, n, passes, fields): {bad[:8]}"
    assert np.array_equal(oa, ob), tag
    assert np.array_equal(ea, eb, equal_nan=True), tag


def _mixed_batch(seed, nsub=240, nmax=3000):
    from hbtplus_gb300 import synthetic as S
    return S.subhalo_batch(nsub=nsub, seed=seed, nmax=nmax)


@pytest.mark.parametrize("precision,max_sample", [(0, 0), (1, 0), (0, 300)])
def test_small_path_equals_batch_path(precision, max_sample):
    from hbtplus_gb300 import synthetic as S
    b = _mixed_batch(31 + precision)
    p = S.default_params(max_sample_size=max_sample)
    ref, st0 = _run(p, b, 0, precision)
    assert st0["small_subhaloes"] == 0
    for cutoff in (256, 2048):
        got, st = _run(p, b, cutoff, precision)
        assert st["small_subhaloes"] > 0
        _same(got, ref, f"precision {precision} cutoff {cutoff}", b["offsets"])
    # only small subhaloes: the hand-over comes at the first round
    n = np.diff(b["offsets"])
    keep = np.nonzero(n <= 2048)[0]
    small = {k: b[k] for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel",
                               "mostbound_id")}
    small = {k: np.asarray(v)[keep] for k, v in small.items()}
    rows = np.concatenate([np.arange(b["offsets"][s], b["offsets"][s + 1]) for s in keep])
    for k in ("id", "pos", "vel", "mass", "type"):
        small[k] = np.asarray(b[k])[rows]
    small["offsets"] = np.concatenate([[0], np.cumsum(n[keep])]).astype(np.int64)
    ref, _ = _run(p, small, 0, precision)
    got, st = _run(p, small, 2048, precision)
    assert st["small_subhaloes"] == int(np.sum(n[keep] >= 2))
    assert st["passes"] == 0
    _same(got, ref, f"precision {precision}: small subhaloes only", small["offsets"])


def test_small_path_edge_cases():
    """Tiny and disrupted subhaloes, a pass cap, no periodic box."""
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(77))
    subs = [S.nfw_subhalo(rng, n, 0.01 * (1 + n / 500), 10.0, contaminant_frac=f,
                          center=rng.uniform(0, 100, 3))
            for n, f in ((0, 0.0), (1, 0.0), (2, 0.0), (3, 0.0), (19, 0.0), (20, 0.5),
                         (21, 0.9), (64, 0.3), (300, 0.6), (900, 0.4), (2048, 0.3))]
    S._assign_ids(rng, subs)
    b = S.concat(subs)
    for par in (S.default_params(), S.default_params(periodic=0),
                S.default_params(min_num_part=100)):
        for max_passes in (0, 1, 2):
            ref, _ = _run(par, b, 0, 0, max_passes)
            got, _ = _run(par, b, 2048, 0, max_passes)
            _same(got, ref, f"periodic {par['periodic']} minpart {par['min_num_part']} "
                            f"max_passes {max_passes}", b["offsets"])


@pytest.mark.parametrize("case", SINGLE_CASES)
def test_small_path_fp64_golden(case):
    """The reference's own Unbind outputs, bit for bit, with the per-subhalo
    loop taking over as early as it can (FP64 mode): a golden subhalo of
    2..2048 particles runs every pass in it, a larger one its last passes
    once its list is that short."""
    from hbtplus_gb300.unbind import Unbinder
    from test_gpu_parity import check_exact
    par, inp, ref = load_case(case)
    n = len(inp["mass"])
    with Unbinder(par, precision=1) as ub:
        ub.set_option("small_cutoff", 2048)
        ub.reset_stats()
        order, energy, res = ub.unbind(inp)
        if 2 <= n <= 2048:
            assert ub.stats()["small_subhaloes"] == 1 and ub.stats()["passes"] == 0
    check_exact(res, order, energy, ref, case, n)
