"""The headline workload at full size: the 2000-subhalo batch (sizes from
dN/dlnN ~ N^-0.9 on [20, 2e5], NFW + Jeans velocities, 20% contaminants,
100 Mpc/h periodic box, 867,289 particles) unbound in one hbtu_unbind_batch
call and compared, subhalo by subhalo, with the C oracle's halo-parallel
Unbind of the same batch (src/subhalo_unbind.cpp:263-431, :495-503).

Two settings of MaxSampleSizeOfPotentialEstimate:
  0     the exact tree (the benchmark's setting);
  1000  the reference's production default: every subhalo above 1000
        particles is first shuffled with the reference's random_shuffle
        (src/subhalo_unbind.cpp:302), both sides get the shuffled particles,
        the tree is built over a 1000-particle sample with scaled masses and
        RefineBindingEnergyOrder reorders the first 1000 bound particles.

Cells below TreeNodeResolution are split by the reference into random
octants with its process-global drand48 stream (src/oct_tree.tpp:112-123) and
kept whole here.  The oracle counts those draws per subhalo (random_splits);
with the batch unbound on many threads, which numbers a subhalo draws depends
on thread timing, so such a subhalo's reference tree changes from run to run.

Subhaloes where the reference split a cell at random (both modes): that
reference tree is one random draw, and this library keeps the cell whole, so
the two trees approximate the same potential differently, at the level of the
tree's own error (up to 1e-4 * max|E| seen: subhalo 446, 78 particles, one
draw).  For them a particle may change side only if |E| <= 1e-3 * max|E_bound|,
Nbound may differ only by the particles that changed side, and the energies of
particles bound in both agree within 1e-3 * max|E_bound|.  The test counts
them.

Every other subhalo:
  FP32 mode: a particle may change side only if its energy lies in the band
    |E| <= 1e-5 * max|E_bound|; Mbound within 1e-5 relative plus one particle
    mass per changed particle; bound energies within 2e-6 * max|E_bound|
    (subhaloes where no particle changed side); iteration counts exact;
    interaction counts within 1e-6 relative (the walk takes the reference's
    opening decision in double near the threshold, but on float coordinates
    relative to the frame, which are exact except near the frame's origin: a
    decision within ~1e-7 of the threshold can then flip); the same
    most-bound particle unless the reference's two lowest energies lie within
    2e-6 * max|E_bound| of each other.
  FP64 mode: Nbound, Mbound, iterations, frames and bound energies bit for
    bit, the order up to runs of equal energy.
"""
import numpy as np
import pytest

from helpers import tie_groups_equal

pytestmark = pytest.mark.gpu

BAND = 1e-5
EREL = 2e-6
TREE_TOL = 1e-3  # the theta = 0.45 tree's own approximation level


@pytest.fixture(scope="module")
def batch():
    from hbtplus_gb300 import synthetic as S
    return S.subhalo_batch(nsub=2000, seed=20261204)


@pytest.fixture(scope="module")
def orc():
    from oracle import Oracle
    return Oracle()


def shuffled(batch, orc, max_sample):
    """The batch with every subhalo above max_sample particles permuted by the
    reference's random_shuffle (seeded per subhalo); mostbound_id keeps the Id
    that was at position 0 before the shuffle."""
    out = {k: np.array(v, copy=True) for k, v in batch.items()}
    off = batch["offsets"]
    for s in range(len(off) - 1):
        o0, o1 = int(off[s]), int(off[s + 1])
        if o1 - o0 > max_sample:
            perm = o0 + orc.reference_shuffle(o1 - o0, 1000 + s)
            for k in ("id", "pos", "vel", "mass", "type"):
                out[k][o0:o1] = batch[k][perm]
    return out


def refined_energies(orc, p, b, a, orf, nbr, r, max_sample):
    """Energies RefineBindingEnergyOrder sorts by (src/subhalo_unbind.cpp:234-262):
    a tree over the first min(Nbound, MaxSample) bound particles of the
    reference's order, their own masses, the final frame."""
    k = min(nbr, max_sample)
    idx = a + orf[:k]
    e, _, _ = orc.binding_energies(dict(p, max_sample_size=0), b["pos"][idx], b["vel"][idx],
                                   b["mass"][idx], r["ref_pos"], r["ref_vel"])
    return e


def split_checks(batch, a, b, g, r, og, orf, eg, erf, tag):
    """A subhalo in which the reference split a sub-resolution cell into random
    octants: its reference tree is one random draw among many, and this
    library keeps the cell whole, so the two trees approximate the same
    potential differently, at the level of the tree's own error (measured up to
    1e-4 * max|E|).  Required: a particle changes side only if |E| <= TREE_TOL *
    max|E_bound|, Nbound differs by at most the particles that changed side,
    and the energies of particles bound in both within TREE_TOL * max|E_bound|."""
    n = b - a
    nb, nbr = int(g["nbound"]), int(r["nbound"])
    if bool(g["disrupted"]) != bool(r["disrupted"]) or n <= 1:
        return
    emax = float(np.max(np.abs(erf[:nbr]))) if nbr else 1.0
    e_ref = np.full(n, np.nan)
    e_ref[orf] = erf
    e_got = np.full(n, np.nan)
    e_got[og] = eg
    mg = np.zeros(n, bool)
    mr = np.zeros(n, bool)
    mg[og[:nb]] = True
    mr[orf[:nbr]] = True
    diff = np.nonzero(mg ^ mr)[0]
    e_side = np.where(np.isnan(e_ref[diff]), e_got[diff], e_ref[diff])
    assert np.all(np.abs(e_side) <= TREE_TOL * emax), f"{tag}: a particle changed side outside the band"
    assert abs(nb - nbr) <= len(diff), tag
    both = mg & mr
    if both.any():
        assert np.max(np.abs(e_got[both] - e_ref[both])) <= TREE_TOL * emax, tag


def compare(batch, got, ref, exact, orc=None, p=None, counts=None):
    """Per-subhalo comparison; returns (particles changed side, subhaloes with
    cells split at random)."""
    max_sample = int(p["max_sample_size"]) if p else 0
    order, energy, res = got
    o_ref, e_ref, r_ref = ref
    off = batch["offsets"]
    changed = 0
    inexact = 0
    if counts is not None:
        counts.clear()
    for s in range(len(off) - 1):
        a, b = int(off[s]), int(off[s + 1])
        n = b - a
        g, r = res[s], r_ref[s]
        tag = f"subhalo {s} (n={n})"
        nb, nbr = int(g["nbound"]), int(r["nbound"])
        og, orf = order[a:b], o_ref[a:b]
        eg, erf = energy[a:b], e_ref[a:b]
        if int(r["random_splits"]) > 0:  # the reference split a cell at random
            split_checks(batch, a, b, g, r, og, orf, eg, erf, tag)
            inexact += 1
            continue
        assert g["disrupted"] == r["disrupted"], tag
        assert g["iterations"] == r["iterations"], tag
        if g["disrupted"] or n <= 1:
            assert nb == nbr and og[0] == orf[0], tag
            continue
        emax = float(np.max(np.abs(erf[:nbr]))) if nbr else 1.0
        if exact:
            assert nb == nbr, tag
            assert g["mbound"] == r["mbound"], tag
            np.testing.assert_array_equal(g["ref_pos"], r["ref_pos"], err_msg=tag)
            np.testing.assert_array_equal(g["ref_vel"], r["ref_vel"], err_msg=tag)
            same = eg[:nb] == erf[:nb]
            if same.all() and g["interactions"] == r["interactions"]:
                if not np.array_equal(og, orf):
                    k = min(nbr, max_sample) if max_sample and nbr > max_sample else 0
                    if k:  # the refined prefix is ordered by the refined energies
                        er = refined_energies(orc, p, batch, a, orf, nbr, r, max_sample)
                        assert tie_groups_equal(og[:k], orf[:k], er), tag
                    assert tie_groups_equal(og[k:], orf[k:], eg[k:]), tag
            else:
                raise AssertionError(f"{tag}: not exact, and the reference drew no random octant")
            continue
        if g["interactions"] != r["interactions"]:
            assert abs(g["interactions"] - r["interactions"]) <= 1e-6 * r["interactions"], tag
            if counts is not None:
                counts.append((s, n, int(g["interactions"] - r["interactions"])))
        mg = np.zeros(n, bool)
        mr = np.zeros(n, bool)
        mg[og[:nb]] = True
        mr[orf[:nbr]] = True
        diff = np.nonzero(mg ^ mr)[0]
        e_of = np.empty(n, np.float64)
        e_of[og] = eg
        e_of[orf[:nbr]] = erf[:nbr]  # the reference's energy where it holds one
        outside = diff[np.abs(e_of[diff]) > BAND * emax]
        assert len(outside) == 0, f"{tag}: {len(outside)} particles changed side outside the band"
        mass = batch["mass"][a:b]
        assert abs(g["mbound"] - r["mbound"]) <= \
            1e-5 * r["mbound"] + float(np.max(mass)) * len(diff) + 1e-12, tag
        changed += len(diff)
        if len(diff) == 0 and nb:
            e_ref_pid = np.empty(n, np.float64)
            e_ref_pid[orf[:nbr]] = erf[:nbr]
            assert np.max(np.abs(eg[:nb] - e_ref_pid[og[:nb]])) <= EREL * emax, tag
            if og[0] != orf[0]:
                if max_sample and nbr > max_sample:  # ordered by the refined energies
                    er = refined_energies(orc, p, batch, a, orf, nbr, r, max_sample)
                    pos = int(np.nonzero(orf[:len(er)] == og[0])[0][0])
                    assert er[pos] - er[0] <= EREL * float(np.max(np.abs(er))), tag
                else:
                    assert nbr > 1 and erf[1] - erf[0] <= EREL * emax, \
                        f"{tag}: most-bound particle"
    return changed, inexact


@pytest.mark.parametrize("max_sample", [0, 1000])
def test_full_batch_against_oracle(batch, orc, max_sample):
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import Unbinder
    b = shuffled(batch, orc, max_sample) if max_sample else batch
    assert int(b["offsets"][-1]) == 867_289 and len(b["offsets"]) == 2001
    p = S.default_params(max_sample_size=max_sample)
    ref = orc.unbind_batch(p, b, nthreads=0)
    for precision in (0, 1):
        with Unbinder(p, precision=precision) as ub:
            got = ub.unbind_batch(b)
        counts = []
        changed, inexact = compare(b, got, ref, exact=precision == 1, orc=orc, p=p,
                                   counts=counts)
        nbound = sum(int(r["nbound"]) for r in got[2])
        print(f"max_sample {max_sample} precision {'fp64' if precision else 'fp32'}: "
              f"nbound {nbound}, {changed} particles changed side (all inside the band), "
              f"{inexact} subhaloes with cells split at random (checked at the tree's "
              f"error level), interaction counts not exact in {len(counts)} other "
              f"subhaloes (subhalo, n, difference): {counts[:10]}")
        assert inexact <= (len(b["offsets"]) - 1) // 10  # the rest is checked strictly
        # size-independent properties of the outputs
        order, energy, res = got
        off = b["offsets"]
        for s in range(len(off) - 1):
            o0, o1 = int(off[s]), int(off[s + 1])
            assert np.array_equal(np.sort(order[o0:o1]), np.arange(o1 - o0))
