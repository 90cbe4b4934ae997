"""Generate the golden fixtures of the unbinding path from the reference itself.

Run here, where the reference sources are available:
    python tests/golden/make_golden.py
It builds oracle/_ref/libhbt_ref.so (the reference's own Subhalo_t::Unbind,
compiled from its unmodified sources by oracle/Makefile) and writes one
compressed .npz per case into tests/golden/.  Each file holds the inputs
(particles in the order Unbind receives them, frame, parameters) and the
reference's outputs (permuted particle order as input indices, Energies,
Nbound, Mbound, frames, kinematics, per-type counts); `first_pass_*` cases hold
the reference tree's BindingEnergy/EvaluatePotential of every particle;
`index_*` cases hold the reference's particle-ID tables and their lookups
(`python tests/golden/make_golden.py index` writes only those); `forest_10`
holds the reference's RecursiveUnbind + TruncateSource over a forest of nested
subhaloes (`... forest`); `props_*` batches hold each subhalo's Unbind followed
by the reference's CalculateProfileProperties and CalculateShape (`... props`).

For sampled cases the stored particles are the ones AFTER the reference's
random_shuffle (what the GPU library and the C oracle take), with
mostbound_id naming the particle that was at position 0 before it.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from hbtplus_gb300 import synthetic as S  # noqa: E402
from oracle import Oracle  # noqa: E402

RESULT_KEYS = ("nbound", "mbound", "ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel",
               "specific_potential", "specific_kinetic", "specific_angmom", "nbound_type",
               "mbound_type", "disrupted", "converged", "too_few")


def scaled(n, seed, c=10.0, cf=0.1, center=None, bulk=(0.0, 0.0, 0.0)):
    rng = np.random.Generator(np.random.PCG64(seed))
    r200 = 0.2 * (n / 1e5) ** (1.0 / 3.0)
    sub = S.nfw_subhalo(rng, n, r200, c, contaminant_frac=cf, center=center,
                        bulk_velocity=bulk)
    S._assign_ids(rng, [sub])
    return sub


def save(name, params, sub, ref, shuffle_seed=0, drand_seed=1):
    order, energy, res = ref.unbind(params, sub, nthreads=1, shuffle_seed=shuffle_seed,
                                    drand_seed=drand_seed)
    out = dict(sub)
    if params["max_sample_size"] > 0 and len(sub["mass"]) > params["max_sample_size"]:
        # store the post-shuffle particles, as the library takes them
        perm = ref.reference_shuffle(len(sub["mass"]), shuffle_seed)
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(perm))
        for k in ("id", "pos", "vel", "mass", "type"):
            out[k] = sub[k][perm]
        out["mostbound_id"] = int(sub["id"][0])
        order = inv[order]
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        **{f"in_{k}": np.asarray(v) for k, v in out.items()},
        **{f"par_{k}": np.asarray(v) for k, v in params.items()},
        ref_order=order, ref_energy=energy, drand_seed=drand_seed,
        **{f"ref_{k}": np.asarray(res[k]) for k in RESULT_KEYS})
    print(f"{name}: n={len(sub['mass'])} nbound={res['nbound']} disrupted={res['disrupted']}")


def save_first_pass(name, params, sub, ref):
    E, pot, _ = ref.binding_energies(params, sub["pos"], sub["vel"], sub["mass"], sub["ref_pos"],
                                     sub["ref_vel"], nthreads=1)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        **{f"in_{k}": np.asarray(v) for k, v in sub.items()},
                        **{f"par_{k}": np.asarray(v) for k, v in params.items()},
                        ref_energy=E, ref_potential=pot)
    print(f"{name}: n={len(sub['mass'])}")


def main():
    ref = Oracle(reference=True)
    p = S.default_params()
    save("nfw_1100", p, scaled(1000, 101), ref)
    save("nfw_3300_corner", p, scaled(3000, 102, c=15.0, center=(0.01, 99.99, 50.0)), ref)
    save("nfw_2200_bulk", p, scaled(2000, 103, c=6.0, bulk=(250.0, -120.0, 40.0)), ref)
    save("nfw_1650_theta07", S.default_params(open_angle=0.7), scaled(1500, 104), ref)
    save("nfw_1100_nonperiodic", S.default_params(periodic=0),
         scaled(1000, 105, center=(40.0, 50.0, 60.0)), ref)
    save("nfw_4400_sampled", S.default_params(max_sample_size=800),
         scaled(4000, 106), ref, shuffle_seed=4242)
    # a subhalo whose particles all move far too fast: disruption
    hot = scaled(200, 107)
    hot["vel"] = (hot["vel"] * 40.0).astype(np.float32)
    save("disrupt_220", p, hot, ref)
    save("tiny_5", p, scaled(5, 108, cf=0.0), ref)
    two = scaled(2, 109, cf=0.0)
    save("two_2", S.default_params(min_num_part=1), two, ref)
    save("one_1", p, scaled(1, 110, cf=0.0), ref)
    # coincident pairs below TreeNodeResolution: the reference's drand48 branch
    co = scaled(800, 111)
    co["pos"][1::7] = co["pos"][0::7][: len(co["pos"][1::7])]
    save("coincident_880", p, co, ref, drand_seed=77)
    save_first_pass("first_pass_nfw_3300", p, scaled(3000, 112), ref)
    save_first_pass("first_pass_corner_2200", p, scaled(2000, 113, center=(99.995, 0.002, 0.5)),
                    ref)
    # a small batch: the halo-parallel loop of RefineParticles
    b = S.subhalo_batch(nsub=48, seed=114, nmax=3000)
    order, energy, res = ref.unbind_batch(p, b, nthreads=1)
    np.savez_compressed(os.path.join(HERE, "batch_48.npz"),
                        **{f"in_{k}": np.asarray(v) for k, v in b.items()},
                        **{f"par_{k}": np.asarray(v) for k, v in p.items()},
                        ref_order=order, ref_energy=energy,
                        **{f"ref_{k}": np.array([r[k] for r in res]) for k in RESULT_KEYS})
    print(f"batch_48: n={b['offsets'][-1]}")


def index_cases(ref):
    """Particle-ID tables (src/hash.tpp): the reference's MappedIndexTable_t
    and FlatIndexTable_t filled with (id, index) pairs, and their answers to
    queries that hit, miss, fall outside the key range or are negative."""
    rng = np.random.Generator(np.random.PCG64(115))
    n = 20000
    ids = rng.choice(10 * n, n, replace=False).astype(np.int64) + 12345  # sparse ids
    vals = rng.permutation(n).astype(np.int64)
    q = np.concatenate([ids[rng.integers(0, n, 5000)], rng.integers(-50, 10 * n + 20000, 5000),
                        np.array([-1, 0, 12344, 12345, ids.min(), ids.max(), ids.max() + 1])])
    q = q.astype(np.int64)
    for flat, name in ((False, "index_mapped"), (True, "index_flat")):
        out = ref.index_lookup(ids, vals, q, flat=flat, null_index=-1)
        qs = np.sort(q)
        outs = ref.index_lookup(ids, vals, qs, flat=flat, null_index=-1, batch=True)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), keys=ids, values=vals,
                            queries=q, ref_out=out, sorted_queries=qs, ref_out_sorted=outs,
                            null_index=np.int64(-1))
        print(f"{name}: {n} keys, {len(q)} queries, {int(np.sum(out != -1))} hits")





def forest_case(seed=116, n_scale=1.0):
    """A forest of nested subhaloes for RecursiveUnbind: two haloes with
    satellites nested three deep, an orphan with a satellite, a satellite that
    disrupts, and a field subhalo.  Satellites sit inside their host's volume
    with their own bulk velocity, so tails do feed the hosts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    box = 100.0
    specs = [  # (n, r200, host, offset from host centre, bulk speed, nbound_prev)
        (4000, 0.25, None, 0.0, 0.0, 4000),     # 0: central of halo A
        (1500, 0.12, 0, 0.10, 250.0, 1500),     # 1: satellite of 0
        (600, 0.07, 1, 0.04, 150.0, 600),       # 2: satellite of 1
        (300, 0.05, 2, 0.02, 120.0, 300),       # 3: satellite of 2 (depth 3)
        (1, 0.01, 0, 0.15, 0.0, 1),             # 4: orphan in 0
        (400, 0.06, 4, 0.03, 100.0, 400),       # 5: satellite of the orphan
        (250, 0.05, 0, 0.12, 300.0, 250),       # 6: a satellite that disrupts (hot)
        (2500, 0.2, None, 0.0, 0.0, 2500),      # 7: central of halo B
        (800, 0.09, 7, 0.08, 200.0, 800),       # 8: satellite of 7
        (700, 0.08, None, 0.0, 0.0, 700),       # 9: field subhalo
    ]
    centres, subs = [], []
    for k, (n, r200, host, off, bulk, _) in enumerate(specs):
        n = max(1, int(n * n_scale)) if n > 1 else 1
        if host is None:
            c = rng.uniform(10.0, 90.0, size=3)
            v = np.zeros(3)
        else:
            u = rng.normal(size=3)
            c = centres[host][0] + off * u / np.linalg.norm(u)
            w = rng.normal(size=3)
            v = centres[host][1] + bulk * w / np.linalg.norm(w)
        centres.append((c, v))
        subs.append(S.nfw_subhalo(rng, n, r200, 8.0, contaminant_frac=0.1 if n > 1 else 0.0,
                                  center=c, bulk_velocity=v, box=box))
    hot = subs[6]  # particles far too fast for their own mass: it disrupts
    hot["vel"] = ((hot["vel"] - centres[6][1]) * 40.0 + centres[6][1]).astype(np.float32)
    S._assign_ids(rng, subs)
    b = S.concat(subs)
    nests = [[] for _ in specs]
    for k, sp in enumerate(specs):
        if sp[2] is not None:
            nests[sp[2]].append(k)
    nest_off = np.concatenate([[0], np.cumsum([len(x) for x in nests])]).astype(np.int64)
    nest_idx = np.array([c for x in nests for c in x], np.int64)
    forest = dict(id=b["id"], pos=b["pos"], vel=b["vel"], mass=b["mass"], type=b["type"],
                  list_off=b["offsets"], nbound_prev=np.array([sp[5] for sp in specs], np.int64),
                  nest_off=nest_off, nest_idx=nest_idx, roots=np.array([0, 7, 9], np.int64),
                  ref_pos=b["ref_pos"], ref_vel=b["ref_vel"], mostbound_pos=b["mostbound_pos"],
                  mostbound_vel=b["mostbound_vel"], mostbound_id=b["mostbound_id"])
    return forest


def forest_cases(ref):
    p = S.default_params()
    forest = forest_case()
    off, pos, res = ref.recursive_unbind(p, forest, relax=3.0)
    np.savez_compressed(os.path.join(HERE, "forest_10.npz"),
                        **{f"in_{k}": np.asarray(v) for k, v in forest.items()},
                        **{f"par_{k}": np.asarray(v) for k, v in p.items()},
                        relax=np.float64(3.0), ref_off=off, ref_pos_out=pos,
                        **{f"ref_{k}": np.array([r[k] for r in res]) for k in RESULT_KEYS})
    print(f"forest_10: {int(forest['list_off'][-1])} particles, final lists {int(off[-1])}, "
          f"nbound {[int(r['nbound']) for r in res]}")


def merge_case(seed=140, n_scale=1.0):
    """Subhaloes for MergeSubhalos, each with its own particles: in halo A a
    central, a satellite sitting in its core (it sinks), a satellite passing
    fast (it does not), a sub-satellite in that satellite's core (it sinks into
    its host), a satellite of the sinking one, an orphan at the central's
    centre and a satellite trapped at an earlier snapshot but still alive; in
    halo B a central and a second top-level subhalo in its core (glued to the
    central's nest while merging); a field subhalo.  The central of A lists
    the sinking satellite's outer particles too (a tail it received while
    unbinding), so the merge has duplicate IDs to drop."""
    rng = np.random.Generator(np.random.PCG64(seed))
    box = 100.0
    specs = [  # (n, r200, parent, offset from parent centre, bulk speed, halo)
        (3000, 0.22, None, 0.0, 0.0, 0),     # 0: central of halo A
        (600, 0.08, 0, 0.0005, 1.0, 0),      # 1: sits in 0's core: sinks into 0
        (500, 0.07, 0, 0.15, 400.0, 0),      # 2: passes fast: stays
        (200, 0.04, 2, 0.0003, 1.0, 0),      # 3: in 2's core: sinks into 2
        (150, 0.03, 1, 0.03, 80.0, 0),       # 4: satellite of 1
        (1, 0.01, 0, 0.0005, 0.0, 0),        # 5: orphan at 0's centre
        (120, 0.03, 0, 0.05, 100.0, 0),      # 6: trapped before (SinkTrackId 0), alive
        (2000, 0.18, None, 0.0, 0.0, 1),     # 7: central of halo B
        (700, 0.08, None, 0.0005, 1.0, 1),   # 8: second head of B, in 7's core
        (400, 0.06, None, 0.0, 0.0, 2),      # 9: field subhalo
    ]
    centres, subs = [], []
    for k, (n, r200, parent, off, bulk, halo) in enumerate(specs):
        n = max(1, int(n * n_scale)) if n > 1 else 1
        anchor = parent if parent is not None else (7 if k == 8 else None)
        if anchor is None:
            c = rng.uniform(10.0, 90.0, size=3)
            v = np.zeros(3)
        else:
            u = rng.normal(size=3)
            c = centres[anchor][0] + off * u / np.linalg.norm(u)
            w = rng.normal(size=3)
            v = centres[anchor][1] + bulk * w / np.linalg.norm(w)
        centres.append((c, v))
        subs.append(S.nfw_subhalo(rng, n, r200, 8.0, contaminant_frac=0.1 if n > 1 else 0.0,
                                  center=c, bulk_velocity=v, box=box))
    S._assign_ids(rng, subs)
    # central 0 also holds satellite 1's last 60 particles
    tail = {k: subs[1][k][-max(1, int(60 * n_scale)):] for k in ("id", "pos", "vel", "mass",
                                                                    "type")}
    for k in tail:
        subs[0][k] = np.concatenate([subs[0][k], tail[k]])
    nests = [[] for _ in specs]
    for k, sp in enumerate(specs):
        if sp[2] is not None:
            nests[sp[2]].append(k)
    groups = [[0, 1, 2, 3, 4, 5, 6], [7, 8], [9]]
    heads = [[0], [7, 8], [9]]
    sink = np.full(len(specs), -1, np.int64)
    sink[6] = 0
    return subs, nests, groups, heads, sink


def merge_state(unbind, params, case):
    """The subhaloes after their unbinding (bound particles first), the input
    of MergeSubhalos: unbind(params, sub) -> (order, result)."""
    subs, nests, groups, heads, sink = case
    rows, nbound, frames = [], [], {k: [] for k in ("ref_pos", "ref_vel", "mostbound_pos",
                                                     "mostbound_vel")}
    for sub in subs:
        order, r = unbind(params, sub)
        rows.append({k: np.asarray(sub[k])[order] for k in ("id", "pos", "vel", "mass", "type")})
        nbound.append(int(r["nbound"]))
        for k in frames:
            frames[k].append(np.asarray(r[k], np.float32))
    def flat(lists):
        off = np.concatenate([[0], np.cumsum([len(x) for x in lists])]).astype(np.int64)
        idx = np.array([c for x in lists for c in x], np.int64)
        return off, idx
    st = {k: np.concatenate([r[k] for r in rows]) for k in ("id", "pos", "vel", "mass", "type")}
    st["list_off"] = np.concatenate([[0], np.cumsum([len(r["id"]) for r in rows])]).astype(
        np.int64)
    st["nbound"] = np.array(nbound, np.int64)
    st.update({k: np.array(v) for k, v in frames.items()})
    st["nest_off"], st["nest_idx"] = flat(nests)
    st["group_off"], st["group_idx"] = flat(groups)
    st["heads_off"], st["heads_idx"] = flat(heads)
    st["sink"] = np.asarray(sink, np.int64)
    st["death"] = np.full(len(subs), -1, np.int32)
    return st


def merge_cases(ref):
    p = S.default_params()

    def unbind(params, sub):
        o, _, r = ref.unbind(params, sub, nthreads=1)
        return o, r

    st = merge_state(unbind, p, merge_case())
    out = ref.merge_subhalos(p, st, isnap=5, relax=3.0)
    np.savez_compressed(
        os.path.join(HERE, "merge_10.npz"),
        **{f"in_{k}": v for k, v in st.items()},
        **{f"par_{k}": np.asarray(v) for k, v in p.items()},
        isnap=np.int32(5), relax=np.float64(3.0),
        ref_off=out["off"], ref_id=out["id"], ref_energy=out["energy"], ref_sink=out["sink"],
        ref_death=out["death"], ref_sink_snap=out["sink_snap"],
        **{f"ref_{k}": np.array([r[k] for r in out["results"]]) for k in RESULT_KEYS})
    print(f"merge_10: nbound {list(st['nbound'])} -> "
          f"{[int(r['nbound']) for r in out['results']]}, sink {list(out['sink'])}, "
          f"death {list(out['death'])}")


PROPS_KEYS = ("rmax_comoving", "vmax_physical", "last_max_vmax_physical",
              "snapshot_of_last_max_vmax", "r2sigma_comoving", "rhalf_comoving",
              "r200crit_comoving", "m200crit", "inertial_tensor", "inertial_tensor_weighted")


def wide_masses(sub, seed, octaves):
    """Particle masses spread over 2^-octaves .. 2^octaves times the base mass,
    with random mantissas (mixed species)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    f = np.exp2(rng.uniform(-octaves, octaves, len(sub["mass"])))
    sub["mass"] = (sub["mass"].astype(np.float64) * f).astype(np.float32)
    return sub


def props_batch(name, params, specs, ref):
    """Each subhalo unbound by the reference's Unbind, then its
    CalculateProfileProperties and CalculateShape (epoch: snapshot 1), stored
    as one batch: inputs, order, results and properties per subhalo."""
    subs, orders, energies, results, props = [], [], [], [], []
    for sub, lm, ls in specs:
        o, e, r, pr = ref.unbind_properties(params, sub, last_max_vmax=lm, last_snap=ls)
        subs.append(sub)
        orders.append(o)
        energies.append(e)
        results.append(r)
        props.append(pr)
    off = np.concatenate([[0], np.cumsum([len(s["mass"]) for s in subs])]).astype(np.int64)
    cat = {k: np.concatenate([s[k] for s in subs]) for k in ("id", "pos", "vel", "mass", "type")}
    per = {k: np.array([s[k] for s in subs]) for k in ("ref_pos", "ref_vel", "mostbound_pos",
                                                       "mostbound_vel")}
    per["mostbound_id"] = np.array([int(s.get("mostbound_id", s["id"][0])) for s in subs])
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        **{f"in_{k}": v for k, v in cat.items()}, **{f"in_{k}": v for k, v in per.items()},
        in_offsets=off, in_last_max_vmax=np.array([s[1] for s in specs], np.float32),
        in_last_snap=np.array([s[2] for s in specs], np.int32), snapshot_index=np.int32(1),
        **{f"par_{k}": np.asarray(v) for k, v in params.items()},
        ref_order=np.concatenate(orders), ref_energy=np.concatenate(energies),
        **{f"ref_{k}": np.array([r[k] for r in results]) for k in RESULT_KEYS},
        **{f"props_{k}": np.array([q[k] for q in props]) for k in PROPS_KEYS})
    print(f"{name}: {len(subs)} subhaloes, nbound {[int(r['nbound']) for r in results]}")


def props_cases(ref):
    p = S.default_params()
    hot = scaled(300, 127)
    hot["vel"] = (hot["vel"] * 40.0).astype(np.float32)
    props_batch("props_10", p, [
        (scaled(3000, 121), 0.0, -1),
        (scaled(1000, 122, c=15.0, center=(0.01, 99.99, 50.0)), 0.0, -1),  # periodic corner
        (scaled(20000, 123, c=8.0), 0.0, -1),
        (scaled(50, 124, cf=0.0), 0.0, -1),
        (scaled(3, 125, cf=0.0), 0.0, -1),
        (scaled(2000, 126), 1e9, 0),       # below the last maximum: kept
        (scaled(2000, 126), 150.0, 0),     # the same subhalo above a lower last maximum
        (hot, 7.0, 0),                      # disrupted: nothing computed, last maximum kept
        (wide_masses(scaled(20000, 128), 129, 8.0), 0.0, -1),   # mixed species
        (wide_masses(scaled(4000, 130), 131, 30.0), 0.0, -1),   # masses over 2^60
    ], ref)
    pa = S.default_params(scale_factor=0.5, hubble=180.0, periodic=0)
    props_batch("props_a05", pa, [
        (scaled(5000, 132, center=(30.0, 40.0, 50.0)), 0.0, -1),
        (scaled(800, 133, c=4.0, center=(60.0, 40.0, 50.0)), 12.0, 0),
    ], ref)


if __name__ == "__main__":
    if sys.argv[1:] == ["index"]:
        index_cases(Oracle(reference=True))
    elif sys.argv[1:] == ["forest"]:
        forest_cases(Oracle(reference=True))
    elif sys.argv[1:] == ["props"]:
        props_cases(Oracle(reference=True))
    elif sys.argv[1:] == ["merge"]:
        merge_cases(Oracle(reference=True))
    else:
        main()
        index_cases(Oracle(reference=True))
        forest_cases(Oracle(reference=True))
        props_cases(Oracle(reference=True))
        merge_cases(Oracle(reference=True))
