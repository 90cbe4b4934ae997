"""Merging of trapped subhaloes: SubhaloSnapshot_t::MergeSubhalos.

After the unbinding of a snapshot the reference looks for subhaloes that have
sunk into the core of one of their hosts (src/subhalo_merge.cpp:187-220):

1. GlueHeadNests (src/subhalo_tracking.cpp:843-862): the other top-level
   subhaloes of a halo join its central's nest for the duration;
2. FillHelpers: each subhalo's host (the subhalo whose nest lists it) and
   its core (first min(Nbound, 20) particles); DetectTraps: a subhalo not yet
   trapped walks up its hosts and sinks into the first whose core is within
   phase-space distance 2 of its most-bound particle;
3. MergeRecursive (:222-232), per halo from its central, depth first: a
   trapped subhalo that is still alive hands its particles to its sink
   (Subhalo_t::MergeTo, :244-262: the union by particle Id, host order first)
   and dies;
4. every subhalo that swallowed a subhalo with Nbound > 1 is unbound again and
   its list cut (TruncateSource).

Here step 2 runs on the GPU for all subhaloes at once (hbtu_merge_detect),
step 4's unbindings are one hbtu_unbind_batch call, and the list unions of
step 3, which follow the halo's depth-first order, run on the host.

    out = merge_subhalos(unbinder, state, isnap=5, relax=3.0)

``state`` holds every subhalo's list after its unbinding (rows id, pos, vel,
mass, type concatenated by list_off, bound first), nbound, the frames
(ref_pos, ref_vel, mostbound_pos, mostbound_vel), the nests
(nest_off/nest_idx), the haloes' members (group_off/group_idx, central first)
and top-level subhaloes (heads_off/heads_idx, central first), sink
(SinkTrackId, -1: none) and death (SnapshotIndexOfDeath, -1: alive).
"""
from __future__ import annotations

import numpy as np

from .refine import source_size


def _lists(off, idx):
    off = np.asarray(off, np.int64)
    idx = np.asarray(idx, np.int64)
    return [idx[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def glued_nests(state: dict):
    """Every subhalo's nest with the haloes' other heads appended to their
    centrals' (GlueHeadNests)."""
    nests = _lists(state["nest_off"], state["nest_idx"])
    groups = _lists(state["group_off"], state["group_idx"])
    heads = _lists(state["heads_off"], state["heads_idx"])
    for g, hd in zip(groups, heads):
        if g:
            nests[g[0]] = nests[g[0]] + hd[1:]
    return nests, groups


def host_track_ids(nsub: int, nests) -> np.ndarray:
    """HostTrackId (FillHostTrackIds, src/subhalo_merge.cpp:162-171): the
    subhalo whose nest lists s; the last such subhalo in index order wins."""
    host = np.full(nsub, -1, np.int64)
    for i, nest in enumerate(nests):
        for c in nest:
            host[c] = i
    return host


def merge_subhalos(ub, state: dict, isnap: int, relax: float = 3.0) -> dict:
    """MergeSubhalos with MergeTrappedSubhalos on.  Returns the lists after
    merging (``lists``: row positions into the state arrays), nbound, sink,
    sink_snap (SnapshotIndexOfSink where a subhalo was trapped now, else -1),
    death, merged (the subhaloes unbound again) and their results."""
    lo = np.asarray(state["list_off"], np.int64)
    nsub = len(lo) - 1
    ids = np.asarray(state["id"], np.int64)
    nests, groups = glued_nests(state)
    host = host_track_ids(nsub, nests)
    parts = {k: state[k] for k in ("pos", "vel", "mass")}
    sink, sink_snap, merged, _ = ub.merge_detect(
        parts, lo, state["nbound"], host, state["mostbound_pos"], state["mostbound_vel"], isnap,
        state["sink"])
    lists = [np.arange(lo[s], lo[s + 1], dtype=np.int64) for s in range(nsub)]
    nbound = np.asarray(state["nbound"], np.int64).copy()
    death = np.asarray(state["death"], np.int32).copy()

    def merge_to(s: int, h: int) -> None:  # Subhalo_t::MergeTo
        if nbound[s] <= 1:
            return
        cid = ids[lists[s]]
        first = np.zeros(len(cid), bool)  # first appearance of each Id in the subhalo's list
        first[np.unique(cid, return_index=True)[1]] = True
        keep = first & ~np.isin(cid, ids[lists[h]])  # and not held by the sink already
        lists[h] = np.concatenate([lists[h], lists[s][keep]])
        nbound[h] += nbound[s]
        lists[s] = lists[s][:1]
        nbound[s] = 1

    for g in groups:  # MergeRecursive from each central, depth first (post-order)
        if not g:
            continue
        stack = [(g[0], False)]
        while stack:
            s, done = stack.pop()
            if not done:
                stack.append((s, True))
                for c in reversed(nests[s]):
                    stack.append((c, False))
                continue
            if sink[s] >= 0 and death[s] < 0:  # IsTrapped() && IsAlive()
                merge_to(s, int(sink[s]))
                death[s] = isnap
    # the merged subhaloes, unbound again in one batch, then truncated
    idx = np.nonzero(merged)[0]
    results = [None] * nsub
    energy = [None] * nsub
    if len(idx):
        rows = [lists[s] for s in idx]
        flat = np.concatenate(rows)
        offsets = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
        batch = {k: np.asarray(state[k])[flat] for k in ("id", "pos", "vel", "mass", "type")}
        batch["offsets"] = offsets
        for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
            batch[k] = np.asarray(state[k])[idx]
        batch["mostbound_id"] = np.array([ids[r[0]] if len(r) else -1 for r in rows], np.int64)
        order, en, res = ub.unbind_batch(batch, check_status=False)
        for j, s in enumerate(idx):
            o0, o1 = int(offsets[j]), int(offsets[j + 1])
            lists[s] = rows[j][order[o0:o1]]
            energy[s] = en[o0:o1]
            nbound[s] = int(res[j]["nbound"])
            results[s] = res[j]
            ns = source_size(int(nbound[s]), len(lists[s]), relax)  # TruncateSource
            lists[s] = lists[s][:ns]
    return dict(lists=lists, nbound=nbound, sink=sink, sink_snap=sink_snap, death=death,
                merged=merged, results=results, energy=energy, host=host)
