"""Nested unbinding: RecursiveUnbind and TruncateSource, batched by depth.

The reference unbinds a halo's subhaloes depth first: every nested subhalo is
unbound before its host, and its unbound tail (Particles[Nbound:]) is appended
to the host's list before the host is unbound; an orphan (Nbound <= 1 in the
last snapshot) is unbound on its own particles only but hands the extended
list to its host (Subhalo_t::RecursiveUnbind, src/subhalo_unbind.cpp:432-447).
Afterwards every list is cut to Nbound * SourceSubRelaxFactor
(TruncateSource, :449-458).  RefineParticles calls this per halo, after
adding the halo's other heads to the central's nested list (:481-494), then
unbinds field and new-born subhaloes (:497-513).

Here every subhalo of one nesting depth is unbound in one hbtu_unbind_batch
call, deepest depth first, so a forest of thousands of subhaloes needs as many
GPU calls as it has levels.

    out = recursive_unbind(unbinder, parts, list_off, nbound_prev, nest_off,
                           nest_idx, roots, frames, relax=3.0)
    out["off"], out["pos"]   # final lists: positions into the input arrays
    out["results"]           # per subhalo: hbtu_result as a dict (None if not reached)
"""
from __future__ import annotations

import numpy as np


def nesting_depth(nsub: int, nest_off, nest_idx, roots) -> np.ndarray:
    """Depth of every subhalo below the roots (-1: not reached).  A subhalo
    reached twice keeps its first depth, as RecursiveUnbind visits it once per
    appearance in a nested list."""
    depth = np.full(nsub, -1, np.int64)
    stack = [(int(r), 0) for r in reversed(list(roots))]
    while stack:
        s, d = stack.pop()
        if depth[s] >= 0:
            continue
        depth[s] = d
        for c in reversed(nest_idx[nest_off[s]:nest_off[s + 1]].tolist()):
            stack.append((int(c), d + 1))
    return depth


def source_size(nbound: int, n: int, relax: float) -> int:
    """TruncateSource's list length: Nbound * SourceSubRelaxFactor, formed as
    the reference does (HBTInt times HBTReal in float, truncated), at most n."""
    if nbound <= 1:
        ns = nbound
    else:
        ns = int(np.float32(nbound) * np.float32(relax))
    return min(ns, n)


def recursive_unbind(ub, parts: dict, list_off, nbound_prev, nest_off, nest_idx, roots,
                     frames: dict, relax: float = 3.0) -> dict:
    """Unbind a forest of subhaloes as RecursiveUnbind + TruncateSource do.

    parts: id, pos, vel, mass, type of every subhalo's own particles,
    concatenated (subhalo s owns rows list_off[s] .. list_off[s+1]).
    frames: ref_pos, ref_vel, mostbound_pos, mostbound_vel, mostbound_id
    per subhalo.  Each subhalo is unbound once (its first appearance)."""
    list_off = np.asarray(list_off, np.int64)
    nest_off = np.asarray(nest_off, np.int64)
    nest_idx = np.asarray(nest_idx, np.int64)
    nbound_prev = np.asarray(nbound_prev, np.int64)
    nsub = len(list_off) - 1
    depth = nesting_depth(nsub, nest_off, nest_idx, roots)
    final = [None] * nsub      # each subhalo's list after its unbinding (input positions)
    nbound = np.zeros(nsub, np.int64)
    results = [None] * nsub
    for d in sorted(set(depth[depth >= 0].tolist()), reverse=True):
        level = np.nonzero(depth == d)[0]
        unb, ext, orphan = [], [], []
        for s in level:
            own = np.arange(list_off[s], list_off[s + 1], dtype=np.int64)
            tails = [final[c][nbound[c]:] for c in nest_idx[nest_off[s]:nest_off[s + 1]]
                     if depth[c] == d + 1 and final[c] is not None]
            e = np.concatenate([own] + tails) if tails else own
            o = nbound_prev[s] <= 1
            ext.append(e)
            unb.append(own if o else e)
            orphan.append(o)
        counts = np.array([len(u) for u in unb], np.int64)
        offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        flat = np.concatenate(unb) if len(unb) else np.zeros(0, np.int64)
        batch = {k: np.asarray(parts[k])[flat] for k in ("id", "pos", "vel", "mass", "type")}
        batch["offsets"] = offsets
        for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel", "mostbound_id"):
            batch[k] = np.asarray(frames[k])[level]
        order, _, res = ub.unbind_batch(batch, check_status=False)
        for j, s in enumerate(level):
            o0, o1 = int(offsets[j]), int(offsets[j + 1])
            nbound[s] = int(res[j]["nbound"])
            results[s] = res[j]
            # an orphan keeps its extended list unpermuted (the swap at :444-446)
            final[s] = ext[j] if orphan[j] else unb[j][order[o0:o1]]
    # TruncateSource on every list
    out_pos, out_off = [], [0]
    for s in range(nsub):
        if final[s] is None:  # not under any root: cut with the last snapshot's Nbound
            lst = np.arange(list_off[s], list_off[s + 1], dtype=np.int64)
            ns = source_size(int(nbound_prev[s]), len(lst), relax)
        else:
            lst = final[s]
            ns = source_size(int(nbound[s]), len(lst), relax)
        out_pos.append(lst[:ns])
        out_off.append(out_off[-1] + ns)
    return dict(off=np.array(out_off, np.int64),
                pos=np.concatenate(out_pos) if out_pos else np.zeros(0, np.int64),
                results=results, depth=depth)
