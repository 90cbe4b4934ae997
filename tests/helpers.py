"""Shared helpers of the test suite: fixtures and comparisons."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SINGLE_CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if not os.path.basename(f).startswith(("first_pass", "batch", "index", "forest",
                                                                     "props", "merge")))
FIRST_PASS_CASES = sorted(os.path.basename(f)[:-4]
                          for f in glob.glob(os.path.join(GOLDEN, "first_pass_*.npz")))


def load_case(name: str):
    """(params, inputs, reference outputs) of a golden fixture."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    par = {k[4:]: z[k].item() for k in z.files if k.startswith("par_")}
    inp = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    for k in ("mostbound_id",):
        if k in inp and inp[k].ndim == 0:
            inp[k] = int(inp[k])
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    extra = {k: z[k] for k in z.files if not k.startswith(("par_", "in_", "ref_"))}
    ref.update(extra)
    return par, inp, ref


def tie_groups_equal(order_a, order_b, energy):
    """Orders agree up to permutations inside runs of bit-equal energy."""
    order_a = np.asarray(order_a)
    order_b = np.asarray(order_b)
    if len(order_a) != len(order_b):
        return False
    if np.array_equal(order_a, order_b):
        return True
    e = np.asarray(energy)
    i = 0
    n = len(e)
    while i < n:
        j = i + 1
        while j < n and e[j] == e[i]:
            j += 1
        if set(order_a[i:j].tolist()) != set(order_b[i:j].tolist()):
            return False
        i = j
    return True


def partition_emulation(E: np.ndarray):
    """The GPU's closed form of PartitionBindingEnergy (prefix counts of the
    sign pattern), in numpy: returns (nbound, permutation of positions)."""
    E = np.asarray(E, np.float32)
    n = len(E)
    if n == 0:
        return 0, np.zeros(0, np.int64)
    if n == 1:
        return int(E[0] < 0), np.zeros(1, np.int64)
    pos = np.nonzero(E[1:] > 0)[0] + 1          # P_1 < P_2 < ...
    neg = np.nonzero(E[1:] < 0)[0][::-1] + 1    # Q_1 > Q_2 > ...
    npos, nneg = len(pos), len(neg)
    mn = min(npos, nneg)
    k = np.arange(1, mn + 1)
    failF = np.nonzero(pos[:mn] >= neg[:mn])[0]
    F = (failF[0] + 1 if len(failF) else mn + 1) - 1
    condG = np.array([(kk + 1 > nneg) or (pos[kk - 1] >= neg[kk]) for kk in k], bool)
    failG = np.nonzero(condG)[0]
    G = min((failG[0] + 1 if len(failG) else 1 << 30) - 1, F)
    src = np.arange(n)
    if nneg == 0:
        mb = mf = vd = 0
    else:
        mb = 1 + G
        mf = G + (1 if G + 1 <= F else 0)
        vd = pos[mf - 1] if mf == mb else neg[mb - 1]
        src[0] = neg[0]
        for kk in range(1, mf + 1):
            src[neg[kk - 1]] = pos[kk - 1]
        for kk in range(1, mb):
            src[pos[kk - 1]] = neg[kk]
    src[vd] = 0
    return int(vd + (E[0] < 0)), src


def recursive_unbind_oracle(orc, params, forest, relax=3.0):
    """RecursiveUnbind + TruncateSource restated literally (depth first, one
    subhalo at a time; src/subhalo_unbind.cpp:432-458) on the C oracle's Unbind.
    Returns (final list offsets, positions into the input rows, nbound)."""
    lo = np.asarray(forest["list_off"], np.int64)
    no = np.asarray(forest["nest_off"], np.int64)
    ni = np.asarray(forest["nest_idx"], np.int64)
    nsub = len(lo) - 1
    final = [np.arange(lo[s], lo[s + 1]) for s in range(nsub)]
    nbound = np.asarray(forest["nbound_prev"], np.int64).copy()

    def unbind(s, rows):
        sub = {k: np.asarray(forest[k])[rows] for k in ("id", "pos", "vel", "mass", "type")}
        for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
            sub[k] = np.asarray(forest[k])[s]
        sub["mostbound_id"] = int(forest["mostbound_id"][s])
        order, _, res = orc.unbind(params, sub)
        return rows[order], int(res["nbound"])

    def rec(s):
        orphan = nbound[s] <= 1
        rows = np.arange(lo[s], lo[s + 1])
        backup = rows.copy() if orphan else None
        for c in ni[no[s]:no[s + 1]]:
            rec(int(c))
            rows = np.concatenate([rows, final[c][nbound[c]:]])
        if orphan:
            rows, backup = backup, rows
        rows, nbound[s] = unbind(s, rows)
        if orphan:
            rows, backup = backup, rows
        final[s] = rows

    for r in forest["roots"]:
        rec(int(r))
    off, out = [0], []
    for s in range(nsub):
        if nbound[s] <= 1:
            ns = nbound[s]
        else:
            ns = int(np.float32(nbound[s]) * np.float32(relax))
        ns = min(ns, len(final[s]))
        out.append(final[s][:ns])
        off.append(off[-1] + ns)
    return np.array(off, np.int64), np.concatenate(out), nbound


class OracleUnbinder:
    """The oracle behind the two calls hbtplus_gb300.merge makes of an
    Unbinder (merge_detect, unbind_batch), so the host orchestration can be
    checked on the CPU against the reference."""

    def __init__(self, orc, params):
        self.orc = orc
        self.params = params

    def merge_detect(self, parts, list_off, nbound, host, mb_pos, mb_vel, isnap, sink):
        return self.orc.merge_detect(self.params, list_off, parts["pos"], parts["vel"],
                                     parts["mass"], nbound, host, mb_pos, mb_vel, isnap, sink)

    def unbind_batch(self, batch, check_status=True):
        off = np.asarray(batch["offsets"], np.int64)
        orders, energies, results = [], [], []
        for s in range(len(off) - 1):
            o0, o1 = int(off[s]), int(off[s + 1])
            sub = {k: np.asarray(batch[k])[o0:o1] for k in ("id", "pos", "vel", "mass", "type")}
            for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
                sub[k] = np.asarray(batch[k])[s]
            sub["mostbound_id"] = int(batch["mostbound_id"][s])
            o, e, r = self.orc.unbind(self.params, sub)
            orders.append(o)
            energies.append(e)
            results.append(r)
        cat = (lambda x, t: np.concatenate(x) if x else np.zeros(0, t))
        return cat(orders, np.int64), cat(energies, np.float32), results
