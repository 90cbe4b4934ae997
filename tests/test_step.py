"""The tracking step around the unbinding (hbtplus_gb300.step): the new
snapshot's ID table, the re-resolve of each subhalo's particle IDs
(GetIndices, src/hash_remote.tpp), the gather, and the batched unbind.

Checks: the GPU re-resolve equals a host re-resolve (numpy), the gathered
particles equal the host-gathered ones, and the unbinding of the gathered
batch equals the same library's unbinding of the host-gathered batch bit for
bit, and so do the profile and shape of every subhalo.  At full size (config
4: 20,000 subhaloes, 3e7 particles in a 200 Mpc/h box, drift, 10% stripping)
the same holds for 20 sampled subhaloes and every ID resolves; and the step's
unbinding of 300 sampled subhaloes (of at most 50,000 particles) agrees with
the C oracle's Unbind of the host-gathered particles (src/subhalo_unbind.cpp:
263-431) within the FP32 tolerances of the full-batch test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_resolve(snap_id, member_id):
    order = np.argsort(snap_id, kind="stable")
    k = np.searchsorted(snap_id[order], member_id)
    k = np.minimum(k, len(order) - 1)
    hit = snap_id[order[k]] == member_id
    return np.where(hit, order[k], -1)


def run_step(d, flat=False):
    import torch
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.step import TrackingStep
    from hbtplus_gb300.unbind import Unbinder
    ub = Unbinder(S.default_params(box_size=200.0))
    step = TrackingStep(ub, flat=flat)
    dev = torch.device("cuda")
    T = {k: torch.from_numpy(np.ascontiguousarray(d[k])).to(dev)
         for k in ("snap_id", "snap_pos", "snap_vel", "snap_mass", "snap_type", "member_id")}
    step.load_snapshot(T["snap_id"], T["snap_pos"], T["snap_vel"], T["snap_mass"],
                       T["snap_type"])
    frames = dict(offsets=d["offsets"], ref_pos=d["ref_pos"], ref_vel=d["ref_vel"],
                  mostbound_pos=d["mostbound_pos"], mostbound_vel=d["mostbound_vel"],
                  mostbound_id=d["mostbound_id"])
    states = ub.make_states(frames)
    out, index = step.run(d["offsets"], T["member_id"], states,
                          properties=dict(snapshot_index=3))
    torch.cuda.synchronize()
    return ub, step, out, index.cpu().numpy(), states


def host_batch(d, index):
    b = {k: d["snap_" + k][index] for k in ("id", "pos", "vel", "mass", "type")}
    for k in ("offsets", "ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel",
              "mostbound_id"):
        b[k] = d[k]
    return b


@pytest.mark.parametrize("flat", [False, True])
def test_step_small_matches_host(flat):
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import results_from_bytes
    d = S.tracking_snapshot(nsub=200, ntot=300_000, seed=31)
    if flat:  # dense IDs for the flat table
        remap = np.empty(d["snap_id"].max() + 1, np.int64)
        remap[d["snap_id"]] = np.arange(len(d["snap_id"]))
        for k in ("snap_id", "member_id", "mostbound_id"):
            d[k] = remap[d[k]]
    ub, step, out, index, states = run_step(d, flat)
    expect = host_resolve(d["snap_id"], d["member_id"])
    assert np.array_equal(index, expect) and (index >= 0).all()
    b = host_batch(d, index)
    order, energy, res = ub.unbind_batch(b)
    gres = results_from_bytes(out["res"].cpu().numpy(), len(d["offsets"]) - 1)
    assert np.array_equal(out["order"].cpu().numpy(), order)
    assert np.array_equal(out["energy"].cpu().numpy(), energy, equal_nan=True)
    assert [r["nbound"] for r in gres] == [r["nbound"] for r in res]
    # the step's profile and shape equal the host call on the host-gathered batch
    from hbtplus_gb300.unbind import props_to_dict
    hp = ub.subhalo_properties(b, order, res, snapshot_index=3)
    for s in range(len(hp)):
        g = props_to_dict(out["props"][s])
        for k, v in hp[s].items():
            assert np.array_equal(np.asarray(g[k]), np.asarray(v), equal_nan=True), (s, k)
    step.close()
    ub.close()


def test_step_config4_full_size():
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.unbind import results_from_bytes
    d = S.tracking_snapshot()  # 20,000 subhaloes, 3e7 particles, 200 Mpc/h
    assert len(d["snap_id"]) == 30_000_000 and len(d["offsets"]) == 20_001
    ub, step, out, index, states = run_step(d)
    assert (index >= 0).all()
    rng = np.random.default_rng(8)
    expect = host_resolve(d["snap_id"], d["member_id"])
    assert np.array_equal(index, expect)
    nsub = len(d["offsets"]) - 1
    gres = results_from_bytes(out["res"].cpu().numpy(), nsub)
    order = out["order"].cpu().numpy()
    b = host_batch(d, index)
    for s in rng.choice(nsub, 20, replace=False):
        sub = S.split(b, int(s))
        o, e, r = ub.unbind(sub)
        o0, o1 = int(d["offsets"][s]), int(d["offsets"][s + 1])
        assert np.array_equal(order[o0:o1], o)
        assert gres[s]["nbound"] == r["nbound"] and gres[s]["mbound"] == r["mbound"]
    # the step's unbinding against the C oracle, on sampled subhaloes
    from oracle import Oracle
    from test_batch_full import compare
    energy = out["energy"].cpu().numpy()
    n = np.diff(d["offsets"])
    pick = rng.choice(np.nonzero(n <= 50_000)[0], 300, replace=False)
    subs = [S.split(b, int(s)) for s in pick]
    sb = S.concat(subs)
    got_order = np.concatenate([order[d["offsets"][s]:d["offsets"][s + 1]] for s in pick])
    got_energy = np.concatenate([energy[d["offsets"][s]:d["offsets"][s + 1]] for s in pick])
    got = (got_order, got_energy, [gres[int(s)] for s in pick])
    p = S.default_params(box_size=200.0)
    ref = Oracle().unbind_batch(p, sb, nthreads=0)
    changed, _ = compare(sb, got, ref, exact=False, p=p)
    print(f"config 4, 300 sampled subhaloes against the oracle: {changed} particles changed "
          f"side, all inside the band")
    step.close()
    ub.close()
