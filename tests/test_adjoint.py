"""Adjoint of the binding energy (hbtu_energy_gradient, hbtplus_gb300.adjoint).

Checks:
  * theta = 0 opens every cell, so the walk is the exact pairwise sum: the GPU
    gradient must equal an FP64 direct-sum gradient to FP32 rounding (1e-5);
  * theta = 0.45 (the reference default): within the tree's own error (2e-2 in
    the relative L2 norm of the position gradient);
  * the FP64 direct-sum gradient itself against central finite differences of
    the FP64 direct-sum E_tot (step 1e-6 Mpc/h, 1000 random particles, the frame
    recomputed at every step);
  * torch.autograd through BindingEnergy gives exactly the library's gradients;
  * one batched launch equals per-subhalo launches (to FP32 rounding);
  * the 1e6-particle subhalo: FP64 direct-sum gradients of 1000 random
    particles, and momentum balance of sum m grad phi;
  * the bound sets of the 2000-subhalo batch after unbinding, differentiated
    in one call: bit for bit the per-subhalo calls (each target's walk and
    sums do not depend on the other subhaloes of a call), and within the
    tree's error of FP64 direct-sum gradients on 1000 random particles.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = 43.0071
HZ = 100.0


def direct(tx, sx, sm, eps, skip_self_index=None, chunk=2_000_000):
    """FP64 direct sum at targets tx (k,3) from sources sx (n,3), masses sm:
    potential phi (k,) and gradient (k,3), reference spline softening (h=2.8 eps),
    positions already relative (no wrap needed)."""
    import torch
    h = 2.8 * eps
    hinv = 1.0 / h
    k = tx.shape[0]
    phi = torch.zeros(k, dtype=torch.float64, device=tx.device)
    grad = torch.zeros((k, 3), dtype=torch.float64, device=tx.device)
    step = max(1, chunk // max(k, 1))
    for j0 in range(0, sx.shape[0], step):
        s = sx[j0:j0 + step]
        m = sm[j0:j0 + step]
        dx = s[None, :, :] - tx[:, None, :]             # x_node - x_target
        r2 = (dx * dx).sum(-1)
        r = torch.sqrt(r2)
        u = r * hinv
        far = r >= h
        rs = torch.where(r2 > 0, r, torch.ones_like(r))
        wp = torch.where(u < 0.5, -2.8 + u * u * (16.0 / 3 + u * u * (6.4 * u - 9.6)),
                         -3.2 + 1.0 / (15 * torch.where(u > 0, u, torch.ones_like(u))) +
                         u * u * (32.0 / 3 + u * (-16.0 + u * (9.6 - 32.0 / 15 * u))))
        dwp = torch.where(u < 0.5, u * (32.0 / 3 + u * u * (32.0 * u - 38.4)),
                          -1.0 / (15 * torch.where(u > 0, u * u, torch.ones_like(u))) +
                          u * (64.0 / 3 + u * (-48.0 + u * (38.4 - 32.0 / 3 * u))))
        pot = torch.where(far, -1.0 / rs, hinv * wp)
        w = torch.where(far, 1.0 / (rs * rs * rs), hinv * hinv * dwp / rs)
        if skip_self_index is not None:
            idx = torch.arange(j0, j0 + s.shape[0], device=tx.device)
            self_mask = idx[None, :] == skip_self_index[:, None]
            pot = torch.where(self_mask, torch.zeros_like(pot), pot)
            w = torch.where(self_mask, torch.zeros_like(w), w)
        w = torch.where(r2 > 0, w, torch.zeros_like(w))
        phi += (pot * m[None, :]).sum(1)
        grad += -((w * m[None, :])[:, :, None] * dx).sum(1)
    return G * phi, G * grad


def etot_fp64(x, v, m, eps):
    """FP64 direct-sum E_tot with the frame at the centre of mass (a=1, no wrap)."""
    import torch
    X = (m[:, None] * x).sum(0) / m.sum()
    V = (m[:, None] * v).sum(0) / m.sum()
    dv = v - V + HZ * (x - X)
    phi, _ = direct(x, x, m, 0.002, skip_self_index=torch.arange(len(m), device=x.device))
    return 0.5 * (m * (dv * dv).sum(1)).sum() + 0.5 * (m * phi).sum()


def _subhalo(n, seed, center=(50.0, 50.0, 50.0)):
    from hbtplus_gb300 import synthetic as S
    rng = np.random.Generator(np.random.PCG64(seed))
    sub = S.nfw_subhalo(rng, n, 0.2 * (n / 1e5) ** (1 / 3), 10.0, contaminant_frac=0.0,
                        center=center)
    S._assign_ids(rng, [sub])
    # frame at the centre of mass (what unbinding converges to)
    m = sub["mass"].astype(np.float64)
    sub["ref_pos"] = (np.sum(sub["pos"] * m[:, None], 0) / m.sum()).astype(np.float32)
    sub["ref_vel"] = (np.sum(sub["vel"] * m[:, None], 0) / m.sum()).astype(np.float32)
    return sub


def _gpu_grads(sub, theta):
    import torch
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.adjoint import energy_gradient
    from hbtplus_gb300.unbind import Unbinder
    p = S.default_params(open_angle=theta)
    with Unbinder(p) as ub:
        t = {k: torch.from_numpy(np.ascontiguousarray(sub[k])).cuda() for k in ("pos", "vel", "mass")}
        E, gp, gv, gm = energy_gradient(ub, t["pos"], t["vel"], t["mass"],
                                        [0, len(sub["mass"])], sub["ref_pos"][None],
                                        sub["ref_vel"][None])
    return float(E[0]), gp.cpu().numpy(), gv.cpu().numpy(), gm.cpu().numpy()


def _fp64_reference(sub):
    import torch
    x = torch.tensor(sub["pos"], dtype=torch.float64, device="cuda")
    v = torch.tensor(sub["vel"], dtype=torch.float64, device="cuda")
    m = torch.tensor(sub["mass"], dtype=torch.float64, device="cuda")
    X = torch.tensor(sub["ref_pos"], dtype=torch.float64, device="cuda")
    V = torch.tensor(sub["ref_vel"], dtype=torch.float64, device="cuda")
    phi, gphi = direct(x, x, m, 0.002, skip_self_index=torch.arange(len(m), device="cuda"))
    dv = v - V + HZ * (x - X)
    E = float(0.5 * (m * (dv * dv).sum(1)).sum() + 0.5 * (m * phi).sum())
    gp = m[:, None] * (HZ * dv + gphi)
    gv = m[:, None] * dv
    gm = 0.5 * (dv * dv).sum(1) + phi
    return E, gp.cpu().numpy(), gv.cpu().numpy(), gm.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_theta0_equals_fp64_direct_sum():
    pytest.importorskip("torch")
    sub = _subhalo(3000, 1)
    E, gp, gv, gm = _gpu_grads(sub, 0.0)
    E64, gp64, gv64, gm64 = _fp64_reference(sub)
    assert abs(E - E64) <= 1e-5 * abs(E64)
    assert _rel(gp, gp64) < 1e-5
    assert _rel(gv, gv64) < 1e-6
    assert _rel(gm, gm64) < 1e-5


def test_theta045_within_tree_error():
    pytest.importorskip("torch")
    sub = _subhalo(5000, 2)
    E, gp, gv, gm = _gpu_grads(sub, 0.45)
    E64, gp64, gv64, gm64 = _fp64_reference(sub)
    assert abs(E - E64) <= 1e-3 * abs(E64)
    assert _rel(gp, gp64) < 2e-2
    assert _rel(gm, gm64) < 2e-3


def test_fp64_gradient_against_central_differences():
    torch = pytest.importorskip("torch")
    sub = _subhalo(1000, 3)
    x = torch.tensor(sub["pos"], dtype=torch.float64, device="cuda")
    v = torch.tensor(sub["vel"], dtype=torch.float64, device="cuda")
    m = torch.tensor(sub["mass"], dtype=torch.float64, device="cuda")
    X = (m[:, None] * x).sum(0) / m.sum()
    V = (m[:, None] * v).sum(0) / m.sum()
    phi, gphi = direct(x, x, m, 0.002, skip_self_index=torch.arange(len(m), device="cuda"))
    dv = v - V + HZ * (x - X)
    gp = (m[:, None] * (HZ * dv + gphi)).cpu().numpy()
    rng = np.random.default_rng(4)
    idx = rng.choice(len(m), size=1000, replace=False)
    step = 1e-6
    errs = []
    for i in idx:                      # each FD sample costs two direct sums
        j = int(rng.integers(3))
        xp = x.clone()
        xm = x.clone()
        xp[i, j] += step
        xm[i, j] -= step
        fd = float((etot_fp64(xp, v, m, 0.002) - etot_fp64(xm, v, m, 0.002)) / (2 * step))
        errs.append(abs(fd - gp[i, j]) / (np.abs(gp[i]).max() + 1e-30))
    assert max(errs) < 1e-4


def test_autograd_and_batched_launch():
    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.adjoint import BindingEnergy, energy_gradient
    from hbtplus_gb300.unbind import Unbinder
    subs = [_subhalo(n, 10 + k, center=(20.0 + 10 * k, 40.0, 60.0)) for k, n in
            enumerate((400, 2500, 90))]
    b = S.concat(subs)
    p = S.default_params()
    with Unbinder(p) as ub:
        pos = torch.tensor(b["pos"], device="cuda", requires_grad=True)
        vel = torch.tensor(b["vel"], device="cuda", requires_grad=True)
        mass = torch.tensor(b["mass"], device="cuda", requires_grad=True)
        E = BindingEnergy.apply(pos, vel, mass, ub, b["offsets"], b["ref_pos"], b["ref_vel"])
        w = torch.tensor([1.0, 2.0, -0.5], dtype=torch.float64, device="cuda")
        (E * w).sum().backward()
        off = b["offsets"]
        for s in range(3):
            a, z = int(off[s]), int(off[s + 1])
            Es, gp, gv, gm = energy_gradient(ub, pos[a:z], vel[a:z], mass[a:z], [0, z - a],
                                             b["ref_pos"][s:s + 1], b["ref_vel"][s:s + 1])
            # each target's walk and sums are its own: batched and single calls agree
            assert float(Es[0]) == float(E[s].detach())
            for got, ref in ((pos.grad[a:z], gp), (vel.grad[a:z], gv), (mass.grad[a:z], gm)):
                ref = (ref * float(w[s])).cpu().numpy()
                assert _rel(got.cpu().numpy(), ref) < 1e-5


def test_million_particle_subhalo_gradients():
    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.adjoint import energy_gradient
    from hbtplus_gb300.unbind import Unbinder
    rng = np.random.Generator(np.random.PCG64(20261206))
    sub = S.nfw_subhalo(rng, 1_000_000, 0.2 * 10 ** (1 / 3), 10.0, contaminant_frac=0.0,
                        center=(50.0, 50.0, 50.0))
    m = sub["mass"].astype(np.float64)
    sub["ref_pos"] = (np.sum(sub["pos"] * m[:, None], 0) / m.sum()).astype(np.float32)
    sub["ref_vel"] = (np.sum(sub["vel"] * m[:, None], 0) / m.sum()).astype(np.float32)
    with Unbinder(S.default_params()) as ub:
        t = {k: torch.from_numpy(np.ascontiguousarray(sub[k])).cuda() for k in ("pos", "vel", "mass")}
        E, gp, gv, gm = energy_gradient(ub, t["pos"], t["vel"], t["mass"], [0, 1_000_000],
                                        sub["ref_pos"][None], sub["ref_vel"][None])
    x = torch.tensor(sub["pos"], dtype=torch.float64, device="cuda")
    mm = torch.tensor(m, device="cuda")
    v = torch.tensor(sub["vel"], dtype=torch.float64, device="cuda")
    X = torch.tensor(sub["ref_pos"], dtype=torch.float64, device="cuda")
    V = torch.tensor(sub["ref_vel"], dtype=torch.float64, device="cuda")
    idx = torch.as_tensor(np.random.default_rng(5).choice(1_000_000, 1000, replace=False),
                          device="cuda")
    phi, gphi = direct(x[idx], x, mm, 0.002, skip_self_index=idx)
    dv = v[idx] - V + HZ * (x[idx] - X)
    ref = (mm[idx][:, None] * (HZ * dv + gphi)).cpu().numpy()
    got = gp[idx].cpu().numpy()
    assert _rel(got, ref) < 2e-2
    # momentum balance: sum_k m_k grad phi_k vanishes for a pairwise sum
    mg = gp.double() - mm[:, None] * HZ * (torch.tensor(sub["vel"], dtype=torch.float64,
                                                         device="cuda") - V + HZ * (x - X))
    assert float(mg.sum(0).norm()) <= 2e-3 * float(mg.norm(dim=1).sum())


def test_batched_backward_of_the_2000_subhalo_batch():
    """Config 3's batch form: the 2000-subhalo workload (867,289 particles)
    unbound, then every subhalo's bound set differentiated in one call."""
    import time

    torch = pytest.importorskip("torch")
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.adjoint import bound_subset, energy_gradient
    from hbtplus_gb300.unbind import Unbinder
    batch = S.subhalo_batch(nsub=2000, seed=20261204)
    p = S.default_params()
    with Unbinder(p) as ub:
        order, _, res = ub.unbind_batch(batch)
        b = bound_subset(batch, order, res)
        t = {k: torch.from_numpy(b[k]).cuda() for k in ("pos", "vel", "mass")}
        E, gp, gv, gm = energy_gradient(ub, t["pos"], t["vel"], t["mass"], b["offsets"],
                                        b["ref_pos"], b["ref_vel"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            energy_gradient(ub, t["pos"], t["vel"], t["mass"], b["offsets"], b["ref_pos"],
                            b["ref_vel"])
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / 3
        print(f"batched backward: {len(b['mass'])} bound particles in 2000 subhaloes, "
              f"{1e3 * dt:.2f} ms per call")
        off = b["offsets"]
        sizes = np.diff(off)
        picks = list(np.argsort(sizes)[-5:]) + list(np.random.default_rng(8).choice(2000, 25))
        for s in picks:
            a, z = int(off[s]), int(off[s + 1])
            if z - a == 0:
                continue
            Es, gps, gvs, gms = energy_gradient(ub, t["pos"][a:z], t["vel"][a:z], t["mass"][a:z],
                                                [0, z - a], b["ref_pos"][s:s + 1],
                                                b["ref_vel"][s:s + 1])
            assert float(Es[0]) == float(E[s]), s
            assert torch.equal(gps, gp[a:z]) and torch.equal(gvs, gv[a:z]), s
            assert torch.equal(gms, gm[a:z]), s
    # FP64 direct-sum gradients of 1000 random bound particles, each from its own
    # subhalo's bound set (positions relative to the frame, periodic wrap)
    rng = np.random.default_rng(9)
    idx = np.sort(rng.choice(len(b["mass"]), 1000, replace=False))
    sub_of = np.searchsorted(off, idx, side="right") - 1
    got = gp[torch.as_tensor(idx, device="cuda")].double().cpu().numpy()
    ref = np.empty_like(got)
    for s in np.unique(sub_of):
        a, z = int(off[s]), int(off[s + 1])
        sel = idx[sub_of == s]
        x = b["pos"][a:z].astype(np.float64) - b["ref_pos"][s].astype(np.float64)
        x = np.where(x > 50.0, x - 100.0, np.where(x < -50.0, x + 100.0, x))
        xt = torch.tensor(x, device="cuda")
        m = torch.tensor(b["mass"][a:z], dtype=torch.float64, device="cuda")
        v = torch.tensor(b["vel"][a:z], dtype=torch.float64, device="cuda")
        V = torch.tensor(b["ref_vel"][s], dtype=torch.float64, device="cuda")
        loc = torch.as_tensor(sel - a, device="cuda")
        phi, gphi = direct(xt[loc], xt, m, 0.002, skip_self_index=loc)
        dv = v[loc] - V + HZ * xt[loc]
        ref[sub_of == s] = (m[loc][:, None] * (HZ * dv + gphi)).cpu().numpy()
    print(f"batched backward vs FP64 direct sum on 1000 particles: rel L2 {_rel(got, ref):.2e}")
    assert _rel(got, ref) < 2e-2
