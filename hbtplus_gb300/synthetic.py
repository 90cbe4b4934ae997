"""Seeded synthetic subhalo populations for the unbinding workloads.

No public particle suite is used by the reference's unbinding path, so the
workloads are generated here: truncated NFW haloes with isotropic
Jeans-equation Maxwellian velocities plus unbound contaminants, placed in a
periodic box.  Units are the reference's defaults (1e10 Msun/h, Mpc/h, km/s),
for which PhysicalConst::G = 43.0071 (src/config_parser.cpp:95) and, at a=1,
Hz = 100 (src/snapshot.h:27-38 with H0 = 100).

Workloads (numpy.random.Generator(PCG64), seed 20261203 + index):
  single_subhalo()  1e5 NFW particles (r200 = 0.2, c = 10, m = 1e-4) plus
                    10% contaminants in a 0.4 Mpc/h sphere moving at three
                    times the local escape speed; random centre in a 100 Mpc/h
                    box; ids a random permutation.
  subhalo_batch()   2000 subhaloes, N from dN/dlnN ~ N^-0.9 on [20, 2e5],
                    c ~ U(5, 20), r200 = 0.2 (N/1e5)^(1/3), 20% contaminants,
                    about 5% of centres within r200 of a box face.
  host_with_clumps() a 2e7-particle NFW host (r200 = 1, c = 5) with 300 Plummer
                    clumps (1e3-1e5 particles, a = 0.01) and 5% contaminants.

A subhalo is a dict with id (int64), pos/vel (n,3 float32), mass, type
(int32), ref_pos/ref_vel (initial frame), mostbound_pos/mostbound_vel
(= particle 0, the particle nearest the centre).  A batch concatenates
subhaloes and adds offsets (nsub+1,) and per-subhalo (nsub,3) frames.
"""
from __future__ import annotations

import numpy as np

G_MPC_KMS = 43.0071
HUBBLE_A1 = 100.0


def default_params(**over) -> dict:
    """The unbinding parameters of the workloads (reference defaults, exact tree)."""
    p = dict(softening=0.002, open_angle=0.45, bound_mass_precision=0.995,
             min_num_part=20, max_sample_size=0, refine_mostbound=1, periodic=1,
             box_size=100.0, G=G_MPC_KMS, hubble=HUBBLE_A1, scale_factor=1.0)
    p.update(over)
    return p


def _mnfw(x):
    return np.log1p(x) - x / (1.0 + x)


def _nfw_profile_tables(c: float, ngrid: int = 2048):
    """Dimensionless radius grid x = r/rs in (0, c], enclosed-mass fraction,
    isotropic Jeans sigma_r^2 in units of G*M/rs, and potential in the same units."""
    x = np.geomspace(1e-6 * c, c, ngrid)
    mc = _mnfw(c)
    menc = _mnfw(x) / mc
    # sigma_r^2(x) = x(1+x)^2 / m(c) * int_x^c m(x') / (x'^3 (1+x')^2) dx'
    integrand = _mnfw(x) / (x ** 3 * (1.0 + x) ** 2)
    seg = 0.5 * (integrand[1:] + integrand[:-1]) * np.diff(x)
    tail = np.concatenate([np.cumsum(seg[::-1])[::-1], [0.0]])
    sig2 = x * (1.0 + x) ** 2 * tail / mc
    # phi(x) = -[m(x)/x + 1/(1+x) - 1/(1+c)] / m(c)   (truncated at r200)
    phi = -(_mnfw(x) / x + 1.0 / (1.0 + x) - 1.0 / (1.0 + c)) / mc
    return x, menc, sig2, phi


def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def nfw_subhalo(rng, n: int, r200: float, c: float, m: float = 1e-4,
                contaminant_frac: float = 0.1, contaminant_radius_factor: float = 2.0,
                center=None, bulk_velocity=(0.0, 0.0, 0.0), box: float = 100.0):
    """One NFW subhalo with Jeans velocities plus unbound contaminants."""
    rs = r200 / c
    mtot = n * m
    x, menc, sig2, phi = _nfw_profile_tables(c)
    u = rng.uniform(size=n)
    xr = np.interp(u, menc, x)
    r = xr * rs
    pos = _unit_vectors(rng, n) * r[:, None]
    sig = np.sqrt(np.maximum(np.interp(xr, x, sig2), 0.0) * G_MPC_KMS * mtot / rs)
    vel = rng.normal(size=(n, 3)) * sig[:, None]
    ncont = int(round(contaminant_frac * n))
    if ncont:
        rc = contaminant_radius_factor * r200 * rng.uniform(size=ncont) ** (1.0 / 3.0)
        xc = rc / rs
        phic = np.where(xc <= c, np.interp(np.minimum(xc, c), x, phi) * G_MPC_KMS * mtot / rs,
                        -G_MPC_KMS * mtot / np.maximum(rc, 1e-12))
        vesc = np.sqrt(2.0 * np.abs(phic))
        pos = np.concatenate([pos, _unit_vectors(rng, ncont) * rc[:, None]])
        vel = np.concatenate([vel, _unit_vectors(rng, ncont) * (3.0 * vesc)[:, None]])
    ntot = len(pos)
    if center is None:
        center = rng.uniform(0.0, box, size=3)
    center = np.asarray(center, np.float64)
    # previous most-bound particle: the one nearest the centre, moved to slot 0
    perm = np.arange(ntot)
    if ntot:
        k = int(np.argmin(np.einsum("ij,ij->i", pos, pos)))
        perm[0], perm[k] = k, 0
    pos = pos[perm]
    vel = vel[perm]
    absolute = np.mod(pos + center, box)
    absolute = np.where(absolute >= box, absolute - box, absolute)
    pos32 = absolute.astype(np.float32)
    pos32 = np.where(pos32 >= np.float32(box), np.float32(0.0), pos32)
    vel32 = (vel + np.asarray(bulk_velocity)).astype(np.float32)
    mass = np.full(ntot, m, np.float32)
    typ = np.ones(ntot, np.int32)
    return dict(pos=pos32, vel=vel32, mass=mass, type=typ,
                ref_pos=center.astype(np.float32),
                ref_vel=np.asarray(bulk_velocity, np.float32),
                mostbound_pos=pos32[0].copy() if ntot else np.zeros(3, np.float32),
                mostbound_vel=vel32[0].copy() if ntot else np.zeros(3, np.float32))


def _assign_ids(rng, subs):
    ntot = sum(len(s["mass"]) for s in subs)
    ids = rng.permutation(ntot).astype(np.int64)
    o = 0
    for s in subs:
        n = len(s["mass"])
        s["id"] = ids[o:o + n].copy()
        s["mostbound_id"] = int(s["id"][0]) if n else -1
        o += n


def single_subhalo(n: int = 100_000, seed: int = 20261203, r200: float = 0.2, c: float = 10.0,
                   contaminant_frac: float = 0.1, box: float = 100.0) -> dict:
    """The 1e5-particle isolated NFW subhalo (+10% contaminants), seeded."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sub = nfw_subhalo(rng, n, r200, c, contaminant_frac=contaminant_frac, box=box)
    _assign_ids(rng, [sub])
    return sub


def plummer(rng, n: int, a: float, m: float = 1e-4, rmax_factor: float = 10.0):
    """Plummer sphere of n particles (scale radius a, truncated at rmax_factor*a)
    with isotropic Gaussian velocities, sigma^2(r) = G M / (6 sqrt(r^2 + a^2))."""
    mt = n * m
    fmax = rmax_factor ** 3 / (1.0 + rmax_factor ** 2) ** 1.5  # mass fraction inside rmax
    u = rng.uniform(size=n) * fmax
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    pos = _unit_vectors(rng, n) * r[:, None]
    sig = np.sqrt(G_MPC_KMS * mt / (6.0 * np.sqrt(r * r + a * a)))
    vel = rng.normal(size=(n, 3)) * sig[:, None]
    return pos, vel


def host_with_clumps(n_host: int = 20_000_000, r200: float = 1.0, c: float = 5.0,
                     nclumps: int = 300, clump_min: float = 1e3, clump_max: float = 1e5,
                     clump_a: float = 0.01, contaminant_frac: float = 0.05,
                     seed: int = 20261205, box: float = 100.0, m: float = 1e-4) -> dict:
    """Large host subhalo: NFW host (r200 = 1 Mpc/h, c = 5) with Jeans velocities,
    nclumps Plummer satellites (sizes log-uniform in [1e3, 1e5], scale radius
    0.01 Mpc/h) placed on the host profile with orbital velocities drawn from the
    host's dispersion there, plus unbound contaminants (5% of the total)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rs = r200 / c
    mtot_host = n_host * m
    x, menc, sig2, phi = _nfw_profile_tables(c)
    xr = np.interp(rng.uniform(size=n_host), menc, x)
    pos = [(_unit_vectors(rng, n_host) * (xr * rs)[:, None]).astype(np.float64)]
    sig = np.sqrt(np.maximum(np.interp(xr, x, sig2), 0.0) * G_MPC_KMS * mtot_host / rs)
    vel = [rng.normal(size=(n_host, 3)) * sig[:, None]]
    del xr, sig
    sizes = np.exp(rng.uniform(np.log(clump_min), np.log(clump_max), size=nclumps)).astype(np.int64)
    for k in range(nclumps):
        xc = np.interp(rng.uniform(0.05, 0.95), menc, x)
        cpos = _unit_vectors(rng, 1)[0] * xc * rs
        csig = np.sqrt(max(np.interp(xc, x, sig2), 0.0) * G_MPC_KMS * mtot_host / rs)
        cvel = rng.normal(size=3) * csig
        p, v = plummer(rng, int(sizes[k]), clump_a, m)
        pos.append(p + cpos)
        vel.append(v + cvel)
    n_in = n_host + int(sizes.sum())
    ncont = int(round(contaminant_frac / (1.0 - contaminant_frac) * n_in))
    rc = 2.0 * r200 * rng.uniform(size=ncont) ** (1.0 / 3.0)
    xcn = rc / rs
    phic = np.where(xcn <= c, np.interp(np.minimum(xcn, c), x, phi) * G_MPC_KMS * mtot_host / rs,
                    -G_MPC_KMS * mtot_host / np.maximum(rc, 1e-12))
    pos.append(_unit_vectors(rng, ncont) * rc[:, None])
    vel.append(_unit_vectors(rng, ncont) * (3.0 * np.sqrt(2.0 * np.abs(phic)))[:, None])
    pos = np.concatenate(pos)
    vel = np.concatenate(vel)
    center = rng.uniform(0.0, box, size=3)
    k0 = int(np.argmin(np.einsum("ij,ij->i", pos, pos)))
    pos[[0, k0]] = pos[[k0, 0]]
    vel[[0, k0]] = vel[[k0, 0]]
    pos32 = np.mod(pos + center, box).astype(np.float32)
    pos32 = np.where(pos32 >= np.float32(box), np.float32(0.0), pos32)
    del pos
    ntot = len(pos32)
    sub = dict(pos=pos32, vel=vel.astype(np.float32), mass=np.full(ntot, m, np.float32),
               type=np.ones(ntot, np.int32), ref_pos=center.astype(np.float32),
               ref_vel=np.zeros(3, np.float32))
    sub["mostbound_pos"] = sub["pos"][0].copy()
    sub["mostbound_vel"] = sub["vel"][0].copy()
    sub["id"] = rng.permutation(ntot).astype(np.int64)
    sub["mostbound_id"] = int(sub["id"][0])
    return sub


def batch_sizes(rng, nsub: int, nmin: float = 20, nmax: float = 2e5, slope: float = -0.9):
    """N drawn from dN/dlnN ~ N^slope on [nmin, nmax] (inverse CDF in ln N)."""
    a, b = np.log(nmin), np.log(nmax)
    u = rng.uniform(size=nsub)
    k = slope
    lnN = np.log(np.exp(k * a) + u * (np.exp(k * b) - np.exp(k * a))) / k
    return np.maximum(np.floor(np.exp(lnN)).astype(np.int64), int(nmin))


def subhalo_batch(nsub: int = 2000, seed: int = 20261204, box: float = 100.0,
                  nmin: float = 20, nmax: float = 2e5, slope: float = -0.9,
                  contaminant_frac: float = 0.2, face_frac: float = 0.05,
                  bulk_sigma: float = 300.0) -> dict:
    """The 2000-subhalo batch (power-law sizes), seeded; sorted by nothing."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = batch_sizes(rng, nsub, nmin, nmax, slope)
    subs = []
    for s in range(nsub):
        n = int(sizes[s])
        c = rng.uniform(5.0, 20.0)
        r200 = 0.2 * (n / 1e5) ** (1.0 / 3.0)
        center = rng.uniform(0.0, box, size=3)
        if rng.uniform() < face_frac:  # straddle a box face
            d = rng.integers(3)
            center[d] = rng.uniform(-r200, r200) % box
        bulk = rng.normal(scale=bulk_sigma, size=3)
        subs.append(nfw_subhalo(rng, n, r200, c, contaminant_frac=contaminant_frac,
                                center=center, bulk_velocity=bulk, box=box))
    _assign_ids(rng, subs)
    return concat(subs)


def concat(subs) -> dict:
    """Concatenate subhalo dicts into a batch dict with offsets."""
    counts = np.array([len(s["mass"]) for s in subs], np.int64)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    out = dict(offsets=off)
    for k in ("id", "mass", "type"):
        out[k] = np.concatenate([s[k] for s in subs]) if subs else np.zeros(0)
    for k in ("pos", "vel"):
        out[k] = np.concatenate([s[k] for s in subs]) if subs else np.zeros((0, 3), np.float32)
    for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
        out[k] = np.stack([s[k] for s in subs]).astype(np.float32)
    out["mostbound_id"] = np.array([s["mostbound_id"] for s in subs], np.int64)
    out["id"] = out["id"].astype(np.int64)
    out["mass"] = out["mass"].astype(np.float32)
    out["type"] = out["type"].astype(np.int32)
    return out


def split(batch: dict, s: int) -> dict:
    """Subhalo s of a batch as a single-subhalo dict."""
    o0, o1 = int(batch["offsets"][s]), int(batch["offsets"][s + 1])
    sub = {k: batch[k][o0:o1] for k in ("id", "pos", "vel", "mass", "type")}
    for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
        sub[k] = batch[k][s]
    sub["mostbound_id"] = int(batch["mostbound_id"][s])
    return sub


def tracking_snapshot(nsub: int = 20_000, ntot: int = 30_000_000, box: float = 200.0,
                      seed: int = 20261207, drift: float = 1e-4, strip: float = 0.1) -> dict:
    """A tracking step's inputs: the new snapshot and the subhaloes of the last one.

    The subhaloes of the 2000-subhalo law, nsub of them in a `box` Mpc/h box,
    plus uniform background particles up to `ntot`.  Particle IDs are a sparse
    random permutation (3 * k + 1), so the ID table is a mapped one.  The new
    snapshot moves every particle by v * drift (Mpc/h per km/s, periodic) and
    stores particles in a fresh random order, so the subhaloes' particle IDs
    must be re-resolved.  Each subhalo keeps the inner (1 - strip) of its
    particles (by distance to its frame centre; its first particle, the
    previous most-bound one, stays first).

    Returns dict(snap_id, snap_pos, snap_vel, snap_mass, snap_type: the new
    snapshot, in its own order; offsets, member_id: each subhalo's particle IDs;
    ref_pos, ref_vel, mostbound_pos, mostbound_vel, mostbound_id: the frames
    the unbinding starts from)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    subs = subhalo_batch(nsub=nsub, seed=seed + 1, box=box)
    nin = int(subs["offsets"][-1])
    nbg = max(0, ntot - nin)
    ntot = nin + nbg
    pos = np.concatenate([subs["pos"], rng.uniform(0.0, box, size=(nbg, 3)).astype(np.float32)])
    vel = np.concatenate([subs["vel"],
                          rng.normal(scale=300.0, size=(nbg, 3)).astype(np.float32)])
    mass = np.concatenate([subs["mass"], np.full(nbg, 1e-4, np.float32)])
    typ = np.concatenate([subs["type"], np.ones(nbg, np.int32)])
    ids = rng.permutation(ntot).astype(np.int64) * 3 + 1
    # the last snapshot's membership, stripped of each subhalo's outer particles
    off = subs["offsets"]
    keep_off = [0]
    members = []
    for s in range(nsub):
        o0, o1 = int(off[s]), int(off[s + 1])
        n = o1 - o0
        if n == 0:
            keep_off.append(keep_off[-1])
            continue
        d = pos[o0:o1].astype(np.float64) - subs["ref_pos"][s].astype(np.float64)
        d -= box * np.round(d / box)
        r2 = np.einsum("ij,ij->i", d, d)
        nkeep = max(1, int(round((1.0 - strip) * n)))
        order = np.argsort(r2[1:], kind="stable")[: nkeep - 1] + 1
        idx = np.concatenate([[0], np.sort(order)]) + o0
        members.append(ids[idx])
        keep_off.append(keep_off[-1] + len(idx))
    # the new snapshot: drifted, in a new order
    newpos = np.mod(pos + vel * np.float32(drift), np.float32(box)).astype(np.float32)
    newpos = np.where(newpos >= np.float32(box), np.float32(0.0), newpos)
    perm = rng.permutation(ntot)
    return dict(snap_id=ids[perm], snap_pos=newpos[perm], snap_vel=vel[perm],
                snap_mass=mass[perm], snap_type=typ[perm],
                offsets=np.array(keep_off, np.int64),
                member_id=np.concatenate(members) if members else np.zeros(0, np.int64),
                ref_pos=subs["ref_pos"], ref_vel=subs["ref_vel"],
                mostbound_pos=subs["mostbound_pos"], mostbound_vel=subs["mostbound_vel"],
                mostbound_id=ids[off[:-1]].astype(np.int64))
