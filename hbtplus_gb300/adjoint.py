"""Adjoint of the binding energy behind torch.autograd.Function.

E_tot(s) = sum_i m_i |dv_i|^2 / 2 + 1/2 sum_i m_i phi_i over the particles of
subhalo s (for example its bound set after unbinding), with dv_i the velocity
relative to the frame (Snapshot_t::RelativeVelocity, src/snapshot.h:100-111)
and phi_i the tree potential of the unbinding walk (src/gravity_tree.cpp:79-164);
the factor 1/2 undoes the double counting of pairs (src/subhalo.h:65).  The
gradients are the gravitational accelerations used for tidal diagnostics:

    dE/dv = m dv,   dE/dx = m (H a dv + grad phi),   dE/dm = |dv|^2 / 2 + phi

(frame at the centre of mass, so its own dependence cancels).  Forward
computes E_tot with one energy walk; backward recomputes the walk with
gradients (hbtu_energy_gradient) instead of storing anything.  Both run in
libhbtu.so on the GPU; a batch of subhaloes is one launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .unbind import Unbinder, _state


def _states(ref_pos, ref_vel):
    nsub = len(ref_pos)
    sts = (_lib.hbtu_state * max(nsub, 1))()
    for s in range(nsub):
        sts[s] = _state(ref_pos[s], ref_vel[s], ref_pos[s], ref_vel[s], -1)
    return sts


def bound_subset(batch: dict, order, results) -> dict:
    """The bound particles of every subhalo of an unbound batch (most bound
    first, as Unbind leaves Particles[0..Nbound)) with its final frame: the
    fixed particle sets whose binding energy is differentiated.  ``order`` and
    ``results`` are what Unbinder.unbind_batch returned for ``batch``."""
    off = np.asarray(batch["offsets"], np.int64)
    rows, counts = [], []
    for s in range(len(off) - 1):
        nb = int(results[s]["nbound"])
        rows.append(int(off[s]) + np.asarray(order[int(off[s]):int(off[s]) + nb], np.int64))
        counts.append(nb)
    rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    out = {k: np.ascontiguousarray(np.asarray(batch[k])[rows]) for k in ("pos", "vel", "mass")}
    out["offsets"] = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    out["ref_pos"] = np.array([r["ref_pos"] for r in results], np.float32).reshape(-1, 3)
    out["ref_vel"] = np.array([r["ref_vel"] for r in results], np.float32).reshape(-1, 3)
    return out


def energy_gradient(ub: Unbinder, pos: torch.Tensor, vel: torch.Tensor, mass: torch.Tensor,
                    offsets, ref_pos, ref_vel, with_grad: bool = True):
    """E_tot per subhalo (float64, device) and, if asked, the gradients
    (float32, device) of device-resident particles pos (N,3), vel (N,3), mass (N)."""
    dev = pos.device
    off = np.ascontiguousarray(offsets, np.int64)
    nsub = len(off) - 1
    n = int(off[-1])
    pos = pos.detach().contiguous().float()
    vel = vel.detach().contiguous().float()
    mass = mass.detach().contiguous().float()
    ids = torch.arange(n, dtype=torch.int64, device=dev)
    p = _lib.hbtu_particles(id=ids.data_ptr(), pos=pos.data_ptr(), vel=vel.data_ptr(),
                            mass=mass.data_ptr(), type=0, location=_lib.HBTU_DEVICE, reserved=0)
    E = torch.empty(max(nsub, 1), dtype=torch.float64, device=dev)
    gp = gv = gm = None
    ptrs = [0, 0, 0]
    if with_grad:
        gp = torch.empty((n, 3), dtype=torch.float32, device=dev)
        gv = torch.empty((n, 3), dtype=torch.float32, device=dev)
        gm = torch.empty(n, dtype=torch.float32, device=dev)
        ptrs = [gp.data_ptr(), gv.data_ptr(), gm.data_ptr()]
    sts = _states(np.asarray(ref_pos, np.float32), np.asarray(ref_vel, np.float32))
    ub.set_stream(torch.cuda.current_stream(dev).cuda_stream)
    rc = ub.lib.hbtu_energy_gradient(ub.handle, C.byref(p), nsub, off.ctypes.data,
                                     C.addressof(sts), E.data_ptr(), *ptrs)
    _lib.check(rc, ub.handle)
    return E[:nsub], gp, gv, gm


class BindingEnergy(torch.autograd.Function):
    """E = BindingEnergy.apply(pos, vel, mass, unbinder, offsets, ref_pos, ref_vel):
    total binding energy of every subhalo (shape (nsub,), float64); backward
    gives d(sum_s w_s E_s)/d(pos, vel, mass) for the incoming weights w."""

    @staticmethod
    def forward(ctx, pos, vel, mass, unbinder, offsets, ref_pos, ref_vel):
        E, _, _, _ = energy_gradient(unbinder, pos, vel, mass, offsets, ref_pos, ref_vel,
                                     with_grad=False)
        ctx.save_for_backward(pos, vel, mass)
        ctx.unbinder = unbinder
        ctx.offsets = np.asarray(offsets, np.int64)
        ctx.frames = (ref_pos, ref_vel)
        return E

    @staticmethod
    def backward(ctx, gE):
        pos, vel, mass = ctx.saved_tensors
        _, gp, gv, gm = energy_gradient(ctx.unbinder, pos, vel, mass, ctx.offsets,
                                        ctx.frames[0], ctx.frames[1], with_grad=True)
        counts = torch.as_tensor(np.diff(ctx.offsets), device=pos.device)
        w = torch.repeat_interleave(gE.to(torch.float32), counts)
        return (gp * w[:, None]).to(pos.dtype), (gv * w[:, None]).to(vel.dtype), \
            (gm * w).to(mass.dtype), None, None, None, None
