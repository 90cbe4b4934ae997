"""A tracking step around the unbinding: ID re-resolve, gather, batched unbind.

Between snapshots the reference keeps each subhalo's particles as IDs and
turns them back into the new snapshot's particles through the snapshot's
ID table (ParticleSnapshot_t::GetIndices, src/snapshot.h:191-224,
src/hash_remote.tpp; ParticleExchanger_t::QueryParticles,
src/particle_exchanger.h:194-208), then unbinds every subhalo
(SubhaloSnapshot_t::RefineParticles, src/subhalo_unbind.cpp:460-516), and
computes each subhalo's profile and shape (Subhalo_t::CalculateProfileProperties
and ::CalculateShape, called at the end of SubhaloSnapshot_t::UpdateTracks,
src/subhalo_tracking.cpp:901-906).  Here the whole step stays on the GPU:

    step = TrackingStep(unbinder, flat=False)
    step.load_snapshot(ids, pos, vel, mass, type)        # CUDA tensors; fills the table
    out, index = step.run(offsets, member_ids, states,   # re-resolve, gather, unbind,
                          properties=dict(snapshot_index=7))   # profile and shape
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .index import FlatIndexTable, MappedIndexTable


class TrackingStep:
    def __init__(self, unbinder, flat: bool = False):
        self.ub = unbinder
        self.table = (FlatIndexTable if flat else MappedIndexTable)(unbinder)
        self.snap = None

    def close(self):
        self.table.close()

    def load_snapshot(self, ids, pos, vel, mass, typ):
        """The new snapshot (CUDA tensors on the handle's device) and its ID
        table: snapshot position i holds particle ids[i]."""
        dev = ids.device
        self.ub.set_stream(torch.cuda.current_stream(dev).cuda_stream)
        self.snap = dict(id=ids.contiguous(), pos=pos.contiguous(), vel=vel.contiguous(),
                         mass=mass.contiguous(), type=typ.contiguous())
        positions = torch.arange(ids.numel(), dtype=torch.int64, device=dev)
        self.table.fill_device(self.snap["id"], positions, null_index=-1)

    def resolve(self, member_ids):
        """Snapshot positions of the members (GetIndices); -1 for an ID the
        snapshot lacks."""
        out = torch.empty_like(member_ids)
        self.table.lookup_device(member_ids.contiguous(), out)
        return out

    def gather(self, index):
        """The members' particles in member order (an ID the snapshot lacks
        raises: the reference drops such particles before unbinding)."""
        if bool((index < 0).any()):
            raise ValueError("a member ID is not in the snapshot")
        return {k: v.index_select(0, index) for k, v in self.snap.items()}

    def run(self, offsets, member_ids, states, properties=None):
        """Re-resolve, gather and unbind every subhalo; returns (order, energy,
        results bytes) as CUDA tensors and the resolved positions.  With
        ``properties`` (a dict of snapshot_index and, optionally, the
        last_max_vmax and last_snap arrays of the subhaloes), out["props"]
        also holds every subhalo's profile and shape (hbtu_props array)."""
        index = self.resolve(member_ids)
        batch = self.gather(index)
        n = member_ids.numel()
        nsub = len(offsets) - 1
        dev = member_ids.device
        out = dict(order=torch.empty(n, dtype=torch.int64, device=dev),
                   energy=torch.empty(n, dtype=torch.float32, device=dev),
                   res=torch.empty(nsub * C.sizeof(_lib.hbtu_result), dtype=torch.uint8,
                                   device=dev))
        self.ub.unbind_batch_device(batch, offsets, states, out)
        if properties is not None:
            out["props"] = self.ub.subhalo_properties_device(
                batch, offsets, out["order"], out["res"],
                last_max_vmax=properties.get("last_max_vmax"),
                last_snap=properties.get("last_snap"),
                snapshot_index=int(properties.get("snapshot_index", 0)))
        return out, index
