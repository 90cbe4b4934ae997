"""hbtplus_gb300 -- HBT+ subhalo unbinding (Subhalo_t::Unbind) on GB300 (sm_103a).

The CUDA library libhbtu.so (built in-tree by hbtplus_gb300.build) implements
the C ABI of include/hbtu.h.  The Python host side over it:

    unbind     Unbinder: Unbind, the batched unbinding, binding energies,
               profile and shape properties, merge trap detection
    refine     RecursiveUnbind + TruncateSource over a forest, batched by depth
    merge      MergeSubhalos: traps, MergeTo unions, re-unbinding
    index      particle-ID tables (MappedIndexTable / FlatIndexTable)
    step       the tracking step: ID table, re-resolve, gather, unbind, properties
    adjoint    gradient of the binding energy (torch.autograd.Function)
    shard      the multi-GPU shard planner
    synthetic  the seeded workloads
"""
from . import synthetic  # noqa: F401

__all__ = ["adjoint", "build", "index", "merge", "refine", "shard", "step", "synthetic",
           "unbind"]
