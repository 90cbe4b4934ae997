"""hbtplus_gb300 -- HBT+ subhalo unbinding (Subhalo_t::Unbind) on GB300 (sm_103a).

The CUDA library libhbtu.so (built in-tree by hbtplus_gb300.build) implements
the C ABI of include/hbtu.h; hbtplus_gb300.unbind is the Python host API over
it and hbtplus_gb300.synthetic generates the seeded workloads.
"""
from . import synthetic  # noqa: F401

__all__ = ["synthetic", "unbind", "build"]
