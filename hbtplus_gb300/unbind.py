"""Python host API over the C ABI, mirroring the reference's unbinding interface.

Reference interface (HBT+ 1.16.2):
  Parameter_t (src/config_parser.h:22-123)       -> Parameters
  Cosmology_t (src/snapshot.h:17-39)             -> Cosmology
  Subhalo_t::Unbind (src/subhalo_unbind.cpp:263) -> Unbinder.unbind
  the per-subhalo loops of RefineParticles       -> Unbinder.unbind_batch
  (src/subhalo_unbind.cpp:460-516)
  GravityTree_t::BindingEnergy over all particles -> Unbinder.binding_energies

Everything here is marshalling; the work runs in libhbtu.so on the GPU, and
there is no CPU fallback: constructing an Unbinder without a compute
capability 10.3 device raises.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib

# keys of the reference configuration file (src/config_parser.cpp:12-72)
_COMPULSORY = ("SnapshotPath", "HaloPath", "SubhaloPath", "SnapshotFileBase",
               "MaxSnapshotIndex", "BoxSize", "SofteningHalo")
_OPTIONAL = ("SnapshotFormat", "GroupFileFormat", "MaxConcurrentIO", "MinSnapshotIndex",
             "MinNumPartOfSub", "GroupParticleIdMask", "MassInMsunh", "LengthInMpch",
             "VelInKmS", "PeriodicBoundaryOn", "SnapshotHasIdBlock", "ParticleIdRankStyle",
             "ParticleIdNeedHash", "SnapshotIdUnsigned", "SaveSubParticleProperties",
             "MergeTrappedSubhalos", "MajorProgenitorMassRatio", "BoundMassPrecision",
             "SourceSubRelaxFactor", "SubCoreSizeFactor", "SubCoreSizeMin", "TreeAllocFactor",
             "TreeNodeOpenAngle", "TreeMinNumOfCells", "MaxSampleSizeOfPotentialEstimate",
             "RefineMostboundParticle", "SnapshotIdList")


@dataclass
class Parameters:
    """The unbinding subset of Parameter_t, with the reference's names and
    defaults (src/config_parser.h:77-110)."""
    SofteningHalo: float = 0.0
    BoxSize: float = 0.0
    TreeNodeOpenAngle: float = 0.45
    BoundMassPrecision: float = 0.995
    MinNumPartOfSub: int = 20
    MaxSampleSizeOfPotentialEstimate: int = 1000
    RefineMostboundParticle: bool = True
    PeriodicBoundaryOn: bool = True
    MassInMsunh: float = 1e10
    LengthInMpch: float = 1.0
    VelInKmS: float = 1.0
    extra: dict = field(default_factory=dict)

    @property
    def G(self) -> float:
        """PhysicalConst::G (src/config_parser.cpp:95), rounded to float."""
        g = 43.0071 * (self.MassInMsunh / 1e10) / self.VelInKmS / self.VelInKmS / self.LengthInMpch
        return float(np.float32(g))

    @property
    def H0(self) -> float:
        """PhysicalConst::H0 (src/config_parser.cpp:96)."""
        return 100.0 * (1.0 / self.VelInKmS) / (1.0 / self.LengthInMpch)

    @classmethod
    def from_config_file(cls, path: str) -> "Parameters":
        """Parse a reference configuration file: `Key value` lines, anything
        after `#` or `[` ignored (src/config_parser.cpp:74-109).  Unknown keys
        raise, missing compulsory keys raise."""
        p = cls()
        seen = set()
        with open(path) as f:
            for line in f:
                for mark in "#[":
                    k = line.find(mark)
                    if k >= 0:
                        line = line[:k]
                line = line.strip()
                if not line:
                    continue
                parts = line.split()
                key, vals = parts[0], parts[1:]
                if key not in _COMPULSORY and key not in _OPTIONAL:
                    raise ValueError(f"unrecognized configuration entry: {key}")
                seen.add(key)
                if hasattr(p, key) and key != "extra":
                    cur = getattr(p, key)
                    if isinstance(cur, bool):
                        setattr(p, key, bool(int(vals[0])))
                    elif isinstance(cur, int):
                        setattr(p, key, int(vals[0]))
                    else:
                        setattr(p, key, float(vals[0]))
                else:
                    p.extra[key] = vals
        missing = [k for k in _COMPULSORY if k not in seen]
        if missing:
            raise ValueError(f"compulsory configuration entries missing: {missing}")
        return p


@dataclass
class Cosmology:
    """Cosmology_t of the snapshot being unbound (src/snapshot.h:17-39)."""
    ScaleFactor: float = 1.0
    Hz: float = 100.0

    @classmethod
    def set(cls, scalefactor: float, omega0: float, omega_lambda0: float,
            H0: float = 100.0) -> "Cosmology":
        a = scalefactor
        hratio = math.sqrt(omega0 / a ** 3 + (1 - omega0 - omega_lambda0) / a ** 2 + omega_lambda0)
        return cls(ScaleFactor=float(np.float32(a)), Hz=float(np.float32(hratio * H0)))


def params_from_dict(p: dict, precision: int = _lib.HBTU_PRECISION_FP32, device: int = 0,
                     max_passes: int = 0) -> _lib.hbtu_params:
    return _lib.hbtu_params(
        softening=p["softening"], open_angle=p["open_angle"],
        bound_mass_precision=p["bound_mass_precision"], min_num_part=int(p["min_num_part"]),
        max_sample_size=int(p["max_sample_size"]), refine_mostbound=int(p["refine_mostbound"]),
        periodic=int(p["periodic"]), box_size=p["box_size"], G=p["G"], hubble=p["hubble"],
        scale_factor=p["scale_factor"], precision=precision, max_passes=max_passes,
        device=device, reserved=0)


def params_from_reference(par: Parameters, cosmo: Cosmology,
                          precision: int = _lib.HBTU_PRECISION_FP32, device: int = 0) -> dict:
    return dict(softening=par.SofteningHalo, open_angle=par.TreeNodeOpenAngle,
                bound_mass_precision=par.BoundMassPrecision, min_num_part=par.MinNumPartOfSub,
                max_sample_size=par.MaxSampleSizeOfPotentialEstimate,
                refine_mostbound=int(par.RefineMostboundParticle),
                periodic=int(par.PeriodicBoundaryOn), box_size=par.BoxSize, G=par.G,
                hubble=cosmo.Hz, scale_factor=cosmo.ScaleFactor)


def result_to_dict(r: _lib.hbtu_result) -> dict:
    out = {}
    for name, _ in _lib.hbtu_result._fields_:
        if name == "reserved":
            continue
        v = getattr(r, name)
        out[name] = np.array(list(v)) if hasattr(v, "__len__") else v
    return out


def results_array(results) -> C.Array:
    """Inverse of result_to_dict over a list: a ctypes hbtu_result array."""
    arr = (_lib.hbtu_result * max(len(results), 1))()
    for s, d in enumerate(results):
        for name, _ in _lib.hbtu_result._fields_:
            if name not in d:
                continue
            v = d[name]
            if hasattr(v, "__len__"):
                dst = getattr(arr[s], name)
                for k in range(len(v)):
                    dst[k] = v[k]
            else:
                setattr(arr[s], name, v.item() if hasattr(v, "item") else v)
    return arr


def props_to_dict(p: _lib.hbtu_props) -> dict:
    out = {}
    for name, _ in _lib.hbtu_props._fields_:
        v = getattr(p, name)
        out[name] = np.array(list(v), np.float32) if hasattr(v, "__len__") else v
    return out


def _state(ref_pos, ref_vel, mb_pos, mb_vel, mb_id) -> _lib.hbtu_state:
    s = _lib.hbtu_state()
    for k in range(3):
        s.ref_pos[k] = float(ref_pos[k])
        s.ref_vel[k] = float(ref_vel[k])
        s.mostbound_pos[k] = float(mb_pos[k])
        s.mostbound_vel[k] = float(mb_vel[k])
    s.mostbound_id = int(mb_id)
    return s


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0


class Unbinder:
    """One library handle: parameters, a CUDA stream and a device workspace."""

    def __init__(self, params: dict, precision: int = _lib.HBTU_PRECISION_FP32,
                 device: int = 0, max_passes: int = 0):
        self.lib = _lib.load()
        self.params = dict(params)
        self.precision = precision
        cp = params_from_dict(params, precision, device, max_passes)
        h = C.c_void_p()
        _lib.check(self.lib.hbtu_create(C.byref(cp), C.byref(h)), None)
        self.handle = h

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.hbtu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_option(self, name: str, value: int) -> None:
        _lib.check(self.lib.hbtu_set_option(self.handle, name.encode(), int(value)), self.handle)

    def get_option(self, name: str) -> int:
        v = C.c_int64()
        _lib.check(self.lib.hbtu_get_option(self.handle, name.encode(), C.byref(v)), self.handle)
        return v.value

    def set_timing(self, on: bool) -> None:
        _lib.check(self.lib.hbtu_set_timing(self.handle, int(bool(on))), self.handle)

    def stats(self) -> dict:
        st = _lib.hbtu_stats()
        _lib.check(self.lib.hbtu_get_stats(self.handle, C.byref(st)), self.handle)
        return {k: getattr(st, k) for k, _ in _lib.hbtu_stats._fields_}

    def reset_stats(self) -> None:
        _lib.check(self.lib.hbtu_reset_stats(self.handle), self.handle)

    def set_stream(self, stream_ptr: int) -> None:
        _lib.check(self.lib.hbtu_set_stream(self.handle, C.c_void_p(stream_ptr)), self.handle)

    # -- host-memory calls --------------------------------------------------
    @staticmethod
    def _host_particles(d: dict):
        ids = np.ascontiguousarray(d["id"], np.int64)
        pos = np.ascontiguousarray(d["pos"], np.float32)
        vel = np.ascontiguousarray(d["vel"], np.float32)
        mass = np.ascontiguousarray(d["mass"], np.float32)
        typ = d.get("type")
        typ = np.ascontiguousarray(typ, np.int32) if typ is not None else None
        keep = (ids, pos, vel, mass, typ)
        p = _lib.hbtu_particles(id=_ptr(ids), pos=_ptr(pos), vel=_ptr(vel), mass=_ptr(mass),
                                type=_ptr(typ) if typ is not None else 0,
                                location=_lib.HBTU_HOST, reserved=0)
        return p, keep

    def unbind(self, sub: dict):
        """Unbind one subhalo held in host arrays; returns (order, energy, result)."""
        n = len(sub["mass"])
        p, keep = self._host_particles(sub)
        st = _state(sub["ref_pos"], sub["ref_vel"], sub["mostbound_pos"], sub["mostbound_vel"],
                    sub.get("mostbound_id", sub["id"][0] if n else -1))
        order = np.zeros(max(n, 1), np.int64)
        energy = np.zeros(max(n, 1), np.float32)
        res = _lib.hbtu_result()
        rc = self.lib.hbtu_unbind(self.handle, C.byref(p), n, C.byref(st), _ptr(order),
                                  _ptr(energy), C.addressof(res))
        _lib.check(rc, self.handle)
        del keep
        return order[:n], energy[:n], result_to_dict(res)

    def unbind_batch(self, batch: dict, check_status: bool = True):
        """Unbind every subhalo of a batch held in host arrays."""
        off = np.ascontiguousarray(batch["offsets"], np.int64)
        nsub = len(off) - 1
        ntot = int(off[-1])
        p, keep = self._host_particles(batch)
        sts = (_lib.hbtu_state * max(nsub, 1))()
        for s in range(nsub):
            o = int(off[s])
            mb_id = batch["mostbound_id"][s] if "mostbound_id" in batch else (
                batch["id"][o] if off[s + 1] > o else -1)
            sts[s] = _state(batch["ref_pos"][s], batch["ref_vel"][s], batch["mostbound_pos"][s],
                            batch["mostbound_vel"][s], mb_id)
        order = np.zeros(max(ntot, 1), np.int64)
        energy = np.zeros(max(ntot, 1), np.float32)
        res = (_lib.hbtu_result * max(nsub, 1))()
        rc = self.lib.hbtu_unbind_batch(self.handle, C.byref(p), nsub, _ptr(off),
                                        C.addressof(sts), _ptr(order), _ptr(energy),
                                        C.addressof(res))
        if check_status or rc != _lib.HBTU_ERR_NOT_CONVERGED:
            _lib.check(rc, self.handle)
        del keep
        return order[:ntot], energy[:ntot], [result_to_dict(res[s]) for s in range(nsub)]

    def binding_energies(self, pos, vel, mass, ref_pos, ref_vel, ids=None):
        """First-pass energies (float) and potentials (double) of every particle."""
        n = len(mass)
        d = dict(id=ids if ids is not None else np.arange(n, dtype=np.int64), pos=pos, vel=vel,
                 mass=mass)
        p, keep = self._host_particles(d)
        rp = np.ascontiguousarray(ref_pos, np.float32)
        rv = np.ascontiguousarray(ref_vel, np.float32)
        E = np.zeros(max(n, 1), np.float32)
        pot = np.zeros(max(n, 1), np.float64)
        rc = self.lib.hbtu_binding_energies(self.handle, C.byref(p), n, _ptr(rp), _ptr(rv),
                                            _ptr(E), _ptr(pot))
        _lib.check(rc, self.handle)
        del keep
        return E[:n], pot[:n]

    def direct_potential(self, pos, mass, targets, vel=None, ids=None):
        """Exact FP64 pairwise potentials (G/a included) of particles `targets`
        from all particles: the quantity the tree walk approximates."""
        n = len(mass)
        d = dict(id=ids if ids is not None else np.arange(n, dtype=np.int64), pos=pos,
                 vel=vel if vel is not None else np.zeros((n, 3), np.float32), mass=mass)
        p, keep = self._host_particles(d)
        t = np.ascontiguousarray(targets, np.int64)
        out = np.zeros(max(len(t), 1), np.float64)
        rc = self.lib.hbtu_direct_potential(self.handle, C.byref(p), n, _ptr(t), len(t),
                                            _ptr(out))
        _lib.check(rc, self.handle)
        del keep
        return out[:len(t)]

    # -- device-resident calls (torch tensors on the handle's device) --------
    def unbind_batch_device(self, dev: dict, offsets: np.ndarray, states, out: dict):
        """Batch call on device-resident torch tensors.  ``dev`` holds id, pos,
        vel, mass (and optionally type) CUDA tensors; ``out`` holds order
        (int64), energy (float32) and res (uint8, nsub*sizeof(hbtu_result))
        CUDA tensors.  ``states`` is a ctypes array of hbtu_state."""
        off = np.ascontiguousarray(offsets, np.int64)
        nsub = len(off) - 1
        p = _lib.hbtu_particles(
            id=dev["id"].data_ptr(), pos=dev["pos"].data_ptr(), vel=dev["vel"].data_ptr(),
            mass=dev["mass"].data_ptr(),
            type=dev["type"].data_ptr() if dev.get("type") is not None else 0,
            location=_lib.HBTU_DEVICE, reserved=0)
        rc = self.lib.hbtu_unbind_batch(self.handle, C.byref(p), nsub, _ptr(off),
                                        C.addressof(states), out["order"].data_ptr(),
                                        out["energy"].data_ptr(), out["res"].data_ptr())
        _lib.check(rc, self.handle)

    # -- properties of the bound part (Subhalo_t::CalculateProfileProperties,
    #    ::CalculateShape, src/subhalo.cpp:242-398) ----------------------------
    def subhalo_properties(self, batch: dict, order, results, last_max_vmax=None,
                           last_snap=None, snapshot_index: int = 0):
        """Properties of every subhalo of a batch that unbind_batch has just
        unbound (host arrays): ``order`` and ``results`` as it returned them,
        ``last_max_vmax`` / ``last_snap`` per subhalo before this snapshot.
        Returns one dict per subhalo (hbtu_props fields)."""
        off = np.ascontiguousarray(batch["offsets"], np.int64)
        nsub = len(off) - 1
        d = dict(batch)
        d.setdefault("vel", np.zeros((int(off[-1]), 3), np.float32))
        d.setdefault("id", np.zeros(int(off[-1]), np.int64))
        p, keep = self._host_particles(d)
        ordr = np.ascontiguousarray(order, np.int64)
        res = results_array(results)
        lm = None if last_max_vmax is None else np.ascontiguousarray(last_max_vmax, np.float32)
        ls = None if last_snap is None else np.ascontiguousarray(last_snap, np.int32)
        out = (_lib.hbtu_props * max(nsub, 1))()
        rc = self.lib.hbtu_subhalo_properties(self.handle, C.byref(p), nsub, _ptr(off),
                                              _ptr(ordr), C.addressof(res),
                                              _ptr(lm) if lm is not None else 0,
                                              _ptr(ls) if ls is not None else 0,
                                              int(snapshot_index), C.addressof(out))
        _lib.check(rc, self.handle)
        del keep
        return [props_to_dict(out[s]) for s in range(nsub)]

    def merge_detect(self, parts: dict, list_off, nbound, host, mostbound_pos, mostbound_vel,
                     snapshot_index: int, sink):
        """Cores and trap detection of the merging step (hbtu_merge_detect):
        ``parts`` holds pos, vel and mass of every subhalo's list (bound
        first), concatenated by ``list_off``.  Returns (sink, sink_snap,
        merged, cores); sink_snap is -1 where nothing was trapped now."""
        off = np.ascontiguousarray(list_off, np.int64)
        nsub = len(off) - 1
        n = int(off[-1])
        d = dict(parts)
        d.setdefault("id", np.zeros(n, np.int64))
        p, keep = self._host_particles(d)
        nb = np.ascontiguousarray(nbound, np.int64)
        hs = np.ascontiguousarray(host, np.int64)
        mbp = np.ascontiguousarray(mostbound_pos, np.float32)
        mbv = np.ascontiguousarray(mostbound_vel, np.float32)
        sk = np.ascontiguousarray(sink, np.int64).copy()
        snap = np.full(max(nsub, 1), -1, np.int32)
        merged = np.zeros(max(nsub, 1), np.int32)
        cores = (_lib.hbtu_core * max(nsub, 1))()
        rc = self.lib.hbtu_merge_detect(self.handle, C.byref(p), nsub, _ptr(off), _ptr(nb),
                                        _ptr(hs), _ptr(mbp), _ptr(mbv), int(snapshot_index),
                                        _ptr(sk), _ptr(snap), _ptr(merged), C.addressof(cores))
        _lib.check(rc, self.handle)
        del keep
        cd = [dict(pos=np.array(list(cores[s].pos), np.float32), sigma_r=cores[s].sigma_r,
                   vel=np.array(list(cores[s].vel), np.float32), sigma_v=cores[s].sigma_v)
              for s in range(nsub)]
        return sk[:nsub], snap[:nsub], merged[:nsub], cd

    def subhalo_properties_device(self, dev: dict, offsets: np.ndarray, order, res,
                                  last_max_vmax=None, last_snap=None, snapshot_index: int = 0):
        """subhalo_properties on device-resident torch tensors: ``dev`` holds
        pos and mass, ``order`` and ``res`` are the outputs of
        unbind_batch_device.  Returns the ctypes hbtu_props array."""
        off = np.ascontiguousarray(offsets, np.int64)
        nsub = len(off) - 1
        p = _lib.hbtu_particles(id=0, pos=dev["pos"].data_ptr(), vel=0,
                                mass=dev["mass"].data_ptr(), type=0,
                                location=_lib.HBTU_DEVICE, reserved=0)
        lm = None if last_max_vmax is None else np.ascontiguousarray(last_max_vmax, np.float32)
        ls = None if last_snap is None else np.ascontiguousarray(last_snap, np.int32)
        out = (_lib.hbtu_props * max(nsub, 1))()
        rc = self.lib.hbtu_subhalo_properties(self.handle, C.byref(p), nsub, _ptr(off),
                                              order.data_ptr(), res.data_ptr(),
                                              _ptr(lm) if lm is not None else 0,
                                              _ptr(ls) if ls is not None else 0,
                                              int(snapshot_index), C.addressof(out))
        _lib.check(rc, self.handle)
        return out

    @staticmethod
    def make_states(batch: dict):
        off = batch["offsets"]
        nsub = len(off) - 1
        sts = (_lib.hbtu_state * max(nsub, 1))()
        for s in range(nsub):
            o = int(off[s])
            mb_id = batch["mostbound_id"][s] if "mostbound_id" in batch else (
                batch["id"][o] if off[s + 1] > o else -1)
            sts[s] = _state(batch["ref_pos"][s], batch["ref_vel"][s], batch["mostbound_pos"][s],
                            batch["mostbound_vel"][s], mb_id)
        return sts


def results_from_bytes(buf: bytes, nsub: int):
    arr = (_lib.hbtu_result * max(nsub, 1)).from_buffer_copy(buf)
    return [result_to_dict(arr[s]) for s in range(nsub)]
