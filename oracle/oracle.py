"""ctypes bindings for the CPU oracle (test infrastructure only).

``Oracle()`` loads oracle/_build/libhbt_oracle.so, the C restatement of the
reference unbinding path (hbt_oracle.c).  ``Oracle(reference=True)`` loads
oracle/_ref/libhbt_ref.so, the reference's own Subhalo_t::Unbind compiled
from its unmodified sources (only present where the reference is).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference's sources are (the harness build and the header checks):
# $HBTPLUS_REFERENCE, else the Makefile's default.  Absent on most hosts.
REFERENCE_DIR = os.environ.get("HBTPLUS_REFERENCE") or subprocess.run(
    ["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True).stdout.strip()
ORACLE_SO = os.path.join(HERE, "_build", "libhbt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhbt_ref.so")


class Params(C.Structure):
    _fields_ = [
        ("softening", C.c_double),
        ("open_angle", C.c_double),
        ("bound_mass_precision", C.c_double),
        ("min_num_part", C.c_int64),
        ("max_sample_size", C.c_int64),
        ("refine_mostbound", C.c_int32),
        ("periodic", C.c_int32),
        ("box_size", C.c_double),
        ("G", C.c_double),
        ("hubble", C.c_double),
        ("scale_factor", C.c_double),
    ]


class State(C.Structure):
    _fields_ = [
        ("ref_pos", C.c_float * 3),
        ("ref_vel", C.c_float * 3),
        ("mostbound_pos", C.c_float * 3),
        ("mostbound_vel", C.c_float * 3),
        ("mostbound_id", C.c_int64),
    ]


class Result(C.Structure):
    _fields_ = [
        ("nbound", C.c_int64),
        ("mbound", C.c_float),
        ("ref_pos", C.c_float * 3),
        ("ref_vel", C.c_float * 3),
        ("mostbound_pos", C.c_float * 3),
        ("mostbound_vel", C.c_float * 3),
        ("specific_potential", C.c_float),
        ("specific_kinetic", C.c_float),
        ("specific_angmom", C.c_float * 3),
        ("nbound_type", C.c_int64 * 6),
        ("mbound_type", C.c_float * 6),
        ("iterations", C.c_int32),
        ("disrupted", C.c_int32),
        ("converged", C.c_int32),
        ("too_few", C.c_int32),
        ("evaluations", C.c_int64),
        ("interactions", C.c_int64),
        ("random_splits", C.c_int64),
    ]


class Core(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("sigma_r", C.c_float), ("vel", C.c_float * 3),
                ("sigma_v", C.c_float)]


class Props(C.Structure):
    _fields_ = [
        ("rmax_comoving", C.c_float), ("vmax_physical", C.c_float),
        ("last_max_vmax_physical", C.c_float), ("snapshot_of_last_max_vmax", C.c_int32),
        ("r2sigma_comoving", C.c_float), ("rhalf_comoving", C.c_float),
        ("r200crit_comoving", C.c_float), ("m200crit", C.c_float),
        ("inertial_tensor", C.c_float * 6), ("inertial_tensor_weighted", C.c_float * 6),
    ]


def props_dict(p: Props) -> dict:
    out = {}
    for name, _ in Props._fields_:
        v = getattr(p, name)
        out[name] = np.array(list(v), np.float32) if hasattr(v, "__len__") else v
    return out


def result_dict(r: Result) -> dict:
    out = {}
    for name, _ in Result._fields_:
        v = getattr(r, name)
        out[name] = np.array(list(v)) if hasattr(v, "__len__") else v
    return out


def make_params(p: dict) -> Params:
    return Params(
        softening=p["softening"], open_angle=p["open_angle"],
        bound_mass_precision=p["bound_mass_precision"],
        min_num_part=int(p["min_num_part"]), max_sample_size=int(p["max_sample_size"]),
        refine_mostbound=int(p["refine_mostbound"]), periodic=int(p["periodic"]),
        box_size=p["box_size"], G=p["G"], hubble=p["hubble"],
        scale_factor=p["scale_factor"])


def make_state(ref_pos, ref_vel, mb_pos, mb_vel, mb_id) -> State:
    s = State()
    for k in range(3):
        s.ref_pos[k] = ref_pos[k]
        s.ref_vel[k] = ref_vel[k]
        s.mostbound_pos[k] = mb_pos[k]
        s.mostbound_vel[k] = mb_vel[k]
    s.mostbound_id = int(mb_id)
    return s


def build(reference: bool = False) -> None:
    """Compile the oracle (and, with reference=True, the reference harness)."""
    target = ["ref", "REF=" + REFERENCE_DIR] if reference else []
    subprocess.run(["make", "-s", "-C", HERE, "-j8"] + target, check=True)


def reference_present() -> bool:
    """True where the reference's sources can be compiled from."""
    return bool(REFERENCE_DIR) and os.path.isdir(os.path.join(REFERENCE_DIR, "src"))


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """The C restatement (default) or the reference build (reference=True)."""

    def __init__(self, reference: bool = False):
        so = REF_SO if reference else ORACLE_SO
        if not os.path.exists(so):
            build(reference)
        self.reference = reference
        self.lib = C.CDLL(so)
        pre = "ref_" if reference else "hbto_"
        self._unbind = getattr(self.lib, pre + "unbind")
        self._batch = getattr(self.lib, pre + "unbind_batch")
        self._energies = getattr(self.lib, pre + "binding_energies")
        self._srand48 = getattr(self.lib, pre + "srand48")
        self._shuffle = self.lib.hbto_reference_shuffle
        self._shuffle.argtypes = [C.c_int64, C.c_uint, C.POINTER(C.c_int64)]
        if not reference:
            self._partition = self.lib.hbto_partition
            self._partition.restype = C.c_int64

    # -- helpers ----------------------------------------------------------
    def srand48(self, seed: int) -> None:
        self._srand48(C.c_long(seed))

    def reference_shuffle(self, n: int, seed: int) -> np.ndarray:
        perm = np.empty(max(n, 1), np.int64)
        self._shuffle(n, seed, _p(perm, C.c_int64))
        return perm[:n]

    def index_lookup(self, keys, values, queries, flat: bool = False, null_index: int = -1,
                     batch: bool = False) -> np.ndarray:
        """Fill a particle-ID table with (keys, values) and look up every query
        (MappedIndexTable_t / FlatIndexTable_t, src/hash.tpp).  batch=True uses
        the reference's GetIndices (reference build only; the mapped table
        expects ascending queries)."""
        k = np.ascontiguousarray(keys, np.int64)
        v = np.ascontiguousarray(values, np.int64)
        q = np.ascontiguousarray(queries, np.int64)
        out = np.empty(max(len(q), 1), np.int64)
        if batch:
            if not self.reference:
                raise ValueError("the batch form exists in the reference build only")
            fn = self.lib.ref_index_lookup_batch
        else:
            fn = getattr(self.lib, ("ref_" if self.reference else "hbto_") + "index_lookup")
        fn.restype = C.c_int
        rc = fn(C.c_int(1 if flat else 0), _p(k, C.c_int64), _p(v, C.c_int64), C.c_int64(len(k)),
                C.c_int64(null_index), _p(q, C.c_int64), C.c_int64(len(q)), _p(out, C.c_int64))
        if rc != 0:
            raise RuntimeError(f"index lookup failed ({rc})")
        return out[:len(q)]

    def unbind_properties(self, params: dict, sub: dict, last_max_vmax: float = 0.0,
                          last_snap: int = -1):
        """The reference's Unbind followed by CalculateProfileProperties and
        CalculateShape (reference build only; the epoch is snapshot 1):
        (order, energy, result, properties)."""
        if not self.reference:
            raise ValueError("exists in the reference build only")
        n = len(sub["mass"])
        ids = np.ascontiguousarray(sub["id"], np.int64)
        pos = np.ascontiguousarray(sub["pos"], np.float32).reshape(-1)
        vel = np.ascontiguousarray(sub["vel"], np.float32).reshape(-1)
        mass = np.ascontiguousarray(sub["mass"], np.float32)
        typ = np.ascontiguousarray(sub.get("type", np.ones(n, np.int32)), np.int32)
        st = State()
        for j in range(3):
            st.ref_pos[j] = float(sub["ref_pos"][j])
            st.ref_vel[j] = float(sub["ref_vel"][j])
            st.mostbound_pos[j] = float(sub["mostbound_pos"][j])
            st.mostbound_vel[j] = float(sub["mostbound_vel"][j])
        st.mostbound_id = int(sub.get("mostbound_id", ids[0] if n else -1))
        order = np.zeros(max(n, 1), np.int64)
        energy = np.zeros(max(n, 1), np.float32)
        res, props = Result(), Props()
        fn = self.lib.ref_unbind_properties
        fn.restype = C.c_int
        rc = fn(C.byref(make_params(params)), C.c_int64(n), _p(ids, C.c_int64), _p(pos, C.c_float),
                _p(vel, C.c_float), _p(mass, C.c_float), _p(typ, C.c_int32), C.byref(st),
                C.c_float(last_max_vmax), C.c_int32(last_snap), _p(order, C.c_int64),
                _p(energy, C.c_float), C.byref(res), C.byref(props))
        if rc != 0:
            raise RuntimeError("ref_unbind_properties failed")
        return order[:n], energy[:n], result_dict(res), props_dict(props)

    def subhalo_properties(self, params: dict, pos, mass, cen, mbound: float,
                           last_max_vmax: float = 0.0, last_snap: int = -1,
                           snapshot_index: int = 1) -> dict:
        """The C restatement of CalculateProfileProperties + CalculateShape on
        a subhalo's bound particles (most-bound first)."""
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        mass = np.ascontiguousarray(mass, np.float32)
        c = (C.c_float * 3)(*[float(x) for x in cen])
        props = Props()
        fn = self.lib.hbto_subhalo_properties
        fn.restype = C.c_int
        fn(C.byref(make_params(params)), C.c_int64(len(mass)), _p(pos, C.c_float),
           _p(mass, C.c_float), c, C.c_float(mbound), C.c_float(last_max_vmax),
           C.c_int32(last_snap), C.c_int32(snapshot_index), C.byref(props))
        return props_dict(props)

    def recursive_unbind(self, params: dict, forest: dict, relax: float = 3.0):
        """The reference's RecursiveUnbind over a forest, then TruncateSource
        (reference build only).  forest: parts (id, pos, vel, mass, type),
        list_off, nbound_prev, nest_off, nest_idx, roots and the frames.
        Returns (final list offsets, positions into the input rows, results)."""
        if not self.reference:
            raise ValueError("the forest entry exists in the reference build only")
        lo = np.ascontiguousarray(forest["list_off"], np.int64)
        nsub = len(lo) - 1
        ntot = int(lo[-1])
        ids = np.ascontiguousarray(forest["id"], np.int64)
        pos = np.ascontiguousarray(forest["pos"], np.float32).reshape(-1)
        vel = np.ascontiguousarray(forest["vel"], np.float32).reshape(-1)
        mass = np.ascontiguousarray(forest["mass"], np.float32)
        typ = np.ascontiguousarray(forest["type"], np.int32)
        nbp = np.ascontiguousarray(forest["nbound_prev"], np.int64)
        no = np.ascontiguousarray(forest["nest_off"], np.int64)
        ni = np.ascontiguousarray(forest["nest_idx"], np.int64)
        roots = np.ascontiguousarray(forest["roots"], np.int64)
        sts = (State * max(nsub, 1))()
        for s in range(nsub):
            for j in range(3):
                sts[s].ref_pos[j] = float(forest["ref_pos"][s][j])
                sts[s].ref_vel[j] = float(forest["ref_vel"][s][j])
                sts[s].mostbound_pos[j] = float(forest["mostbound_pos"][s][j])
                sts[s].mostbound_vel[j] = float(forest["mostbound_vel"][s][j])
            sts[s].mostbound_id = int(forest["mostbound_id"][s])
        out_off = np.zeros(nsub + 1, np.int64)
        cap = max(ntot * max(nsub, 1), 1)  # a particle can end in several lists
        out_pos = np.zeros(cap, np.int64)
        res = (Result * max(nsub, 1))()
        par = make_params(params)
        fn = self.lib.ref_recursive_unbind
        fn.restype = C.c_int
        rc = fn(C.byref(par), C.c_double(relax), C.c_int64(nsub), _p(lo, C.c_int64),
                _p(ids, C.c_int64), _p(pos, C.c_float), _p(vel, C.c_float), _p(mass, C.c_float),
                _p(typ, C.c_int32), _p(nbp, C.c_int64), sts, _p(no, C.c_int64),
                _p(ni, C.c_int64), C.c_int64(len(roots)), _p(roots, C.c_int64),
                _p(out_off, C.c_int64), _p(out_pos, C.c_int64), C.c_int64(cap), res)
        if rc != 0:
            raise RuntimeError(f"ref_recursive_unbind failed ({rc})")
        return out_off, out_pos[:out_off[-1]], [result_dict(res[s]) for s in range(nsub)]

    def merge_detect(self, params: dict, list_off, pos, vel, mass, nbound, host, mb_pos, mb_vel,
                     isnap: int, sink):
        """FillCores + DetectTraps (C restatement): returns (sink, sink_snap,
        merged, cores) with sink_snap -1 where nothing was trapped now."""
        lo = np.ascontiguousarray(list_off, np.int64)
        nsub = len(lo) - 1
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1)
        mass = np.ascontiguousarray(mass, np.float32)
        nb = np.ascontiguousarray(nbound, np.int64)
        host = np.ascontiguousarray(host, np.int64)
        mbp = np.ascontiguousarray(mb_pos, np.float32).reshape(-1)
        mbv = np.ascontiguousarray(mb_vel, np.float32).reshape(-1)
        sink = np.ascontiguousarray(sink, np.int64).copy()
        snap = np.full(max(nsub, 1), -1, np.int32)
        merged = np.zeros(max(nsub, 1), np.int32)
        cores = (Core * max(nsub, 1))()
        fn = self.lib.hbto_merge_detect
        fn.restype = C.c_int
        rc = fn(C.byref(make_params(params)), C.c_int64(nsub), _p(lo, C.c_int64),
                _p(pos, C.c_float), _p(vel, C.c_float), _p(mass, C.c_float), _p(nb, C.c_int64),
                _p(host, C.c_int64), _p(mbp, C.c_float), _p(mbv, C.c_float), C.c_int32(isnap),
                _p(sink, C.c_int64), _p(snap, C.c_int32), _p(merged, C.c_int32), cores)
        if rc != 0:
            raise RuntimeError("hbto_merge_detect: a host chain has a cycle")
        cd = [dict(pos=np.array(list(cores[s].pos), np.float32), sigma_r=cores[s].sigma_r,
                   vel=np.array(list(cores[s].vel), np.float32), sigma_v=cores[s].sigma_v)
              for s in range(nsub)]
        return sink[:nsub], snap[:nsub], merged[:nsub], cd

    def merge_subhalos(self, params: dict, state: dict, isnap: int, relax: float = 3.0):
        """The reference's SubhaloSnapshot_t::MergeSubhalos (reference build
        only).  state: every subhalo's list (id, pos, vel, mass, type rows,
        list_off, bound first), nbound, frames, nest_off/nest_idx,
        group_off/group_idx (central first), heads_off/heads_idx, sink, death.
        Returns dict(off, id, energy, sink, death, sink_snap, results)."""
        if not self.reference:
            raise ValueError("exists in the reference build only")
        a = {k: np.ascontiguousarray(state[k], np.int64)
             for k in ("list_off", "nbound", "nest_off", "nest_idx", "group_off", "group_idx",
                       "heads_off", "heads_idx", "sink", "id")}
        death = np.ascontiguousarray(state["death"], np.int32)
        pos = np.ascontiguousarray(state["pos"], np.float32).reshape(-1)
        vel = np.ascontiguousarray(state["vel"], np.float32).reshape(-1)
        mass = np.ascontiguousarray(state["mass"], np.float32)
        typ = np.ascontiguousarray(state["type"], np.int32)
        nsub = len(a["list_off"]) - 1
        nhalo = len(a["group_off"]) - 1
        sts = (State * max(nsub, 1))()
        for s in range(nsub):
            for j in range(3):
                sts[s].ref_pos[j] = float(state["ref_pos"][s][j])
                sts[s].ref_vel[j] = float(state["ref_vel"][s][j])
                sts[s].mostbound_pos[j] = float(state["mostbound_pos"][s][j])
                sts[s].mostbound_vel[j] = float(state["mostbound_vel"][s][j])
            lo = int(a["list_off"][s])
            sts[s].mostbound_id = int(a["id"][lo]) if a["list_off"][s + 1] > lo else -1
        cap = max(2 * int(a["list_off"][-1]), 1)
        out_off = np.zeros(nsub + 1, np.int64)
        out_id = np.zeros(cap, np.int64)
        out_e = np.zeros(cap, np.float32)
        sink = np.zeros(max(nsub, 1), np.int64)
        dout = np.zeros(max(nsub, 1), np.int32)
        ssnap = np.zeros(max(nsub, 1), np.int32)
        res = (Result * max(nsub, 1))()
        fn = self.lib.ref_merge_subhalos
        fn.restype = C.c_int
        rc = fn(C.byref(make_params(params)), C.c_double(relax), C.c_int32(isnap),
                C.c_int64(nsub), _p(a["list_off"], C.c_int64), _p(a["id"], C.c_int64),
                _p(pos, C.c_float), _p(vel, C.c_float), _p(mass, C.c_float), _p(typ, C.c_int32),
                _p(a["nbound"], C.c_int64), sts, _p(a["nest_off"], C.c_int64),
                _p(a["nest_idx"], C.c_int64), C.c_int64(nhalo), _p(a["group_off"], C.c_int64),
                _p(a["group_idx"], C.c_int64), _p(a["heads_off"], C.c_int64),
                _p(a["heads_idx"], C.c_int64), _p(a["sink"], C.c_int64), _p(death, C.c_int32),
                C.c_int64(cap), _p(out_off, C.c_int64), _p(out_id, C.c_int64),
                _p(out_e, C.c_float), _p(sink, C.c_int64), _p(dout, C.c_int32),
                _p(ssnap, C.c_int32), res)
        if rc != 0:
            raise RuntimeError(f"ref_merge_subhalos failed ({rc})")
        n = int(out_off[-1])
        return dict(off=out_off, id=out_id[:n], energy=out_e[:n], sink=sink[:nsub],
                    death=dout[:nsub], sink_snap=ssnap[:nsub],
                    results=[result_dict(res[s]) for s in range(nsub)])

    def partition(self, E: np.ndarray):
        E = np.ascontiguousarray(E, np.float32).copy()
        idx = np.arange(len(E), dtype=np.int64)
        nb = self._partition(_p(E, C.c_float), _p(idx, C.c_int64), C.c_int64(len(E)))
        return int(nb), E, idx

    # -- the path -----------------------------------------------------------
    def unbind(self, params: dict, sub: dict, nthreads: int = 1, shuffle_seed: int = 0,
               drand_seed: int = 1):
        """Unbind one subhalo.  ``sub`` holds id, pos (n,3), vel (n,3), mass,
        type, ref_pos, ref_vel, mostbound_pos, mostbound_vel (and optionally
        mostbound_id).  For the C restatement the particles are taken as given
        (already shuffled when sampling applies); the reference harness takes
        them before the shuffle and shuffles with ``shuffle_seed``."""
        n = len(sub["mass"])
        ids = np.ascontiguousarray(sub["id"], np.int64)
        pos = np.ascontiguousarray(sub["pos"], np.float32).reshape(-1)
        vel = np.ascontiguousarray(sub["vel"], np.float32).reshape(-1)
        mass = np.ascontiguousarray(sub["mass"], np.float32)
        typ = np.ascontiguousarray(sub.get("type", np.ones(n, np.int32)), np.int32)
        mb_id = sub.get("mostbound_id", ids[0] if n else -1)
        st = make_state(sub["ref_pos"], sub["ref_vel"], sub["mostbound_pos"],
                        sub["mostbound_vel"], mb_id)
        order = np.zeros(max(n, 1), np.int64)
        energy = np.zeros(max(n, 1), np.float32)
        res = Result()
        par = make_params(params)
        self.srand48(drand_seed)
        args = [C.byref(par), C.c_int64(n), _p(ids, C.c_int64), _p(pos, C.c_float),
                _p(vel, C.c_float), _p(mass, C.c_float), _p(typ, C.c_int32), C.byref(st),
                _p(order, C.c_int64), _p(energy, C.c_float), C.byref(res), C.c_int(nthreads)]
        if self.reference:
            args.append(C.c_uint(shuffle_seed))
        rc = self._unbind(*args)
        if rc != 0:
            raise RuntimeError(f"oracle unbind failed with status {rc}")
        return order[:n], energy[:n], result_dict(res)

    def unbind_batch(self, params: dict, batch: dict, nthreads: int = 0,
                     shuffle_seed: int = 0, drand_seed: int = 1):
        """Unbind every subhalo of a batch (see hbtplus_gb300.synthetic)."""
        off = np.ascontiguousarray(batch["offsets"], np.int64)
        nsub = len(off) - 1
        ntot = int(off[-1])
        ids = np.ascontiguousarray(batch["id"], np.int64)
        pos = np.ascontiguousarray(batch["pos"], np.float32).reshape(-1)
        vel = np.ascontiguousarray(batch["vel"], np.float32).reshape(-1)
        mass = np.ascontiguousarray(batch["mass"], np.float32)
        typ = np.ascontiguousarray(batch.get("type", np.ones(ntot, np.int32)), np.int32)
        sts = (State * max(nsub, 1))()
        for s in range(nsub):
            o = int(off[s])
            mb_id = batch["mostbound_id"][s] if "mostbound_id" in batch else (
                ids[o] if off[s + 1] > o else -1)
            sts[s] = make_state(batch["ref_pos"][s], batch["ref_vel"][s],
                                batch["mostbound_pos"][s], batch["mostbound_vel"][s], mb_id)
        order = np.zeros(max(ntot, 1), np.int64)
        energy = np.zeros(max(ntot, 1), np.float32)
        res = (Result * max(nsub, 1))()
        par = make_params(params)
        self.srand48(drand_seed)
        args = [C.byref(par), C.c_int64(nsub), _p(off, C.c_int64), _p(ids, C.c_int64),
                _p(pos, C.c_float), _p(vel, C.c_float), _p(mass, C.c_float),
                _p(typ, C.c_int32), sts, _p(order, C.c_int64), _p(energy, C.c_float), res,
                C.c_int(nthreads)]
        if self.reference:
            args.append(C.c_uint(shuffle_seed))
        rc = self._batch(*args)
        if rc != 0:
            raise RuntimeError(f"oracle batch unbind failed with status {rc}")
        return order[:ntot], energy[:ntot], [result_dict(res[s]) for s in range(nsub)]

    def tree_potentials(self, params: dict, pos, mass, targets, open_angles,
                        nthreads: int = 0, drand_seed: int = 1):
        """EvaluatePotential of the particles ``targets`` from one reference
        tree over all particles, at each opening angle (C restatement only):
        (potentials (len(open_angles), len(targets)), interactions per angle)."""
        if self.reference:
            raise ValueError("tree_potentials exists in the C restatement only")
        f = self.lib.hbto_tree_potentials
        n = len(mass)
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        mass = np.ascontiguousarray(mass, np.float32)
        t = np.ascontiguousarray(targets, np.int64)
        th = np.ascontiguousarray(open_angles, np.float64)
        pot = np.zeros((len(th), max(len(t), 1)), np.float64)
        cnt = np.zeros(max(len(th), 1), np.int64)
        par = make_params(params)
        self.srand48(drand_seed)
        rc = f(C.byref(par), C.c_int64(n), _p(pos, C.c_float), _p(mass, C.c_float),
               C.c_int64(len(t)), _p(t, C.c_int64), C.c_int32(len(th)), _p(th, C.c_double),
               _p(pot, C.c_double), _p(cnt, C.c_int64), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle tree potentials failed with status {rc}")
        return pot[:, :len(t)], cnt[:len(th)]

    def binding_energies(self, params: dict, pos, vel, mass, ref_pos, ref_vel,
                         nthreads: int = 1, drand_seed: int = 1):
        """First-pass energies and potentials of every particle (tree over all)."""
        n = len(mass)
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1)
        mass = np.ascontiguousarray(mass, np.float32)
        rp = np.ascontiguousarray(ref_pos, np.float32)
        rv = np.ascontiguousarray(ref_vel, np.float32)
        E = np.zeros(max(n, 1), np.float32)
        pot = np.zeros(max(n, 1), np.float64)
        cnt = C.c_int64(0)
        par = make_params(params)
        self.srand48(drand_seed)
        self._energies(C.byref(par), C.c_int64(n), _p(pos, C.c_float), _p(vel, C.c_float),
                       _p(mass, C.c_float), _p(rp, C.c_float), _p(rv, C.c_float),
                       _p(E, C.c_float), _p(pot, C.c_double), C.byref(cnt), C.c_int(nthreads))
        return E[:n], pot[:n], cnt.value
