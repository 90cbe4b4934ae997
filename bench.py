"""Benchmark of the batched subhalo-unbinding path on GB300.

Workload (one step): unbinding of the 2000-subhalo batch -- sizes drawn from
dN/dlnN ~ N^-0.9 on [20, 2e5], NFW haloes with Jeans velocities and 20%
unbound contaminants, centres uniform in a 100 Mpc/h periodic box (about 5%
straddling a face) -- in one hbtu_unbind_batch call (seeded synthetic data:
no public particle suite exists for this path).  Parameters are the
reference's defaults with the exact tree (MaxSampleSizeOfPotentialEstimate 0),
softening 0.002 Mpc/h, opening angle 0.45.

  value  subhalo unbinds/s with inputs resident in HBM, CUDA events on the
         library's stream, L2 flushed (256 MB write) before every timed step
  e2e    the same through the C ABI with pinned host buffers: host->device
         copy of the particles and device->host read of order, energies and
         per-subhalo results inside the timed region
  plain  the same batch unbound one subhalo per call (hbtu_unbind)
  cpu_baseline  the reference CPU path on the same batch on this host's cores

python bench.py [--steps K] [--warmup W] [--impl reference]; under torchrun
the job is one global batch split across the ranks by the planner of
hbtplus_gb300.shard (greedy LPT on n log n; no device collective, the results
are gathered on the host afterwards): by default N copies of the workload with
different seeds (weak scaling), with --scaling strong one workload split N ways.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("subhalo unbinds/s & particle-potentials/s, batched vs plain, same GB300, "
          "≤1e-4 mass err")
UNIT = "subhalo unbinds/s"
FLOPS_PER_INTERACTION = 14  # 3 sub, 5 for r^2, 4 for rsqrt, 2 for the potential update
HBM_BYTES_PER_EVALUATION = 44  # read pos, vel, mass (28 B); write E and index (16 B)
FP32_LANES_PER_SM = 128
# DRAM bytes (read + write) of the first-pass walk launch, from one ncu capture of
# the same workload (summaries in profiles/); None until captured for this kernel.
WALK1_DRAM_BYTES = {"batch": 79971584}
WALK1_PROFILE = {"batch": "walk_lean_pass1_batch2000.md"}
# The same capture: the walk is limited by the L1 data path, not by DRAM or the FP32 pipe.
WALK1_LIMITER = {"batch": "L1 data path: l1tex throughput 90% of peak at a 97% L1 hit rate, "
                          "22 sectors per warp request (one 32-byte node record per lane per "
                          "step; the lanes walk apart)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nsub", type=int, default=2000)
    ap.add_argument("--workload", default="batch",
                    choices=["batch", "single", "host2e7", "step", "adjoint"],
                    help="batch: the 2000-subhalo batch (default); single: the isolated "
                         "1e5-particle NFW subhalo (+10%% contaminants); host2e7: the "
                         "2e7-particle host with 300 clumps (+5%% contaminants); step: a "
                         "tracking step of 20,000 subhaloes in a 3e7-particle snapshot (ID "
                         "re-resolve, gather, unbind); adjoint: the batched backward of the "
                         "2000-subhalo batch's bound sets (one hbtu_energy_gradient call)")
    ap.add_argument("--open-angle", type=float, default=0.45)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--leaf-runs", type=int, default=-1,
                    help="walk_leaf_runs option of the FP32 walk (-1: library default)")
    ap.add_argument("--max-sample", type=int, default=0,
                    help="MaxSampleSizeOfPotentialEstimate: 0 exact (parity, the default), "
                         "1000 the reference's production default")
    ap.add_argument("--walk-layout", type=int, default=-1,
                    help="walk_layout option of the FP32 walk (-1: library default)")
    ap.add_argument("--walk-schedule", type=int, default=-1,
                    help="walk_schedule option of the FP32 walk (-1: library default)")
    ap.add_argument("--small-cutoff", type=int, default=-1,
                    help="small_cutoff option: once every active subhalo's list is at most "
                         "this long, one block per subhalo finishes the loop (-1: library "
                         "default, 0: off)")
    ap.add_argument("--small-blocks", type=int, default=-1,
                    help="small_blocks_per_sm option (-1: library default)")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="under torchrun: weak (default) -- a global batch of N workloads, "
                         "one per rank's worth, split across the ranks by the LPT planner; "
                         "strong -- one workload split N ways")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(nsub: int, rank: int, kind: str = "batch", theta: float = 0.45,
             max_sample: int = 0):
    from hbtplus_gb300 import synthetic as S
    p = S.default_params(open_angle=theta, max_sample_size=max_sample)
    if kind == "single":
        return S.concat([S.single_subhalo(seed=20261203 + 1000 * rank)]), p
    if kind == "host2e7":
        return S.concat([S.host_with_clumps(seed=20261205 + 1000 * rank)]), p
    b = S.subhalo_batch(nsub=nsub, seed=20261204 + 1000 * rank)
    return b, p


def global_workload(args, ws):
    """The whole job's batch: ws workloads (seeds per rank) concatenated for weak
    scaling, one workload for strong scaling; every rank builds the same."""
    from hbtplus_gb300 import synthetic as S
    copies = ws if args.scaling == "weak" else 1
    parts, params = [], None
    for r in range(copies):
        b, params = workload(args.nsub, r, args.workload, args.open_angle, args.max_sample)
        parts.append(b)
    if copies == 1:
        return parts[0], params
    subs = [S.split(b, s) for b in parts for s in range(len(b["offsets"]) - 1)]
    return S.concat(subs), params


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_reference_time(params, batch, threads):
    """(seconds, kind) of one unbinding of the batch by the reference CPU path:
    the reference's own Unbind when its harness is built here, else the C
    restatement (oracle/hbt_oracle.c), halo-parallel on `threads` threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    kind = "reference" if os.path.exists(O.REF_SO) else "port"
    if kind == "port" and not os.path.exists(O.ORACLE_SO):
        O.build(reference=False)
    orc = O.Oracle(reference=(kind == "reference"))
    off = batch["offsets"]
    if len(off) == 2:  # one subhalo: the reference's particle-parallel inner loops
        sub = {k: batch[k] for k in ("id", "pos", "vel", "mass", "type") if k in batch}
        for k in ("ref_pos", "ref_vel", "mostbound_pos", "mostbound_vel"):
            sub[k] = np.asarray(batch[k])[0]
        if "mostbound_id" in batch:
            sub["mostbound_id"] = int(np.asarray(batch["mostbound_id"])[0])
        t = time.perf_counter()
        _, _, r = orc.unbind(params, sub, nthreads=threads)
        return time.perf_counter() - t, kind, [r]
    t = time.perf_counter()
    _, _, res = orc.unbind_batch(params, batch, nthreads=threads)
    return time.perf_counter() - t, kind, res


def cpu_schedule(nsub: int) -> str:
    """How the reference CPU path parallelises this workload."""
    if nsub == 1:
        return "one Unbind, particle-parallel OpenMP inner loops (src/subhalo_unbind.cpp:319-354)"
    return "halo-parallel OpenMP schedule(dynamic,1) (src/subhalo_unbind.cpp:495-503)"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def copy_times(pin, dev, outs, stream, steps):
    """(host->device ms, device->host ms) per step: the pinned input arrays copied
    to their device buffers, and the device outputs to pinned host buffers,
    each bracketed by CUDA events on `stream`, averaged over `steps`."""
    import torch
    h2d, d2h = [], []
    for _ in range(max(1, steps)):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record(stream)
        for k, v in pin.items():
            dev[k].copy_(v, non_blocking=True)
        e[1].record(stream)
        for host, d in outs:
            host.copy_(d, non_blocking=True)
        e[2].record(stream)
        torch.cuda.synchronize()
        h2d.append(e[0].elapsed_time(e[1]))
        d2h.append(e[1].elapsed_time(e[2]))
    return statistics.mean(h2d), statistics.mean(d2h)


def run_reference_arm(args, ws, rank):
    if rank != 0:
        return
    if args.workload in ("step", "host2e7", "adjoint"):
        print(json.dumps({"impl": "reference", "unavailable":
                          f"the {args.workload} workload has no CPU reference run: one pass "
                          "of the reference over it takes minutes on the host"}), flush=True)
        return
    batch, params = workload(args.nsub, 0, args.workload, args.open_angle, args.max_sample)
    threads = cpu_threads()
    for _ in range(args.warmup):
        cpu_reference_time(params, batch, threads)
    times, kind = [], "port"
    for _ in range(args.steps):
        t, kind, _ = cpu_reference_time(params, batch, threads)
        times.append(t)
    total = sum(times)
    nsub = len(batch["offsets"]) - 1
    value = nsub * args.steps / total
    nsum = int(batch["offsets"][-1])
    sample = (f"the full {nsub}-subhalo workload ({nsum} particles) per step, "
              f"{cpu_schedule(nsub)}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args, batch),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(args, batch):
    nsub = len(batch["offsets"]) - 1
    if args.workload == "single":
        name = ("single subhalo: 1e5-particle NFW (r200 0.2 Mpc/h, c 10) + 10% contaminants, "
                "100 Mpc/h periodic box")
    elif args.workload == "host2e7":
        name = ("large host: 2e7-particle NFW (r200 1 Mpc/h, c 5) + 300 Plummer clumps "
                "(1e3-1e5 particles) + 5% contaminants, 100 Mpc/h periodic box")
    else:
        name = (f"{nsub}-subhalo batch: dN/dlnN ~ N^-0.9 on [20, 2e5], NFW + Jeans, "
                "20% contaminants, 100 Mpc/h periodic box")
    return {"workload": name,
            "nsub": nsub, "particles": int(batch["offsets"][-1]),
            "max_subhalo": int(np.max(np.diff(batch["offsets"]))),
            "softening": 0.002, "open_angle": args.open_angle,
            "max_sample_size": args.max_sample,
            "precision": args.precision, "walk_leaf_runs": args.leaf_runs if args.leaf_runs >= 0 else 1,
            "walk_schedule": args.walk_schedule if args.walk_schedule >= 0 else 0,
            "walk_layout": args.walk_layout if args.walk_layout >= 0 else 1,
            "l2": "flushed before each timed step (256 MB write)"}


def run_tracking_step(args, ws, rank, local):
    """The tracking step of 20,000 subhaloes (2000-subhalo law) in a 3e7-particle,
    200 Mpc/h snapshot: the snapshot's ID table, the re-resolve of every
    subhalo's particle IDs after a drift and 10% outer stripping, the gather,
    the batched unbinding and every subhalo's profile and shape, all on the
    GPU."""
    import torch

    from hbtplus_gb300 import _lib
    from hbtplus_gb300 import synthetic as S
    from hbtplus_gb300.step import TrackingStep
    from hbtplus_gb300.unbind import Unbinder

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    d = S.tracking_snapshot(seed=20261207 + 1000 * rank)
    params = S.default_params(box_size=200.0)
    nsub = len(d["offsets"]) - 1
    nmem = int(d["offsets"][-1])
    nsnap = len(d["snap_id"])
    ub = Unbinder(params, device=local)
    step = TrackingStep(ub)
    T = {k: torch.from_numpy(np.ascontiguousarray(d[k])).to(dev)
         for k in ("snap_id", "snap_pos", "snap_vel", "snap_mass", "snap_type", "member_id")}
    frames = {k: d[k] for k in ("offsets", "ref_pos", "ref_vel", "mostbound_pos",
                                "mostbound_vel", "mostbound_id")}
    states = ub.make_states(frames)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    props_args = dict(snapshot_index=1)

    def one():
        step.load_snapshot(T["snap_id"], T["snap_pos"], T["snap_vel"], T["snap_mass"],
                           T["snap_type"])
        return step.run(d["offsets"], T["member_id"], states, properties=props_args)

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    ub.set_timing(True)
    ub.reset_stats()
    times, phase = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
            e[0].record(stream)
            step.load_snapshot(T["snap_id"], T["snap_pos"], T["snap_vel"], T["snap_mass"],
                               T["snap_type"])
            e[1].record(stream)
            index = step.resolve(T["member_id"])
            batch = step.gather(index)
            e[2].record(stream)
            out = dict(order=torch.empty(nmem, dtype=torch.int64, device=dev),
                       energy=torch.empty(nmem, dtype=torch.float32, device=dev),
                       res=torch.empty(nsub * C.sizeof(_lib.hbtu_result), dtype=torch.uint8,
                                       device=dev))
            ub.unbind_batch_device(batch, d["offsets"], states, out)
            e[3].record(stream)
            ub.subhalo_properties_device(batch, d["offsets"], out["order"], out["res"],
                                         snapshot_index=1)
            e[4].record(stream)
            times.append(e)
        torch.cuda.synchronize()
    ms = [a[0].elapsed_time(a[4]) for a in times]
    fill_ms = statistics.mean(a[0].elapsed_time(a[1]) for a in times)
    rg_ms = statistics.mean(a[1].elapsed_time(a[2]) for a in times)
    un_ms = statistics.mean(a[2].elapsed_time(a[3]) for a in times)
    pr_ms = statistics.mean(a[3].elapsed_time(a[4]) for a in times)
    ms_per_step = sum(ms) / args.steps
    st = ub.stats()
    clocks = clk.summary()
    # e2e: snapshot and member IDs from pinned host memory, results back to the host
    pin = {k: v.cpu().pin_memory() for k, v in T.items()}
    res_host = torch.empty(nsub * C.sizeof(_lib.hbtu_result), dtype=torch.uint8).pin_memory()
    order_host = torch.empty(nmem, dtype=torch.int64).pin_memory()
    G = {k: torch.empty_like(v) for k, v in T.items()}  # device buffers, kept across steps

    def e2e_one():
        for k, v in pin.items():
            G[k].copy_(v, non_blocking=True)
        step.load_snapshot(G["snap_id"], G["snap_pos"], G["snap_vel"], G["snap_mass"],
                           G["snap_type"])
        out, _ = step.run(d["offsets"], G["member_id"], states, properties=props_args)
        order_host.copy_(out["order"], non_blocking=True)
        res_host.copy_(out["res"], non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_one()
    e2e_t = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_one()
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_t) / args.steps
    h2d = sum(int(v.numel() * v.element_size()) for v in pin.values())
    d2h = nmem * 8 + nsub * (C.sizeof(_lib.hbtu_result) + C.sizeof(_lib.hbtu_props))
    # HBM view of the re-resolve + gather phase: per member 8 B id + 8 B index
    # written and read back + 40 B particle read and written
    rg_bytes = nmem * (8 + 8 + 8 + 40 + 40)
    peaks, peak_kind = measured_peaks()
    line = {
        "metric": "subhalo unbinds/s in a tracking step (ID re-resolve + gather + unbind + "
                  "profile and shape)",
        "value": ws * nsub / (ms_per_step / 1e3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded: 2000-subhalo law, uniform background, drift, stripping)",
        "config": {"workload": "tracking step: 20,000 subhaloes, 3e7-particle 200 Mpc/h "
                               "snapshot, v*dt drift, 10% outer stripping, mapped ID table",
                   "nsub": nsub, "members": nmem, "snapshot_particles": nsnap,
                   "l2": "flushed before each timed step (256 MB write)"},
        "phase_ms_per_step": {"table_fill": fill_ms, "resolve_gather": rg_ms, "unbind": un_ms,
                              "properties": pr_ms,
                              "tree": st["tree_ms"] / args.steps,
                              "walk": st["walk_ms"] / args.steps},
        "roofline": {"kernel": "ID re-resolve + gather phase", "bound": "hbm",
                     "achieved": rg_bytes / (rg_ms / 1e3) / 1e9, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": rg_bytes / (rg_ms / 1e3) / 1e9 / peaks["hbm_gbs"],
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": None, "algorithmic_bytes": rg_bytes},
        "cpu_baseline": None,
        "cpu_baseline_note": "not measured for this workload (one reference pass over it "
                             "takes minutes on the host)",
        "e2e": {"value": ws * nsub / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s},
        "gpu_launches": int(st["kernel_launches"]),  # all timed steps
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    step.close()
    ub.close()


def run_adjoint(args, ws, rank, local):
    """The batched backward of config 3: the 2000-subhalo batch is unbound, and
    the binding energies of all its bound sets are differentiated with respect
    to positions, velocities and masses in one hbtu_energy_gradient call."""
    import torch

    from hbtplus_gb300 import _lib
    from hbtplus_gb300.adjoint import bound_subset, energy_gradient
    from hbtplus_gb300.unbind import Unbinder, _state

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    batch, params = workload(args.nsub, rank, "batch", args.open_angle, 0)
    ub = Unbinder(params, device=local)
    order, _, res = ub.unbind_batch(batch)
    b = bound_subset(batch, order, res)
    nsub = len(b["offsets"]) - 1
    npart = int(b["offsets"][-1])
    T = {k: torch.from_numpy(b[k]).to(dev) for k in ("pos", "vel", "mass")}
    stream = torch.cuda.current_stream(dev)
    ub.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    off = np.ascontiguousarray(b["offsets"], np.int64)
    sts = (_lib.hbtu_state * nsub)()
    for s in range(nsub):
        sts[s] = _state(b["ref_pos"][s], b["ref_vel"][s], b["ref_pos"][s], b["ref_vel"][s], -1)
    # the timed call: device-resident inputs and outputs through the C ABI
    d_ids = torch.arange(npart, dtype=torch.int64, device=dev)
    d_E = torch.empty(nsub, dtype=torch.float64, device=dev)
    d_g = [torch.empty((npart, 3), dtype=torch.float32, device=dev),
           torch.empty((npart, 3), dtype=torch.float32, device=dev),
           torch.empty(npart, dtype=torch.float32, device=dev)]
    p_dev = _lib.hbtu_particles(id=d_ids.data_ptr(), pos=T["pos"].data_ptr(),
                                vel=T["vel"].data_ptr(), mass=T["mass"].data_ptr(), type=0,
                                location=_lib.HBTU_DEVICE, reserved=0)

    def step():
        rc = ub.lib.hbtu_energy_gradient(ub.handle, C.byref(p_dev), nsub, off.ctypes.data,
                                         C.addressof(sts), d_E.data_ptr(), d_g[0].data_ptr(),
                                         d_g[1].data_ptr(), d_g[2].data_ptr())
        _lib.check(rc, ub.handle)

    # the same gradient as the autograd path's (hbtplus_gb300.adjoint)
    _, gp_ref, _, _ = energy_gradient(ub, T["pos"], T["vel"], T["mass"], b["offsets"],
                                      b["ref_pos"], b["ref_vel"])
    step()
    torch.cuda.synchronize()
    assert torch.equal(gp_ref, d_g[0])

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ub.reset_stats()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(c) for a, c in times) / args.steps
    launches = int(ub.stats()["kernel_launches"])  # all timed steps
    # end to end: host arrays through the C ABI, gradients back to the host
    pin = {k: torch.from_numpy(b[k]).pin_memory() for k in ("pos", "vel", "mass")}
    ids = torch.arange(npart, dtype=torch.int64).pin_memory()
    gp = torch.empty((npart, 3), dtype=torch.float32).pin_memory()
    gv = torch.empty((npart, 3), dtype=torch.float32).pin_memory()
    gm = torch.empty(npart, dtype=torch.float32).pin_memory()
    E = np.zeros(nsub, np.float64)
    p_host = _lib.hbtu_particles(id=ids.data_ptr(), pos=pin["pos"].data_ptr(),
                                 vel=pin["vel"].data_ptr(), mass=pin["mass"].data_ptr(), type=0,
                                 location=_lib.HBTU_HOST, reserved=0)

    def e2e_step():
        rc = ub.lib.hbtu_energy_gradient(ub.handle, C.byref(p_host), nsub, off.ctypes.data,
                                         C.addressof(sts), E.ctypes.data, gp.data_ptr(),
                                         gv.data_ptr(), gm.data_ptr())
        _lib.check(rc, ub.handle)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_t) / args.steps
    h2d = npart * (12 + 12 + 4 + 8) + off.nbytes + C.sizeof(sts)
    d2h = npart * (12 + 12 + 4) + nsub * 8
    line = {
        "metric": "subhalo binding-energy gradients/s (batched backward of the bound sets)",
        "value": ws * nsub / (ms / 1e3), "unit": "subhalo gradients/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the 2000-subhalo batch, unbound; its bound sets)",
        "config": {"workload": "adjoint: d E_tot / d(x, v, m) of the bound sets of the "
                               "2000-subhalo batch in one call", "nsub": nsub,
                   "bound_particles": npart, "open_angle": args.open_angle,
                   "l2": "flushed before each timed step (256 MB write)"},
        "particles_per_s": ws * npart / (ms / 1e3),
        "e2e": {"value": ws * nsub / e2e_s, "unit": "subhalo gradients/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s},
        "gpu_launches": launches,
        "cpu_baseline": None,
        "cpu_baseline_note": "the reference has no adjoint",
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ub.close()


def main():
    args = parse()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload in ("step", "adjoint"):
        (run_tracking_step if args.workload == "step" else run_adjoint)(args, ws, rank, local)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    import torch

    from hbtplus_gb300 import _lib
    from hbtplus_gb300 import unbind as U

    from hbtplus_gb300 import shard

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    job, params = global_workload(args, ws)
    job_sizes = np.diff(job["offsets"])
    plan = shard.plan_shards(job_sizes, ws)
    batch = shard.take(job, plan[rank])  # this rank's shard of the job
    nsub_job = len(job_sizes)
    nsub = len(batch["offsets"]) - 1
    ntot = int(batch["offsets"][-1])
    prec = 1 if args.precision == "fp64" else 0
    ub = U.Unbinder(params, precision=prec, device=local)
    if args.leaf_runs >= 0:
        ub.set_option("walk_leaf_runs", args.leaf_runs)
    if args.walk_schedule >= 0:
        ub.set_option("walk_schedule", args.walk_schedule)
    if args.walk_layout >= 0:
        ub.set_option("walk_layout", args.walk_layout)
    if args.small_cutoff >= 0:
        ub.set_option("small_cutoff", args.small_cutoff)
    if args.small_blocks >= 0:
        ub.set_option("small_blocks_per_sm", args.small_blocks)
    small_cutoff = ub.get_option("small_cutoff")
    small_blocks = ub.get_option("small_blocks_per_sm")

    stream = torch.cuda.current_stream(dev)
    ub.set_stream(stream.cuda_stream)

    # -- device-resident inputs and outputs ---------------------------------
    d_in = {k: torch.from_numpy(np.ascontiguousarray(batch[k])).to(dev)
            for k in ("id", "pos", "vel", "mass", "type")}
    d_out = dict(order=torch.empty(ntot, dtype=torch.int64, device=dev),
                 energy=torch.empty(ntot, dtype=torch.float32, device=dev),
                 res=torch.empty(nsub * C.sizeof(_lib.hbtu_result), dtype=torch.uint8,
                                 device=dev))
    states = ub.make_states(batch)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        ub.unbind_batch_device(d_in, batch["offsets"], states, d_out)

    # reference interactions/evaluations of the job (identical walk): a host call on
    # this rank's shard, the shards' results gathered on rank 0 in job order
    h_order, h_energy, host_res = ub.unbind_batch(batch)
    tagged = [dict(r, _n=int(job_sizes[s])) for r, s in zip(host_res, plan[rank])]
    gathered = shard.gather_results(plan, rank, ws, (h_order, h_energy, tagged))
    job_res = gathered[2] if gathered is not None else []
    interactions = sum(int(r["interactions"]) for r in job_res)
    evaluations = sum(int(r["evaluations"]) for r in job_res)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ub.set_timing(False)  # the timed steps run as a user's calls do: no phase events
    ub.reset_stats()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in times]
    total_ms = sum(step_ms)
    # the phase split (and the first walk launch of the roofline) from as many
    # further steps with the library's per-phase CUDA events on, untimed
    ub.set_timing(True)
    ub.reset_stats()
    for _ in range(args.steps):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    st = ub.stats()
    ub.set_timing(False)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    ms_per_step = total_ms / args.steps
    value = nsub_job / (ms_per_step / 1e3)  # the whole job's subhaloes / the slowest rank
    clocks = clk.summary()

    # -- roofline of the dominant kernel launch: the first pass's energy walk ----
    walk_ms = st["walk_ms"] / args.steps
    walk1_ms = st["walk1_ms"] / args.steps
    walk1_inter = st["walk1_interactions"] / args.steps
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clocks.get("sm_mhz") or 1965.0
    fp32_peak = sm_count * FP32_LANES_PER_SM * 2 * mhz * 1e6 / 1e12
    achieved = walk1_inter * FLOPS_PER_INTERACTION / (walk1_ms / 1e3) / 1e12 if walk1_ms else 0.0
    achieved_all = interactions * FLOPS_PER_INTERACTION / (walk_ms / 1e3) / 1e12 if walk_ms else 0
    peaks, peak_kind = measured_peaks()
    first_evals = ntot  # the first pass evaluates every particle once
    hbm_achieved = (first_evals * HBM_BYTES_PER_EVALUATION / (walk1_ms / 1e3) / 1e9
                    if walk1_ms else 0.0)
    traffic = WALK1_DRAM_BYTES.get(args.workload) if args.precision == "fp32" else None
    roofline = {
        "kernel": "k_walk_fp32_lean, first pass of the step (Barnes-Hut energy walk, one "
                  "walk per lane, sibling-block node records)",
        "limiter": WALK1_LIMITER.get(args.workload) if args.precision == "fp32" else None,
        "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
        "frac": achieved / fp32_peak if fp32_peak else None,
        "peak_source": f"{sm_count} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 flop at the "
                       f"measured median SM clock {mhz:.0f} MHz (FP32 FMA rate; no FP32 figure "
                       "in MEASURED_PEAKS.json)",
        "traffic": traffic,
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of this launch, "
                           "profiles/" + WALK1_PROFILE[args.workload]) if traffic else None,
        "flops_per_interaction": FLOPS_PER_INTERACTION,
        "interactions_per_launch": walk1_inter, "launch_ms": walk1_ms,
        "all_walk_launches": {"achieved": achieved_all, "interactions_per_step": interactions,
                              "walk_ms_per_step": walk_ms,
                              "share_of_step": walk_ms / ms_per_step if ms_per_step else None},
        "hbm": {"bound": "hbm", "achieved": hbm_achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": hbm_achieved / peaks["hbm_gbs"],
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "bytes_per_evaluation": HBM_BYTES_PER_EVALUATION,
                "algorithmic_bytes_per_launch": first_evals * HBM_BYTES_PER_EVALUATION},
    }

    # -- e2e: host buffers through the C ABI, pinned memory -----------------------
    pin = {k: torch.from_numpy(np.ascontiguousarray(batch[k])).pin_memory()
           for k in ("id", "pos", "vel", "mass", "type")}
    out_order = torch.empty(ntot, dtype=torch.int64).pin_memory()
    out_energy = torch.empty(ntot, dtype=torch.float32).pin_memory()
    out_res = (_lib.hbtu_result * nsub)()
    offsets = np.ascontiguousarray(batch["offsets"], np.int64)
    p_host = _lib.hbtu_particles(id=pin["id"].data_ptr(), pos=pin["pos"].data_ptr(),
                                 vel=pin["vel"].data_ptr(), mass=pin["mass"].data_ptr(),
                                 type=pin["type"].data_ptr(), location=_lib.HBTU_HOST,
                                 reserved=0)

    def e2e_step():
        rc = ub.lib.hbtu_unbind_batch(ub.handle, C.byref(p_host), nsub, offsets.ctypes.data,
                                      C.addressof(states), out_order.data_ptr(),
                                      out_energy.data_ptr(), C.addressof(out_res))
        _lib.check(rc, ub.handle)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_t) / args.steps
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = sum(int(v.numel() * v.element_size()) for v in pin.values()) + offsets.nbytes + \
        C.sizeof(states)
    d2h = ntot * (8 + 4) + nsub * C.sizeof(_lib.hbtu_result)
    h2d_ms, d2h_ms = copy_times(pin, d_in, [(out_order, d_out["order"]),
                                            (out_energy, d_out["energy"])],
                                stream, args.steps)
    e2e = {"value": nsub_job / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s,
           "h2d_ms": h2d_ms, "d2h_ms": d2h_ms,
           "copies_note": "h2d_ms / d2h_ms: the particle copies in and the order and energy "
                          "copies out, timed alone with CUDA events (the e2e call overlaps "
                          "nothing: its copies run on the library's stream in order)"}

    # -- plain form: one subhalo per call on the same GB300 ------------------------
    plain = None
    if not args.no_plain and nsub > 1 and ws == 1:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        order_np = np.empty(ntot, np.int64)
        for s in range(nsub):
            o0, o1 = int(offsets[s]), int(offsets[s + 1])
            n = o1 - o0
            p1 = _lib.hbtu_particles(
                id=d_in["id"].data_ptr() + 8 * o0, pos=d_in["pos"].data_ptr() + 12 * o0,
                vel=d_in["vel"].data_ptr() + 12 * o0, mass=d_in["mass"].data_ptr() + 4 * o0,
                type=d_in["type"].data_ptr() + 4 * o0, location=_lib.HBTU_DEVICE, reserved=0)
            rc = ub.lib.hbtu_unbind(ub.handle, C.byref(p1), n, C.byref(states[s]),
                                    d_out["order"].data_ptr() + 8 * o0,
                                    d_out["energy"].data_ptr() + 4 * o0,
                                    d_out["res"].data_ptr() + s * C.sizeof(_lib.hbtu_result))
            _lib.check(rc, ub.handle)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        del order_np
        plain = {"value": nsub / plain_s, "unit": UNIT, "ms_per_step": 1e3 * plain_s,
                 "form": "hbtu_unbind once per subhalo, device-resident inputs"}

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # -- CPU baseline (reference path on this host's cores) and accuracy ----------------
    cpu = None
    accuracy = None
    if args.workload == "host2e7":
        args.no_cpu = True  # the CPU path needs several minutes per unbinding of 2.7e7 particles
    if not args.no_cpu and ws == 1:  # the CPU baseline: rank 0 at N = 1 only
        threads = cpu_threads()
        t_cpu, kind, cres = cpu_reference_time(params, batch, threads)
        cpu = {"value": nsub / t_cpu, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"the full {nsub}-subhalo workload, one run, {cpu_schedule(nsub)}",
               "seconds": t_cpu}
        rel = [abs(g["mbound"] - c["mbound"]) / c["mbound"] for g, c in zip(host_res, cres)
               if c["mbound"] > 0]
        nb_diff = sum(abs(int(g["nbound"]) - int(c["nbound"])) for g, c in zip(host_res, cres))
        accuracy = {"max_rel_mass_err": max(rel) if rel else 0.0,
                    "mean_rel_mass_err": float(np.mean(rel)) if rel else 0.0,
                    "total_nbound_difference": nb_diff,
                    # the reference's own harness does not count passes (reported as 0)
                    "iterations_equal": (all(g["iterations"] == c["iterations"]
                                             for g, c in zip(host_res, cres))
                                         if any(c["iterations"] for c in cres) else None)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": args.scaling, "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded NFW/Jeans subhaloes, no public suite exists for this path)",
        "config": config_of(args, job),
        "potentials_per_s": evaluations / (ms_per_step / 1e3),
        "interactions_per_s": interactions / (ms_per_step / 1e3),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": int(st["kernel_launches"]),
        "clocks": clocks,
        "plain": plain,
        "batched_over_plain": (value / ws) / plain["value"] if plain else None,
        "accuracy_vs_cpu_reference": accuracy,
        "phase_ms_per_step": {"small": st["small_ms"] / args.steps,
                              "tree": st["tree_ms"] / args.steps, "walk": walk_ms,
                              "loop": st["loop_ms"] / args.steps,
                              "passes": st["passes"] / args.steps,
                              "small_subhaloes": st["small_subhaloes"] / args.steps},
    }
    line["config"]["parallelism"] = (f"{ws} rank(s), one GPU each: the job's {nsub_job} "
                                     "subhaloes in LPT shards (hbtplus_gb300.shard), results "
                                     "gathered on the host")
    line["config"]["job_subhaloes"] = nsub_job
    line["config"]["job_particles"] = int(job["offsets"][-1])
    line["gathered_subhaloes"] = len(job_res)
    line["config"]["small_cutoff"] = small_cutoff
    line["config"]["small_blocks_per_sm"] = small_blocks
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
