#!/usr/bin/env python
"""Throughput of the MGLET RK time step on GB300 (cell-updates/s).

Workload (default): 4096 grids of 24^3 cells with two ghost layers
(16 x 16 x 16 tiling of a periodic box of side 2*pi, 56.6 M cells), the 3-D
Taylor-Green field plus seeded uniform noise of amplitude 1e-2 on u, v, w
(splitmix64, seed 42), nu = 1/1600, Williamson RK3, dt = 5e-4, hyperplane
SIP with ninner = 5, nouter = 9, epcorr = 1e-10.  One step = one time step
= three RK stages, each with its full pressure solve.  Inputs and the
working set (>10 GB) are far larger than L2, so no flush is needed.

The headline is the batched mixed-precision form (FP32 flux stencils and SIP
sweeps under the FP64 defect-correction outer loop, one CUDA graph per RK
stage); the plain FP64 form, bit-identical to the CPU restatement, is timed
in the same run and reported beside it.  The timed region runs unprofiled;
per-kernel times for the roofline come from a second, profiled pass of the
same number of steps (per-launch CUDA events on the solver's stream).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed|plain]
  python bench.py --impl reference   # the CPU restatement on the host cores
  python bench.py --sphere [--sphere-check]   # multi-level ghost-cell case
  python bench.py --precision [--tiles 8 8 8] [--steps 200]
      # mixed form against the plain FP64 form (bit-identical to the CPU
      # restatement) from a solenoidal random field: relative L2 error of
      # u, v, w, p every 50 steps

Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mglet-base_gb300"))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s per RK step: mixed/batched vs plain FP64, 1 GB300; % HBM roofline"
UNIT = "cell-updates/s"

# Algorithmic bytes per interior cell and launch of the kernel families:
# every operand read once and every result written once (FP64 8 B, FP32 4 B).
PLAIN_BYTES = {
    "tstle4": 8 * (5 + 3),          # read u,v,w,p,g; write uo,vo,wo
    "rkstep": 8 * 4,                # read p,dp,rhs; write p,dp (per component) / 1.25 ~ 4+1
    "laplacephi": 8 * 3,            # read phi, ap; write res (bp is skipped where it is 1.0)
    "sipiter1": 8 * 7,              # read rhs, res, lw, ls, lb, lpr; write res
    "sipiter2": 8 * 7,              # read res, ue, un, ut, phi; write res, phi
    "divcal": 8 * 4,                # read u, v, w; write rhs
    "rescal_maxabs": 8 * 3,         # read rhs, res; write rhs
    "accumulate": 8 * 4,            # read dp, hilf; write dp, hilf (whole slab)
    "mgpcorr": 8 * 9,               # read dp,u,v,w,p; write u,v,w,p
}
MIXED_BYTES = {
    "mx_flux": 8 * 4 + 4 * 6 + 8 * 3,   # read u,v,w,p (f64), du,dv,dw (f32); write du,dv,dw, u,v,w
    "mx_divcal": 8 * 3 + 4 * 2,         # read u,v,w; write rhs (float-float)
    "mx_mgpcorr": 8 + 8 * 4 * 2,        # read dp, u,v,w,p; write u,v,w,p
    "mx_scatter": 4 * 2 + 8,            # read dp (float-float, plane order); write DP
}


# DRAM bytes per launch measured by ncu on the default workload itself (4096
# grids of 24^3): dram__bytes_read.sum and dram__bytes_write.sum of single
# launches in steady state, averaged over the five inner iterations of one
# outer iteration (the first of them starts from hilf = 0); scaled by cells
# for other tilings.
NCU_DRAM_4096 = {
    "mx_sip_pre": (472.8e6, 184.3e6),
    "mx_sip_fwd": (373.2e6, 168.0e6),
    "mx_sip_bwd": (509.5e6, 177.3e6),
    "mx_outer": (1263.3e6, 848.9e6),
}
NCU_CELLS = 4096 * 13824


# FP64 thread instructions (DADD, DMUL, DFMA and the conversions the FP64 pipe
# issues) per interior cell and launch of the plain FP64 kernels, measured by
# ncu (sm__inst_executed_pipe_fp64 x 32 over one launch on 1024 grids of 24^3,
# parity build without FMA contraction); with the measured FP64 issue rate
# they give each kernel's fraction of the second roof.
FP64_INSTR_PER_CELL = {
    "tstle4": 232650752 * 32 / (1024 * 13824),      # 525.9 (uniform-G shortcut)
    "laplacephi": 5750784 * 32 / (1024 * 13824),    # 13.0
    "sipiter1": 3850240 * 32 / (1024 * 13824),      # 8.70
    "sipiter2": 3330048 * 32 / (1024 * 13824),      # 7.53
}


def kernel_bytes(name, case, ninner):
    """Algorithmic bytes of one launch of a kernel family on this case.
    FP32 plane-order SIP kernels: the pre-pass reads hilf and rhs and writes
    (rhs + laplacian) x lpr; the forward recurrence reads that and writes res
    over it; the backward sweep reads res and hilf and writes hilf; the outer
    step reads hilf and the float-float residual and correction and writes
    both back.  The first inner iteration of an outer iteration starts from
    hilf = 0 and reads no hilf.  Ghost faces: three res faces read per grid
    and sweep, six hilf faces read by the pre-pass and the outer step, all
    gathered from the neighbours' arrays.
    Class coefficients, shared by all grids of a class and served from L2,
    are not counted."""
    cells = case.ncells
    nk, nj, ni = case.kk - 4, case.jj - 4, case.ii - 4
    face = case.ngrid * 4 * ((max(nj * nk, ni * nk, ni * nj) + 3) // 4 * 4)
    hz = 1.0 / ninner
    if name == "mx_sip_pre":
        return cells * (12 - 4 * hz) + face * 6 * (1 - hz)
    if name == "mx_sip_fwd":
        return cells * 8 + face * 3
    if name == "mx_sip_bwd":
        return cells * (12 - 4 * hz) + face * 3
    if name == "mx_outer":
        return cells * (4 + 4 * 4 + 4 * 4) + face * 6
    per = MIXED_BYTES.get(name, PLAIN_BYTES.get(name))
    return per * cells if per else None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["plain", "mixed"], default="mixed")
    ap.add_argument("--tiles", type=int, nargs=3, default=None,
                    help="level-1 tiling (default 16 16 16; 8 8 8 for --precision and --adjoint)")
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 form timed beside the mixed headline")
    ap.add_argument("--no-profile", action="store_true",
                    help="skip the profiled pass (per-kernel times, roofline)")
    ap.add_argument("--persistent", action="store_true",
                    help="mixed form: run each pressure solve as the persistent cooperative "
                         "launch (the fastest variant that applies) instead of the per-phase graph")
    ap.add_argument("--precision", action="store_true",
                    help="error of the mixed form against the plain FP64 form")
    ap.add_argument("--precision-field", choices=["solenoidal", "taylor-green"],
                    default="solenoidal",
                    help="with --precision: the solenoidal random field (nu=1e-3, dt=2e-4) or "
                         "Taylor-Green plus noise (nu=1/1600, dt=5e-4)")
    ap.add_argument("--parity", action="store_true",
                    help="one time step of the plain FP64 form and of the CPU restatement on the "
                         "full tiling, compared bit for bit")
    ap.add_argument("--adjoint", action="store_true",
                    help="dJ/df of the final kinetic energy by the discrete adjoint, timed, with a "
                         "finite-difference check")
    ap.add_argument("--sphere", action="store_true",
                    help="the multi-level ghost-cell case: a sphere in a channel, 16x8x8 level-1 "
                         "grids of 24^3 and two refinement levels, both forms")
    ap.add_argument("--sphere-check", action="store_true",
                    help="with --sphere: one RK stage of the full case on the GPU and on the CPU "
                         "restatement, compared bit for bit")
    ap.add_argument("--channel", action="store_true",
                    help="the sphere channel's three-level hierarchy without the body (1024 + 704 "
                         "+ 2112 grids of 24^3, FIX inflow, OP1 outflow): the mixed form timed "
                         "against the plain FP64 form, and their difference after the timed steps")
    ap.add_argument("--fd-dirs", type=int, default=20,
                    help="random directions of the adjoint's finite-difference check")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_case(args):
    from mglet_gb300 import cases
    nx, ny, nz = args.tiles
    return cases.periodic_box(nx, ny, nz, n=args.n)


def init_fields(case):
    from mglet_gb300 import cases
    u, v, w, p = cases.taylor_green(case)
    u, v, w = cases.add_noise(case, (u, v, w), amplitude=1e-2, seed=42)
    return u, v, w, p


DT = 5e-4


def flow_params(form):
    from mglet_gb300 import abi
    forms = {"mixed": abi.FORM_MIXED, "plain": abi.FORM_PLAIN, "plain_fma": abi.FORM_PLAIN_FMA}
    return abi.make_flow_params(gmol=1.0 / 1600, rho=1.0, epcorr=1e-10, nouter=9, ninner=5,
                                nouter_min=0, form=forms[form])


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return out
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for q, nm in enumerate(names):
                if r[5 + q].lower() == "active":
                    reasons.add(nm)
        out["sm_mhz"] = sm[len(sm) // 2] if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_sample(threads=None, tiles=(8, 8, 8), steps=4, warmup=1):
    """The CPU restatement on a bounded sample of the same workload: a
    periodic 8x8x8 tiling of 24^3 grids (7.1 M cells), Williamson RK3,
    about ten seconds of host work."""
    from oracle import binding
    from mglet_gb300 import cases
    binding.build()
    if threads:
        binding.set_threads(threads)
    nthreads = binding.max_threads()
    case = cases.periodic_box(*tiles, n=24)
    o = binding.Oracle(case, flow_params("plain"))
    for nm, a in zip("UVWP", init_fields(case)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = binding.rk_scheme("williamson")
    it = 0
    for _ in range(warmup):
        it += 1
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
    t0 = time.perf_counter()
    for _ in range(steps):
        it += 1
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, 5e-4, irk, rk)
    dt = time.perf_counter() - t0
    value = case.ncells * steps / dt
    return value, nthreads, (f"{tiles[0]}x{tiles[1]}x{tiles[2]} periodic tiling of 24^3 grids "
                             f"({case.ncells} cells), {steps} steps after {warmup} warm-up, "
                             f"{dt:.1f} s")


def run_reference(args, rank):
    """The CPU restatement of the reference path on the host cores, on the
    same workload as the GPU arm (the full tiling, Taylor-Green + noise,
    Williamson RK3, dt = 5e-4, the same SIP settings).  A time step of the
    full tiling takes about half a minute on 16 cores, so the arm times at
    most REF_STEPS of the requested steps after one warm-up step and says so
    in its sample; the value is cell-updates per second of those steps."""
    if rank != 0:
        return 0
    from oracle import binding
    binding.build()
    case = make_case(args)
    o = binding.Oracle(case, flow_params("plain"))
    for nm, a in zip("UVWP", init_fields(case)):
        o.set(nm, a)
    o.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = binding.rk_scheme("williamson")
    nthreads = binding.max_threads()
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, REF_STEPS))
    it = 0
    for _ in range(warm):
        it += 1
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, DT, irk, rk)
    t0 = time.perf_counter()
    for _ in range(steps):
        it += 1
        for irk in range(1, 4):
            o.timeintegrate_flow(it, it, 0.0, DT, irk, rk)
    dt = time.perf_counter() - t0
    value = case.ncells * steps / dt
    sample = (f"{args.tiles[0]}x{args.tiles[1]}x{args.tiles[2]} periodic tiling of {args.n}^3 grids "
              f"({case.ncells} cells, the GPU arm's workload), {steps} timed steps after {warm} "
              f"warm-up, {dt:.1f} s on {nthreads} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: Taylor-Green + splitmix64 noise (seed 42)",
        "config": {"workload": f"periodic {case.ngrid} x {args.n}^3 grids "
                               f"({args.tiles[0]}x{args.tiles[1]}x{args.tiles[2]}), TG+noise, RK3 "
                               "dt=5e-4, SIP ninner=5 nouter=9 epcorr=1e-10",
                   "timed_steps": steps, "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# time steps of the full tiling the reference arm times (about 30 s each on
# 16 host cores)
REF_STEPS = 3


def reduce_max(value, dist):
    """The largest value over all ranks (the step time every rank reports is
    the slowest rank's); the identity without a process group."""
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_form(args, form, case, fields, local, dist, profile=True):
    """K unprofiled steps on the device (CUDA events on the solver's stream),
    then, if asked, K profiled steps for the per-kernel times.  Returns the
    solver (still open), the step time and the kernel table."""
    import torch
    from mglet_gb300 import gpu

    prm = flow_params(form)
    s = gpu.Solver(case, prm, device=local)
    if form == "mixed" and getattr(args, "persistent", False):
        # 256-thread variants, fastest first as measured on 24^3 grids
        for v in (5, 2, 4, 1, 3, 0):
            try:
                s.force_variant("mx_sip_solve", v)
                break
            except gpu.MgletError:
                continue
    for nm, a in zip("UVWP", fields):
        s.set(nm, a)
    s.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = gpu.rk_scheme("williamson")
    stream = torch.cuda.ExternalStream(s.stream, device=local)
    state = {"it": 0}

    def step():
        state["it"] += 1
        st = None
        for irk in range(1, 4):
            st = s.timeintegrate_flow(state["it"], state["it"], 0.0, DT, irk, rk)
        return st

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    s.synchronize()
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    l0 = s.launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks.start()
    ipcs = []
    e0.record(stream)
    for _ in range(args.steps):
        ipcs.append(step().ipc)
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = s.launches - l0
    ms = reduce_max(ms, dist)
    kern, prof_ms = {}, None
    if profile:
        s.profile(True)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.steps):
            step()
        p1.record(stream)
        p1.synchronize()
        prof_ms = p0.elapsed_time(p1)
        for name in s.profile_names():
            tot, n = s.profile_get(name)
            kern[name] = (tot, n)
        s.profile(False)
    return {"solver": s, "ms": ms, "launches": launches, "clocks": clk, "ipcs": ipcs,
            "kern": kern, "prof_ms": prof_ms, "step": step, "prm": prm, "tuning": s.tuning()}


def roofline(kern, case, ninner, prof_ms):
    """Roofline object of the dominant kernel family of the profiled pass."""
    if not kern:
        return None
    peak, peak_kind = measured_peaks()
    top = max(kern, key=lambda k: kern[k][0])
    tot, n = kern[top]
    b = kernel_bytes(top, case, ninner)
    if not b or not n:
        return None
    achieved = b / (tot / n / 1e3) / 1e9
    rw = NCU_DRAM_4096.get(top) if case.n_interior == 24 else None
    scale = case.ncells / NCU_CELLS
    traffic = (rw[0] + rw[1]) * scale if rw else None
    return {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "traffic_read": rw[0] * scale if rw else None,
            "traffic_write": rw[1] * scale if rw else None,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch on "
                               "4096 x 24^3 grids, mean over one outer iteration's launches"
                               + ("" if scale == 1.0 else ", scaled by cells") if rw else None),
            "share": tot / prof_ms if prof_ms else None,
            "algorithmic_bytes_per_launch": b, "avg_launch_ms": tot / n}


def kernel_roofs(kern, case, ninner, fp64=None):
    """Per kernel family: average launch time, algorithmic bytes and flops
    per launch, the fraction of the measured HBM bandwidth and, for the FP64
    kernels with a known instruction count, the fraction of the measured FP64
    issue rate; "bound" names the larger of the two."""
    peak, _ = measured_peaks()
    out = {}
    for name, (tot, n) in kern.items():
        if not n:
            continue
        ms = tot / n
        row = {"avg_launch_ms": ms, "launches": n}
        b = kernel_bytes(name, case, ninner)
        if b:
            row["bytes_per_launch"] = b
            row["hbm_frac"] = b / (ms / 1e3) / 1e9 / peak
        ipc = FP64_INSTR_PER_CELL.get(name)
        if ipc and fp64:
            rate = ipc * case.ncells / (ms / 1e3)
            row["fp64_instr_per_cell"] = ipc
            row["fp64_frac"] = rate / fp64["dfma"]
        if "hbm_frac" in row or "fp64_frac" in row:
            row["bound"] = ("fp64" if row.get("fp64_frac", 0) > row.get("hbm_frac", 0)
                            else "hbm")
        out[name] = row
    return out


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    case = make_case(args)
    fields = init_fields(case)
    prof = not args.no_profile
    from mglet_gb300 import gpu
    fp64 = gpu.fp64_roof(local)
    r = time_form(args, args.form, case, fields, local, dist, profile=prof)
    s = r["solver"]
    ms = r["ms"]
    value = case.ncells * args.steps * world / (ms / 1e3)
    roof = roofline(r["kern"], case, r["prm"].ninner, r["prof_ms"])

    # end to end through the public API with host buffers: every step uploads
    # u, v, w, p from pinned host memory and downloads them again
    e2e = None
    if not args.no_e2e:
        n = case.idim3d
        host = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(4)]
        for h, a in zip(host, fields):
            h.copy_(torch.from_numpy(a))
        ksteps = args.steps
        s.synchronize()
        t0 = time.perf_counter()
        for _ in range(ksteps):
            for nm, h in zip("UVWP", host):
                s.set_ptr(nm, h.data_ptr(), n)
            r["step"]()
            for nm, h in zip("UVWP", host):
                s.get_ptr(nm, h.data_ptr(), n)
        s.synchronize()
        te = time.perf_counter() - t0
        e2e = {"value": case.ncells * ksteps * world / te, "unit": UNIT,
               "h2d_bytes_per_step": 4 * n * 8, "d2h_bytes_per_step": 4 * n * 8,
               "steps": ksteps}
    s.close()

    plain = None
    if args.form == "mixed" and not args.no_plain:
        q = time_form(args, "plain", case, fields, local, dist, profile=prof)
        parity = [q["solver"].get(nm) for nm in "UVWP"]
        q["solver"].close()
        pv = case.ncells * args.steps * world / (q["ms"] / 1e3)
        plain = {"value": pv, "unit": UNIT, "ms_per_step": q["ms"] / args.steps,
                 "gpu_launches": q["launches"], "clocks": q["clocks"],
                 "roofline": roofline(q["kern"], case, q["prm"].ninner, q["prof_ms"]),
                 "kernel_roofs": kernel_roofs(q["kern"], case, q["prm"].ninner, fp64),
                 "kernels_ms": {k: {"total_ms": v[0], "launches": v[1]}
                                for k, v in q["kern"].items()},
                 "mixed_over_plain": value / pv}
        # the same steps with the contracted build of the plain kernels
        f = time_form(args, "plain_fma", case, fields, local, dist, profile=prof)
        fv = case.ncells * args.steps * world / (f["ms"] / 1e3)
        diff = {}
        for nm, a in zip("UVWP", parity):
            b = f["solver"].get(nm)
            if nm == "P":
                a, b = a - a.mean(), b - b.mean()
            diff[nm] = float(np.linalg.norm(b - a) / np.linalg.norm(a))
        f["solver"].close()
        del parity
        plain["fma_build"] = {
            "value": fv, "unit": UNIT, "ms_per_step": f["ms"] / args.steps,
            "over_parity_build": fv / pv, "mixed_over_plain_fma": value / fv,
            "rel_l2_vs_parity_build": diff,
            "what": "MGLET_FORM_PLAIN_FMA: the plain flux and Poisson kernels compiled with "
                    "multiply-add contraction; relative L2 against the bit-exact build after "
                    "the same steps (pressure with its mean removed)",
            "kernels_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in f["kern"].items()},
        }

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            v, nth, sample = cpu_sample()
            cpu = {"value": v, "unit": UNIT, "cores": nth, "kind": "port", "sample": sample}
            v1, _, sample1 = cpu_sample(threads=1, tiles=(2, 2, 2), steps=2)
            cpu["single_thread"] = {"value": v1, "unit": UNIT, "cores": 1, "sample": sample1}
            from oracle import binding
            binding.set_threads(nth)
        except Exception as ex:   # the baseline never blocks the GPU line
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                   "sample": f"failed: {ex}"}

    if rank == 0:
        ipcs = r["ipcs"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.form == "plain" else "f64+f32",
            "data": "synthetic: Taylor-Green + splitmix64 noise (seed 42)",
            "config": {"workload": f"periodic {case.ngrid} x {args.n}^3 grids "
                                   f"({args.tiles[0]}x{args.tiles[1]}x{args.tiles[2]}), "
                                   "TG+noise, RK3 dt=5e-4, SIP ninner=5 nouter=9 epcorr=1e-10",
                       "form": args.form, "cells": case.ncells,
                       "step": "one time step = 3 RK stages with their pressure solves",
                       "l2": "working set > L2 (no flush needed)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "ipc_per_stage_last": ipcs[-1] if ipcs else None,
                       "kernel_times": "separate profiled pass of the same step count"},
            "clocks": r["clocks"],
            "e2e": e2e,
            "gpu_launches": r["launches"],
            "tuning": r["tuning"],
            "roofline": roof,
            "kernels_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in r["kern"].items()},
            "kernel_roofs": kernel_roofs(r["kern"], case, r["prm"].ninner, fp64),
            "fp64_roof": {"dfma_per_s": fp64["dfma"], "dadd_per_s": fp64["dadd"],
                          "dmul_per_s": fp64["dmul"], "tflops_fma": 2 * fp64["dfma"] / 1e12,
                          "how": "independent FP64 chains on every SM, CUDA events, best of 5"},
            "plain_fp64": plain,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_precision(args, rank, local):
    """Precision of the mixed form: 24^3 grids tiling a periodic box of side
    2 pi, a seeded solenoidal random field (Gaussian shell around k = 4, rms
    velocity 1) projected once by the FP64 pressure solve, nu = 1e-3,
    Williamson RK3 at dt = 2e-4, pressure solved to max|rhs|/prefak < 1e-10
    (up to 40 outer iterations).  The plain FP64 form, bit-identical to the
    CPU restatement, is the reference; the error is the relative L2 norm over
    the interior (pressure with its mean removed)."""
    import numpy as np
    import torch
    from mglet_gb300 import abi, cases, gpu

    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    case = cases.periodic_box(*args.tiles, n=args.n)
    tg = args.precision_field == "taylor-green"
    if tg:
        u, v, w, p = init_fields(case)
        nu, dtp = 1.0 / 1600, DT
    else:
        u, v, w = cases.divergence_free_modes(case, nmodes=48, kpeak=4.0, urms=1.0, seed=4242)
        p = np.zeros_like(u)
        nu, dtp = 1e-3, 2e-4

    def prm(form):
        return abi.make_flow_params(gmol=nu, rho=1.0, epcorr=1e-10, nouter=40, ninner=5,
                                    nouter_min=0, form=form)
    ref = gpu.Solver(case, prm(abi.FORM_PLAIN), device=local)
    for nm, a in zip("UVWP", (u, v, w, p)):
        ref.set(nm, a)
    ref.connect(0, 2, "U", "V", "W", "P", corners=True)
    if not tg:
        ref.mgpoisl(1.0)   # discrete projection of the initial field
        ref.set("P", p)
    init = [ref.get(nm) for nm in "UVWP"]
    div0 = ref.itinfo(dtp).divmax
    mix = gpu.Solver(case, prm(abi.FORM_MIXED), device=local)
    for nm, a in zip("UVWP", init):
        mix.set(nm, a)
    mix.connect(0, 2, "U", "V", "W", "P", corners=True)
    rk = gpu.rk_scheme("williamson")

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    rows = []
    ipc = {"mixed": 0, "plain": 0}
    t0 = time.perf_counter()
    for it in range(1, args.steps + 1):
        for irk in range(1, 4):
            ipc["plain"] += ref.timeintegrate_flow(it, it, 0.0, dtp, irk, rk).ipc
            ipc["mixed"] += mix.timeintegrate_flow(it, it, 0.0, dtp, irk, rk).ipc
        if it % 50 == 0 or it == args.steps:
            fr = {nm: case.interior(ref.get(nm)) for nm in "UVWP"}
            fm = {nm: case.interior(mix.get(nm)) for nm in "UVWP"}
            row = {"step": it}
            for nm in "UVW":
                row[nm.lower()] = rel(fm[nm], fr[nm])
            row["p"] = rel(fm["P"] - fm["P"].mean(), fr["P"] - fr["P"].mean())
            num = sum(np.sum((fm[nm] - fr[nm]) ** 2) for nm in "UVW")
            den = sum(np.sum(fr[nm] ** 2) for nm in "UVW")
            row["velocity"] = float(np.sqrt(num / den))
            row["divmax_mixed"] = mix.itinfo(dtp).divmax
            row["divmax_plain"] = ref.itinfo(dtp).divmax
            rows.append(row)
            # progress on stderr: a run cut short still leaves its rows
            print(json.dumps(row), file=sys.stderr, flush=True)
    field = ("Taylor-Green + splitmix64 noise 1e-2 (seed 42), nu=1/1600, RK3 dt=5e-4" if tg else
             "solenoidal random field (k ~ 4, rms 1), nu=1e-3, RK3 dt=2e-4")
    line = {"precision": "mixed vs plain FP64", "workload":
            f"periodic {case.ngrid} x {args.n}^3 grids, {field}, epcorr=1e-10 (nouter<=40)",
            "steps": args.steps, "initial_divmax": div0, "errors": rows,
            "pressure_iterations": ipc, "seconds": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)
    mix.close()
    ref.close()
    return 0


def run_parity(args, rank, local):
    """The plain FP64 form against the CPU restatement on the bench workload
    itself (4096 grids of 24^3, Taylor-Green + noise, dt = 5e-4): one time
    step (three stages) on each, every field compared bit for bit."""
    import numpy as np
    import torch
    from mglet_gb300 import gpu
    from oracle import binding

    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    binding.build()
    case = make_case(args)
    fields = init_fields(case)
    prm = flow_params("plain")
    g = gpu.Solver(case, prm, device=local)
    o = binding.Oracle(case, prm)
    for s in (g, o):
        for nm, a in zip("UVWP", fields):
            s.set(nm, a)
        s.connect(0, 2, "U", "V", "W", "P", corners=True)
    rkg, rko = gpu.rk_scheme("williamson"), binding.rk_scheme("williamson")
    t0 = time.perf_counter()
    stats = []
    for irk in range(1, 4):
        sg = g.timeintegrate_flow(1, 1, 0.0, DT, irk, rkg)
        so = o.timeintegrate_flow(1, 1, 0.0, DT, irk, rko)
        stats.append({"ipc": [sg.ipc, so.ipc], "maxrhs": [sg.maxrhs, so.maxrhs]})
    eq = {nm: bool(np.array_equal(g.get(nm), o.get(nm)))
          for nm in ("U", "V", "W", "P", "DU", "DV", "DW")}
    line = {"parity": "plain FP64 GPU form vs CPU restatement, one time step",
            "workload": f"periodic {case.ngrid} x {args.n}^3 grids ({case.ncells} cells), "
                        "Taylor-Green + noise, RK3 dt=5e-4, SIP ninner=5 nouter=9",
            "bit_exact": eq, "stages": stats, "seconds": time.perf_counter() - t0,
            "oracle_threads": binding.max_threads()}
    print(json.dumps(line), flush=True)
    g.close()
    return 0


def run_adjoint(args, rank, local):
    """dJ/df of the kinetic energy after 50 RK3 steps with respect to a
    steady body force: 512 grids of 24^3 tiling a periodic box of side 2 pi,
    the force drawn from a seeded Gaussian random field (rms 0.1, correlation
    length 0.5), nu = 5e-3, dt = 1e-3, from rest, checkpoints every 10 steps,
    the pressure solve at a fixed 12 outer iterations (so that J is a smooth
    function of f).  The gradient (forward + recompute + adjoint) is timed
    beside one forward run, and checked against central differences
    (h = 1e-6) along seeded random directions, taken with the plain FP64
    forward solver (bit-identical to the CPU restatement)."""
    import numpy as np
    import torch
    from mglet_gb300 import abi, cases, gpu

    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    nsteps, ncheck, dt = args.steps, 10, 1e-3
    case = cases.periodic_box(*args.tiles, n=args.n)
    f = cases.gaussian_force(case, rms=0.1, length=0.5, seed=2025)
    prm = abi.make_flow_params(gmol=5e-3, rho=1.0, epcorr=0.0, nouter=12, ninner=5, nouter_min=12,
                               form=abi.FORM_PLAIN)
    rk = gpu.rk_scheme("williamson")
    s = gpu.Solver(case, prm, device=local)
    zero = case.zeros()

    def reset(force):
        for nm in "UVWP":
            s.set(nm, zero)
        for nm in ("DU", "DV", "DW"):
            s.set(nm, zero)
        s.set_body_force(*force)

    def energy(force):
        reset(force)
        for it in range(1, nsteps + 1):
            for irk in range(1, 4):
                s.timeintegrate_flow(it, it, 0.0, dt, irk, rk)
        return s.itinfo(dt).energy

    J0 = energy(f)                                    # warm-up and the reference value
    s.synchronize()
    t0 = time.perf_counter()
    J1 = energy(f)
    s.synchronize()
    t_fwd = time.perf_counter() - t0
    reset(f)
    s.synchronize()
    t0 = time.perf_counter()
    J, grad = s.energy_gradient(nsteps, ncheck, dt, rk)
    s.synchronize()
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(77)
    h = 1e-6
    errs = []
    for _ in range(args.fd_dirs):
        d = [rng.standard_normal(case.idim3d) for _ in range(3)]
        fd = (energy([a + h * b for a, b in zip(f, d)]) - energy([a - h * b for a, b in zip(f, d)])) / (2 * h)
        ad = sum(float(np.dot(g, b)) for g, b in zip(grad, d))
        errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
    line = {"adjoint": "dJ/df, J = kinetic energy after the run",
            "workload": f"periodic {case.ngrid} x {args.n}^3 grids, Gaussian body force (rms 0.1, "
                        f"length 0.5), nu=5e-3, RK3 dt=1e-3, {nsteps} steps from rest, "
                        f"checkpoints every {ncheck}, 12 outer pressure iterations",
            "J": J, "J_forward": J0, "J_repeat": J1,
            "forward_s": t_fwd, "gradient_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
            "fd": {"directions": args.fd_dirs, "h": h, "max_rel_err": max(errs) if errs else None,
                   "median_rel_err": float(np.median(errs)) if errs else None},
            "data": "synthetic"}
    print(json.dumps(line), flush=True)
    s.close()
    return 0


def perturb_fp32(s, case, seed=5):
    """Multiplies the interior of U, V, W by 1 +- 2^-24 (one FP32 unit
    roundoff, random signs): the start of the FP64 form's sensitivity run,
    which measures how far rounding at FP32 level alone carries the flow."""
    import numpy as np
    rng = np.random.default_rng(seed)
    for nm in "UVW":
        a = s.get(nm)
        it = case.interior(a)
        it *= 1.0 + 2.0 ** -24 * rng.choice((-1.0, 1.0), size=it.shape)
        s.set(nm, a)


def field_diff(fa, fb):
    """Relative L2 of the velocity vector and of the pressure (mean removed)
    between two sets of interior fields."""
    import numpy as np
    num = sum(np.sum((fa[n] - fb[n]) ** 2) for n in "UVW")
    den = sum(np.sum(fb[n] ** 2) for n in "UVW")
    pa, pb = fa["P"] - fa["P"].mean(), fb["P"] - fb["P"].mean()
    return {"velocity_rel_l2": float(np.sqrt(num / den)),
            "pressure_rel_l2": float(np.linalg.norm(pa - pb) / np.linalg.norm(pb))}


def run_sphere(args, rank, local):
    """The sphere in a channel, 8D x 4D x 4D: level 1 = 16 x 8 x 8 grids of
    24^3, levels 2 and 3 refined around the sphere (1024 + 704 + 2112
    grids, 53.1 M cells), the ghost-cell IB built from the sphere's signed
    distance, FIX inflow u = 1, OP1 outflow, periodic in y and z, Re_D = 300,
    dt = 0.25 h / U on the finest level, which holds the measured CFL number
    (itinfo's cflmax: the flow speeds up around the body) at about 0.5 -- at
    0.5 h / U the impulsive start drives it above 1 and the run diverges
    within seven steps in both forms; Williamson RK3, SIP ninner = 5,
    nouter = 9, epcorr = 1e-10.  The mixed form and the plain FP64 form each
    run the warm-up and the timed steps from the same start (CUDA events on
    each solver's stream); the line reports the form --form names (mixed by
    default) with the other beside it and the relative L2 difference of the
    fields after the run, and beside that the same difference for the FP64
    form started from a state perturbed by one FP32 unit roundoff (how far
    rounding alone carries this flow)."""
    import numpy as np
    import torch
    from mglet_gb300 import abi, channel, gpu

    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    sc = channel.SphereChannel()
    case = sc.case
    lists = sc.lists
    t_setup = time.perf_counter() - t0
    dt = sc.dt(0.25)
    rk = gpu.rk_scheme("williamson")
    res, fields = {}, {}
    for form in ("mixed", "plain", "perturbed"):
        prm = sc.flow_params(abi.FORM_MIXED if form == "mixed" else abi.FORM_PLAIN, epcorr=1e-10,
                             nouter=9, ninner=5)
        s = gpu.Solver(case, prm, device=local)
        sc.setup(s)
        if form == "perturbed":
            perturb_fp32(s, case)
        stream = torch.cuda.ExternalStream(s.stream, device=local)
        state = {"it": 0}

        def step():
            state["it"] += 1
            st = None
            for irk in range(1, 4):
                st = s.timeintegrate_flow(state["it"], state["it"], 0.0, dt, irk, rk)
            return st

        for _ in range(args.warmup):
            step()
        s.synchronize()
        clocks = Clocks(local)
        torch.cuda.synchronize()
        l0 = s.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks.start()
        ipcs = []
        e0.record(stream)
        for _ in range(args.steps):
            ipcs.append(step().ipc)
        e1.record(stream)
        e1.synchronize()
        clk = clocks.stop()
        ms = e0.elapsed_time(e1)
        info = s.itinfo(dt)
        res[form] = {"value": case.ncells * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                     "launches": s.launches - l0, "clocks": clk,
                     "ipc_per_stage_last": ipcs[-1] if ipcs else None,
                     "itinfo": {"cflmax": info.cflmax, "divmax": info.divmax, "energy": info.energy},
                     "tuning": s.tuning() if form == "mixed" else ""}
        fields[form] = {nm: case.interior(s.get(nm)) for nm in "UVWP"}
        if form == "mixed" and not args.no_profile:
            # per-kernel times of one more step, issued eagerly with events
            s.profile(True)
            step()
            s.synchronize()
            res[form]["kernels_ms"] = {n: s.profile_get(n)[0] for n in s.profile_names()}
            s.profile(False)
        s.close()
    check = None
    if args.sphere_check:
        from oracle import binding
        binding.build()
        prm1 = sc.flow_params(epcorr=1e-10, nouter=9, ninner=5, nouter_min=9)
        g1 = gpu.Solver(case, prm1, device=local)
        o = binding.Oracle(case, prm1)
        tc = time.perf_counter()
        for x in (g1, o):
            sc.setup(x)
        sg = g1.timeintegrate_flow(1, 1, 0.0, dt, 1, rk)
        so = o.timeintegrate_flow(1, 1, 0.0, dt, 1, binding.rk_scheme("williamson"))
        eq = {n: bool(np.array_equal(g1.get(n), o.get(n))) for n in ("U", "V", "W", "P")}
        check = {"form": "plain", "stage": 1, "bit_exact": eq, "ipc": [sg.ipc, so.ipc],
                 "maxrhs": [sg.maxrhs, so.maxrhs], "seconds": time.perf_counter() - tc}
        g1.close()
    levels = [int((case.level == lv).sum()) for lv in (1, 2, 3)]
    form = "plain" if args.form == "plain" else "mixed"
    other = "mixed" if form == "plain" else "plain"
    main, side = res[form], res[other]
    line = {
        "metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if form == "plain" else "f32 fluxes/sweeps, f64 storage",
        "data": "synthetic: uniform inflow past a sphere given by its signed distance",
        "config": {"workload": f"sphere channel 8D x 4D x 4D, {levels[0]}+{levels[1]}+{levels[2]} "
                               f"grids of 24^3 on 3 levels ({case.ncells} cells), ghost-cell IB, "
                               "FIX inflow, OP1 outflow, Re_D=300, measured CFL ~0.5 (dt = 0.25 h/U), RK3, SIP ninner=5 "
                               "nouter=9 epcorr=1e-10",
                   "form": form, "cells": case.ncells, "grids_per_level": levels,
                   "ghost_cell_entries": int(sum(gl[1][0] + gl[2][0] + gl[3][0] for gl in lists)),
                   "intersected_cells": int(sc.geo["icells"].sum()), "dt": dt,
                   "setup_s": t_setup, "ipc_per_stage_last": main["ipc_per_stage_last"],
                   "l2": "working set > L2 (no flush needed)"},
        "clocks": main["clocks"], "gpu_launches": main["launches"], "itinfo": main["itinfo"],
        "tuning": res["mixed"]["tuning"],
        "kernels_ms_mixed_step": res["mixed"].get("kernels_ms"),
        other + "_form": {k: side[k] for k in ("value", "ms_per_step", "launches", "itinfo")},
        "mixed_vs_plain": {"steps": args.warmup + args.steps,
                           **field_diff(fields["mixed"], fields["plain"])},
        "fp64_sensitivity": {"what": "plain form from a start perturbed by 2^-24 vs plain form",
                             **field_diff(fields["perturbed"], fields["plain"])},
        "oracle_check": check,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_channel(args, rank, local):
    """The sphere channel's hierarchy without the sphere: 16 x 8 x 8 level-1
    grids of 24^3 refined twice around the quarter point (1024 + 704 + 2112
    grids, 53.1 M cells), FIX inflow u = 1, OP1 outflow, periodic in y and z,
    nu = 1/300, a Taylor-Green perturbation of 10 % on the mean flow, dt =
    0.25 h / U on the finest level (measured CFL about 0.5), Williamson RK3,
    SIP ninner = 5, nouter = 9,
    epcorr = 1e-10.  The mixed form and the plain FP64 form each run the
    warm-up and the timed steps from the same start (CUDA events on each
    solver's stream); the line reports the mixed form and, beside it, the
    plain one and the relative L2 difference of the fields after the run,
    and the same difference for the FP64 form started from a state
    perturbed by one FP32 unit roundoff (how far rounding alone carries this
    flow)."""
    import numpy as np
    import torch
    from mglet_gb300 import abi, cases, gpu

    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    case = cases.body_refined(16, 8, 8, n=24, length=(8.0, 4.0, 4.0), center=(2.0, 2.0, 2.0),
                              refine_radii=(1.0, 1.0), walls={1: abi.BC_FIX, 2: abi.BC_OP1})
    levels = [int((case.level == lv).sum()) for lv in (1, 2, 3)]
    u, v, w, p = cases.taylor_green(case)
    init = dict(zip("UVWP", (1.0 + 0.1 * u, 0.1 * v, 0.1 * w, 0.01 * p)))
    one = np.ones(case.kk * case.jj)
    dt = 0.25 * float(case.ddx.min())
    rk = gpu.rk_scheme("williamson")
    out = {}
    fields = {}
    for name in ("mixed", "plain", "perturbed"):
        form = abi.FORM_MIXED if name == "mixed" else abi.FORM_PLAIN
        prm = abi.make_flow_params(gmol=1.0 / 300.0, epcorr=1e-10, nouter=9, ninner=5, nouter_min=0,
                                   form=form)
        s = gpu.Solver(case, prm, device=local)
        s.set_hierarchy(case.iparent, case.position)
        for g in range(case.ngrid):
            if case.bctype[g, 0] == abi.BC_FIX:
                s.set_buffer("U", g + 1, 1, one)
        for nm, a in init.items():
            s.set(nm, a)
        for lvl in (1, 2, 3):
            s.connect(lvl, 2, v1="U", v2="V", v3="W", s1="P", corners=True)
        for lvl in (3, 2):
            s.ftoc_multiple(lvl, v=("U", "V", "W"), s=("P",))
        for lvl in (1, 2, 3):
            s.connect(lvl, 1, v1="U", v2="V", v3="W", normal=True, forward=1)
            s.parent(lvl, v=("U", "V", "W"), s=("P",))
            s.bound_flow(lvl)
        if name == "perturbed":
            perturb_fp32(s, case)
        stream = torch.cuda.ExternalStream(s.stream, device=local)
        it = [0]

        def step():
            it[0] += 1
            st = None
            for irk in range(1, 4):
                st = s.timeintegrate_flow(it[0], it[0], 0.0, dt, irk, rk)
            return st

        for _ in range(args.warmup):
            step()
        s.synchronize()
        clocks = Clocks(local)
        torch.cuda.synchronize()
        l0 = s.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks.start()
        e0.record(stream)
        last = None
        for _ in range(args.steps):
            last = step()
        e1.record(stream)
        e1.synchronize()
        clk = clocks.stop()
        ms = e0.elapsed_time(e1)
        info = s.itinfo(dt)
        out[name] = {"itinfo": {"cflmax": info.cflmax, "divmax": info.divmax, "energy": info.energy},
                     "value": case.ncells * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                     "launches": s.launches - l0, "clocks": clk,
                     "nouter_last": last.nouter_done if last else None,
                     "tuning": s.tuning() if name == "mixed" else ""}
        fields[name] = {nm: case.interior(s.get(nm)) for nm in "UVWP"}
        s.close()
    mixed, plain = out["mixed"], out["plain"]
    line = {
        "metric": METRIC, "value": mixed["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mixed["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 fluxes/sweeps, f64 storage",
        "data": "synthetic: uniform inflow with a Taylor-Green perturbation",
        "config": {"workload": f"channel 8 x 4 x 4, {levels[0]}+{levels[1]}+{levels[2]} grids of 24^3 "
                               f"on 3 levels ({case.ncells} cells), FIX inflow, OP1 outflow, nu=1/300, "
                               "measured CFL ~0.5 (dt = 0.25 h/U), RK3, SIP ninner=5 nouter=9 epcorr=1e-10",
                   "form": "mixed", "cells": case.ncells, "grids_per_level": levels, "dt": dt,
                   "l2": "working set > L2 (no flush needed)"},
        "clocks": mixed["clocks"], "gpu_launches": mixed["launches"],
        "nouter_last": mixed["nouter_last"], "tuning": mixed["tuning"], "itinfo": mixed["itinfo"],
        "plain_fp64": {k: plain[k] for k in ("value", "ms_per_step", "launches", "nouter_last", "itinfo")},
        "mixed_vs_plain": {"steps": args.warmup + args.steps,
                           **field_diff(fields["mixed"], fields["plain"])},
        "fp64_sensitivity": {"what": "plain form from a start perturbed by 2^-24 vs plain form",
                             **field_diff(fields["perturbed"], fields["plain"])},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.adjoint:
        if args.steps == 5:
            args.steps = 50
        args.tiles = args.tiles or [8, 8, 8]
        return run_adjoint(args, rank, local)
    if args.precision:
        if args.steps == 5:
            args.steps = 200
        args.tiles = args.tiles or [8, 8, 8]
        return run_precision(args, rank, local)
    if args.sphere:
        if args.tiles:
            raise SystemExit("--sphere runs the full configuration only")
        return run_sphere(args, rank, local)
    if args.channel:
        return run_channel(args, rank, local)
    args.tiles = args.tiles or [16, 16, 16]
    if args.parity:
        return run_parity(args, rank, local)
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
