"""Benchmark of the RK4 residual path on one GB300 (or N replicas).

Default run (N=1): three configurations, each measured end to end.
  * Headline: Sod shock tube at scale, 256x128x128 Hexa8 cells (4,194,304)
    on 1.0x0.5x0.5, rho/p = 1/1 | 0.125/0.1, second order with Green-Gauss
    gradients and the Venkatakrishnan limiter, viscous (constant mu = 1.8e-5,
    Pr = 0.72), dt from CFL 0.5 at t = 0, plain FP64; K timed steps.
  * The first-order inviscid Sod tube on 128x16x16 (dt 1e-5) and the viscous
    flat plate on 512x128x128 (Mach 0.3, Van Albada), each timed over its
    configured step count (200 and 50).
A "step" is one RK4 time step (4 stages) over the whole mesh; the unit of
work is one cell-stage, metric Mcell-stage/s = cells * 4 * steps / s / 1e6.

Timing: W warm-up steps, then the timed steps as CUDA graph launches
bracketed by a barrier and device synchronisation, timed with CUDA events on
the solver's stream. The large meshes' working sets (3-7 GB) are far above
the 129 MB L2; the 32,768-cell mesh fits in L2 and runs back to back as a
solve does. The mixed form (FP32 flux/gradient/limiter, FP64 accumulation and
RK update) is timed on the same meshes, its error against FP64 taken after
each configuration's own step count (200 / 100 / 50). The end-to-end figure
times, per step, the host->device copy of the state from pinned memory, the
step and the device->host copy of the result, all through the C ABI. The CPU
baseline is the oracle port on all host threads, built as the reference's
Makefile builds (-O3, default contraction; the -O2 no-contraction parity
build is timed beside it on the headline). Then the batched ensemble and the
serving loop (saturating stream and 25/50/90 % offered loads). The JSON
line ends with a compact summary of every configuration.

--impl reference times the CPU restatement of the reference's Kokkos OpenMP
loops (oracle port, -O3 timing build, all host threads) on the headline
configuration, with the same config dict.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: options, description
    "sod_2nd_viscous_256x128x128": dict(
        problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=256, ny=128, nz=128, second_order_space=1, viscous=1,
        viscosity_model=1, mu=1.8e-5, prandtl=0.72, ic=1, sod_left=[1.0, 1.0], sod_right=[0.125, 0.1], cfl=0.5,
        ntimesteps=100),
    "sod_1st_inviscid_128x16x16": dict(
        problem_type=0, lx=1.0, ly=0.1, lz=0.1, nx=128, ny=16, nz=16, second_order_space=0, viscous=0,
        ic=1, sod_left=[1.0, 1.0], sod_right=[0.125, 0.1], dt=1e-5, ntimesteps=200),
    # Same physics as the default at 262,144 cells: small case for ncu captures.
    "sod_2nd_viscous_64x64x64": dict(
        problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=64, ny=64, nz=64, second_order_space=1, viscous=1,
        viscosity_model=1, mu=1.8e-5, prandtl=0.72, ic=1, sod_left=[1.0, 1.0], sod_right=[0.125, 0.1], cfl=0.5,
        ntimesteps=100),
    # 2,097,152 cells: the mixed form's arrays (~1 GB) exceed L2, for ncu captures of the mixed kernels.
    "sod_2nd_viscous_128x128x128": dict(
        problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=128, ny=128, nz=128, second_order_space=1, viscous=1,
        viscosity_model=1, mu=1.8e-5, prandtl=0.72, ic=1, sod_left=[1.0, 1.0], sod_right=[0.125, 0.1], cfl=0.5,
        ntimesteps=100),
    "flat_plate_vanalbada_512x128x128": dict(
        problem_type=1, lx=2.0, ly=0.5, lz=0.5, nx=512, ny=128, nz=128, second_order_space=1, viscous=1,
        limiter=1, viscosity_model=1, mu=1.8e-5, prandtl=0.72, ic=2, cfl=0.5, ntimesteps=50),
}
DEFAULT_WORKLOAD = "sod_2nd_viscous_256x128x128"


def kernel_bytes(md, kind, w, second_viscous=True):
    """Algorithmic (compulsory) DRAM bytes of one launch: every array the
    kernel touches read or written once, neighbour data counted once (w =
    bytes of the flux/gradient type). Second-order viscous form on axis-aligned
    faces whose centroid offsets lie along the face axis: the flux reads one
    component each of n, n/|n|, t/|t|, b/|b|, the two offsets, and |n| (7
    values per internal face); the sweep one area component and the cell's
    offset per face."""
    C, Fi = md.ncells, md.internal.nfaces
    Fb = sum(b.nfaces for b in md.bc)
    if kind == "sweep_gradient_limiter":
        # W, V, 1/V, 3 contribution lists, axis flag; writes grad, phi; per face
        # one area component and the offset of each side.
        return C * (5 * w + 8 + 8 + 72 + 1 + 15 * w + 5 * w) + Fi * 3 * w + Fb * 2 * w
    if kind == "internal_face_flux":
        # W, grad and phi of both cells; W only in the first-order inviscid form.
        return Fi * (8 + 7 * w + 5 * w) + C * (25 if second_viscous else 5) * w
    if kind == "boundary_face_flux":
        return Fb * (4 + 16 * w + 5 * w) + Fb * 5 * w
    if kind == "residual_rk_update":
        # flux list, V, U_n and U_np1 (read + write), W; each face flux read once.
        return C * (24 + 8 + 120 + 5 * w) + (Fi + Fb) * 5 * w
    return 0


FP64_LANES_PER_SM_CYCLE = 2   # ncu sm__sass_thread_inst_executed_op_dfma_pred_on.peak_sustained on GB300
NUM_SMS = 152

# Two-sweep compulsory model of a whole RK stage, bytes per cell-stage for the
# second-order viscous path: sweep 1 (gradient, min/max, limiter) reads U 40,
# x_c 24, V 8 and 3 faces x (n 24 + x_f 24 + conn 8), writes grad 120 and
# phi 40 (400 B); sweep 2 (flux, boundary, gather, RK4) reads U 40, grad 120,
# phi 40, x_c 24, V 8, 3 faces x (n, t, b, x_f 96 + conn 8), U_n 40, U_np1 40
# and writes U_np1 40, U_tmp 40 (704 B). The mixed form holds grad, phi and
# geometry in FP32: 232 + 464 B.
STAGE_BYTES_PER_CELL = {8: 1104, 4: 696}


def stage_roofline(C, prof, w):
    """Whole-stage achieved bandwidth under the two-sweep model: bytes per
    cell-stage x cells / (summed kernel time of one stage)."""
    stage_ms = sum(ms / n for ms, n in prof.values())  # one launch of each kind per stage
    peak, peak_kind = load_peaks()
    achieved = STAGE_BYTES_PER_CELL[w] * C / (stage_ms / 1e3) / 1e9
    return {"model": "two-sweep compulsory bytes per cell-stage", "bytes_per_cell_stage": STAGE_BYTES_PER_CELL[w],
            "stage_ms": stage_ms, "achieved": achieved, "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
            "frac": achieved / peak}


def fp64_ceiling(kernel, rates):
    """Measured FP64 ceiling (thread instructions/s) for one kernel's
    instruction mix: its fused multiply-adds at the measured FMA rate, every
    other FP64-pipe instruction at the measured add/multiply rate (the lower
    one on GB300), from the per-item counts of the ncu summary."""
    n = (load_traffic("fp64_thread_inst_per_item") or {}).get(kernel)
    f = (load_traffic("fp64_fma_inst_per_item") or {}).get(kernel)
    if not rates or not n or f is None:
        return None
    addmul = 0.5 * (rates["add"] + rates["mul"])
    return n / (f / rates["fma"] + (n - f) / addmul)


def kernel_rooflines(md, prof, w, sm_mhz, fp64_rates=None, counted=True, second_viscous=True, traffic_key=None):
    """Per-kernel time share, achieved algorithmic GB/s and, where the ncu
    summary gives FP64 instructions per item, FP64-pipe throughput against
    the nominal 2 per SM per clock and against the rates measured on this
    device (fp64_rates: {"add", "mul", "fma"} thread instructions/s).
    counted: the workload has the physics the per-item counts were captured
    on (Sod, second order, viscous, Venkatakrishnan); otherwise no FP64
    fractions are reported. traffic_key: the ncu summary's table of DRAM
    bytes per launch when it was scaled to this workload, else None."""
    total_ms = sum(v[0] for v in prof.values())
    peak, peak_kind = load_peaks()
    fp64 = (load_traffic("fp64_thread_inst_per_item") or {}) if counted else {}
    items = {"sweep_gradient_limiter": md.ncells, "internal_face_flux": md.internal.nfaces,
             "boundary_face_flux": sum(b.nfaces for b in md.bc), "residual_rk_update": md.ncells}
    clock = (sm_mhz or 2070.0) * 1e6
    fp64_peak = FP64_LANES_PER_SM_CYCLE * NUM_SMS * clock
    kernels = {}
    for k, (ms, n) in prof.items():
        per = ms / n
        b = kernel_bytes(md, k, w, second_viscous)
        e = {"ms_per_launch": per, "launches": n, "share": ms / total_ms, "algorithmic_bytes": b,
             "achieved_GBps": b / (per / 1e3) / 1e9}
        if w == 8 and k in fp64:
            inst = fp64[k] * items[k]
            e["fp64_pipe_frac"] = inst / (per / 1e3) / fp64_peak
            ceiling = fp64_ceiling(k, fp64_rates)
            if ceiling:
                e["fp64_measured_ceiling_frac"] = inst / (per / 1e3) / ceiling
        kernels[k] = e
    dom = max(kernels, key=lambda k: kernels[k]["share"])
    d = kernels[dom]
    roofline = {"kernel": dom, "bound": "hbm", "achieved": d["achieved_GBps"], "peak": peak,
                "peak_source": peak_kind, "unit": "GB/s", "frac": d["achieved_GBps"] / peak,
                "traffic": (load_traffic(traffic_key) or {}).get(dom) if traffic_key else None,
                "algorithmic_bytes_per_launch": d["algorithmic_bytes"], "ms_per_launch": d["ms_per_launch"]}
    if roofline["traffic"] is not None:
        roofline["traffic_scaled_from"] = ("128^3 ncu capture (sod_2nd_viscous_128x128x128), scaled by the items "
                                           "per launch; profiles/ncu_traffic.json")
    if "fp64_pipe_frac" in d:
        roofline["fp64_pipe"] = {"frac": d["fp64_pipe_frac"], "peak_inst_per_s": fp64_peak,
                                 "note": "FP64 thread instructions per item from the ncu summary; the plain form "
                                         "is bound by this pipe, not by HBM"}
        if fp64_rates:
            roofline["fp64_pipe"]["measured_rates_inst_per_s"] = fp64_rates
        ceiling = fp64_ceiling(dom, fp64_rates)
        if ceiling:
            roofline["fp64_pipe"].update({
                "measured_ceiling_inst_per_s": ceiling,
                "frac_of_measured": d["fp64_measured_ceiling_frac"],
                "ceiling_note": "add, multiply and fma streams timed on this device by ma_debug_fp64_rate, "
                                "weighted by the kernel's FMA share of FP64 instructions"})
    return roofline, kernels


def flat_plate_inflow(mach=0.3, T=300.0, p=1e5):
    R, g = 287.05, 1.4
    rho = p / (R * T)
    u = mach * (g * R * T) ** 0.5
    return [rho, rho * u, 0.0, 0.0, rho * (R / (g - 1.0) * T + 0.5 * u * u)]


def make_options(ma, name, precision="fp64"):
    kw = dict(WORKLOADS[name])
    o = ma.Options(**kw)
    if name.startswith("flat_plate"):
        o.inflow_state = flat_plate_inflow()
        o.inflow_given = 1
    o.precision = {"mixed": ma.MA_PREC_MIXED, "fp64_fma": ma.MA_PREC_FP64_FMA}.get(precision, ma.MA_PREC_FP64)
    return o


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(key):
    """One table of the committed ncu summary (profiles/ncu_traffic.json), if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except Exception:
        return None


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl != "reference" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, value):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# The configurations the default run measures: (workload, RK4 steps the
# configuration specifies; the mixed form's error is taken after that many
# steps). The Sod 256x128x128 mesh is the headline (value, e2e, roofline).
CONFIG_SUITE = [("sod_1st_inviscid_128x16x16", 200), ("sod_2nd_viscous_256x128x128", 100),
                ("flat_plate_vanalbada_512x128x128", 50)]
DATA_NOTE = "synthetic (seeded mesh generator; analytic Sod / flat-plate initial states)"


def rel_errors(Um, U):
    """Relative L2 error per conserved variable, momentum components against
    the momentum norm (a component that is zero in exact arithmetic, like the
    transverse momentum of Sod, has no meaningful relative error)."""
    mom = max(float(np.linalg.norm(U[:, 1:4])), 1e-300)
    return [float(np.linalg.norm(Um[:, k] - U[:, k]) / (mom if k in (1, 2, 3) else
                                                         max(np.linalg.norm(U[:, k]), 1e-300))) for k in range(5)]


def measure_config(ma, args, world, rank, local, name, err_steps, timed_steps, cpu=("timing",), cpu_seconds=10.0):
    """One configuration end to end: FP64 throughput device-resident and
    through the C ABI with host copies, per-kernel rooflines, the mixed form's
    throughput and its error after the configured steps, and the CPU
    baseline(s) on rank 0."""
    import torch
    o = make_options(ma, name, "fp64")
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    C = md.ncells
    dmesh = ma.DeviceMesh(md)
    solver = ma.TimeSolverExplicitRK4(md, o, device_mesh=dmesh)
    solver.set_state(U0)
    dt = solver.dt
    solver.step(args.warmup)
    solver.synchronize()
    U_start = solver.get_state()  # state entering the timed region (AOS)

    # ---- timed region: K steps from device-resident state ----
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    ms = time_steps(ma, solver, timed_steps)
    clocks = sampler.stop()
    barrier(world)
    ms = allreduce_max(world, ms)
    launches = solver.launches_per_step * timed_steps
    value = world * C * 4 * timed_steps / (ms / 1e3) / 1e6

    # ---- per-kernel durations (same workload, kernels launched one by one) ----
    prof = solver.profile_steps(max(2, min(timed_steps, 10)))
    fp64_rates = {op: ma.fp64_rate(op) for op in ("add", "mul", "fma")}
    wl = WORKLOADS[name]
    second_viscous = bool(wl.get("second_order_space") and wl.get("viscous"))
    # The ncu per-item FP64 counts were captured on the Sod second-order
    # viscous workloads; the traffic table is scaled to the 256x128x128 mesh.
    counted = name.startswith("sod_2nd_viscous")
    scaled = name == DEFAULT_WORKLOAD
    roofline, kernels = kernel_rooflines(md, prof, 8, clocks.get("sm_mhz"), fp64_rates, counted, second_viscous,
                                         "traffic_bytes_per_launch" if scaled else None)
    roofline["stage"] = stage_roofline(C, prof, 8) if second_viscous else None

    # ---- FP64 and mixed after the configured step count, from the initial state ----
    solver.set_state(U0)
    solver.dt = dt
    solver.step(err_steps)
    solver.synchronize()
    U_fp64 = solver.get_state()
    om = make_options(ma, name, "mixed")
    msolver = ma.TimeSolverExplicitRK4(md, om, device_mesh=dmesh)
    msolver.set_state(U0)
    msolver.dt = dt
    msolver.step(err_steps)
    msolver.synchronize()
    errs = rel_errors(msolver.get_state(), U_fp64)
    msolver.set_state(U_start)
    msolver.dt = dt
    msolver.step(args.warmup)
    msolver.synchronize()
    mms = allreduce_max(world, time_steps(ma, msolver, timed_steps))
    mvalue = world * C * 4 * timed_steps / (mms / 1e3) / 1e6
    mprof = msolver.profile_steps(2)
    msolver.close()
    # ---- the opt-in contracted FP64 form: throughput and deviation from the bits ----
    fo = make_options(ma, name, "fp64_fma")
    fsolver = ma.TimeSolverExplicitRK4(md, fo, device_mesh=dmesh)
    fsolver.set_state(U0)
    fsolver.dt = dt
    fsolver.step(err_steps)
    fsolver.synchronize()
    U_fma = fsolver.get_state()
    scale = np.abs(U_fp64).max(axis=0)
    scale[1:4] = scale[1:4].max()
    fma_err = (np.abs(U_fma - U_fp64).max(axis=0) / scale).tolist()
    fsolver.set_state(U_start)
    fsolver.dt = dt
    fsolver.step(args.warmup)
    fsolver.synchronize()
    fms = allreduce_max(world, time_steps(ma, fsolver, timed_steps))
    fvalue = world * C * 4 * timed_steps / (fms / 1e3) / 1e6
    fsolver.close()
    mroofline, mkernels = kernel_rooflines(md, mprof, 4, clocks.get("sm_mhz"), None, counted, second_viscous,
                                           "traffic_bytes_per_launch_mixed" if scaled else None)
    mroofline["stage"] = stage_roofline(C, mprof, 4) if second_viscous else None

    # ---- end to end through the C ABI with pinned host buffers ----
    eo = make_options(ma, name, "fp64")
    eo.cfl = 0.0
    eo.dt = dt
    esolver = ma.TimeSolverExplicitRK4(md, eo, device_mesh=dmesh)
    # Component-major host buffers (MA_LAYOUT_SOA): each step uploads the
    # state that entered the timed region above and reads back its successor.
    hU = torch.empty((5, C), dtype=torch.float64).pin_memory()
    hU.numpy()[:] = U_start.T
    hOut = torch.empty((5, C), dtype=torch.float64).pin_memory()
    state_bytes = C * 5 * 8
    L = ma._lib.lib()
    inp = ma._lib.f64p(hU.numpy())
    outp = ma._lib.f64p(hOut.numpy())

    def e2e_step():
        ma._lib.check(L.ma_solver_set_state(esolver._h, inp, ma.MA_LAYOUT_SOA))
        ma._lib.check(L.ma_solver_step(esolver._h, 1))
        ma._lib.check(L.ma_solver_get_state(esolver._h, outp, ma.MA_LAYOUT_SOA))

    for _ in range(max(1, min(args.warmup, 2))):
        e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(timed_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = allreduce_max(world, time.perf_counter() - t0)
    barrier(world)
    e2e_value = world * C * 4 * timed_steps / e2e_s / 1e6
    # The SoA round trip must give the bits of the same step through the AOS path.
    esolver.set_state(U_start)
    esolver.step(1)
    e2e_verified = bool(np.array_equal(esolver.get_state(), hOut.numpy().T))
    esolver.close()
    solver.close()

    cpu_results = {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        for build in cpu:
            cpu_results[build] = cpu_baseline_sample(ma, oracle, md, o, U0, dt, seconds=cpu_seconds,
                                                     timing=(build == "timing"))
    dmesh.close()
    res = {
        "config": config_dict(name, md, o, world), "dt": dt, "timed_steps": timed_steps,
        "value": value, "ms_per_step": ms / timed_steps, "clocks": clocks, "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "Mcell-stage/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes,
                "path": "ma_solver_set_state + ma_solver_step + ma_solver_get_state, pinned host SoA buffers",
                "input": "state after the warm-up steps", "verified_vs_aos_path": e2e_verified},
        "roofline": roofline, "kernels": kernels,
        "mixed": {"value": mvalue, "unit": "Mcell-stage/s", "ms_per_step": mms / timed_steps,
                  "speedup_vs_fp64": mvalue / value, "rel_l2_error_vs_fp64": errs,
                  "error_note": "momentum components relative to the momentum norm",
                  "error_after_steps": err_steps, "roofline": mroofline, "kernels": mkernels},
        "fp64_fma": {"value": fvalue, "unit": "Mcell-stage/s", "ms_per_step": fms / timed_steps,
                     "speedup_vs_fp64": fvalue / value, "max_rel_error_vs_fp64": fma_err,
                     "error_note": "max over cells of |U_fma - U_fp64| over each variable's largest magnitude "
                                   "(momentum components share one scale)",
                     "error_after_steps": err_steps},
        "cpu_baseline": cpu_results.get("timing"),
    }
    if "parity" in cpu_results:
        res["cpu_baseline_parity_build"] = cpu_results["parity"]
    return res


def one_launch_value(ma, name, steps, warmup, blocks=(128, 256)):
    """The configuration as a one-member batch in single-launch mode: all
    `steps` RK4 steps in one cooperative launch (no per-kernel launches), at
    each block size in `blocks`; the faster is reported."""
    out = {}
    for block in blocks:
        for prec_name, r in _one_launch(ma, name, steps, warmup, block).items():
            if prec_name not in out or r["value"] > out[prec_name]["value"]:
                out[prec_name] = dict(r, tried_blocks=list(blocks))
    return out


def _one_launch(ma, name, steps, warmup, block):
    import torch
    out = {}
    for prec_name in ("fp64", "mixed"):
        o = make_options(ma, name, prec_name)
        md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
        U0 = ma.initial_state(md, o)
        dm = ma.DeviceMesh(md)
        b = ma.Batch(o, capacity=1, budget_bytes=64 << 30)
        grid = b.set_single_launch(block)
        b.add(dm, U0, dt=(o.dt if not o.cfl > 0 else 0.0))
        b.step(warmup)
        b.synchronize()
        stream = torch.cuda.ExternalStream(b.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(steps)
        e1.record(stream)
        b.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec_name] = {"value": md.ncells * 4 * steps / (ms / 1e3) / 1e6, "unit": "Mcell-stage/s",
                          "steps": steps, "launches": 1, "block": block, "grid": grid}
        b.close()
        dm.close()
    return out


def _r(x, n=4):
    """Rounds to n significant digits for the compact summary."""
    if x is None or not isinstance(x, float) or x == 0.0 or not math.isfinite(x):
        return x
    return float("%.*g" % (n, x))


def compact(name, r):
    """A few numbers per configuration for the end of the JSON line."""
    cpu = r.get("cpu_baseline") or {}
    st = (r["roofline"].get("stage") or {})
    mst = (r["mixed"]["roofline"].get("stage") or {})
    out = {"cells": r["config"]["cells"], "timed_steps": r["timed_steps"], "fp64": _r(r["value"]),
           "e2e": _r(r["e2e"]["value"]), "cpu": _r(cpu.get("value")),
           "e2e_vs_cpu": _r(r["e2e"]["value"] / cpu["value"]) if cpu.get("value") else None,
           "fp64_fma": _r(r["fp64_fma"]["value"]), "fma_err": _r(max(r["fp64_fma"]["max_rel_error_vs_fp64"]), 2),
           "mixed": _r(r["mixed"]["value"]), "mixed_speedup": _r(r["mixed"]["speedup_vs_fp64"]),
           "mixed_err": [_r(e, 2) for e in r["mixed"]["rel_l2_error_vs_fp64"]],
           "err_steps": r["mixed"]["error_after_steps"]}
    if r.get("one_launch"):
        out["fp64_one_launch"] = _r(r["one_launch"]["fp64"]["value"])
        out["mixed_one_launch"] = _r(r["one_launch"]["mixed"]["value"])
    if st:
        out["stage_hbm_frac"] = _r(st["frac"], 3)
    if mst:
        out["mixed_stage_hbm_frac"] = _r(mst["frac"], 3)
    return out


def run_ours(args, world, rank, local):
    import torch
    import miniaero_gb300 as ma
    torch.cuda.set_device(local)
    suite = [(n, s) for n, s in CONFIG_SUITE if args.workload == "all" or n == args.workload]
    if args.workload not in ("all",) and not suite:
        suite = [(args.workload, WORKLOADS[args.workload].get("ntimesteps", 100))]
    headline = DEFAULT_WORKLOAD if any(n == DEFAULT_WORKLOAD for n, _ in suite) else suite[0][0]
    results = {}
    for name, err_steps in suite:
        if name == headline:
            timed, cpu = args.steps, ("timing", "parity")
        else:
            # Secondary configurations: their own step counts are timed (the
            # small mesh takes 200 steps of ~0.4 ms; the 8.4 M-cell flat plate 50).
            timed, cpu = max(args.steps, err_steps), ("timing",)
        results[name] = measure_config(ma, args, world, rank, local, name, err_steps, timed, cpu,
                                       cpu_seconds=(12.0 if name == headline else 8.0))
        if results[name]["config"]["cells"] < 1_000_000:
            # A small mesh is launch- and latency-sensitive: also time it as
            # one cooperative launch for all its steps.
            results[name]["one_launch"] = one_launch_value(ma, name, timed, args.warmup)

    batched = serving = None
    # The batch and serving sections describe one GPU: with replicas (N > 1)
    # they would hold every GPU for minutes to report rank 0's copy again.
    if not args.no_extras and world == 1:
        batched = run_batched(ma, steps=max(2, min(args.steps, 10)), warmup=args.warmup)
        serving = run_serving_suite(ma, n_requests=args.serve_requests)

    if rank == 0:
        h = results[headline]
        line = {
            "metric": "Mcell-stage/s", "value": h["value"], "unit": "Mcell-stage/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": h["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA_NOTE, "config": h["config"], "clocks": h["clocks"], "e2e": h["e2e"],
            "gpu_launches": h["gpu_launches"], "roofline": h["roofline"], "cpu_baseline": h["cpu_baseline"],
            "cpu_baseline_parity_build": h.get("cpu_baseline_parity_build"),
            "kernels": h["kernels"], "mixed": h["mixed"],
            "other_configs": {n: {k: v for k, v in r.items() if k not in ("kernels",)}
                              for n, r in results.items() if n != headline},
            "batched": batched,
            "serving": serving,
        }
        # Last, so that a reader of only the end of the output sees them: the
        # key numbers of every configuration, the batch and the serving loads.
        summary = {n: compact(n, r) for n, r in results.items()}
        if batched:
            summary["batched_64_sod_boxes"] = {
                "fp64": _r(batched["fp64"]["value"]), "mixed": _r(batched["mixed"]["value"]),
                "fp64_one_launch": _r(batched["fp64"]["single_launch"]["value"]),
                "mixed_one_launch": _r(batched["mixed"]["single_launch"]["value"])}
        if serving:
            summary["serving"] = serving["summary"]
        line["summary"] = summary
        print(json.dumps(line), flush=True)


ORACLE_BUILDS = {
    True: "oracle port at -O3 with the compiler's default multiply-add contraction (the reference Makefile's "
          "flags, kokkos/Makefile:17)",
    False: "oracle port at -O2 -ffp-contract=off (the parity build)",
}


def cpu_baseline_sample(ma, oracle, md, o, U0, dt, seconds=15.0, nthreads=None, timing=True):
    """Times the oracle port (OpenMP, all host threads) on whole-mesh steps.
    timing=True uses its -O3 timing build, False the parity build."""
    nthreads = nthreads or os.cpu_count() or 1
    st = oracle.Stepper(md, o, U0, dt=dt, nthreads=nthreads, timing=timing)
    t0 = time.perf_counter()
    st.step(1)
    per_step = time.perf_counter() - t0
    untimed = 1
    if per_step < 0.5:
        # A small mesh: the first step carries the thread pool's start-up, so
        # the step time is estimated again over 10 more untimed steps.
        t0 = time.perf_counter()
        st.step(10)
        per_step = (time.perf_counter() - t0) / 10
        untimed += 10
    # As many whole-mesh steps as fill `seconds` (a small mesh takes thousands).
    nsteps = max(1, min(100000, int(seconds / max(per_step, 1e-6))))
    t0 = time.perf_counter()
    st.step(nsteps)
    elapsed = time.perf_counter() - t0
    st.close()
    value = md.ncells * 4 * nsteps / elapsed / 1e6
    return {"value": value, "unit": "Mcell-stage/s", "cores": nthreads, "kind": "port",
            "build": ORACLE_BUILDS[bool(timing)],
            "sample": "%d RK4 steps of the full %d-cell mesh after %d untimed step%s (%.1f s)"
                      % (nsteps, md.ncells, untimed, "" if untimed == 1 else "s", elapsed)}


def config_dict(name, md, o, world):
    """The workload as both arms report it (identical keys and values)."""
    wl = WORKLOADS[name]
    cfg = {"workload": name, "cells": md.ncells, "internal_faces": md.internal.nfaces, "precision": "fp64"}
    if wl.get("cfl"):
        cfg["cfl"] = wl["cfl"]
    else:
        cfg["dt"] = wl["dt"]
    state_mb = md.ncells * 0.8e-3  # ~0.8 KB of device arrays per cell in the FP64 form
    if state_mb > 1000.0:
        cfg["l2"] = "working set ~%.0f GB >> 129 MB L2 (no flush needed)" % (state_mb / 1e3)
    else:
        cfg["l2"] = ("working set ~%.0f MB fits the 129 MB L2; steps run back to back as a solve does (no flush)"
                     % state_mb)
    cfg["parallelism"] = "replicas" if world > 1 else "single GPU"
    return cfg


def run_reference(args, world, rank):
    import miniaero_gb300 as ma
    import oracle
    if rank != 0:
        return
    name = args.workload
    o = make_options(ma, name)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    dt = o.dt
    if o.cfl > 0:
        dt = cfl_dt_host(md, U0, o.cfl)
    nthreads = os.cpu_count() or 1
    st = oracle.Stepper(md, o, U0, dt=dt, nthreads=nthreads, timing=True)
    tw = time.perf_counter()
    st.step(args.warmup)
    per_step = (time.perf_counter() - tw) / max(args.warmup, 1)
    # Each timed step is a whole-mesh RK4 step; the timed region is bounded to
    # about two minutes, timing fewer steps when K steps would not fit.
    timed = max(1, min(args.steps, int(120.0 / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    st.step(timed)
    elapsed = time.perf_counter() - t0
    st.close()
    value = md.ncells * 4 * timed / elapsed / 1e6
    sample = "%d RK4 steps of the full %d-cell mesh after %d warm-up steps" % (timed, md.ncells, args.warmup)
    if timed < args.steps:
        sample += " (bounded: %d of the %d requested steps timed)" % (timed, args.steps)
    line = {
        "impl": "reference", "metric": "Mcell-stage/s", "value": value, "unit": "Mcell-stage/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / timed * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA_NOTE, "config": config_dict(name, md, o, world),
        "cpu_baseline": {"value": value, "unit": "Mcell-stage/s", "cores": nthreads, "kind": "port",
                         "build": ORACLE_BUILDS[True], "sample": sample},
        "e2e": {"value": value, "unit": "Mcell-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cfl_dt_host(md, U, cfl):
    """Host restatement of the device CFL rule (used by the CPU-only arm)."""
    R, g = 287.05, 1.4
    r = U[:, 0]
    u, v, w = U[:, 1] / r, U[:, 2] / r, U[:, 3] / r
    T = (U[:, 4] / r - 0.5 * (u * u + v * v + w * w)) * (g - 1.0) / R
    a = np.sqrt(g * R * T)
    s = np.zeros(md.ncells)

    def add(cells, nrm):
        nn = np.sqrt((nrm ** 2).sum(1))
        un = np.abs(u[cells] * nrm[:, 0] + v[cells] * nrm[:, 1] + w[cells] * nrm[:, 2])
        np.add.at(s, cells, un + a[cells] * nn)

    fi = md.internal
    add(fi.conn[:, 0], fi.normal)
    add(fi.conn[:, 1], fi.normal)
    for b in md.bc:
        add(b.conn[:, 0], b.normal)
    return float(cfl * np.min(md.cell_volumes / s))


def time_steps(ma, solver, K):
    import torch
    stream = torch.cuda.ExternalStream(solver.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    solver.step(K)
    e1.record(stream)
    solver.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def ensemble_members(ma, n=64, seed=0, lo=16, hi=96):
    """Batched-ensemble workload: n Sod boxes on 1.0x0.5x0.5, per-axis cell
    counts log-uniform in [lo, hi], left/right density and pressure ratios
    uniform in [2, 20] over rho = 0.125, p = 0.1 (seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        dims = [int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))) for _ in range(3)]
        rr, pr = rng.uniform(2.0, 20.0, 2)
        o = ma.Options(problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=dims[0], ny=dims[1], nz=dims[2],
                       second_order_space=1, viscous=1, viscosity_model=1, mu=1.8e-5, prandtl=0.72, ic=1,
                       sod_left=[0.125 * rr, 0.1 * pr], sod_right=[0.125, 0.1], cfl=0.5)
        out.append(o)
    return out


def run_batched(ma, steps, warmup, n_members=64):
    """64 meshes in one batch, FP64 and mixed, autotuned launch shapes."""
    import torch
    members = ensemble_members(ma, n_members)
    t0 = time.perf_counter()
    built = []
    for o in members:
        md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
        built.append((o, md, ma.initial_state(md, o), ma.DeviceMesh(md)))
    setup_s = time.perf_counter() - t0
    cells = sum(b[1].ncells for b in built)
    res = {"workload": "64 Sod boxes, per-axis cells log-uniform [16, 96] (seed 0), 2nd order viscous, CFL 0.5",
           "meshes": n_members, "cells": cells, "host_setup_s": setup_s, "timed_steps": steps}
    for prec_name, prec in (("fp64", ma.MA_PREC_FP64), ("mixed", ma.MA_PREC_MIXED)):
        phys = members[0].copy()
        phys.precision = prec
        b = ma.Batch(phys, capacity=n_members, budget_bytes=200 << 30)
        ids = [b.add(dm, U0) for (o, md, U0, dm) in built]
        # Tune on the flow the timed steps see: the limiter's cost depends on
        # how much of each box the waves cover (the autotuner restores states).
        b.step(warmup)
        b.synchronize()
        tuned = b.autotune(reps=2)
        stream = torch.cuda.ExternalStream(b.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        b.step(steps)
        e1.record(stream)
        b.synchronize()
        ms = e0.elapsed_time(e1)
        # The same step with the kernels launched one by one between events.
        bprof = b.profile_steps(2)
        # Same members one after another through the single-mesh solver.
        seq_ms = 0.0
        for (o, md, U0, dm) in built:
            so = o.copy()
            so.precision = prec
            s = ma.TimeSolverExplicitRK4(md, so, device_mesh=dm)
            s.set_state(U0)
            s.step(1)
            s.synchronize()
            st = torch.cuda.ExternalStream(s.stream)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(st)
            s.step(steps)
            a1.record(st)
            s.synchronize()
            seq_ms += a0.elapsed_time(a1)
            s.close()
        block, grid = b.launch
        # The same steps as one cooperative launch (all steps, all members).
        sgrid = b.set_single_launch(256)
        b.step(1)
        b.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        b.step(steps)
        s1.record(stream)
        b.synchronize()
        sms = s0.elapsed_time(s1)
        b.set_single_launch(0)
        b.set_launch(block, grid)
        res[prec_name] = {"value": cells * 4 * steps / (ms / 1e3) / 1e6, "unit": "Mcell-stage/s",
                          "single_launch": {"value": cells * 4 * steps / (sms / 1e3) / 1e6,
                                            "unit": "Mcell-stage/s", "launches": 1, "steps_per_launch": steps,
                                            "block": 256, "grid": sgrid},
                          "ms_per_step": ms / steps,
                          "sequential_single_mesh_value": cells * 4 * steps / (seq_ms / 1e3) / 1e6,
                          "autotuned": {"block": block, "grid": grid, "ms_per_launch": tuned.tolist()},
                          "kernels_in_step": {k: {"ms_per_launch": v[0] / v[1], "launches": v[1]}
                                              for k, v in bprof.items()},
                          "kernels_ms_per_step": sum(v[0] for v in bprof.values()) / 2,
                          "launches_per_step": 16}
        b.close()
    return res


SERVE_SIZES = [32, 48, 64, 96, 128]
SERVE_STEPS = 500


def serving_requests(ma, n_requests, rate, seed=1):
    """The serving stream's requests: Poisson arrivals at `rate` per second
    (seeded), flat-plate solves with Mach uniform in [0.1, 0.6] on n^3 meshes,
    n uniform from SERVE_SIZES. The same seed gives the same request mix at
    every rate; only the arrival times scale."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0, n_requests)
    arrivals = np.cumsum(gaps) / rate
    return [(float(a), int(rng.choice(SERVE_SIZES)), float(rng.uniform(0.1, 0.6))) for a in arrivals]


def serving_physics(ma):
    return ma.Options(problem_type=1, second_order_space=1, viscous=1, limiter=ma.MA_LIMITER_VANALBADA,
                      viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72, precision=ma.MA_PREC_MIXED,
                      cfl=0.5)


def run_serving(ma, reqs, static, budget=150 << 30, tick=25, max_running_cells=8_000_000, nsteps=SERVE_STEPS,
                preload=True):
    """Serves the requests (arrival offset s, n, Mach) through ma.Server:
    admitted under the HBM budget with at most max_running_cells cells
    running at once (the latency control: it bounds how many requests share
    a tick), run with the launch shapes the autotuner picked for the same
    requests as one static batch (tuned once for the workload, before the
    stream starts). Latency = finish - submit per request."""
    phys = serving_physics(ma)
    srv = ma.Server(phys, budget_bytes=budget, tick_steps=tick, capacity=512, thread=True)
    srv.set_max_running_cells(max_running_cells)
    srv.set_launch(*static["launch"])
    t0 = time.perf_counter()
    if preload:
        for n in sorted({n for _, n, _ in reqs}):  # mesh cache warm-up: one device mesh per size
            srv.preload(ma.Server.request(n, n, n, 2.0, 0.5, 0.5, flat_plate_inflow(0.3), nsteps))
    setup_s = time.perf_counter() - t0
    ids = []
    start = time.perf_counter()
    for at, n, mach in reqs:
        now = time.perf_counter() - start
        if at > now:
            time.sleep(at - now)
        ids.append(srv.submit(ma.Server.request(n, n, n, 2.0, 0.5, 0.5, flat_plate_inflow(mach), nsteps)))
    for rid in ids:
        srv.wait(rid, timeout=3600.0)
    wall = time.perf_counter() - start
    infos = [srv.query(r) for r in ids]
    st = srv.stats()
    srv.close()
    lat = np.array([(i.t_finish_ns - i.t_submit_ns) / 1e9 for i in infos])
    queue = np.array([(i.t_admit_ns - i.t_submit_ns) / 1e9 for i in infos])
    done = sum(1 for i in infos if i.state == 2)
    cell_stages = sum(i.cells * 4 * nsteps for i in infos if i.state == 2)
    span = reqs[-1][0] if reqs[-1][0] > 0 else 1.0
    offered = sum(n ** 3 * 4 * nsteps for _, n, _ in reqs) / span
    return {"requests": len(reqs), "completed": done, "tick_steps": tick, "budget_bytes": budget,
            "max_running_cells": max_running_cells, "mesh_cache_setup_s": setup_s,
            "offered_load_mcell_stage_s": offered / 1e6,
            "throughput": {"value": cell_stages / wall / 1e6, "unit": "Mcell-stage/s (wall, first arrival to last)"},
            "throughput_busy": {"value": st["cell_stages"] / max(st["busy_seconds"], 1e-9) / 1e6,
                                "unit": "Mcell-stage/s (while requests run)"},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "queue_wait_s": {"p50": float(np.percentile(queue, 50)), "p99": float(np.percentile(queue, 99))},
            "peak_running": st["peak_running"], "peak_bytes": st["peak_bytes"],
            "saturated": bool(offered / 1e6 > cell_stages / wall / 1e6),
            "serving_vs_batched": (cell_stages / wall / 1e6) / static["value"]}


def run_serving_suite(ma, n_requests=32, rate=200.0, loads=(0.25, 0.5, 0.9), n_load_requests=16,
                      budget=150 << 30):
    """Serving at the configured saturating stream (Poisson 200/s, more work
    offered than one GPU carries: throughput against the static batch) and at
    offered loads of 25, 50 and 90 % of the static batch's throughput (same
    request mix, seeded; latency below saturation)."""
    phys = serving_physics(ma)
    sat_reqs = serving_requests(ma, n_requests, rate)
    static = run_static_batch(ma, phys, sat_reqs, budget)
    mean_work = float(np.mean([n ** 3 for n in SERVE_SIZES])) * 4 * SERVE_STEPS  # cell-stages per request
    out = {"workload": "Poisson arrivals of flat-plate requests, Mach U[0.1,0.6], sizes {32,48,64,96,128}^3, "
                       "%d steps, mixed precision, 150 GiB budget" % SERVE_STEPS,
           "launch": {"block": static["launch"][0], "grid": static["launch"][1]},
           "batched_same_requests": static,
           "latency_control": "max_running_cells caps the cells running at once; the HBM budget "
                              "(150 GiB) never binds for these request sizes"}
    out["saturating_200_per_s"] = run_serving(ma, sat_reqs, static, budget=budget)
    for load in loads:
        r = load * static["value"] * 1e6 / mean_work
        out["load_%d_pct" % round(load * 100)] = dict(
            run_serving(ma, serving_requests(ma, n_load_requests, r), static, budget=budget),
            arrival_rate_per_s=r, target_load_of_static_batch=load)
    # Host mesh generation of the largest serving size, geometry on the host's
    # threads and on the device (the server's mesh thread uses the device).
    mo = ma.Options(problem_type=1, nx=128, ny=128, nz=128, lx=2.0, ly=0.5, lz=0.5)
    times = {}
    for dev in (False, True):
        ma.Parallel3DMesh.from_options(mo).fill_mesh_data(device_geometry=dev)  # warm (module load)
        t0 = time.perf_counter()
        md128 = ma.Parallel3DMesh.from_options(mo).fill_mesh_data(device_geometry=dev)
        times["device_geometry" if dev else "host_geometry"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    dm128 = ma.DeviceMesh(md128)
    times["device_upload"] = time.perf_counter() - t0
    dm128.close()
    del md128
    out["mesh_build_128_cubed_s"] = times
    # The 50 % load again with an empty mesh cache: every first request of a
    # size waits for its mesh, built by the server's mesh thread while the
    # running requests keep stepping.
    r = 0.5 * static["value"] * 1e6 / mean_work
    out["load_50_pct_uncached_meshes"] = dict(
        run_serving(ma, serving_requests(ma, n_load_requests, r), static, budget=budget, preload=False),
        arrival_rate_per_s=r, target_load_of_static_batch=0.5)
    summ = {}
    for key in (["saturating_200_per_s"] + ["load_%d_pct" % round(x * 100) for x in loads]
                + ["load_50_pct_uncached_meshes"]):
        v = out[key]
        summ[key] = {"thru": _r(v["throughput"]["value"]), "p50_s": _r(v["latency_s"]["p50"], 3),
                     "p99_s": _r(v["latency_s"]["p99"], 3), "vs_batched": _r(v["serving_vs_batched"], 3)}
    summ["static_batch"] = _r(static["value"])
    out["summary"] = summ
    return out


def run_static_batch(ma, phys, reqs, budget, steps=40, warmup=3, tune_after=25):
    """The serving stream's requests as one static batch (all resident from
    the start, stepped together, autotuned): the batched form's throughput
    on the serving workload."""
    import torch
    meshes = {}
    b = ma.Batch(phys, capacity=len(reqs), budget_bytes=budget)
    cells = 0
    for _, n, mach in reqs:
        o = phys.copy()
        o.nx = o.ny = o.nz = n
        o.lx, o.ly, o.lz = 2.0, 0.5, 0.5
        o.inflow_state = flat_plate_inflow(mach)
        o.inflow_given = 1
        if n not in meshes:
            md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
            meshes[n] = (md, ma.DeviceMesh(md))
        md, dm = meshes[n]
        b.add(dm, ma.initial_state(md, o), inflow_state=flat_plate_inflow(mach))
        cells += md.ncells
    # Tune on a developed flow: at t = 0 the requests are uniform and the
    # limiter idle, so the sweep's timing would not be the serving run's.
    b.step(tune_after)
    b.synchronize()
    b.autotune(reps=2)
    launch = b.launch
    b.step(warmup)
    b.synchronize()
    stream = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(steps)
    e1.record(stream)
    b.synchronize()
    ms = e0.elapsed_time(e1)
    b.close()
    for md, dm in meshes.values():
        dm.close()
    return {"value": cells * 4 * steps / (ms / 1e3) / 1e6, "unit": "Mcell-stage/s", "members": len(reqs),
            "cells": cells, "timed_steps": steps, "launch": launch}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="all", choices=["all"] + sorted(WORKLOADS),
                    help="all: the configuration suite (small Sod, Sod 256x128x128 as the headline, flat plate); "
                         "the reference arm times the headline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and serving sections")
    ap.add_argument("--serve-requests", type=int, default=32)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        if args.workload == "all":
            args.workload = DEFAULT_WORKLOAD
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
