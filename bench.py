#!/usr/bin/env python3
"""k-eigenvalue solves/s of the GB300 hot path, one JSON line on stdout (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one complete k-eigenvalue solve (flat start to convergence, |dk| < 1e-10,
fission-source change < 1e-9) of the workload's synthetic input, generated from a fixed
seed in the reference's .pmp format.  Default workload: 2-group S8 (80 directions)
discrete ordinates on a 3D Cartesian 64x64x32 mesh of 2 cm cells in FP64 (~21M angular
unknowns), pure upwind, reflective -x/-y/-z, vacuum +x/+y/+z.

* value: solves/s with the operator and iterates already resident in HBM, device time
  from CUDA events on the library's launching stream, max over ranks; the L2 is flushed
  (256 MB write) between timed solves.
* e2e: the same metric through the drop-in C API with host buffers: pampa_initialize
  (parse + host assembly) + pampa_solve (upload + solve) + pampa_get_field of the scalar
  flux, angular flux and power + pampa_finalize, wall-clock per step.
* roofline: the transport-sweep kernel, algorithmic bytes (psi written and read once per
  cell-group-direction update, source, moment and material id per cell-group) over its
  CUDA-event time inside the timed solves; peak = measured HBM copy bandwidth.
* cpu_baseline / parity: one complete k-eigenvalue solve of the same input on the host
  cores by oracle/sn_cpu.py (the same power iteration with GMRES over transport sweeps,
  FP64, C + OpenMP sweeps on all host threads), after the timed region; its k and fluxes
  are compared with the GPU's ("parity").
* mixed: the same workload in mixed precision (FP32 sweeps and GMRES, FP64 residual
  refinement), device-timed on the same problem; served: the serving stream's summary.
* --impl reference: complete CPU solves of the same input by oracle/sn_cpu.py, one per
  step (the reference's own LU + Krylov-Schur on this operator would need ~82 GB of AIJ
  storage and is not buildable here).

Multi-GPU: the path does not shard (one solve is one GPU); --gpus N under torchrun runs N
independent replicas and value is the total over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "sn_s8_64x64x32_g2": dict(kind="sn", args=dict(), precision="fp64", dtype="f64",
                               desc="2-group S8 SN k-eigenvalue, 3D Cartesian 64x64x32 (2 cm), ~21M angular unknowns"),
    "sn_s8_64x64x32_g2_mixed": dict(kind="sn", args=dict(), precision="mixed", dtype="f32+f64",
                                     desc="same, FP32 sweeps/GMRES with FP64 residual refinement"),
    "diffusion_2d_34x34_g2": dict(kind="diffusion2d", args=dict(), precision="fp64", dtype="f64",
                                  desc="2-group diffusion k-eigenvalue, 2D Cartesian 34x34 (5 cm)"),
}
WORKLOADS["diffusion_7g_256x256x128_mixed"] = dict(
    kind="diffusion7g", args=dict(), precision="mixed", dtype="f32+f64",
    desc="7-group diffusion k-eigenvalue, 3D Cartesian 256x256x128 (2 cm), 6 materials in 8^3 blocks, "
         "58.7M unknowns, FP32 BiCGStab with FP64 refinement")
WORKLOADS["diffusion_7g_256x256x128"] = dict(
    kind="diffusion7g", args=dict(), precision="fp64", dtype="f64",
    desc="same 7-group 3D diffusion problem, FP64 BiCGStab")
# the Wielandt shift of this problem (k ~ 0.42, high dominance ratio) was measured: 0.02
# takes 641 sweeps per solve against 951 at the SN default 0.05 (1241 at 0.1)
WORKLOADS["sn_hex_s8_g4_mixed"] = dict(
    kind="snhex", args=dict(), precision="mixed", dtype="f32+f64", shift=0.02,
    desc="4-group S8 SN k-eigenvalue on 200x200 hexagonal prisms x 40 layers (1.6M cells, 512M angular "
         "unknowns), vacuum, FP32 level-set sweeps with FP64 refinement")
WORKLOADS["serve_diffusion"] = dict(
    kind="serve", args=dict(), precision="mixed", dtype="f32+f64",
    desc="stream of k-eigenvalue diffusion requests (3D Cartesian 16x16x4..128x128x64 log-uniform, G in {2,4,7}, "
         "+-5% lognormal XS perturbations), continuous batching, k to 1e-8; capacity with the whole stream queued, "
         "p50/p99 latency with Poisson arrivals at 80% of capacity")
DEFAULT = "sn_s8_64x64x32_g2"
# DRAM bytes (read + write) of one launch of each workload's dominant kernel, from ncu
# captures summarised under profiles/: k_sweep_flow on the full S8 workload, FP64 and FP32
# (k_sweep_flow_sn_s8_64x64x32.md); k_bicg_v_cell<float, 7> captured at 128x128x64
# (7.34M rows, 320.7 MB) and scaled by the 8x rows of 256x256x128, its traffic being
# proportional to the rows (k_bicg_v_cell_diffusion_7g_128x128x64.md).
TRAFFIC = {"sn_s8_64x64x32_g2": 108907520, "sn_s8_64x64x32_g2_mixed": 58752768,
           "diffusion_7g_256x256x128_mixed": 2565486592}


def reduce_over_ranks(value: float, dist, device: str, op: str = "max") -> float:
    """`value` reduced over the job's ranks: the maximum for times, the sum for
    throughputs.  Without a process group (one rank) the value itself."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_input(name: str, out_dir: str, size: str | None = None) -> str:
    """The workload's input; `size` ("NXxNYxNZ", profiling captures only) shrinks the box."""
    from pampa_gb300 import workloads as wl
    w = WORKLOADS[name]
    args = dict(w["args"])
    if size and w["kind"] in ("sn", "diffusion7g"):
        args.update(zip(("nx", "ny", "nz"), (int(v) for v in size.lower().split("x"))))
    if w["kind"] == "sn":
        return wl.sn_3d(out_dir, **args)
    if w["kind"] == "diffusion7g":
        return wl.diffusion_3d_7g(out_dir, **args)
    if w["kind"] == "snhex":
        if size:
            args.update(zip(("nq", "nr", "nz"), (int(v) for v in size.lower().split("x"))))
        return wl.sn_hex(out_dir, **args)
    return wl.diffusion_2d(out_dir, **w["args"])


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return dict(hbm_gbs=float(d["hbm_gbs"]), source="measured")
    return dict(hbm_gbs=6800.0, source="fallback")


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"])
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(smax) if smax else None,
                    reasons=sorted(reasons), samples=len(sm))


def cpu_solve(input_path: str) -> dict:
    """One complete CPU k-eigenvalue solve (oracle/sn_cpu.py) of an SN input, with the
    setup (operator tables, upwind orders) outside the timed part."""
    from oracle import pampa_oracle as po, sn_cpu
    S = sn_cpu.SNCpu(po.read_problem(input_path))
    return S.solve()


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    w = WORKLOADS[args.workload]
    if w["kind"] == "diffusion2d":
        return run_reference_diffusion(args, world)
    if w["kind"] != "sn":
        print(json.dumps({"impl": "reference", "unavailable": "the reference's own method (LU + Krylov-Schur on the "
                          "assembled matrix) is timed for the 2D diffusion and the S8 workloads only; this "
                          "workload's matrix is too large for it on this host, or (serving) the reference "
                          "has no counterpart"}))
        return 0
    with tempfile.TemporaryDirectory() as d:
        path = make_input(args.workload, d, args.size)
        from oracle import pampa_oracle as po, sn_cpu
        S = sn_cpu.SNCpu(po.read_problem(path))
        # warm-up steps: solves capped at two outer iterations (page-in, thread start-up)
        for _ in range(args.warmup):
            try:
                S.solve(max_outer=2)
            except RuntimeError:
                pass
        per, res = [], None
        for _ in range(args.steps):
            res = S.solve()
            per.append(res["seconds"])
    t = statistics.mean(per)
    cpu = dict(value=1.0 / t, unit="solves/s", cores=res["threads"], kind="port",
               sample=f"complete k-eigenvalue solves of this workload by oracle/sn_cpu.py (power iteration "
                      f"with GMRES over C + OpenMP transport sweeps, FP64, {res['threads']} threads), one per "
                      f"step: {res['sweeps']} sweeps, {res['outer_iterations']} outer iterations")
    line = dict(metric="k-eigen solves/s", value=1.0 / t, unit="solves/s", n_gpus=world, steps=args.steps,
                warmup=args.warmup, ms_per_step=1e3 * t, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f64", data="synthetic (seeded generator, reference .pmp format)",
                config=dict(workload=args.workload, description=w["desc"], keff=res["keff"],
                            **(dict(size_override=args.size) if args.size else {})), impl="reference",
                cpu_baseline=cpu, e2e=dict(value=1.0 / t, unit="solves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))
    return 0


def oracle_solve_seconds(path: str) -> tuple[float, dict]:
    """One complete k-eigenvalue solve by the oracle (the reference's method restated:
    assembled R and F, SuperLU factor of R, ARPACK on R^-1 F), wall-clock seconds."""
    from oracle import pampa_oracle as po
    t0 = time.perf_counter()
    ref = po.run_input(path)
    return time.perf_counter() - t0, ref


def run_reference_diffusion(args, world):
    w = WORKLOADS[args.workload]
    with tempfile.TemporaryDirectory() as d:
        path = make_input(args.workload, d)
        per = []
        for i in range(args.warmup + args.steps):
            t, ref = oracle_solve_seconds(path)
            if i >= args.warmup:
                per.append(t)
    t = statistics.mean(per)
    cpu = dict(value=1.0 / t, unit="solves/s", cores=1, kind="port",
               sample="complete solves of this workload by oracle/pampa_oracle.py (parse, assembly, SuperLU + "
                      "ARPACK shift-invert, normalisation), one per step")
    line = dict(metric="k-eigen solves/s", value=1.0 / t, unit="solves/s", n_gpus=world, steps=args.steps,
                warmup=args.warmup, ms_per_step=1e3 * t, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f64", data="synthetic (seeded generator, reference .pmp format)",
                config=dict(workload=args.workload, description=w["desc"], keff=ref["keff"]), impl="reference",
                cpu_baseline=cpu, e2e=dict(value=1.0 / t, unit="solves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))
    return 0


def run_ours(args, rank, world, local):
    import ctypes as C
    import numpy as np
    import torch
    import pampa_gb300 as pg

    dev = local
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))

    def barrier():
        if dist is not None:
            dist.barrier()

    w = WORKLOADS[args.workload]
    tmp = tempfile.mkdtemp(prefix=f"bench_r{rank}_")
    path = make_input(args.workload, tmp, args.size)
    if args.shift is not None:
        w = dict(w, shift=args.shift)
    prec = ["-pgpu_precision", w["precision"]]
    if w.get("shift"):
        prec += ["-pgpu_shift", str(w["shift"])]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    # ---- device-resident solves ---------------------------------------------------
    p = pg.Pampa(path, "-silent", "-pgpu_device", str(dev), *prec)
    h = C.c_void_p(None)
    err = C.c_int(0)
    pg.lib().pampa_get_problem(C.byref(h), C.byref(err))
    if err.value:
        raise RuntimeError(pg.last_error())
    opts = pg.default_options(precision=pg.PGPU_MIXED if w["precision"] == "mixed" else pg.PGPU_FP64)
    stats = pg.pgpu_stats()

    if w.get("shift"):
        opts.shift = w["shift"]
    if args.profile_outer:
        opts.max_outer = args.profile_outer

    def solve(profile: int):
        opts.profile = profile
        st = pg.lib().pgpu_problem_solve(h, C.byref(opts), C.byref(stats))
        if st != pg.PGPU_OK and not (args.profile_outer and st == pg.PGPU_ERR_NOT_CONVERGED):
            raise RuntimeError(f"solve failed: {pg.last_error()}")
        return {k: getattr(stats, k) for k, _ in pg.pgpu_stats._fields_}

    # With per-launch events a solve drives its inner iterations from the host one at a time
    # (no CUDA graph chunks for BiCGStab, no graph of conditional Arnoldi steps for GMRES),
    # so the timed region runs the normal path and the dominant kernel's timing comes from
    # one more solve with events right after it (same kernels, same launch shapes).
    for _ in range(args.warmup):
        solve(0)
    results = []
    torch.cuda.synchronize()
    barrier()
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            results.append(solve(0))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier()
    dev_time = reduce_over_ranks(sum(r["seconds"] for r in results), dist, f"cuda:{dev}", "max")
    keff = results[-1]["keff"]
    kres = [solve(1)]
    kres_time = sum(r["seconds"] for r in kres)
    kern_s = sum(r["kernel_seconds"] for r in kres)
    kern_b = sum(r["kernel_bytes"] for r in kres)
    kern_n = sum(r["kernel_launches"] for r in kres)
    launches = sum(r["launches"] for r in results)
    sweeps = results[-1]["sweeps"]
    upload = int(pg.lib().pgpu_problem_upload_bytes(h))
    n_phi = p.field_size("scalar-flux")
    n_psi = p.field_size("angular-flux") if w["kind"] in ("sn", "snhex") else 0
    n_cells = p.field_size("power")

    def fields():
        """Normalised scalar and angular flux of the problem's last solve (host copies)."""
        phi = np.zeros(n_phi)
        if pg.lib().pgpu_problem_get_scalar_flux(h, phi.ctypes.data_as(C.POINTER(C.c_double))) != pg.PGPU_OK:
            raise RuntimeError(pg.last_error())
        psi = None
        if n_psi:
            psi = np.zeros(n_psi)
            if pg.lib().pgpu_problem_get_angular_flux(h, psi.ctypes.data_as(C.POINTER(C.c_double))) != pg.PGPU_OK:
                raise RuntimeError(pg.last_error())
        return phi, psi

    phi64, psi64 = fields() if not args.profile_outer else (None, None)

    # ---- the same problem in mixed precision (FP32 sweeps and GMRES, FP64 refinement) ----
    mixed = None
    if w["kind"] == "sn" and w["precision"] == "fp64" and not args.profile_outer and not args.no_mixed:
        opts.precision = pg.PGPU_MIXED
        for _ in range(args.warmup):
            solve(0)
        mres = []
        torch.cuda.synchronize()
        barrier()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            mres.append(solve(0))
        torch.cuda.synchronize()
        barrier()
        mtime = reduce_over_ranks(sum(r["seconds"] for r in mres), dist, f"cuda:{dev}", "max")
        phim, psim = fields()
        rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
        mixed = dict(value=world * args.steps / mtime, unit="solves/s", ms_per_step=1e3 * mtime / args.steps,
                     dtype="f32+f64", speedup_vs_fp64=(args.steps / mtime) / (args.steps / dev_time),
                     keff=mres[-1]["keff"], dk_vs_fp64=abs(mres[-1]["keff"] - keff),
                     flux_l2_vs_fp64=rel(phim, phi64), psi_l2_vs_fp64=rel(psim, psi64),
                     sweeps_per_solve=mres[-1]["sweeps"], outer_iterations=mres[-1]["outer_iterations"],
                     gmres_iterations=mres[-1]["inner_iterations"],
                     # one FP64 residual sweep per outer iteration and the final FP64 sweep for
                     # psi; the GMRES correction sweeps are FP32
                     sweeps_fp64=mres[-1]["outer_iterations"] + 1,
                     sweeps_fp32=mres[-1]["sweeps"] - mres[-1]["outer_iterations"] - 1,
                     gpu_launches=int(sum(r["launches"] for r in mres)),
                     timing="device time (CUDA events) of the same number of complete solves as the FP64 "
                            "line, same problem resident in HBM, L2 flushed between solves")
        opts.precision = pg.PGPU_FP64
    p.finalize()

    # ---- end-to-end through the drop-in API -------------------------------------
    e2e_times = []
    for i in range(0 if args.profile_outer else max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        q = pg.Pampa(path, "-silent", "-pgpu_device", str(dev), *prec)
        q.solve()
        q.field("scalar-flux")
        if n_psi:
            q.field("angular-flux")
        q.field("power")
        q.finalize()
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t1)
    e2e_t = reduce_over_ranks(statistics.mean(e2e_times) if e2e_times else float("inf"), dist, f"cuda:{dev}", "max")

    peaks = measured_peaks()
    achieved = kern_b / kern_s / 1e9 if kern_s > 0 else None
    kname = kres[-1]["kernel_name"]
    kname = kname.decode() if isinstance(kname, bytes) else str(kname)
    roof = dict(bound="hbm", kernel=kname,
                achieved=achieved, peak=peaks["hbm_gbs"], unit="GB/s",
                frac=(achieved / peaks["hbm_gbs"]) if achieved else None, peak_source=peaks["source"],
                traffic=None, launches=kern_n,
                kernel_share_of_solve=kern_s / kres_time if kres_time > 0 else None,
                timing="CUDA events around every launch of the kernel in one solve right after the timed ones")
    if w["kind"] == "sn" and kern_s > 0:
        # the transport sweep is bound by FP64 issue on GB300 (FP64 = 1/64 of FP32): per
        # (cell, group, direction) update one multiply and three FMAs (7 flops); the
        # mixed-precision workload's correction sweeps are FP32 and only its residual
        # sweeps count here.  Peak: nominal GB300 FP64, 1.25 TFLOP/s (no measured figure).
        sw = kern_n / 2.0 if kname == "k_sweep_flow" else float(sum(r["sweeps"] for r in kres))
        # the sweep's own rate: (cell, group, direction) updates per second of sweep time
        roof["updates_per_s"] = n_psi * sw / kern_s
        if w["precision"] == "fp64":
            ach = 7.0 * n_psi * sw / kern_s / 1e12
            roof["fp64"] = dict(flops_per_update=7, achieved_tflops=ach, nominal_peak_tflops=1.25,
                                frac_of_nominal=ach / 1.25)
    roof["traffic"] = TRAFFIC.get(args.workload)

    line = dict(metric="k-eigen solves/s", value=world * args.steps / dev_time, unit="solves/s", n_gpus=world,
                steps=args.steps, warmup=args.warmup, ms_per_step=1e3 * dev_time / args.steps,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype=w["dtype"],
                data="synthetic (seeded generator, reference .pmp format)",
                config=dict(workload=args.workload, description=w["desc"], keff=keff,
                            sweeps_per_solve=sweeps, outer_iterations=results[-1]["outer_iterations"],
                            inner_iterations=results[-1]["inner_iterations"],
                            inner_solver="GMRES over sweeps" if w["kind"].startswith("sn") else "BiCGStab",
                            l2="flushed (256 MB write) between steps",
                            parallelism=f"replicas x{world}" if world > 1 else "1 GPU",
                            wall_ms_per_step=1e3 * wall / args.steps,
                            wielandt_shift=w.get("shift") or "solver default",
                            **(dict(size_override=args.size) if args.size else {})),
                e2e=dict(value=world / e2e_t, unit="solves/s", h2d_bytes_per_step=upload,
                         d2h_bytes_per_step=8 * (n_phi + n_psi + n_cells),
                         note="drop-in pampa_* API: parse + host assembly + upload + solve + field reads; "
                              "host buffers are pageable"),
                gpu_launches=launches, roofline=roof, clocks=clk.summary())
    if args.profile_outer:
        line["profile_run"] = f"solves capped at {args.profile_outer} outer iterations; not a benchmark result"
    if rank == 0 and world == 1 and w["kind"] == "diffusion2d" and not args.no_cpu and not args.profile_outer:
        try:
            t, _ = oracle_solve_seconds(path)
            line["cpu_baseline"] = dict(value=1.0 / t, unit="solves/s", cores=1, kind="port",
                                        sample="one complete solve by oracle/pampa_oracle.py (SuperLU + ARPACK)")
        except Exception as e:
            line["cpu_baseline"] = dict(value=None, unavailable=str(e))
    if mixed is not None:
        line["mixed"] = mixed
    if rank == 0 and world == 1 and w["kind"] == "sn" and not args.no_cpu and not args.profile_outer:
        # one complete CPU solve of the same input: the CPU baseline, and the parity check
        # of the GPU result at the workload's full size
        try:
            cpu = cpu_solve(path)
            rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
            line["cpu_baseline"] = dict(
                value=1.0 / cpu["seconds"], unit="solves/s", cores=cpu["threads"], kind="port",
                sample=f"one complete k-eigenvalue solve of this workload by oracle/sn_cpu.py (power iteration with "
                       f"GMRES over C + OpenMP transport sweeps, FP64, {cpu['threads']} threads; {cpu['sweeps']} "
                       f"sweeps, {cpu['outer_iterations']} outer iterations)")
            line["parity"] = dict(
                vs="oracle/sn_cpu.py complete FP64 CPU solve of the same input (checked against the oracle's direct "
                   "solve on small meshes by the CPU tests)",
                dk=abs(keff - cpu["keff"]), flux_l2=rel(phi64, cpu["phi"]),
                psi_l2=rel(psi64, cpu["psi"]) if psi64 is not None else None,
                k_tol=1e-6, flux_tol=1e-5)
            if mixed is not None:
                line["parity"]["mixed_dk"] = abs(mixed["keff"] - cpu["keff"])
                line["parity"]["mixed_k_tol"] = 1e-5
        except Exception as e:  # the baseline never decides the GPU result
            line["cpu_baseline"] = dict(value=None, unavailable=str(e))
    if world == 1 and args.workload == DEFAULT and not args.no_serve and not args.profile_outer and not args.size:
        served = serve_stream(args, rank, dev, dist)
        line["served"] = {k: served[k] for k in (
            "value", "unit", "speedup_vs_fp64_one_at_a_time", "fp64_one_at_a_time", "mixed_one_at_a_time",
            "latency", "dk_max_vs_fp64", "dk_max_between_passes", "gpu_launches")}
        line["served"]["config"] = {k: served["config"][k] for k in (
            "workload", "description", "requests", "slots", "mean_unknowns", "mean_outer_iterations",
            "mean_inner_iterations")}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_serve(args, rank, world, local):
    """Serving workload: a stream of diffusion requests of uneven size through the
    pgpu_serve_* continuous-batching server (FP32 inner solves + FP64 refinement), next to
    the plain FP64 path solving the first requests one at a time.

    Two passes over the same requests: (1) capacity: every request is submitted at once,
    value = requests / time to the last answer; (2) latency: Poisson arrivals at 80 % of
    that capacity, p50/p99 of submit-to-answer.  Requests are built before the timed
    passes (in a process pool), so the host generator is not what is measured.  Every rank
    serves its own stream (replicas); value is the total over ranks."""
    import torch

    dev = local
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    line = serve_stream(args, rank, dev, dist)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def serve_stream(args, rank, dev, dist) -> dict:
    """Builds the seeded request stream and measures it (see run_serve); returns the line."""
    import math
    import multiprocessing as mp
    import queue
    import threading

    import numpy as np
    import torch

    import pampa_gb300 as pg
    from pampa_gb300 import workloads as wl

    rng = np.random.default_rng(4 + rank)
    nreq = args.requests
    world = dist.get_world_size() if dist is not None else 1

    def loguni(lo, hi):
        return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))

    specs = [(loguni(16, 128), loguni(16, 128), loguni(4, 64), int(rng.choice([2, 4, 7]))) for _ in range(nreq)]
    seeds = rng.integers(0, 2**31 - 1, size=nreq)
    procs = max(1, min(16, (os.cpu_count() or 2) // max(1, world)))
    with mp.get_context("spawn").Pool(procs) as pool:
        ops = pool.map(wl.diffusion_request_op, [(*specs[k], int(seeds[k])) for k in range(nreq)], chunksize=4)

    # power iteration to 1e-8 on k and 1e-7 on the fission source, as the small plain
    # workload is specified (served answers are compared at 1 pcm)
    fp64 = pg.default_options(precision=pg.PGPU_FP64, tol_k=1e-8, tol_flux=1e-7)
    mixed = pg.default_options(precision=pg.PGPU_MIXED, tol_k=1e-8, tol_flux=1e-7)
    if args.shift is not None:
        fp64.shift = mixed.shift = args.shift
    # 0. plain FP64, one request at a time, on the first requests of the stream
    sample = min(nreq, args.serve_sample) if args.serve_sample > 0 else nreq
    def one_at_a_time(opts):
        """keff and run seconds of the sample's requests solved one after the other."""
        ks, runs = [], []
        with pg.Server(dev, slots=1) as srv:
            srv.wait(srv.submit_diffusion(ops[0], opts))  # warm-up
            t0 = time.perf_counter()
            for op in ops[:sample]:
                out = srv.wait(srv.submit_diffusion(op, opts))
                if out["status"] != pg.PGPU_OK:
                    raise RuntimeError(f"one-at-a-time solve failed: {out.get('error')}")
                ks.append(out["keff"])
                runs.append(out["run_s"])
            return ks, runs, time.perf_counter() - t0

    k64, run64, t64 = one_at_a_time(fp64)
    rate64 = sample / t64
    _, run32, t32 = one_at_a_time(mixed)
    rate32 = sample / t32

    def serve(arrivals):
        """Submits request k at arrivals[k] seconds after the start; returns the results
        (with completion times) and the wall time from the start to the last answer."""
        results = [None] * nreq
        ids = queue.Queue()
        with pg.Server(dev, slots=args.slots, sm_share=args.sm_share) as srv:
            srv.wait(srv.submit_diffusion(ops[0], mixed))  # warm-up

            def waiter():
                while True:
                    item = ids.get()
                    if item is None:
                        return
                    k, rid = item
                    results[k] = srv.wait(rid)
                    results[k]["t_done"] = time.perf_counter()

            wt = [threading.Thread(target=waiter, daemon=True) for _ in range(4)]
            for t in wt:
                t.start()
            t_start = time.perf_counter()
            for k in range(nreq):
                delay = t_start + arrivals[k] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                ids.put((k, srv.submit_diffusion(ops[k], mixed)))
            for _ in wt:
                ids.put(None)
            for t in wt:
                t.join()
        bad = [(k, r) for k, r in enumerate(results) if r["status"] != pg.PGPU_OK]
        if bad:
            raise RuntimeError(f"{len(bad)} served solves failed: " + "; ".join(
                f"#{k} {specs[k]} status {r['status']} {r.get('error', '')}" for k, r in bad[:8]))
        return results, max(r["t_done"] for r in results) - t_start

    # 1. capacity: the whole stream at once
    with ClockSampler(dev) as clk:
        results, wall = serve(np.zeros(nreq))
    value = nreq / wall
    lat_sat = np.array([r["latency_s"] for r in results])
    # 2. latency at 80 % of capacity, Poisson arrivals
    load = 0.8 * value
    arrivals = np.cumsum(rng.exponential(1.0 / load, size=nreq))
    results_p, wall_p = serve(arrivals)
    lat = np.array([r["latency_s"] for r in results_p])
    run_s = np.array([r["run_s"] for r in results_p])

    # work of the stream: unknowns x inner iterations summed over requests (a BiCGStab
    # iteration streams each unknown's vectors and matrix row a fixed number of times)
    inner = np.array([r["stats"]["inner_iterations"] for r in results], dtype=float)
    unk_it = float(np.sum(np.array([a * b * c * G for a, b, c, G in specs], dtype=float) * inner))
    dk = max(abs(results[k]["keff"] - k64[k]) for k in range(sample))
    # where the time goes, by request size (quartiles of unknowns over the FP64 sample)
    unk = np.array([a * b * c * G for a, b, c, G in specs], dtype=float)
    edges = np.quantile(unk[:sample], [0.25, 0.5, 0.75])
    by_size = []
    for q in range(4):
        lo = edges[q - 1] if q > 0 else -1.0
        hi = edges[q] if q < 3 else np.inf
        ks = [k for k in range(sample) if lo < unk[k] <= hi]
        if not ks:
            continue
        by_size.append(dict(requests=len(ks), mean_unknowns=float(np.mean(unk[ks])),
                            mean_inner_iterations=float(np.mean(inner[ks])),
                            fp64_alone_mean_ms=1e3 * float(np.mean([run64[k] for k in ks])),
                            fp64_alone_share=float(np.sum([run64[k] for k in ks]) / np.sum(run64)),
                            mixed_alone_mean_ms=1e3 * float(np.mean([run32[k] for k in ks])),
                            served_run_mean_ms=1e3 * float(np.mean([results[k]["run_s"] for k in ks]))))
    dk_mix = max(abs(a["keff"] - b["keff"]) for a, b in zip(results, results_p))
    launches = sum(r["stats"]["launches"] for r in results)
    cells = np.array([a * b * c for a, b, c, _ in specs], dtype=float)
    unknowns = np.array([a * b * c * G for a, b, c, G in specs], dtype=float)
    value = reduce_over_ranks(value, dist, f"cuda:{dev}", "sum")
    pct = lambda a, q: 1e3 * float(np.percentile(a, q))  # noqa: E731
    line = dict(metric="k-eigen solves/s (served, continuous batching)", value=value, unit="solves/s",
                n_gpus=world, steps=nreq, warmup=1, ms_per_step=1e3 * wall / nreq, higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="f32+f64", data="synthetic (seeded request generator)",
                config=dict(workload="serve_diffusion", description=WORKLOADS["serve_diffusion"]["desc"],
                            requests=nreq, slots=args.slots, sm_share=args.sm_share or "server default",
                            mean_cells=float(cells.mean()),
                            mean_unknowns=float(unknowns.mean()),
                            capacity_pass="all requests submitted at once; value = requests / time to last answer",
                            mean_outer_iterations=float(np.mean([r["stats"]["outer_iterations"] for r in results])),
                            mean_inner_iterations=float(np.mean([r["stats"]["inner_iterations"] for r in results])),
                            unknown_iterations=unk_it, unknown_iterations_per_s=unk_it / wall,
                            l2="requests are independent problems; no flush", parallelism="1 GPU"),
                latency=dict(arrivals="Poisson at 80% of the measured capacity", rate=load,
                             achieved_rate=nreq / wall_p, p50_ms=pct(lat, 50), p99_ms=pct(lat, 99),
                             mean_ms=1e3 * float(lat.mean()), run_p50_ms=pct(run_s, 50), run_p99_ms=pct(run_s, 99)),
                latency_saturated=dict(p50_ms=pct(lat_sat, 50), p99_ms=pct(lat_sat, 99),
                                       note="capacity pass: every request queued at t = 0"),
                fp64_one_at_a_time=dict(value=rate64, unit="solves/s", sample=sample,
                                        note="plain FP64 path, one request at a time, on the first `sample` "
                                             "requests of the same stream"),
                mixed_one_at_a_time=dict(value=rate32, unit="solves/s", sample=sample,
                                         note="the served precision, one request at a time (no batching)"),
                speedup_vs_fp64_one_at_a_time=value / rate64, by_size=by_size,
                capacity_pass_mean_in_flight=float(sum(r["run_s"] for r in results) / wall),
                dk_max_vs_fp64=dk, dk_max_between_passes=dk_mix,
                e2e=dict(value=value, unit="solves/s",
                         h2d_bytes_per_step=int(float(np.mean(unknowns * 56 + cells * 36))),
                         d2h_bytes_per_step=8,
                         note="the served rate is end to end: host operator arrays in, keff out"),
                gpu_launches=int(launches), roofline=None, clocks=clk.summary())
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline and parity leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision object of the default line")
    ap.add_argument("--no-serve", action="store_true", help="skip the served object of the default line")
    ap.add_argument("--size", default=None,
                    help="profiling captures only: NXxNYxNZ box (hexagonal workload: NQxNRxNZ lattice) instead "
                         "of the workload's (the line is then not the workload's result)")
    ap.add_argument("--requests", type=int, default=256,
                    help="serve_diffusion: requests in the stream (built up front: about 19 MB of host memory each)")
    ap.add_argument("--slots", type=int, default=16, help="serve_diffusion: solves in flight at most")
    ap.add_argument("--shift", type=float, default=None,
                    help="relative Wielandt shift of every solve (default: the workload's, else the solver's)")
    ap.add_argument("--sm-share", type=int, default=None,
                    help="serve_diffusion: SMs each served solve sizes its grids for (default: the server's)")
    ap.add_argument("--serve-sample", type=int, default=0,
                    help="serve_diffusion: requests (first of the stream) solved one at a time in FP64 for "
                         "the reference rate; 0: all of them")
    ap.add_argument("--profile-outer", type=int, default=0,
                    help="profiling runs under ncu only: cap every solve at this many outer iterations, "
                         "skip the e2e and CPU legs; the printed line is not a benchmark result")
    args = ap.parse_args()
    if args.warmup < 3 and not args.profile_outer:
        args.warmup = 3  # a benchmark result needs at least 3 warm-up solves
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import pampa_gb300.build as b
    b.build()
    if WORKLOADS[args.workload]["kind"] == "serve":
        return run_serve(args, rank, world, local)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
