"""Benchmark of the GB300 CD hot path (one JSON line on rank 0).

Workload (the precision configuration of the reference's CD3D path): CD3D on
the unit cube, 32^3 hexahedra, Q2 (274,625 DOFs), eps=1e-3,
b=(1,1,1)/sqrt(3), c=0, SUPG with delta = h/(2|b|) (SDFEM_TYPE 5, h = edge
length), manufactured u = x y z (1-x)(1-y)(1-z) exp(x), 3x3x3 Gauss
quadrature.  One step = ConvectionDiffusion::assemble (all 4 multigrid
levels) + Solver::solve: FGMRES(30) in FP64 preconditioned by a 4-level
geometric multigrid V(2,2) with damped Jacobi (omega=0.8) in FP32 and an FP64
dense coarse solve, to a relative residual of 1e-10.  The all-FP64 run of the
same solve is measured beside it.  Synthetic data only (generated mesh and
manufactured solution; no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload cd3d_q2_32|tcd3d_p2_48|cd2d_q1_64|cd3d_q2_96]

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, per-quadrature-point assembly with row-search scatter, FP64
multigrid) on all host cores, one solve per core per step.

Other workloads (--workload), each printing its own JSON line:
  tcd3d_p2_48  time-dependent CD3D on 48^3 cubes x 6 tetrahedra (Kuhn), finest
               interior vertices perturbed by U(+-0.2h) (seed 2024), P2
               (912,673 DOFs), eps=1e-4, b=(-(y-1/2), x-1/2, 0.2), Gaussian bump
               sigma=0.1 at (0.3,0.5,0.5), Crank-Nicolson dt=1e-3; one step =
               reassembly of stiffness and rhs on all 4 levels + CN rhs and
               system + FGMRES(30) with FP32 MG V(2,2) (omega 0.45, 5 levels, coarse
               3^3x6) warm-started to 1e-10.
  cd2d_q1_64   stationary CD2D, 64x64 Q1 (4,225 DOFs), eps=1e-2, b=(1,0.5), c=1,
               u=sin(pi x)sin(pi y), Galerkin, 3x3 Gauss, FP64 FGMRES(50)+Jacobi
               to 1e-10.
  cd3d_q2_96   stationary CD3D, 96^3 Q2 hexahedra (7,189,057 DOFs), eps=1e-6,
               SUPG, b=(1,0.25,0.1), u=sin(2 pi x)sin(2 pi y)sin(2 pi z), 6-level
               FP32 MG V(3,3) (damped Jacobi omega 0.5) inside FP64 FGMRES(30)
               to 1e-10.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CD solves/s, p50/p99 latency, mixed vs FP64 GPU at 1e-10 res; assembly GDOF/s"

# stationary workloads: mesh, problem data, solver (the reference's database keys)
STATIONARY = {
    "cd3d_q2_32": dict(
        workload="CD3D 32^3 Q2 SUPG eps=1e-3 b=(1,1,1)/sqrt3 c=0, FGMRES(30)+MG V(2,2) 4 levels "
                 "to 1e-10",
        dim=3, order=2, roots=1, nref=5, levels=4, example="POLYEXP", freq=1.0, eps=1e-3,
        b=(1 / np.sqrt(3.0),) * 3, c=0.0, supg=True, sdfem_type=5, delta0=1.0, cell_measure=2,
        problem_linear=1, quadrature="3x3x3 Gauss", sdfem="type 5, delta=h/(2|b|), h=edge length",
        precond="multigrid", restart=30, n_pre=2, n_post=2, damp=0.8, precisions=("mixed", "fp64"),
        cpu_sample=None, profile_tag="k_sell_f64_cd3d_q2_32"),
    "cd2d_q1_64": dict(
        workload="CD2D 64^2 Q1 Galerkin eps=1e-2 b=(1,.5) c=1 u=sin(pi x)sin(pi y), "
                 "FGMRES(50)+Jacobi FP64 to 1e-10",
        dim=2, order=1, roots=1, nref=6, levels=1, example="SINE", freq=1.0, eps=1e-2,
        b=(1.0, 0.5), c=1.0, supg=False, sdfem_type=2, delta0=1.0, cell_measure=0,
        problem_linear=0, quadrature="Gauss rule of degree 3 (reference map)", sdfem="none",
        precond="jacobi", restart=50, n_pre=0, n_post=0, damp=1.0, precisions=("fp64",),
        cpu_sample=None, profile_tag="k_spmv_f64_cd2d_q1_64"),
    "cd3d_q2_96": dict(
        workload="CD3D 96^3 Q2 SUPG eps=1e-6 b=(1,.25,.1) c=0 u=sin(2pi x)sin(2pi y)sin(2pi z), "
                 "FGMRES(30)+MG V(3,3) omega .5 6 levels to 1e-10",
        dim=3, order=2, roots=3, nref=5, levels=6, example="SINE", freq=2.0, eps=1e-6,
        b=(1.0, 0.25, 0.1), c=0.0, supg=True, sdfem_type=5, delta0=1.0, cell_measure=2,
        problem_linear=1, quadrature="3x3x3 Gauss", sdfem="type 5, delta=h/(2|b|), h=edge length",
        # omega 0.5: with 0.8 the Jacobi smoother amplifies high modes of this
        # convection-dominated Q2 SUPG operator and FGMRES stagnates
        precond="multigrid", restart=30, n_pre=3, n_post=3, damp=0.5, precisions=("mixed", "fp64"),
        cpu_sample=dict(roots=3, nref=3, levels=4), profile_tag="k_sell_f64_cd3d_q2_96"),
}


def spec_assembly(pg, w):
    return pg.assembly_params(
        example=getattr(pg, "EX_" + w["example"]), eps=w["eps"], b=w["b"], c=w["c"],
        freq=w["freq"], space_discretization_type="supg" if w["supg"] else "galerkin",
        sdfem_type=w["sdfem_type"], delta0=w["delta0"], cell_measure=w["cell_measure"],
        problem_linear=w["problem_linear"])


def spec_solver(pg, w, precision, levels=None):
    return pg.solver_params(
        w["precond"], precision=precision, max_n_iterations=5000, gmres_restart=w["restart"],
        residual_tolerance=0.0, residual_reduction=1e-10,
        multigrid_n_levels=levels or w["levels"], multigrid_cycle_type="V",
        multigrid_n_pre_smooth=w["n_pre"], multigrid_n_post_smooth=w["n_post"],
        jacobi_damp=w["damp"], multigrid_correction_damp_factor=1.0,
        multigrid_smoother_coarse="direct_solve")


# ---------------------------------------------------------------------------
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc, self.lines = gpu, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(kernel_tag):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.md line 'traffic_bytes_per_launch <tag> <bytes>')."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith((".md", ".txt")):
            continue
        for ln in open(os.path.join(pdir, fn)):
            f = ln.split()
            if len(f) >= 3 and f[0] == "traffic_bytes_per_launch" and f[1] == kernel_tag:
                try:
                    return float(f[2])
                except ValueError:
                    pass
    return None


# ---------------------------------------------------------------------------
EXTRA = {"on": False}   # a short record run embedded in the headline line


def timed_hierarchies(pg, ctx, args, kw, levels):
    """The hierarchy built on the host and on the GPU (DOF numbering and CSR
    patterns of every level), both timed; the GPU-built one is checked
    bit-exact against the host one and used for the run."""
    if EXTRA["on"]:
        t0 = time.perf_counter()
        dev = pg.Hierarchy(*args, ctx=ctx, **kw)
        return dev, {"hierarchy_device_s": time.perf_counter() - t0,
                     "bit_exact": "not checked in the embedded record run"}
    t0 = time.perf_counter()
    host = pg.Hierarchy(*args, **kw)
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    dev = pg.Hierarchy(*args, ctx=ctx, **kw)
    t_dev = time.perf_counter() - t0
    same = True
    for lvl in range(levels):
        ra, ca = host.pattern(lvl)
        rb, cb = dev.pattern(lvl)
        same = same and host.info(lvl) == dev.info(lvl) and np.array_equal(
            host.dofs(lvl), dev.dofs(lvl)) and np.array_equal(ra, rb) and np.array_equal(ca, cb)
    if not same:
        raise RuntimeError("GPU-built hierarchy differs from the host one")
    return dev, {"hierarchy_host_s": t_host, "hierarchy_device_s": t_dev, "bit_exact": same}


def run_gpu(args):
    import torch
    import parmoon2022_gb300 as pg
    w = STATIONARY[args.workload]
    rank, world, local = dist_env()
    dist = init_dist(world)
    torch.cuda.set_device(local)
    ctx = pg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    LEVELS = w["levels"]
    hkw = dict(n_levels=LEVELS, roots=w["roots"])
    hier, setup = timed_hierarchies(pg, ctx, (w["dim"], w["order"], w["nref"]), hkw, LEVELS)
    t0 = time.perf_counter()
    cd = pg.ConvectionDiffusion(ctx, hier)
    setup["problem_create_s"] = time.perf_counter() - t0
    a = spec_assembly(pg, w)
    precs = w["precisions"]
    cd64 = cd
    if precs[0] == "mixed":
        # the mixed solve's intermediate multigrid levels are FP32-only:
        # assembled on the tensor cores; the FP64 side runs on its own problem
        cd.set_fp32_tensor_levels(True)
        cd64 = pg.ConvectionDiffusion(ctx, hier)
    s_main = spec_solver(pg, w, precs[0])
    s_fp64 = spec_solver(pg, w, "fp64")
    info = [cd.info(l) for l in range(LEVELS)]
    n = info[0]["ndof"]

    def step(s, prob=None):
        prob = prob or cd
        prob.set_solution(None)   # start iterate 0 on the device (assemble sets Dirichlet values)
        prob.assemble(a)
        return prob.solve(s)

    def timed(s, k, w_, prob=None):
        for _ in range(w_):
            step(s, prob)
        barrier(dist)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        l0 = ctx.launches()
        stats = []
        for i in range(k):
            ev[i][0].record(stream)
            stats.append(step(s, prob))
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        barrier(dist)
        return [e0.elapsed_time(e1) for e0, e1 in ev], stats, ctx.launches() - l0

    cd.set_solution(np.zeros(n))
    if args.profile:
        # one step between cudaProfilerStart/Stop (ncu --profile-from-start off)
        for _ in range(2):
            step(s_main)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        l0 = ctx.launches()
        st = step(s_main)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_step": True, "launches": ctx.launches() - l0,
                          "iterations": st.iterations}))
        return
    # headline: inputs resident in HBM
    clocks = ClockSampler(local)
    clocks.start()
    per_m, st_m, launches = timed(s_main, args.steps, args.warmup)
    clk = clocks.stop()
    err_m = cd.errors(a)
    x_m = cd.solution()
    fp64_side = len(precs) > 1
    if fp64_side:
        # side by side: all-FP64 GPU solve of the same problem
        per_d, st_d, _ = timed(s_fp64, max(2, min(args.steps, 5)), 1, cd64)
        err_d = cd64.errors(a)
        x_d = cd64.solution()
    # assembly only (all levels, FP64)
    for _ in range(2):
        cd.assemble(a)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ka = max(3, args.steps)
    e0.record(stream)
    for _ in range(ka):
        cd.assemble(a)
    e1.record(stream)
    torch.cuda.synchronize()
    t_asm = e0.elapsed_time(e1) / ka / 1e3
    dofs_all = sum(i["ndof"] for i in info)
    # e2e: the reference-facing call with host buffers (pinned), copies inside
    sol_in = torch.zeros(n, dtype=torch.float64).pin_memory()
    sol_out = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    nul = dp()

    def e2e_step():
        st = pg.SolveStats()
        pg._chk(pg.lib().cdg_problem_assemble_solve(
            cd.p, ctypes.byref(a), ctypes.byref(s_main),
            ctypes.cast(sol_in.data_ptr(), dp), nul, ctypes.cast(sol_out.data_ptr(), dp),
            ctypes.byref(st)))
        return st
    for _ in range(args.warmup):
        e2e_step()
    barrier(dist)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(dist, (time.perf_counter() - te) / args.steps)
    # dominant kernel: the FP32 Jacobi smoothing SpMV of the finest level (MG),
    # the FP64 operator SpMV (Jacobi-preconditioned FGMRES)
    ms_smooth = cd.time_kernel(0, a, level=0, reps=50)
    ms_spmv64 = cd.time_kernel(1, a, level=0, reps=50)
    ms_contract = cd.time_kernel(2, a, level=0, reps=5)
    nnz0 = info[0]["nnz"]
    # the smoother reads the entries of the active rows only (Dirichlet rows
    # are identity rows): val + col of those, row_ptr, x, b, invd, y
    nnz_act0 = int(hier.pattern(0)[0][info[0]["nactive"]])
    bytes_smooth = 8 * nnz_act0 + 4 * (n + 1) + 4 * 4 * n
    bytes_spmv64 = 12 * nnz0 + 4 * (n + 1) + 8 * 2 * n
    peak, peak_kind = measured_peak_hbm()
    mg = w["precond"] == "multigrid"
    lay = cd.operator_layout(0)
    # roofline kernel: the FP64 operator w = A z of the finest level, the one
    # kernel on the path that streams an assembled matrix from HBM every
    # FGMRES iteration (sliced ELLPACK copy where the level has one)
    rl_kernel = ("k_sell<double,%d,8,0> (FP64 operator, finest level, sliced ELLPACK)"
                 % lay["lanes"]) if lay["lanes"] else \
        "k_spmv<double,...,0> (FP64 operator, finest level, CSR)"
    achieved = bytes_spmv64 / (ms_spmv64 * 1e-3) / 1e9
    rl_bytes = bytes_spmv64
    traffic = profile_traffic(w["profile_tag"])
    smoother, tuning = None, None
    if mg:
        # the FP32 smoothing step of every multigrid level as the tuner chose
        # it (CSR or matrix-free), with the tuner's timings of both kernels
        tuning = []
        for l in range(LEVELS - 1):
            c, (t_csr, t_mf), (lanes, cap) = cd.tuning_detail(l)
            tuning.append({"level": l, "dofs": info[l]["ndof"],
                           "kernel": {-2: "not tuned", -1: "csr (no matrix-free operator)",
                                      0: "csr", 1: "matrix-free"}[c],
                           "csr_lanes_per_row": lanes,
                           "matrix_free_blocks_per_sm": cap if c == 1 else None,
                           "ms_csr": t_csr, "ms_matrix_free": t_mf})
        if cd.tuning(0)[0] == 1:
            nc0 = info[0]["ncells"]
            if cd.tuning_detail(0)[2][1] <= -100:
                # stencil sweep: lattice map, x, b, D^-1, x' (the halo's
                # re-reads of map and x hit L2); the eight stencils are 3 KB
                zt = -100 - cd.tuning_detail(0)[2][1]
                mf_bytes = 4 * n + 4 * 4 * n
                mf_kernel = ("k_mf_stencil<2,%d> (lattice stencil Jacobi step, finest level, "
                             "eight 125-point stencils from one element matrix)" % zt)
            elif cd.tuning_detail(0)[2][1] < 0:
                # one launch: gdof_c + entry slots, row ranges, x, b, D^-1, x'
                # (the cells recomputed by neighbouring tiles hit L2)
                mf_bytes = 2 * 27 * nc0 * 4 + 4 * (info[0]["nactive"] + 1) + 4 * 4 * n
                mf_kernel = ("k_mf_fused<2,%d> (one-launch matrix-free Jacobi step, finest "
                             "level, one element matrix, 256-row tiles)"
                             % -cd.tuning_detail(0)[2][1])
            else:
                # gdof_c + pos_c + results (written, read), row ranges, x, b, D^-1, x'
                mf_bytes = 4 * 27 * nc0 * 4 + 4 * (info[0]["nactive"] + 1) + 4 * 4 * n
                mf_kernel = ("k_mf_uniform + k_mf_gather<2> (matrix-free Jacobi step, "
                             "finest level, one element matrix)")
            smoother = {"kernel": mf_kernel,
                        "bound": "latency (dependent L2 gathers); neither FP32 issue nor HBM",
                        "ms": ms_smooth, "bytes": mf_bytes,
                        "achieved_gbs": mf_bytes / (ms_smooth * 1e-3) / 1e9,
                        # multiply-adds formed: 729 per cell (tiles), or
                        # 25 (dx, dy) x 3 or 5 dz per lattice point (stencil)
                        "fp32_gflop": (2 * 100 * info[0]["nactive"] if "stencil" in mf_kernel
                                       else 2 * 729 * nc0) / 1e9,
                        "csr_step_ms": cd.tuning(0)[1][0], "csr_bytes": bytes_smooth}
        else:
            smoother = {"kernel": "k_spmv<float,8,8,2> (CSR Jacobi step, finest level)",
                        "bound": "hbm", "ms": ms_smooth, "bytes": bytes_smooth,
                        "achieved_gbs": bytes_smooth / (ms_smooth * 1e-3) / 1e9,
                        "frac": bytes_smooth / (ms_smooth * 1e-3) / 1e9 / peak}

    t_step_m = max_over_ranks(dist, sum(per_m) / len(per_m) / 1e3)
    if fp64_side:
        t_step_d = max_over_ranks(dist, sum(per_d) / len(per_d) / 1e3)
    value = world / t_step_m
    if rank != 0:
        return
    cpu = cpu_baseline_sample(args.workload) if not args.skip_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step_m * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 FGMRES + f32 multigrid (mixed)" if precs[0] == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": w["workload"], "dofs": n, "nnz": nnz0,
                   "levels_dofs": [i["ndof"] for i in info], "quadrature": w["quadrature"],
                   "sdfem": w["sdfem"],
                   "l2": ("working set > L2 (finest CSR alone %.0f MB); no flush"
                          % (nnz0 * 16 / 1e6)) if nnz0 * 16 > 129e6 else
                         "working set fits in L2 (%.1f MB); no flush, latency-bound"
                         % (nnz0 * 16 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "p50_ms": statistics.median(per_m), "p99_ms": float(np.percentile(per_m, 99)),
        "iterations": st_m[-1].iterations,
        "rel_residual": st_m[-1].residual / st_m[-1].initial_residual,
        "errors": {"L2": err_m[0], "H1_semi": err_m[1]},
        "assembly_gdofs": dofs_all / t_asm / 1e9,
        "assembly_ms": t_asm * 1e3,
        "kernels_ms": {"jacobi_smooth_f32_L0": ms_smooth, "spmv_f64_L0": ms_spmv64,
                       "element_contract_f64_L0": ms_contract},
        "smoother": smoother,
        "tuning": tuning,
        "roofline": {"bound": "hbm", "kernel": rl_kernel, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": rl_bytes, "traffic": traffic},
        "cpu_baseline": cpu,
        "e2e": {"value": world / t_e2e, "unit": "solves/s",
                "h2d_bytes_per_step": 8 * n + 2 * 136,
                "d2h_bytes_per_step": 8 * n + 8 * 4},
        "clocks": clk,
        "gpu_launches": launches,
        "setup": setup,
    }
    if fp64_side:
        rel = float(np.max(np.abs(x_m - x_d)) / np.max(np.abs(x_d)))
        line["errors"].update({"L2_fp64": err_d[0], "H1_semi_fp64": err_d[1],
                               "solution_rel_diff_vs_fp64": rel})
        line["fp64"] = {"value": world / t_step_d, "ms_per_step": t_step_d * 1e3,
                        "iterations": st_d[-1].iterations}
        line["mixed_over_fp64"] = t_step_d / t_step_m
    if args.workload == "cd3d_q2_32" and world == 1 and not EXTRA["on"] and not args.no_extra:
        line["extra_workloads"] = extra_workloads()
    print(json.dumps(line))


def extra_workloads():
    """The other workloads as short child runs of this script (3 timed steps,
    no CPU sample), each line embedded as reported; the headline numbers above
    are measured before any of them starts."""
    out = {}
    for wl, steps in (("cd2d_q1_64", 5), ("tcd3d_p2_48", 5), ("cd3d_q2_96", 3), ("serve", 0)):
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", wl, "--skip-cpu",
               "--extra"]
        if steps:
            cmd += ["--steps", str(steps), "--warmup", "3"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            rec = json.loads(lines[-1]) if r.returncode == 0 and lines else {
                "error": "rc %d: %s" % (r.returncode, r.stderr.strip().splitlines()[-1:])}
        except Exception as e:  # a failed record run must not lose the headline line
            rec = {"error": repr(e)}
        rec["wall_s"] = time.perf_counter() - t0
        out[wl] = rec
    return out


# ---------------------------------------------------------------------------
# time-dependent CD3D on perturbed P2 tetrahedra (Crank-Nicolson)
# ---------------------------------------------------------------------------
TCD = dict(roots=3, nref=4, levels=5, perturb=0.2, seed=2024, eps=1e-4, b=(0.5, -0.5, 0.2),
           b_grad=((0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
           ic=(0.3, 0.5, 0.5, 0.1), tau=1e-3)
TCD_WORKLOAD = ("TCD3D 48^3x6 P2 tetrahedra perturbed 0.2h, eps=1e-4, b=(-(y-.5),x-.5,.2), "
                "bump sigma .1 at (.3,.5,.5), CN dt=1e-3, FGMRES(30)+MG V(2,2) omega .45 5 levels "
                "to 1e-10")
TCD_METRIC = "TCD steps/s (reassembly + CN solve to 1e-10), mixed vs FP64; assembly GDOF/s"


def tcd_solver_kw(levels):
    # the Crank-Nicolson system tau/2 A + M is mass dominated; for P2
    # tetrahedra the Jacobi-scaled spectrum reaches ~4.2, so damped Jacobi
    # needs omega < 2/4.2: omega = 0.45 (0.8 amplifies the high modes)
    return dict(max_n_iterations=1000, gmres_restart=30, residual_tolerance=0.0,
                residual_reduction=1e-10, multigrid_n_levels=levels, multigrid_cycle_type="V",
                multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.45,
                multigrid_correction_damp_factor=1.0, multigrid_smoother_coarse="direct_solve")


def tcd_params(pg, t):
    return pg.assembly_params(example=pg.EX_BUMP, eps=TCD["eps"], b=TCD["b"],
                              b_grad=TCD["b_grad"], t=t, ic=TCD["ic"])


def run_gpu_tcd(args):
    import torch
    import parmoon2022_gb300 as pg
    rank, world, local = dist_env()
    dist = init_dist(world)
    torch.cuda.set_device(local)
    ctx = pg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    L = TCD["levels"] - (1 if args.small else 0)
    nref = TCD["nref"] - (1 if args.small else 0)
    hier, setup = timed_hierarchies(pg, ctx, (3, 2, nref),
                                    dict(n_levels=L, roots=TCD["roots"], tetra=True,
                                         perturb=TCD["perturb"], seed=TCD["seed"]), L)
    t0 = time.perf_counter()
    cd = pg.ConvectionDiffusion(ctx, hier)
    setup["problem_create_s"] = time.perf_counter() - t0
    info = [cd.info(l) for l in range(L)]
    n = info[0]["ndof"]
    tau = TCD["tau"]
    s_mixed = pg.solver_params("multigrid", precision="mixed", **tcd_solver_kw(L))
    s_fp64 = pg.solver_params("multigrid", precision="fp64", **tcd_solver_kw(L))

    def run(s, k, w):
        """initial condition, w untimed steps, k timed steps (event per step)"""
        cd.tcd_initialize(tcd_params(pg, 0.0))
        t = 0.0
        for _ in range(w):
            t += tau
            cd.tcd_step(tcd_params(pg, t), tau, s)
        barrier(dist)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        l0 = ctx.launches()
        stats = []
        for i in range(k):
            t += tau
            ev[i][0].record(stream)
            stats.append(cd.tcd_step(tcd_params(pg, t), tau, s))
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        barrier(dist)
        return [e0.elapsed_time(e1) for e0, e1 in ev], stats, ctx.launches() - l0, t

    if args.profile:
        # one mixed step between cudaProfilerStart/Stop (ncu --profile-from-start off)
        run(s_mixed, 1, 2)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        l0 = ctx.launches()
        st = cd.tcd_step(tcd_params(pg, 4 * tau), tau, s_mixed)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_step": True, "launches": ctx.launches() - l0,
                          "iterations": st.iterations}))
        return
    clocks = ClockSampler(local)
    clocks.start()
    per_m, st_m, launches, t_end = run(s_mixed, args.steps, args.warmup)
    clk = clocks.stop()
    x_m = cd.solution()
    per_d, st_d, _, _ = run(s_fp64, args.steps, args.warmup)
    x_d = cd.solution()
    # stationary assembly of the same stiffness and rhs on all levels (FP64)
    a_end = tcd_params(pg, t_end)
    for _ in range(2):
        cd.assemble(a_end)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ka = 10
    e0.record(stream)
    for _ in range(ka):
        cd.assemble(a_end)
    e1.record(stream)
    torch.cuda.synchronize()
    t_asm = e0.elapsed_time(e1) / ka / 1e3
    dofs_all = sum(i["ndof"] for i in info)
    # e2e: each step through the C-ABI with the solution read back to pinned host memory
    import ctypes
    sol_out = torch.empty(n, dtype=torch.float64).pin_memory()
    dp = ctypes.POINTER(ctypes.c_double)
    cd.tcd_initialize(tcd_params(pg, 0.0))
    t = 0.0
    ke = args.steps
    for i in range(args.warmup + ke):
        if i == args.warmup:
            torch.cuda.synchronize()
            te = time.perf_counter()
        t += tau
        a_t = tcd_params(pg, t)
        st = pg.SolveStats()
        pg._chk(pg.lib().cdg_problem_tcd_step(cd.p, ctypes.byref(a_t), tau, ctypes.byref(s_mixed),
                                             ctypes.byref(st)))
        pg._chk(pg.lib().cdg_problem_get_solution(cd.p, ctypes.cast(sol_out.data_ptr(), dp)))
    t_e2e = max_over_ranks(dist, (time.perf_counter() - te) / ke)
    # dominant kernels of a step
    ms_smooth = cd.time_kernel(0, a_end, level=0, reps=50)
    ms_spmv64 = cd.time_kernel(1, a_end, level=0, reps=50)
    ms_contract = cd.time_kernel(2, a_end, level=0, reps=5)
    nnz0 = info[0]["nnz"]
    nnz_act0 = int(hier.pattern(0)[0][info[0]["nactive"]])   # entries of active rows
    bytes_smooth = 8 * nnz_act0 + 4 * (n + 1) + 4 * 4 * n
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_smooth / (ms_smooth * 1e-3) / 1e9
    chunk = cd.operator_layout(0)["smoother_chunk"]
    rl_kernel = ("k_spmv_bulk<%d,4,2> (Jacobi smoothing, finest level, %d-entry chunks staged "
                 "by cp.async.bulk)" % (8192 // chunk, chunk)) if chunk else (
                 "k_spmv<float,4,8,2> (Jacobi smoothing, finest level)")
    traffic = profile_traffic("k_spmv_f32_jacobi_tcd3d_p2_48")
    t_step_m = max_over_ranks(dist, sum(per_m) / len(per_m) / 1e3)
    t_step_d = max_over_ranks(dist, sum(per_d) / len(per_d) / 1e3)
    if rank != 0:
        return
    cpu = cpu_baseline_tcd() if not args.skip_cpu else None
    rel = float(np.max(np.abs(x_m - x_d)) / np.max(np.abs(x_d)))
    its = [s.iterations for s in st_m]
    print(json.dumps({
        "metric": TCD_METRIC, "value": world / t_step_m, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step_m * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 FGMRES + f32 multigrid (mixed)", "data": "synthetic",
        "config": {"workload": TCD_WORKLOAD, "dofs": n, "nnz": nnz0,
                   "cells": info[0]["ncells"], "levels_dofs": [i["ndof"] for i in info],
                   "quadrature": "collapsed Gauss 5^3 (degree 6)",
                   "l2": "working set > L2 (finest stiffness+mass+system CSR %.0f MB); no flush"
                         % (nnz0 * 32 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "p50_ms": statistics.median(per_m), "p99_ms": float(np.percentile(per_m, 99)),
        "iterations_per_step": {"min": min(its), "max": max(its), "mean": sum(its) / len(its)},
        "rel_residual": st_m[-1].residual / max(st_m[-1].initial_residual, 1e-300),
        "solution_rel_diff_vs_fp64": rel,
        "fp64": {"value": world / t_step_d, "ms_per_step": t_step_d * 1e3,
                 "iterations_last": st_d[-1].iterations},
        "mixed_over_fp64": t_step_d / t_step_m,
        "assembly_gdofs": dofs_all / t_asm / 1e9, "assembly_ms": t_asm * 1e3,
        "kernels_ms": {"jacobi_smooth_f32_L0": ms_smooth, "spmv_f64_L0": ms_spmv64,
                       "element_contract_f64_L0": ms_contract},
        "roofline": {"bound": "hbm", "kernel": rl_kernel,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "algorithmic_bytes": bytes_smooth,
                     "traffic": traffic},
        "cpu_baseline": cpu,
        "e2e": {"value": world / t_e2e, "unit": "steps/s", "h2d_bytes_per_step": 136 + 136,
                "d2h_bytes_per_step": 8 * n + 8 * 4},
        "clocks": clk, "gpu_launches": launches, "setup": setup,
    }))


# ---------------------------------------------------------------------------
# served form: a Poisson stream of stationary solves of differing meshes and
# coefficients through the request server
# ---------------------------------------------------------------------------
SERVE = dict(classes=[(2, 1, n) for n in (16, 32, 64, 128, 256)] +
             [(2, 2, n) for n in (16, 32, 64, 128, 256)] +
             [(3, 1, n) for n in (8, 12, 16, 24, 32, 48)],
             rates=(10, 100, 500, 1000, 2000), seconds_per_rate=6.0, slots=8,
             seed=1234)
SERVE_WORKLOAD = ("served CD: Poisson arrivals (seeded), rate swept 10-2000 req/s; 2D Q1/Q2 "
                  "N in {16,32,64,128,256}, 3D Q1 N in {8,12,16,24,32,48}; eps log-U[1e-4,1], "
                  "b = unit direction x U[0,1], c = U[0,1], f = 1, SUPG (SDFEM_TYPE 2); FGMRES(30) "
                  "+ MG V(2,2) omega .5 to 1e-10")
SERVE_METRIC = "served CD solves/s with p50/p99 latency vs one-at-a-time FP64"


def serve_stream(count, seed):
    """(dim, order, n, eps, b, c) of `count` requests, drawn as the served
    configuration asks: dimension 2 or 3 with equal probability, then the
    element order and N uniformly"""
    rng = np.random.default_rng(seed)
    c2 = [k for k in SERVE["classes"] if k[0] == 2]
    c3 = [k for k in SERVE["classes"] if k[0] == 3]
    out = []
    for _ in range(count):
        cls = c2[rng.integers(len(c2))] if rng.uniform() < 0.5 else c3[rng.integers(len(c3))]
        d = rng.standard_normal(cls[0])
        d /= np.linalg.norm(d)
        out.append((cls[0], cls[1], cls[2], float(10 ** rng.uniform(-4, 0)),
                    tuple(d * rng.uniform(0, 1)), float(rng.uniform(0, 1))))
    return out


def serve_request(pg, q, precision):
    # omega 0.5: with 0.8 the Jacobi smoother amplifies high modes when the
    # convection dominates and is nearly grid-aligned (a 2D Q1 32^2 request
    # with eps 1.4e-4, b ~ -x stalls; 0.5 converges in 48 iterations)
    dim, order, n, eps, b, c = q
    a = pg.assembly_params(example=pg.EX_CONST_F, eps=eps, b=b, c=c,
                           space_discretization_type="supg", sdfem_type=2)
    s = pg.solver_params("multigrid", max_n_iterations=500, gmres_restart=30,
                         residual_tolerance=0.0, residual_reduction=1e-10, multigrid_n_levels=0,
                         multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.5,
                         precision=precision)
    return pg.request(dim, order, n, a, s)


def run_stream(pg, srv, qs, arrivals, precision):
    """submit qs at the given arrival times (seconds); wait for all; returns
    (wall seconds, results)"""
    reqs = [serve_request(pg, q, precision) for q in qs]
    tickets = []
    t0 = time.perf_counter()
    for r, ta in zip(reqs, arrivals):
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(r))
    res = [srv.wait(t)[0] for t in tickets]
    return time.perf_counter() - t0, res


def run_gpu_serve(args):
    import torch
    import parmoon2022_gb300 as pg
    rank, world, local = dist_env()
    dist = init_dist(world)
    torch.cuda.set_device(local)
    if args.slots:
        SERVE["slots"] = args.slots
    srv = pg.Server(local, n_slots=SERVE["slots"])
    # warm the pools: one request of every mesh class (hierarchies, device
    # instances, captured graphs), not timed
    warm = [(d, o, n, 1e-2, (0.6, 0.8, 0.0)[:d], 0.5) for d, o, n in SERVE["classes"]]
    t_cold = time.perf_counter()
    run_stream(pg, srv, warm, [0.0] * len(warm), "mixed")
    t_cold = time.perf_counter() - t_cold
    c0 = srv.counters()
    clocks = ClockSampler(local)
    clocks.start()
    sweep = []
    rng = np.random.default_rng(SERVE["seed"])
    rates = (100, 500, 2000) if EXTRA["on"] else SERVE["rates"]
    secs = 1.5 if EXTRA["on"] else SERVE["seconds_per_rate"]
    for k, lam in enumerate(rates):
        # about seconds_per_rate of arrivals, at most 2500 requests per rate
        # (8,160 requests over the full sweep)
        cnt = int(min(2500, max(40, lam * secs)))
        qs = serve_stream(cnt, SERVE["seed"] + k)
        arrivals = np.cumsum(rng.exponential(1.0 / lam, cnt))
        wall, res = run_stream(pg, srv, qs, arrivals, "mixed")
        lat = np.array([r.latency_seconds for r in res]) * 1e3
        qt = np.array([r.queue_seconds for r in res]) * 1e3
        bad = sum(1 for r in res if r.status != 0 or
                  r.stats.residual > 1e-10 * r.stats.initial_residual * 1.0001)
        sweep.append({"rate": lam, "requests": cnt, "solves_per_s": cnt / wall,
                      "p50_ms": float(np.percentile(lat, 50)),
                      "p99_ms": float(np.percentile(lat, 99)),
                      "queue_p50_ms": float(np.percentile(qt, 50)),
                      "iterations_mean": float(np.mean([r.stats.iterations for r in res])),
                      "not_converged": bad})
    clk = clocks.stop()
    c1 = srv.counters()
    srv.close()
    # one-at-a-time FP64 (and mixed) on the same requests, back to back;
    # 600 requests (~1.7 s one at a time) so that the concurrent pass's
    # start and tail are a small part of it
    base_q = serve_stream(600, SERVE["seed"] + 99)
    # (each server first runs the same requests untimed, so its pool holds
    # the instances the timed pass needs: steady state, not setup)
    one = {}
    # (per-launch batching off: every request on the slot's stream)
    os.environ["CDG_SERVER_BATCH"] = "0"
    for prec in ("fp64", "mixed"):
        s1 = pg.Server(local, n_slots=1)
        run_stream(pg, s1, base_q, [0.0] * len(base_q), prec)
        wall, res = run_stream(pg, s1, base_q, [0.0] * len(base_q), prec)
        one[prec] = len(base_q) / wall
        s1.close()
    del os.environ["CDG_SERVER_BATCH"]
    # saturated concurrent throughput on the same requests
    s8 = pg.Server(local, n_slots=SERVE["slots"])
    run_stream(pg, s8, base_q, [0.0] * len(base_q), "mixed")
    wall, _ = run_stream(pg, s8, base_q, [0.0] * len(base_q), "mixed")
    sat = len(base_q) / wall
    s8.close()
    # the largest class's FP32 smoothing SpMV against the HBM roofline
    ctx = pg.Context(local)
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 2, 8, n_levels=7))
    a = serve_request(pg, (2, 2, 256, 1e-2, (0.6, 0.8), 0.5), "mixed").a
    cd.assemble(a)
    ms = cd.time_kernel(0, a, level=0, reps=50)
    i0 = cd.info(0)
    nnz_act = int(cd.hier.pattern(0)[0][i0["nactive"]])
    bytes_smooth = 8 * nnz_act + 4 * (i0["ndof"] + 1) + 16 * i0["ndof"]
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_smooth / (ms * 1e-3) / 1e9
    chunk = cd.operator_layout(0)["smoother_chunk"]
    tpr = {True: 8, False: 4}[i0["nnz"] / i0["ndof"] > 32]
    rl_kernel = ("k_spmv_bulk<%d,%d,2> (smoothing, 2D Q2 256^2, %d-entry chunks staged by "
                 "cp.async.bulk)" % (8192 // chunk, tpr, chunk)) if chunk else (
                 "k_spmv<float,%d,8,2> (smoothing, 2D Q2 256^2)" % tpr)
    cd.close()
    ctx.close()
    if rank != 0:
        return
    cpu = cpu_baseline_serve() if not args.skip_cpu else None
    # latency at the highest offered rate the server keeps up with (beyond
    # saturation the queue, not the solve, sets the latency)
    kept = [e for e in sweep if e["solves_per_s"] >= 0.9 * e["rate"]]
    top = kept[-1] if kept else sweep[0]
    ndof_mean = float(np.mean([(o * n + 1) ** d for d, o, n, *_ in base_q]))
    print(json.dumps({
        "metric": SERVE_METRIC, "value": sat, "unit": "solves/s", "n_gpus": world,
        "steps": len(base_q), "warmup": len(warm), "ms_per_step": 1e3 / sat,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 FGMRES + f32 multigrid (mixed)", "data": "synthetic",
        "config": {"workload": SERVE_WORKLOAD, "slots": SERVE["slots"],
                   "classes": len(SERVE["classes"]), "mean_dofs": ndof_mean,
                   "l2": "mixed sizes; no flush", "parallelism": "single GPU, %d streams" % SERVE["slots"]},
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "latency_at_rate": top["rate"],
        "sweep": sweep,
        "one_at_a_time": {"fp64_solves_per_s": one["fp64"], "mixed_solves_per_s": one["mixed"]},
        "served_over_one_at_a_time_fp64": sat / one["fp64"],
        "server": {k: c1[k] - c0.get(k, 0)
                   if k in ("completed", "launches", "evictions", "batch_launches", "batched")
                   else c1[k] for k in c1},
        "roofline": {"bound": "hbm", "kernel": rl_kernel,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "algorithmic_bytes": bytes_smooth, "traffic": None},
        "cpu_baseline": cpu,
        "e2e": {"value": sat, "unit": "solves/s", "h2d_bytes_per_step": 400,
                "d2h_bytes_per_step": int(8 * ndof_mean)},
        "clocks": clk, "gpu_launches": c1["launches"] - c0["launches"],
        "cold_start_s": t_cold,
    }))


def oracle_serve_solve(q):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    dim, order, n, eps, b, c = q
    roots = 3 if n % 3 == 0 else 1
    nref = int(round(np.log2(n // roots)))
    levels = nref + 1 if roots == 3 else max(1, nref - 1)
    kw = dict(eps=eps, b=b, c=c, supg=True, sdfem_type=2)
    if roots == 1:
        p = po.Problem(po.make_config(dim, order, nref, po.EX_CONST_F, **kw), levels)
    else:
        import parmoon2022_gb300 as pg
        h = pg.Hierarchy(dim, order, nref, n_levels=levels, roots=roots)
        arrays = []
        for l in range(levels):
            rp, col = h.pattern(l)
            i = h.info(l)
            arrays.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"],
                               nactive=i["nactive"], row_ptr=rp, col=col))
        p = po.Problem(po.make_config(dim, order, 0, po.EX_CONST_F, **kw), arrays=arrays)
    t0 = time.perf_counter()
    p.assemble()
    p.solve(po.make_solver("multigrid", max_it=500, restart=30, reduction=1e-10, mg_levels=levels,
                           n_pre=2, n_post=2, jacobi_damp=0.5))
    return time.perf_counter() - t0


def cpu_baseline_serve(budget_s=20.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    qs = serve_stream(400, SERVE["seed"] + 99)
    t, k = 0.0, 0
    for q in qs:
        t += oracle_serve_solve(q)
        k += 1
        if t > budget_s:
            break
    return {"value": k / t, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": "the first %d requests of the one-at-a-time stream solved back to back "
                      "(%.1f s) by the C restatement of the reference, 1 thread" % (k, t)}


def _worker_serve(q, idx, stride, budget_s):
    qs = serve_stream(4000, SERVE["seed"] + 99)
    t, k = 0.0, 0
    for qq in qs[idx::stride]:
        t += oracle_serve_solve(qq)
        k += 1
        if t > budget_s:
            break
    q.put((k, t))


def oracle_tcd_step_time(roots, nref, levels):
    """Seconds of one Crank-Nicolson step (reassembly + FP64 MG solve) by the
    CPU oracle on a roots*2^nref tetrahedral mesh of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    import parmoon2022_gb300 as pg
    h = pg.Hierarchy(3, 2, nref, n_levels=levels, roots=roots, tetra=True,
                     perturb=TCD["perturb"], seed=TCD["seed"])
    arrays = []
    for l in range(levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        arrays.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"],
                           nactive=i["nactive"], row_ptr=rp, col=col))
    cfg = po.make_config(3, 2, 0, po.EX_BUMP, eps=TCD["eps"], b=TCD["b"], b_grad=TCD["b_grad"],
                         ic=TCD["ic"], tetra=True)
    p = po.Problem(cfg, arrays=arrays)
    p.tcd_initialize()
    s = po.make_solver("multigrid", max_it=1000, restart=30, reduction=1e-10, mg_levels=levels,
                       n_pre=2, n_post=2, jacobi_damp=0.45)
    t0 = time.perf_counter()
    it, _, _ = p.tcd_step(TCD["tau"], TCD["tau"], s)
    return time.perf_counter() - t0, it, h.info(0)["ndof"]


def cpu_baseline_tcd():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    dt, it, nd = oracle_tcd_step_time(3, 3, 4)
    scale = 912673 / nd
    return {"value": 1.0 / (dt * scale), "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": "one CN step (reassembly + FP64 MG solve, %d its) of the same workload on "
                      "24^3x6 tetrahedra (%d DOFs, %.1f s), scaled by DOFs x%.2f to 912,673 DOFs; "
                      "C restatement of the reference, 1 thread" % (it, nd, dt, scale)}


# ---------------------------------------------------------------------------
def oracle_solve_once(name, sample=None):
    """One assemble + solve of a stationary workload by the CPU oracle
    (reference algorithm); sample: smaller mesh (roots, nref, levels)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    w = STATIONARY[name]
    roots, nref, levels = (w["roots"], w["nref"], w["levels"]) if sample is None else (
        sample["roots"], sample["nref"], sample["levels"])
    kw = dict(eps=w["eps"], b=w["b"], c=w["c"], freq=w["freq"], supg=w["supg"],
              sdfem_type=w["sdfem_type"], delta0=w["delta0"], cell_measure=w["cell_measure"],
              problem_linear=w["problem_linear"])
    ex = getattr(po, "EX_" + w["example"])
    if roots == 1:
        cfg = po.make_config(w["dim"], w["order"], nref, ex, **kw)
        p = po.Problem(cfg, levels)
    else:
        import parmoon2022_gb300 as pg
        h = pg.Hierarchy(w["dim"], w["order"], nref, n_levels=levels, roots=roots)
        arrays = []
        for l in range(levels):
            rp, col = h.pattern(l)
            i = h.info(l)
            arrays.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"],
                               nactive=i["nactive"], row_ptr=rp, col=col))
        cfg = po.make_config(w["dim"], w["order"], 0, ex, **kw)
        p = po.Problem(cfg, arrays=arrays)
    ndof = p.info(0)["ndof"]
    t0 = time.perf_counter()
    p.assemble()
    t1 = time.perf_counter()
    it, res, ini = p.solve(po.make_solver(w["precond"], max_it=5000, restart=w["restart"],
                                          tol_abs=0.0, reduction=1e-10, mg_levels=levels,
                                          mg_cycle="V", n_pre=w["n_pre"], n_post=w["n_post"],
                                          jacobi_damp=w["damp"], correction_damp=1.0,
                                          coarse_direct=True))
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, it, ndof


def full_ndof(name):
    w = STATIONARY[name]
    n1 = w["roots"] * 2 ** w["nref"] * w["order"] + 1
    return n1 ** w["dim"]


def cpu_baseline_sample(name):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    w = STATIONARY[name]
    t, t_asm, it, nd = oracle_solve_once(name, w["cpu_sample"])
    scale = full_ndof(name) / nd
    if w["cpu_sample"] is None:
        sample = ("one full solve (assemble %d levels %.1f s + FGMRES %d its) of the same "
                  "workload by the C restatement of the reference, 1 thread" % (w["levels"], t_asm, it))
    else:
        sample = ("one solve (assemble + FGMRES %d its, %.1f s) of the same problem on %d DOFs, "
                  "scaled by DOFs x%.1f to the full size; C restatement of the reference, 1 thread"
                  % (it, t, nd, scale))
    return {"value": 1.0 / (t * scale), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": sample}


def _worker(q, name):
    w = STATIONARY[name]
    t, _, _, nd = oracle_solve_once(name, w["cpu_sample"])
    q.put(t * full_ndof(name) / nd)


def _worker_tcd(q):
    dt, it, nd = oracle_tcd_step_time(3, 3, 4)
    q.put(dt * 912673 / nd)


BATCH_CLASSES = [(2, 1, 4, 3), (2, 2, 4, 3), (3, 1, 3, 2)]   # (dim, order, nref, levels)
BATCH_METRIC = "batched small CD solves/s (one block per request, one launch)"


def run_gpu_batch(args):
    """Many small stationary solves in one launch (cdg_solve_batched) against
    the same problems solved one at a time by the stream-level solver.  A
    step is one launch over K = 2 x SMs requests of one class (host
    preparation of the K problems included, assembly not); the headline class
    is 2D Q1 16^2 (289 DOFs), the served mix's smallest."""
    import torch
    import parmoon2022_gb300 as pg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    ctx = pg.Context(local)
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    K = 2 * nsm
    rng = np.random.default_rng(17)
    records = []
    for dim, order, nref, levels in BATCH_CLASSES:
        h = pg.Hierarchy(dim, order, nref, n_levels=levels)
        probs, params_ = [], []
        for q in range(K):
            d = rng.standard_normal(dim)
            d /= np.linalg.norm(d)
            a = pg.assembly_params(example=pg.EX_CONST_F, eps=float(10 ** rng.uniform(-2, 0)),
                                   b=tuple(d * rng.uniform(0, 1)), c=float(rng.uniform(0, 1)),
                                   space_discretization_type="supg", sdfem_type=2)
            cd = pg.ConvectionDiffusion(ctx, h)
            cd.assemble(a)
            probs.append(cd)
            params_.append(pg.solver_params(
                "multigrid", precision="mixed", max_n_iterations=500, gmres_restart=30,
                residual_tolerance=0.0, residual_reduction=1e-10, multigrid_n_levels=levels,
                multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.5))
        x0 = [p.solution() for p in probs]
        walls, its, launches = [], [], []
        for step in range(args.warmup + args.steps):
            for p, x in zip(probs, x0):
                p.set_solution(x)
            ctx.synchronize()
            l0 = ctx.launches()
            t0 = time.perf_counter()
            out = pg.solve_batched(ctx, probs, params_)
            t = time.perf_counter() - t0
            launches.append(ctx.launches() - l0)
            assert all(s == 0 and st.residual <= 1e-10 * st.initial_residual for s, st in out)
            if step >= args.warmup:
                walls.append(t)
                its.append(float(np.mean([st.iterations for _, st in out])))
        # the same problems one at a time (stream-level solver), 32 of them
        t_one = []
        for p, x, sp in list(zip(probs, x0, params_))[:32]:
            p.set_solution(x)
            ctx.synchronize()
            t0 = time.perf_counter()
            p.solve(sp)
            t_one.append(time.perf_counter() - t0)
        wall = float(np.median(walls))
        records.append({"class": "%dD Q%d %d^%d" % (dim, order, 2 ** nref, dim),
                        "dofs": probs[0].info(0)["ndof"], "requests_per_launch": K,
                        "launch_ms": wall * 1e3, "solves_per_s": K / wall,
                        "one_at_a_time_solves_per_s": 1.0 / float(np.mean(t_one)),
                        "iterations_mean": float(np.mean(its)),
                        "launches_per_step": int(launches[-1])})
        for p in probs:
            p.close()
    if rank != 0:
        return
    head = records[0]
    print(json.dumps({
        "metric": BATCH_METRIC, "value": head["solves_per_s"], "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["launch_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 FGMRES + f32 multigrid (mixed)", "data": "synthetic",
        "config": {"workload": "batched: K = 2 x SMs small SUPG CD requests per launch, "
                               "f = 1, eps log-U[1e-2,1], random b, c; FGMRES(30) + MG "
                               "V(2,2) omega .5 to 1e-10", "l2": "small problems; no flush"},
        "classes": records,
        "batched_over_one_at_a_time": head["solves_per_s"] / head["one_at_a_time_solves_per_s"],
        "gpu_launches": head["launches_per_step"] * args.steps}))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "batch":
        print(json.dumps({"impl": "reference", "unavailable": "the reference solves one "
                          "problem per call; see --workload serve for its one-at-a-time rate"}))
        return
    tcd = args.workload == "tcd3d_p2_48"
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import multiprocessing as mp
    import pyoracle as po
    po.build()
    cores = os.cpu_count() or 1
    ctxm = mp.get_context("spawn")
    if args.workload == "serve":
        # every core serves its share of the request stream for ~20 s
        q = ctxm.Queue()
        procs = [ctxm.Process(target=_worker_serve, args=(q, i, cores, 20.0))
                 for i in range(cores)]
        for pr in procs:
            pr.start()
        for pr in procs:
            pr.join()
        got = [q.get() for _ in range(cores)]
        solves = sum(k for k, _ in got)
        wall = max(t for _, t in got)
        value = solves / wall
        print(json.dumps({
            "metric": SERVE_METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": solves, "warmup": 0, "ms_per_step": 1e3 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "config": {"workload": SERVE_WORKLOAD},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": "%d host processes, each solving its share of the request "
                                       "stream back to back for ~20 s; C restatement of the "
                                       "reference" % cores},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }))
        return
    # each step: every core solves one instance; bounded to keep the run short
    steps = max(1, min(args.steps, 3))
    warm = 1 if args.warmup > 0 else 0
    times = []
    for i in range(warm + steps):
        q = ctxm.Queue()
        procs = [ctxm.Process(target=_worker_tcd, args=(q,)) if tcd else
                 ctxm.Process(target=_worker, args=(q, args.workload)) for _ in range(cores)]
        t0 = time.perf_counter()
        for pr in procs:
            pr.start()
        for pr in procs:
            pr.join()
        dt = time.perf_counter() - t0
        if i >= warm:
            times.append(max(q.get() for _ in range(cores)))
    t = sum(times) / len(times)
    value = cores / t
    if tcd:
        print(json.dumps({
            "metric": TCD_METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": t * 1e3 / cores,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": TCD_WORKLOAD, "dofs": 912673},
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": "each step: %d concurrent CN steps (one per host core) of "
                                       "the workload on 24^3x6 tetrahedra, each scaled by DOFs "
                                       "to 912,673 DOFs; C restatement of the reference" % cores},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }))
        return
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": STATIONARY[args.workload]["workload"],
                   "dofs": full_ndof(args.workload)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "each step: %d concurrent solves (one per host core) by the C "
                                   "restatement of the reference%s; steps capped at 3" % (
                                       cores, "" if STATIONARY[args.workload]["cpu_sample"] is None
                                       else " on a smaller mesh, each scaled by DOFs to the "
                                            "full size")},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline sample")
    ap.add_argument("--workload", default="cd3d_q2_32",
                    choices=["cd3d_q2_32", "tcd3d_p2_48", "cd2d_q1_64", "cd3d_q2_96", "serve",
                             "batch"])
    ap.add_argument("--profile", action="store_true",
                    help="run one bracketed step for an ncu capture and exit")
    ap.add_argument("--slots", type=int, default=0,
                    help="serve: concurrent request slots (default 8)")
    ap.add_argument("--small", action="store_true",
                    help="with --profile: the 24^3x6 tetrahedral mesh (for detailed captures)")
    ap.add_argument("--no-extra", action="store_true",
                    help="headline only: no embedded record runs of the other workloads")
    ap.add_argument("--extra", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    EXTRA["on"] = args.extra
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "tcd3d_p2_48":
        run_gpu_tcd(args)
    elif args.workload == "serve":
        run_gpu_serve(args)
    elif args.workload == "batch":
        run_gpu_batch(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
