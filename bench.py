#!/usr/bin/env python3
"""Benchmark: design iterations/s of the voxel-SIMP inner loop on one GB300.

Workload (the large single-GPU configuration): a 256x128x128 hex8 cantilever
(4,194,304 elements, 12,830,211 DOFs), E0 = 1, nu = 0.3, p = 3, rho_min = 1e-3
(the reference's material law), filter radius 1.5, volume fraction 0.3, move 0.2,
MG-PCG to a relative residual of 1e-8 on the FP64 residual.  The x = 0 face is
clamped; a unit -z load sits at a seeded uniform point (numpy default_rng(0)) of
the x = nx end face, spread bilinearly to its four nodes.  Synthetic, seeded.

A step is one design iteration on a resident job (filter, penalised solve,
sensitivities, OC update with its bisection), timed with CUDA events on the job's
stream; `value` is the mixed-precision form (FP32 V-cycle inside FP64 iterative
refinement), the plain FP64 form is reported beside it.  `e2e` covers the same
iteration window through the public job API with host buffers: every step writes
the design from host memory, runs the iteration and reads the design and the
physical density back.  Inputs are larger than L2 (the fine vectors alone are
100 MB each), so no L2 flush is needed.

--impl reference times the reference's CPU path on the host cores: whole design
iterations of the same problem by the oracle's C restatement of the reference's
MG-PCG design iteration (oracle/oracle_mg.c; the reference tree itself is not
present on the GPU host), iterations 1..--ref-iterations from the uniform start.
The in-arm `cpu_baseline` runs the same code on the first iterations of the
timed window (the GPU job's design and displacement where the window starts).

Secondary workloads (--workload; one JSON line each, not the headline):
  batch  -- 64 seeded designs of the batched workload (nx in [32,128], ny, nz in
            [16,64]) run concurrently through the serving loop, mixed precision;
            value = aggregate design iterations/s; beside it the plain FP64 form
            one design at a time on a sample of the same designs.
  homog  -- periodic homogenization of 512 seeded 32^3 gyroid/octet cells at
            relative densities U[0.1, 0.4], six strain columns each, tol 1e-8,
            mixed precision; value = cells/s; the FP64 form on a sample of the
            cells beside it, with the tensors' relative difference.
  serve  -- an open-loop Poisson stream (4 jobs/s, --serve-seconds of arrivals;
            the reference's 10-minute stream is shortened so the run stays within
            minutes) of jobs log-uniform between 24^3 and 192x96x96 elements, 40
            design iterations each, 150 GB HBM budget; p50/p99 latency, jobs/s and
            GPU occupancy, beside the plain FP64 one-at-a-time service time.
  gatev2 -- the two Gate V2 problems (cantilever 24x8x8, clamped beam 48x8x8)
            under the locked projected formulation, 300 iterations each, in
            both forms with their gate metrics; the oracle's time beside them.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(nx=256, ny=128, nz=128)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(nx, ny, nz):
    """DRAM bytes per launch of the FP32 fine operator from the committed ncu
    capture of the same workload (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", f"fine_op_fp32_column_{nx}x{ny}x{nz}.txt")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":")[1])
    except OSError:
        pass
    return None


def cantilever_random_load(nx, ny, nz, seed=0):
    from topopt_gb300.workloads import cantilever_seeded_load
    return cantilever_seeded_load(nx, ny, nz, seed)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ CPU side
def host_cores():
    """Host cores this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_port():
    """The oracle's C restatement with its parallel loops on every host core
    (torchrun exports OMP_NUM_THREADS=1 to its ranks; the CPU legs override it)."""
    from oracle.oracle import OracleLib
    port = OracleLib("port")
    port.set_threads(host_cores())
    return port


def cpu_iterations(nx, ny, nz, n, x0=None, u0=None):
    """Whole design iterations of the benchmark problem on the host cores: the
    oracle's CPU restatement of the reference's MG-PCG design iteration
    (oracle/oracle_mg.c: filter, modulus, reduced system, Galerkin hierarchy,
    MG-PCG warm-started from the previous displacement, sensitivities, OC),
    from design x0 (the uniform start when None) and warm start u0."""
    from oracle.oracle import Problem
    port = oracle_port()
    bcs, loads = cantilever_random_load(nx, ny, nz)
    o = Problem(nx, ny, nz, 1.0, None, bcs, loads)
    x = np.full(o.nv, 0.3) if x0 is None else x0
    r = port.design_iterations_mg(o, x, n, u=u0, cg_tol=1e-8)
    per = r["seconds"].sum(axis=1)
    return dict(value=n / float(per.sum()), unit="design_iters/s", cores=port.threads(),
                kind="port", seconds=r["seconds"], cg=[int(c) for c in r["cg"]],
                compliance=[float(c) for c in r["compliance"]], per_iter_s=per)


def cpu_phase_note(r):
    ph = r["seconds"].mean(axis=0)
    return (f"per iteration {r['per_iter_s'].mean():.1f} s: filter {ph[0]:.2f}, reduced system + "
            f"hierarchy {ph[1]:.2f}, MG-PCG {ph[2]:.2f} ({'/'.join(str(c) for c in r['cg'])} "
            f"iterations), sensitivities {ph[3]:.2f}, OC {ph[4]:.2f} s")


def run_reference(args, world, rank, pg):
    """The reference's CPU path on the host cores: whole design iterations
    1..n of the benchmark problem from the uniform start (the reference's own
    first iterations), timed end to end per iteration."""
    if rank != 0:
        return
    nx, ny, nz = args.nx, args.ny, args.nz
    n = max(1, min(args.steps, args.ref_iterations))
    r = cpu_iterations(nx, ny, nz, n)
    v = r["value"]
    sample = (f"oracle/oracle_mg.c (CPU restatement of the reference's MG-PCG design iteration), "
              f"{nx}x{ny}x{nz} design iterations 1..{n} from the uniform start, whole "
              f"iterations timed; " + cpu_phase_note(r))
    line = {"impl": "reference", "metric": "design_iters_per_s", "value": v,
            "unit": "design_iters/s", "n_gpus": world, "steps": n, "warmup": 0,
            "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(args),
            "cpu_baseline": {"value": v, "unit": "design_iters/s", "cores": r["cores"],
                             "kind": r["kind"], "sample": sample},
            "cg_iterations": r["cg"], "compliance": r["compliance"],
            "e2e": {"value": v, "unit": "design_iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": f"cantilever {args.nx}x{args.ny}x{args.nz} hex8 SIMP, seeded end-face load",
            "elements": args.nx * args.ny * args.nz,
            "dofs": 3 * (args.nx + 1) * (args.ny + 1) * (args.nz + 1),
            "volfrac": 0.3, "rmin": 1.5, "move": 0.2, "penal": 3, "cg_tol": 1e-8,
            "solver": "MG-PCG (Galerkin, damped Jacobi 1+1, dense Cholesky coarsest)",
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas"}


# ----------------------------------------------------------------- our arm
def run_ours(args, world, rank, local, pg):
    import topopt_gb300 as tg
    from topopt_gb300.build import build
    build()
    tg.lib().tg_set_device(local)
    nx, ny, nz = args.nx, args.ny, args.nz
    bcs, loads = cantilever_random_load(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, bcs, loads)
    params = tg.SimpParams()

    def opts(prec, K):
        return tg.SimpOptions(volume_fraction=0.3, filter_radius=1.5, move=0.2, change_tol=0.0,
                              cg_tolerance=1e-8, max_iterations=K,
                              solve=tg.SolveOptions(precision=prec, mg_levels=args.mg_levels,
                                                    graph_mode=tg.GRAPH_OFF if args.no_graph
                                                    else tg.GRAPH_ON))

    fp64_peak, fp32_peak = tg.device_fma_peaks() if not args.profile else (None, None)
    forms = {}
    order = ["mixed", "fp64"] if not args.skip_fp64 else ["mixed"]
    for form in order:
        prec = tg.PREC_MIXED if form == "mixed" else tg.PREC_FP64
        job = tg.SimpJob(pb, params, opts(prec, args.warmup + args.steps + 1))
        sched = tg.fp32_schedule(nx, ny, nz)
        for _ in range(args.warmup):
            job.step()
        if form == "mixed":  # the state the timed window starts from (CPU baseline input)
            window_x, _ = job.read()
            window_u = job.read_displacement()
        barrier(pg)
        launches0 = tg.kernel_launches()
        rows = []
        with ClockSampler(local) as cs:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                rows.append(job.step())
            wall = time.perf_counter() - t0
        launches = tg.kernel_launches() - launches0
        dev_s = sum(r["t_device_ms"] for r in rows) / 1e3
        dev_s = max_over_ranks(pg, dev_s)
        forms[form] = dict(
            design_iters_per_s=sum_over_ranks(pg, args.steps) / dev_s,
            ms_per_step=1e3 * dev_s / args.steps, wall_s=wall, launches=launches,
            clocks=cs.summary(),
            solve_ms=statistics.median(r["t_solve_ms"] for r in rows),
            cg_iterations=[r["cg_iterations"] for r in rows],
            fine_matvecs_fp64=statistics.median(r["fine_matvecs"] for r in rows),
            fine_matvecs_fp32=statistics.median(r["fine_matvecs_lowp"] for r in rows),
            oc_volume_evals=statistics.median(r["oc_volume_evals"] for r in rows),
            oc_volume_passes=statistics.median(r["oc_volume_passes"] for r in rows),
            compliance=[r["compliance"] for r in rows],
            device_gb=job.device_bytes / 1e9)
        if form == "mixed":
            forms[form]["fp32_schedule"] = {"kind": sched[0], "shape": sched[1], "kz": sched[2],
                                            "source": "measured on the job's first use of the grid"}
            forms[form]["op_level1_tc_ms"] = job.time_operator(tg.APPLY_L1_TC, 10)
            forms[form]["op_level1_stencil_ms"] = job.time_operator(tg.APPLY_L1_STENCIL, 10)
        # Dominant-kernel timing (CUDA events, job stream).
        forms[form]["op_fp64_ms"] = job.time_operator(tg.PREC_FP64, 5)
        if form == "mixed":
            forms[form]["op_df_residual_ms"] = job.time_operator(2, 5)
        if form == "mixed":
            forms[form]["op_fp32_ms"] = job.time_operator(tg.PREC_MIXED, 20)
            design, _ = job.read()
        job.close()
    # Mixed vs FP64 accuracy on the same design (compliance and displacement).
    acc = {}
    if not args.skip_fp64 and not args.profile:
        r64 = tg.simp_compliance(pb, params, _phys_of(tg, pb, design), tolerance=1e-8,
                                 options=tg.SolveOptions(precision=tg.PREC_FP64))
        r32 = tg.simp_compliance(pb, params, _phys_of(tg, pb, design), tolerance=1e-8,
                                 options=tg.SolveOptions(precision=tg.PREC_MIXED))
        acc = {"compliance_rel_err": abs(r32["compliance"] - r64["compliance"]) / abs(r64["compliance"]),
               "u_rel_maxnorm_err": float(np.abs(r32["u"] - r64["u"]).max() / np.abs(r64["u"]).max()),
               "solve_ms_fp64": r64["cg"].t_solve_ms, "solve_ms_mixed": r32["cg"].t_solve_ms,
               "cg_iters_fp64": r64["cg"].iterations, "cg_iters_mixed_inner": r32["cg"].iterations,
               "refinements_mixed": r32["cg"].refinements}
    # End to end through the public host API, the same iteration window as
    # `value`: a second job takes the same warm-up steps untimed, then every
    # timed step writes the design from host memory, runs the iteration and
    # reads the design and physical density back (page-locked host buffers from
    # tg_host_alloc, both ways).
    K = args.steps
    e2e_wall = None
    if not args.profile:
        job = tg.SimpJob(pb, params, opts(tg.PREC_MIXED, args.warmup + K + 1))
        for _ in range(args.warmup):
            job.step()
        xh, xph = tg.host_array(pb.nv), tg.host_array(pb.nv)
        job.read(xh, xph)
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(K):
            job.write_design(xh)
            job.step()
            job.read(xh, xph)
        e2e_wall = max_over_ranks(pg, time.perf_counter() - t0)
        job.close()
    nv, ndof = pb.nv, pb.ndof
    h2d = nv * 8  # the design, every step
    d2h = 2 * nv * 8  # the design and the physical density, every step
    hbm, src = peaks()
    m = forms["mixed"]
    op_bytes32 = 2 * ndof * 4 + nv * 4
    achieved = op_bytes32 / (m["op_fp32_ms"] * 1e-3) / 1e9
    fp64_alg_flops = 1152 * nv
    line = {
        "metric": "design_iters_per_s", "value": m["design_iters_per_s"], "unit": "design_iters/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded cantilever)", "config": workload_config(args),
        "clocks": m["clocks"], "gpu_launches": int(m["launches"]),
        "e2e": {"value": sum_over_ranks(pg, K) / e2e_wall if e2e_wall else None,
                "unit": "design_iters/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "includes": f"design iterations {args.warmup + 1}..{args.warmup + K} (the "
                            "window of value) through the job API: host design written, "
                            "iteration, design and physical density read back, every step "
                            "(page-locked host buffers, tg_host_alloc)"},
        "roofline": {"bound": "hbm", "kernel": "fine operator apply, FP32 (mixed V-cycle)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": src, "bytes_per_launch": op_bytes32,
                     "traffic": committed_traffic(nx, ny, nz),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one "
                                       "launch of the same workload (committed capture)",
                     "ms_per_launch": m["op_fp32_ms"]},
        "fp64_operator": {"ms_per_launch": m["op_fp64_ms"],
                          "reference_flops_per_launch": fp64_alg_flops,
                          "reference_equiv_tflops": fp64_alg_flops / (m["op_fp64_ms"] * 1e-3) / 1e12,
                          "executed_fp64_ops_per_element": 212,
                          "executed_tflops": 212 * nv / (m["op_fp64_ms"] * 1e-3) / 1e12,
                          "fp64_fma_peak_tflops": fp64_peak, "fp32_fma_peak_tflops": fp32_peak},
        "forms": forms, "mixed_vs_fp64": acc,
    }
    if rank == 0 and not args.no_cpu:
        n = max(1, args.ref_iterations)
        cb = cpu_iterations(nx, ny, nz, n, window_x, window_u)
        line["cpu_baseline"] = {
            "value": cb["value"], "unit": cb["unit"], "cores": cb["cores"], "kind": cb["kind"],
            "sample": (f"oracle/oracle_mg.c (CPU restatement of the reference's MG-PCG design "
                       f"iteration), design iterations {args.warmup + 1}..{args.warmup + n} of "
                       f"the same run (the GPU job's design and displacement at the start of the "
                       f"timed window), whole iterations timed; " + cpu_phase_note(cb))}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_op_only(args):
    """Operator launches on a resident job of the benchmark workload (its kept
    mask and element factors), for ncu captures: three launches of the FP32 or
    FP64 fine operator, or of the level-1 tensor-core operator ("l1tc").  The
    FP32 schedule comes from --fp32-schedule (kind,shape,kz), so no autotuning
    launches precede the captured ones."""
    import topopt_gb300 as tg
    from topopt_gb300.build import build
    build()
    if args.fp32_schedule:
        tg.set_fp32_schedule(*(int(v) for v in args.fp32_schedule.split(",")))
    nx, ny, nz = args.nx, args.ny, args.nz
    bcs, loads = cantilever_random_load(nx, ny, nz)
    pb = tg.Problem(nx, ny, nz, 1.0, None, bcs, loads)
    prec = tg.PREC_FP64 if args.op_only == "fp64" else tg.PREC_MIXED
    job = tg.SimpJob(pb, tg.SimpParams(), tg.SimpOptions(
        volume_fraction=0.3, filter_radius=1.5, move=0.2, change_tol=0.0, cg_tolerance=1e-8,
        max_iterations=2, solve=tg.SolveOptions(precision=prec, mg_levels=args.mg_levels)))
    form = {"fp32": tg.PREC_MIXED, "fp64": tg.PREC_FP64, "l1tc": tg.APPLY_L1_TC}[args.op_only]
    ms = job.time_operator(form, 3)
    job.close()
    print(json.dumps({"op_only": args.op_only, "ms_per_launch": ms,
                      "fp32_schedule": tg.fp32_schedule(nx, ny, nz)}))


# ------------------------------------------------------ secondary workloads
def _oracle_problem(pb):
    from oracle.oracle import Problem
    return Problem(pb.nx, pb.ny, pb.nz, pb.spacing, pb.tags, pb.bcs, pb.loads)


def _cpu_design_sample(designs, iters):
    """Whole OC design iterations of a few designs on the host cores, one design
    at a time: the oracle's CPU restatement of the reference's MG-PCG design
    iteration.  Returns (iterations/s, cores, note)."""
    port = oracle_port()
    n, t = 0, 0.0
    for pb, prm, opt in designs:
        o = _oracle_problem(pb)
        x0 = np.full(o.nv, opt.volume_fraction)
        r = port.design_iterations_mg(o, x0, iters, volfrac=opt.volume_fraction,
                                      radius=opt.filter_radius, move=opt.move, cg_tol=1e-8)
        n += iters
        t += float(r["seconds"].sum())
    return n / t, port.threads(), f"{len(designs)} designs x {iters} iterations, {t:.1f} s"


def _fp32_roofline(tg, pb, prm, opt, label):
    """The FP32 fine operator on one design (CUDA events on its job's stream)."""
    hbm, src = peaks()
    job = tg.SimpJob(pb, prm, tg.SimpOptions(
        volume_fraction=opt.volume_fraction, filter_radius=opt.filter_radius, move=opt.move,
        change_tol=0.0, max_iterations=2, solve=tg.SolveOptions(precision=tg.PREC_MIXED)))
    job.step()
    ms = job.time_operator(tg.PREC_MIXED, 20)
    job.close()
    byt = 2 * pb.ndof * 4 + pb.nv * 4
    ach = byt / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": f"fine operator apply, FP32, {label}", "achieved": ach,
            "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_source": src,
            "bytes_per_launch": byt, "ms_per_launch": ms, "traffic": None}


def _pctl(v, q):
    return float(np.percentile(np.asarray(v, dtype=float), q)) if len(v) else None


def run_batch(args):
    import topopt_gb300 as tg
    from topopt_gb300 import workloads
    from topopt_gb300.build import build
    build()
    K = args.steps
    jobs = [workloads.design(s, precision=tg.PREC_MIXED, iterations=K) for s in range(64)]
    # Warm-up: one small job through the library.
    pb, prm, opt = workloads.design(999, iterations=2, sizes=(32, 16, 16))
    tg.simp_optimize(pb, prm, opt)
    srv = tg.Server(hbm_budget_bytes=150 << 30, max_active=args.max_active)
    with ClockSampler(0) as cs:
        t0 = time.perf_counter()
        tickets = [srv.submit(pb, prm, opt) for pb, prm, opt in jobs]
        res = [srv.wait(t, fields=False) for t in tickets]
        wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    iters = sum(r["iterations"] for r in res)
    launches = None
    # Plain FP64, one design at a time, on a sample.
    sample = [workloads.design(s, precision=tg.PREC_FP64, iterations=K) for s in range(4)]
    t0 = time.perf_counter()
    for pb, prm, opt in sample:
        tg.simp_optimize(pb, prm, opt)
    t64 = time.perf_counter() - t0
    line = {"metric": "design_iters_per_s", "value": iters / wall, "unit": "design_iters/s",
            "n_gpus": 1, "steps": K, "warmup": 1, "higher_is_better": True, "dtype": "f32+f64",
            "data": "synthetic (64 seeded designs)", "impl": "ours",
            "config": {"workload": "batched SIMP, 64 designs, nx in [32,128], ny,nz in [16,64]",
                       "elements_total": int(sum(pb.nv for pb, _, _ in jobs)),
                       "form": "mixed, concurrent resident jobs (serving loop)",
                       "max_active": args.max_active},
            "wall_s": wall, "clocks": cs.summary(), "server": st,
            "fp64_one_at_a_time": {"design_iters_per_s": 4 * K / t64, "designs": 4},
            "speedup_vs_fp64_one_at_a_time": (iters / wall) / (4 * K / t64)}
    # The whole batch already runs through the public API with host buffers.
    h2d = sum(pb.nv + 16 * (pb.nbc + pb.nloads) for pb, _, _ in jobs)
    d2h = sum(2 * pb.nv * 8 for pb, _, _ in jobs)
    line["e2e"] = {"value": iters / wall, "unit": "design_iters/s",
                   "h2d_bytes_per_step": h2d / max(1, iters), "d2h_bytes_per_step": d2h / max(1, iters),
                   "includes": "submission of every design (host problem), all iterations, results "
                               "(design and physical density) read back"}
    big = max(jobs, key=lambda j: j[0].nv)
    line["roofline"] = _fp32_roofline(tg, *big, f"largest design of the batch "
                                                  f"({big[0].nx}x{big[0].ny}x{big[0].nz})")
    if not args.no_cpu:
        v, cores, note = _cpu_design_sample(jobs[:3], 2)
        line["cpu_baseline"] = {"value": v, "unit": "design_iters/s", "cores": cores,
                                "kind": "port",
                                "sample": "oracle/oracle_mg.c (CPU restatement of the reference's "
                                          "MG-PCG design iteration), one design at a time: " + note}
    print(json.dumps(line), flush=True)


def run_homog(args):
    import topopt_gb300 as tg
    from topopt_gb300 import lattice
    from topopt_gb300.build import build
    build()
    cells, meta = lattice.batch(args.cells, vpc=32, seed=0)
    tg.homogenize(cells[:1], tolerance=1e-8, precision=tg.PREC_MIXED)  # warm-up
    with ClockSampler(0) as cs:
        t0 = time.perf_counter()
        ch32, info = tg.homogenize(cells, tolerance=1e-8, precision=tg.PREC_MIXED)
        wall = time.perf_counter() - t0
    ns = min(args.cells, 32)
    t0 = time.perf_counter()
    ch64, info64 = tg.homogenize(cells[:ns], tolerance=1e-8, precision=tg.PREC_FP64)
    t64 = time.perf_counter() - t0
    err = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(ch32[:ns], ch64))
    line = {"metric": "cells_per_s", "value": args.cells / wall, "unit": "cells/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32+f64", "impl": "ours",
            "data": "synthetic (seeded gyroid/octet cells)",
            "config": {"workload": f"periodic homogenization, {args.cells} cells of 32^3, 6 strains",
                       "tol": 1e-8, "solver": "batched Jacobi-PCG (FP32 inner, FP64 refinement)"},
            "wall_s": wall, "clocks": cs.summary(), "info": info,
            "fp64": {"cells_per_s": ns / t64, "cells": ns, "info": info64},
            "ch_rel_err_mixed_vs_fp64": err,
            "mean_density": float(np.mean([m[2] for m in meta]))}
    line["e2e"] = {"value": args.cells / wall, "unit": "cells/s",
                   "h2d_bytes_per_step": 32 ** 3, "d2h_bytes_per_step": 36 * 8,
                   "includes": "tg_homogenize on host cell arrays: upload, batched solves, tensors "
                               "read back (per cell)"}
    line["roofline"] = None
    line["roofline_note"] = ("the batched periodic operator runs inside the lock-step solve only; "
                             "its kernel is the pencil operator of the FP64 form (see the headline "
                             "line for the fine operator's roofline)")
    if not args.no_cpu:
        port = oracle_port()
        nc = 2
        t0 = time.perf_counter()
        for c in cells[:nc]:
            port.homogenize(32, 32, 32, solid=np.ascontiguousarray(c).ravel(), tol=1e-8)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nc / tc, "unit": "cells/s", "cores": 1, "kind": "port",
                                "sample": f"oracle homogenize (FP64 Jacobi-PCG, the harness's "
                                          f"method; its periodic operator is a serial loop), "
                                          f"{nc} cells of the batch, one core"}
    print(json.dumps(line), flush=True)


def run_serve(args):
    import threading
    import topopt_gb300 as tg
    from topopt_gb300 import workloads
    from topopt_gb300.build import build
    build()
    tg.set_sync_mode(args.sync_mode)
    stream = workloads.stream(0, rate=4.0, duration=args.serve_seconds, precision=tg.PREC_MIXED)
    pb, prm, opt = workloads.design(999, iterations=2, sizes=(32, 16, 16))
    tg.simp_optimize(pb, prm, opt)  # warm-up
    srv = tg.Server(hbm_budget_bytes=150 << 30, max_active=args.max_active)
    tickets = []
    with ClockSampler(0) as cs:
        t0 = time.perf_counter()

        def feeder():
            for at, pb, prm, opt in stream:
                d = at - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                tickets.append(srv.submit(pb, prm, opt))

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        res = [srv.wait(t, fields=False) for t in tickets]
        wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = [r["t_latency_ms"] for r in res]
    # The plain FP64 form, one job at a time, on a sample of the same stream.
    sample = [(p, q, o) for _, p, q, o in stream[:6]]
    t1 = time.perf_counter()
    for p, q, o in sample:
        o.solve = tg.SolveOptions(precision=tg.PREC_FP64)
        tg.simp_optimize(p, q, o)
    svc64 = (time.perf_counter() - t1) / len(sample)
    line = {"metric": "p50_p99_job_latency_ms", "value": _pctl(lat, 50), "p99_ms": _pctl(lat, 99),
            "unit": "ms", "n_gpus": 1, "higher_is_better": False, "dtype": "f32+f64",
            "impl": "ours", "data": "synthetic (seeded Poisson job stream)",
            "config": {"workload": "serving: Poisson 4 jobs/s, 24^3..192x96x96, 40 iterations",
                       "arrival_seconds": args.serve_seconds, "jobs": len(stream),
                       "hbm_budget_gb": 150, "max_active": args.max_active},
            "jobs_per_s": len(res) / wall, "wall_s": wall,
            "host_busy_frac": st["busy_ms"] / st["uptime_ms"] if st["uptime_ms"] else None,
            "queue_ms_p50": _pctl([r["t_queue_ms"] for r in res], 50),
            "queue_ms_p99": _pctl([r["t_queue_ms"] for r in res], 99),
            "server": st, "clocks": cs.summary(),
            "fp64_one_at_a_time": {"mean_service_s": svc64, "jobs_per_s": 1.0 / svc64,
                                   "sample_jobs": len(sample)}}
    line["host_busy_note"] = ("fraction of the loop's uptime with at least one job admitted "
                              "(host-side), not device occupancy")
    line["e2e"] = {"value": _pctl(lat, 50), "unit": "ms",
                   "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                   "includes": "arrival (host problem) to result read back, through tg_server"}
    if not args.no_cpu:
        small = sorted(stream, key=lambda a: a[1].nv)[:2]
        v, cores, note = _cpu_design_sample([(p, q, o) for _, p, q, o in small], 2)
        its = small[0][3].max_iterations
        line["cpu_baseline"] = {"value": 1e3 * its / v, "unit": "ms (service time of a job, "
                                "one at a time)", "cores": cores, "kind": "port",
                                "sample": "oracle/oracle_mg.c design iterations on the two "
                                          f"smallest jobs of the stream ({note}), scaled to "
                                          f"{its} iterations per job"}
    print(json.dumps(line), flush=True)


def run_gatev2(args):
    """The Gate V2 benchmark problems end to end (300 projected OC iterations,
    beta 1 -> 32) in both forms, their gates, and the oracle's time for the same
    run on the host cores."""
    import topopt_gb300 as tg
    from oracle.oracle import CONTINUATION, GATE_V2, gate_v2_metrics, gate_v2_problem
    from topopt_gb300.build import build
    build()
    out = {}
    for name in GATE_V2:
        o = gate_v2_problem(name)
        pb = tg.Problem(o.nx, o.ny, o.nz, 1.0, None, list(zip(o.bc_node, o.bc_comp, o.bc_val)),
                        list(zip(o.ld_node, o.ld_comp, o.ld_val)))
        row = {}
        for form, prec in (("mixed", tg.PREC_MIXED), ("fp64", tg.PREC_FP64)):
            opt = tg.SimpOptions(volume_fraction=0.3, filter_radius=2.5, change_tol=0.0,
                                 cg_tolerance=1e-9, projection=list(CONTINUATION),
                                 solve=tg.SolveOptions(precision=prec))
            tg.simp_optimize(pb, tg.SimpParams(), tg.SimpOptions(
                volume_fraction=0.3, filter_radius=2.5, change_tol=0.0, cg_tolerance=1e-9,
                projection=[(1.0, 0.2, 3)], solve=tg.SolveOptions(precision=prec)))  # warm-up
            t0 = time.perf_counter()
            s = tg.simp_optimize(pb, tg.SimpParams(), opt)
            wall = time.perf_counter() - t0
            hc = [h["compliance"] for h in s["history"]]
            ncomp, mnd, ysym = gate_v2_metrics(o.nx, o.ny, o.nz, s["physical_density"])
            row[form] = {"wall_s": wall, "iters_per_s": s["iterations"] / wall,
                         "stage_end_compliance": [hc[50 * k + 49] for k in range(6)],
                         "final_compliance": s["compliance"],
                         "volume_fraction": s["volume_fraction"], "components": ncomp,
                         "mnd": mnd, "y_symmetry": ysym,
                         "oc_volume_passes": int(sum(h["oc_volume_passes"]
                                                     for h in s["history"])),
                         "cg_iterations": int(sum(h["cg_iterations"] for h in s["history"]))}
        if not args.no_cpu:
            port = oracle_port()
            t0 = time.perf_counter()
            r = port.simp_optimize(o, volfrac=0.3, radius=2.5, change_tol=0.0,
                                   cg_tol=1e-9, stages=CONTINUATION)
            row["cpu_port"] = {"wall_s": time.perf_counter() - t0, "cores": port.threads(),
                               "final_compliance": r["compliance"]}
        out[name] = row
    tot = sum(r["mixed"]["wall_s"] for r in out.values())
    line = {"metric": "gate_v2_runs_per_s", "value": len(out) / tot, "unit": "runs/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f32+f64", "impl": "ours",
            "data": "the Gate V2 benchmark problems (cantilever 24x8x8, clamped beam 48x8x8)",
            "config": {"workload": "projected SIMP, 6 stages x 50 OC iterations, rmin 2.5, "
                                   "cg_tol 1e-9", "form": "mixed (fp64 beside it)"},
            "runs": out}
    if not args.no_cpu:
        cpu = sum(r["cpu_port"]["wall_s"] for r in out.values())
        cores = max(r["cpu_port"]["cores"] for r in out.values())
        line["cpu_baseline"] = {"value": len(out) / cpu, "unit": "runs/s", "cores": cores,
                                "kind": "port", "sample": "both problems, full 300 iterations"}
    print(json.dumps(line), flush=True)


def _phys_of(tg, pb, design):
    return tg.make_density_filter(pb, 1.5).filter_density(design)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=WORKLOAD["nx"])
    ap.add_argument("--ny", type=int, default=WORKLOAD["ny"])
    ap.add_argument("--nz", type=int, default=WORKLOAD["nz"])
    ap.add_argument("--mg-levels", type=int, default=7)
    # Whole CPU design iterations timed by the reference arm and the CPU baseline
    # (each ~20-40 s at 16 host threads on the 256x128x128 cantilever).
    ap.add_argument("--ref-iterations", type=int, default=2)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--op-only", choices=["fp32", "fp64", "l1tc"], default=None,
                    help="profiling aid: three launches of one operator on a resident job")
    ap.add_argument("--fp32-schedule", default=None,
                    help="profiling aid: kind,shape,kz of the FP32 operator (tg_set_fp32_schedule)")
    ap.add_argument("--profile", action="store_true",
                    help="profiling aid: allow warmup < 3, skip e2e and the CPU baseline")
    ap.add_argument("--no-graph", action="store_true",
                    help="profiling aid: drive the mixed inner PCG loop from the host (same "
                         "kernels, same results) instead of one CUDA graph")
    ap.add_argument("--workload", choices=["cantilever", "batch", "homog", "serve", "gatev2"],
                    default="cantilever")
    ap.add_argument("--cells", type=int, default=512)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    # 32 concurrent resident jobs: measured best for the serving mix (16: p50 8.3 s,
    # 32: 5.8 s, 48: 5.9 s; the GPU is saturated at ~2.4 jobs/s from 32 on).
    ap.add_argument("--max-active", type=int, default=32)
    ap.add_argument("--sync-mode", type=int, default=0,
                    help="host wait mode for the serving workloads: 0 default, 2 yield, 3 blocking")
    args = ap.parse_args()
    if args.workload != "cantilever":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "secondary workloads are GPU-only; the CPU baseline is reported on "
                              "the cantilever workload"}), flush=True)
            return
        {"batch": run_batch, "homog": run_homog, "serve": run_serve,
         "gatev2": run_gatev2}[args.workload](args)
        return
    if args.op_only:
        run_op_only(args)
        return
    if args.warmup < 3 and not args.profile:
        args.warmup = 3
    if args.profile:
        args.no_cpu = True
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
