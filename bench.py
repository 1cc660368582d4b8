"""Benchmark: pressure solves/s on the 256x256x96 sloping-beach workload.

One step = one PCGPME solve (setup + BiCGSTAB to ERR <= 1e-10, the reference's
stop tests) of the assembled pressure system.  ``value`` is measured with the
matrix, right-hand side and workspace resident in HBM (as inside the
reference's ik loop); ``e2e`` is the same solve through the host-array drop-in
``pcgpme_gpu`` (the call the Fortran model makes), with the host->device copy
of AL, LL, D, B, X and the device->host copy of X inside the timed region.

``--impl reference`` times the reference algorithm on the host cores instead:
the oracle's OpenMP restatement of PCGPME (the Fortran reference cannot be
compiled here: ifort-only, no Fortran compiler on either machine).

Multi-GPU: the solve is one coupled system, so N GPUs run N independent
replicas (one solve each per step, weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__ as ge  # noqa: E402

WORKLOAD = "beach_256x256x96"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# Algorithmic bytes (the fixed count roofline.achieved uses): floating-point
# streams only, at the stored word size w (8 FP64, 4 FP32); index traffic and
# gathered neighbour values are not counted.  One operator application PM A x:
# AXSUB D + 6 AL + x + y = 9w, LDUSUB sweeps 1-4 3w each = 12w, sweep 5/6
# AL5 + AL6 + in + out = 4w -> 25w.  One iteration: 2 applications (50w) + RQ 2w
# + e 3w + AMU/SS 2w + x/r 7w + p 4w = 68w.  Setup of a solve: scaling 16w,
# PM b 16w, PM A x0 25w, r0 pass 5w = 62w.  So FP64: N (496 + 544 iters).
# Mixed: N [96 + sum over sweeps (248 + 272 inner iters) + 100 per sweep]
# (FP32 inner iterations; 100 B per sweep for the FP64 refinement residual and
# accumulation; 96 B for the FP64 -> FP32 conversion).
# Measured DRAM bytes per row and iteration of the loop graph (ncu, the graph as
# one unit, beach_256x256x96): profiles/pcgpme_loop_dram_beach_256x256x96.md.
TRAFFIC_ROW_ITER_FP64 = 434.2
TRAFFIC_ROW_ITER_MIXED = 224.6

# What pins the CPU port: run on one thread it reproduces the reference's own
# PCGPME, executed from its Fortran source, bit for bit.
PORT_PARITY = ("serially bit-identical to the reference's PCGPME run from its source text "
               "(tests/test_oracle_reference_runs.py)")

# FP64 arithmetic of one iteration per row, in fused multiply-adds (a multiply or
# an add counts as one): AXSUB D x + 6 AL = 7 and LDUSUB 6 sweeps = 6 per
# application (26 for two), RQ 1, e 1, AMU and SS 2, x 2, r 1, RN and C1 2, p 2
# -> 37 (pcgpme_para.F90:147-352).  The kernels issue about 41 (ncu counters:
# warp sums of the dot products and rows of partial chunks):
# profiles/pcgpme_kernels_full_beach_192x192x64.md.
FMA_ROW_ITER_FP64 = 37


def bytes_solve_fp64(n: int, iters: int) -> float:
    return float(n) * (496 + 544 * iters)


def bytes_solve_mixed(n: int, inner_iters: int, outer: int) -> float:
    return float(n) * (96 + 248 * outer + 272 * inner_iters + 100 * outer)


# The same count with the 4-byte column-index streams added (6 + 4 + 2 per
# application: 96 B per iteration, 72 B in the setup), reported beside it.
def bytes_solve_fp64_with_indices(n: int, iters: int) -> float:
    return float(n) * (496 + 72 + (544 + 96) * iters)


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu_index = gpu_index
        self.path = pathlib.Path(tempfile.gettempdir()) / f"clowns_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.path.read_text().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("CLOWNS_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    """Slowest rank's time (the job's time).  CPU tensor under gloo."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference_solve(ora, sy, eps, threads):
    t0 = time.perf_counter()
    r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=eps, nthreads=threads)
    return time.perf_counter() - t0, r


def run_reference(args, world, rank):
    """Reference arm: the oracle's OpenMP PCGPME on all host cores."""
    if rank != 0:
        return
    pkg = ge.load_package()
    ora = ge.load_oracle()
    ora.build()
    case = workload_case(pkg, args.workload)
    cls, sm, sy = ora.prepare(case)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_solve(ora, sy, case.eps0, threads)
    times = []
    last = None
    for _ in range(args.steps):
        t, last = cpu_reference_solve(ora, sy, case.eps0, threads)
        times.append(t)
    tot = sum(times)
    value = args.steps / tot
    line = {
        "impl": "reference", "metric": "pressure solves/s", "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "rows": sy.mnoe, "tol": case.eps0, "iters": last.iters},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": f"full solves of {args.workload} (N={sy.mnoe}, {last.iters} iterations), "
                                   f"OpenMP restatement of pcgpme_para.F90, {threads} threads",
                         "port_parity": PORT_PARITY},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def true_residual(ds, x):
    """||b - A x|| / ||b|| of the assembled (unscaled, unpreconditioned) system,
    evaluated on the device with torch outside the timed region (alu/llu are
    (6, mm2) column blocks, llu 1-based with 0 = no neighbour)."""
    import torch
    n = ds.mnoe
    xv = x[:n]
    ax = ds.de[:n] * xv
    for k in range(ds.alu.shape[0]):
        c = ds.llu[k, :n].long()
        g = torch.where(c > 0, xv[(c - 1).clamp(min=0)], torch.zeros_like(xv))
        ax = ax + ds.alu[k, :n] * g
    b = ds.b[:n]
    return float(torch.linalg.norm(b - ax) / torch.linalg.norm(b))


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.processor() or platform.machine()


def time_device(fn, steps, stream):
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    out = [fn() for _ in range(steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), out


def workload_case(pkg, name):
    wl = pkg.workload
    if name == "beach_256x256x96":
        return wl.beach_256x256x96(seed=1)
    if name == "beach_512x384x128":
        return wl.beach_512x384x128()
    if name == "beach_192x192x64":
        return wl.beach_192x192x64()
    if name == "tank_64x64x32":
        return wl.tank_64x64x32()
    if name.startswith("beach_"):
        nx, ny, nz = (int(v) for v in name.split("_")[1].split("x"))
        return wl.beach_case(nx, ny, nz, seed=1)
    raise SystemExit(f"unknown workload {name}")


def run_ensemble(args):
    """Batched ensemble (64 members, grids U[96,256] x U[96,192] x U[48,80], slopes
    U(1/30,1/10), 0-40 obstacles, amplitudes U(0.01,0.1)): one batched mixed solve
    and one batched FP64 solve against serial per-member launches of the plain
    FP64 and mixed paths.  Prints one JSON line."""
    import torch
    pkg = ge.load_package()
    pkg.build()
    specs = pkg.workload.ensemble_members(n=args.members, seed=3, scale=args.member_scale)
    systems, xs, sizes = [], [], []
    t0 = time.perf_counter()
    for sp in specs:
        case = pkg.workload.ensemble_case(sp)
        dc, ds = pkg.prepare_dev(case)
        del dc
        systems.append((ds.alu, ds.llu, ds.de, ds.b))
        xs.append(torch.zeros(ds.mm2, dtype=torch.float64, device="cuda"))
        sizes.append(ds.mnoe)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    eps = 1e-10

    def zero():
        for x in xs:
            x.zero_()

    def serial(kind):
        solvers = [pkg.Solver(n) if kind == "fp64" else pkg.MixedSolver(n) for n in sizes]

        def run():
            zero()
            return [sv.solve(*sy, x, eps=eps) for sv, sy, x in zip(solvers, systems, xs)]
        return run

    def batched(prec):
        bs = pkg.BatchedSolver(sizes, prec)

        def run():
            zero()
            return bs.solve(systems, xs, eps=eps)
        return run

    out = {}
    for name, fn in (("serial_fp64", serial("fp64")), ("serial_mixed", serial("mixed")),
                     ("batched_fp64", batched(pkg.PREC_FP64)), ("batched_mixed", batched(pkg.PREC_MIXED))):
        for _ in range(max(1, args.warmup)):
            fn()
        ms, res = time_device(fn, args.steps, stream)
        infos = res[-1]
        row_iters = float(sum(n * i.iter for n, i in zip(sizes, infos)))
        out[name] = {"ms_per_ensemble": ms / args.steps, "solves_per_s": len(sizes) * args.steps / (ms / 1000.0),
                     "iters_total": int(sum(i.iter for i in infos)), "max_eps": max(i.eps for i in infos),
                     "ier": sorted(set(int(i.ier) for i in infos)),
                     # sum over members of rows x iterations (inner ones for mixed), and the time per unit
                     "row_iterations": row_iters, "ps_per_row_iteration": ms / args.steps * 1e9 / row_iters}
    line = {"metric": "ensemble pressure solves/s", "unit": "solves/s", "members": len(sizes),
            "rows_total": int(sum(sizes)), "rows_min": int(min(sizes)), "rows_max": int(max(sizes)),
            "tol": eps, "generation_s": t_gen, "legs": out,
            "batched_mixed_vs_serial_fp64": out["batched_mixed"]["solves_per_s"] / out["serial_fp64"]["solves_per_s"],
            "batched_mixed_vs_serial_mixed": out["batched_mixed"]["solves_per_s"] / out["serial_mixed"]["solves_per_s"],
            "batched_fp64_vs_serial_fp64": out["batched_fp64"]["solves_per_s"] / out["serial_fp64"]["solves_per_s"]}
    print(json.dumps(line), flush=True)


def run_will(args):
    """PCGPME_WILL (the 2DH dispersion solve) on a seeded 2DH system of
    --will-grid cells (built like disp_param): device-resident solves/s, end to
    end through the host drop-in, and the oracle's OpenMP restatement on the
    host cores (rank 0).  Prints one JSON line."""
    import torch
    pkg = ge.load_package()
    pkg.build()
    nx, ny = (int(v) for v in args.will_grid.split("x"))
    ds = pkg.workload.dispersion_system(nx, ny, seed=11)
    n = ds.n
    eps = 1e-10
    al, ll, d = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (ds.al, ds.ll, ds.d))
    b0 = torch.from_numpy(ds.b).cuda()
    b = torch.empty_like(b0)
    solver = pkg.WillSolver(n)
    stream = torch.cuda.current_stream()

    def step():
        b.copy_(b0)
        return solver.solve(al, ll, d, b, eps=eps)

    for _ in range(max(3, args.warmup)):
        step()
    ms, infos = time_device(step, args.steps, stream)
    info = infos[-1]
    alh, llh = np.ascontiguousarray(ds.al), np.ascontiguousarray(ds.ll)
    bh = ds.b.copy()
    pkg.pcgpme_will(alh, llh, ds.d, bh, n, eps=eps)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bh[:] = ds.b
        pkg.pcgpme_will(alh, llh, ds.d, bh, n, eps=eps)
    e2e_s = (time.perf_counter() - t0) / args.steps
    ora = ge.load_oracle()
    ora.build()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    bo, it_o, reason = ora.pcgpme_will(ds.al, ds.ll, ds.d, ds.b, n, eps=eps, nthreads=threads)
    t_cpu = time.perf_counter() - t0
    bg = b.cpu().numpy()
    line = {"metric": "2DH dispersion solves/s (PCGPME_WILL)", "unit": "solves/s", "grid": args.will_grid,
            "rows": n, "tol": eps, "iters": info.iter, "iters_oracle": it_o,
            "value": args.steps / (ms / 1000.0), "ms_per_solve": ms / args.steps,
            "e2e": {"value": 1.0 / e2e_s, "unit": "solves/s",
                    "h2d_bytes_per_step": n * (4 * 8 + 4 * 4 + 2 * 8), "d2h_bytes_per_step": n * 8},
            "rel_l2_vs_oracle": float(np.linalg.norm(bg - bo) / np.linalg.norm(bo)),
            "tuned_shape": pkg.tuned_shape([n], 0),
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "solves/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"one solve, OpenMP restatement of pcgpme_2DH.f90 on {threads} threads"}}
    print(json.dumps(line), flush=True)


def run_ingest(args):
    """Real-case ingestion: the workload written in the reference's case-file
    format (sparse .xyzn and dense .xyz forms) to a scratch directory, then
    timed from files to converged pressure -- read_case on the host, upload,
    classification, coefficients, rows, assembly and the FP64 solve on the
    device, the pressure read back.  Checks that the system built from the
    files equals the one built from the generator bit for bit.  The host leg
    runs the same files through the oracle (16-thread PCGPME).  One JSON line."""
    import shutil
    import tempfile
    import torch
    pkg = ge.load_package()
    pkg.build()
    case = workload_case(pkg, args.workload)
    tmp = tempfile.mkdtemp(prefix="clowns_case_")
    try:
        out = {}
        for form in ("sparse", "dense"):
            prefix = os.path.join(tmp, f"{args.workload}_{form}")
            paths = pkg.ingest.write_case(prefix, case, sparse=(form == "sparse"))
            nbytes = sum(os.path.getsize(v) for v in paths.values())
            times = []
            for _ in range(max(1, args.steps)):
                t0 = time.perf_counter()
                got = pkg.ingest.read_case(prefix, eps0=case.eps0)
                times.append(time.perf_counter() - t0)
            t_read = statistics.median(times)
            out[form] = {"file_mb": nbytes / 1e6, "read_s": t_read, "read_mb_per_s": nbytes / 1e6 / t_read,
                         "prefix": prefix}
        prefix = out["sparse"].pop("prefix")
        out["dense"].pop("prefix")
        # parity: the system from the files against the system from the generator, whose spacings get
        # the rounding the reference's reader applies (set_dx, 1sub-main.F90:53-74)
        got = pkg.ingest.read_case(prefix, eps0=case.eps0).case
        gen = case.copy()
        gen.x, gen.dx = pkg.ingest.set_dx(gen.dims, gen.x)
        dc0, ds0 = pkg.prepare_dev(gen)
        dc1, ds1 = pkg.prepare_dev(got)
        torch.cuda.synchronize()
        same = (ds0.mnoe == ds1.mnoe and torch.equal(ds0.alu, ds1.alu) and torch.equal(ds0.llu, ds1.llu)
                and torch.equal(ds0.de, ds1.de) and torch.equal(ds0.b, ds1.b))
        n = ds1.mnoe
        solver = pkg.Solver(n)

        def files_to_pressure():
            c = pkg.ingest.read_case(prefix, eps0=case.eps0).case
            dc, ds = pkg.prepare_dev(c)
            x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
            info = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=case.eps0)
            return info, x[:ds.mnoe].cpu().numpy()

        for _ in range(max(1, args.warmup)):
            files_to_pressure()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            info, xg = files_to_pressure()
        torch.cuda.synchronize()
        t_e2e = (time.perf_counter() - t0) / args.steps
        line = {"metric": "case files to converged pressure per second", "unit": "cases/s",
                "workload": args.workload, "rows": n, "cells": int(case.inne2),
                "value": 1.0 / t_e2e, "s_per_case": t_e2e, "iters": info.iter, "tol": case.eps0,
                "files": out, "system_from_files_equals_generated": bool(same),
                "note": "the reader rounds grid spacings as the reference does (set_dx); the generated case "
                        "is compared after the same rounding"}
        if not args.no_cpu:
            ora = ge.load_oracle()
            ora.build()
            threads = os.cpu_count() or 1
            t0 = time.perf_counter()
            c = pkg.ingest.read_case(prefix, eps0=case.eps0).case
            cls, sm, sy = ora.prepare(c)
            ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=case.eps0, nthreads=threads)
            t_cpu = time.perf_counter() - t0
            line["rel_l2_vs_oracle"] = float(np.linalg.norm(xg - ref.x) / np.linalg.norm(ref.x))
            line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "cases/s", "cores": threads, "kind": "port",
                                    "cpu_model": cpu_model(),
                                    "sample": "one case: read_case, the oracle's set_nflag, init_matrix, rows, "
                                              f"assembly and PCGPME on {threads} threads"}
        print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_session(args):
    """The whole pressure-correction ik loop of one time step on the device
    (clowns_session_pressure_loop: row numbering, RHS and dmax, assembly, PCGPME,
    pressure and velocity correction, repeated until dmax < d0;
    1sub-momentum.F90:41-60) for --workload, against the oracle running the same
    loop on the host cores (rank 0).  Each timed step resets the fields first
    (host upload outside the device timing, inside the end-to-end one).  Prints
    one JSON line."""
    import torch
    pkg = ge.load_package()
    pkg.build()
    case = workload_case(pkg, args.workload)
    d0, eps0 = 1e-5, case.eps0
    p0 = np.zeros(case.inne2 + 2)
    s = pkg.Session(case)

    def reset():
        s.set_fields(case.nf, case.nfb, case.f, case.fb, case.a, case.un, case.sp, p0)
        return s.classify()

    reset()
    out = s.pressure_loop(case.dt, d0=d0, eps0=eps0)             # warm-up (autotuning, graphs)
    dev_ms, e2e_s, outs = [], [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        reset()
        torch.cuda.synchronize()
        ev0.record()
        out = s.pressure_loop(case.dt, d0=d0, eps0=eps0)
        ev1.record()
        torch.cuda.synchronize()
        got = s.fields()
        e2e_s.append(time.perf_counter() - t0)
        dev_ms.append(ev0.elapsed_time(ev1))
        outs.append(out)
    s.close()
    ora = ge.load_oracle()
    ora.build()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    cls = ora.set_nflag(case)
    sm = ora.init_matrix(case, cls)
    c = case.copy()
    c.f = cls.f.copy()
    pc = np.zeros(case.inne2 + 2)
    un = case.un.copy()
    ik = 0
    while True:
        c.un = un
        sy = ora.rows_rhs_assemble(c, cls, sm)
        if sy.dmax < d0 or ik >= 1000:
            break
        ik += 1
        r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=eps0, nthreads=threads)
        pc, un = ora.correct(c, cls, sy, r.x, pc, un)
    t_cpu = time.perf_counter() - t0
    ms = statistics.median(dev_ms)
    line = {"metric": "pressure-correction steps/s (whole ik loop on the device)", "unit": "steps/s",
            "workload": args.workload, "rows": int(got["mnoe"]), "ik_passes": outs[-1]["ik"], "ik_passes_oracle": ik,
            "solve_iters_last_pass": outs[-1]["iter"], "dmax": outs[-1]["dmax"], "icon": outs[-1]["icon"],
            "value": 1000.0 / ms, "ms_per_step": ms,
            "e2e": {"value": 1.0 / statistics.median(e2e_s), "unit": "steps/s"},
            "rel_l2_p_vs_oracle": float(np.linalg.norm(got["p"] - pc) / np.linalg.norm(pc)),
            "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"one step: the oracle's set_nflag, init_matrix and {ik} passes of numbering, "
                                       f"RHS, assembly, PCGPME ({threads} threads) and correction"}}
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Adjoint on the 192x192x64 beach: J = sum of 16 seeded gauge pressures with
    weights U(0.5,1.5); dJ/da for 200 seeded face fractions against central
    differences at relative step 1e-6 (evaluated through the exact difference
    identity) and dJ/db = lambda.  Prints one JSON line."""
    import torch
    sys.path.insert(0, str(ROOT / "tests"))
    from adjoint_harness import PressureSolve, PressureSystem, central_difference, fd_faces, gauges
    pkg = ge.load_package()
    pkg.build()
    case = pkg.workload.beach_192x192x64()
    system = PressureSystem(case)
    n = system.n
    rows, w = gauges(n)
    wt = torch.zeros(n, dtype=torch.float64, device="cuda")
    wt[torch.from_numpy(rows).cuda()] = torch.from_numpy(w).cuda()
    a0 = system.dc.a.clone()
    a = a0.clone().requires_grad_(True)
    b = system.b0[:n].clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = PressureSolve.apply(a, b, system)
    J = (wt * x).sum()
    J.backward()
    torch.cuda.synchronize()
    t_fwd_adj = time.perf_counter() - t0
    ga = a.grad.cpu().numpy()
    faces = fd_faces(system, count=args.faces)
    fd, ad = [], []
    t0 = time.perf_counter()
    for owner, l in faces:
        fd.append(central_difference(system, wt, a0, owner, l, x.detach()))
        ad.append(ga[owner, l])
    t_fd = time.perf_counter() - t0
    fd, ad = np.array(fd), np.array(ad)
    line = {"metric": "adjoint gradient vs central differences", "workload": "beach_192x192x64", "rows": n,
            "faces": len(faces), "fd_step_rel": 1e-6,
            "rel_l2_error": float(np.linalg.norm(ad - fd) / np.linalg.norm(fd)),
            "max_rel_error_face": float(np.max(np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-300))),
            "forward_plus_adjoint_s": t_fwd_adj, "fd_s": t_fd}
    print(json.dumps(line), flush=True)


def run_gpu(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    pkg = ge.load_package()
    pkg.build()
    case = workload_case(pkg, args.workload)
    dc, ds = pkg.prepare_dev(case)
    n = ds.mnoe
    solver = pkg.Solver(n)
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    launches = []

    def plain_step():
        x.zero_()                       # xe = 0 before every solve (1sub-momentum.F90:269)
        info = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=case.eps0)
        launches.append(pkg.last_kernel_launches())
        return info

    for _ in range(args.warmup):
        plain_step()
    launches.clear()
    # ---- device-resident timing (plain FP64: the headline value)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.5)
    barrier(world)
    torch.cuda.synchronize()
    ms, infos = time_device(plain_step, args.steps, stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = max_over_ranks(ms, world)
    info = infos[-1]
    it = int(round(statistics.mean(i.iter for i in infos)))
    per_solve_s = ms / 1000.0 / args.steps
    value = world * args.steps / (ms / 1000.0)
    peak, peak_kind = measured_peaks()
    alg = bytes_solve_fp64(n, it)
    achieved = alg / per_solve_s / 1e9
    args.fma_peak = pkg.fp64_fma_rate(stream)          # measured here, outside the timed region
    args.fma_achieved = FMA_ROW_ITER_FP64 * float(n) * it / per_solve_s
    x_plain = x[:n].cpu().numpy().copy()
    args.res_plain = true_residual(ds, x)

    legs = set(args.legs.split(","))
    if "apply" in legs:
        run_apply_profile(pkg, args, ds, stream)
    minfo = None
    m_value = ms_m = m_alg = None
    x_mixed = None
    # ---- mixed precision on the same system (FP32 storage + FP64 refinement)
    if "mixed" in legs:
        m_value, ms_m, minfo, m_alg, x_mixed = run_mixed(pkg, args, ds, case, world, stream)
    e2e_value = None
    if "e2e" in legs:
        e2e_value = run_e2e(pkg, args, ds, case, world)
    h2d = n * 6 * 8 + n * 6 * 4 + 3 * n * 8
    d2h = n * 8
    args.timed_launches = sum(launches)          # the library's kernels (the x = 0 fill is torch's)
    _report(pkg, args, world, rank, case, n, ms, infos, info, it, value, alg, achieved, peak, peak_kind,
            clk, x_plain, legs, m_value, ms_m, minfo, m_alg, x_mixed, e2e_value, h2d, d2h)


def run_apply_profile(pkg, args, ds, stream):
    """Operator application y = PM (W A) x through the test hook (row scaling,
    sort, AXSUB and the five LDUSUB sweeps as plain launches, so that a profiler
    can attribute them kernel by kernel)."""
    import torch
    n = ds.mnoe
    xv = torch.ones(n, dtype=torch.float64, device="cuda")
    for _ in range(max(1, args.steps)):
        pkg.apply_pm_a_dev(ds.alu, ds.llu, ds.de, n, xv)
    torch.cuda.synchronize()


def run_mixed(pkg, args, ds, case, world, stream):
    import torch
    n = ds.mnoe
    msolver = pkg.MixedSolver(n)
    xm = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")

    def mixed_step():
        xm.zero_()
        return msolver.solve(ds.alu, ds.llu, ds.de, ds.b, xm, eps=case.eps0, inner_tol=args.inner_tol)

    for _ in range(args.warmup):
        mixed_step()
    torch.cuda.synchronize()
    ms_m, minfos = time_device(mixed_step, args.steps, stream)
    ms_m = max_over_ranks(ms_m, world)
    minfo = minfos[-1]
    m_value = world * args.steps / (ms_m / 1000.0)
    m_alg = bytes_solve_mixed(n, minfo.iter, minfo.outer)
    x_mixed = xm[:n].cpu().numpy().copy()
    args.res_mixed = true_residual(ds, xm)
    return m_value, ms_m, minfo, m_alg, x_mixed


def run_e2e(pkg, args, ds, case, world):
    """Same solve through the host-array drop-in (Fortran call shape)."""
    import torch
    n = ds.mnoe
    al = ds.alu.cpu().numpy()
    ll = ds.llu.cpu().numpy()
    de = ds.de.cpu().numpy()
    b = ds.b.cpu().numpy()
    xh = np.zeros(ds.mm2)
    for _ in range(max(1, args.warmup)):
        xh[:] = 0.0
        pkg.pcgpme(al, ll, de, b, xh, n, eps=case.eps0)
    barrier(world)
    e2e_times = []
    for _ in range(args.steps):
        xh[:] = 0.0
        t0 = time.perf_counter()
        eps_o, it_o, ier = pkg.pcgpme(al, ll, de, b, xh, n, eps=case.eps0)
        e2e_times.append(time.perf_counter() - t0)
    barrier(world)
    e2e_s = max_over_ranks(sum(e2e_times), world)
    return world * args.steps / e2e_s


def _report(pkg, args, world, rank, case, n, ms, infos, info, it, value, alg, achieved, peak, peak_kind,
            clk, x_plain, legs, m_value, ms_m, minfo, m_alg, x_mixed, e2e_value, h2d, d2h):
    # ---- CPU baseline: the oracle on the host cores (rank 0, N=1 only)
    cpu = None
    err_plain = err_mixed = None
    if rank == 0 and world == 1 and not args.no_cpu and "cpu" in legs:
        ora = ge.load_oracle()
        ora.build()
        cls, sm, sy = ora.prepare(case)
        threads = os.cpu_count() or 1
        # all host cores: 3 warm-up solves, then the median of 10 full solves
        for _ in range(3):
            cpu_reference_solve(ora, sy, case.eps0, threads)
        times = []
        for _ in range(10):
            t, r = cpu_reference_solve(ora, sy, case.eps0, threads)
            times.append(t)
        t_med = statistics.median(times)
        # one thread: one full solve, measured
        t1, r1 = cpu_reference_solve(ora, sy, case.eps0, 1)
        cpu = {"value": 1.0 / t_med, "unit": "solves/s", "cores": threads, "kind": "port",
               "cpu_model": cpu_model(),
               "sample": f"median of 10 full solves of {args.workload} (N={sy.mnoe}, {r.iters} iterations) after 3 "
                         f"warm-ups, OpenMP restatement of pcgpme_para.F90 on {threads} threads "
                         f"(min {min(times):.3f} s, max {max(times):.3f} s)",
               "port_parity": PORT_PARITY,
               "one_thread": {"value": 1.0 / t1, "unit": "solves/s", "iters": r1.iters,
                              "sample": f"one full solve on 1 thread, measured ({t1:.1f} s)"}}
        nrm = np.linalg.norm(r.x)
        err_plain = float(np.linalg.norm(x_plain - r.x) / nrm)
        if x_mixed is not None:
            err_mixed = float(np.linalg.norm(x_mixed - r.x) / nrm)

    if rank == 0:
        line = {
            "metric": "pressure solves/s", "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": args.workload, "rows": n, "tol": case.eps0, "iters": it,
                       "stop": pkg.STOP_NAMES.get(info.reason), "eps": info.eps,
                       "rel_l2_vs_oracle": err_plain, "true_rel_residual": args.res_plain,
                       "l2": "inputs larger than L2 (matrix %.0f MB)" % (n * 80 / 1e6),
                       "path": "plain FP64", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "kernel": "pcgpme FP64 solve (one graph launch)",
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": TRAFFIC_ROW_ITER_FP64 * n * it,
                         "traffic_source": "ncu DRAM bytes of the loop graph per row-iteration, "
                                           "profiles/pcgpme_loop_dram_beach_256x256x96.md",
                         "frac_with_index_streams": bytes_solve_fp64_with_indices(n, it) / alg * achieved / peak,
                         "algorithmic_bytes_per_solve": alg},
            "roofline_fp64": {"bound": "fp64", "kernel": "pcgpme FP64 solve (one graph launch)",
                              "achieved": args.fma_achieved / 1e9, "peak": args.fma_peak / 1e9,
                              "peak_kind": "measured (clowns_fp64_fma_rate, this run)", "unit": "G FMA/s",
                              "frac": args.fma_achieved / args.fma_peak,
                              "fma_per_row_iter": FMA_ROW_ITER_FP64},
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": args.timed_launches,
            "tuned_shape": {"fp64": pkg.tuned_shape([n], 0), "mixed": pkg.tuned_shape([n], 1)},
            "clocks": clk,
        }
        if minfo is not None:
            line["mixed"] = {"value": m_value, "unit": "solves/s", "speedup_vs_fp64": m_value / value,
                             "inner_iters": minfo.iter, "outer": minfo.outer, "eps": minfo.eps,
                             "rel_l2_vs_oracle": err_mixed, "true_rel_residual": args.res_mixed,
                             "ms_per_solve": ms_m / args.steps,
                             "achieved_gbs": m_alg / (ms_m / 1000.0 / args.steps) / 1e9,
                             "traffic": TRAFFIC_ROW_ITER_MIXED * n * minfo.iter,
                             "algorithmic_bytes_per_solve": m_alg}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--legs", default="plain,mixed,e2e,cpu",
                    help="measurement legs to run (the plain FP64 leg always runs)")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="inner (FP32) tolerance of the mixed path; 0 = library default")
    ap.add_argument("--ensemble", action="store_true", help="batched ensemble measurement instead")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--member-scale", type=float, default=1.0)
    ap.add_argument("--adjoint", action="store_true", help="adjoint vs finite differences instead")
    ap.add_argument("--will", action="store_true", help="PCGPME_WILL (2DH dispersion solve) instead")
    ap.add_argument("--session", action="store_true", help="the whole ik loop on the device instead")
    ap.add_argument("--ingest", action="store_true", help="case files to converged pressure instead")
    ap.add_argument("--will-grid", default="1600x1200", help="2DH plan grid of the --will leg")
    ap.add_argument("--faces", type=int, default=200)
    ap.add_argument("--workload", default=WORKLOAD,
                    help="beach_256x256x96 (default), beach_512x384x128, beach_192x192x64, "
                         "tank_64x64x32 or beach_NXxNYxNZ")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.ensemble:
        import torch
        torch.cuda.set_device(local)
        run_ensemble(args)
        return
    if args.adjoint:
        import torch
        torch.cuda.set_device(local)
        run_adjoint(args)
        return
    if args.will:
        import torch
        torch.cuda.set_device(local)
        run_will(args)
        return
    if args.session:
        import torch
        torch.cuda.set_device(local)
        run_session(args)
        return
    if args.ingest:
        import torch
        torch.cuda.set_device(local)
        run_ingest(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
