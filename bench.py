"""Benchmark: DOF/s assembled + solved to 1e-8 FP64 relative residual on one GB300.

Workload: 3-D lognormal diffusion, 128^3 Q1 hexahedra (2,048,383 free dofs), kappa a seeded
lognormal Gaussian random field (correlation length 8h, contrast 1e4), f ~ N(0,1) per node,
homogeneous Dirichlet on the boundary. One step = what AffineFEOperator + solve do:
symbolic assembly (pattern on the device), numeric assembly of A and b (FP64), and the
linear solve to ||b - A x|| <= 1e-8 ||b|| (FP64 residual).

  value (headline arm)  mixed precision: FP32 Jacobi-PCG with FP64 reliable updates (x and
                        the true residual in FP64), inputs resident in HBM;
  plain_fp64            FP64 assembly + FP64 Jacobi-PCG, same inputs (the plain FP64 base path);
  e2e                   the headline arm through the C ABI with pinned host buffers:
                        cell ids, kappa and f copied in, x copied out, every step.

`--impl reference` times the oracle (the CPU restatement of Gridap's algorithm) on the host
cores on a bounded sample of the same workload.

Multi-GPU: the path does not shard (one problem per GPU); N>1 runs N independent replicas
and reports the DOF of all replicas over the slowest replica's time.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import os
import pathlib
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DOF/s assembled+solved to 1e-8 rel. residual: mixed/learned vs plain FP64, 1 GB300"
UNIT = "DOF/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_step_ms(ms: float, device) -> float:
    """Step time of a replicas-only run: every rank solves its own problem, the slowest rank
    sets the time (max over ranks). No other data crosses ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(nfree_per_rank: int, world: int, step_ms: float) -> float:
    """Whole-job DOF/s: all ranks' free dofs over the max-over-ranks step time."""
    return world * nfree_per_rank / (step_ms * 1e-3)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons (every 50 ms) around the timed regions;
    `window()` marks a timed region and the summary keeps only samples taken inside one."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []      # (host time, fields)
        self.windows = []   # (t0, t1) of the timed regions
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0:  # sampler running
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def window(self):
        sampler = self

        class _W:
            def __enter__(self):
                self.t0 = time.perf_counter()

            def __exit__(self, *a):
                sampler.windows.append((self.t0, time.perf_counter()))
        return _W()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = [r for t, r in self.rows
                if not self.windows or any(a <= t <= b for a, b in self.windows)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows), "period_ms": 50}


def mg_levels(n):
    """Cell counts per direction of the multigrid levels (halved while even and >= 8)."""
    lv = [n]
    while lv[-1] % 2 == 0 and lv[-1] >= 8:
        lv.append(lv[-1] // 2)
    return lv


def vcycle_bytes(n):
    """Algorithmic bytes of one V-cycle (FP32): per level with R rows, C cells and Rc coarse
    rows, the first sweep (b, D read, x written: 12 R), three fused sweeps (kappa 4 C; x, b,
    D read and x written 16 R each), the fused residual (kappa 4 C; x, b read, r written
    12 R), restriction (r read 4 R, 4 Rc written) and prolongation (4 Rc and x read, x
    written 8 R): 16 C + 84 R + 8 Rc per level; the coarsest level the first sweep and four
    fused ones."""
    lv = mg_levels(n)
    tot = 0
    for i, m in enumerate(lv):
        R, C = (m - 1) ** 3, m ** 3
        if i + 1 < len(lv):
            tot += 16 * C + 84 * R + 8 * (lv[i + 1] - 1) ** 3
        else:
            tot += 12 * R + 4 * (4 * C + 16 * R)
    return tot


def assembly_bytes(nnz, n, ncells, nnodes):
    """Class-sum numeric assembly of Cartesian Q1 diffusion: kappa (8 B per cell) and the
    nodal source (8 B per node) read, every stored value and b written (8 B)."""
    return ncells * 8 + nnodes * 8 + nnz * 8 + n * 8


def spmv_bytes(nnz, n, s):
    """Algorithmic bytes of one CSR SpMV: values + column ids + row pointers + x + y."""
    return nnz * (s + 4) + (n + 1) * 4 + n * 2 * s


def profile_traffic(kind: str):
    """Per-launch DRAM traffic of a kernel at the bench workload, from the committed ncu
    summaries under profiles/ (a line `traffic_bytes_per_launch_<kind>: <bytes>`)."""
    for p in sorted((ROOT / "profiles").glob("*.md")):
        m = re.search(rf"traffic_bytes_per_launch_{kind}:\s*([0-9.eE+]+)", p.read_text())
        if m:
            return float(m.group(1))
    return None


def workload_config(n, nfree, ncells, nnz, rtol, world):
    """The workload both arms report (identical keys and values for the same problem)."""
    return {"workload": f"lognormal_3d {n}^3 Q1 diffusion", "free_dofs": int(nfree),
            "cells": int(ncells), "nnz": int(nnz), "rtol": rtol,
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (matrix %.2f GB)" % (nnz * 12 / 1e9)}


def load_synthetic():
    """The numpy-only input generator (gridap.jl_gb300/synthetic.py), loaded by path so that
    the CPU arm never imports the package (and never maps the CUDA library)."""
    import importlib.util
    if "gfe_synthetic" in sys.modules:
        return sys.modules["gfe_synthetic"]
    spec = importlib.util.spec_from_file_location(
        "gfe_synthetic", ROOT / "gridap.jl_gb300" / "synthetic.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gfe_synthetic"] = mod
    spec.loader.exec_module(mod)
    return mod


def export_csr(lib, h, base):
    """(rowptr, colval, nzval) of a device matrix as int64/int64/float64 host arrays."""
    import ctypes
    from gridap_gb300 import _lib
    nr, nnz = ctypes.c_int64(), ctypes.c_int64()
    lib.gfe_matrix_info(h, ctypes.byref(nr), None, ctypes.byref(nnz))
    rp = np.empty(nr.value + 1, np.int64)
    cv = np.empty(nnz.value, np.int64)
    nz = np.empty(nnz.value)
    _lib.check(lib.gfe_matrix_export_csr(h, base, _lib.ptr(rp), _lib.ptr(cv), _lib.ptr(nz)))
    return rp, cv, nz


def csr_parity(csr, csc, b=None, b_ref=None):
    """Device CSR (1-based) against the oracle's CSC (1-based; equal arrays for these
    symmetric matrices): pattern bit-exact, values |a - a_ref| / max|row of a_ref|, vector
    max |b - b_ref| / max |b_ref|."""
    rp, cv, nz = csr
    cp, rv, zv = csc
    same = bool(np.array_equal(rp, cp) and np.array_equal(cv, rv))
    out = {"pattern_bit_exact": same, "nnz": int(zv.shape[0]), "nnz_device": int(nz.shape[0])}
    if same:
        lens = np.diff(cp)
        nonempty = lens > 0
        rowmax = np.zeros(lens.shape[0])
        rowmax[nonempty] = np.maximum.reduceat(np.abs(zv), (cp[:-1] - 1)[nonempty])
        scale = np.repeat(np.maximum(rowmax, 1e-300), lens)
        out["matrix_max_rowscaled_err"] = float(np.max(np.abs(nz - zv) / scale))
        out["matrix_bit_exact_fraction"] = float(np.mean(nz == zv))
    if b is not None:
        out["vector_max_rel_err"] = float(np.abs(b - b_ref).max() / np.abs(b_ref).max())
    return out


def solution_parity(orc, csc, b_ref, x, x_ref=None):
    """FP64 relative residual of a device solution in the oracle's system, and its distance
    to the oracle's own solution."""
    r = b_ref - orc.csc_mul(*csc, x)
    out = {"relres_in_oracle_system": float(np.linalg.norm(r) / np.linalg.norm(b_ref))}
    if x_ref is not None:
        out["rel_l2_vs_oracle_solution"] = float(np.linalg.norm(x - x_ref) /
                                                 np.linalg.norm(x_ref))
    return out


def headline_parity(args, kept, ref):
    """The headline step's assembled matrix, vector and solutions against the oracle on the
    same inputs at full size (the CPU baseline's arrays when it ran)."""
    from oracle import oracle as orc
    if ref is None:
        syn = load_synthetic()
        kappa, f = syn.lognormal_inputs(args.n)
        with orc.cell_threads(os.cpu_count() or 1):
            r = orc.poisson_q1((0, 1, 0, 1, 0, 1), (args.n,) * 3, ("boundary",), kappa=kappa,
                               fkind=orc.F_NODAL, fdata=f)
        ref = {"csc": r["csc"], "b": r["b"], "x": None, "relres": None}
    out = {"oracle": "CPU restatement of Gridap's assembly (serial InserterCSC loop in cell "
                     "order) and Jacobi-PCG, same seeded inputs, full size",
           "tolerance": {"pattern": "bit-exact", "matrix": 1e-12, "vector": 1e-12,
                         "solution_relres": 1e-8}}
    out.update(csr_parity(kept["csr"], ref["csc"], kept["b"], ref["b"]))
    out["solution"] = solution_parity(orc, ref["csc"], ref["b"], kept["x"], ref.get("x"))
    out["solution_plain_fp64"] = solution_parity(orc, ref["csc"], ref["b"], kept["x_plain"],
                                                 ref.get("x"))
    if ref.get("relres") is not None:
        out["oracle_pcg_relres"] = ref["relres"]
    out["pass"] = bool(out["pattern_bit_exact"] and out["matrix_max_rowscaled_err"] <= 1e-12
                       and out["vector_max_rel_err"] <= 1e-12
                       and out["solution"]["relres_in_oracle_system"] <= 1e-8 * (1 + 1e-3))
    return out


# ---- GPU arm ------------------------------------------------------------------------------
def run_gpu(args):
    import ctypes

    import torch

    import __graft_entry__ as ge
    gg = ge.load_package()
    from gridap_gb300 import _lib, workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    ctx = gg.Context(local)
    lib = _lib.load()
    dev = torch.device("cuda", local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)

    w = workloads.lognormal_3d(n=args.n)
    V = w.space
    nfree = V.num_free_dofs()
    ids_h = V.cell_dof_ids
    ncells, nd = ids_h.shape
    # device-resident inputs
    ids_d = torch.from_numpy(ids_h).to(dev)
    kap_d = torch.from_numpy(w.kappa).to(dev)
    f_d = torch.from_numpy(w.source.values).to(dev)
    b_d = torch.zeros(nfree, dtype=torch.float64, device=dev)
    x_d = torch.zeros(nfree, dtype=torch.float64, device=dev)
    # pinned host inputs for the end-to-end arm
    ids_p = torch.from_numpy(ids_h).pin_memory()
    kap_p = torch.from_numpy(w.kappa).pin_memory()
    f_p = torch.from_numpy(w.source.values).pin_memory()
    x_p = torch.zeros(nfree, dtype=torch.float64).pin_memory()
    b_scratch = torch.zeros(nfree, dtype=torch.float64, device=dev)

    def problem(ids, kap, f):
        prep = gg.prepare_problem(V, V, w.measure, gg.CellField(kap), gg.NodalField(f),
                                  cell_dof_ids=ids)
        return prep

    def step(ids, kap, f, x, solver, b, keep=None):
        prep = problem(ids, kap, f)
        h = ctypes.c_void_p()
        # the symbolic loop with the model in hand, as SparseMatrixAssembler(U, V) runs it
        _lib.check(lib.gfe_symbolic_loop_matrix_problem(ctx.handle, ctypes.byref(prep.p),
                                                        ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(ctx.handle, ctypes.byref(prep.p), h,
                                                          _lib.ptr(b)))
            o = solver.opts()
            rep = _lib.SolveReport()
            if isinstance(solver, gg.FCGSolver):
                _lib.check(lib.gfe_solve_fcg(ctx.handle, h,
                                             solver.pc.handle if solver.pc is not None else None,
                                             ctypes.byref(o), _lib.ptr(b), _lib.ptr(x),
                                             ctypes.byref(rep)))
            else:
                _lib.check(lib.gfe_solve(ctx.handle, h, ctypes.byref(o), _lib.ptr(b),
                                         _lib.ptr(x), ctypes.byref(rep)))
            if keep is not None:  # the assembled system and solution, for the oracle parity
                keep["csr"] = export_csr(lib, h, 1)
                keep["b"] = b.cpu().numpy().copy()
                keep["x"] = x.cpu().numpy().copy()
        finally:
            lib.gfe_matrix_destroy(h)
        return rep

    # headline: flexible CG (FP32, FP64 reliable updates) with the multigrid V-cycle; the
    # Jacobi mixed CG of the same precision scheme and the plain FP64 CG are measured beside
    mixed_cg = gg.MixedCGSolver(rtol=w.rtol, inner_rtol=args.delta)
    mixed = gg.FCGSolver(rtol=w.rtol, pc="mg") if args.solver == "mg" else mixed_cg
    plain = gg.CGSolver(rtol=w.rtol)

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = []  # the clock sampler while the headline arms run

    def timed(label, fn, steps, warmup, kernel_timing=True):
        for _ in range(warmup):
            fn()
        barrier()
        ctx.set_timing(kernel_timing)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = ctx.kernel_launches()
        reps = []
        with clocks[0].window() if clocks else contextlib.nullcontext():
            with torch.cuda.stream(stream):
                e0.record(stream)
            t0 = time.perf_counter()
            for _ in range(steps):
                reps.append(fn())
            with torch.cuda.stream(stream):
                e1.record(stream)
            barrier()
            wall = time.perf_counter() - t0
        kt = {k: ctx.kernel_time(k) for k in (_lib.GFE_KT_SPMV64, _lib.GFE_KT_SPMV32,
                                              _lib.GFE_KT_ASSEMBLE, _lib.GFE_KT_RESIDUAL64,
                                              _lib.GFE_KT_PRECOND, _lib.GFE_KT_VECTOR,
                                              _lib.GFE_KT_ELEMENT)}
        ctx.set_timing(False)
        ms = e0.elapsed_time(e1) / steps
        if world > 1:
            ms = replica_step_ms(ms, dev)
        return dict(ms=ms, wall_ms=1e3 * wall / steps, reps=reps, kt=kt,
                    launches=ctx.kernel_launches() - l0)

    mixed_dev = lambda: step(ids_d, kap_d, f_d, x_d, mixed, b_d)  # noqa: E731
    plain_dev = lambda: step(ids_d, kap_d, f_d, x_d, plain, b_d)  # noqa: E731

    def mixed_e2e():
        rep = step(ids_p, kap_p, f_p, x_p, mixed, b_scratch)
        return rep

    # The headline steps run as a user runs them: CG iteration chunks replayed from CUDA
    # graphs. Kernel durations need CUDA events around each SpMV, which the library records
    # only on its direct-launch path, so the same steps are then repeated with kernel timing
    # on; the roofline comes from that instrumented repeat (its ms_per_step is reported too).
    if args.profile:
        # the headline steps alone, for a profiler's launch list (no JSON line: a number taken
        # under a profiler is not a measurement). Kernel timing is on, so that the solver
        # launches its iterations from the host: kernels inside the device-driven loop (a
        # graph with a conditional node) are invisible to a per-kernel profiler.
        ctx.set_timing(True)
        for _ in range(args.warmup + args.steps):
            mixed_dev()
        barrier()
        if rank == 0:
            print(f"profile run: {args.warmup + args.steps} headline steps")
        return
    with ClockSampler(local) as clk:
        clocks.append(clk)
        r_mixed = timed("mixed", mixed_dev, args.steps, args.warmup, kernel_timing=False)
        r_mixed_kt = timed("mixed_kt", mixed_dev, args.steps, 1)
        r_plain = timed("plain", plain_dev, args.steps, max(3, args.warmup),
                        kernel_timing=False)
        r_plain_kt = timed("plain_kt", plain_dev, args.steps, 1)
        x_plain = x_d.clone()
        mixed_dev()
        x_mixed = x_d.clone()
        err_vs_fp64 = float(torch.linalg.norm(x_mixed - x_plain) / torch.linalg.norm(x_plain))
        kept = {}
        if not args.no_parity and rank == 0:
            step(ids_d, kap_d, f_d, x_d, mixed, b_d, keep=kept)
            kept["x_plain"] = x_plain.cpu().numpy()
        r_e2e = timed("e2e", mixed_e2e, args.steps, max(3, args.warmup), kernel_timing=False)
        r_mcg = (timed("mixed_cg", lambda: step(ids_d, kap_d, f_d, x_d, mixed_cg, b_d),
                       args.steps, 3, kernel_timing=False) if mixed is not mixed_cg else r_mixed)
        clocks.clear()

    # learned arm: FCG with the learned block preconditioner (weights trained offline on
    # 64^3 draws), and FCG with Jacobi on the same vectors for comparison
    learned_out = None
    from gridap_gb300 import learned as learned_mod
    if learned_mod.WEIGHTS_FILE.exists() and not args.no_learned:
        # the learned preconditioner (weights trained offline on residual / error pairs of FP64
        # solves of 64^3 draws): as the fine-level smoother of the V-cycle (the learned arm),
        # alone, and beside them FCG with Jacobi and with the Jacobi-smoothed V-cycle; every
        # arm is the same step as the headline (pattern, FP64 assembly, solve to 1e-8)
        pc = learned_mod.LearnedBlockPreconditioner(V, w.kappa, ctx)
        pc.load_default_weights()
        arms = {"learned_mg": gg.FCGSolver(rtol=w.rtol, pc=pc, multigrid=True),
                "learned_alone": gg.FCGSolver(rtol=w.rtol, pc=pc),
                "fcg_jacobi": gg.FCGSolver(rtol=w.rtol, pc=None),
                "fcg_multigrid": gg.FCGSolver(rtol=w.rtol, pc="mg")}
        res = {}
        for name, solver in arms.items():
            r = timed(name, lambda: step(ids_d, kap_d, f_d, x_d, solver, b_d), args.steps, 3,
                      kernel_timing=False)
            rep = r["reps"][-1]
            res[name] = {"value": world * nfree / (r["ms"] * 1e-3), "ms_per_step": r["ms"],
                         "iterations": rep.iterations, "relres": rep.relres,
                         "fallback_to_jacobi": bool(rep.fallback)}
        r_kt = timed("learned_mg_kt", lambda: step(ids_d, kap_d, f_d, x_d, arms["learned_mg"],
                                                    b_d), 1, 1)
        lm = res["learned_mg"]
        learned_out = dict(lm)
        learned_out.update({
            "solver": "flexible CG (FP32 inner, FP64 reliable updates) preconditioned by the "
                      "multigrid V-cycle whose fine-level smoother is the learned block MLP "
                      "(BF16 on tcgen05): pre x = M(b), post x += M(b - A x); coarser levels "
                      "damped Jacobi; Jacobi-PCG fallback on stagnation",
            "precond_ms_per_apply": (r_kt["kt"][_lib.GFE_KT_PRECOND][0] /
                                     max(r_kt["kt"][_lib.GFE_KT_PRECOND][1], 1)),
            "learned_alone": res["learned_alone"], "fcg_jacobi": res["fcg_jacobi"],
            "fcg_multigrid": dict(res["fcg_multigrid"], preconditioner=(
                "geometric multigrid V-cycle on the lattice operator (FP32, 2+2 damped Jacobi "
                "sweeps)")),
            "training": "residual / error pairs (r_k = b - A x_k, e_k = x* - x_k) of FP64 CG "
                        "iterates from x* + white noise (k = 0, 1, 2, 4), x* the FP64 solution, "
                        "on 200 independent 64^3 kappa draws (seeds 5000..5199)"})

    # dominant kernel: the CG SpMV, timed with CUDA events inside the timed regions
    def avg_ms(r, k):
        tot, n = r["kt"][k]
        return tot / n if n else float("nan")
    nnz_c = ctypes.c_int64()
    hA = ctypes.c_void_p()
    _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                            _lib.ptr(ids_d), nfree, nfree, ctypes.byref(hA)))
    lib.gfe_matrix_info(hA, None, None, ctypes.byref(nnz_c))
    lib.gfe_matrix_destroy(hA)
    prof = {"nnz": nnz_c.value, "fp32_ms": avg_ms(r_mixed_kt, _lib.GFE_KT_SPMV32),
            "fp64_ms": avg_ms(r_plain_kt, _lib.GFE_KT_SPMV64),
            "fp32_launches": r_mixed_kt["kt"][_lib.GFE_KT_SPMV32][1],
            "assemble_ms": avg_ms(r_plain_kt, _lib.GFE_KT_ASSEMBLE)}

    rep_m, rep_p = r_mixed["reps"][-1], r_plain["reps"][-1]
    for rp in r_mixed["reps"] + r_plain["reps"] + r_e2e["reps"] + r_mcg["reps"]:
        if not rp.relres <= w.rtol * (1 + 1e-6):
            raise RuntimeError(f"solve did not reach rtol: relres={rp.relres}")
    value = replica_value(nfree, world, r_mixed["ms"])
    plain_value = replica_value(nfree, world, r_plain["ms"])
    e2e_value = replica_value(nfree, world, r_e2e["ms"])
    h2d = ids_h.nbytes + w.kappa.nbytes + w.source.values.nbytes
    d2h = nfree * 8
    peak, peak_kind = peaks()
    nnz = prof["nnz"]
    fmt = rep_m.operator_format
    # algorithmic bytes of one launch of each timed kernel class (FP32 inner iteration)
    #   matrix-free lattice SpMV: kappa per cell + p read + q written
    #   diagonal format: values + p + q (no column ids); sliced ELL: the CSR formula
    #   vector updates (update + direction): x, r, p, q, dinv read + x, r written, then
    #   p, r, dinv read + p written = 44 B per row
    if fmt == 2:
        alg, kname = ncells * 4 + nfree * 8, ("k_cg_spmv_dot<float, LatticeQ1Op> (matrix-free "
                                              "FP32 Q1 operator + p.q)")
    elif fmt == 1:
        alg, kname = nnz * 4 + nfree * 8, (f"k_cg_spmv_dot<float, DiaOp<float>> (diagonal "
                                           f"format, {rep_m.ndiag} diagonals, + p.q)")
    else:
        alg, kname = spmv_bytes(nnz, nfree, 4), "k_cg_spmv_dot<float, SellOp<float>>"
    kinds = {
        "spmv32": dict(kernel=kname, alg=alg, kt=r_mixed_kt["kt"][_lib.GFE_KT_SPMV32],
                       traffic=profile_traffic({2: "fp32_lattice", 1: "fp32_dia"}.get(
                           fmt, "fp32_sell"))),
        "vector32": dict(kernel="k_cg_update4 + k_cg_direction4 (FP32 CG vector updates)",
                         alg=44 * nfree, kt=r_mixed_kt["kt"][_lib.GFE_KT_VECTOR],
                         traffic=profile_traffic("fp32_vector")),
        "assembly": dict(kernel="k_assemble_cart_q1 (class-sum numeric assembly, FP64; "
                                "FP64-pipe bound)",
                         alg=assembly_bytes(nnz, nfree, ncells, (args.n + 1) ** 3),
                         traffic=profile_traffic("assembly"),
                         kt=r_mixed_kt["kt"][_lib.GFE_KT_ASSEMBLE]),
    }
    if isinstance(mixed, gg.FCGSolver):
        # FCG on the lattice multigrid: the SpMV applies the operator to z and folds in the
        # direction update (kappa per cell, z read; p, q read and written; r read: 4 C + 24 R),
        # the update kernel moves x, r, p, q (x, r, p, q read, x, r written: 24 R), and the
        # V-cycle, one graph launch timed as a whole, also reads q in its last sweep (the beta
        # dot: 4 R)
        kinds["spmv32"].update(kernel="k_lattice_spmv_dir (matrix-free FP32 Q1 operator on z; "
                                      "p = z + beta p, q = A z + beta q; p.q, p.r)",
                               alg=ncells * 4 + nfree * 24,
                               traffic=profile_traffic("fp32_lattice_dir"))
        kinds["vector32"].update(kernel="k_fcg_update4 (x += a p, r -= a q, r.r)",
                                 alg=24 * nfree, traffic=None)
        kinds["vcycle"] = dict(kernel="multigrid V-cycle (CUDA graph over %d levels: "
                                      "k_mg_jacobi0, k_mg_smooth, k_mg_pre, k_mg_residual, "
                                      "k_mg_restrict, k_mg_prolong, k_mg_coarse; the last "
                                      "sweep k_mg_smooth_dot forms the FCG beta)"
                                      % len(mg_levels(args.n)),
                               alg=vcycle_bytes(args.n) + 4 * nfree,
                               traffic=profile_traffic("vcycle"),
                               kt=r_mixed_kt["kt"][_lib.GFE_KT_PRECOND])
    table = {}
    for k, d in kinds.items():
        tot, cnt = d["kt"]
        ms_avg = tot / cnt if cnt else float("nan")
        ach = d["alg"] / (ms_avg * 1e-3) / 1e9 if cnt else float("nan")
        table[k] = {"kernel": d["kernel"], "algorithmic_bytes_per_launch": d["alg"],
                    "avg_launch_ms": ms_avg, "launches_timed": cnt, "achieved": ach,
                    "frac": ach / peak, "traffic": d["traffic"],
                    "share_of_step_time": tot / (r_mixed_kt["ms"] * args.steps)}
    dom = max(table, key=lambda k: table[k]["share_of_step_time"])
    alg64 = spmv_bytes(nnz, nfree, 8)
    achieved64 = alg64 / (prof["fp64_ms"] * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r_mixed["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-refinement",
        "data": "synthetic (seeded lognormal GRF kappa, N(0,1) nodal f)",
        "config": workload_config(args.n, nfree, ncells, nnz, w.rtol, world),
        "method": {"solver": (f"flexible CG, FP32 vectors with FP64 reliable updates, "
                              f"preconditioned by a geometric multigrid V-cycle on the "
                              f"matrix-free lattice operator ({len(mg_levels(args.n))} levels, "
                              f"2+2 damped Jacobi sweeps); FP64 x and true residual"
                              if isinstance(mixed, gg.FCGSolver) else
                              f"mixed CG: FP32 Jacobi-PCG with FP64 reliable updates "
                              f"(delta {args.delta}), FP64 x and true residual; inner "
                              f"operator {rep_m.operator_format}"),
                   "assembly": "FP64 class-sum assembly into the closed-form Cartesian "
                               "CSR pattern"},
        "iterations": {"mixed": rep_m.iterations, "mixed_reliable_updates": rep_m.refinements,
                       "plain_fp64": rep_p.iterations},
        "plain_fp64": {"value": plain_value, "ms_per_step": r_plain["ms"],
                       "solver": "FP64 Jacobi-PCG", "relres": rep_p.relres},
        "mixed_over_plain": value / plain_value,
        "mixed_cg_jacobi": {"value": replica_value(nfree, world, r_mcg["ms"]),
                            "ms_per_step": r_mcg["ms"],
                            "iterations": r_mcg["reps"][-1].iterations,
                            "relres": r_mcg["reps"][-1].relres,
                            "solver": f"FP32 Jacobi-PCG with FP64 reliable updates (delta "
                                      f"{args.delta}) on the matrix-free lattice operator"},
        "error_vs_fp64": {"rel_l2_solution_vs_plain_fp64_gpu": err_vs_fp64,
                          "relres_mixed": rep_m.relres,
                          "vs_fp64_oracle": "parity.solution (the oracle's FP64 system)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": r_e2e["ms"]},
        "roofline": {"bound": "hbm", "achieved": table[dom]["achieved"], "peak": peak,
                     "unit": "GB/s", "frac": table[dom]["frac"],
                     "traffic": table[dom]["traffic"], "kernel": table[dom]["kernel"],
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": table[dom]["algorithmic_bytes_per_launch"],
                     "avg_launch_ms": table[dom]["avg_launch_ms"],
                     "launches_timed": table[dom]["launches_timed"],
                     "share_of_step_time": table[dom]["share_of_step_time"],
                     "timed_in": "instrumented repeat of the timed steps (CUDA events around "
                                 "each launch on the library's stream), "
                                 f"{r_mixed_kt['ms']:.2f} ms/step",
                     "kernels": table,
                     "fp64_spmv": {"kernel": "k_cg_spmv_dot<double, SellOp<double>> (plain path)",
                                   "achieved": achieved64, "frac": achieved64 / peak,
                                   "algorithmic_bytes_per_launch": alg64,
                                   "avg_launch_ms": prof["fp64_ms"],
                                   "traffic": profile_traffic("fp64_sell")}},
        "assembly": {"class_sum_ms": prof["assemble_ms"]},
        "learned_fcg": (dict(learned_out, over_plain_fp64=learned_out["value"] / plain_value)
                        if learned_out else None),
        "gpu_launches": r_mixed["launches"],
        "clocks": clk.summary(),
    }
    if "vcycle" in table:
        # the V-cycle's vectors and kappa stay in L2 between its kernels: its bound is L2
        # latency and launch overhead, its L2 traffic the relevant byte count
        m = re.search(r"l2_bytes_per_launch_vcycle:\s*([0-9.eE+]+)",
                      "".join(p.read_text() for p in sorted((ROOT / "profiles").glob("*.md"))))
        l2b = float(m.group(1)) if m else None
        vc = table["vcycle"]
        out["roofline"]["vcycle_l2"] = {
            "l2_bytes_per_launch": l2b,
            "l2_gbs": l2b / (vc["avg_launch_ms"] * 1e-3) / 1e9 if l2b else None,
            "note": "L2-resident (8.2 MB vectors at 128^3); DRAM traffic per cycle is the "
                    "cold-cache ncu figure; bound by L2 latency and launch overhead"}
    if not args.no_batch:
        out["batched"] = bench_batched(args, gg, ctx, lib, barrier)
    if not args.no_elasticity:
        out["elasticity_p2"] = bench_elasticity(args, gg, ctx, lib, timed)
    if not args.no_q2:
        out["q2_tensor_cores"] = bench_q2(args, gg, ctx, lib, timed)
    if not args.no_poisson2d:
        out["poisson_2d"] = bench_poisson2d(args, gg, ctx, lib, timed)
    if not args.no_nonlinear:
        out["nonlinear_plaplacian"] = bench_nonlinear(args, gg, ctx, lib, timed)
    if not args.no_reordering:
        out["reordering_rcm"] = bench_reordering(args, gg, ctx, lib, timed)
    if not args.no_multifield:
        out["multifield_stokes"] = bench_multifield(args, gg, ctx, lib, timed)
    if rank == 0:
        ref = None
        if not args.no_cpu_baseline:
            out["cpu_baseline"], ref = cpu_baseline(args, keep=not args.no_parity)
        if not args.no_parity:
            out["parity"] = headline_parity(args, kept, ref)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---- batched problems ----------------------------------------------------------------------
def bench_batched(args, gg, ctx, lib, barrier):
    """256 independent diffusion problems div(kappa grad u) = 1 on unit cubes with n^3 cells,
    n uniform in 16..64, per-cell lognormal kappa (sigma 1.5), u = 0 on the boundary: one
    batched assemble+solve call (one persistent launch: matrix-free FP32 Jacobi-PCG per problem
    with FP64 reliable updates, autotuned launch shape) against the same problems solved one
    after the other through the single-problem path (symbolic + numeric assembly + FP64
    Jacobi-PCG per problem)."""
    import ctypes
    import torch
    from gridap_gb300 import _lib, workloads
    sizes, kappas = workloads.batched_diffusion(args.batch_problems)
    rtol = 1e-8
    B = gg.BatchedPoissonProblems(sizes, kappas, ctx)
    dev = torch.device("cuda", ctx.device)
    xb = torch.empty(B.nfree, dtype=torch.float64, device=dev)
    for _ in range(2):
        B.assemble_solve(1.0, rtol, 0, xb)
    barrier()
    steps = 3
    t0 = time.perf_counter()
    l0 = ctx.kernel_launches()
    for _ in range(steps):
        B.assemble_solve(1.0, rtol, 0, xb)
    barrier()
    t_batch = (time.perf_counter() - t0) / steps
    launches = (ctx.kernel_launches() - l0) // steps
    it_b = B.iterations.copy()
    assert B.nconverged == len(sizes)
    # sequential: the single-problem path, one problem after the other
    one = np.ones(1)
    seq = []
    for n, k in zip(sizes, kappas):
        ids = torch.from_numpy(workloads.box_cell_dofs(n)).to(dev)
        kd = torch.from_numpy(np.ascontiguousarray(k, np.float64)).to(dev)
        nf = (n - 1) ** 3
        seq.append((n, ids, kd, nf, torch.zeros(nf, dtype=torch.float64, device=dev),
                    torch.zeros(nf, dtype=torch.float64, device=dev)))
    o = gg.CGSolver(rtol=rtol).opts()

    def solve_one(n, ids, kd, nf, b, x):
        p = _lib.Problem()
        p.dim, p.reffe, p.ncomp, p.degree = 3, 1, 1, 2
        p.ncells, p.nd, p.cell_dof_ids, p.nfree = n ** 3, 8, _lib.ptr(ids), nf
        p.geometry = _lib.GFE_GEOM_CARTESIAN
        for d in range(3):
            p.partition[d] = n
            p.domain[2 * d], p.domain[2 * d + 1] = 0.0, 1.0
        p.form = _lib.GFE_FORM_DIFFUSION
        p.coef_kind, p.coef = _lib.GFE_COEF_CELL, _lib.ptr(kd)
        p.source_kind, p.source, p.source_len = _lib.GFE_SRC_CONST, _lib.ptr(one), 1
        p.precision = _lib.GFE_PREC_FP64
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, n ** 3, 8, _lib.ptr(ids),
                                                _lib.ptr(ids), nf, nf, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(ctx.handle, ctypes.byref(p), h,
                                                          _lib.ptr(b)))
            rep = _lib.SolveReport()
            _lib.check(lib.gfe_solve(ctx.handle, h, ctypes.byref(o), _lib.ptr(b), _lib.ptr(x),
                                     ctypes.byref(rep)))
        finally:
            lib.gfe_matrix_destroy(h)
        return rep.iterations

    for s in seq[:4]:
        solve_one(*s)
    barrier()
    t0 = time.perf_counter()
    it_s = [solve_one(*s) for s in seq]
    barrier()
    t_seq = time.perf_counter() - t0
    # same answers: the batched solution of every problem against its sequential one
    xs = B.split(xb.cpu().numpy())
    err = max(float(np.linalg.norm(xs[i] - seq[i][5].cpu().numpy()) /
                    np.linalg.norm(seq[i][5].cpu().numpy())) for i in range(len(seq)))
    dofs = B.nfree
    return {"problems": len(sizes), "free_dofs": dofs, "cells": B.ncells,
            "sizes": "n^3 cells, n uniform in 16..64 (seeded)", "rtol": rtol,
            "ms_per_step": 1e3 * t_batch, "problems_per_s": len(sizes) / t_batch,
            "dof_per_s": dofs / t_batch, "gpu_launches_per_step": launches,
            "launch_shape": {"threads_per_cta": B.shape()[0], "ctas_per_cluster": B.shape()[1],
                             "cluster_threshold": B.shape()[2]},
            "max_iterations": int(it_b.max()), "mean_iterations": float(it_b.mean()),
            "sequential": {"ms": 1e3 * t_seq, "problems_per_s": len(sizes) / t_seq,
                           "dof_per_s": dofs / t_seq, "timing": "host clock, one pass"},
            "speedup_vs_sequential": t_seq / t_batch,
            "max_iteration_difference": int(np.max(np.abs(it_b - np.asarray(it_s)))),
            "max_rel_l2_vs_sequential": err}


# ---- vector P2 elasticity on a simplexified box ----------------------------------------------
def bench_elasticity(args, gg, ctx, lib, timed):
    """simplexify(48^3) vector P2 elasticity (6 tets per cube, 30 dofs per tet), per-cell
    lognormal Lamé coefficients, body force (0,0,-1), x = 0 clamped: symbolic + numeric
    assembly + FCG (Jacobi, FP32 inner iterations with FP64 reliable updates) to 1e-8, with
    FP64 and with FP32 cell matrices (FP64 scatter)."""
    import ctypes
    import torch
    from gridap_gb300 import _lib, workloads
    model, V, dO, lame, force = workloads.elasticity_3d(args.elast_n)
    nfree = V.num_free_dofs()
    dev = torch.device("cuda", ctx.device)
    ids_d = torch.from_numpy(V.cell_dof_ids).to(dev)
    lam, mu = gg.CellField(lame[:, 0]), gg.CellField(lame[:, 1])
    b = torch.zeros(nfree, dtype=torch.float64, device=dev)
    x = torch.zeros(nfree, dtype=torch.float64, device=dev)
    solver = gg.FCGSolver(rtol=1e-8, pc="mg")
    jacobi = gg.FCGSolver(rtol=1e-8)
    preps = {p: gg.prepare_problem(V, V, dO, (lam, mu), force, precision=p)
             for p in ("fp64", "fp32")}
    ncells, nd = V.cell_dof_ids.shape
    info = {}

    def step(prec, keep=False, slv=None):
        slv = slv or solver
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                                _lib.ptr(ids_d), nfree, nfree, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(
                ctx.handle, ctypes.byref(preps[prec].p), h, _lib.ptr(b)))
            if "nnz" not in info:
                nnz = ctypes.c_int64()
                lib.gfe_matrix_info(h, None, None, ctypes.byref(nnz))
                info["nnz"] = nnz.value
            if keep:
                info["csr_" + prec] = export_csr(lib, h, 1)
                info["b_" + prec] = b.cpu().numpy().copy()
                return None
            o = slv.opts()
            rep = _lib.SolveReport()
            _lib.check(lib.gfe_solve_fcg(ctx.handle, h, None, ctypes.byref(o), _lib.ptr(b),
                                         _lib.ptr(x), ctypes.byref(rep)))
        finally:
            lib.gfe_matrix_destroy(h)
        return rep

    out = {"workload": f"simplexify({args.elast_n}^3) vector P2 elasticity",
           "free_dofs": nfree, "cells": ncells, "quadrature": "Witherden-Vincent degree 4 "
           "(14 points)", "solver": "FCG (FP32 inner / FP64 reliable updates, 1e-8) with the "
           "two-level preconditioner: Chebyshev-Jacobi on P2, the P1 elasticity matrix of the "
           "same tets solved by 30 Jacobi-PCG steps; FCG with Jacobi beside it (`fcg_jacobi`)"}
    sols = {}
    for prec in ("fp64", "fp32"):
        r = timed("elast_" + prec, lambda: step(prec), 1, 1)
        rep = r["reps"][-1]
        if not rep.relres <= 1e-8 * (1 + 1e-6):
            raise RuntimeError(f"elasticity solve did not reach 1e-8: {rep.relres}")
        out[prec] = {"value": nfree / (r["ms"] * 1e-3), "unit": "DOF/s", "ms_per_step": r["ms"],
                     "iterations": rep.iterations, "relres": rep.relres,
                     "assembly_ms_per_launch": (r["kt"][_lib.GFE_KT_ASSEMBLE][0] /
                                                max(r["kt"][_lib.GFE_KT_ASSEMBLE][1], 1))}
        sols[prec] = x.clone()
    rj = timed("elast_jacobi", lambda: step("fp64", slv=jacobi), 1, 0, kernel_timing=False)
    out["fp64"]["fcg_jacobi"] = {"value": nfree / (rj["ms"] * 1e-3), "ms_per_step": rj["ms"],
                                 "iterations": rj["reps"][-1].iterations,
                                 "relres": rj["reps"][-1].relres}
    out["nnz"] = info.get("nnz")
    # the element kernels of general affine tets (node coordinates) on the same mesh: the
    # FP32 cells come from the tensor cores (k_p2_metric + k_p2_cells_tc), the FP64 cells from
    # the CUDA-core kernel; assembly only
    preps_n = {p: gg.prepare_problem(V, V, dO, (lam, mu), force, precision=p, geometry="nodal")
               for p in ("fp64", "fp32")}

    def assemble_nodal(prec):
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                                _lib.ptr(ids_d), nfree, nfree, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(
                ctx.handle, ctypes.byref(preps_n[prec].p), h, _lib.ptr(b)))
        finally:
            lib.gfe_matrix_destroy(h)

    tc = {}
    peak, _ = peaks()
    for prec in ("fp32", "fp64"):
        r = timed("elast_nodal_" + prec, lambda: assemble_nodal(prec), 2, 1)
        el_tot, el_n = r["kt"][_lib.GFE_KT_ELEMENT]
        el_ms = el_tot / el_n if el_n else float("nan")
        # algorithmic: the 9 x 9 by 9 x 100 product per cell; bytes: the FP32 (FP64) cell
        # matrix and the FP64 cell vector written, vertex ids, coordinates and Lame read
        flops = 2.0 * 900 * 9 * ncells
        esz = 4 if prec == "fp32" else 8
        nbytes = ncells * (900 * esz + 30 * 8 + 4 * 4 + 4 * 3 * 8 + 16)
        tc[prec] = {"element_kernel_ms": el_ms,
                    "element_tflops": flops / (el_ms * 1e-3) / 1e12,
                    "element_gbs": nbytes / (el_ms * 1e-3) / 1e9,
                    "element_frac_of_hbm": nbytes / (el_ms * 1e-3) / 1e9 / peak,
                    "assembly_ms_per_step": r["ms"]}
    tc["fp32"]["kernel"] = ("k_p2_metric + k_p2_cells_tc: tcgen05 kind::f16 with split FP16 "
                            "operands (about 22 significant bits), M=128 entries, N=144 (9 "
                            "(k,l) x 16 cells), K=32; output-bound")
    tc["fp64"]["kernel"] = "k_p2_elasticity_cells<double> (thread per tet, CUDA cores)"
    out["general_tet_element_kernels"] = tc
    out["fp32_cells_solution_rel_l2_vs_fp64"] = float(
        torch.linalg.norm(sols["fp32"] - sols["fp64"]) / torch.linalg.norm(sols["fp64"]))
    if not args.no_parity:
        # FP64 and FP32 assemblies and both solutions against the oracle at full size
        from oracle import oracle as orc
        step("fp64", keep=True)
        step("fp32", keep=True)
        n = args.elast_n
        t0 = time.perf_counter()
        with orc.cell_threads(os.cpu_count() or 1):
            ref = orc.elasticity_p2((0, 1, 0, 1, 0, 1), (n, n, n), lame, assemble=False)
        cd = ref["cell_dofs"]
        if not np.array_equal(cd, V.cell_dof_ids):
            raise RuntimeError("elasticity: device-path dof ids differ from the oracle's")
        csc = orc.assemble_csc(cd, cd, ref["cellmats"], ref["nfree"], ref["nfree"])
        del ref["cellmats"]
        bref = orc.assemble_vector(cd, ref["cellvecs"], ref["nfree"])
        t_orc = time.perf_counter() - t0
        par = {"oracle": f"CPU restatement of Gridap's P2 elasticity assembly on simplexify("
                         f"{n}^3), same Lame coefficients ({t_orc:.1f} s)"}
        for prec in ("fp64", "fp32"):
            par[prec] = csr_parity(info["csr_" + prec], csc, info["b_" + prec], bref)
            par[prec]["solution"] = solution_parity(orc, csc, bref, sols[prec].cpu().numpy())
        p64 = par["fp64"]
        par["pass_fp64"] = bool(p64["pattern_bit_exact"] and p64["matrix_max_rowscaled_err"]
                                <= 1e-12 and p64["vector_max_rel_err"] <= 1e-12 and
                                p64["solution"]["relres_in_oracle_system"] <= 1e-8 * (1 + 1e-3))
        out["parity"] = par
    return out


# ---- Q2 on jittered hexahedra: FP64 cells vs tensor-core cells ------------------------------
def bench_q2(args, gg, ctx, lib, timed):
    """64^3 Q2 Poisson on jittered hexahedra (2,048,383 free dofs): symbolic + numeric
    assembly + mixed CG (FP32 inner, FP64 reliable updates) to 1e-8, once with FP64 cell
    matrices and once with tensor-core cell matrices (tcgen05 kind::f16, per-cell-scaled FP16
    operands with TF32's 11 significant bits, FP32 accumulation and geometry), FP64 scatter in
    both. Reports the element kernel's rate against the dense bf16 tensor peak, and the
    tensor-core result's error against FP64."""
    import ctypes
    import torch
    from gridap_gb300 import _lib, workloads
    model, V, dO = workloads.jittered_q2_3d(args.q2_n)
    nfree = V.num_free_dofs()
    ncells, nd = V.cell_dof_ids.shape
    dev = torch.device("cuda", ctx.device)
    ids_d = torch.from_numpy(V.cell_dof_ids).to(dev)
    b = torch.zeros(nfree, dtype=torch.float64, device=dev)
    x = torch.zeros(nfree, dtype=torch.float64, device=dev)
    solvers = {"mixed_cg": gg.MixedCGSolver(rtol=1e-8), "pmg_fcg": gg.FCGSolver(rtol=1e-8, pc="mg")}
    preps = {p: gg.prepare_problem(V, V, dO, 1.0, 1.0, precision=p) for p in ("fp64", "fp32")}
    vals = {}

    def step(prec, keep=False, solver_name="pmg_fcg"):
        solver = solvers[solver_name]
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                                _lib.ptr(ids_d), nfree, nfree, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(
                ctx.handle, ctypes.byref(preps[prec].p), h, _lib.ptr(b)))
            if keep:
                vals[prec] = export_csr(lib, h, 1)
                vals["b_" + prec] = b.cpu().numpy().copy()
            o = solver.opts()
            rep = _lib.SolveReport()
            if isinstance(solver, gg.FCGSolver):
                _lib.check(lib.gfe_solve_fcg(ctx.handle, h, None, ctypes.byref(o), _lib.ptr(b),
                                             _lib.ptr(x), ctypes.byref(rep)))
            else:
                _lib.check(lib.gfe_solve(ctx.handle, h, ctypes.byref(o), _lib.ptr(b),
                                         _lib.ptr(x), ctypes.byref(rep)))
        finally:
            lib.gfe_matrix_destroy(h)
        return rep

    out = {"workload": f"{args.q2_n}^3 Q2 Poisson, jittered nodes (+-0.2h), degree 4",
           "free_dofs": nfree, "cells": ncells,
           "solver": "flexible CG (FP32 inner, FP64 reliable updates) with the p-multigrid "
                     "preconditioner (damped Jacobi on Q2, Q1 lattice V-cycle below), 1e-8; "
                     "mixed CG with Jacobi beside it (`mixed_cg_jacobi`)"}
    sols = {}
    peak_tf = None
    try:
        mp = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        peak_tf = mp.get("bf16_tflops")
    except (OSError, ValueError):
        pass
    flops = 34.4e9 * ncells / 262144  # Q2 per-cell contraction count (27 q x (push-forward +
    # 27^2 x 3 x 2 products)) at 64^3
    for prec in ("fp64", "fp32"):
        step(prec, keep=True)
        r = timed("q2_" + prec, lambda: step(prec), 1, 1)
        rep = r["reps"][-1]
        if not rep.relres <= 1e-8 * (1 + 1e-6):
            raise RuntimeError(f"Q2 solve did not reach 1e-8: {rep.relres}")
        el_tot, el_n = r["kt"][_lib.GFE_KT_ELEMENT]
        el_ms = el_tot / el_n if el_n else float("nan")
        out[prec] = {"value": nfree / (r["ms"] * 1e-3), "unit": "DOF/s", "ms_per_step": r["ms"],
                     "iterations": rep.iterations, "relres": rep.relres,
                     "element_kernel_ms": el_ms,
                     "element_tflops": flops / (el_ms * 1e-3) / 1e12 if el_n else None,
                     "assembly_ms_per_launch": (r["kt"][_lib.GFE_KT_ASSEMBLE][0] /
                                                max(r["kt"][_lib.GFE_KT_ASSEMBLE][1], 1))}
        sols[prec] = x.clone()
        rj = timed("q2_jac_" + prec, lambda: step(prec, solver_name="mixed_cg"), 1, 1,
                   kernel_timing=False)
        out[prec]["mixed_cg_jacobi"] = {"value": nfree / (rj["ms"] * 1e-3),
                                        "ms_per_step": rj["ms"],
                                        "iterations": rj["reps"][-1].iterations,
                                        "relres": rj["reps"][-1].relres}
    out["fp32"]["element_kernel"] = ("k_q2_metric (FP32 geometry -> FP16 metric tiles in the "
                                     "MMA operand layout, FP32 load vectors) + k_q2_cells_tc "
                                     "(tcgen05 kind::f16, per-cell-scaled FP16 operands with "
                                     "TF32's 11 significant bits, FP32 accumulate: every cell "
                                     "matrix one column of [729 x 176] x [176 x cells], M=128 "
                                     "matrix entries, N=64 cells, K=176; metric tiles by TMA "
                                     "bulk copies; zero row sums kept exact)")
    if peak_tf and out["fp32"]["element_tflops"]:
        out["fp32"]["element_frac_of_bf16_dense_peak"] = out["fp32"]["element_tflops"] / peak_tf
    rp, _, z64 = vals["fp64"]
    _, _, z32 = vals["fp32"]
    rowmax = np.maximum.reduceat(np.abs(z64), rp[:-1] - 1)
    out["tf32_cells_matrix_err_rowscaled"] = float(
        np.max(np.abs(z32 - z64) / np.repeat(rowmax, np.diff(rp))))
    out["tf32_cells_solution_rel_l2_vs_fp64"] = float(
        torch.linalg.norm(sols["fp32"] - sols["fp64"]) / torch.linalg.norm(sols["fp64"]))
    if not args.no_parity:
        # FP64 and TF32 assemblies and both solutions against the oracle at full size
        from oracle import oracle as orc
        syn = load_synthetic()
        n = args.q2_n
        t0 = time.perf_counter()
        with orc.cell_threads(os.cpu_count() or 1):
            ref = orc.poisson_q2((0, 1, 0, 1, 0, 1), (n, n, n), ("boundary",), kappa=None,
                                 fconst=1.0, degree=4, jitter=syn.q2_jitter(n))
        t_orc = time.perf_counter() - t0
        del ref["cellmats"]
        par = {"oracle": f"CPU restatement of Gridap's Q2 assembly on the same jittered {n}^3 "
                         f"mesh ({t_orc:.1f} s)"}
        par["fp64"] = csr_parity(vals["fp64"], ref["csc"], vals["b_fp64"], ref["b"])
        par["fp64"]["solution"] = solution_parity(orc, ref["csc"], ref["b"],
                                                  sols["fp64"].cpu().numpy())
        par["tf32"] = csr_parity(vals["fp32"], ref["csc"], vals["b_fp32"], ref["b"])
        par["tf32"]["solution"] = solution_parity(orc, ref["csc"], ref["b"],
                                                  sols["fp32"].cpu().numpy())
        p64 = par["fp64"]
        par["pass_fp64"] = bool(p64["pattern_bit_exact"] and p64["matrix_max_rowscaled_err"]
                                <= 1e-12 and p64["vector_max_rel_err"] <= 1e-12 and
                                p64["solution"]["relres_in_oracle_system"] <= 1e-8 * (1 + 1e-3))
        par["pass_tf32"] = bool(par["tf32"]["pattern_bit_exact"] and
                                par["tf32"]["matrix_max_rowscaled_err"] <= 2e-3)
        out["parity"] = par
    return out


# ---- 2-D Poisson, the configuration Gridap runs on CPU -------------------------------------
def bench_poisson2d(args, gg, ctx, lib, timed):
    """256^2 Q1 Poisson, f = sum of 8 seeded sinusoids, CG (FP64, Jacobi) to 1e-10, against
    the oracle (Gridap's algorithm on the host) for the same problem."""
    import ctypes
    import torch
    from gridap_gb300 import _lib, workloads
    w = workloads.poisson_2d(256)
    V = w.space
    nfree = V.num_free_dofs()
    ncells, nd = V.cell_dof_ids.shape
    dev = torch.device("cuda", ctx.device)
    ids_d = torch.from_numpy(V.cell_dof_ids).to(dev)
    b = torch.zeros(nfree, dtype=torch.float64, device=dev)
    x = torch.zeros(nfree, dtype=torch.float64, device=dev)
    prep = gg.prepare_problem(V, V, w.measure, None, w.source)
    solver = gg.CGSolver(rtol=w.rtol)

    def step():
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                                _lib.ptr(ids_d), nfree, nfree, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(ctx.handle, ctypes.byref(prep.p), h,
                                                          _lib.ptr(b)))
            o = solver.opts()
            rep = _lib.SolveReport()
            _lib.check(lib.gfe_solve(ctx.handle, h, ctypes.byref(o), _lib.ptr(b), _lib.ptr(x),
                                     ctypes.byref(rep)))
        finally:
            lib.gfe_matrix_destroy(h)
        return rep

    r = timed("poisson2d", step, 5, 3, kernel_timing=False)
    rep = r["reps"][-1]
    out = {"workload": "256^2 Q1 Poisson, sinusoid-sum source, CG 1e-10", "free_dofs": nfree,
           "value": nfree / (r["ms"] * 1e-3), "unit": "DOF/s", "ms_per_step": r["ms"],
           "iterations": rep.iterations, "relres": rep.relres}
    if not args.no_parity:
        # the same assembly kept, against the oracle on the same source at full size
        from oracle import oracle as orc
        h = ctypes.c_void_p()
        _lib.check(lib.gfe_symbolic_loop_matrix(ctx.handle, ncells, nd, _lib.ptr(ids_d),
                                                _lib.ptr(ids_d), nfree, nfree, ctypes.byref(h)))
        try:
            _lib.check(lib.gfe_assemble_matrix_and_vector(ctx.handle, ctypes.byref(prep.p), h,
                                                          _lib.ptr(b)))
            csr = export_csr(lib, h, 1)
        finally:
            lib.gfe_matrix_destroy(h)
        ref = orc.poisson_q1((0, 1, 0, 1), (256, 256), ("boundary",), f_callable=w.source)
        xr, itr, rrr = orc.pcg(*ref["csc"], ref["b"], w.rtol)
        par = {"oracle": "CPU restatement of Gridap's assembly and Jacobi-PCG, full size"}
        par.update(csr_parity(csr, ref["csc"], b.cpu().numpy(), ref["b"]))
        par["solution"] = solution_parity(orc, ref["csc"], ref["b"], x.cpu().numpy(), xr)
        par["oracle_pcg"] = {"iterations": itr, "relres": rrr}
        par["pass"] = bool(par["pattern_bit_exact"] and par["matrix_max_rowscaled_err"] <= 1e-12
                           and par["vector_max_rel_err"] <= 1e-12 and
                           par["solution"]["relres_in_oracle_system"] <= w.rtol * (1 + 1e-3))
        out["parity"] = par
    return out


def bench_nonlinear(args, gg, ctx, lib, timed):
    """Newton on the 3-D p-Laplacian (p = 3, eps2 = 1e-2): n^3 Q1 cells, u = x + y + z on the
    boundary, f = 1, degree 4 (8 points). Timed: the residual + Jacobian re-assembly into the
    fixed pattern (what every Newton step repeats) and a whole Newton solve (NLSolver, CG
    1e-10 on the SPD Jacobian) from a seeded random start; vectors stay on the device."""
    import torch
    n = args.nl_n
    m = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (n, n, n))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    U = gg.TrialFESpace(V, lambda x: x[:, 0] + x[:, 1] + x[:, 2])
    dO = gg.Measure(gg.Triangulation(m), 4)
    flux = gg.PowerLawFlux(3.0, 1e-2)
    op = gg.FEOperator(lambda u, v: gg.integrate(gg.inner(gg.grad(v), flux(gg.grad(u)))
                                                 - 1.0 * v, dO), U, V,
                       assem=gg.SparseMatrixAssembler(U, V, ctx=ctx))
    nfree = V.num_free_dofs()
    dev = torch.device("cuda", ctx.device)
    gen = torch.Generator(device="cpu").manual_seed(17)
    x0 = torch.rand(nfree, generator=gen, dtype=torch.float64).to(dev)
    x = x0.clone()
    b = torch.empty(nfree, dtype=torch.float64, device=dev)
    A = op.allocate_jacobian()
    r = timed("nl_reassembly", lambda: op.residual_and_jacobian_(b, A, x), args.steps,
              max(3, args.warmup))
    el_ms, el_n = r["kt"][_lib_const(lib, "GFE_KT_ELEMENT")]
    asm_ms, asm_n = r["kt"][_lib_const(lib, "GFE_KT_ASSEMBLE")]
    nls = gg.NLSolver(gg.CGSolver(rtol=1e-10), method="newton", ftol=1e-9)

    def newton():
        x.copy_(x0)
        nls.solve_(x, op.get_algebraic_operator())
        return nls.iterations

    rs = timed("nl_newton", newton, 1, 1, kernel_timing=False)
    its = rs["reps"][-1]
    return {"workload": f"{n}^3 Q1 p-Laplacian (p=3, eps2=1e-2), Newton (NLSolver), CG 1e-10",
            "free_dofs": nfree, "cells": m.num_cells(),
            "reassembly": {"ms_per_call": r["ms"], "dof_per_s": nfree / (r["ms"] * 1e-3),
                           "element_ms": el_ms / max(el_n, 1), "row_gather_ms":
                           asm_ms / max(asm_n, 1),
                           "what": "residual + Jacobian at the state: element kernel "
                                   "(k_quasilinear_cells) + row gather into the fixed pattern"},
            "newton": {"ms": rs["ms"], "iterations": its, "ms_per_newton_step": rs["ms"] / its,
                       "final_residual_inf": nls.residual_norm}}


def bench_reordering(args, gg, ctx, lib, timed):
    """Free-dof RCM on the jittered Q2 space (n^3 cells, Gridap's first-touch numbering):
    the device permutation against the oracle's sequential restatement on one host core
    (same permutation), and FP64 CG iterations on the matrix before and after reordering
    (100 iterations each, same arithmetic up to the permutation)."""
    import ctypes
    import torch
    from gridap_gb300 import _lib, workloads
    from gridap_gb300.reindexing import bandwidth
    model, V, dO = workloads.jittered_q2_3d(args.ro_n)
    nfree = V.num_free_dofs()
    ids = np.ascontiguousarray(V.cell_dof_ids, np.int32)
    iperm = np.empty(nfree, np.int64)

    def rcm():
        _lib.check(lib.gfe_dof_permutation(ctx.handle, ids.shape[0], ids.shape[1],
                                           _lib.ptr(ids), nfree, _lib.GFE_REORDER_RCM, 1, 2,
                                           _lib.ptr(iperm)))

    r = timed("rcm", rcm, 1, 1, kernel_timing=False)
    W = gg.reindex_free_dof_ids(V, iperm.copy())
    dev = torch.device("cuda", ctx.device)
    out = {"workload": f"{args.ro_n}^3 Q2 jittered, free dofs {nfree}",
           "rcm_gpu_ms": r["ms"]}
    cg = gg.CGSolver(rtol=1e-30, maxiter=100)
    for name, S in (("natural", V), ("rcm", W)):
        prep = gg.prepare_problem(S, S, dO, None, 1.0)
        A = gg.symbolic_loop_matrix(gg.SparseMatrixAssembler(S, S, ctx=ctx),
                                    (None, S.cell_dof_ids, S.cell_dof_ids))
        b = torch.zeros(nfree, dtype=torch.float64, device=dev)
        x = torch.zeros(nfree, dtype=torch.float64, device=dev)
        _lib.check(lib.gfe_assemble_matrix_and_vector(ctx.handle, ctypes.byref(prep.p), A.handle,
                                                      _lib.ptr(b)))
        ns = gg.numerical_setup(gg.symbolic_setup(cg, A), A)
        rs = timed("cg_" + name, lambda: gg.solve_(x, ns, b), 3, 2, kernel_timing=False)
        out[name] = {"bandwidth": bandwidth(A), "ms_per_cg_iteration": rs["ms"] / 100}
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        t0 = time.perf_counter()
        want = orc.dof_permutation(ids, nfree, "rcm")
        out["rcm_cpu_oracle_s"] = time.perf_counter() - t0
        out["rcm_cpu_cores"] = 1
        out["same_permutation_as_oracle"] = bool(np.array_equal(want, iperm))
    return out


def bench_multifield(args, gg, ctx, lib, timed):
    """Stokes Taylor-Hood assembly (StokesTaylorHoodTests.jl's form: vector Q2 velocity, Q1
    pressure, a = ∫ ∇v⊙∇u - (∇⋅v)p + q(∇⋅u), l = ∫ v⋅f + q g, u = u_exact on the boundary)
    on n^3 cells, consecutive (one matrix) and block (2 x 2 grid) layouts. Timed: the whole
    AffineFEOperator assembly call (host form classification and tables, device geometry and
    cell integrals, symbolic and numeric loops, vector with the Dirichlet lift)."""
    n = args.mf_n
    m = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (n, n, n))
    u = lambda x: np.stack([x[:, 1] ** 2, x[:, 2] ** 2 + x[:, 0], x[:, 0] * x[:, 1]], 1)  # noqa
    f = lambda x: np.tile([-2.0, -2.0, 0.0], (x.shape[0], 1))  # noqa: E731
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags="boundary")
    Q = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1))
    U, P = gg.TrialFESpace(V, u), gg.TrialFESpace(Q)
    dO = gg.Measure(gg.Triangulation(m), 4)
    a = lambda x, y: gg.integrate(gg.inner(gg.grad(y[0]), gg.grad(x[0]))  # noqa: E731
                                  - gg.div(y[0]) * x[1] + y[1] * gg.div(x[0]), dO)
    l = lambda y: gg.integrate(gg.inner(y[0], f), dO)  # noqa: E731
    assem = gg.SparseMatrixAssembler(gg.MultiFieldFESpace([U, P]), gg.MultiFieldFESpace([V, Q]),
                                     ctx=ctx)
    out = {"workload": f"{n}^3 Stokes Taylor-Hood (vector Q2 / Q1), degree 4 (27 points)"}
    for name, style in (("consecutive", None), ("block", gg.BlockMultiFieldStyle())):
        X = gg.MultiFieldFESpace([U, P], style=style)
        Y = gg.MultiFieldFESpace([V, Q], style=style)
        steps = max(1, args.steps // 2)
        r = timed("mf_" + name, lambda: gg.assemble_matrix_and_vector(a, l, X, Y, assem),
                  steps, max(3, args.warmup))
        el_ms, el_n = r["kt"][_lib_const(lib, "GFE_KT_ELEMENT")]
        asm_ms, asm_n = r["kt"][_lib_const(lib, "GFE_KT_ASSEMBLE")]
        nd = X.num_free_dofs()
        out[name] = {"ms_per_assembly": r["ms"], "dof_per_s": nd / (r["ms"] * 1e-3),
                     "cell_integral_ms": el_ms / steps, "row_gather_ms": asm_ms / steps,
                     "kernel_launches_per_assembly": {"cell_integrals": el_n // steps,
                                                      "row_gather": asm_n // steps}}
    out["free_dofs"] = X.num_free_dofs()
    out["cells"] = m.num_cells()
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        ns = 8
        ms = gg.CartesianDiscreteModel((0, 1, 0, 1, 0, 1), (ns, ns, ns))
        Vs = gg.FESpace(ms, gg.ReferenceFE(gg.lagrangian, 3, 2), dirichlet_tags="boundary")
        Qs = gg.FESpace(ms, gg.ReferenceFE(gg.lagrangian, float, 1))
        Us = gg.TrialFESpace(Vs, u)
        t0 = time.perf_counter()
        xq = orc.qpoints(3, ms.cell_node_ids, ms.node_coords, 4)
        fq = f(xq.reshape(-1, 3)).reshape(xq.shape[0], xq.shape[1], 3)
        terms = [(0, 1, 0, 1, 1.0, None, None), (0, 2, 1, 0, -1.0, None, None),
                 (1, 0, 0, 2, 1.0, None, None), (0, 0, None, None, 1.0, None, fq)]
        K, F = orc.multifield_cell_arrays(3, ms.node_coords, ms.cell_node_ids, [(2, 3), (1, 1)],
                                          terms, 4)
        nu = Vs.num_free_dofs()
        ip = Qs.get_cell_dof_ids()
        orc.multifield_assemble([Vs.get_cell_dof_ids(), np.where(ip > 0, ip + nu, ip)],
                                [nu, Qs.num_free_dofs()], K, F,
                                [Us.get_dirichlet_dof_values(), None])
        t = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "kind": "port", "cores": 1,
            "sample": f"oracle (numpy cell integrals + serial CSC assembly) on {ns}^3 cells, "
                      f"{t:.2f} s, scaled per cell",
            "ms_per_assembly_scaled": 1e3 * t * m.num_cells() / ms.num_cells()}
    return out


def _lib_const(lib, name):
    from gridap_gb300 import _lib
    return getattr(_lib, name)


# ---- CPU baseline / reference arm ---------------------------------------------------------
def cpu_baseline(args, keep=False, serial=True):
    """The oracle (CPU restatement of Gridap's algorithm) on the host cores, the whole step
    on the same seeded inputs as the device arm (numpy-generated; no package import):
      - serial: the assembly exactly like Gridap's numeric loop, one thread (cell arrays,
        InserterCSC insertions in cell order);
      - threaded (the reported value): the cell arrays on all host threads and the
        colour-parallel InserterCSC assembly (greedy cell colouring, cells of one colour in
        parallel), then Jacobi-PCG to the same 1e-8 FP64 relative residual on all host
        threads.
    Returns (summary, oracle arrays for the parity check or None)."""
    from oracle import oracle as orc
    syn = load_synthetic()
    n = args.n
    kappa, f = syn.lognormal_inputs(n)
    rtol = 1e-8
    nthreads = os.cpu_count() or 1
    dom, part = (0, 1, 0, 1, 0, 1), (n, n, n)
    ref, t_asm = None, None
    if serial:
        t0 = time.perf_counter()
        ref = orc.poisson_q1(dom, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL, fdata=f)
        t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    with orc.cell_threads(nthreads):
        r2 = orc.poisson_q1(dom, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL, fdata=f,
                            assemble=False)
    nfree = r2["nfree"]
    colors = orc.color_cells(r2["cell_dofs"], nfree)
    csc2, b2 = orc.assemble_colored(r2["cell_dofs"], r2["cellmats"], r2["cellvecs"], nfree,
                                    nthreads, colors)
    t_asm_omp = time.perf_counter() - t0
    del r2
    same_pattern, omp_err = None, None
    if ref is not None:
        cp, rv, zv = ref["csc"]
        same_pattern = bool(np.array_equal(csc2[0], cp) and np.array_equal(csc2[1], rv))
        omp_err = float(np.abs(csc2[2] - zv).max() / np.abs(zv).max())
        bvec = ref["b"]
    else:
        (cp, rv, zv), bvec = csc2, b2
    t1 = time.perf_counter()
    x, it, relres = orc.pcg(cp, rv, zv, bvec, rtol, nthreads=nthreads)
    t_solve = time.perf_counter() - t1
    total = t_asm_omp + t_solve
    summary = {
        "value": nfree / total, "unit": UNIT, "cores": nthreads, "kind": "port",
        "sample": (f"oracle on the full {n}^3 workload, the whole step: cell arrays + "
                   f"colour-parallel InserterCSC assembly ({colors[1]} colours, "
                   f"{t_asm_omp:.2f} s on {nthreads} threads) + Jacobi-PCG to {rtol:g} "
                   f"({it} iterations, {t_solve:.2f} s on {nthreads} threads)"),
        "assembly_s": t_asm_omp, "solve_s": t_solve, "iterations": it, "relres": relres,
        "serial_assembly": None if t_asm is None else {
            "assembly_s": t_asm, "cores": 1,
            "value_with_threaded_solve": nfree / (t_asm + t_solve),
            "what": "Gridap's numeric loop as written: one thread, InserterCSC insertions in "
                    "cell order"},
        "threaded_assembly_same_pattern": same_pattern,
        "threaded_assembly_max_err_vs_serial": omp_err,
        "nfree": nfree, "ncells": n ** 3, "nnz": int(zv.shape[0])}
    keep_out = None
    if keep and ref is not None:
        keep_out = {"csc": ref["csc"], "b": ref["b"], "x": x, "relres": relres}
    return summary, keep_out


def run_reference(args):
    """The CPU arm: the oracle (Gridap's algorithm restated in C, all host threads) on the same
    workload and metric. Imports neither the package nor the CUDA library."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    vals, times = [], []
    cb = None
    for k in range(args.warmup + args.steps):
        cb, _ = cpu_baseline(args, serial=False)
        if k >= args.warmup:
            vals.append(cb["value"])
            times.append(1e3 * (cb["assembly_s"] + cb["solve_s"]))
    v = float(np.median(vals))
    cb["value"] = v
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median(times)),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded lognormal GRF kappa, N(0,1) nodal f)",
           "config": workload_config(args.n, cb["nfree"], cb["ncells"], cb["nnz"], 1e-8, world),
           "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gfe", choices=["gfe", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--solver", default="mg", choices=["mg", "mixed"],
                    help="headline solver: multigrid-preconditioned flexible CG or Jacobi mixed CG")
    ap.add_argument("--delta", type=float, default=0.01,
                    help="residual reduction between FP64 reliable updates of the mixed CG")
    ap.add_argument("--profile", action="store_true",
                    help="run only the headline steps and print no JSON (for ncu launch lists)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size comparisons with the oracle")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-elasticity", action="store_true")
    ap.add_argument("--elast-n", type=int, default=48)
    ap.add_argument("--no-q2", action="store_true")
    ap.add_argument("--q2-n", type=int, default=64)
    ap.add_argument("--no-poisson2d", action="store_true")
    ap.add_argument("--no-nonlinear", action="store_true")
    ap.add_argument("--nl-n", type=int, default=64)
    ap.add_argument("--no-reordering", action="store_true")
    ap.add_argument("--ro-n", type=int, default=48)
    ap.add_argument("--no-multifield", action="store_true")
    ap.add_argument("--mf-n", type=int, default=24)
    ap.add_argument("--batch-problems", type=int, default=256)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gfe":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
