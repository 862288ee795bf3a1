#!/usr/bin/env python
"""Coupled solves/s at 1e-8 relative residual on one GB300.

Workload (the "plain vs mixed-precision on GPU" configuration): a
two-region conjugate-heat-transfer temperature system, fluid 128^3 over solid
128x128x64 (n = 3,145,728 cells, 9,371,648 faces incl. the 16,384-face
interface), conductivity log-uniform in [0.1, 50] per cell (seeded), in
monolithic LDU form.  One step = one solve to foam-normalised residual 1e-8
(relTol 0): coefficient upload (views + DIC factor) and the Krylov solve.

  value   mixed form (FP32 PCG + multi-colour DIC inside FP64 iterative
          refinement) with coefficients, b and x0 already resident in HBM
  e2e     the same through the host-pointer C ABI (mrg_coeffs_upload +
          mrg_solve from pinned host memory; copies inside the timed region)
  plain   the plain method, FP64 PCG+DIC in foam's order, reported beside

Every result carries its max-norm error against the FP64 oracle: the CPU
oracle's foam-order solve of the same system converged to 1e-13 (1e-12 for
the many small systems), computed after the GPU timing.

The working set (~1 GB per solve) is far larger than the 129 MB L2, so no
L2 flush is needed between steps.

Beside the headline, the line carries the other configurations:
  c3        the asymmetric, non-conformal pair (96^3-scale convection-
            diffusion, permuted numbering, 3:2 GGI interface with weights
            built on the device; 737,280 cells): PBiCG + DILU plain FP64,
            mixed with BiCGStab and with PBiCG inner solves, and the GGI
            gather of a random face field (--c3-scale, 0 skips)
  batched   512 independent CHT systems (8k-260k cells) in one batch, mixed
            vs plain FP64, solves/s (--batched N, 0 skips)
  block     a 4x4 block-coupled system (48^3 cells, the shape of a
            BlockLduMatrix<vector4>) expanded to its scalar LDU system and
            solved by BiCGStab + DILU, mixed vs plain FP64 (--block-n N)
  gamg      GAMG (GaussSeidel smoother, the tutorials' fluid p / T settings)
            on a 64^3-cell CHT system, FP64 foam order, beside plain PCG +
            DIC on the same system (--gamg-n N, 0 skips)
  served    Poisson-arriving requests over recurring meshes (100 meshes of
            10k-2M cells, 70% symmetric CHT with DIC, 30% asymmetric
            convection-diffusion with DILU, 20 time steps each with 5%
            coefficient drift per step: 2000 requests) through the
            continuous-batching server under a 150 GB HBM budget, for each
            arrival rate of the sweep (default 200 and 2000 /s; the plain
            server at 2000 /s): solves/s, p50/p99 ms, for the mixed form and the plain
            FP64 method; the plain drop-in one request at a time beside
            (--served-meshes / --served-steps / --served-rates, 0 meshes
            skips)
  cpu_baseline  the CPU oracle (foam's algorithm in C, FP64 PCG + DIC) on
            the same headline system, full solves to 1e-8 timed: one core
            alone, and every core at once (one solve per process)

--impl reference times the reference algorithm's CPU implementation (the
project's C oracle; foam-extend itself cannot be built here): full solves
of the same system on every host core.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TOL = 1e-8
SEED = 0
C3_SEED = 2
REF_TOL = 1e-13          # FP64 oracle solution of a single system
REF_TOL_MANY = 1e-12     # ... of the batched / served / block members


def peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(name):
    """dram bytes per launch from a committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_system(rank, scale):
    from multiregionfoam_gb300 import cases
    return cases.c2(form="global", seed=SEED + rank, scale=scale)


_T0 = time.perf_counter()


def log(msg):
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f} s] {msg}", file=sys.stderr, flush=True)


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def err_stats(errs):
    errs = [e for e in errs if e is not None]
    if not errs:
        return None
    return {"max": float(np.max(errs)), "p99": float(np.percentile(errs, 99)), "n": len(errs)}


# ------------------------------------------------------------------ CPU leg
# The CPU oracle (foam's algorithm restated in C; test infrastructure) runs
# only here: as the timed CPU baseline and as the checker that gives every
# GPU result its error against an FP64 solution.  Worker processes are
# spawned (never forked after CUDA initialised) and rebuild their systems
# from the seeds.

_W = {}


def _w_setup():
    for p in (ROOT, os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle as O
    return O


def _w_matrix(s):
    O = _w_setup()
    return O.OracleMatrix(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.iface)


def _w_c2(scale):
    if ("c2", scale) not in _W:
        from multiregionfoam_gb300 import cases
        _w_setup()
        s = cases.c2(form="global", seed=SEED, scale=scale)
        _W[("c2", scale)] = (s, _w_matrix(s))
    return _W[("c2", scale)]


def _w_c2_solves(arg):
    """`count` full foam-order PCG + DIC solves of the headline system to
    1e-8 in this process; returns the per-solve seconds and iterations."""
    scale, count = arg
    s, A = _w_c2(scale)
    out = []
    for _ in range(count):
        t = time.perf_counter()
        _, p = A.solve(s.b, s.x0, "PCG", "DIC", tol=TOL, max_iter=20000)
        out.append((time.perf_counter() - t, p["n_iter"], bool(p["converged"])))
    return out


def _w_reference(job):
    """The FP64 oracle solution of one system, rebuilt from its description."""
    from multiregionfoam_gb300 import cases
    O = _w_setup()
    kind = job[0]
    if kind == "c2":
        s = cases.c2(form="global", seed=SEED, scale=job[1])
        solver, pc, tol = "PCG", "DIC", REF_TOL
    elif kind == "c3":
        def weights(fa, fb):
            return O.ggi_weights(*fa, *fb)
        s = cases.c3(weights, scale=job[1], seed=C3_SEED)[0]
        solver, pc, tol = "PBiCG", "DILU", REF_TOL
    elif kind == "c4":
        _, count, idx = job
        nx, ny, nzf, nzs = cases.batch_shapes(count, seed=SEED)[idx]
        s = cases.cht_system(nx, ny, nzf, nzs, seed=SEED + 1 + idx, k_range=(0.1, 50.0))
        solver, pc, tol = "PCG", "DIC", REF_TOL_MANY
    elif kind == "c5":
        _, count, mesh, step = job
        spec = cases.c5_specs(count, seed=SEED)[mesh]
        s = cases.c5_step(cases.c5_mesh(spec), mesh, step, SEED)
        solver, pc, tol = ("PBiCG", "DILU", REF_TOL_MANY) if spec[0] else ("PCG", "DIC", REF_TOL_MANY)
    elif kind == "block":
        import block_oracle as BO
        c = cases.block_case(job[1], job[1], job[1], bs=4, seed=SEED)
        lo, up, d, uc, lc = BO.expand(c["n"], c["lower"], c["upper"], 4, c["D"], c["U"], c["L"])
        n_s = 4 * c["n"]
        s = cases.LduSystem(n_s, lo, up, d, uc, lc, c["b"].ravel(), np.zeros(n_s), None)
        solver, pc, tol = "BiCGStab", "DILU", REF_TOL_MANY
    else:
        raise ValueError(kind)
    x, p = _w_matrix(s).solve(s.b, s.x0, solver, pc, tol=tol, max_iter=40000)
    return job, x, p


class CpuLeg:
    """A spawned pool of oracle workers on the host cores."""

    def __init__(self, procs=None):
        import multiprocessing as mp
        O = _w_setup()
        O.build()
        self.cores = len(os.sched_getaffinity(0))
        self.procs = procs or self.cores
        self.pool = mp.get_context("spawn").Pool(self.procs)

    def c2_solves(self, scale, counts):
        """One task per process with its solve count, all started together;
        returns the per-process lists of (seconds, iterations, converged)."""
        return self.pool.map(_w_c2_solves, [(scale, k) for k in counts], chunksize=1)

    def references(self, jobs):
        """FP64 oracle solutions {job: (x, perf)}, largest systems first."""
        out = {}
        for job, x, p in self.pool.imap_unordered(_w_reference, jobs):
            out[job] = (x, p)
        return out

    def close(self):
        self.pool.terminate()
        self.pool.join()


def cpu_baseline(scale, leg):
    """Measured full solves of the headline system: one core alone, then
    every core at once (one full solve per process)."""
    leg.c2_solves(scale, [0] * leg.procs)                       # every worker builds the system
    one = leg.c2_solves(scale, [1])[0][0]
    allc = leg.c2_solves(scale, [1] * leg.procs)
    t_all = [r[0][0] for r in allc]
    rate_all = float(sum(1.0 / t for t in t_all))
    return {"value": rate_all, "unit": "solves/s", "cores": leg.procs, "kind": "port",
            "sample": (f"oracle PCG+DIC FP64 (foam order), full solves to {TOL:g} ({one[1]} iterations) measured: "
                       f"{leg.procs} processes one solve each at once, median {np.median(t_all):.1f} s; throughput "
                       f"= sum of per-process rates"),
            "single_core": {"value": 1.0 / one[0], "unit": "solves/s", "cores": 1, "solve_s": one[0],
                            "iters": one[1]},
            "all_cores_median_solve_s": float(np.median(t_all))}


def run_reference(args):
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    s = make_system(0, args.scale)
    leg = CpuLeg(min(args.steps, len(os.sched_getaffinity(0))))
    P = leg.procs
    leg.c2_solves(args.scale, [0] * P)                       # every worker builds the system (untimed)
    # warm-up: W full solves spread over the workers (untimed)
    leg.c2_solves(args.scale, [args.warmup // P + (1 if i < args.warmup % P else 0) for i in range(P)])
    # timed: K full solves spread over the workers, all started together;
    # throughput = sum over workers of solves / that worker's busy time
    counts = [args.steps // P + (1 if i < args.steps % P else 0) for i in range(P)]
    t0 = time.perf_counter()
    res = leg.c2_solves(args.scale, counts)
    wall = time.perf_counter() - t0
    leg.close()
    solves = [r for rr in res for r in rr]
    rate = float(sum(len(rr) / sum(t for t, _, _ in rr) for rr in res if rr))
    med = float(np.median([t for t, _, _ in solves]))
    iters = int(solves[0][1])
    sample = (f"oracle PCG+DIC FP64 (foam order), {len(solves)} full solves to {TOL:g} ({iters} iterations each) on "
              f"{P} processes at once, median {med:.1f} s per solve, wall {wall:.1f} s; throughput = sum of "
              f"per-process rates")
    line = {"metric": "coupled solves/s at 1e-8 rel. residual", "value": rate, "unit": "solves/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            # a step is one solve; the solves run P at a time, so the timed
            # region's wall over the steps is the time a step takes
            "ms_per_step": wall * 1e3 / len(solves), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded C2 system)",
            "config": {"workload": "cht-2region-128^3+128x128x64", "n_cells": s.n, "n_faces": s.nf,
                       "tolerance": TOL},
            "cpu_baseline": {"value": rate, "unit": "solves/s", "cores": P, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU forms
def run_c3(args, ctx, mrgpu):
    """The asymmetric, non-conformal configuration: GGI weights built on
    the device (mrg_ggi_build); per form one warm solve and `reps` timed
    steps (coefficient upload + factor + solve, device resident); the GGI
    gather of a random face field U(-1, 1) in both directions."""
    from multiregionfoam_gb300 import cases

    def weights(fa, fb):
        ga, gb = mrgpu.Ggi.build(ctx, *fa, *fb)
        out = (ga.csr(), gb.csr())
        ga.close()
        gb.close()
        return out

    s, ggi = cases.c3(weights, scale=args.c3_scale, seed=C3_SEED)
    f = s.iface
    m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper, f)
    d_d, d_u, d_l = ctx.to_device(s.diag), ctx.to_device(s.upper_c), ctx.to_device(s.lower_c)
    d_ib = ctx.to_device(f["bou"])
    d_b, d_x0 = ctx.to_device(s.b), ctx.to_device(s.x0)
    d_x = ctx.dev_alloc(8 * s.n)
    out = {"cells": s.n, "faces": s.nf, "iface_faces": [int(ggi["n_a"]), int(ggi["n_b"])], "tolerance": TOL,
           "seed": C3_SEED}
    xs = {}
    forms = (("plain_fp64", "PBiCG", "fp64", "exact"), ("mixed", "BiCGStab", "mixed", "colour"),
             ("mixed_pbicg_inner", "PBiCG", "mixed", "colour"))
    for name, solver, prec, order in forms:
        ctl = mrgpu.controls(tol=TOL, max_iter=20000, solver=solver, precond="DILU", precision=prec,
                             ordering=order, inner_rel_tol=args.inner_tol)
        ms, perf = [], None
        for rep in range(1 + args.c3_reps):
            m.upload_device(d_d, d_u, d_l, d_ib)
            ctx.copy_d2d(d_x, d_x0, 8 * s.n)
            ctx.record(48)
            perf = m.solve_device(d_b, d_x, ctl)
            ctx.record(49)
            if rep:
                ms.append(ctx.elapsed_ms(48, 49))
        xs[name] = ctx.from_device(d_x, np.empty(s.n))
        best = min(ms)
        out[name] = {"solver": f"{solver}+DILU", "solves_per_s": 1e3 / best, "ms_per_step": best,
                     "iters": int(perf["n_iter"]), "outer": int(perf.get("n_outer", 0)),
                     "final_residual": perf["final_residual"], "converged": bool(perf["converged"])}
    out["speedup_mixed_vs_plain"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    rng = np.random.default_rng(3)
    gg = {}
    for key, (ptr, addr, w), n_src in (("a_from_b", ggi["a_from_b"], ggi["n_b"]),
                                       ("b_from_a", ggi["b_from_a"], ggi["n_a"])):
        g = mrgpu.Ggi(ctx, ptr, addr, w, n_src)
        d_src = ctx.to_device(rng.uniform(-1.0, 1.0, n_src))
        d_dst = ctx.dev_alloc(8 * g.n_dst)
        gg[key] = {"n_dst": g.n_dst, "n_src": n_src, "nnz": int(len(addr)),
                   "us_per_gather": 1e3 * g.time_device(d_src, d_dst, 200)}
        g.close()
        ctx.dev_free(d_src)
        ctx.dev_free(d_dst)
    out["ggi_gather"] = gg
    for a in (d_d, d_u, d_l, d_ib, d_b, d_x0, d_x):
        ctx.dev_free(a)
    m.close()
    return out, xs


def run_batched(args, ctx, mrgpu):
    """Batched configuration: `args.batched` independent two-region CHT
    systems (cells log-uniform in [8k, 260k], random aspect ratios,
    conductivity log-uniform in [0.1, 50]) solved in one batch, device
    resident; mixed (colour) and plain FP64 (exact order)."""
    from multiregionfoam_gb300 import cases
    systems = cases.c4(args.batched, seed=SEED)
    meshes = []
    for s in systems:
        m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper)
        m.upload(s.diag, s.upper_c)
        meshes.append(m)
    d_b = [ctx.to_device(s.b) for s in systems]
    d_x0 = [ctx.to_device(s.x0) for s in systems]
    d_x = [ctx.dev_alloc(8 * s.n) for s in systems]
    out = {"systems": len(systems), "cells": int(sum(s.n for s in systems)),
           "faces": int(sum(s.nf for s in systems))}
    xs = {}
    for name, prec, order in (("mixed", "mixed", "colour"), ("plain_fp64", "fp64", "exact")):
        bt = mrgpu.Batch(ctx, meshes, order)
        ctl = mrgpu.controls(tol=TOL, max_iter=20000, solver="PCG", precond="DIC", precision=prec, ordering=order,
                             inner_rel_tol=args.inner_tol)
        tune = bt.tune(d_b, d_x0, ctl)
        ms = []
        for rep in range(1 + args.batched_reps):
            for sy, a, b in zip(systems, d_x, d_x0):
                ctx.copy_d2d(a, b, 8 * sy.n)
            ctx.record(50)
            perfs = bt.solve_device(d_b, d_x, ctl)
            ctx.record(51)
            if rep:
                ms.append(ctx.elapsed_ms(50, 51))
        bt.close()
        xs[name] = [ctx.from_device(a, np.empty(sy.n)) for sy, a in zip(systems, d_x)]
        its = [p["n_iter"] for p in perfs]
        best = min(ms)
        out[name] = {"solves_per_s": len(systems) / (best * 1e-3), "ms_per_batch": best,
                     "iters_max": int(max(its)), "iters_mean": float(np.mean(its)),
                     "converged": int(sum(p["converged"] for p in perfs)), "tuning": tune}
    out["speedup_mixed_vs_plain"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    for a in d_b + d_x0 + d_x:
        ctx.dev_free(a)
    for m in meshes:
        m.close()
    return out, xs


def run_block(args, ctx, mrgpu):
    """Block-coupled configuration: a 4 x 4 block system (the shape of
    foam-extend's BlockLduMatrix<vector4>) on an args.block_n^3 hex block,
    expanded to its scalar LDU system on the host (mrg_block_addressing +
    mrg_block_coeffs, timed) and solved, device resident, by BiCGStab +
    DILU to 1e-8: mixed (colour) and plain FP64 (exact order).  A step is
    coefficient upload + factor + solve, as for the headline workload."""
    from multiregionfoam_gb300 import cases
    c = cases.block_case(args.block_n, args.block_n, args.block_n, bs=4, seed=SEED)
    t0 = time.perf_counter()
    n_s, lo, up, d, uc, lc = mrgpu.block_system(c["n"], c["lower"], c["upper"], 4, c["D"], c["U"], c["L"])
    t_expand = time.perf_counter() - t0
    m = mrgpu.Mesh(ctx, n_s, lo, up)
    m.set_blocks(4, c["n"], c["lower"], c["upper"])
    d_d, d_u, d_l = ctx.to_device(d), ctx.to_device(uc), ctx.to_device(lc)
    d_b, d_x0 = ctx.to_device(c["b"].ravel()), ctx.to_device(np.zeros(n_s))
    d_x = ctx.dev_alloc(8 * n_s)
    out = {"block_cells": c["n"], "block_size": 4, "scalar_cells": n_s, "scalar_faces": int(len(lo)),
           "expand_ms": t_expand * 1e3, "solver": "BiCGStab+DILU (block_cholesky: BiCGStab + the block "
                                                   "Cholesky preconditioner on the 4x4 blocks)", "tolerance": TOL}
    xs = {}
    for name, prec, order, pc in (("mixed", "mixed", "colour", "DILU"), ("plain_fp64", "fp64", "exact", "DILU"),
                                  ("block_cholesky", "fp64", "exact", "block")):
        ctl = mrgpu.controls(tol=TOL, max_iter=20000, solver="BiCGStab", precond=pc, precision=prec,
                             ordering=order, inner_rel_tol=args.inner_tol)
        ms, perf = [], None
        for rep in range(4):   # the first untimed: plans, views, graphs
            m.upload_device(d_d, d_u, d_l)
            ctx.copy_d2d(d_x, d_x0, 8 * n_s)
            ctx.record(60)
            perf = m.solve_device(d_b, d_x, ctl)
            ctx.record(61)
            if rep:
                ms.append(ctx.elapsed_ms(60, 61))
        xs[name] = ctx.from_device(d_x, np.empty(n_s))
        best = min(ms)
        out[name] = {"solves_per_s": 1e3 / best, "ms_per_step": best, "iters": int(perf["n_iter"]),
                     "final_residual": perf["final_residual"], "converged": bool(perf["converged"])}
    out["speedup_mixed_vs_plain"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    out["speedup_block_cholesky_vs_plain"] = out["block_cholesky"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    for a in (d_d, d_u, d_l, d_b, d_x0, d_x):
        ctx.dev_free(a)
    m.close()
    return out, xs


def run_gamg(args, ctx, mrgpu):
    """GAMG with the tutorials' fluid p / T settings (GaussSeidel smoother,
    agglomerator faceAreaPair, nCellsInCoarsestLevel 10, 2 post / 2 finest
    sweeps, scaleCorrection) on a two-region CHT system of args.gamg_n^3
    cells (global form), FP64 in foam order, to 1e-8, beside the same with
    algebraicPair and plain PCG + DIC on the same system.  A step is coefficient upload +
    solve; the first GAMG solve (agglomeration, cached afterwards) is timed
    on its own."""
    from multiregionfoam_gb300 import cases
    n = args.gamg_n
    s = cases.cht_system(n, n, n // 2, n - n // 2, seed=SEED, form="global")
    m = mrgpu.Mesh(ctx, s.n, s.lower, s.upper)
    m.set_face_areas(cases.face_area_vectors(s))
    d_diag, d_up = ctx.to_device(s.diag), ctx.to_device(s.upper_c)
    d_b, d_x0 = ctx.to_device(s.b), ctx.to_device(s.x0)
    d_x = ctx.dev_alloc(8 * s.n)
    out = {"cells": s.n, "faces": s.nf, "tolerance": TOL}
    words = dict(solver="GAMG", smoother="GaussSeidel", n_coarsest_cells=10, n_post_sweeps=2, n_finest_sweeps=2,
                 scale_correction=True)
    for name, kw in (("gamg", dict(words, agglomerator="faceAreaPair")),
                     ("gamg_algebraic", dict(words, agglomerator="algebraicPair")),
                     ("pcg_dic", dict(solver="PCG", precond="DIC"))):
        ctl = mrgpu.controls(tol=TOL, max_iter=5000, precision="fp64", ordering="exact", **kw)
        ms, perf = [], None
        for rep in range(4):   # rep 0: setup (GAMG hierarchy, plans, views)
            m.upload_device(d_diag, d_up)
            ctx.copy_d2d(d_x, d_x0, 8 * s.n)
            ctx.record(62)
            perf = m.solve_device(d_b, d_x, ctl)
            ctx.record(63)
            ms.append(ctx.elapsed_ms(62, 63))
        best = min(ms[1:])
        out[name] = {"solves_per_s": 1e3 / best, "ms_per_step": best, "first_ms": ms[0], "iters": int(perf["n_iter"]),
                     "final_residual": perf["final_residual"], "converged": bool(perf["converged"])}
    out["speedup_gamg_vs_pcg"] = out["gamg"]["solves_per_s"] / out["pcg_dic"]["solves_per_s"]
    out["speedup_gamg_algebraic_vs_pcg"] = out["gamg_algebraic"]["solves_per_s"] / out["pcg_dic"]["solves_per_s"]
    for a in (d_diag, d_up, d_b, d_x0, d_x):
        ctx.dev_free(a)
    m.close()
    return out


def run_served(args, ctx, mrgpu):
    """Served configuration: `served_meshes` meshes (cells log-uniform in
    [10k, 2M], 70% CHT with DIC, 30% convection-diffusion with DILU), each
    recurring `served_steps` time steps with its coefficients re-drawn at 5%
    perturbation per step (cases.c5_step), one request per mesh and step,
    Poisson arrivals at each rate of the sweep; 150 GB HBM budget.  Every
    form is warmed (plans, views, factors, graphs) before it is timed.  One
    request per mesh (step i mod steps) keeps its solution for the error
    against the FP64 oracle."""
    from multiregionfoam_gb300 import cases
    specs = cases.c5_specs(args.served_meshes, seed=SEED)
    t0 = time.perf_counter()

    def generate(i):
        """Mesh i's addressing and its time steps' coefficient arrays
        (cases.c5_step's sequence, one step after the other)."""
        cur = cases.c5_mesh(specs[i])
        seq = [dict(diag=cur.diag, upper=cur.upper_c, lower=cur.lower_c, b=cur.b, x0=cur.x0)]
        for k in range(1, args.served_steps):
            cur = cases.perturb_step(cur, np.random.default_rng((SEED, i, k)))
            seq.append(dict(diag=cur.diag, upper=cur.upper_c, lower=cur.lower_c, b=cur.b, x0=seq[0]["x0"]))
        return cur.n, cur.lower, cur.upper, seq

    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=len(os.sched_getaffinity(0))) as ex:
        gen = list(ex.map(generate, range(len(specs))))
    meshes = [mrgpu.Mesh(ctx, n, lo, up) for n, lo, up, _ in gen]
    steps = [seq for _, _, _, seq in gen]
    del gen
    t_gen = time.perf_counter() - t0
    asym = [sp[0] for sp in specs]
    n_req = len(specs) * args.served_steps
    sample = {i: i % args.served_steps for i in range(len(specs))}      # mesh -> sampled step
    rates = [float(r) for r in args.served_rates.split(",") if r.strip()]
    plain_rates = rates if not args.served_plain_rates else \
        [float(r) for r in args.served_plain_rates.split(",") if r.strip()]
    out = {"requests": n_req, "meshes": len(specs), "steps_per_mesh": args.served_steps, "rates_per_s": rates,
           "iters_per_launch": args.served_k, "cells_mean": float(np.mean([m.n for m in meshes])),
           "asym_meshes": int(sum(asym)), "hbm_budget_gb": 150, "generate_s": t_gen}
    # the fast form: mixed PCG + colour DIC for the symmetric requests; for
    # the asymmetric (convection-diffusion) ones FP64 PBiCG + colour DILU,
    # which on this mix finished in less time than the mixed BiCGStab form:
    # over the perturbed time steps a few FP32-inner solves stall and end in
    # the FP64 continuation (one request of 2000 did not converge there);
    # --served-mixed-asym serves them with mixed BiCGStab
    forms = [("mixed", "mixed", "colour", "BiCGStab" if args.served_mixed_asym else "PBiCG-fp64"),
             ("plain_fp64", "fp64", "exact", "PBiCG")]
    if args.served_pbicg_inner:
        forms.insert(1, ("mixed_pbicg_inner", "mixed", "colour", "PBiCG"))
    out["forms"] = {f[0]: {"precision": f[1], "ordering": f[2], "sym_solver": "PCG+DIC",
                           "asym_solver": (f[3].replace("-fp64", "") + "+DILU FP64" if f[3].endswith("-fp64")
                                           else f[3] + "+DILU")}
                    for f in forms}

    def server(prec, order, asym_solver):
        kw = dict(tol=TOL, max_iter=20000, ordering=order, inner_rel_tol=args.inner_tol,
                  iters_per_launch=args.served_k)
        aprec = "fp64" if asym_solver.endswith("-fp64") else prec
        return mrgpu.Server(ctx, mrgpu.controls(solver="PCG", precond="DIC", precision=prec, **kw),
                            mrgpu.controls(solver=asym_solver.replace("-fp64", ""), precond="DILU", precision=aprec,
                                           **kw), hbm_budget=150 * 2**30)

    order_req = [(i, k) for k in range(args.served_steps) for i in range(len(specs))]
    xbuf = [np.empty(m.n) for m in meshes]          # a mesh's steps run one after another
    xs = {}
    by_rate = {}
    for name, prec, order, asym_solver in forms:
        srv = server(prec, order, asym_solver)      # warm-up: every mesh once
        wid = [srv.submit(meshes[i], steps[i][0]["b"], steps[i][0]["x0"], steps[i][0]["diag"],
                          steps[i][0]["upper"], steps[i][0]["lower"], asym=asym[i], x_out=xbuf[i])
               for i in range(len(specs))]
        for r in wid:
            srv.wait(r, 600000.0)
        srv.close()
        form_rates = plain_rates if name == "plain_fp64" else rates
        for ri, rate in enumerate(form_rates):
            arrivals = np.cumsum(np.random.default_rng((SEED, 11, rates.index(rate) if rate in rates else ri))
                                 .exponential(1.0 / rate, n_req))
            keep = ri == len(form_rates) - 1
            srv = server(prec, order, asym_solver)
            ids = []
            t0 = time.perf_counter()
            for (i, k), ta in zip(order_req, arrivals):
                dt = ta - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                st = steps[i][k]
                xo = np.empty(meshes[i].n) if (keep and sample[i] == k) else xbuf[i]
                ids.append(srv.submit(meshes[i], st["b"], st["x0"], st["diag"], st["upper"], st["lower"],
                                      asym=asym[i], x_out=xo))
            lat, conv, unconv = [], 0, []
            for (i, k), r in zip(order_req, ids):
                x, p, l = srv.wait(r, 600000.0)
                lat.append(l)
                conv += p["converged"]
                if not p["converged"]:
                    unconv.append({"mesh": i, "step": k, "cells": meshes[i].n, "asym": bool(asym[i]),
                                   "iters": int(p["n_iter"]), "final_residual": p["final_residual"]})
                if keep and sample[i] == k:
                    xs[(name, i, k)] = x
            wall = time.perf_counter() - t0
            stt = srv.stats()
            srv.close()
            log(f"served {name} rate {rate:g}: {len(ids) / wall:.1f} solves/s, wall {wall:.1f} s")
            by_rate.setdefault(f"{rate:g}", {})[name] = {
                "solves_per_s": len(ids) / wall, "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "converged": int(conv), "not_converged": unconv[:5],
                "peak_running": stt["peak_running"], "peak_inflight_gb": stt["peak_inflight_bytes"] / 2**30}
    for r in by_rate.values():
        if "mixed" in r and "plain_fp64" in r:
            r["speedup_mixed_vs_plain"] = r["mixed"]["solves_per_s"] / r["plain_fp64"]["solves_per_s"]
    out["by_rate"] = by_rate
    # The plain drop-in solver as foam would call it: one request at a time,
    # device-resident, FP64 in foam's order.  Timed on the first time step of
    # every mesh (the request mix's sizes and families) and reported as
    # requests per second of solve time.
    plain_ms = []
    for i in range(len(specs)):
        st = steps[i][0]
        ctl = mrgpu.controls(tol=TOL, max_iter=20000, solver="PBiCG" if asym[i] else "PCG",
                             precond="DILU" if asym[i] else "DIC", precision="fp64", ordering="exact")
        meshes[i].upload(st["diag"], st["upper"], st["lower"])
        d_b, d_x = ctx.to_device(st["b"]), ctx.to_device(st["x0"])
        meshes[i].solve_device(d_b, d_x, ctl)          # warm (plan, graphs)
        ctx.dev_free(d_x)
        d_x = ctx.to_device(st["x0"])
        ctx.record(52)
        meshes[i].solve_device(d_b, d_x, ctl)
        ctx.record(53)
        plain_ms.append(ctx.elapsed_ms(52, 53))
        ctx.dev_free(d_b)
        ctx.dev_free(d_x)
    seq_rate = len(plain_ms) / (sum(plain_ms) * 1e-3)
    out["plain_fp64_one_at_a_time"] = {"solves_per_s": seq_rate, "requests_timed": len(plain_ms),
                                       "mean_ms": float(np.mean(plain_ms))}
    top = by_rate[f"{rates[-1]:g}"]
    out["speedup_served_mixed_vs_plain_one_at_a_time"] = top["mixed"]["solves_per_s"] / seq_rate
    out["asym_of_mesh"] = [bool(a) for a in asym]
    for m in meshes:
        m.close()
    return out, xs


def run_gpu(args):
    from multiregionfoam_gb300 import _build, mrgpu
    rank, world, local, dist = dist_setup(args.gpus)
    _build.build()
    L = mrgpu.load()
    s = make_system(rank, args.scale)
    n, nf = s.n, s.nf
    ctx = mrgpu.Context(local)
    mesh = mrgpu.Mesh(ctx, n, s.lower, s.upper)
    d_diag, d_up = ctx.to_device(s.diag), ctx.to_device(s.upper_c)
    d_b, d_x0 = ctx.to_device(s.b), ctx.to_device(s.x0)
    d_x = ctx.dev_alloc(8 * n)
    mixed = mrgpu.controls(tol=TOL, max_iter=20000, solver="PCG", precond="DIC", precision="mixed",
                           ordering="colour", inner_rel_tol=args.inner_tol)
    plain = mrgpu.controls(tol=TOL, max_iter=20000, solver="PCG", precond="DIC", precision="fp64",
                           ordering="exact")

    def step(ctl):
        mesh.upload_device(d_diag, d_up)
        ctx.copy_d2d(d_x, d_x0, 8 * n)
        return mesh.solve_device(d_b, d_x, ctl)

    def timed(ctl, k, slot0):
        barrier(dist)
        ctx.record(slot0)
        perfs = []
        for i in range(k):
            perfs.append(step(ctl))
            ctx.record(slot0 + 1 + i)
        tot = ctx.elapsed_ms(slot0, slot0 + k)
        per = [ctx.elapsed_ms(slot0 + i, slot0 + i + 1) for i in range(k)]
        return tot, per, perfs

    # autotune the launch shapes of both forms (never changes a result bit)
    ctx.copy_d2d(d_x, d_x0, 8 * n)
    mesh.upload_device(d_diag, d_up)
    tuning = {"mixed": mesh.tune(d_b, d_x, mixed), "plain_fp64": mesh.tune(d_b, d_x, plain)}
    for _ in range(args.warmup):
        step(mixed)
    for _ in range(min(args.warmup, 2)):
        step(plain)

    clocks = Clocks(local)
    l0 = mrgpu.kernel_launches()
    tot_mixed, per_mixed, perf_mixed = timed(mixed, args.steps, 0)
    launches = mrgpu.kernel_launches() - l0
    x_mixed = ctx.from_device(d_x, np.empty(n))
    k_plain = max(1, min(args.steps, args.plain_steps))
    tot_plain, per_plain, perf_plain = timed(plain, k_plain, 42)
    clk = clocks.stop()
    x_plain = ctx.from_device(d_x, np.empty(n))
    tot_mixed = max_over_ranks(dist, tot_mixed)
    tot_plain = max_over_ranks(dist, tot_plain)

    # e2e through the host-pointer ABI from pinned memory
    h_diag = mrgpu.host_array(None, n); h_diag[:] = s.diag
    h_up = mrgpu.host_array(None, nf); h_up[:] = s.upper_c
    h_b = mrgpu.host_array(None, n); h_b[:] = s.b
    h_x = mrgpu.host_array(None, n)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    perf = mrgpu.Perf()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        h_x[:] = s.x0
        barrier(dist)
        ctx.record(40)
        mrgpu._check(L.mrg_coeffs_upload(mesh.h, dp(h_diag), dp(h_up), None, None, None))
        mrgpu._check(L.mrg_solve(mesh.h, dp(h_b), dp(h_x), C.byref(mixed), C.byref(perf)))
        ctx.record(41)
        if i >= args.warmup:
            e2e_ms.append(ctx.elapsed_ms(40, 41))
    e2e_tot = max_over_ranks(dist, float(np.sum(e2e_ms)))
    x_e2e = h_x.copy()

    # dominant-kernel roofline: Amul + (q,p) of the FP32 inner loop
    peak, peak_kind = peaks()
    step(mixed)
    ms_spmv32 = mesh.time_kernel(mixed, 0, 50)
    ms_prec32 = mesh.time_kernel(mixed, 1, 20)
    step(plain)
    ms_spmv64 = mesh.time_kernel(plain, 0, 50)
    ms_prec64 = mesh.time_kernel(plain, 1, 5)
    bytes32 = 12 * n + 12 * nf          # FP32 values, int32 addressing (sym)
    bytes64 = 24 * n + 16 * nf
    ach32 = bytes32 / (ms_spmv32 * 1e-3) / 1e9
    ach64 = bytes64 / (ms_spmv64 * 1e-3) / 1e9
    traffic = profile_traffic("spmv_fp32_c2.txt")
    mesh.close()
    for a in (d_diag, d_up, d_b, d_x0, d_x):
        ctx.dev_free(a)

    log("headline done")
    c3, x_c3 = run_c3(args, ctx, mrgpu) if args.c3_scale > 0 else (None, {})
    log("c3 done")
    batched, x_c4 = run_batched(args, ctx, mrgpu) if args.batched > 0 else (None, {})
    log("batched done")
    block, x_block = run_block(args, ctx, mrgpu) if args.block_n > 0 else (None, {})
    log("block done")
    gamg = run_gamg(args, ctx, mrgpu) if args.gamg_n > 0 else None
    log("gamg done")
    served, x_c5 = run_served(args, ctx, mrgpu) if args.served_meshes > 0 else (None, {})
    log("served done")
    ctx.close()

    if rank != 0:
        return
    k = args.steps
    value = world * k / (tot_mixed * 1e-3)
    plain_rate = world * k_plain / (tot_plain * 1e-3)

    # CPU leg: the measured baseline, then the FP64 oracle solutions every
    # GPU result is checked against
    cpu, refs = None, {}
    if world == 1 and not args.no_cpu:
        leg = CpuLeg()
        cpu = cpu_baseline(args.scale, leg)
        log("cpu baseline done")
        jobs = [("c2", args.scale)]
        if c3 is not None:
            jobs.append(("c3", args.c3_scale))
        c5_every = max(1, args.ref_every // 2)
        jobs += [("c5", args.served_meshes, i, st) for (_, i, st) in x_c5 if _ == "mixed" and i % c5_every == 0]
        if block is not None:
            jobs.append(("block", args.block_n))
        if batched is not None:
            jobs += [("c4", args.batched, i) for i in range(0, args.batched, args.ref_every)]
        t0 = time.perf_counter()
        refs = leg.references(jobs)
        leg.close()
        cpu["references_s"] = time.perf_counter() - t0
        log("oracle references done")

    def err(key, x):
        return rel_err(x, refs[key][0]) if key in refs else None

    pm, pp = perf_mixed[-1], perf_plain[-1]
    rc2 = refs.get(("c2", args.scale))
    if c3 is not None:
        for f in ("plain_fp64", "mixed", "mixed_pbicg_inner"):
            c3[f]["err_vs_fp64_oracle"] = err(("c3", args.c3_scale), x_c3[f])
        if ("c3", args.c3_scale) in refs:
            p3 = refs[("c3", args.c3_scale)][1]
            c3["fp64_oracle"] = {"kind": "CPU oracle, foam order", "tolerance": REF_TOL, "iters": p3["n_iter"]}
    if batched is not None:
        for f in ("mixed", "plain_fp64"):
            batched[f]["err_vs_fp64_oracle"] = err_stats(
                [err(("c4", args.batched, i), x) for i, x in enumerate(x_c4[f])])
    if block is not None:
        for f in ("mixed", "plain_fp64", "block_cholesky"):
            block[f]["err_vs_fp64_oracle"] = err(("block", args.block_n), x_block[f])
    if served is not None:
        fam = served.pop("asym_of_mesh")
        served["err_vs_fp64_oracle"] = {
            "sample": f"one request per {max(1, args.ref_every // 2)}-th mesh (time step mesh % steps) of the last "
                      f"rate's runs; the FP64 oracle converged to {REF_TOL_MANY:g}",
            **{f"{f}_{kind}": err_stats([err(("c5", args.served_meshes, i, st), x) for (ff, i, st), x in x_c5.items()
                                         if ff == f and fam[i] == (kind == "asym")])
               for f in ("mixed", "plain_fp64") for kind in ("sym", "asym")}}

    line = {
        "metric": "coupled solves/s at 1e-8 rel. residual", "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": k, "warmup": args.warmup, "ms_per_step": tot_mixed / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64",
        "data": "synthetic (seeded C2 system)",
        "config": {"workload": "cht-2region-128^3+128x128x64", "n_cells": n, "n_faces": nf,
                   "tolerance": TOL, "form": "mixed FP32 PCG + colour DIC inside FP64 refinement",
                   "l2": "inputs larger than L2 (~1 GB working set)", "parallelism": f"replicas x{world}"},
        "p50_ms": float(np.percentile(per_mixed, 50)), "p99_ms": float(np.percentile(per_mixed, 99)),
        "mixed": {"iters": pm["n_iter"], "outer": pm["n_outer"], "final_residual": pm["final_residual"],
                  "converged": pm["converged"], "rel_err_vs_plain": rel_err(x_mixed, x_plain),
                  "err_vs_fp64_oracle": err(("c2", args.scale), x_mixed),
                  "e2e_err_vs_fp64_oracle": err(("c2", args.scale), x_e2e)},
        "fp64_oracle": None if rc2 is None else {
            "kind": "CPU oracle (foam order, C)", "tolerance": REF_TOL, "iters": rc2[1]["n_iter"],
            "final_residual": rc2[1]["final_residual"], "note": "max-norm errors relative to this FP64 solution"},
        "plain_fp64": {"value": plain_rate, "unit": "solves/s", "ms_per_step": tot_plain / k_plain,
                       "iters": pp["n_iter"], "final_residual": pp["final_residual"],
                       "err_vs_fp64_oracle": err(("c2", args.scale), x_plain),
                       "p50_ms": float(np.percentile(per_plain, 50)), "p99_ms": float(np.percentile(per_plain, 99)),
                       "steps": k_plain},
        "speedup_mixed_vs_plain": value / plain_rate,
        "e2e": {"value": world * k / (e2e_tot * 1e-3), "unit": "solves/s",
                "h2d_bytes_per_step": 8 * (n + nf) + 16 * n, "d2h_bytes_per_step": 8 * n,
                "p99_ms": float(np.percentile(e2e_ms, 99))},
        "roofline": {"kernel": "Amul+(q,p) FP32 (mixed inner loop)", "bound": "hbm", "achieved": ach32,
                     "peak": peak, "unit": "GB/s", "frac": ach32 / peak, "traffic": traffic,
                     "algorithmic_bytes": bytes32, "ms_per_launch": ms_spmv32, "peak_source": peak_kind},
        "kernels": {"spmv_fp64": {"ms": ms_spmv64, "GB/s": ach64, "frac": ach64 / peak},
                    "precondition_fp32_colour_ms": ms_prec32, "precondition_fp64_exact_ms": ms_prec64},
        "tuning": tuning,
        "c3": c3,
        "batched": batched,
        "block": block,
        "gamg": gamg,
        "served": served,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=1, help="divide the mesh dimensions (testing only)")
    ap.add_argument("--plain-steps", type=int, default=3, help="timed plain FP64 steps (at most 5)")
    ap.add_argument("--inner-tol", type=float, default=1e-5)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the oracle errors")
    ap.add_argument("--c3-scale", type=int, default=1, help="asymmetric GGI configuration: 96/scale (0: skip)")
    ap.add_argument("--c3-reps", type=int, default=3)
    ap.add_argument("--batched", type=int, default=512, help="systems of the batched configuration (0: skip)")
    ap.add_argument("--batched-reps", type=int, default=2)
    ap.add_argument("--block-n", type=int, default=48, help="4x4 block configuration: n^3 cells (0: skip)")
    ap.add_argument("--gamg-n", type=int, default=64, help="GAMG configuration: n^3 cells (0: skip)")
    ap.add_argument("--served-meshes", type=int, default=100, help="meshes of the served configuration (0: skip)")
    ap.add_argument("--served-steps", type=int, default=20)
    ap.add_argument("--served-rates", default="200,2000",
                    help="Poisson arrival rates of the mixed server's sweep, requests/s (the full C5 sweep: "
                         "50,100,200,500,1000,2000)")
    ap.add_argument("--served-plain-rates", default="2000",
                    help="arrival rates of the plain FP64 server's sweep (empty: --served-rates)")
    ap.add_argument("--ref-every", type=int, default=8,
                    help="FP64 oracle errors for every n-th batched system and every (n/2)-th served mesh")
    ap.add_argument("--served-k", type=int, default=8, help="server: Krylov iterations per launch")
    ap.add_argument("--served-pbicg-inner", action="store_true",
                    help="also serve with mixed FP32 PBiCG for the asymmetric requests")
    ap.add_argument("--served-mixed-asym", action="store_true",
                    help="serve the asymmetric requests with mixed FP32 BiCGStab (default: FP64 PBiCG + colour DILU)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.steps > 39 or args.plain_steps > 5:
        ap.error("--steps at most 39 and --plain-steps at most 5 (CUDA event slots of the timing)")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
