#!/usr/bin/env python
"""Benchmark of the operator path (assembly + H-matrix application) on one GB300.

Default workload: Helmholtz Burton-Miller at kappa = 8 on the ellipsoid with semi-axes
(1, 0.7, 0.5) at icosphere level 6 (81920 triangles), P1 trace space (40962 complex dofs),
H-matrix leaf 20, eta = 2, ACA eps = 1e-8, intorder 3, 32 incident plane waves (directions
uniform on the sphere, seeded).  Synthetic data: mesh and right-hand sides are generated.

A step is one application Y = C X of the combined-field H-matrix to the 32 right-hand sides
(the product every batched-GMRES iteration makes) in mixed precision: complex64 factors,
split-TF32 tcgen05 products with FP32 accumulation.  X and the operator are resident in HBM;
L2 is flushed before every step (a 512 MiB write, then a 512 MiB read of a second buffer, so
that the write-back of the flush's dirty lines does not land inside the step); each step is
timed with CUDA events on the launch stream.  value = single-right-hand-side H-matvecs per
second (32 per step) over all ranks.  e2e = the same step through the host-buffer C-ABI entry
point (page-locked X and Y, staged by one bulk copy each way).

The same line carries the metric's other half and its comparators: assembly seconds of the
mixed and the plain FP64 GPU path, the batched 32-right-hand-side solve of both paths, the
FP64 path's application rate, the solution error of the mixed path against the FP64 path,
the products' errors against the FP64 path and the FP64 oracle, the roofline of the
tensor-core GEMM kernels and the FP64 oracle on the host cores (cpu_baseline).

--impl reference times the reference algorithm's CPU implementation (the FP64 C++ oracle, all
host threads: the combined-field H-matrix assembled on the host cores, then per step its
product with a bounded sample of the 32 right-hand sides, one vector at a time as the
reference's HMatrix::Mult does) and prints the same JSON line with impl=reference.  That arm
loads only the oracle's library: the mesh and right-hand-side generators are loaded from their
source files without the package (whose import loads the CUDA library).

--workload dtn (Laplace Dirichlet-to-Neumann, icosphere level 5, single-vector V matvec),
shape (batched energy + shape gradient) and maxwell (EFIE on RT0) print secondary lines.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly s + H-matvec/s at 1e-6 rel.err vs FP64 plain path, 1 GB300"
SEED = 20261203 + 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=None, help="mesh level (bm: 6, dtn: 5, maxwell: 5)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-path comparison")
    ap.add_argument("--no-gmres", action="store_true", help="skip the DtN GMRES solve (profiling runs)")
    ap.add_argument("--workload", default="bm", choices=["bm", "dtn", "shape", "maxwell"],
                    help="bm: Helmholtz Burton-Miller kappa 8 on the L6 ellipsoid, 32 plane waves (default, "
                         "the headline); dtn: Laplace DtN on the L5 icosphere, single-vector V matvec; shape: "
                         "batched single-layer energy + adjoint shape gradient over 64 perturbed icospheres "
                         "(L2..L5); maxwell: EFIE on RT0 of the L5 icosphere")
    ap.add_argument("--apply-only", action="store_true",
                    help="bm: assemble the mixed operator, then only the warm-up and timed applications "
                         "(profiling runs: no FP64 path, no solves, no host-buffer steps)")
    ap.add_argument("--ref-sample", type=int, default=4,
                    help="bm reference arm: right-hand sides per step (the oracle applies one vector at a time)")
    ap.add_argument("--l2-flush", default="write+read", choices=["write+read", "write"],
                    help="before every step: write a 512 MiB buffer, then (default) read another 512 MiB "
                         "buffer so that the write-back of the dirty lines is not charged to the step")
    return ap.parse_args()


L2_NOTE = {"write+read": "flushed before every step: 512 MiB write, then 512 MiB read of another buffer "
                        "(no operator data and no dirty lines left in L2)",
           "write": "flushed before every step: 512 MiB write (dirty lines written back during the step)"}


def workload(level, l2="write+read"):
    return {"workload": f"laplace_dtn_icosphere_L{level}", "mesh": f"unit icosphere level {level}",
            "triangles": 20 * 4 ** level, "V": "laplace SL P0->P0", "K": "laplace DL P1->P0",
            "leafsize": 20, "eta": 2.0, "eps": 1e-8, "intorder": 3, "precision": "mixed",
            "step": "one H-matvec y = V x", "l2": L2_NOTE[l2],
            "gmres": "V u = (M/2 + K) g, g = x^2 - y^2, tol 1e-8, CUDA graph"}


BM_KAPPA, BM_NRHS, BM_AXES = 8.0, 32, (1.0, 0.7, 0.5)
BM_OPTS = dict(intorder=3, leafsize=20, eta=2.0, eps=1e-8)
BM_SEED = SEED + 3


def bm_workload(level, l2="write+read"):
    nt = 20 * 4 ** level
    return {"workload": f"helmholtz_bm_ellipsoid_L{level}_kappa8_32rhs",
            "mesh": f"ellipsoid, semi-axes (1, 0.7, 0.5), icosphere level {level}", "triangles": nt,
            "dofs": nt // 2 + 2, "space": "P1 (H1 order 1), complex",
            "operator": "Helmholtz combined field C = K - i kappa V; system (M/2 + C) u = f",
            "kappa": BM_KAPPA, "nrhs": BM_NRHS,
            "rhs": "32 incident plane waves exp(i kappa d.x), d uniform on the sphere (seeded)",
            "leafsize": 20, "eta": 2.0, "eps": 1e-8, "intorder": 3,
            "precision": "mixed: FP64 Sauter-Schwab pairs; complex64 regular near field, ACA and factors; "
                         "split-TF32 tensor-core products, FP32 accumulation",
            "step": "one application Y = C X to the 32 right-hand sides (the batched-GMRES product)",
            "l2": L2_NOTE[l2], "gmres": "batched, 32 right-hand sides in lockstep, tol 1e-8, restart 100"}


def assembly_rates(info):
    """Kernel evaluations per second of the two assembly phases that dominate (from the
    operator's counters and its CUDA-event phase times).  ACA counts, per far block and kernel
    component, (steps + 1) x (row + column points) evaluations; the near field counts its
    regular pairs x nq^2 (its time also holds the Sauter-Schwab pairs, which run concurrently
    in the same phase)."""
    r = {"aca_evals": info["aca_evals"], "nf_regular_evals": info["nf_regular_evals"],
         "n_singular_pairs": info["n_singular_pairs"]}
    if info["ms_aca"] > 0:
        r["aca_evals_per_s"] = info["aca_evals"] / (info["ms_aca"] * 1e-3)
    if info["ms_nearfield"] > 0:
        r["nf_regular_evals_per_s"] = info["nf_regular_evals"] / (info["ms_nearfield"] * 1e-3)
    return r


def bm_rhs(meshes, forms, level):
    """The ellipsoid and its 32 Burton-Miller plane-wave load vectors (n x 32, complex128)."""
    mesh = meshes.ellipsoid(level, BM_AXES)
    d = forms.random_directions(BM_NRHS, BM_SEED)
    return mesh, forms.p1_load_vector(mesh, forms.plane_wave_bm_source(BM_KAPPA, d), order=6)


def traffic_from_profile(kernel, summary="mv_fused_kernel_laplace_dtn_L5.md"):
    """DRAM bytes per launch of `kernel` from a committed ncu summary (profiles/), or None.

    The summary holds a line 'traffic_bytes_per_launch <kernel-name> <bytes>' taken from
    dram__bytes_read.sum + dram__bytes_write.sum of one capture of the same workload."""
    name = kernel.split()[0]
    path = os.path.join(ROOT, "profiles", summary)
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.strip().strip("`").split()
        if len(f) == 3 and f[0] == "traffic_bytes_per_launch" and f[1] == name:
            return float(f[2])
    return None


def _pure_modules():
    """ngbem_gb300/meshes.py and forms.py loaded from their source files, without the package's
    __init__ (which loads the CUDA library): the reference arm maps no library of this repo
    except the oracle's."""
    import importlib.util
    import types
    pkg_name = "_ngbem_sources"
    if pkg_name not in sys.modules:
        pkg = types.ModuleType(pkg_name)
        pkg.__path__ = [os.path.join(ROOT, "ngbem_gb300")]
        sys.modules[pkg_name] = pkg
    out = []
    for m in ("meshes", "forms"):
        full = f"{pkg_name}.{m}"
        if full not in sys.modules:
            spec = importlib.util.spec_from_file_location(full, os.path.join(ROOT, "ngbem_gb300", m + ".py"))
            mod = importlib.util.module_from_spec(spec)
            sys.modules[full] = mod
            spec.loader.exec_module(mod)
        out.append(sys.modules[full])
    return tuple(out)


class ClockSampler:
    """nvidia-smi clocks sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.idx), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
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
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of timings over all ranks of the process group (the
    values themselves when there is no group): the whole job takes as long as its slowest
    replica."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t]


def whole_job_rate(world, units_per_rank, seconds):
    """Units processed by all ranks per second of the slowest rank (replicas: every rank does
    the same work)."""
    return world * units_per_rank / seconds


# ---------------------------------------------------------------------------------------------
def cpu_reference(level, nthreads=0, steps=20, warmup=2):
    """Oracle (FP64 C++ restatement of the reference, all host threads): assembly of V and
    matvec throughput on the Laplace DtN workload."""
    import numpy as np
    from oracle import pyoracle as O
    meshes, _ = _pure_modules()
    O.build()
    m = meshes.icosphere(level)
    t0 = time.perf_counter()
    V = O.OracleOperator("laplace_sl", m, "P0", intorder=3, leafsize=20, eta=2.0, eps=1e-8, nthreads=nthreads)
    t_asm = time.perf_counter() - t0
    x = np.random.default_rng(SEED).standard_normal(V.width)
    for _ in range(warmup):
        V.mult(x)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        V.mult(x)
        times.append(time.perf_counter() - t)
    cores = nthreads or os.cpu_count()
    return {"matvec_per_s": steps / sum(times), "assembly_s": t_asm, "cores": cores, "nze": V.nze,
            "ms_per_step": 1e3 * sum(times) / steps, "oracle": V, "x": x}


def cpu_reference_bm(level, sample, steps, warmup, nthreads=0):
    """Oracle on the Burton-Miller workload: the combined-field H-matrix assembled on all host
    threads (CalcHMatrix restated), then per step its product with `sample` of the 32
    right-hand sides, one vector at a time (HMatrix::Mult restated), cycling through them."""
    from oracle import pyoracle as O
    meshes, forms = _pure_modules()
    O.build()
    mesh, X = bm_rhs(meshes, forms, level)
    t0 = time.perf_counter()
    Cop = O.OracleOperator("helmholtz_cf", mesh, "P1", kappa=BM_KAPPA, nthreads=nthreads, **BM_OPTS)
    t_asm = time.perf_counter() - t0
    ys = {}

    def step(k):
        for c in range(sample):
            col = (k * sample + c) % X.shape[1]
            ys[col] = Cop.mult(X[:, col])

    for k in range(warmup):
        step(k)
    times = []
    for k in range(steps):
        t = time.perf_counter()
        step(warmup + k)
        times.append(time.perf_counter() - t)
    cores = nthreads or os.cpu_count()
    return {"matvec_per_s": steps * sample / sum(times), "assembly_s": t_asm, "cores": cores, "nze": Cop.nze,
            "max_rank": Cop.max_rank, "nfallback": Cop.nfallback, "ms_per_step": 1e3 * sum(times) / steps,
            "products": ys, "X": X}


def run_reference(args):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    if args.workload == "bm":
        L = args.level or 6
        r = cpu_reference_bm(L, args.ref_sample, args.steps, args.warmup)
        cfg = bm_workload(L, args.l2_flush)
        sample = (f"oracle FP64 assembly of C on {r['cores']} threads ({r['assembly_s']:.1f} s, untimed), then per "
                  f"step C applied to {args.ref_sample} of the 32 right-hand sides, one vector at a time")
        extra = {"assembly_s": r["assembly_s"], "nze": r["nze"], "max_rank": r["max_rank"],
                 "nfallback": r["nfallback"]}
    else:
        L = args.level or 5
        r = cpu_reference(L, 0, steps=args.steps, warmup=args.warmup)
        cfg = workload(L, args.l2_flush)
        sample = f"full workload: oracle assembly of V ({r['assembly_s']:.2f} s) then {args.steps} timed matvecs"
        extra = {"assembly_s": r["assembly_s"], "nze": r["nze"]}
    v = r["matvec_per_s"]
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "matvec/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.workload == "bm"
            else "f64", "data": "synthetic", "config": cfg, **extra,
            "cpu_baseline": {"value": v, "unit": "matvec/s", "cores": r["cores"], "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "matvec/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def dtn_solve(nb, mesh, P0, P1, V, K, V64, K64, dev, acc):
    """Dirichlet-to-Neumann solve V u = (M/2 + K) g for g = x^2 - y^2 (exact u = 2 g on the sphere)."""
    import numpy as np
    import torch
    M = nb.MassOperator(P1, P0)
    vt = mesh.vertices
    g = torch.from_numpy(vt[:, 0] ** 2 - vt[:, 1] ** 2).to(dev)
    rhs = (0.5 * M + K.mat) * g
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = nb.GMRes(V.mat, rhs, maxsteps=500, tol=1e-8, restart=500)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    gm = dict(nb.GMRes.last)
    c = mesh.centroids()
    c = c / np.linalg.norm(c, axis=1)[:, None]
    exact = 2.0 * (c[:, 0] ** 2 - c[:, 1] ** 2)
    areas = mesh.areas()
    uh = u.cpu().numpy()
    gm["solve_s"] = t_solve
    gm["l2_err_vs_exact"] = float(np.sqrt(np.sum(areas * (uh - exact) ** 2) / np.sum(areas * exact ** 2)))
    if V64 is not None:
        rhs64 = (0.5 * M + K64.mat) * g
        u64 = nb.GMRes(V64.mat, rhs64, maxsteps=500, tol=1e-8, restart=500)
        acc["solution_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(u - u64) / torch.linalg.vector_norm(u64))
        gm["iterations_fp64"] = nb.GMRes.last["iterations"]
    return gm


# ---------------------------------------------------------------------------------------------
def run_dtn(args):
    import numpy as np
    import torch

    import ngbem_gb300 as nb

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    L = args.level or 5
    mesh = nb.icosphere(L)
    P0 = nb.SurfaceL2(mesh, order=0)
    P1 = nb.H1(mesh, order=1)
    opts = dict(intorder=3, leafsize=20, eta=2.0, eps=1e-8)

    # ---- assembly (mixed precision): one warm-up construction, then timed constructions
    def assemble(prec):
        # fresh spaces: the cluster trees (cached per space) are built inside the timed region;
        # V and K share the P0 tree as they share the space
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P0a, P1a = nb.SurfaceL2(mesh, order=0), nb.H1(mesh, order=1)
        V = nb.SingleLayerPotentialOperator(P0a, precision=prec, **opts)
        K = nb.DoubleLayerPotentialOperator(P1a, P0a, precision=prec, **opts)
        torch.cuda.synchronize()
        return V, K, time.perf_counter() - t0

    V, K, _ = assemble("mixed")
    del V, K
    asm = []
    for _ in range(2):
        V, K, t = assemble("mixed")
        asm.append(t)
    assembly_s = min(asm)
    info_V, info_K = V.mat.info, K.mat.info

    # matvec decomposition picked by the autotuner (piece size, single launch or four passes)
    tuned = V.mat.autotune(reps=10)

    rng = np.random.default_rng(SEED)
    x_h = rng.standard_normal(P0.ndof)
    x = torch.from_numpy(x_h).to(dev)
    acc = {}
    # the timed matvec is the one GMRES iterates with: FP32 storage, plain FP32 arithmetic
    V.mat.set_accuracy(False)
    K.mat.set_accuracy(False)
    if not args.no_fp64:
        V64, K64, t64 = assemble("fp64")
        acc["assembly_s_fp64"] = t64
        y32 = V.mat * x
        y64 = V64.mat * x
        acc["V_matvec_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(y32 - y64) / torch.linalg.vector_norm(y64))
        V.mat.set_accuracy(True)
        yc = V.mat * x
        acc["V_matvec_compensated_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(yc - y64) /
                                                            torch.linalg.vector_norm(y64))
        V.mat.set_accuracy(False)
        xk = torch.from_numpy(rng.standard_normal(P1.ndof)).to(dev)
        k32, k64 = K.mat * xk, K64.mat * xk
        acc["K_matvec_rel_err_vs_fp64"] = float(torch.linalg.vector_norm(k32 - k64) / torch.linalg.vector_norm(k64))

    # ---- DtN solve: V u = (M/2 + K) g
    gm = {}
    if not args.no_gmres:
        gm = dtn_solve(nb, mesh, P0, P1, V, K, V64 if not args.no_fp64 else None,
                       K64 if not args.no_fp64 else None, dev, acc)
    if not args.no_fp64:
        del V64, K64
    # ---- timed steps: y = V x, L2 flushed before each step, CUDA events on the stream
    y = V.mat.CreateColVector()
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    sweep = torch.zeros(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev) if args.l2_flush == "write+read" else None
    sweep_out = torch.zeros((), dtype=torch.float32, device=dev)

    def flush_l2():
        flush.fill_(1.0)
        if sweep is not None:
            torch.amax(sweep, dim=0, out=sweep_out)

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        flush_l2()
        V.mat.Mult(x, y)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush_l2()
        evs[k][0].record(stream)
        V.mat.Mult(x, y)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    dev_ms = sum(step_ms)
    # kernel times from a separate, untimed pass with the operator's event profiling on
    V.mat.set_profiling(True)
    for _ in range(min(args.steps, 20)):
        flush_l2()
        V.mat.Mult(x, y)
    torch.cuda.synchronize()
    kms, kcount = V.mat.kernel_times()
    V.mat.set_profiling(False)
    per_step_launches = sum(kcount) / max(1, min(args.steps, 20))
    # the same steps with the compensated (error-free) arithmetic used for GMRES residuals
    V.mat.set_accuracy(True)
    for _ in range(2):
        V.mat.Mult(x, y)
    cms = []
    for k in range(min(args.steps, 20)):
        flush_l2()
        evs[k][0].record(stream)
        V.mat.Mult(x, y)
        evs[k][1].record(stream)
        cms.append(evs[k])
    torch.cuda.synchronize()
    comp_ms = sum(a.elapsed_time(b) for a, b in cms) / len(cms)
    V.mat.set_accuracy(False)

    # ---- e2e: host pinned buffers through bem_operator_mult_host
    xh = torch.from_numpy(x_h).pin_memory()
    yh = torch.zeros(P0.ndof, dtype=torch.float64).pin_memory()
    xh_np, yh_np = xh.numpy(), yh.numpy()
    for _ in range(args.warmup):
        V.mat.mult_host(xh_np, y=yh_np)
    e2e_t = []
    for _ in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t = time.perf_counter()
        V.mat.mult_host(xh_np, y=yh_np)
        e2e_t.append(time.perf_counter() - t)
    clocks = sampler.stop()
    e2e_check = float(np.linalg.norm(yh_np - y.cpu().numpy()) / np.linalg.norm(y.cpu().numpy()))

    dev_ms, e2e_sum = max_over_ranks([dev_ms, sum(e2e_t)], dev)
    value = whole_job_rate(world, args.steps, dev_ms / 1e3)
    e2e_value = whole_job_rate(world, args.steps, e2e_sum)

    # ---- roofline of the dominant kernel (apply: dense near field + U2 t)
    import json as _j
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(_j.load(open(peaks_path))["hbm_gbs"]), "measured"
    iv = info_V
    vs = 4  # fp32 storage
    n, m = V.mat.width, V.mat.height
    # algorithmic bytes of one matvec: the stored blocks once, x read once, y written once (FP64)
    matvec_bytes = iv["bytes_dense"] + iv["bytes_lowrank"] + n * 8 + m * 8
    fused = kcount[1] == 0 and kcount[2] > 0
    if fused:
        # one cooperative launch per matvec (mv_fused_kernel): the whole matvec is the kernel
        kernel, alg_bytes = "mv_fused_kernel", matvec_bytes
        launch_ms = kms[2] / kcount[2]
        extra = {}
    else:
        kernel = "mv_tma_kernel (apply pass)"
        alg_bytes = iv["bytes_dense"] + iv["bytes_lowrank_u"] + n * vs + iv["sum_rank"] * vs + m * 8
        stage1_bytes = (iv["bytes_lowrank"] - iv["bytes_lowrank_u"]) + n * vs + iv["sum_rank"] * vs
        launch_ms = kms[2] / max(kcount[2], 1)
        stage1_ms = kms[1] / max(kcount[1], 1)
        extra = {"stage1_GBps": stage1_bytes / (stage1_ms * 1e-3) / 1e9, "stage1_avg_ms": stage1_ms}
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic_from_profile(kernel),
                "algorithmic_bytes": alg_bytes, "avg_launch_ms": launch_ms,
                "matvec_GBps": matvec_bytes / (dev_ms / args.steps * 1e-3) / 1e9, **extra}
    launches = int(round(per_step_launches * args.steps))

    line = {"metric": METRIC, "value": value, "unit": "matvec/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload(L, args.l2_flush), "assembly_s": assembly_s,
            "assembly_breakdown_ms": {"V": {k: iv[k] for k in ("ms_setup", "ms_aca", "ms_nearfield", "ms_projection", "ms_mvitems", "ms_total")},
                                      "K": {k: info_K[k] for k in ("ms_setup", "ms_aca", "ms_nearfield", "ms_projection", "ms_mvitems", "ms_total")}},
            "hmatrix": {"V": {k: iv[k] for k in ("nblocks", "nnear", "nfar", "nfallback", "nze", "max_rank",
                                                 "bytes_dense", "bytes_lowrank", "n_singular_pairs", "n_regular_pairs",
                                                 "mv_items", "mv_segments", "mv_ranges")},
                        "K": {k: info_K[k] for k in ("nblocks", "nfar", "nfallback", "nze", "max_rank")}},
            "accuracy": acc, "gmres": gm, "roofline": roofline, "gpu_launches": launches, "autotune": tuned,
            "matvec_compensated": {"value": 1e3 / comp_ms, "unit": "matvec/s",
                                   "note": "error-free FP32 products and sums (GMRES residuals)"},
            "wall_s_timed_region": t_wall, "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": "matvec/s", "h2d_bytes_per_step": P0.ndof * 8,
                    "d2h_bytes_per_step": P0.ndof * 8, "check_rel_err": e2e_check}}

    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_reference(L, 0, steps=10, warmup=1)
        # the oracle's matvec on the same x, against our FP64-accumulated mixed result
        yo = r["oracle"].mult(x_h)
        line["accuracy"]["V_matvec_rel_err_vs_oracle"] = float(np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo))
        line["cpu_baseline"] = {"value": r["matvec_per_s"], "unit": "matvec/s", "cores": r["cores"], "kind": "port",
                                "assembly_s": r["assembly_s"],
                                "sample": f"full workload: oracle FP64 assembly of V ({r['assembly_s']:.2f} s, "
                                          f"{r['cores']} threads) then 10 timed matvecs"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_shape(args):
    """Batched energy + gradient: 64 icospheres, levels 2..5 (16 each), radial noise
    0.05 N(0,1) (seeded), densities N(0,1), mixed precision; a step is one forward energy and
    one backward pass (dE/dX, dE/du) through the torch.autograd.Function, inputs resident on
    the device.  Each step touches only the 1.6 MB of coordinates and densities; the work is
    compute-bound (kernel evaluations), so L2 state is irrelevant."""
    import numpy as np
    import torch

    from ngbem_gb300.meshes import perturbed_icosphere
    from ngbem_gb300.shape import SingleLayerEnergyBatch

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    dev = torch.device("cuda", local)
    levels = [2, 3, 4, 5]
    meshes = [perturbed_icosphere(L, 0.05, SEED + 5 + 100 * L + k) for L in levels for k in range(16)]
    b = SingleLayerEnergyBatch(meshes, intorder=3, intorder_singular=4, precision="mixed")
    X0 = b.coordinates()
    g = torch.Generator().manual_seed(SEED + 5)
    u0 = torch.randn(b.nt_total, dtype=torch.float64, generator=g).to(dev)
    info = b.info()

    def step():
        X = X0.clone().requires_grad_(True)
        u = u0.clone().requires_grad_(True)
        E = b(X, u)
        E.sum().backward()
        return E, X.grad, u.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    # forward and backward separately, for the rates below
    fw = []
    for _ in range(3):
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        b.evaluate(X0, u0)
        a1.record()
        torch.cuda.synchronize()
        fw.append(a0.elapsed_time(a1))
    ms, = max_over_ranks([ms], dev)
    nq = 4
    pairs = info["regular_pairs"] + info["singular_pairs"]
    line = {"metric": "batched SL energy + shape gradient (64 meshes) per second",
            "value": whole_job_rate(world, args.steps, ms / 1e3),
            "unit": "batch/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (regular pairs) / f64 (singular pairs)", "data": "synthetic",
            "config": {"workload": "sl_energy_gradient_batch64_L2-L5", "meshes": "64 icospheres L2..L5 (16 each), radial noise 0.05",
                       "triangles": b.nt_total, "vertices": b.nv_total, "intorder": 3, "intorder_singular": 4,
                       "precision": "mixed", "step": "forward energy + backward (dE/dX, dE/du)"},
            "pairs": pairs, "regular_pairs": info["regular_pairs"], "singular_pairs": info["singular_pairs"],
            "forward_ms": min(fw), "regular_kernel_evals_per_s": info["regular_pairs"] * nq * nq / (min(fw) / 1e3),
            "gpu_launches": 3 * 2 * args.steps, "clocks": clocks}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_bm(args):
    """Burton-Miller (M/2 + C) u = f at kappa 8 on the ellipsoid (1, 0.7, 0.5), icosphere level
    args.level (default 6: 81920 triangles, 40962 complex P1 dofs), 32 plane waves.  Both the
    mixed path and the plain FP64 GPU path assemble C (timed, fresh space so that the cluster tree
    is built inside the timed region) and solve the 32 right-hand sides with the batched GMRES to
    1e-8.  The timed steps apply the mixed C to the 32 right-hand sides (tensor cores)."""
    import ctypes as C

    import numpy as np
    import torch

    import ngbem_gb300 as nb
    from ngbem_gb300 import _lib
    from ngbem_gb300.forms import p1_load_vector, plane_wave_bm_source, random_directions

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    dev = torch.device("cuda", local)
    L = args.level or 6
    nrhs = BM_NRHS

    if args.apply_only:
        run_bm_apply(args, nb, _lib, dev, L)
        return
    # untimed warm-up of both paths on a small ellipsoid (module loading, workspaces, graphs,
    # the tensor-core self-test)
    wm = nb.ellipsoid(2, BM_AXES)
    wP = nb.H1(wm, complex=True)
    wF = torch.from_numpy(p1_load_vector(wm, plane_wave_bm_source(BM_KAPPA, random_directions(nrhs, 1)))).to(dev)
    for prec in ("mixed", "fp64"):
        wC = nb.HelmholtzCombinedFieldOperator(wP, wP, kappa=BM_KAPPA, precision=prec, **BM_OPTS)
        nb.GMRes(0.5 * nb.MassOperator(wP, wP, complex=True) + wC.mat, wF, maxsteps=50, tol=1e-8, restart=100)
        wC.mat.Mult(wF, torch.empty_like(wF))
        del wC
    torch.cuda.synchronize()

    mesh = nb.ellipsoid(L, BM_AXES)
    Fh = p1_load_vector(mesh, plane_wave_bm_source(BM_KAPPA, random_directions(nrhs, BM_SEED)), order=6)
    F = torch.from_numpy(Fh).to(dev)
    Xc = F.t().contiguous()  # column-major n x 32: one contiguous column per right-hand side
    M = nb.MassOperator(nb.H1(mesh, complex=True), None, complex=True)
    stream = torch.cuda.current_stream()
    one, zero = _lib.cplx2(1.0), _lib.cplx2(0.0)

    def apply(op, X, Y):
        _lib.check(_lib.lib.bem_operator_mult(op.h, 0, one, C.c_void_p(X.data_ptr()), zero,
                                              C.c_void_p(Y.data_ptr()), nrhs, C.c_void_p(stream.cuda_stream)))

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed_apply(op, X, Y, reps):
        apply(op, X, Y)
        e0.record(stream)
        for _ in range(reps):
            apply(op, X, Y)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    info_keys = ("ms_setup", "ms_aca", "ms_nearfield", "ms_projection", "ms_mvitems", "ms_total")
    paths, ops, sols = {}, {}, {}
    for prec in ("mixed", "fp64"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P1 = nb.H1(mesh, complex=True)
        Cop = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=BM_KAPPA, precision=prec, **BM_OPTS)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        U = nb.GMRes(0.5 * M + Cop.mat, F, maxsteps=1000, tol=1e-8, restart=100)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        last = dict(nb.GMRes.last)
        info = Cop.mat.info
        paths[prec] = {"assembly_s": t1 - t0, "solve_s": t2 - t1, "total_s": t2 - t0,
                       "iterations": last["iterations"], "max_residual": last["residual"], "nze": info["nze"],
                       "max_rank": info["max_rank"], "nfallback": info["nfallback"],
                       "bytes_stored": info["bytes_dense"] + info["bytes_lowrank"],
                       "assembly_breakdown_ms": {k: info[k] for k in info_keys},
                       "assembly_rates": assembly_rates(info)}
        ops[prec], sols[prec] = Cop, U
    Cm, C64 = ops["mixed"].mat, ops["fp64"].mat
    Y = torch.empty_like(Xc)
    # the FP64 GPU path's application to the same 32 right-hand sides
    t64 = timed_apply(C64, Xc, Y, 3)
    Y64 = Y.clone()
    # mixed, error-free FP32 products on the CUDA cores (the GMRES residuals)
    Cm.set_accuracy(True)
    t_comp = timed_apply(Cm, Xc, Y, 3)
    Ycomp = Y.clone()
    # mixed, plain accuracy: the tensor-core products of the GMRES iterations (the timed step),
    # with the stage plan picked by the autotuner on this operator
    Cm.set_accuracy(False)
    tc_tune = Cm.autotune_tensor_cores(reps=5)
    tc = dict(Cm.tensor_cores(), autotune=tc_tune)

    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev)
    sweep = torch.zeros(512 * 2 ** 20 // 4, dtype=torch.float32, device=dev) if args.l2_flush == "write+read" else None
    sweep_out = torch.zeros((), dtype=torch.float32, device=dev)

    def flush_l2():
        flush.fill_(1.0)
        if sweep is not None:
            torch.amax(sweep, dim=0, out=sweep_out)

    for _ in range(args.warmup):
        flush_l2()
        apply(Cm, Xc, Y)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush_l2()
        evs[k][0].record(stream)
        apply(Cm, Xc, Y)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    Ytc = Y.clone()

    # e2e: page-locked host buffers through bem_operator_mult_host (the kernels read X and
    # write Y across the host link inside every step)
    xh = Xc.cpu().pin_memory()
    yh = torch.zeros_like(xh).pin_memory()

    def apply_host():
        _lib.check(_lib.lib.bem_operator_mult_host(Cm.h, 0, one, C.c_void_p(xh.data_ptr()), zero,
                                                   C.c_void_p(yh.data_ptr()), nrhs))

    for _ in range(args.warmup):
        apply_host()
    e2e_t = []
    for _ in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t = time.perf_counter()
        apply_host()
        e2e_t.append(time.perf_counter() - t)
    clocks = sampler.stop()
    e2e_check = float(torch.linalg.vector_norm(yh - Ytc.cpu()) / torch.linalg.vector_norm(Ytc.cpu()))

    # kernel times from a separate, untimed pass with the operator's event profiling on:
    # [X panels, GEMM pass 0, GEMM pass 1, partial-row sum + output]
    nprof = 10
    Cm.set_profiling(True)
    for _ in range(nprof):
        flush_l2()
        apply(Cm, Xc, Y)
    torch.cuda.synchronize()
    kms, kcount = Cm.kernel_times()
    Cm.set_profiling(False)
    per_app = [kms[i] / max(1, kcount[i]) for i in range(4)]
    launches_per_step = sum(kcount) / nprof

    dev_ms, e2e_sum = max_over_ranks([dev_ms, sum(e2e_t)], dev)
    value = whole_job_rate(world, args.steps * nrhs, dev_ms / 1e3)
    e2e_value = whole_job_rate(world, args.steps * nrhs, e2e_sum)

    # ---- accuracy against the FP64 GPU path (per right-hand side, max over the 32)
    def colmax(a, b):
        d = torch.linalg.vector_norm(a - b, dim=1) / torch.linalg.vector_norm(b, dim=1)
        return float(d.max())

    um, u64 = sols["mixed"].t(), sols["fp64"].t()
    acc = {"solution_rel_err_vs_fp64": colmax(um, u64),
           "solution_rel_err_vs_fp64_median": float((torch.linalg.vector_norm(um - u64, dim=1) /
                                                     torch.linalg.vector_norm(u64, dim=1)).median()),
           "C_matvec_tensor_core_rel_err_vs_fp64": colmax(Ytc, Y64),
           "C_matvec_compensated_rel_err_vs_fp64": colmax(Ycomp, Y64),
           "C_matvec_tensor_core_rel_err_vs_compensated": colmax(Ytc, Ycomp)}

    # ---- roofline of the tensor-core GEMM passes (tc_gemm_kernel<0> + <1>)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    im = Cm.info
    n = Cm.width
    # algorithmic bytes: the stored operator once (complex64 dense blocks and factors) plus the
    # 32 right-hand sides read and the 32 results written once (complex64)
    alg_bytes = im["bytes_dense"] + im["bytes_lowrank"] + 2 * n * nrhs * 8
    gemm_ms = per_app[1] + per_app[2]
    achieved = alg_bytes / (gemm_ms * 1e-3) / 1e9
    t0p = traffic_from_profile("tc_gemm_kernel<0>", f"tc_gemm_kernel_bm_ellipsoid_L{L}.md")
    t1p = traffic_from_profile("tc_gemm_kernel<1>", f"tc_gemm_kernel_bm_ellipsoid_L{L}.md")
    roofline = {"bound": "hbm", "kernel": "tc_gemm_kernel<0> + tc_gemm_kernel<1>", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                "traffic": (t0p + t1p) if (t0p is not None and t1p is not None) else None,
                "algorithmic_bytes": alg_bytes, "avg_launch_ms": gemm_ms,
                "kernel_ms": {"tc_xprep": per_app[0], "tc_gemm_pass0": per_app[1], "tc_gemm_pass1": per_app[2],
                              "tc_ysum_out": per_app[3]},
                "application_GBps": alg_bytes / (dev_ms / args.steps * 1e-3) / 1e9,
                "tensor_flops_per_step": 8 * im["nze"] * nrhs,
                "tensor_TFLOPs": 8 * im["nze"] * nrhs / (gemm_ms * 1e-3) / 1e12}

    mixed, fp64 = paths["mixed"], paths["fp64"]
    mixed.update({"matvec32_ms": dev_ms / args.steps, "matvec32_compensated_ms": t_comp, "tensor_cores": tc})
    fp64.update({"matvec32_ms": t64, "matvec_per_s": nrhs / (t64 * 1e-3)})
    vs_fp64 = {"assembly": fp64["assembly_s"] / mixed["assembly_s"], "solve": fp64["solve_s"] / mixed["solve_s"],
               "assembly_plus_solve": fp64["total_s"] / mixed["total_s"],
               "matvec": t64 / (dev_ms / args.steps),
               "target": ">= 5x for assembly + solve at solution error <= 1e-6"}
    line = {"metric": METRIC, "value": value, "unit": "matvec/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c64 (split-TF32 tensor-core products, FP32 accumulation)", "data": "synthetic",
            "config": bm_workload(L, args.l2_flush), "assembly_s": mixed["assembly_s"],
            "assembly_s_fp64": fp64["assembly_s"], "solve_s": mixed["solve_s"], "vs_fp64": vs_fp64,
            "mixed": mixed, "fp64": fp64, "accuracy": acc, "roofline": roofline,
            "gpu_launches": int(round(launches_per_step * args.steps)), "wall_s_timed_region": t_wall,
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": "matvec/s", "h2d_bytes_per_step": n * nrhs * 16,
                    "d2h_bytes_per_step": n * nrhs * 16, "check_rel_err": e2e_check,
                    "note": "page-locked host buffers, staged by one bulk copy each way (products above 1 MiB)"}}

    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_reference_bm(L, 2, 2, 0)
        # the oracle's products against the GPU paths' products of the same columns
        errs = {"fp64": [], "tensor_core": [], "compensated": []}
        for col, yo in r["products"].items():
            yo_t = torch.from_numpy(yo)
            for k, Yk in (("fp64", Y64), ("tensor_core", Ytc), ("compensated", Ycomp)):
                yg = Yk[col].cpu()
                errs[k].append(float(torch.linalg.vector_norm(yg - yo_t) / torch.linalg.vector_norm(yo_t)))
        for k, v in errs.items():
            line["accuracy"][f"C_matvec_{k}_rel_err_vs_oracle"] = max(v)
        line["accuracy"]["oracle_columns"] = sorted(r["products"])
        line["cpu_baseline"] = {"value": r["matvec_per_s"], "unit": "matvec/s", "cores": r["cores"], "kind": "port",
                                "assembly_s": r["assembly_s"], "nze": r["nze"],
                                "sample": f"oracle FP64 assembly of C on {r['cores']} threads "
                                          f"({r['assembly_s']:.1f} s), then 4 of the 32 right-hand sides "
                                          f"applied one vector at a time (2 timed steps of 2)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_bm_apply(args, nb, _lib, dev, L):
    """Profiling form of the Burton-Miller line: the mixed operator is assembled, then W warm-up
    and K timed applications to the 32 right-hand sides run back to back (kernel launches in
    order: per application tc_xprep, tc_gemm pass 0, tc_gemm pass 1, tc_ysum_out)."""
    import ctypes as C

    import torch

    from ngbem_gb300.forms import p1_load_vector, plane_wave_bm_source, random_directions
    nrhs = BM_NRHS
    mesh = nb.ellipsoid(L, BM_AXES)
    Fh = p1_load_vector(mesh, plane_wave_bm_source(BM_KAPPA, random_directions(nrhs, BM_SEED)), order=6)
    Xc = torch.from_numpy(Fh).to(dev).t().contiguous()
    P1 = nb.H1(mesh, complex=True)
    Cop = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=BM_KAPPA, precision="mixed", **BM_OPTS)
    Cm = Cop.mat
    Cm.set_accuracy(False)
    Cm.set_tensor_cores(True)
    Y = torch.empty_like(Xc)
    stream = torch.cuda.current_stream()
    one, zero = _lib.cplx2(1.0), _lib.cplx2(0.0)

    def apply():
        _lib.check(_lib.lib.bem_operator_mult(Cm.h, 0, one, C.c_void_p(Xc.data_ptr()), zero,
                                              C.c_void_p(Y.data_ptr()), nrhs, C.c_void_p(stream.cuda_stream)))

    for _ in range(args.warmup):
        apply()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        apply()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    info = Cm.info
    print(json.dumps({"metric": "tensor-core application to 32 right-hand sides (profiling form)",
                      "value": nrhs * 1e3 / ms, "unit": "matvec/s", "ms_per_step": ms, "steps": args.steps,
                      "warmup": args.warmup, "config": dict(bm_workload(L), l2="not flushed (back to back)"),
                      "bytes_stored": info["bytes_dense"] + info["bytes_lowrank"], "nze": info["nze"],
                      "tensor_cores": Cm.tensor_cores()}), flush=True)


def run_maxwell(args):
    """Maxwell EFIE: single layer on RT0 of the unit icosphere at level args.level (default 5:
    20480 triangles, 30720 edge dofs), kappa = 2, H-matrix leaf 20, eta 2, ACA eps 1e-6,
    intorder 3.  Assembly and single-vector matvec time of the mixed path (complex64 far field,
    complex128 singular pairs) and the plain FP64 GPU path, and the matvec error of the mixed
    path against FP64 on a seeded random complex vector."""
    import numpy as np
    import torch

    import ngbem_gb300 as nb

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    L = args.level or 5
    mesh = nb.icosphere(L)
    # warm-up on a small sphere (module loading)
    wR = nb.HDivSurface(nb.icosphere(2), complex=True)
    for prec in ("mixed", "fp64"):
        nb.MaxwellSingleLayerPotentialOperator(wR, kappa=2.0, leafsize=20, eps=1e-6, precision=prec)
    rng = np.random.default_rng(SEED + 4)
    out, ys = {}, {}
    for prec in ("mixed", "fp64"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        RT = nb.HDivSurface(mesh, complex=True)
        op = nb.MaxwellSingleLayerPotentialOperator(RT, kappa=2.0, intorder=3, leafsize=20, eta=2.0, eps=1e-6,
                                                    precision=prec)
        torch.cuda.synchronize()
        t_asm = time.perf_counter() - t0
        if prec == "mixed":
            xh = rng.standard_normal(RT.ndof) + 1j * rng.standard_normal(RT.ndof)
            x = torch.from_numpy(xh).cuda()
        tuned = op.mat.autotune(reps=5)
        y = torch.empty_like(x)
        for _ in range(args.warmup):
            op.mat.Mult(x, y)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            op.mat.Mult(x, y)
        e1.record()
        torch.cuda.synchronize()
        info = op.mat.info
        ys[prec] = y.cpu().numpy()
        out[prec] = {"assembly_s": t_asm, "matvec_ms": e0.elapsed_time(e1) / args.steps, "nze": info["nze"],
                     "bytes": info["bytes_dense"] + info["bytes_lowrank"], "max_rank": info["max_rank"],
                     "nfallback": info["nfallback"], "autotune": tuned}
        del op
        torch.cuda.empty_cache()
    err = float(np.linalg.norm(ys["mixed"] - ys["fp64"]) / np.linalg.norm(ys["fp64"]))
    line = {"metric": "Maxwell EFIE H-matvec/s (mixed) and assembly s", "value": 1e3 / out["mixed"]["matvec_ms"],
            "unit": "matvec/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out["mixed"]["matvec_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 far field / c128 singular pairs", "data": "synthetic",
            "config": {"workload": f"maxwell_efie_rt0_icosphere_L{L}_kappa2", "triangles": mesh.nt,
                       "dofs": int(3 * mesh.nt // 2), "kappa": 2.0, "leafsize": 20, "eta": 2.0, "eps": 1e-6,
                       "intorder": 3, "l2": "not flushed (timed back to back)"},
            "mixed": out["mixed"], "fp64": out["fp64"], "matvec_rel_err_mixed_vs_fp64": err,
            "assembly_speedup": out["fp64"]["assembly_s"] / out["mixed"]["assembly_s"],
            "matvec_speedup": out["fp64"]["matvec_ms"] / out["mixed"]["matvec_ms"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.workload == "maxwell":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the dtn workload carries the CPU baseline"}))
            return
        run_maxwell(args)
        return
    if args.workload == "bm":
        if args.impl == "reference":
            run_reference(args)
        else:
            run_bm(args)
        return
    if args.workload == "shape":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no shape derivatives; "
                              "the energy's CPU restatement is the oracle's dense matrix (tests)"}))
            return
        run_shape(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_dtn(args)


if __name__ == "__main__":
    main()
