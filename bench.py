#!/usr/bin/env python3
"""BEM solves/s on GB300 -- the headline benchmark.

Workload (the precision configuration): rigid (Neumann, bc = (0, 1, 0)) unit
sphere as an icosphere at subdivision 5 (10242 nodes, 20480 triangles) at
ka = 10, a plane wave from a seeded random direction, 32 seeded CHIEF points
uniform in r < 0.5; system (10274 x 10242) complex.

One step = one complete surface solve through the library:
  assembly  -- FP32 regular quadrature, FP64 singular and near-singular pairs
               (eta = 1, depth 2), c64 storage, rewritten every step;
  solve     -- GMRES on the normal equations with FP32 matrix products and
               FP64 Arnoldi/Givens, inside FP64 iterative refinement to a
               relative normal-equation residual of 1e-8.

value: solves/s with inputs resident in HBM.  e2e: the same through the C ABI
from pinned host buffers (geometry, sources in; surface pressure out).
The plain FP64 path (FP64 assembly + Householder QR, one solve) is run once
and the mixed solution's error against it is reported.

--impl reference times the CPU restatement of the path (the FP64 oracle,
OpenMP on every host core) on a bounded sample of the same workload.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = "rigid-sphere icosphere s5 (N=10242, E=20480), ka=10, seeded plane wave, 32 CHIEF"
METRIC = "BEM solves/s (surface solve, <=1e-5 rel err vs FP64)"
UNIT = "solves/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--subdiv", type=int, default=5)
    ap.add_argument("--ka", type=float, default=10.0)
    ap.add_argument("--chief", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eta", type=float, default=1.0)
    ap.add_argument("--depth", type=int, default=2)
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 reference solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="precision: skip the rhs (256 sources) and serve (request stream) objects of the line")
    ap.add_argument("--config", default="precision", choices=["precision", "rhs", "freq", "serve"],
                    help="precision: the headline workload (one plane wave); rhs: perturbed ellipsoid, "
                         "8 kHz, 256 point sources solved together (block GMRES); freq: 64 frequencies of "
                         "uneven mesh size as one batch; serve: Poisson request stream through the server")
    ap.add_argument("--sources", type=int, default=256, help="rhs: point sources (the configuration has 256)")
    ap.add_argument("--max-iter", type=int, default=100,
                    help="rhs/freq/serve: block GMRES iterations per refinement cycle")
    ap.add_argument("--inner-tol", type=float, default=1e-4, help="rhs: inner GMRES relative tolerance")
    ap.add_argument("--slots", type=int, default=8, help="freq/serve: requests in flight at once")
    ap.add_argument("--rate", type=float, default=2.0, help="serve: mean request arrivals per second")
    ap.add_argument("--requests", type=int, default=40, help="serve: requests in the stream")
    ap.add_argument("--gemm", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 4, 5, 6],
                    help="block-solve GEMM mode (-1 auto, 0 FP32, 1 split-BF16 FP32-accurate, 2 TF32, 3 TF32x3, "
                         "4 TF32x3 in the 3M form, 5 FP32 streaming kernels on the CUDA cores, 6 tcgen05 "
                         "tensor-core fp16 split products)")
    ap.add_argument("--far-variant", type=int, default=-1,
                    help="profile mode: fixed far-field launch shape (-1: autotuned)")
    ap.add_argument("--mode", default="bench",
                    choices=["bench", "profile", "cpu-validate", "products", "qr-tc", "tc-gemm"],
                    help="profile: one warm-up solve and one more solve, nothing timed (for ncu captures); "
                         "cpu-validate: the CPU legs' sample extrapolation against full FP64 CPU solves of "
                         "the workload at icosphere subdivisions 3 and 4; products: the block solve's product "
                         "pair per GEMM mode at 16, 64 and 256 sources on the rhs configuration's matrix; "
                         "qr-tc: the tensor-core QR least squares on the workload's c64 system (--steps solves "
                         "after one warm-up; phase times of the last, error against the FP64 QR); tc-gemm: "
                         "the tensor-core GEMM on 4096 x 16384 x 512 and its transposed-A twin, twice each "
                         "(a small case for ncu captures)")
    return ap.parse_args()


def run_profile(args):
    """Two solves of the workload and nothing else, so that an ncu capture
    (-k <kernel> -s/-c) sees the kernels of a steady-state solve."""
    import bem_gpu_clean_cpp_gb300 as bem
    pts, elems, chief, srcs, k, bc, _ = select_workload(args)
    rhs = args.config == "rhs"
    s = bem.Solver(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=1e-4,
                   max_iter=100 if rhs else 300, max_refine=10, block_tol=1e-8, gemm_mode=args.gemm,
                   far_variant=args.far_variant)
    s.set_geometry(pts, elems, bc=bc, chief=chief)
    s.set_sources(srcs)
    method = bem.SOLVE_BLOCK_GMRES if rhs else bem.SOLVE_GMRES_REFINED
    for _ in range(2):
        s.assemble(k, bem.PREC_C64)
        info = s.solve(method)
    s.sync()
    print(json.dumps({"mode": "profile", "iterations": info.iterations, "refinements": info.refinements,
                      "rel_residual": info.rel_residual, "far_variant": s.far_variant()}))
    return 0


# ---------------------------------------------------------------------------
# Synthetic inputs (numpy, shared by both arms)
# ---------------------------------------------------------------------------
def icosphere(subdiv: int, radius: float = 1.0):
    """Icosahedron subdivided `subdiv` times, projected to the sphere, faces
    wound so that (p1-p3) x (p2-p3) points inwards."""
    t = (1 + 5 ** 0.5) / 2
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
         [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
         [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                cache[key] = len(v) - 1
            return cache[key]
        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        f = nf
    p = np.array(v) * radius
    f = np.array(f, dtype=np.int32)
    n = np.cross(p[f[:, 0]] - p[f[:, 2]], p[f[:, 1]] - p[f[:, 2]])
    out = np.einsum("ij,ij->i", n, p[f].sum(axis=1)) > 0
    f[out, 0], f[out, 1] = f[out, 1].copy(), f[out, 0].copy()
    return p, f


WORKLOAD_RHS = ("perturbed ellipsoid 0.075/0.09/0.11 m (SH l<=8, 5%), geodesic nu=39 (N=15212, E=30420), "
                "8 kHz, Fibonacci point sources at 1 m (256), 32 CHIEF, block GMRES")


def workload_rhs(args):
    """The multi-right-hand-side configuration (rigid body)."""
    import bem_gpu_clean_cpp_gb300 as bem
    m = bem.Mesh.geodesic(39).perturbed_ellipsoid(0.075, 0.09, 0.11, lmax=8, amp=0.05, seed=args.seed)
    pts, elems = m.points(), m.elems()
    rng = np.random.default_rng(args.seed)
    u = rng.random((args.chief, 3))
    r = 0.5 * 0.075 * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    srcs = [("point", s, 1.0) for s in bem.fibonacci_sphere(args.sources, 1.0)]
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (elems.shape[0], 1))
    k = 2 * np.pi * 8000.0 / 343.21
    return pts, elems, chief, srcs, k, bc


def workload(args):
    rng = np.random.default_rng(args.seed)
    pts, elems = icosphere(args.subdiv)
    u = rng.random((args.chief, 3))
    r = 0.5 * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    chief = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)
    d = rng.standard_normal(3)
    d /= np.linalg.norm(d)
    bc = np.tile(np.array([0, 1, 0], dtype=np.complex128), (elems.shape[0], 1))
    return pts, elems, chief, d, float(args.ka), bc


WORKLOAD_FREQ = ("64 log-spaced frequencies 100 Hz-12 kHz, perturbed ellipsoid 0.075/0.09/0.11 m seeded per "
                 "frequency, icosphere s2-s6 (10 elements per wavelength on the longest edge), 16 point sources, "
                 "16 CHIEF each; all problems submitted at once to the request server")
WORKLOAD_SERVE = ("Poisson request stream: ellipsoid semi-axes U[0.05,0.2] m, subdivision U{3..6}, "
                  "f U[200 Hz, 10 kHz], 1-64 point sources; a quarter of the requests repeat an earlier "
                  "(mesh, frequency) with new sources")


def _max_edge(p, e):
    return max(float(np.linalg.norm(p[e[:, a]] - p[e[:, b]], axis=1).max()) for a, b in ((0, 1), (1, 2), (2, 0)))


def _chief_in(rng, rmax, n):
    u = rng.random((n, 3))
    r = rmax * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    return np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)


def freq_problems(args, nfreq=64):
    """The multi-frequency family: per frequency a seeded perturbed ellipsoid
    at the coarsest subdivision in 2..6 whose longest edge is <= lambda/10."""
    import bem_gpu_clean_cpp_gb300 as bem
    out = []
    srcs = [("point", s, 1.0) for s in bem.fibonacci_sphere(16, 1.0)]
    for i, f in enumerate(np.geomspace(100.0, 12000.0, nfreq)):
        lam = 343.21 / f
        for sub in range(2, 7):
            m = bem.Mesh.icosphere(sub).perturbed_ellipsoid(0.075, 0.09, 0.11, lmax=8, amp=0.05, seed=args.seed + i)
            p, e = m.points(), m.elems()
            if sub == 6 or _max_edge(p, e) <= lam / 10.0:
                break
        rng = np.random.default_rng(1000 + args.seed + i)
        out.append(dict(pnts=p, elems=e, k=2 * np.pi * f / 343.21, srcs=srcs, chief=_chief_in(rng, 0.0375, 16),
                        f=float(f), subdiv=sub))
    return out


def serve_requests(args, n=40):
    """Seeded request stream with arrival times (Poisson, rate args.rate/s)."""
    import bem_gpu_clean_cpp_gb300 as bem
    rng = np.random.default_rng(args.seed + 77)
    t, out, scenes = 0.0, [], []
    for i in range(n):
        t += rng.exponential(1.0 / args.rate)
        S = int(rng.integers(1, 65))
        rot = np.linalg.qr(rng.standard_normal((3, 3)))[0]
        srcs = [("point", s, 1.0) for s in bem.fibonacci_sphere(S, 1.0) @ rot.T]
        if scenes and rng.random() < 0.25:
            sc = scenes[int(rng.integers(0, len(scenes)))]
        else:
            ax = rng.uniform(0.05, 0.2, 3)
            sub = int(rng.integers(3, 7))
            m = bem.Mesh.icosphere(sub).perturbed_ellipsoid(*ax, lmax=8, amp=0.05, seed=args.seed + 500 + i)
            f = rng.uniform(200.0, 10000.0)
            sc = dict(pnts=m.points(), elems=m.elems(), k=2 * np.pi * f / 343.21,
                      chief=_chief_in(rng, 0.4 * ax.min(), 16), subdiv=sub, f=float(f))
            scenes.append(sc)
        out.append(dict(sc, srcs=srcs, t=t))
    return out


def select_workload(args):
    """(pts, elems, chief, sources, k, bc, workload name) of the chosen config."""
    if args.config == "rhs":
        pts, elems, chief, srcs, k, bc = workload_rhs(args)
        return pts, elems, chief, srcs, k, bc, WORKLOAD_RHS
    pts, elems, chief, d, k, bc = workload(args)
    return pts, elems, chief, [("plane", d, 1.0)], k, bc, WORKLOAD


# ---------------------------------------------------------------------------
# Distributed helpers (replicas: every rank solves its own copy)
# ---------------------------------------------------------------------------
def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    def __init__(self, use_cuda: bool):
        self.rank, self.world, self.local = dist_info()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group(backend="nccl" if use_cuda else "gloo")
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if self.pg.get_backend() == "nccl" else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# Clock sampling during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU restatement timing (the oracle), bounded sample of the same workload
# ---------------------------------------------------------------------------
# Sample of the CPU legs (the cpu_baseline of our arm and the --impl
# reference arm use the same): assembly of CPU_ROWS rows, Householder QR of a
# (CPU_QR + 32) x CPU_QR system (out of cache, like the full one).
CPU_ROWS = 256
CPU_QR = 2048


def cpu_sample(pts, elems, chief, srcs, k, bc, eta, depth, threads, rows=CPU_ROWS, n_qr=CPU_QR):
    """FP64 CPU time of one surface solve, extrapolated from a sample:
    assembly of `rows` rows (all elements and sources, x (N+M)/rows) plus a
    Householder QR least-squares solve of an (n_qr+32) x n_qr system (x flop
    ratio (8mn^2 - 8n^3/3) of the full system), divided by the number of
    sources that share the factorisation."""
    import oracle
    oracle.build()
    oracle.set_threads(threads)
    R, N = pts.shape[0] + chief.shape[0], pts.shape[0]
    allp = np.vstack([pts, chief])
    prm = oracle.params(near_eta=eta, near_depth=depth)
    t0 = time.perf_counter()
    oracle.assemble(allp, elems, k, N, srcs, bc=bc, prm=prm, rows=(0, rows))
    t_asm = (time.perf_counter() - t0) * R / rows
    rng = np.random.default_rng(1)
    m_s = n_qr + 32
    Aq = rng.standard_normal((m_s, n_qr)) + 1j * rng.standard_normal((m_s, n_qr))
    Bq = rng.standard_normal((m_s, 1)) + 1j * rng.standard_normal((m_s, 1))
    t0 = time.perf_counter()
    oracle.lsq_qr(Aq, Bq)
    t_qr_s = time.perf_counter() - t0
    S = len(srcs)
    # factorisation once, then Q^H b and the triangular solve per source
    flops = lambda m, n, s: 8.0 * m * n * n - 8.0 / 3.0 * n ** 3 + s * (8.0 * m * n)
    t_qr = t_qr_s * flops(R, N, S) / flops(m_s, n_qr, 1)
    total = t_asm + t_qr
    return {"value": S / total, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"oracle FP64: assembly of {rows}/{R} rows with {S} source(s) (x{R / rows:.1f}) + "
                      f"Householder LS-QR {m_s}x{n_qr} (x{flops(R, N, S) / flops(m_s, n_qr, 1):.0f} by flop "
                      f"count); extrapolated {total:.1f} s for {S} solve(s) (assembly {t_asm:.1f} s, "
                      f"QR {t_qr:.1f} s)"}


def run_qr_tc(args):
    """BEM_SOLVE_QR_TC on the workload's c64 system: one warm-up solve, then
    --steps solves; the library's phase timer on the last one, its wall time,
    refinement steps, and the relative difference from BEM_SOLVE_QR on the same
    c64 system (cuSOLVER's FP32 QR: mostly that solve's own FP32 error, since
    QR_TC refines to the FP64 least-squares solution)."""
    import bem_gpu_clean_cpp_gb300 as bem
    pts, elems, chief, srcs, k, bc, _ = select_workload(args)
    s = bem.Solver(near_eta=args.eta, near_depth=args.depth)
    s.set_geometry(pts, elems, bc=bc, chief=chief)
    s.set_sources(srcs)
    s.assemble(k, bem.PREC_C64)
    s.sync()
    info = s.solve(bem.SOLVE_QR_TC)
    s.sync()
    walls = []
    for rep in range(max(1, args.steps)):
        last = rep == max(1, args.steps) - 1
        if last:
            bem.profile_enable(True)
        t0 = time.perf_counter()
        info = s.solve(bem.SOLVE_QR_TC)
        s.sync()
        walls.append((time.perf_counter() - t0) * 1e3)
    prof = {n: [c, round(t, 3)] for n, (c, t) in bem.profile_report().items()}
    bem.profile_enable(False)
    x_tc = s.solution()
    s.solve(bem.SOLVE_QR)
    x_qr = s.solution()
    print(json.dumps({"mode": "qr-tc", "wall_ms": walls, "wall_ms_median": statistics.median(walls),
                      "refinements": info.refinements, "rel_residual": info.rel_residual,
                      "rel_diff_vs_cusolver_c64_qr": float(np.linalg.norm(x_tc - x_qr) / np.linalg.norm(x_qr)),
                      "phases_ms": prof}))
    return 0


def run_tc_gemm(args):
    """The tensor-core GEMM on C = A B (4096 x 16384 by 16384 x 512) and
    C = A^T B (A 8192 x 8192, B the first 8192 rows), two parts, twice each:
    a small steady case for ncu captures of tc_gemm_kernel."""
    import bem_gpu_clean_cpp_gb300 as bem
    bem.lib()
    rng = np.random.default_rng(0)
    M, K, N = 4096, 16384, 512
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    At = rng.standard_normal((K // 2, 2 * M)).astype(np.float32)
    for _ in range(2):
        C = bem.tc_gemm(A, B, trans=False, parts=2)
        C2 = bem.tc_gemm(At, B[:K // 2], trans=True, parts=2)
    print(json.dumps({"mode": "tc-gemm", "shapes": [list(C.shape), list(C2.shape)]}))
    return 0


def run_products(args):
    """The block solve's product pair (T = A V, W = A^H T) per GEMM mode on the
    rhs configuration's matrix (15244 x 15212 c64) for the first 16, 64 and
    256 of its sources: a short block solve (20 inner iterations, one cycle)
    per case under the library's kernel timer; per-product averages."""
    import bem_gpu_clean_cpp_gb300 as bem
    bem.lib()
    a = argparse.Namespace(**vars(args))
    a.config, a.sources = "rhs", 256
    pts, elems, chief, srcs, k, bc = workload_rhs(a)
    out = []
    for S in (16, 64, 256):
        for mode in (6, 4, 3, 1, 5):
            if mode == 5 and S > 32:
                continue
            s = bem.Solver(near_eta=args.eta, near_depth=args.depth, max_iter=20, max_refine=1, block_tol=1e-8,
                           gemm_mode=mode)
            s.set_geometry(pts, elems, bc=bc, chief=chief)
            s.set_sources(srcs[:S])
            s.assemble(k, bem.PREC_C64)
            s.solve(bem.SOLVE_BLOCK_GMRES, check=False)   # warm-up (planes, tuning, kernels)
            s.sync()
            bem.profile_enable(True)
            s.solve(bem.SOLVE_BLOCK_GMRES, check=False)
            s.sync()
            prof = bem.profile_report()
            bem.profile_enable(False)
            row = {"sources": S, "mode": GEMM_NAMES[mode]}
            for name in ("gemm_AV", "gemm_AhT"):
                c, t = prof.get(name, (0, 0.0))
                row[name + "_ms"] = t / max(c, 1)
            row["pair_ms"] = row["gemm_AV_ms"] + row["gemm_AhT_ms"]
            out.append(row)
            del s
    print(json.dumps({"mode": "products", "nodes": pts.shape[0], "rows": pts.shape[0] + chief.shape[0],
                      "results": out}), flush=True)
    return 0


def run_cpu_validate(args):
    """The extrapolation behind cpu_baseline and the reference arm, checked
    against full FP64 CPU solves (every row assembled, the full least-squares
    QR) of the headline workload at subdivisions 3 and 4 (642 and 2562
    nodes), with the sample the CPU legs take at subdivision 5 (256 rows, a
    QR of 2048 columns), capped at the problem's size: at subdivision 4 the
    rows are extrapolated x10 and the QR x1.9 by flop count."""
    import oracle
    threads = os.cpu_count() or 1
    out = []
    for sub in (3, 4):
        a = argparse.Namespace(**vars(args))
        a.subdiv = sub
        pts, elems, chief, d, k, bc = workload(a)
        srcs = [("plane", d, 1.0)]
        R, N = pts.shape[0] + chief.shape[0], pts.shape[0]
        rows, n_qr = min(CPU_ROWS, R), min(CPU_QR, N)
        est = cpu_sample(pts, elems, chief, srcs, k, bc, args.eta, args.depth, threads, rows=rows, n_qr=n_qr)
        prm = oracle.params(near_eta=args.eta, near_depth=args.depth)
        t0 = time.perf_counter()
        Ao, Bo = oracle.assemble(np.vstack([pts, chief]), elems, k, N, srcs, bc=bc, prm=prm)
        t_asm = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.lsq_qr(Ao, Bo)
        t_qr = time.perf_counter() - t0
        full = t_asm + t_qr
        extrap = 1.0 / est["value"]
        out.append({"subdiv": sub, "nodes": N, "rows": R, "sample_rows": rows, "sample_qr_columns": n_qr,
                    "extrapolated_s": extrap, "full_s": full, "full_assembly_s": t_asm, "full_qr_s": t_qr,
                    "extrapolated_over_full": extrap / full, "sample": est["sample"], "cores": threads})
    print(json.dumps({"mode": "cpu-validate", "results": out}), flush=True)
    return 0


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    pts, elems, chief, srcs, k, bc, name = select_workload(args)
    threads = os.cpu_count() or 1
    vals = []
    # the same sample as our arm's cpu_baseline; a step is one sample (a few
    # seconds), warm-up steps capped at one so the run stays within minutes
    for i in range(min(args.warmup, 1) + args.steps):
        r = cpu_sample(pts, elems, chief, srcs, k, bc, args.eta, args.depth, threads)
        if i >= min(args.warmup, 1):
            vals.append(r["value"])
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "subdiv": args.subdiv, "ka": args.ka, "chief": args.chief,
                       "sources": len(srcs), "seed": args.seed, "near_eta": args.eta},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": r["sample"] + "; one sample per step"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# Our arm
# ---------------------------------------------------------------------------
# Algorithmic bytes per launch of the HBM-bound kernels (A is (N+M) x N c64);
# normal_op reads A once for w = A^H (A v) (v in, w out; its FP64 sum of the
# clusters' partial w is a separate kernel, timed as normal_op_sum).
def kernel_bytes(name, R, N):
    a = 8.0 * R * N
    return {"normal_op": a + 24.0 * N,
            "gemv_c64": a + 16.0 * N + 8.0 * R,
            "gemv_h_c64": a + 8.0 * R + 16.0 * N,
            "resid": a + 16.0 * N + 32.0 * R,
            "gemv_h_f64": a + 16.0 * R + 16.0 * N}.get(name)


def run_ours(args):
    import torch
    import bem_gpu_clean_cpp_gb300 as bem

    dist = Dist(use_cuda=True)
    torch.cuda.set_device(dist.local)
    bem.lib()
    pts, elems, chief, src, k, bc, name = select_workload(args)
    if args.config == "rhs":
        method = bem.SOLVE_BLOCK_GMRES
        opts = dict(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=args.inner_tol,
                    max_iter=args.max_iter, max_refine=10, block_tol=1e-8, gemm_mode=args.gemm)
    else:
        d = src[0][1]
        method = bem.SOLVE_GMRES_REFINED
        opts = dict(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=1e-4, max_iter=300,
                    max_refine=10)
    N, E, M = pts.shape[0], elems.shape[0], chief.shape[0]
    R = N + M
    S = len(src)

    s = bem.Solver(**opts)
    s.set_geometry(pts, elems, bc=bc, chief=chief)
    s.set_sources(src)
    stream = torch.cuda.ExternalStream(s.stream())
    infos = []

    def step():
        s.assemble(k, bem.PREC_C64)
        infos.append(s.solve(method))

    for _ in range(max(3, args.warmup)):
        step()
    s.sync()
    torch.cuda.synchronize()

    # ---- timed region: inputs resident, K steps ----
    infos.clear()
    dev_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(dist.local)).split(",")[0]) \
        if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else dist.local
    clocks = Clocks(dev_index)
    bem.profile_enable(True)
    l0 = bem.launch_count()
    dist.barrier()
    torch.cuda.synchronize()
    s.sync()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    s.sync()
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches = bem.launch_count() - l0
    prof = bem.profile_report()
    bem.profile_enable(False)
    lat = [a.elapsed_time(b) for a, b in ev]
    total_ms = ev[0][0].elapsed_time(ev[-1][1])
    total_ms = dist.max(total_ms)
    value = dist.world * args.steps * S / (total_ms / 1000.0)     # one solve per source

    # ---- e2e: host buffers through the C ABI, pinned memory ----
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_pts, h_elems, h_chief, h_bc = pin(pts), pin(elems), pin(chief), pin(bc)
    h_x = torch.empty((S, N), dtype=torch.complex128).pin_memory().numpy().T
    s2 = bem.Solver(**opts)
    # Bytes the library copies host -> device per step: nodes (24N), row
    # points in double and hi/lo float (24R + 32R), elements (16E), bc (48E),
    # one column tile's element records (32E) and column map (4N + 12), the
    # source record (48); device -> host: the surface pressure (16N) plus the
    # 8-byte residual estimates read by the solver loop.
    h2d = 24 * N + 56 * R + 64 * E + 32 * E + 4 * N + 12 + 48 * S
    d2h = h_x.nbytes

    def e2e_step():
        s2.set_geometry(h_pts, h_elems, bc=h_bc, chief=h_chief)
        s2.set_sources(src)
        s2.assemble(k, bem.PREC_C64)
        s2.solve(method)
        s2.solution(out=h_x)

    for _ in range(max(1, min(2, args.warmup))):
        e2e_step()
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = dist.world * args.steps * S / e2e_s
    x_mixed = h_x.copy()
    if infos:
        d2h += 8 * int(np.mean([i.iterations + 2 * i.refinements + 1 for i in infos]))

    # ---- plain FP64 path (FP64 assembly + Householder QR): one warm-up solve
    # (handles, library workspace, kernel loading), then the median of 3 ----
    fp64 = None
    if not args.no_fp64:
        s3 = bem.Solver(**opts)
        s3.set_geometry(pts, elems, bc=bc, chief=chief)
        s3.set_sources(src)
        st3 = torch.cuda.ExternalStream(s3.stream())
        runs = []
        for rep in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st3)
            s3.assemble(k, bem.PREC_C128)
            s3.solve(bem.SOLVE_QR)
            b.record(st3)
            s3.sync()
            if rep > 0:
                runs.append(a.elapsed_time(b))
        ms64 = statistics.median(runs)
        x64_all = s3.solution()
        x64 = x64_all[:, 0]
        err = max(float(np.abs(x_mixed[:, j] - x64_all[:, j]).max() / np.abs(x64_all[:, j]).max())
                  for j in range(S))
        # this library's own least-squares QR (tensor-core trailing updates,
        # FP64 refinement) on the c64 assembly: one warm-up, median of 3
        qr_runs, qinfo = [], None
        for rep in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s3.assemble(k, bem.PREC_C64)
            s3.sync()
            if rep == 3:
                bem.profile_enable(True)
            a.record(st3)
            qinfo = s3.solve(bem.SOLVE_QR_TC)
            b.record(st3)
            s3.sync()
            if rep == 3:
                qprof = bem.profile_report()
                bem.profile_enable(False)
            if rep > 0:
                qr_runs.append(a.elapsed_time(b))
        xq = s3.solution()
        qr_tc = {"solve_ms": statistics.median(qr_runs), "ms_runs": qr_runs,
                 "refinements": qinfo.refinements, "rel_residual": qinfo.rel_residual,
                 "rel_err_vs_fp64": max(float(np.abs(xq[:, j] - x64_all[:, j]).max() / np.abs(x64_all[:, j]).max())
                                        for j in range(S)),
                 "kernels_ms": {n: round(t, 3) for n, (c, t) in qprof.items() if n.startswith("qr_") or
                                n in ("resid", "gemv_h_f64")},
                 "note": "BEM_SOLVE_QR_TC on the c64 assembly (solve only, assembly excluded): cluster "
                         "panels, tcgen05 trailing updates, FP64 semi-normal-equation refinement"}
        fp64 = {"ms": ms64, "ms_runs": runs, "spread": (max(runs) - min(runs)) / ms64,
                "solves_per_s": S * 1000.0 / ms64, "rel_err_mixed_vs_fp64": err,
                "speedup_mixed_vs_fp64": value / dist.world / (S * 1000.0 / ms64),
                "timing": "median of 3 after one warm-up solve"}
        del s3

    # ---- the reference's own GPU path on this GB300, once ----
    # (its assembly kernels from the cubin built from its sources, launched as
    # atomicGenSystem does, and qrSolver's cuSOLVER sequence; FP32, no
    # near-singular rule)
    ref_gpu = None
    if not args.no_fp64 and dist.rank == 0 and args.config == "precision":
        try:
            from oracle import ref as refk
            from oracle import ref_build
            ref_build.build_if_possible()
            if refk.available():
                rows = np.vstack([pts, chief]).astype(np.float32)
                bc_ref = np.tile(np.array([0, 1, 0], dtype=np.complex128), (E, 1))
                asm_runs, qr_runs = [], []
                for rep in range(4):   # one warm-up, then 3 timed
                    Ar, Br, ms_asm = refk.assemble(rows, elems, N, k, srcs=[(1e6, 1e6, 1e6)], strength=0.0,
                                                   bc=bc_ref)
                    inc = np.exp(-1j * k * (rows.astype(np.float64) @ d)).astype(np.complex64)   # plane wave RHS
                    xr, ms_qr = refk.qr(Ar, (Br[:, 0] + inc).reshape(-1, 1))
                    if rep > 0:
                        asm_runs.append(ms_asm)
                        qr_runs.append(ms_qr)
                err_ref = None
                if fp64:
                    err_ref = float(np.abs(xr[:, 0] - x64).max() / np.abs(x64).max())
                ma, mq = statistics.median(asm_runs), statistics.median(qr_runs)
                ref_gpu = {"assembly_ms": ma, "qr_ms": mq, "solve_ms": ma + mq, "solves_per_s": 1000.0 / (ma + mq),
                           "assembly_ms_runs": asm_runs, "qr_ms_runs": qr_runs,
                           "rel_err_vs_fp64": err_ref,
                           "note": "reference kernels + cusolver Cgeqrf/Cunmqr/cublasCtrsm, FP32, plain 6x6 "
                                   "rule for near pairs; timed with its own event spans; median of 3 after "
                                   "one warm-up"}
                del Ar, Br
        except Exception as exc:   # reported, not fatal: the reference path is a comparison only
            ref_gpu = {"unavailable": str(exc)[:200]}

    # ---- roofline of the dominant kernel ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "of measured" if "hbm_gbs" in peaks else "of fallback"
    per_kernel = {n: {"launches": c, "total_ms": ms, "avg_ms": ms / max(c, 1)} for n, (c, ms) in prof.items()}
    dev_kernels = [n for n in per_kernel if not n.startswith("host:")]
    dom = max(dev_kernels, key=lambda n: per_kernel[n]["total_ms"]) if dev_kernels else None
    hbm_kernels = [n for n in per_kernel if kernel_bytes(n, R, N)]
    hbm_dom = max(hbm_kernels, key=lambda n: per_kernel[n]["total_ms"]) if hbm_kernels else None
    traffic_tab = {}
    try:
        traffic_tab = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
    except (OSError, ValueError):
        pass
    roofline_hbm = None
    if hbm_dom:
        bpl = kernel_bytes(hbm_dom, R, N)
        ach = bpl / (per_kernel[hbm_dom]["avg_ms"] / 1000.0) / 1e9
        roofline_hbm = {"kernel": hbm_dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                        "frac": ach / hbm_peak, "traffic": traffic_tab.get(hbm_dom, {}).get("bytes_per_launch"),
                        "peak_source": peak_src, "algorithmic_bytes_per_launch": bpl}
    asm = per_kernel.get("far_assembly_f32")
    pairs = R * E
    roofline = None
    if asm:
        # The dominant kernel, bounded by the FP32 pipe.  The reference's
        # per-point arithmetic is 60 FP32 flops (+ 3 MUFU) per quadrature
        # point, 36 points per (row, element) pair, counted once whatever the
        # implementation; of those, the moments of G that the BCs multiply by
        # zero are not needed: 8 flops per point (the S1, S2 sums of G) when
        # alpha = 0 on every element, 4 more (S0) when gamma = 0 too.  The
        # frac is taken on the needed count; the fixed tally is reported
        # beside it.  MEASURED_PEAKS.json holds no FP32 figure: the peak is
        # the nominal rate of this device's SMs (queried) at the SM clock
        # sampled during the timed region.
        bca = np.asarray(bc)
        a_zero = not np.any(bca[:, 0] != 0)
        c_zero = a_zero and not np.any(bca[:, 2] != 0)
        per_point = 60.0 - (8.0 if a_zero else 0.0) - (4.0 if c_zero else 0.0)
        sec = asm["avg_ms"] / 1000.0
        tflops = per_point * 36 * pairs / sec / 1e12
        mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
        sms = torch.cuda.get_device_properties(dist.local).multi_processor_count
        fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12
        tally = 60.0 * 36 * pairs / sec / 1e12
        roofline = {"kernel": "far_assembly_f32", "bound": "fp32", "achieved": tflops, "unit": "TFLOP/s",
                    "peak": fp32_peak, "frac": tflops / fp32_peak,
                    "traffic": traffic_tab.get("far_assembly_f32", {}).get("bytes_per_launch"),
                    "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 flops at the sampled {mhz:.0f} MHz "
                                   "(no FP32 figure in MEASURED_PEAKS.json)",
                    "pairs_per_launch": pairs, "flops_per_pair": 36 * per_point,
                    "flops_per_pair_note": "the reference's 2160 per pair less the G moments the BCs zero "
                                           f"(alpha = 0: {a_zero}, gamma = 0: {c_zero})",
                    "fixed_tally": {"flops_per_pair": 2160, "achieved": tally, "frac": tally / fp32_peak},
                    "mufu_per_pair": 108, "mufu_tops": 108.0 * pairs / sec / 1e12,
                    "algorithmic_bytes_per_launch": 8.0 * R * N}
    it = [i.iterations for i in infos]
    A_bytes = 8.0 * R * N
    B_bytes = 16.0 * R
    asm_ms = (per_kernel.get("far_assembly_f32", {"avg_ms": 0})["avg_ms"] +
              per_kernel.get("near_assembly", {"avg_ms": 0})["avg_ms"])

    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        cpu = cpu_sample(pts, elems, chief, src, k, bc, args.eta, args.depth, os.cpu_count() or 1)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (FP32) + f64", "data": "synthetic",
        "config": {"workload": name, "sources": S, "nodes": N, "triangles": E, "chief": M,
                   **({"subdiv": args.subdiv, "ka": args.ka} if args.config == "precision" else
                      {"k": k, "solver": "block GMRES: %s GEMMs, FP32 Arnoldi, FP64 Givens, FP64-accurate "
                                          "refinement residual to 1e-8" % GEMM_NAMES[args.gemm],
                       "gemm_used": GEMM_NAMES.get(s.block_gemm_mode(), None)}),
                   "seed": args.seed, "near_eta": args.eta, "near_depth": args.depth,
                   "refine_tol": 1e-8, "parallelism": f"replicas x{dist.world}",
                   "l2": "inputs larger than L2: A (%.0f MB c64) is rewritten every step" % (A_bytes / 1e6)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "min": min(lat), "max": max(lat)},
        "solver": {"inner_iterations_per_solve": float(np.mean(it)) if it else None,
                   "refinements": max(i.refinements for i in infos) if infos else None,
                   "rel_residual": max(i.rel_residual for i in infos) if infos else None},
        "assembly_gbs": (A_bytes + B_bytes) / (asm_ms / 1000.0) / 1e9 if asm_ms else None,
        "fp64_plain": fp64,
        "qr_tc": qr_tc if fp64 else None,
        "reference_gpu": ref_gpu,
        "roofline": roofline,
        "roofline_hbm": roofline_hbm,
        "kernels": per_kernel,
        "dominant_kernel": dom,
        "far_variant": s.far_variant() if args.config == "precision" or args.config == "rhs" else None,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "cpu_baseline": cpu,
    }
    if dist.rank == 0 and args.config == "precision" and not args.no_extras:
        del s, s2
        line["rhs"] = rhs_extra(args)
        line["serve"] = serve_extra(args)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.barrier()
    dist.close()
    return 0


# ---------------------------------------------------------------------------
# Batching over frequencies and serving: both through the request server
# ---------------------------------------------------------------------------
def _fp64_solve(bem, p, opts):
    s = bem.Solver(**opts)
    s.set_geometry(p["pnts"], p["elems"], chief=p["chief"])
    s.set_sources(p["srcs"])
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.assemble(p["k"], bem.PREC_C128)
    s.solve(bem.SOLVE_QR)
    x = s.solution()
    return x, time.perf_counter() - t0


def server_passes(bem, args, probs, opts, cache, steps, saturated=False, slots=None):
    """Timed passes of the request server over `probs` (a fresh server per
    pass: empty cache every time).  Poisson arrivals at each problem's time
    "t", or all submitted at once when saturated (capacity).  Returns the
    solves/s, wall time, per-request latencies, the servers' statistics and
    the last pass's results."""
    import torch
    slots = slots or args.slots

    def one_pass(srv):
        tickets = [None] * len(probs)
        t0 = time.perf_counter()

        def feed():
            for i, p in enumerate(probs):
                if not saturated and "t" in p:
                    dt = p["t"] - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                tickets[i] = srv.submit(p["pnts"], p["elems"], p["k"], p["srcs"], chief=p["chief"])

        th = threading.Thread(target=feed)
        th.start()
        out = []
        for i in range(len(probs)):
            while tickets[i] is None:
                time.sleep(0.0002)
            out.append(srv.wait(tickets[i]))
        th.join()
        return out

    solves = sum(len(p["srcs"]) for p in probs)
    elapsed, lat, stats, last = 0.0, [], [], None
    for _ in range(steps):
        with bem.Server(slots=slots, cache_systems=cache, **opts) as srv:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            last = one_pass(srv)
            torch.cuda.synchronize()
            elapsed += time.perf_counter() - t0
            stats.append(srv.stats())
            lat += [r["latency_ms"] for _, r in last]
    return {"solves": solves, "elapsed": elapsed, "value": steps * solves / elapsed, "lat": lat, "stats": stats,
            "last": last, "one_pass": one_pass}


def server_warmup(bem, args, probs, opts, passes=0):
    """Library, handles and kernels warmed on a separate server."""
    import torch
    with bem.Server(slots=args.slots, cache_systems=0, **opts) as w:
        small = [p for p in probs if p["pnts"].shape[0] <= 2562][:max(3, args.warmup)]
        for p in small:
            w.wait(w.submit(p["pnts"], p["elems"], p["k"], p["srcs"], chief=p["chief"]))
    if passes:
        server_passes(bem, args, probs, opts, 0, passes, saturated=True)
    torch.cuda.synchronize()


def server_fp64_check(bem, probs, last, opts):
    """Every problem up to 10242 nodes (one at 10242) against its plain FP64
    solve (c128 assembly + Householder QR), and the one-at-a-time FP64 time."""
    errs, fp64_t, worst_cases = [], {}, []
    checked_s5 = 0
    for i, p in enumerate(probs):
        n = p["pnts"].shape[0]
        if n > 10242 or (n == 10242 and checked_s5 >= 1):
            continue
        checked_s5 += n == 10242
        x64, t64 = _fp64_solve(bem, p, opts)
        x = last[i][0]
        errs.append(float(max(np.abs(x[:, j] - x64[:, j]).max() / np.abs(x64[:, j]).max()
                              for j in range(x.shape[1]))))
        worst_cases.append({"request": i, "nodes": n, "f_hz": round(p["f"], 1), "sources": len(p["srcs"]),
                            "k_times_max_edge": round(p["k"] * _max_edge(p["pnts"], p["elems"]), 3),
                            "rel_err": errs[-1]})
        fp64_t.setdefault(n, []).append(t64)
    per_n = {n: float(np.mean(v)) for n, v in fp64_t.items()}
    if 10242 in per_n:
        per_n.setdefault(40962, per_n[10242] * (40962 / 10242) ** 3)   # QR cost ~ N^3
    est = sum(per_n.get(p["pnts"].shape[0], 0.0) for p in probs)
    return {"checked_problems": len(errs), "max_rel_err_vs_fp64": max(errs) if errs else None,
            "seconds_by_nodes": {str(k): v for k, v in sorted(per_n.items())},
            "estimated_one_at_a_time_s": est,
            "largest_errors": sorted(worst_cases, key=lambda c: -c["rel_err"])[:5],
            "note": "plain FP64 = c128 assembly + Householder QR per problem, timed for every problem up to "
                    "10242 nodes (one at 10242), 40962-node problems extrapolated by N^3 from 10242"}


def run_server_bench(args):
    import torch
    import bem_gpu_clean_cpp_gb300 as bem

    dist = Dist(use_cuda=True)
    torch.cuda.set_device(dist.local)
    bem.lib()
    opts = dict(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=1e-4, max_iter=args.max_iter,
                max_refine=10, block_tol=1e-8, gemm_mode=args.gemm)
    if args.config == "freq":
        probs, name, cache = freq_problems(args), WORKLOAD_FREQ, 0
    else:
        probs, name, cache = serve_requests(args, args.requests), WORKLOAD_SERVE, 16
    server_warmup(bem, args, probs, opts, passes=max(0, args.warmup - 2) if args.config == "freq" else 0)
    dev_index = dist.local
    clocks = Clocks(dev_index)
    l0 = bem.launch_count()
    dist.barrier()
    clocks.start()
    res = server_passes(bem, args, probs, opts, cache, args.steps, saturated=args.config == "freq")
    clk = clocks.stop()
    launches = bem.launch_count() - l0
    elapsed = dist.max(res["elapsed"])
    solves, lat, stats, last = res["solves"], res["lat"], res["stats"], res["last"]
    value = dist.world * args.steps * solves / elapsed

    # ---- accuracy against the plain FP64 solve, and its one-at-a-time time ----
    fp64 = server_fp64_check(bem, probs, last, opts)
    est = fp64["estimated_one_at_a_time_s"]
    fp64["solves_per_s"] = solves / est if est else None
    fp64["speedup_vs_fp64_plain"] = value / (solves / est) if est else None
    sizes = sorted({p["pnts"].shape[0] for p in probs})
    by_sub = {}
    for p, (_, r) in zip(probs, last):
        d = by_sub.setdefault(str(p["subdiv"]), {"requests": 0, "nodes": p["pnts"].shape[0], "solves": 0,
                                                  "service_ms": 0.0, "iterations": 0, "max_latency_ms": 0.0})
        d["requests"] += 1
        d["solves"] += len(p["srcs"])
        d["service_ms"] += r["service_ms"]
        d["iterations"] += r["iterations"]
        d["max_latency_ms"] = max(d["max_latency_ms"], r["latency_ms"])
    for d in by_sub.values():
        d["mean_service_ms"] = d.pop("service_ms") / d["requests"]
        d["mean_iterations"] = d.pop("iterations") / d["requests"]
    h2d = sum(24 * p["pnts"].shape[0] + 12 * p["elems"].shape[0] + 24 * 16 + 48 * len(p["srcs"]) for p in probs)
    d2h = sum(16 * p["pnts"].shape[0] * len(p["srcs"]) for p in probs)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (FP32) + f64", "data": "synthetic",
        "config": {"workload": name, "problems": len(probs), "solves_per_step": solves, "node_counts": sizes,
                   "slots": args.slots, "cache_systems": cache, "rate_per_s": args.rate if args.config == "serve"
                   else None, "parallelism": f"replicas x{dist.world}",
                   "timing": "wall clock between device synchronisations around each pass (several streams)"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(max(lat))},
        "server": stats[-1],
        "per_subdivision": by_sub,
        "fp64_plain": fp64,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "note": "the server path takes host arrays and returns host arrays: value is end to end"},
        "roofline": None, "cpu_baseline": None,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


# ---------------------------------------------------------------------------
# The batching configurations inside the default line (secondary objects)
# ---------------------------------------------------------------------------
GEMM_NAMES = {-1: "auto", 0: "FP32 (cuBLAS)", 1: "split-BF16 (cuBLAS)", 2: "TF32 (cuBLAS)", 3: "TF32x3 (cuBLAS)",
              4: "TF32x3 3M (cuBLAS)", 5: "CUDA-core streaming FP32", 6: "tcgen05 fp16 split (this library)"}


def rhs_extra(args):
    """Config 3 at full size: 256 point sources on the perturbed ellipsoid
    (15212 nodes), all solved together by block GMRES with the default (AUTO)
    products.  One warm-up step, then 3 timed steps (assembly + block solve,
    CUDA events on the solver's stream, median); per-source max error against
    the plain FP64 solve (c128 assembly + Householder QR) of the same system."""
    import torch
    import bem_gpu_clean_cpp_gb300 as bem
    a = argparse.Namespace(**vars(args))
    a.config, a.sources = "rhs", 256
    pts, elems, chief, srcs, k, bc = workload_rhs(a)
    N, E, M, S = pts.shape[0], elems.shape[0], chief.shape[0], len(srcs)
    R = N + M
    s = bem.Solver(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=1e-4, max_iter=100,
                   max_refine=10, block_tol=1e-8, gemm_mode=-1)
    s.set_geometry(pts, elems, bc=bc, chief=chief)
    s.set_sources(srcs)
    st = torch.cuda.ExternalStream(s.stream())
    s.assemble(k, bem.PREC_C64)
    s.solve(bem.SOLVE_BLOCK_GMRES)
    s.sync()
    bem.profile_enable(True)
    runs, infos = [], []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.assemble(k, bem.PREC_C64)
        infos.append(s.solve(bem.SOLVE_BLOCK_GMRES))
        e1.record(st)
        s.sync()
        runs.append(e0.elapsed_time(e1))
    prof = bem.profile_report()
    bem.profile_enable(False)
    mode = s.block_gemm_mode()
    x = s.solution()
    s.assemble(k, bem.PREC_C128)
    s.solve(bem.SOLVE_QR)
    x64 = s.solution()
    err = max(float(np.abs(x[:, j] - x64[:, j]).max() / np.abs(x64[:, j]).max()) for j in range(S))
    del s
    ms = statistics.median(runs)
    prods = {}
    for name in ("gemm_AV", "gemm_AhT"):
        if name in prof:
            c, t = prof[name]
            prods[name] = {"launches": c, "avg_ms": t / max(c, 1)}
    tensor = None
    if mode == 6 and "gemm_AV" in prods and "gemm_AhT" in prods:
        # complex product counted as 8 R N S flops (whatever the method); the
        # fp16 split runs 3 tensor products per real product of the
        # interleaved form (24 R N S fp16 flops on the tensor pipe)
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except (OSError, ValueError):
            pass
        pk = peaks.get("bf16_tflops", 1900.0)
        avg = 0.5 * (prods["gemm_AV"]["avg_ms"] + prods["gemm_AhT"]["avg_ms"])
        alg = 8.0 * R * N * S / (avg / 1000.0) / 1e12
        tensor = {"kernel": "tc_gemm_kernel", "bound": "tensor", "unit": "TFLOP/s",
                  "achieved_algorithmic": alg, "achieved_tensor_pipe": 3 * alg, "peak": pk,
                  "frac": 3 * alg / pk,
                  "peak_source": ("of measured" if "bf16_tflops" in peaks else "of fallback") +
                                 " dense bf16 (fp16 runs at the same rate)",
                  "note": "per product including its operand packing; 8 R N S algorithmic flops, 3x that on the "
                          "tensor pipe (hh + hl + lh fp16 products)"}
    return {"workload": WORKLOAD_RHS, "nodes": N, "triangles": E, "chief": M, "sources": S, "k": k,
            "gemm_mode": GEMM_NAMES.get(mode, mode), "ms_per_step": ms, "ms_runs": runs,
            "solves_per_s": S * 1000.0 / ms,
            "iterations": [i.iterations for i in infos], "refinements": [i.refinements for i in infos],
            "max_rel_err_vs_fp64": err, "products": prods, "roofline_products": tensor,
            "timing": "assembly + block solve per step, median of 3 after one warm-up step"}


def serve_extra(args):
    """Config 5 inside the default line: the seeded stream of 40 requests
    (1-64 sources, subdivision 3-6) through the request server with 8 slots,
    once at the Poisson arrival rate (2/s) and once saturated (all submitted
    at t = 0: the server's capacity), then every request up to 10242 nodes
    (one at 10242) checked against its plain FP64 solve."""
    import bem_gpu_clean_cpp_gb300 as bem
    a = argparse.Namespace(**vars(args))
    a.config, a.requests, a.rate, a.slots, a.max_iter, a.gemm = "serve", 40, 2.0, 8, 100, -1
    probs = serve_requests(a, a.requests)
    opts = dict(near_eta=args.eta, near_depth=args.depth, tol=1e-8, inner_tol=1e-4, max_iter=a.max_iter,
                max_refine=10, block_tol=1e-8, gemm_mode=-1)
    server_warmup(bem, a, probs, opts)
    out = {"workload": WORKLOAD_SERVE, "requests": len(probs), "slots": a.slots,
           "solves": sum(len(p["srcs"]) for p in probs)}
    last = None
    for key, sat in (("poisson", False), ("saturated", True)):
        r = server_passes(bem, a, probs, opts, 16, 1, saturated=sat)
        out[key] = {"solves_per_s": r["value"], "wall_s": r["elapsed"],
                    "p50_ms": float(np.percentile(r["lat"], 50)), "p99_ms": float(np.percentile(r["lat"], 99)),
                    "max_in_flight": r["stats"][-1].get("max_in_flight")}
        if not sat:
            out[key]["rate_per_s"] = a.rate
            last = r["last"]
    chk = server_fp64_check(bem, probs, last, opts)
    out["max_rel_err_vs_fp64"] = chk["max_rel_err_vs_fp64"]
    out["checked_problems"] = chk["checked_problems"]
    out["largest_errors"] = chk["largest_errors"][:3]
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        if args.config in ("freq", "serve"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference solves one problem per process; "
                                                                  "its arm runs the precision and rhs configs"}))
            return 0
        return run_reference(args)
    if args.config in ("freq", "serve"):
        return run_server_bench(args)
    if args.mode == "profile":
        return run_profile(args)
    if args.mode == "cpu-validate":
        return run_cpu_validate(args)
    if args.mode == "products":
        return run_products(args)
    if args.mode == "qr-tc":
        return run_qr_tc(args)
    if args.mode == "tc-gemm":
        return run_tc_gemm(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
