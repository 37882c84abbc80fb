#!/usr/bin/env python
"""Headline benchmark: fused FE loss + adjoint, hex8 linear elasticity, 64^3.

Workload (one "step" = one pass of the hot path over one batch):
  * structured unit-cube hex8 mesh, 64^3 elements (274,625 nodes, 823,875
    dofs), 2x2x2 Gauss; two-phase voxel Young's modulus (seeded white noise,
    Gaussian-smoothed sigma = 3 voxels, thresholded at 0 -> E in {1.0, 0.1}),
    nu = 0.3, one value per element; u = 0 on z = 0, u_z = 0.05 on z = 1;
  * input dofs: the uniaxial field u_z = 0.05 z plus seeded N(0, 0.01^2) noise
    (synthetic, seeded);
  * one step = FE loss (energy u^T(K u - f) summed over elements) plus its
    adjoint: dLoss/du (823,875 dofs) and dLoss/dE (262,144 elements).

Metric: M elements/s of fused loss + adjoint.  Reported beside it: the plain
GPU path (element matrices materialised in HBM, separate backward pass), the
end-to-end number through the public API with host buffers, the dominant
kernel's roofline, and the C FP64 oracle timed on the host cores.

`--impl reference` times the C FP64 oracle (the reference's element algorithm;
the reference itself is JAX, absent here) with every host core on the whole
workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024
FLUSH_BYTES = 512 * 1024 * 1024
# algorithmic work of the fused element kernel per element, 2x2x2 Gauss:
# per Gauss point J (72 FMA), det + inverse (~30 flops), dN/dx (72 FMA),
# grad u (72 FMA), stress (~20), B^T sigma (72 FMA), energy and dE (~25):
# 4 x 72 x 2 + 75 = 651 flops, x 8 points = 5,208 flops; plus gathers ~0.
FLOPS_PER_ELEMENT = 5208.0
# FP32 operations of the uniform-box element (variants 20-24), counted from
# the kernel source: forward Hadamard transforms 72 FADD, eight 3x3 block
# products 24 FMUL + 48 FFMA, u.K u 24 FFMA, energy 1 FFMA, scaling 24 FMUL,
# transposed transforms 72 FADD, control gradient 1 FMUL (FFMA = 2 flops).
BOX_FLOPS_PER_ELEMENT = 72 + 24 + 96 + 48 + 2 + 24 + 72 + 1
# kernel variants by family (the autotuner's index)
BOX_VARIANTS, GRID_VARIANTS = (20, 21, 22), (23, 24)
# ncu figures of one launch of the fused element kernel on the 64^3 workload,
# per kernel variant (the autotuner's index): DRAM bytes read + written
# (dram__bytes_read.sum + dram__bytes_write.sum) and warp instructions
# (smsp__inst_executed.sum; the kernel's real limit is instruction issue, 4
# warp instructions per clock per SM).  Variants without a capture report null.
#   6:  k_hex8_elastic_regs, 128 threads / 96 registers, point sums
#   13: k_hex8_elastic_tma, persistent, TMA-staged rows, paired points
#   16, 17: the same with the next tile's nodes prefetched to L1 / L2
# (13, 16, 17 with the affine-element path; ncu's printed precision for the
# DRAM bytes: 17.60 MB read, a few KB written)
#   21: k_hex8_box, 256 threads, uniform box element (the records, 33.5 MB,
#       stay in L2 for the gather: 8 KB written to DRAM)
#   23: k_hex8_box_grid, the whole step in one launch (its outputs stay in L2:
#       no DRAM writes inside the launch; its FP32 count includes the halo
#       elements and the node sums: 534 per owned element)
# fp32_flops: ncu's FP32 thread-instruction counts of one launch, fadd + fmul +
# 2 ffma + 2 fadd2 + 2 fmul2 + 4 ffma2 (variant 16: 1,699 flops per element,
# against the naive 5,208 of FLOPS_PER_ELEMENT; variant 21: 357).
NCU_FIGURES = {64: {6: {"traffic": 17_498_624 + 108_544, "warp_instructions": 16_144_605},
                    13: {"traffic": 17_600_000 + 4_860, "warp_instructions": 10_652_202},
                    16: {"traffic": 17_600_000 + 28_200, "warp_instructions": 10_935_648,
                         "fp32_flops": 445_300_000},
                    17: {"traffic": 17_600_000 + 8_960, "warp_instructions": 10_964_421},
                    21: {"traffic": 13_100_000 + 7_940, "warp_instructions": 4_817_046,
                         "fp32_flops": 93_490_000},
                    23: {"traffic": 4_482_560 + 0, "warp_instructions": 7_515_845,
                         "fp32_flops": 139_940_000}}}


def ncu_figure(n, variant, key):
    return NCU_FIGURES.get(n, {}).get(variant, {}).get(key)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--plain-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-soak", action="store_true", help="skip the one-second clock soak (profiling runs)")
    ap.add_argument("--no-extras", action="store_true", help="skip the PCG / batched / neo-Hooke measurements")
    ap.add_argument("--only-extras", action="store_true",
                    help="run only the --extras measurements and print them (profiling runs; no bench line)")
    ap.add_argument("--hex8-variant", type=int, default=None,
                    help="force one hex8 kernel variant (0-17) instead of autotuning (profiling runs)")
    ap.add_argument("--minimiser-n", type=int, default=16,
                    help="cells per side of the tet split the loss minimiser is solved on (minimiser extra)")
    ap.add_argument("--extras", default="jittered,small,pcg,batched,neohooke,minimiser,newton,fourier",
                    help="comma list of the extra measurements to run (jittered, small, pcg, batched, neohooke, "
                         "minimiser, newton, fourier; fused: the headline step alone, for profiling)")
    return ap.parse_args()


def workload(n, seed, jitter=0.0):
    from folax_gb300 import workloads
    return workloads.hex8_elastic(n, seed, jitter)


def workload_config(n, B):
    E = n ** 3
    N = (n + 1) ** 3
    return {"workload": f"hex8 linear-elastic fused loss+adjoint, {n}^3 elements, 2x2x2 Gauss",
            "elements": E, "nodes": N, "dofs": 3 * N, "instances_per_step": B,
            "material": "two-phase voxel E in {1.0, 0.1} (sigma 3), nu 0.3, per element",
            "l2": "flushed before every timed step (512 MB write)"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.path = None
        self.index = device_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

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
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def issue_roofline(n, variant, elem_ms, clk, peaks):
    """Instruction-issue roofline of the element kernel: ncu's warp-instruction
    count over 152 SMs x 4 issue slots per clock at the sampled SM clock."""
    wi = ncu_figure(n, variant, "warp_instructions")
    if wi is None:
        return None
    mhz = (clk or {}).get("sm_mhz") or (peaks or {}).get("sm_max_mhz", 2070.0)
    bound_us = wi / (152 * 4 * mhz * 1e6) * 1e6
    return {"warp_instructions": wi, "issue_bound_us": bound_us, "measured_us": elem_ms * 1e3,
            "frac": bound_us / (elem_ms * 1e3), "sm_mhz": mhz}


def max_over_ranks(x: float) -> float:
    """The largest x over all ranks of the default process group (the
    whole-job time is the slowest rank's); CUDA tensors under NCCL, host
    tensors under gloo."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def _c_oracle(n, seed, threads):
    """The C oracle (FP64, OpenMP) set up on the bench workload: returns
    (oracle, control, full dof vector)."""
    from oracle import c_oracle
    mesh, settings, E, u = workload(n, seed)
    L = c_oracle.CLossOracle("hex8", "elastic", mesh.nodes_coordinates, mesh.elements_nodes["hexahedron"],
                             dirichlet=settings["dirichlet_bc_dict"], node_sets=mesh.node_sets,
                             control_layout="element", threads=threads)
    return L, E.astype(np.float64), L.py.full_dof_vector(u.astype(np.float64))


def _host_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_baseline_port(n, seed, budget_s=10.0):
    """C oracle (FP64 restatement of the reference's element algorithm, OpenMP
    over every host core) on the full bench workload: loss + adjoint of the
    whole mesh per repetition, as many repetitions as fit in about budget_s.
    Falls back to the NumPy oracle on a 12^3 sample when the C oracle does not
    build."""
    threads = _host_threads()
    try:
        L, ctrl, u = _c_oracle(n, seed, threads)
    except Exception as exc:  # noqa: BLE001
        return _cpu_baseline_numpy(reason=f"C oracle unavailable ({type(exc).__name__}: {exc})")
    L.loss_adjoint(ctrl, u)
    t0 = time.perf_counter()
    reps = 0
    while True:
        L.loss_adjoint(ctrl, u)
        reps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = (time.perf_counter() - t0) / reps
    E = n ** 3
    return {"value": E / dt / 1e6, "unit": "M elements/s", "cores": L.max_threads, "kind": "port",
            "sample": f"C FP64 oracle (OpenMP, {L.max_threads} threads), hex8 elastic loss+adjoint of the whole "
                      f"{n}^3 mesh ({E} elements), {reps} repetitions, {dt * 1e3:.1f} ms each"}


def _cpu_baseline_numpy(n_sample=12, seed=7, reason=""):
    """NumPy FP64 oracle, one thread, on a 12^3 sample (fallback)."""
    from oracle import fe_oracle as fo
    from folax_gb300 import fields
    from folax_gb300.mesh import create_3D_box_mesh
    m = create_3D_box_mesh(n_sample, n_sample, n_sample)
    L = fo.FELossOracle("hex8", "elastic", m.nodes_coordinates, m.elements_nodes["hexahedron"],
                        dirichlet={"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.05}},
                        node_sets=m.node_sets, control_layout="element")
    ctrl = fields.two_phase_voxels(n_sample, seed)
    u = 0.01 * np.random.default_rng(seed).standard_normal(L.total_dofs)
    L.batch_loss_and_grads(ctrl[None], u[None])
    t0 = time.perf_counter()
    reps = 0
    while True:
        L.batch_loss_and_grads(ctrl[None], u[None])
        reps += 1
        if time.perf_counter() - t0 > 10.0:
            break
    dt = (time.perf_counter() - t0) / reps
    E = n_sample ** 3
    return {"value": E / dt / 1e6, "unit": "M elements/s", "cores": 1, "kind": "port",
            "sample": f"NumPy FP64 oracle, hex8 elastic loss+adjoint on a {n_sample}^3 mesh ({E} elements), "
                      f"{reps} repetitions, {dt * 1e3:.1f} ms each. {reason}"}


# GPU results kept for the CPU leg's checks against the FP64 oracle
_CPU_CHECKS = {}


def cpu_check_pcg():
    """FP64 Jacobi-CG (C oracle, every host core) of the system the GPU PCG
    solved, at the GPU solve's rtol (the same algorithm and stopping rule)
    and converged (rtol 1e-12): the GPU solution's relative error against
    both."""
    if "pcg" not in _CPU_CHECKS:
        return None
    from oracle import c_oracle
    indptr, indices, vals, r, dx, rtol = _CPU_CHECKS.pop("pcg")
    t0 = time.perf_counter()
    x_same, it_same, _ = c_oracle.pcg(indptr, indices, vals, -r, rtol=rtol, threads=_host_threads())
    x, it, rel = c_oracle.pcg(indptr, indices, vals, -r, rtol=1e-12, threads=_host_threads())
    err = lambda y: float(np.linalg.norm(dx - y) / np.linalg.norm(y))
    return {"error_vs_fp64_cg_same_rtol": err(x_same), "fp64_cg_same_rtol_iterations": it_same,
            "error_vs_fp64_cg_converged": err(x), "fp64_cg_converged_iterations": it,
            "fp64_cg_converged_relative_residual": rel, "fp64_checks_s": time.perf_counter() - t0,
            "check": "FP64 Jacobi-CG (x0 = 0) of the same assembled fp32 system on the host (C oracle), at the "
                     "GPU solve's rtol and at rtol 1e-12"}


def _events_ms(torch, fn, steps, flush=None):
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        if flush is not None:
            flush.zero_()
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / steps


def extra_pcg(args, loss, ctrl):
    """C1: CSR stiffness assembly + Jacobi-PCG (rtol 1e-8, fp64 dots) on the
    64^3 hex8 workload; time per iteration and SpMV bandwidth."""
    import ctypes as C
    import torch
    from folax_gb300 import _capi
    from folax_gb300.solvers import FiniteElementLinearResidualBasedSolver
    lib = _capi.load()
    u0 = loss.ApplyDirichletBCOnDofVector(torch.zeros(loss.GetTotalNumberOfDOFs(), device="cuda"))
    c = ctrl[0]
    loss.ComputeJacobianMatrixAndResidualVector(c, u0)          # builds the CSR tables once
    torch.cuda.synchronize()
    ms_asm = _events_ms(torch, lambda: loss.ComputeJacobianMatrixAndResidualVector(c, u0), 3)
    jac, r = loss.ComputeJacobianMatrixAndResidualVector(c, u0)
    solver = FiniteElementLinearResidualBasedSolver("pcg", loss, {"linear_solver_settings": {
        "solver": "GB300-pcg", "tol": 1e-8, "maxiter": 20000, "check_every": 64}})
    solver.Initialize()
    # the default engine (one cooperative launch per solve), timed with events
    # around the whole solve call (the graph launch and the report read)
    solver.LinearSolve(jac, r)  # builds and caches the solve graph
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    dx = solver.LinearSolve(jac, r)
    ev1.record()
    torch.cuda.synchronize()
    grid_ms = ev0.elapsed_time(ev1)
    grid_info = dict(solver.last_linear_info)
    # the kernel-loop engine with per-kernel events (kernel tracing runs it)
    lib.folgb_trace_enable(1)
    lib.folgb_trace_reset()
    t0 = time.perf_counter()
    dx_k = solver.LinearSolve(jac, r)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    n_s, t_s, n_u, t_u = C.c_int64(), C.c_double(), C.c_int64(), C.c_double()
    lib.folgb_trace_read(_capi.KERNEL_IDS["pcg_spmv"], C.byref(n_s), C.byref(t_s))
    lib.folgb_trace_read(_capi.KERNEL_IDS["pcg_update"], C.byref(n_u), C.byref(t_u))
    lib.folgb_trace_enable(0)
    info = solver.last_linear_info
    it = max(1, info["iterations"])
    # true residual of the returned fp32 solution, fp64 on the host (the
    # solver's own figure is that of its fp64 iterate)
    A = jac.to_scipy()
    dx_h, r_h = dx.double().cpu().numpy(), r.double().cpu().numpy()
    res = np.linalg.norm(A @ dx_h + r_h) / np.linalg.norm(r_h)
    # kept for the CPU leg, which checks dx against an FP64 CG of this system
    _CPU_CHECKS["pcg"] = (A.indptr, A.indices, A.data, r_h, dx_h, 1e-8)
    plan = jac.plan
    N = plan.num_nodes
    nnz = plan.nnz
    pairs = nnz // 9
    # plain SpMV y = A x (folgb_spmv), timed alone: values, adjacency, x and y
    xv = torch.randn(plan.total_dofs, device="cuda")
    yv = torch.empty_like(xv)
    spmv = lambda: _capi.check("folgb_spmv", lib.folgb_spmv(plan.handle, _capi.ptr(jac.data), _capi.ptr(xv),
                                                          _capi.ptr(yv), _capi.stream_handle()))
    for _ in range(3):
        spmv()
    spmv_ms = _events_ms(torch, spmv, 20)
    spmv_bytes = 4 * nnz + 4 * pairs + 4 * (N + 1) + 4 * 3 * N + 4 * 3 * N
    peaks = measured_peaks() or {}
    git = max(1, grid_info["iterations"])
    return {"dofs": plan.total_dofs, "nnz": nnz, "assembly_ms": ms_asm,
            "grid_engine": {"iterations": grid_info["iterations"], "status": grid_info["status"],
                            "solve_ms": grid_ms, "ms_per_iteration": grid_ms / git,
                            "relative_residual": grid_info["relative_residual"],
                            "timing": "CUDA events around the solve call: one cooperative launch for the whole "
                                      "solve, SpMV and vector update fused per iteration"},
            "kernels_engine_iterations": info["iterations"],
            "status": info["status"], "kernels_engine_solve_ms": wall * 1e3,
            "kernels_engine_ms_per_iteration": wall * 1e3 / it,
            "kernel_ms_per_iteration": (t_s.value + t_u.value) / it,
            "pcg_spmv_kernel_ms": t_s.value / max(1, n_s.value), "pcg_update_kernel_ms": t_u.value / max(1, n_u.value),
            "pcg_launches": [n_s.value, n_u.value], "spmv_ms": spmv_ms,
            "spmv_gbs": spmv_bytes / (spmv_ms * 1e-3) / 1e9,
            "spmv_hbm_frac": spmv_bytes / (spmv_ms * 1e-3) / 1e9 / peaks.get("hbm_gbs", 6800.0),
            "iterate_relative_residual": info["relative_residual"],
            "returned_fp32_relative_residual": float(res),
            "note": "Jacobi-PCG, fp32 matrix/vectors, fp64 dots, norms and iterate, reliable updates; the solver "
                    "stops on the fp64 iterate's true residual (iterate_relative_residual); the solution it "
                    "returns is that iterate rounded to fp32 (returned_fp32_relative_residual); "
                    "wall time includes one host flag read per 64 iterations"}


def extra_small_thermal(args, n=50, seed=5):
    """C0 on the GPU: quad4 steady heat conduction on the unit square, 50 x 50
    elements, k = 0.1 + 0.9 sigmoid(16 Fourier modes) per element, T = 1 at
    x = 0, T = 0 at x = 1: CSR assembly + Jacobi-PCG to rtol 1e-10 (fp32
    vectors, fp64 dots and iterate: the single-cluster solver), as a linear FE
    solve (fe_linear_residual_based_solver.py:15-22) through the public API."""
    import torch
    from folax_gb300 import workloads
    from folax_gb300.loss import ThermalLoss2DQuad
    from folax_gb300.solvers import FiniteElementLinearResidualBasedSolver
    m, settings, k = workloads.square_thermal(n, seed)
    loss = ThermalLoss2DQuad("c0", settings, m)
    loss.Initialize()
    solver = FiniteElementLinearResidualBasedSolver("c0", loss, {"linear_solver_settings": {
        "solver": "GB300-pcg", "tol": 1e-10, "maxiter": 20000, "vector_precision": "fp32"}})
    solver.Initialize()
    kt = torch.tensor(k, dtype=torch.float32, device="cuda")
    T0 = torch.zeros(loss.GetTotalNumberOfDOFs(), device="cuda")
    for _ in range(3):
        solver.Solve(kt, T0)
    torch.cuda.synchronize()
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        T = solver.Solve(kt, T0)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    info = solver.last_linear_info
    return {"mesh": f"{n}x{n} quad4", "dofs": loss.GetTotalNumberOfDOFs(), "ms_per_solve": ms,
            "iterations": info["iterations"], "status": info["status"],
            "ms_per_iteration": ms / max(1, info["iterations"]), "rtol": 1e-10,
            "relative_residual": info["relative_residual"],
            "note": "wall time of assembly + Dirichlet + PCG + update through the solver API, one host sync per solve"}


def extra_batched(args, n_inst=512, seed=11):
    """C3: 512 quad4 thermal instances, side n ~ U{16..128}, own Fourier
    conductivity each: fused loss + adjoint + Adam on the nodal field as one
    CUDA graph (elements per tile chosen by the autotuner), against the same
    step as per-instance launches."""
    import torch
    from folax_gb300 import workloads
    from folax_gb300.batched import AdamState, BatchedFELoss, capture_step
    from folax_gb300.loss import ThermalLoss2DQuad
    meshes, settings, ks = workloads.thermal_instances(n_inst, seed)
    t0 = time.perf_counter()
    bl = BatchedFELoss("quad", "thermal", meshes, settings, elements_per_tile=1024)
    t_plan = time.perf_counter() - t0
    ctrl = torch.tensor(np.concatenate(ks), dtype=torch.float32, device="cuda")
    T = torch.rand(bl.total_dofs, device="cuda", generator=torch.Generator(device="cuda").manual_seed(seed))
    out = (torch.empty(n_inst, device="cuda"), torch.empty_like(T), torch.empty_like(ctrl))
    tune = bl.Autotune(ctrl, T, repeats=5)  # elements per tile of the launch
    adam = AdamState(T, lr=1e-3)

    def step():
        bl.ComputeLossAndGrad(ctrl, T, out=out)
        adam.update(T, out[1])

    g, _ = capture_step(step, warmup=3)
    steps = 20
    ms_graph = _events_ms(torch, g.replay, steps)
    # per-instance launches: the same work, one loss object and launch set
    # (element kernel + gather + Adam) per instance
    per = []
    offs_c, offs_d = bl.control_offsets, bl.dof_offsets
    for i, m in enumerate(meshes):
        L = ThermalLoss2DQuad("i", dict(settings), m)
        L.Initialize()
        ci = ctrl[offs_c[i]:offs_c[i + 1]][None]
        Ti = T[offs_d[i]:offs_d[i + 1]].clone()[None]
        per.append((L, ci, Ti, AdamState(Ti[0], lr=1e-3)))

    def per_step():
        for L, ci, Ti, st in per:
            _, _, _, du, _ = L.ComputeBatchLossAndGrad(ci, Ti)
            st.update(Ti[0], du[0])

    per_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    per_steps = 3
    for _ in range(per_steps):
        per_step()
    torch.cuda.synchronize()
    ms_per = (time.perf_counter() - t0) * 1e3 / per_steps
    # the same per-instance launch sets captured as one CUDA graph: no host
    # dispatch, only the per-instance launches themselves
    g_per, _ = capture_step(per_step, warmup=1)
    ms_per_graph = _events_ms(torch, g_per.replay, 5)
    E = bl.num_elements
    return {"instances": n_inst, "elements": E, "nodes": bl.num_nodes, "plan_s": t_plan,
            "autotune": {"elements_per_tile": tune["chosen"],
                         "ms_per_tile_size": dict(zip(map(str, BatchedFELoss.BATCH_TILES), tune["ms"]))},
            "graph_ms_per_step": ms_graph, "graph_melem_s": E / (ms_graph * 1e-3) / 1e6,
            "per_instance_graph_ms_per_step": ms_per_graph,
            "per_instance_graph_melem_s": E / (ms_per_graph * 1e-3) / 1e6,
            "per_instance_eager_ms_per_step": ms_per, "per_instance_eager_melem_s": E / (ms_per * 1e-3) / 1e6,
            "speedup_batched_vs_per_instance": ms_per_graph / ms_graph,
            "speedup_batched_vs_per_instance_eager": ms_per / ms_graph,
            "step": "fused loss + adjoint (one persistent launch + gather) + Adam on the nodal field, one CUDA graph",
            "per_instance_step": "the same work as one launch set (element kernel, gather, Adam) per instance; "
                                 "graph: all 512 launch sets captured as one CUDA graph (the speed-up denominator); "
                                 "eager: the same from the Python API (wall clock)"}


def extra_neohooke(args, n=64, batch=16, seed=2024):
    """C4: tet4 Neo-Hookean (6-tet split of a 64^3 hex grid, 1 Gauss point),
    mu/lambda scaled by the two-phase field, 16 microstructures: fused loss +
    adjoint throughput (element kernel + node gather)."""
    import torch
    from folax_gb300 import workloads
    from folax_gb300.loss import NeoHookeMechanicalLoss3DTetra
    mesh, settings, E_b, u_b = workloads.neohooke_tets(n, batch, seed)
    loss = NeoHookeMechanicalLoss3DTetra("nh", settings, mesh)
    loss.Initialize()
    U = torch.tensor(u_b, device="cuda")
    Cb = torch.tensor(E_b, device="cuda")
    for _ in range(3):
        loss.ComputeBatchLossAndGrad(Cb, U)
    torch.cuda.synchronize()
    ms = _events_ms(torch, lambda: loss.ComputeBatchLossAndGrad(Cb, U), 10)
    loss.CheckDeviceStatus()  # no non-finite value or inverted element in the timed work
    E = len(mesh.elements_nodes["tetra"])
    return {"tets": E, "batch": batch, "ms_per_step": ms, "melem_s": batch * E / (ms * 1e-3) / 1e6,
            "microstructures": "one two-phase field per instance"}


def extra_minimiser(args, n=16, seed=2024):
    """The Newton oracle of the C4 loss minimiser on the n^3 split
    (newton_minimiser; n = --minimiser-n, 16 by default).  The reference Neo-Hookean model is not stress-free
    at C = I (S = -mu I): its tangent is indefinite near u = 0 and full
    Newton steps from u = 0 invert elements beyond ~6^3, so the minimiser is
    found with the energy line search."""
    return newton_minimiser(n, seed)


def newton_minimiser(n, seed, abs_tol=1e-7):
    """The Newton oracle of the loss minimiser (one instance): neo-Hookean
    (AD) on the 6-tet split of an n^3 grid with the consistent shear
    convention (residual = energy gradient), the reference's 5 load steps,
    device-resident Newton with the energy line search, fp64-vector BiCGSTAB
    (rtol 1e-8) for the tangent systems, to |r| < abs_tol; then the fused
    loss gradient at the root against its value at u = 0."""
    import torch
    from folax_gb300 import workloads
    from folax_gb300.loss import NeoHookeMechanicalLoss3DTetra
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    mesh, settings, E_b, _ = workloads.neohooke_tets(n, 1, seed)
    settings = dict(settings, voigt_shear_mode="consistent")
    loss = NeoHookeMechanicalLoss3DTetra("nh_newton", settings, mesh)
    loss.Initialize()
    solver = FiniteElementNonLinearResidualBasedSolver("nl", loss, {
        "linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-8, "maxiter": 50000,
                                   "vector_precision": "fp64", "check_every": 64},
        "nonlinear_solver_settings": {"load_incr": 5, "maxiter": 60, "abs_tol": abs_tol, "rel_tol": 1e-12,
                                      "device_resident": True, "line_search": True}})
    solver.Initialize()
    u0 = np.zeros(loss.GetTotalNumberOfDOFs(), dtype=np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    err = None
    try:
        u = solver.Solve(E_b[0], u0)
    except Exception as exc:  # noqa: BLE001
        err = f"{type(exc).__name__}: {exc}"
        u = None
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    h = solver.history
    info = solver.last_newton_info or {}
    res = {"mesh": f"{n}^3 hex split into {len(mesh.elements_nodes['tetra'])} tets",
           "dofs": loss.GetTotalNumberOfDOFs(), "abs_tol": abs_tol, "solve_ms": wall * 1e3,
           "newton_iterations": len(h), "ms_per_newton_iteration": wall * 1e3 / max(1, len(h)),
           "iterations_per_load_step": [sum(1 for x in h if x["load_step"] == k) for k in range(1, 6)],
           "final_res_norm": h[-1]["res_norm"] if h else None, "newton_info": info, "error": err,
           "solve": "one CUDA graph: load steps x Newton iterations, assembly, fp64-vector BiCGSTAB, "
                    "energy line search"}
    if u is not None:
        z = np.zeros((1, loss.GetTotalNumberOfDOFs()), dtype=np.float32)
        g0 = loss.ComputeBatchLossAndGrad(E_b[:1], z)[3]
        g1 = loss.ComputeBatchLossAndGrad(E_b[:1], u[None])[3]
        res["loss_gradient_at_root_relative"] = float(g1.norm() / g0.norm())
    return res


def fp32_peak(torch, lib):
    """Measured FP32 peak of this GPU: the library's FMA-chain probe
    (folgb_fp32_peak_probe: 8 blocks of 256 threads per SM, 8 independent
    packed-pair FMA chains per thread), timed with CUDA events.  Changes no
    GPU setting.  Returns (TFLOP/s, ms per launch)."""
    import ctypes as C
    from folax_gb300 import _capi
    sink = torch.zeros(1, device="cuda")
    flops = C.c_double()

    def run():
        _capi.check("folgb_fp32_peak_probe", lib.folgb_fp32_peak_probe(_capi.ptr(sink), 8, 4096, C.byref(flops),
                                                                       _capi.stream_handle()))

    for _ in range(3):
        run()
    ms = _events_ms(torch, run, 10)
    return flops.value / (ms * 1e-3) / 1e12, ms


def extra_fused(args, loss, ctrl, u):
    """The headline step alone, eager, for profiling runs: 8 fused loss +
    adjoint calls on the 64^3 workload (the plan's kernel variant:
    --hex8-variant forces one), then 3 calls of the plain path (element
    matrices in HBM + separate backward) on the same inputs."""
    import torch
    for _ in range(8):
        loss.ComputeBatchLossAndGrad(ctrl, u)
    torch.cuda.synchronize()
    loss.CheckDeviceStatus()
    for _ in range(3):
        loss.ComputeBatchLossAndGrad(ctrl, u, plain=True)
    torch.cuda.synchronize()
    return {"fused_calls": 8, "plain_calls": 3, "variant": args.hex8_variant}


def extra_jittered(args):
    """The headline step (fused loss + adjoint, 64^3 hex8, graph replay, L2
    flushed) on a mesh whose interior nodes are moved by N(0, (0.1 h)^2): no
    element is a parallelepiped, so the element kernel takes its general
    (non-affine) path at every Gauss point."""
    import torch
    from folax_gb300.batched import capture_step
    from folax_gb300.loss import MechanicalLoss3DHexa
    mesh, settings, E_h, u_h = workload(args.n, args.seed, jitter=0.1)
    loss = MechanicalLoss3DHexa("jittered", settings, mesh)
    loss.Initialize()
    ctrl = torch.from_numpy(E_h).cuda()[None]
    u = torch.from_numpy(u_h).cuda()[None]
    tune = loss.Autotune(ctrl, u, repeats=3)
    g, _ = capture_step(lambda: loss.ComputeBatchLossAndGrad(ctrl, u), warmup=3)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    ms = _events_ms(torch, g.replay, 20, flush)
    nE = args.n ** 3
    return {"mesh": f"{args.n}^3 hex8, interior nodes jittered by N(0, (0.1 h)^2)", "ms_per_step": ms,
            "melem_s": nE / (ms * 1e-3) / 1e6, "chosen_variant": tune["chosen"],
            "timing": "CUDA-graph replay of the fused step, L2 flushed before every step"}


def extra_fourier(args, n=64, batch=4, freqs=4, seed=2024):
    """FOL training step with a Fourier-parametrised Young's modulus on the
    64^3 hex8 workload (fourier_control.py:24-59 in front of fe_loss.py:250-262):
    coefficients -> nodal E -> fused loss + adjoint -> dL/dcoefficients ->
    Adam on the coefficients, batch 4, 4 x 4 x 4 frequencies, one CUDA graph
    (L2 flushed before every timed step); and the control's VJP alone."""
    import torch
    from folax_gb300.batched import AdamState, capture_step
    from folax_gb300.fields import FourierControl
    from folax_gb300.loss import MechanicalLoss3DHexa
    mesh, settings, _, u_h = workload(n, seed)
    settings = dict(settings, control_layout="nodal")
    loss = MechanicalLoss3DHexa("fourier", settings, mesh)
    loss.Initialize()
    fr = np.arange(1, freqs + 1)
    fc = FourierControl("E", {"x_freqs": fr, "y_freqs": fr, "z_freqs": fr, "beta": 20.0, "min": 0.1, "max": 1.0},
                        mesh)
    fc.Initialize()
    gen = torch.Generator(device="cuda").manual_seed(seed)
    coeffs = torch.rand((batch, fc.GetNumberOfVariables()), device="cuda", generator=gen)
    u = loss.ApplyDirichletBCOnDofVector(torch.tensor(u_h, device="cuda")).reshape(1, -1).repeat(batch, 1)
    adam = AdamState(coeffs, lr=1e-3)

    def step():
        E = fc.ComputeBatchControlledVariables(coeffs)
        _, _, losses, du, dE = loss.ComputeBatchLossAndGrad(E, u)
        dc = fc.ComputeBatchControlledVariablesVJP(coeffs, dE)
        adam.update(coeffs, dc)
        return losses, dc

    g, _ = capture_step(step, warmup=3)
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    steps = 20
    ms_step = _events_ms(torch, g.replay, steps, flush)
    E0 = fc.ComputeBatchControlledVariables(coeffs)
    dv = torch.ones_like(E0)
    ms_vjp = _events_ms(torch, lambda: fc.ComputeBatchControlledVariablesVJP(coeffs, dv), steps, flush)
    ms_fwd = _events_ms(torch, lambda: fc.ComputeBatchControlledVariables(coeffs), steps, flush)
    nE = n ** 3
    return {"mesh": f"{n}^3 hex8", "instances": batch, "coefficients": fc.GetNumberOfVariables(),
            "graph_ms_per_step": ms_step, "melem_s": batch * nE / (ms_step * 1e-3) / 1e6,
            "control_forward_ms": ms_fwd, "control_vjp_ms": ms_vjp,
            "step": "Fourier control forward + fused loss/adjoint + control VJP + Adam, one CUDA graph, L2 flushed"}


def extra_newton(args, n=10, seed=7, steps=5):
    """A whole nonlinear solve, Saint-Venant-Kirchhoff hex8 on an n^3 box
    (two-phase nodal Young's modulus, bottom fixed, top stretched by 0.1 in
    4 load steps): the device-resident Newton solve (one CUDA graph) against
    the host-driven Newton loop, wall time per solve with the result on the
    device."""
    import torch
    from folax_gb300 import fields
    from folax_gb300.loss import SaintVenantMechanicalLoss3DHexa
    from folax_gb300.mesh import create_3D_box_mesh
    from folax_gb300.solvers import FiniteElementNonLinearResidualBasedSolver
    mesh = create_3D_box_mesh(n, n, n)
    settings = {"dirichlet_bc_dict": {"Ux": {"bottom": 0.0}, "Uy": {"bottom": 0.0}, "Uz": {"bottom": 0.0, "top": 0.1}},
                "material_dict": {"young_modulus": 1.0, "poisson_ratio": 0.3}}
    loss = SaintVenantMechanicalLoss3DHexa("svk", dict(settings), mesh)
    loss.Initialize()
    Ee = fields.two_phase_voxels(n, seed)
    ctrl = np.zeros(mesh.GetNumberOfNodes())
    cnt = np.zeros(mesh.GetNumberOfNodes())
    conn = mesh.elements_nodes["hexahedron"]
    np.add.at(ctrl, conn, Ee[:, None])
    np.add.at(cnt, conn, 1.0)
    ctrl = (ctrl / cnt).astype(np.float32)
    out = {"mesh": f"{n}^3 hex8, Saint-Venant-Kirchhoff", "dofs": loss.GetTotalNumberOfDOFs()}
    for resident in (True, False):
        solver = FiniteElementNonLinearResidualBasedSolver("nl", loss, {
            "linear_solver_settings": {"solver": "JAX-bicgstab", "tol": 1e-8, "maxiter": 5000},
            "nonlinear_solver_settings": {"load_incr": 4, "maxiter": 10, "abs_tol": 1e-6, "rel_tol": 1e-7,
                                          "device_resident": resident}})
        solver.Initialize()
        u0 = np.zeros(loss.GetTotalNumberOfDOFs(), dtype=np.float32)
        for _ in range(2):
            solver.Solve(ctrl, u0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            x = solver.Solve(ctrl, u0)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / steps * 1e3
        key = "device_resident" if resident else "host_loop"
        out[key] = {"ms_per_solve": ms, "newton_iterations": len(solver.history),
                    "final_res_norm": solver.history[-1]["res_norm"] if solver.history else None}
        if resident:
            out[key]["krylov_iterations"] = (solver.last_newton_info or {}).get("krylov_iterations")
        out[key + "_solution_norm"] = float(torch.linalg.vector_norm(x.double()).item())
    out["speedup_device_resident"] = out["host_loop"]["ms_per_solve"] / out["device_resident"]["ms_per_solve"]
    return out


def run_reference(args):
    """The reference's algorithm on the host cores: the C oracle (FP64,
    OpenMP over every core; the reference itself is JAX, which is not
    installed) evaluates loss + adjoint of the whole bench mesh each step.
    Rank 0 only; other ranks exit without work."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = _host_threads()
    try:
        L, ctrl, u = _c_oracle(args.n, args.seed, threads)
    except Exception as exc:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"C oracle did not build: {type(exc).__name__}"}))
        return
    for _ in range(max(1, args.warmup)):
        L.loss_adjoint(ctrl, u)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.loss_adjoint(ctrl, u)
    dt = (time.perf_counter() - t0) / args.steps
    E = args.n ** 3
    value = E / dt / 1e6
    line = {"metric": "M elements/s, FE loss+adjoint vs plain assembly on same GPU, at 1e-5 rel err",
            "impl": "reference", "value": value, "unit": "M elements/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded two-phase voxels, noisy uniaxial u)",
            "config": workload_config(args.n, 1),
            "cpu_baseline": {"value": value, "unit": "M elements/s", "cores": L.max_threads, "kind": "port",
                             "sample": f"C FP64 oracle restating the reference's element algorithm (the reference "
                                       f"is JAX, not installed): the whole {args.n}^3 mesh ({E} elements) per step, "
                                       f"{L.max_threads} OpenMP threads"},
            "e2e": {"value": value, "unit": "M elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_extras(args, loss, ctrl, u=None):
    """The extra measurements named by --extras; a failed one is reported, not hidden."""
    import torch
    extras = {}
    wanted = set(args.extras.split(","))
    for key, name, fn in (("fused", "fused_step_hex8_64", lambda: extra_fused(args, loss, ctrl, u)),
                          ("jittered", "jittered_hex8_64", lambda: extra_jittered(args)),
                          ("small", "plain_small_quad4_thermal_50", lambda: extra_small_thermal(args)),
                          ("pcg", "pcg_hex8_64", lambda: extra_pcg(args, loss, ctrl)),
                          ("batched", "batched_quad4_512", lambda: extra_batched(args)),
                          ("neohooke", "neohooke_tet4_batch16", lambda: extra_neohooke(args)),
                          ("minimiser", f"newton_minimiser_tet4_{args.minimiser_n}",
                           lambda: extra_minimiser(args, n=args.minimiser_n)),
                          ("newton", "newton_svk_hex8_10", lambda: extra_newton(args)),
                          ("fourier", "fourier_hex8_64_batch4", lambda: extra_fourier(args))):
        if key not in wanted:
            continue
        try:
            extras[name] = fn()
        except Exception as exc:  # noqa: BLE001
            extras[name] = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()
    return extras


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist
    from folax_gb300 import _capi
    from folax_gb300.loss import HEX8_VARIANT_NAMES, MechanicalLoss3DHexa
    import ctypes as C

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    mesh, settings, E_h, u_h = workload(args.n, args.seed)
    if args.hex8_variant is not None:
        settings["kernel_variant"] = int(args.hex8_variant)
    loss = MechanicalLoss3DHexa("bench", settings, mesh)
    loss.Initialize()
    lib = _capi.load()
    ctrl = torch.from_numpy(E_h).cuda()[None]
    u = torch.from_numpy(u_h).cuda()[None]
    if args.only_extras:  # profiling runs: the extra workloads alone
        print(json.dumps({"extras": run_extras(args, loss, ctrl, u)}))
        return
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    nE = args.n ** 3
    B = 1

    def timed(fn, steps):
        total = 0.0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev[k][0].record()
            fn()
            ev[k][1].record()
        torch.cuda.synchronize()
        for a, b in ev:
            total += a.elapsed_time(b)
        return total / steps

    tune = loss.Autotune(ctrl, u, repeats=5)
    fused = lambda: loss.ComputeBatchLossAndGrad(ctrl, u)
    plain = lambda: loss.ComputeBatchLossAndGrad(ctrl, u, plain=True)
    for _ in range(args.warmup):
        fused()
    torch.cuda.synchronize()
    # the step as a CUDA graph (the same kernels; no host launch overhead)
    from folax_gb300.batched import capture_step
    graph, _ = capture_step(fused, warmup=1)
    step = graph.replay
    barrier()
    torch.cuda.synchronize()
    # clocks are sampled from before a one-second untimed soak (steady clocks,
    # enough samples) to the end of the timed region
    clocks = Clocks(local)
    clocks.start()
    t_end = time.perf_counter() + (0.0 if args.no_soak else 1.0)
    while time.perf_counter() < t_end:
        for _ in range(20):
            step()
        torch.cuda.synchronize()
    ms = timed(step, args.steps)
    clk = clocks.stop()
    ms_eager = timed(fused, args.steps)
    torch.cuda.synchronize()
    barrier()
    if world > 1:
        ms = max_over_ranks(ms)
    value = world * B * nE / (ms * 1e-3) / 1e6

    # dominant kernel: tracing events around the element kernel
    lib.folgb_trace_enable(1)
    lib.folgb_trace_reset()
    timed(fused, max(3, args.steps // 2))
    n_l, t_ms = C.c_int64(), C.c_double()
    lib.folgb_trace_read(_capi.KERNEL_IDS["elem_loss"], C.byref(n_l), C.byref(t_ms))
    elem_ms = t_ms.value / max(1, n_l.value)
    lib.folgb_trace_read(_capi.KERNEL_IDS["gather"], C.byref(n_l), C.byref(t_ms))
    gather_ms = t_ms.value / max(1, n_l.value)
    lib.folgb_trace_enable(0)

    # plain path
    for _ in range(2):
        plain()
    ms_plain_eager = timed(plain, args.plain_steps)
    graph_plain, _ = capture_step(plain, warmup=1)
    ms_plain = timed(graph_plain.replay, args.plain_steps)
    value_plain = B * nE / (ms_plain * 1e-3) / 1e6

    # end to end through the public API with host buffers
    u_pin = torch.from_numpy(u_h).pin_memory()[None]
    c_pin = torch.from_numpy(E_h).pin_memory()[None]
    out_du = torch.empty_like(u_pin).pin_memory()
    out_dc = torch.empty_like(c_pin).pin_memory()
    out_l = torch.empty(1).pin_memory()

    def e2e_step():
        # the public API with pinned host buffers: the dofs are copied in, the
        # element controls read in place, the gradients stored straight into
        # the host result buffers by the kernels, the loss copied out; each
        # step's timed region ends when all of it has reached host memory
        loss.ComputeBatchLossAndGrad(c_pin, u_pin, out=(out_l, out_du, out_dc))

    for _ in range(3):
        e2e_step()
    ms_e2e = timed(e2e_step, args.steps)
    h2d = u_pin.numel() * 4 + c_pin.numel() * 4
    d2h = out_du.numel() * 4 + out_dc.numel() * 4 + 4

    # roofline of the element kernel (for the grid variants: the whole step,
    # one kernel).  Algorithmic bytes: control 4 B + dLoss/dE 4 B per
    # element, dofs 12 B + dLoss/du 12 B per node (each node read and written
    # once); the connectivity 32 B per element where the kernel reads it (not
    # the structured grid) and the coordinates 12 B per node where it reads
    # them (the pointwise variants).  The element records of the two-kernel
    # variants are intermediate traffic, not algorithmic.  Flops: the FP32
    # operations of the variant's element (ncu-counted where a capture
    # exists; the box element counted from its source).  bound: the resource
    # whose measured peak the kernel comes closer to.
    N = (args.n + 1) ** 3
    chosen = tune["chosen"]
    alg_bytes = nE * (4 + 4) + N * (12 + 12)
    if chosen not in GRID_VARIANTS:
        alg_bytes += nE * 32
    if chosen not in BOX_VARIANTS + GRID_VARIANTS:
        alg_bytes += N * 12
    kernel_ms = elem_ms  # the grid variants launch no gather
    achieved_gbs = alg_bytes / (kernel_ms * 1e-3) / 1e9
    peaks = measured_peaks()
    hbm = (peaks or {}).get("hbm_gbs", 6800.0)
    fp32_tflops, fp32_probe_ms = fp32_peak(torch, lib)
    flops_launch = ncu_figure(args.n, chosen, "fp32_flops")
    flops_src = "ncu-counted FP32 operations of this kernel variant"
    if flops_launch is None and chosen in BOX_VARIANTS + GRID_VARIANTS:
        flops_launch = BOX_FLOPS_PER_ELEMENT * nE
        flops_src = "box element counted from the kernel source (owned elements; the grid kernel's halo elements " \
                    "and node sums not included)"
    elif flops_launch is None:
        flops_launch = FLOPS_PER_ELEMENT * nE
        flops_src = "naive per-element count, an upper bound (no ncu figure for this variant)"
    fp32_achieved = flops_launch / (kernel_ms * 1e-3) / 1e12
    issue = issue_roofline(args.n, chosen, kernel_ms, clk, peaks) or {}
    fp32_frac, hbm_frac = fp32_achieved / fp32_tflops, achieved_gbs / hbm
    fp32_bound = fp32_frac >= hbm_frac
    roofline = {"bound": "fp32" if fp32_bound else "hbm",
                "achieved": fp32_achieved if fp32_bound else achieved_gbs,
                "peak": fp32_tflops if fp32_bound else hbm,
                "unit": "TFLOP/s" if fp32_bound else "GB/s",
                "frac": fp32_frac if fp32_bound else hbm_frac,
                "traffic": ncu_figure(args.n, chosen, "traffic"),
                "traffic_unit": "bytes per launch (ncu dram read + write)",
                "fp32_achieved_tflops": fp32_achieved, "fp32_peak_tflops": fp32_tflops, "fp32_frac": fp32_frac,
                "flops_per_launch": flops_launch, "flops_source": flops_src,
                "naive_flops_per_element": FLOPS_PER_ELEMENT,
                "fp32_peak_source": "measured in this run: folgb_fp32_peak_probe (FFMA2 chains on every SM), "
                                    f"{fp32_probe_ms:.3f} ms per probe launch",
                "hbm_achieved_gbs": achieved_gbs, "hbm_peak_gbs": hbm, "hbm_frac": hbm_frac,
                "hbm_peak_source": "of measured: MEASURED_PEAKS.json hbm_gbs" if peaks else "of fallback 6800 GB/s",
                "algorithmic_bytes": alg_bytes,
                "issue_frac": issue.get("frac"), "issue_bound_us": issue.get("issue_bound_us"),
                "warp_instructions": issue.get("warp_instructions"),
                "kernel_us": kernel_ms * 1e3,
                "kernel": "hex8 2x2x2 element kernel, variant %d (%s)" % (chosen, HEX8_VARIANT_NAMES[chosen])}

    extras = run_extras(args, loss, ctrl) if rank == 0 and not args.no_extras else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_port(args.n, args.seed)
        chk = cpu_check_pcg()
        if chk is not None and extras and isinstance(extras.get("pcg_hex8_64"), dict):
            extras["pcg_hex8_64"].update(chk)
    if rank == 0:
        line = {"metric": "M elements/s, FE loss+adjoint vs plain assembly on same GPU, at 1e-5 rel err",
                "value": value, "unit": "M elements/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "ms_per_step_eager_api": ms_eager,
                "timing": "CUDA-graph replay of the fused step (memset + element kernel + gather, or memset + "
                          "the one-launch grid kernel for variants 23-24); "
                          "ms_per_step_eager_api = the same step through the Python API call",
                "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded two-phase voxels, noisy uniaxial u)",
                "config": workload_config(args.n, B),
                "plain": {"value": value_plain, "unit": "M elements/s", "ms_per_step": ms_plain,
                          "ms_per_step_eager_api": ms_plain_eager,
                          "timing": "CUDA-graph replay, like the fused step",
                          "speedup_fused_vs_plain": value / value_plain},
                "kernels": {"elem_loss_ms": elem_ms, "gather_ms": gather_ms,
                            "autotune": {"chosen_variant": tune["chosen"], "ms_per_variant": tune["ms"],
                                         "variants": HEX8_VARIANT_NAMES}},
                "roofline": roofline,
                "e2e": {"value": B * nE / (ms_e2e * 1e-3) / 1e6, "unit": "M elements/s", "ms_per_step": ms_e2e,
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "cpu_baseline": cpu,
                "clocks": clk,
                "gpu_launches": (1 if chosen in GRID_VARIANTS else 2) * args.steps,
                "extras": extras}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
