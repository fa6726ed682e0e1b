"""Benchmark of the FP64 element-stiffness-and-assembly path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload plate|beam|truss|batch|adjoint|separate|loads|pcg|results]

A step is one numeric assembly pass over the whole mesh into the FP64 CSR
global stiffness (element kernels + deterministic block reduction), with the
CSR pattern built once before timing.  `value` is elements/s of that pass with
the mesh resident in HBM (CUDA events on the library's stream, L2 flushed
between steps); `e2e` is elements/s of the full drop-in call sequence from
host arrays (create, add_nodes, add_plates/beams, assemble, CSR read-back to
host); `roofline` reports the dominant kernel against the measured HBM copy
bandwidth and the measured FP64 FMA rate; `cpu_baseline` times the CPU oracle
(the reference algorithm restated in C, one thread, eager insertion order) on
a bounded sample.  `--impl reference` times the multi-threaded CPU port of the
reference algorithm on all host cores instead.  The path does not shard across
GPUs: `--gpus N` under torchrun runs N independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from finite_element_method_gb300 import FEM, meshes  # noqa: E402

# FP64 peak of a GB300: 2 DFMA per clock per SM (ncu: sm__sass_thread_inst_executed_op_dfma_pred_on
# peak_sustained = 304/cycle on 152 SMs) at the 2070 MHz maximum SM clock, FMA = 2 flops: 1.2586 TFLOP/s.
# (A dependent-chain DFMA loop reached 1.009 TFLOP/s; the hardware figure is the stricter denominator.)
FP64_PEAK_FLOPS = 2 * 152 * 2070e6 * 2

# Algorithmic FP64 work per element of the numeric pass, counted from the kernels' formulation by
# compiling element_math.cuh with an operation-counting double type (FMA = 2 flops, add/mul/div = 1):
#   plate in a global plane (R = I): rotation test and local coordinates 15 add + 6 mul, core 20 add +
#   145 mul + 208 fma + 2 div, 10 node-pair blocks 20 mul + 154 fma = 932
#   plate off the global planes (general R): rotation and local coordinates 30 add + 39 mul + 21 fma + 3 div +
#   3 sqrt, core as above, 10 blocks with their rotation R^T K R on the structural entries 548 mul + 616 fma
#   = 2480
#   beam, I12 != 0: 57 add + 213 mul + 201 fma + 19 div + 7 sqrt (trig as polynomial fma chains) = 698 when
#   I11 >= I22, 897 when I11 < I22 (one more turn of the principal-axes loop: arctangent, sine and cosine);
#   I12 == 0 (principal axes along the section axes, no arctangent and series): 515 when I11 >= I22, and
#   714 when I11 < I22 (one turn of the loop)
#   truss: 20 add + 46 mul + 9 fma + 4 div + 4 sqrt
PLATE_FLOPS = {"flat": (15 + 6) + (20 + 145 + 2 * 208 + 2) + (20 + 2 * 154),
               "tilted": (30 + 39 + 2 * 21 + 3 + 3) + (20 + 145 + 2 * 208 + 2) + (548 + 2 * 616)}
WORK = {
    "plate": dict(elem_flops=PLATE_FLOPS["flat"], pairs=10),
    "beam": dict(elem_flops=57 + 213 + 2 * 201 + 19 + 7, pairs=3),
    "truss": dict(elem_flops=20 + 46 + 2 * 9 + 4 + 4, pairs=3),
}
BEAM_FLOPS = {"general": 698, "general_turn": 897, "aligned": 515, "aligned_turn": 714}


def element_flops(workload, mesh):
    """algorithmic FP64 work of one numeric pass's element kernel over the mesh"""
    if workload == "plate" and mesh.meta.get("rotation") is not None:
        return PLATE_FLOPS["tilted"] * mesh.n_elements
    if workload != "beam":
        return WORK[workload]["elem_flops"] * mesh.n_elements
    b = mesh.beams
    aligned = np.asarray(b["i12"]) == 0.0
    turn = np.asarray(b["i11"]) < np.asarray(b["i22"])
    return (BEAM_FLOPS["general"] * int((~aligned & ~turn).sum()) + BEAM_FLOPS["general_turn"] * int((~aligned & turn).sum())
            + BEAM_FLOPS["aligned"] * int((aligned & ~turn).sum()) + BEAM_FLOPS["aligned_turn"] * int((aligned & turn).sum()))
# bytes per element read by the element kernel (connectivity, coordinates of its nodes, properties)
IN_BYTES = {"plate": 4 * 4 + 4 * 24 + 4 * 8, "beam": 2 * 4 + 2 * 24 + 11 * 8, "truss": 2 * 4 + 2 * 24 + 3 * 8}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per element of one launch of the element kernel,
# from an ncu capture of k_plate on the 500 x 500 plate mesh (250,000 plates: 46.4 MB read + 230.4 MB written),
# scaled by the element count (the kernel's traffic is per element: its inputs and its packed blocks)
TRAFFIC_PER_ELEMENT = {"plate": (46394368 + 230444800) / 250000}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def max_over_ranks(x: float) -> float:
    """the largest of x over the ranks of the default process group (x itself when there is none): every
    replica times the same work, and the job takes as long as its slowest replica"""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """SM clocks and throttle reasons sampled by one `nvidia-smi -lms` process that runs exactly while the timed
    region runs (started on entry, terminated on exit; every line it printed is a sample from inside)."""

    QUERY = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, period_ms=20):
        self.samples, self.max_mhz, self.reasons = [], None, set()
        self._idx, self._period, self._p = gpu_index, period_ms, None

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self._idx), f"--query-gpu={self.QUERY}",
                                        "--format=csv,noheader,nounits", "-lms", str(self._period)],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._p = None
        return self

    def __exit__(self, *exc):
        if self._p is None:
            return
        self._p.terminate()
        try:
            out, _ = self._p.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self._p.kill()
            out, _ = self._p.communicate()
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 6:
                continue
            try:
                self.samples.append(float(f[0]))
                self.max_mhz = float(f[1])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[2:6]):
                if v.lower().startswith("active"):
                    self.reasons.add(name)

    def summary(self):
        return {"sm_mhz": float(np.median(self.samples)) if self.samples else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.samples)}


def tilt_rotation(seed=7):
    """the seeded orthogonal matrix that takes the plate mesh off the global planes (--tilt)"""
    q, _ = np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))
    return q


def make_mesh(workload, nx=1000, tilt=False):
    if workload == "plate":
        n = nx
        if tilt:
            m = meshes.plate_mesh(n, n, rotation=tilt_rotation())
            m.meta["rotation"] = "seeded orthogonal Q (numpy PCG64 seed 7)"
            return m, (f"plate_mesh_{n}x{n} tilted by a seeded orthogonal Q ({n * n:,} 4-node plates off the "
                       f"global planes, general rotation, {(n + 1) ** 2:,} nodes, 6 DOF/node)")
        return meshes.plate_mesh(n, n), (f"plate_mesh_{n}x{n} ({n * n:,} 4-node plates, {(n + 1) ** 2:,} nodes, "
                                         "6 DOF/node)")
    if workload == "beam":
        return meshes.beam_frame(), "beam_frame_101x101x21 (628,220 2-node beams, 214,221 nodes)"
    if workload == "truss":
        return meshes.truss_lattice(), "truss_lattice_11x11x11 (4,630 bars, 1,331 nodes)"
    raise SystemExit(f"unknown workload {workload}")


def sample_mesh(workload):
    """bounded sample of the same workload for the CPU legs (~10 s of one-thread work)."""
    if workload == "plate":
        return meshes.plate_mesh(400, 400), "plate_mesh 400x400 (160,000 plates), same generator"
    if workload == "beam":
        return meshes.beam_frame(41, 41, 21), "beam_frame 41x41x21 (104,140 beams), same generator"
    return meshes.truss_lattice(), "full truss lattice"


def cpu_oracle_eager(mesh):
    """one-thread eager assembly (the reference algorithm: element matrix, T^T K T, zero-skip, hash accumulate
    in call order), from host arrays to CSR; returns elements/s."""
    from oracle.fem_oracle import OracleFEM

    t0 = time.perf_counter()
    o = OracleFEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(o, mesh)
    o.csr()
    dt = time.perf_counter() - t0
    return mesh.n_elements / dt, dt


def run_reference(args):
    """--impl reference: the multi-threaded CPU port of the reference algorithm on all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import fem_oracle

    fem_oracle.lib()
    mesh, sample_desc = sample_mesh(args.workload)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        fem_oracle.assemble_parallel(mesh, cores)
    times = []
    for _ in range(args.steps):
        sec, nnz, _ = fem_oracle.assemble_parallel(mesh, cores)
        times.append(sec)
    t = float(np.mean(times))
    v = mesh.n_elements / t
    line = {"impl": "reference", "metric": "elements/s assembled to FP64 CSR", "value": v, "unit": "elements/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "sample": sample_desc, "nnz": nnz},
            "cpu_baseline": {"value": v, "unit": "elements/s", "cores": cores, "kind": "port",
                             "sample": sample_desc},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """512 independent structures (log-uniform sizes in [1e3, 2e5], seeded kind mix).  (a) From host arrays:
    one plain call sequence per structure (FEM + add_nodes + add_* + assemble) against one batch built from the
    same arrays (Batch.from_meshes: the checks of every structure in bulk on the GPU, one symbolic phase, one
    graph-captured numeric pass).  (b) The numeric pass alone: one batched pass (a CUDA graph with the autotuned
    element phase) against 512 plain per-structure passes.  Returns the result line."""
    import torch

    from finite_element_method_gb300 import Batch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    structures = meshes.batch_structures(n_structures=64 if args.small else 512)
    n_el = sum(m.n_elements for m in structures)
    counts = np.array([m.counts() for m in structures]).sum(0)
    tol = (meshes.REL_TOL, meshes.ABS_TOL)

    def plain_sequences(keep):
        models = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for m in structures:
            g = FEM(*tol, m.nodes_number)
            meshes.load(g, m)
            g.assemble()
            if keep:
                models.append(g)
            else:
                g.close()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, models

    # the batch's input: the same arrays laid out structure after structure (built once, outside the timing)
    t0 = time.perf_counter()
    laid_out = Batch.structures(structures)
    layout_s = time.perf_counter() - t0

    def batch_build():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b = Batch.from_structures(laid_out, *tol)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, b

    # each path once untimed (device memory pool growth, module loading), then timed
    plain_sequences(False)
    _, b = batch_build()
    b.close()
    reps = max(1, min(5, args.e2e_steps))
    t_plain = []
    for _ in range(reps - 1):
        t_plain.append(plain_sequences(False)[0])
    t, models = plain_sequences(True)
    t_plain.append(t)
    t_batch = []
    for _ in range(reps - 1):
        t, b = batch_build()
        b.close()
        t_batch.append(t)
    t, b = batch_build()
    t_batch.append(t)
    phases = b.build_ms()
    # identical results
    for i in (0, len(structures) // 2, len(structures) - 1):
        rp, ci, va = models[i].stiffness_csr()
        brp, bci, bva = b.csr(i)
        assert np.array_equal(rp, brp) and np.array_equal(ci, bci)
        assert np.array_equal(va.view(np.uint64), bva.view(np.uint64))
    # (b) numeric passes
    t0 = time.perf_counter()
    table = b.autotune(reps=5, cache_path=os.path.join(ROOT, "finite_element_method_gb300", "lib",
                                                       "batch_autotune.json"))
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        b.assemble()
    batch_ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            b.assemble_async()
            e1.record(stream)
            e1.synchronize()
            batch_ms.append(e0.elapsed_time(e1))
    b.assemble()  # checks the patterns
    plain_ms = []
    for _ in range(args.warmup):
        for g in models:
            g.assemble_numeric_async()
        torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for g in models:
            g.assemble_numeric_async()
        torch.cuda.synchronize()
        plain_ms.append((time.perf_counter() - t0) * 1e3)
    t0 = time.perf_counter()
    for g in models:
        g.assemble()
    plain_sync_ms = (time.perf_counter() - t0) * 1e3
    for g in models:
        g.close()
    t_b, t_p = float(np.median(batch_ms)), float(np.median(plain_ms))
    tp_e2e, tb_e2e = float(np.median(t_plain)), float(np.median(t_batch))
    line = {"metric": "elements/s assembled to FP64 CSR (batched)", "value": n_el / (t_b * 1e-3),
            "unit": "elements/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_b,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"batch of {len(structures)} structures, log-uniform sizes in [1e3, 2e5], "
                       f"{n_el:,} elements (truss {counts[0]:,}, beam {counts[1]:,}, plate {counts[2]:,})",
                       "l2": "flushed (256 MB write) between steps", "autotune_s": tune_s},
            "batch": {"from_arrays": {"plain_sequences_s": tp_e2e, "batch_s": tb_e2e,
                                      "speedup": tp_e2e / tb_e2e,
                                      "layout_s": layout_s,
                                      "batch_phase_end_ms": {k: float(v) for k, v in zip(
                                          ("nodes", "trusses", "beams", "plates", "checks_read",
                                           "symbolic_and_numeric", "per_structure_csr", "graph_captured"),
                                          phases)},
                                      "what": "host arrays in, every structure's CSR assembled on the device: "
                                              "FEM + add_nodes + add_* + assemble per structure, against "
                                              "fem_gpu_batch_create_from_arrays on the same arrays laid out "
                                              "structure after structure (the layout, layout_s, built before "
                                              "the timing; median of %d)" % reps},
                      "numeric": {"batched_ms": t_b, "plain_async_ms": t_p, "plain_sync_ms": plain_sync_ms,
                                  "speedup_vs_plain_async": t_p / t_b, "speedup_vs_plain_sync": plain_sync_ms / t_b},
                      "autotune_best": table["best"], "autotune_best_ms": table["best_ms"],
                      "autotune_candidates": len(table["candidates"])},
            "gpu_launches": args.steps * ((1 if table["best"]["persistent"] else sum(1 for c in counts if c)) + 2),
            "clocks": clocks.summary()}
    b.close()
    return line


def run_adjoint(args):
    """vector-Jacobian product on the 51 x 51 x 11 frame + 500 x 500 slab model for 64 (u, lambda) pairs
    ~ N(0, 1), against the forward numeric assembly of the same model."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mesh = meshes.adjoint_model(frame=(21, 21, 5), slab=(200, 200)) if args.small else meshes.adjoint_model()
    n_el = mesh.n_elements
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    rng = np.random.default_rng(64)
    n = 6 * mesh.nodes_number
    U = rng.normal(size=(args.pairs, n))
    L = rng.normal(size=(args.pairs, n))
    for _ in range(args.warmup):
        g.vjp(U, L)
    vjp_ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            grads = g.vjp(U, L)
            vjp_ms.append(g.vjp_last_ms())
    fwd_ms = []
    for _ in range(args.warmup):
        g.assemble_numeric_async()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        g.assemble_numeric_async()
        a, b = g.last_numeric_timing()
        fwd_ms.append(a + b)
    g.check_pattern()
    t_v, t_f = float(np.median(vjp_ms)), float(np.median(fwd_ms))
    n_params = 5 * len(mesh.beams["numbers"]) + 2 * len(mesh.plates["numbers"]) + 3 * mesh.nodes_number
    line = {"metric": "adjoint vjp elements/s (64 (u, lambda) pairs)", "value": n_el / (t_v * 1e-3),
            "unit": "elements/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{'x'.join(map(str, mesh.meta['frame']))} beam frame "
                       f"({len(mesh.beams['numbers']):,} beams) + {'x'.join(map(str, mesh.meta['slab']))} plate "
                       f"slab ({len(mesh.plates['numbers']):,} plates), {args.pairs} (u, lambda) pairs ~ N(0, 1), "
                       f"{n_params:,} parameters (E, A, I11, I22, It per beam; E, t per plate; node xyz)"},
            "adjoint": {"vjp_ms": t_v, "forward_numeric_ms": t_f, "vjp_over_forward": t_v / t_f,
                        "vjp_per_pair_over_forward": t_v / args.pairs / t_f,
                        "accuracy": "tests/test_gpu_vjp.py: central differences (step 1e-6 relative) on 200 "
                                    "parameters of this model and a 50-digit reference derivative"},
            "clocks": clocks.summary()}
    g.close()
    return line


def run_separate(args):
    """Sparse separation of the 1000 x 1000 plate stiffness (118 M entries) with the four edges restrained:
    separate_stiffness_matrix_sparse_iterative on the GPU against its numpy restatement on the host."""
    import torch

    from oracle.separate import separate_sparse

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mesh = meshes.plate_mesh(args.nx, args.nx)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    x, y = mesh.xyz[:, 0], mesh.xyz[:, 1]
    edge = np.flatnonzero((x == 0.0) | (y == 0.0) | (x == x.max()) | (y == y.max()))
    imp = np.zeros(6 * mesh.nodes_number, np.uint8)
    for d in range(6):
        imp[6 * edge + d] = 1
    nnz = g.csr_sizes()[1]
    for _ in range(args.warmup):
        g._check(g._L.fem_gpu_separate_sparse(g._h, ptr_u8(imp)))
    ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g._check(g._L.fem_gpu_separate_sparse(g._h, ptr_u8(imp)))
            ms.append((time.perf_counter() - t0) * 1e3)
    t = float(np.median(ms))
    rp, ci, va = g.stiffness_csr()
    t0 = time.perf_counter()
    separate_sparse(rp, ci, va, imp, g.index_node_numbers())
    t_cpu = time.perf_counter() - t0
    # bytes: CSR read twice (count, fill: 12 B per entry + row pointers), blocks written (12 B per entry)
    n_rows = 6 * mesh.nodes_number
    traffic = 2 * (nnz * 12 + n_rows * 8) + nnz * 12
    line = {"metric": "stiffness entries separated/s (K_aa, K_ab, K_ba, K_bb)", "value": nnz / (t * 1e-3),
            "unit": "entries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plate_mesh_{args.nx}x{args.nx} stiffness, {nnz:,} entries, "
                                   f"{len(edge):,} edge nodes restrained in all 6 DOFs",
                       "timing": "host wall time of the call (its three host synchronisations included)"},
            "roofline": {"bound": "hbm", "achieved": traffic / (t * 1e-3) / 1e9, "peak": measured_peaks()[0],
                         "unit": "GB/s", "frac": traffic / (t * 1e-3) / 1e9 / measured_peaks()[0],
                         "traffic": None},
            "cpu_baseline": {"value": nnz / t_cpu, "unit": "entries/s", "cores": 1, "kind": "port",
                             "sample": "the same stiffness, numpy restatement, one run"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_loads(args):
    """A uniformly distributed surface load on every plate of the 1000 x 1000 mesh (1 M loads, 4 M nodal
    contributions): the GPU conversion and call-ordered summation into the forces vector, against the
    CPU restatement on a 100,000-plate sample."""
    import torch

    from oracle.loads import forces_vector

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mesh = meshes.plate_mesh(args.nx, args.nx)
    n = len(mesh.plates["numbers"])
    dofs = np.full(n, 2, np.uint8)
    q = np.random.default_rng(7).uniform(-2e3, -1e3, n)
    ms = []
    with ClockSampler(0) as clocks:
        for it in range(args.warmup + args.steps):
            g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
            meshes.load(g, mesh)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g.add_uniformly_distributed_surface_loads(mesh.plates["numbers"], dofs, q)
            f = g.forces_vector()
            if it >= args.warmup:
                ms.append((time.perf_counter() - t0) * 1e3)
            g.close()
    t = float(np.median(ms))
    k = min(n, 100000)
    pn = mesh.plates["nodes"].astype(np.int64) - 1
    t0 = time.perf_counter()
    forces_vector(mesh.nodes_number, mesh.xyz, [("surface", i, 2, q[i]) for i in range(k)], plate_nodes=pn)
    t_cpu = time.perf_counter() - t0
    line = {"metric": "surface loads converted and summed into the forces vector per second", "value": n / (t * 1e-3),
            "unit": "loads/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plate_mesh_{args.nx}x{args.nx}: one surface load (Z) per plate, {n:,} loads",
                       "timing": "host wall time of the bulk call and the forces read-back (6 M doubles)"},
            "cpu_baseline": {"value": k / t_cpu, "unit": "loads/s", "cores": 1, "kind": "port",
                             "sample": f"the first {k:,} loads, Python loop over the C element restatement"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_pcg(args):
    """PCG (node-block Jacobi) on the separated 1000 x 1000 plate stiffness, all four edges restrained and a
    surface load on every plate: a fixed number of iterations, timed per iteration."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mesh = meshes.plate_mesh(args.nx, args.nx)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    g.add_uniformly_distributed_surface_loads(mesh.plates["numbers"], np.full(len(mesh.plates["numbers"]), 2, np.uint8),
                                              -1e3)
    x, y = mesh.xyz[:, 0], mesh.xyz[:, 1]
    edge = np.flatnonzero((x == 0.0) | (y == 0.0) | (x == x.max()) | (y == y.max()))
    imp = np.zeros(6 * mesh.nodes_number, np.uint8)
    for d in range(6):
        imp[6 * edge + d] = 1
    sep = g.separate_stiffness_matrix_sparse_iterative(imp)
    r_a = g.compose_r_a_vector(sep.k_aa_indexes)
    iters = args.pcg_iters
    ms = []
    for it in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            g.find_ua_vector_iterative_pcg_block_jacobi_sparse(sep, r_a, None, iters)
        except Exception as e:  # a fixed iteration count: the no-convergence status is expected
            assert "no convergence" in str(e), e
        if it >= args.warmup:
            ms.append((time.perf_counter() - t0) * 1e3)
    t = float(np.median(ms)) / iters
    nnz = int(sep.blocks["k_aa"][0][-1])
    n = sep.n_aa
    # bytes one iteration must move: K_aa (values + columns + row starts), the product's p gather, q write and
    # the p . q read (24 B per row), the update (p, q, x, r read, x, r written: 48), the block preconditioner
    # (a 6-double inverse row + block index per DOF, r read, z written: 68) and the direction (z, p read, p
    # written: 24)
    traffic = nnz * 12 + (n + 1) * 8 + n * (24 + 48 + 68 + 24)
    gbs = traffic / (t * 1e-3) / 1e9
    line = {"metric": "PCG iterations/s (block Jacobi, K_aa of the plate mesh)", "value": 1e3 / t, "unit": "iterations/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plate_mesh_{args.nx}x{args.nx}, edges restrained: K_aa {n:,} DOFs, "
                                   f"{nnz:,} entries; {iters} iterations per call",
                       "timing": "host wall time of the call / iterations (set-up of the preconditioner and of the "
                                 "sliced K_aa copy included; the state is read once per batch of iterations)"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": measured_peaks()[0], "unit": "GB/s",
                         "frac": gbs / measured_peaks()[0], "traffic": None,
                         "algorithmic": f"{traffic / 1e9:.2f} GB per iteration (K_aa product, vector sweeps, "
                                        "block preconditioner)"}}
    print(json.dumps(line), flush=True)


# Algorithmic FP64 work per plate of the element-results kernel (k_plate_results, flat mesh: R = I), counted
# from its formulation (FMA = 2 flops, add / mul / div / sqrt = 1): normal 15, local coordinates 39, local
# fields 100, edge vectors, lengths, differences and tying values 72, corner determinants 12 and their shared
# reciprocal 12, edge weights 24, strain sums 58, shear sums 18, material constants 19, results 18.
RESULTS_FLOPS_PER_PLATE = 15 + 39 + 100 + 72 + 12 + 12 + 24 + 58 + 18 + 19 + 18
# bytes per plate the kernel must move: connectivity 16 + properties 32 + results 64, and per node (about one
# per plate in the 1000 x 1000 mesh) coordinates 24 + displacements 48
RESULTS_BYTES = dict(per_plate=16 + 32 + 64, per_node=24 + 48)


def run_results(args):
    """Element results (membrane forces, bending moments, shear forces) of every plate of the 1000 x 1000 mesh
    from a displacements vector: device-resident kernel time (`value`), the host API end to end (`e2e`), and
    the CPU restatement on all host threads."""
    import torch

    from oracle import fem_oracle as fo

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    mesh = meshes.plate_mesh(args.nx, args.nx)
    n_pl, n_nd = len(mesh.plates["numbers"]), mesh.nodes_number
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, n_nd)
    meshes.load(g, mesh)
    disp = np.random.default_rng(17).standard_normal(6 * n_nd) * 1e-3
    d_disp = torch.from_numpy(disp).cuda()
    d_out = torch.empty((n_pl, 8), dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # larger than the 129 MB L2
    ms = []
    with ClockSampler(dev) as clocks:
        for it in range(args.warmup + args.steps):
            flush.fill_(it & 0xFF)
            torch.cuda.synchronize()
            g.element_results_device(d_disp.data_ptr(), 0, 0, d_out.data_ptr())
            torch.cuda.synchronize()
            if it >= args.warmup:
                ms.append(g.results_last_ms())
    t = float(np.mean(ms))
    # end to end through the host API: pinned displacements in, pinned results out
    h_disp = torch.empty(6 * n_nd, dtype=torch.float64, pin_memory=True).numpy()
    h_disp[:] = disp
    h_out = {"truss": torch.empty((0, 1), dtype=torch.float64, pin_memory=True).numpy(),
             "beam": torch.empty((0, 10), dtype=torch.float64, pin_memory=True).numpy(),
             "plate": torch.empty((n_pl, 8), dtype=torch.float64, pin_memory=True).numpy()}
    e2e_ms = []
    for it in range(max(args.warmup, 3) + args.steps):
        flush.fill_(it & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.element_results(h_disp, out=h_out)
        if it >= max(args.warmup, 3):
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    t_e2e = float(np.median(e2e_ms))
    ok = bool(np.array_equal(h_out["plate"], d_out.cpu().numpy()))
    line = {"metric": "plate element results per second", "value": n_pl / (t * 1e-3), "unit": "elements/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"plate_mesh_{args.nx}x{args.nx}: {n_pl:,} plates, {n_nd:,} nodes, random "
                                   "displacements (N(0, 1e-3), seed 17)",
                       "timing": "CUDA events around the result kernel on the model's stream; L2 flushed (256 MB "
                                 "write) before every step", "host_and_device_agree": ok},
            "e2e": {"value": n_pl / (t_e2e * 1e-3), "unit": "elements/s", "ms_per_step": t_e2e,
                    "h2d_bytes_per_step": 8 * 6 * n_nd, "d2h_bytes_per_step": 8 * 8 * n_pl,
                    "api": "FEM.element_results (fem_gpu_element_results), pinned host buffers"},
            "gpu_launches": args.steps}
    fl = RESULTS_FLOPS_PER_PLATE * n_pl / (t * 1e-3)
    by = (RESULTS_BYTES["per_plate"] * n_pl + RESULTS_BYTES["per_node"] * n_nd) / (t * 1e-3) / 1e9
    hbm = measured_peaks()[0]
    line["roofline"] = {"bound": "fp64", "achieved": fl / 1e12, "peak": FP64_PEAK_FLOPS / 1e12, "unit": "TFLOP/s",
                        "frac": fl / FP64_PEAK_FLOPS, "traffic": None,
                        "algorithmic": f"{RESULTS_FLOPS_PER_PLATE} flops per plate (FMA = 2); "
                                       f"{by:.0f} GB/s of algorithmic bytes = {by / hbm:.3f} of measured HBM",
                        "peak_source": "2 DFMA/clk/SM x 152 SMs x 2070 MHz"}
    line["clocks"] = clocks.summary()
    # the beams of the 101 x 101 x 21 frame too (device-resident, same timing)
    frame = meshes.beam_frame()
    n_bm = len(frame.beams["numbers"])
    gb = FEM(meshes.REL_TOL, meshes.ABS_TOL, frame.nodes_number)
    meshes.load(gb, frame)
    bdisp = torch.from_numpy(np.random.default_rng(18).standard_normal(6 * frame.nodes_number) * 1e-3).cuda()
    bout = torch.empty((n_bm, 10), dtype=torch.float64, device="cuda")
    bms = []
    for it in range(args.warmup + args.steps):
        flush.fill_(it & 0xFF)
        torch.cuda.synchronize()
        gb.element_results_device(bdisp.data_ptr(), 0, bout.data_ptr(), 0)
        torch.cuda.synchronize()
        if it >= args.warmup:
            bms.append(gb.results_last_ms())
    tb = float(np.mean(bms))
    line["beam"] = {"workload": f"beam_frame_101x101x21: {n_bm:,} beams", "ms": tb, "value": n_bm / (tb * 1e-3),
                    "unit": "elements/s"}
    gb.close()
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        secs = []
        for _ in range(3):
            out, sec = fo.element_results(mesh, disp, n_threads=threads)
            secs.append(sec)
        line["cpu_baseline"] = {"value": n_pl / min(secs), "unit": "elements/s", "cores": threads, "kind": "port",
                                "sample": f"all {n_pl:,} plates, C restatement (oracle) on {threads} threads, "
                                          "best of 3",
                                "matches_gpu": bool(np.array_equal(out["plate"], h_out["plate"]))}
    print(json.dumps(line), flush=True)
    g.close()


def copy_ceiling(nbytes, reps=5):
    """The link's copy rates on this machine: one cudaMemcpyAsync of `nbytes` between a device buffer and pinned
    host memory each way (CUDA events, best of `reps`), in GB/s -- the ceiling of the e2e read-back."""
    import torch

    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    out = {}
    for name, dst, src in (("d2h_gbs", host, dev), ("h2d_gbs", dev, host)):
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / (best * 1e-3) / 1e9
    out["bytes"] = int(nbytes)
    del dev, host
    return out


def run_numeric(args):
    """The numeric pass of the plate, beam or truss workload (the line's value), its roofline, the CPU
    baseline and the e2e drop-in sequence.  Returns the result line."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)

    mesh, desc = make_mesh(args.workload, args.nx, args.tilt)
    n_el = mesh.n_elements
    fem = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    t0 = time.perf_counter()
    meshes.load(fem, mesh)
    fem.assemble()  # symbolic (pattern, groups, destination map) + first numeric pass
    setup_s = time.perf_counter() - t0
    n_rows, nnz = fem.csr_sizes()

    stream = torch.cuda.ExternalStream(fem.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(args.warmup):
        fem.assemble_numeric_async()
    torch.cuda.synchronize()
    fem.check_pattern()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, elem_ms, red_ms = [], [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            fem.assemble_numeric_async()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            a, b = fem.last_numeric_timing()
            elem_ms.append(a)
            red_ms.append(b)
    torch.cuda.synchronize()
    fem.check_pattern()
    t_step = max_over_ranks(float(np.sum(step_ms)) / args.steps)
    value = n_el * world / (t_step * 1e-3)

    # roofline of the dominant kernel
    hbm_gbs, peak_src = measured_peaks()
    w = WORK[args.workload]
    n_blocks, n_contrib, scratch, sum_slots = fem.pattern_stats()
    # element kernels: inputs + per-contribution offset and mask (16 B) + packed blocks written to scratch
    elem_bytes = n_el * IN_BYTES[args.workload] + n_contrib * 16 + scratch * 8
    # reduction: packed scratch read once; per block-sum slot an 8-byte descriptor read and the sum written
    # and gathered once; the CSR source map (4 B) read and the CSR values (8 B) written once
    red_bytes = scratch * 8 + 3 * sum_slots * 8 + nnz * (4 + 8)
    t_e, t_r = float(np.mean(elem_ms)), float(np.mean(red_ms))
    kern = {"element": dict(ms=t_e, bytes=elem_bytes, flops=element_flops(args.workload, mesh)),
            "reduce": dict(ms=t_r, bytes=red_bytes, flops=scratch)}  # <= one FP64 add per packed entry
    dom = max(kern, key=lambda k: kern[k]["ms"])
    kd = kern[dom]
    gbs = kd["bytes"] / (kd["ms"] * 1e-3) / 1e9
    fl = kd["flops"] / (kd["ms"] * 1e-3)
    frac_hbm, frac_fp64 = gbs / hbm_gbs, fl / FP64_PEAK_FLOPS
    if frac_fp64 > frac_hbm:
        roof = {"bound": "fp64", "achieved": fl / 1e12, "peak": FP64_PEAK_FLOPS / 1e12, "unit": "TFLOP/s",
                "frac": frac_fp64}
    else:
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm_gbs, "unit": "GB/s", "frac": frac_hbm}
    traffic = TRAFFIC_PER_ELEMENT.get(args.workload) if dom == "element" and not args.tilt else None
    roof.update({"kernel": dom, "traffic": None if traffic is None else int(traffic * n_el),
                 "traffic_source": "ncu DRAM bytes of k_plate on the 500 x 500 mesh, scaled per plate"
                 if traffic is not None else None,
                 "peak_source": f"hbm: {peak_src} copy bandwidth; fp64: 2 DFMA/clk/SM x 152 SMs x 2070 MHz",
                 "algorithmic": {k: {"bytes": int(v["bytes"]), "flops": int(v["flops"])} for k, v in kern.items()},
                 "per_kernel_ms": {k: v["ms"] for k, v in kern.items()},
                 "per_kernel_frac": {k: {"hbm": v["bytes"] / (v["ms"] * 1e-3) / 1e9 / hbm_gbs,
                                         "fp64": v["flops"] / (v["ms"] * 1e-3) / FP64_PEAK_FLOPS}
                                     for k, v in kern.items()},
                 "pass_frac": {"hbm": (elem_bytes + red_bytes) / (t_step * 1e-3) / 1e9 / hbm_gbs,
                               "fp64": (kern["element"]["flops"] + kern["reduce"]["flops"]) / (t_step * 1e-3)
                               / FP64_PEAK_FLOPS}})

    # e2e: the drop-in call sequence from pinned host arrays to a pinned host CSR
    def pinned(a):
        """a copy of `a` in page-locked host memory (torch allocates it; numpy views it)."""
        tdt = {1: torch.uint8, 4: torch.int32, 8: torch.int64}[a.dtype.itemsize]
        t = torch.empty(a.shape, dtype=tdt, pin_memory=True)
        out = t.numpy().view(a.dtype)
        out[...] = a
        return out, t

    keep = []
    pn, pt = pinned(mesh.node_numbers)
    px, pxt = pinned(mesh.xyz)
    keep += [pt, pxt]
    pmesh = meshes.Mesh(mesh.name, pn, px)
    for kind in ("trusses", "beams", "plates"):
        d = getattr(mesh, kind)
        if d is not None:
            pd = {}
            for k, v in d.items():
                if v is None:
                    pd[k] = None
                else:
                    arr, t = pinned(np.ascontiguousarray(v))
                    keep.append(t)
                    pd[k] = arr
            setattr(pmesh, kind, pd)
    h2d = pmesh.xyz.nbytes + pmesh.node_numbers.nbytes
    for d in (pmesh.trusses, pmesh.beams, pmesh.plates):
        if d is not None:
            h2d += sum(v.nbytes for k, v in d.items() if v is not None)
    d2h = (n_rows + 1) * 8 + nnz * (4 + 8)
    rp, t_rp = pinned(np.empty(n_rows + 1, np.int64))
    ci, t_ci = pinned(np.empty(nnz, np.int32))
    va, t_va = pinned(np.empty(nnz, np.float64))
    e2e_ms, phases = [], []
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f2 = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
        f2.add_nodes(pmesh.node_numbers, pmesh.xyz)
        t1 = time.perf_counter()
        meshes.load_elements(f2, pmesh)
        t2 = time.perf_counter()
        got = f2.assemble_to_host(rp, ci, va)  # the pattern comes back while the numeric pass runs
        assert got == nnz
        t3 = time.perf_counter()
        e2e_ms.append((t3 - t0) * 1e3)
        phases.append([(t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3])
        f2.close()
    if not e2e_ms:
        e2e_ms, phases = [float("nan")], [[float("nan")] * 3]
    e2e_t = max_over_ranks(float(np.median(e2e_ms)))
    ph = np.median(np.array(phases), axis=0)
    e2e = {"value": n_el * world / (e2e_t * 1e-3), "unit": "elements/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_t,
           "phases_ms": {"add_nodes": ph[0], "add_elements": ph[1], "assemble_to_host": ph[2]},
           "what": "create + add_nodes + add_* + assemble (symbolic + numeric) with the CSR read back to pinned "
                   "host buffers (fem_gpu_assemble_to_host: the pattern's read-back overlaps the numeric pass)"}
    if args.e2e_steps:
        e2e["copy_ceiling"] = copy_ceiling(d2h)

    cpu = None
    if rank == 0 and not args.no_cpu:
        smesh, sdesc = sample_mesh(args.workload)
        v, dt = cpu_oracle_eager(smesh)
        cpu = {"value": v, "unit": "elements/s", "cores": 1, "kind": "port", "sample": sdesc + f", {dt:.1f} s"}

    launches = fem.numeric_launch_count() * args.steps
    line = {"metric": "elements/s assembled to FP64 CSR", "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "nnz": int(nnz), "n_rows": int(n_rows), "l2": "flushed (256 MB write) "
                       "between steps", "parallelism": f"replicas x{world}", "setup_s": setup_s},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks.summary()}
    fem.close()
    return line




def ptr_u8(a):
    import ctypes

    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plate", choices=["plate", "beam", "truss", "batch", "adjoint", "separate", "loads", "pcg",
                                                         "results"])
    ap.add_argument("--pairs", type=int, default=64, help="(u, lambda) pairs of the adjoint workload")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--tilt", action="store_true",
                    help="plate workload: the mesh tilted off the global planes (general rotation path)")
    ap.add_argument("--nx", type=int, default=1000, help="plate mesh size (nx x nx); 1000 is the full workload")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-aux", action="store_true",
                    help="default workload: skip the beam frame, batch and adjoint results appended as aux")
    ap.add_argument("--pcg-iters", type=int, default=200, help="PCG iterations per step of the pcg workload")
    ap.add_argument("--small", action="store_true",
                    help="profiling-sized batch (64 structures) and adjoint (21x21x5 frame + 200x200 slab) cases")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "batch":
        print(json.dumps(run_batch(args)), flush=True)
        return
    if args.workload == "adjoint":
        print(json.dumps(run_adjoint(args)), flush=True)
        return
    if args.workload == "separate":
        run_separate(args)
        return
    if args.workload == "loads":
        run_loads(args)
        return
    if args.workload == "results":
        run_results(args)
        return
    if args.workload == "pcg":
        run_pcg(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    line = run_numeric(args)
    if args.workload == "plate" and not args.no_aux and world == 1 and not args.tilt:
        line["aux"] = aux_results(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def aux_results(args):
    """Compact results of the other configurations, measured in the same run: the beam frame's numeric pass
    (value, roofline), the batch of 512 structures (from host arrays and the numeric pass alone, against
    plain per-structure calls) and the adjoint vjp's cost against the forward pass; each with its clocks."""
    import copy

    out = {}
    a = copy.copy(args)
    a.workload, a.e2e_steps, a.no_cpu, a.small = "beam", 0, True, False
    beam = run_numeric(a)
    out["beam_frame"] = {"workload": beam["config"]["workload"], "value": beam["value"], "unit": beam["unit"],
                         "ms_per_step": beam["ms_per_step"],
                         "roofline": {k: beam["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac",
                                                                       "kernel")},
                         "clocks": beam["clocks"]}
    a = copy.copy(args)
    a.e2e_steps = 5
    batch = run_batch(a)
    out["batch"] = {"workload": batch["config"]["workload"], "value": batch["value"], "unit": batch["unit"],
                    "from_arrays": batch["batch"]["from_arrays"], "numeric": batch["batch"]["numeric"],
                    "clocks": batch["clocks"]}
    adj = run_adjoint(copy.copy(args))
    out["adjoint"] = {"workload": adj["config"]["workload"], "vjp_ms": adj["adjoint"]["vjp_ms"],
                      "forward_numeric_ms": adj["adjoint"]["forward_numeric_ms"],
                      "vjp_over_forward": adj["adjoint"]["vjp_over_forward"],
                      "vjp_per_pair_over_forward": adj["adjoint"]["vjp_per_pair_over_forward"],
                      "clocks": adj["clocks"]}
    return out


if __name__ == "__main__":
    main()
