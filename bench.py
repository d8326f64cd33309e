"""Benchmark: FV1 assembly throughput on the 64^3 hexahedral workload.

Workload (the 3D assembly configuration): 64^3 hexahedra on the unit cube
(274,625 nodes, 4 unknowns per node), kinematic viscosity 0.0025, linear-
profile-skewed upwind + FLOW stabilisation, seeded solenoidal state (curl of a
random vector potential, seed 1) and p ~ U[-1, 1]. One step = one global
defect + one global Jacobian assembly (FP64, plain method). The FP32-Jacobian
mode (FP64 defect + FP32 Jacobian) is measured beside it.

value: elements/s of one defect + Jacobian assembly with inputs resident in
HBM (device-timed with CUDA events, L2 flushed between steps). e2e: the same
through the C ABI with host buffers: H2D of u and D2H of the defect and the
Jacobian values inside the timed region.

Two more workloads print their own line (not the default run):
--workload batched  256 lid-driven cavities, N ~ U{32,...,256}, Re ~ logU[10, 1000],
                    lid ~ U[0.5, 2] (seed 3), full upwind + FLOW; one step = the whole
                    batch solved by the batched Newton (FP32 Jacobian / FP64 defect,
                    multigrid-preconditioned GMRES, one persistent launch per Newton
                    step replayed from a CUDA graph) to ||d|| <= 1e-8 ||d(0)|| per instance.
--workload transient  1024^2 jittered grid split into 2,097,152 triangles (seed 2), backward
                    Euler dt 0.01 x 20 steps, nu 0.001, full upwind + FIELDS, cavity walls; each
                    step one Newton solve to 1e-6 relative (FP32 Jacobian and block inverses,
                    block-Jacobi BiCGStab to 1e-4 with FP64 Krylov vectors, FP64 defect /
                    update / line search); the all-FP64 run beside it.
--workload cavity   the plain method on one 64^2 lid-driven cavity (nu 0.01, zero initial guess,
                    Newton to 1e-8); full upwind with FLOW: with FIELDS the 64^2 cavity enters a
                    period-2 upwind cycle at 9.8e-4 and never reaches 1e-8 (same in the oracle).
--workload learned  the warm-start MLP trained on 2048 solves of 128^2 cavities (seed 4),
                    then 256 held-out draws (seed 5); one step = the held-out batch solved
                    from the network's iterate (FP32 Jacobian), plain FP64 from zero beside.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload assembly|batched|learned]
"""
from __future__ import annotations

import argparse
from collections import Counter
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 64
NU = 0.0025
UPWIND = "lps"
STAB = "flow"


def workload():
    from plugin_navierstokes_gb300 import mesh

    roid, X, C = mesh.structured_hexes(N_CELLS)
    U = mesh.solenoidal_state(X, seed=1)
    return roid, X, C, U


def config_dict(extra=None):
    d = {"workload": f"FV1 defect+Jacobian assembly, {N_CELLS}^3 hexahedra ({(N_CELLS + 1) ** 3} nodes, b=4), "
                     f"LPS upwind + FLOW, nu={NU}, solenoidal seeded state",
         "elements": N_CELLS ** 3, "nodes": (N_CELLS + 1) ** 3, "block_size": 4,
         "upwind": UPWIND, "stabilization": STAB, "l2": "flushed between timed steps (512 MiB write)"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
            "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import statistics

        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def cpu_baseline_run(roid, X, C, U, nthreads):
    """The oracle (scalar C++ restatement of the reference path) on the host cores: one
    defect + Jacobian assembly of the full mesh, timed; returns (elements/s, oracle, D, J)
    so that the same outputs check the GPU's."""
    import oracle

    o = oracle.Oracle(3)
    o.set_kinematic_viscosity(NU)
    o.set_upwind(UPWIND)
    o.set_stabilization(STAB)
    o.set_mesh(roid, X, C)
    t0 = time.perf_counter()
    Dref, Jref = o.assemble(U, defect=True, jacobian=True, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return C.shape[0] / dt, o, Dref, Jref


def measured_peak():
    """(HBM GB/s, source): the measured copy bandwidth of this GPU type, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        return float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def rel_err(a, b):
    """max |a - b| / max |b| over whole arrays (the parity tests' measure), in chunks."""
    import numpy as np

    num, den = 0.0, 0.0
    step = 1 << 24
    for i in range(0, b.size, step):
        x, y = a[i:i + step].astype(np.float64), b[i:i + step]
        num = max(num, float(np.abs(x - y).max()))
        den = max(den, float(np.abs(y).max()))
    return num / den if den > 0 else num


def oracle_check(o, d, Dref, Jref, D, J64, J32):
    """The FP64 oracle's full-size outputs against the GPU's: sparsity pattern and element
    colouring bit-exact, defect and FP64 Jacobian within 1e-12, FP32 Jacobian within 2e-5
    (max |gpu - oracle| / max |oracle| per array)."""
    import numpy as np

    rp, ci = d.pattern()
    orp, oci = o.pattern()
    col = d.coloring()
    ocol, _ = o.coloring()
    out = {"pattern_bit_exact": bool(np.array_equal(rp, orp) and np.array_equal(ci, oci)),
           "coloring_bit_exact": bool(np.array_equal(col, ocol)),
           "oracle_err_defect": rel_err(D, Dref), "oracle_err_jacobian_f64": rel_err(J64, Jref),
           "oracle_err_jacobian_f32": rel_err(J32, Jref), "tolerance_f64": 1e-12, "tolerance_f32": 2e-5}
    out["pass"] = bool(out["pattern_bit_exact"] and out["coloring_bit_exact"] and out["oracle_err_defect"] <= 1e-12
                       and out["oracle_err_jacobian_f64"] <= 1e-12 and out["oracle_err_jacobian_f32"] <= 2e-5)
    return out


def count_launches(fn):
    """Kernel launches of one call of fn, counted by the CUDA profiler interface
    (torch.profiler / CUPTI): {kernel name: launches} of this library's kernels (namespace
    nsfv1), plus the total of all kernels. None if the profiler is unavailable."""
    import torch

    try:
        from torch.profiler import ProfilerActivity, profile

        torch.cuda.synchronize()
        with profile(activities=[ProfilerActivity.CUDA]) as prof:
            fn()
            torch.cuda.synchronize()
        names = {}
        total = 0
        for e in prof.events():
            if getattr(e, "device_type", None) != torch.autograd.DeviceType.CUDA:
                continue
            if "memset" in e.name.lower() or "memcpy" in e.name.lower():
                continue
            total += 1
            if "nsfv1" in e.name:
                key = e.name.split("(")[0].replace("void ", "")
                names[key] = names.get(key, 0) + 1
        return {"ours": sum(names.values()), "all_kernels": total, "by_kernel": names}
    except Exception as ex:  # noqa: BLE001 - the count is evidence, not a requirement of the run
        return {"ours": None, "error": str(ex)[:200]}


def run_reference(args):
    """The oracle's assembly (the reference's CPU path restated) on all host cores: the
    disc and its pattern are set up once, each step times one defect + Jacobian assembly."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle

    roid, X, C, U = workload()
    nthreads = os.cpu_count() or 1
    o = oracle.Oracle(3)
    o.set_kinematic_viscosity(NU)
    o.set_upwind(UPWIND)
    o.set_stabilization(STAB)
    o.set_mesh(roid, X, C)
    for _ in range(max(args.warmup, 1)):
        o.assemble(U, defect=True, jacobian=True, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.assemble(U, defect=True, jacobian=True, nthreads=nthreads)
    elapsed = time.perf_counter() - t0
    value = C.shape[0] * args.steps / elapsed
    line = {"impl": "reference", "metric": "assembly elems/s", "value": value, "unit": "elems/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded solenoidal state)",
            "config": config_dict({"threads": nthreads}),
            "cpu_baseline": {"value": value, "unit": "elems/s", "cores": nthreads, "kind": "port",
                             "sample": f"full {N_CELLS}^3 mesh, one defect + Jacobian assembly per step (OpenMP over element colours)"},
            "e2e": {"value": value, "unit": "elems/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="assembly", choices=["assembly", "batched", "learned", "transient", "cavity"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-launch-count", action="store_true", help="skip the profiler-interface launch count (for runs under ncu)")
    ap.add_argument("--cells", type=int, default=64, help="assembly workload: cells per side (64 is the benchmark; smaller for profiling)")
    ap.add_argument("--time-steps", type=int, default=20, help="transient workload: backward-Euler steps (20 is the benchmark)")
    ap.add_argument("--instances", type=int, default=256, help="batched workload: first K of the 256 draws (256 is the benchmark)")
    ap.add_argument("--warm-start", default="zero", choices=["zero", "learned"],
                    help="batched workload: initial iterate of the main path (learned: the network trained on 2048 solves of 128^2 cavities)")
    args = ap.parse_args()
    global N_CELLS
    N_CELLS = args.cells
    if args.steps is None:
        args.steps = 10 if args.workload == "assembly" else 3
    if args.workload == "transient":
        return run_transient(args)
    if args.workload == "cavity":
        return run_cavity(args)
    if args.workload != "assembly":
        return run_solves(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from plugin_navierstokes_gb300 import NavierStokesFV1, build

    build.build()
    roid, X, C, U = workload()
    n_el = C.shape[0]
    d = NavierStokesFV1("u,v,w,p", "Inner")
    d.set_kinematic_viscosity(NU)
    d.set_upwind(UPWIND)
    d.set_stabilization(STAB)
    d.set_mesh(roid, X, C)
    info = d.pattern_info()
    nnzb = info["nnz_blocks"]
    b = 4
    stream = torch.cuda.Stream(device=dev)
    tu = torch.tensor(U.ravel(), dtype=torch.float64, device=dev)
    D = torch.empty_like(tu)
    J64 = torch.empty(nnzb * b * b, dtype=torch.float64, device=dev)
    J32 = torch.empty(nnzb * b * b, dtype=torch.float32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step64():
        d.assemble_defect_jacobian(tu, D, J64, stream=stream)

    def step32():
        d.assemble_defect_jacobian(tu, D, J32, stream=stream)

    # CTA size of the colour launches from the assembly autotuner
    asm_threads, asm_ms = d.assembly_autotune(tu, "f64", (32, 64, 128), stream=stream)
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step64()
            step32()
    torch.cuda.synchronize()

    def timed(calls, k):
        """per-step device times (ms) of each call in calls; L2 flushed before each step"""
        out = [[] for _ in calls]
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                evs = [ev() for _ in range(len(calls) + 1)]
                evs[0].record(stream)
                for i, c in enumerate(calls):
                    c()
                    evs[i + 1].record(stream)
            evs[-1].synchronize()
            for i in range(len(calls)):
                out[i].append(evs[i].elapsed_time(evs[i + 1]))
        return out

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        (t64,) = timed([step64], args.steps)
        (t32,) = timed([step32], args.steps)
    torch.cuda.synchronize()
    ms64 = sum(t64) / args.steps
    ms32 = sum(t32) / args.steps
    J32f = J32.cpu().numpy()   # the FP32 Jacobian of the defect + Jacobian call, for the oracle check
    # the FP32 Jacobian kernel alone (the Newton loop assembles it at an iterate whose defect is known)
    (tjac32,) = timed([lambda: d.assemble_jacobian(tu, J32, stream=stream)], args.steps)
    if world > 1:
        t = torch.tensor([ms64, ms32], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms64, ms32 = t.tolist()
    value = world * n_el / (ms64 * 1e-3)
    # the separate FP64 defect and Jacobian calls, for comparison with the fused pass
    tdef64, tjac64 = timed([lambda: d.assemble_defect(tu, D, stream=stream),
                            lambda: d.assemble_jacobian(tu, J64, stream=stream)], max(2, args.steps // 2))

    # e2e through the C ABI with host buffers (pinned): u in, defect + Jacobian out
    hu = torch.tensor(U.ravel(), dtype=torch.float64).pin_memory()
    hD = torch.empty(tu.numel(), dtype=torch.float64).pin_memory()
    hJ = torch.empty(nnzb * b * b, dtype=torch.float64).pin_memory()
    du = torch.empty_like(tu)
    e2e_times = []
    with torch.cuda.stream(stream):
        for it in range(max(1, args.steps // 2) + 1):
            flush.fill_(1.0)
            e0, e1 = ev(), ev()
            e0.record(stream)
            du.copy_(hu, non_blocking=True)
            d.assemble_defect_jacobian(du, D, J64, stream=stream)
            hD.copy_(D, non_blocking=True)
            hJ.copy_(J64, non_blocking=True)
            e1.record(stream)
            e1.synchronize()
            if it > 0:
                e2e_times.append(e0.elapsed_time(e1))
    e2e_ms = sum(e2e_times) / len(e2e_times)
    h2d = hu.numel() * 8
    d2h = (hD.numel() + hJ.numel()) * 8

    # the same host-buffer steps back to back: step k's device-to-host copies (a copy stream)
    # overlap step k+1's upload and assembly (two device buffer sets); every step still copies
    # its state in and its defect and Jacobian out
    ov_steps = max(2, args.steps // 2)
    copy_stream = torch.cuda.Stream(device=dev)
    bufs = [(torch.empty_like(tu), torch.empty_like(D), J64), (torch.empty_like(tu), torch.empty_like(D), torch.empty_like(J64))]
    done_asm = [torch.cuda.Event() for _ in bufs]
    done_copy = [torch.cuda.Event() for _ in bufs]
    torch.cuda.synchronize()
    flush.fill_(1.0)
    torch.cuda.synchronize()
    o0, o1 = ev(), ev()
    o0.record(stream)
    for k in range(ov_steps):
        bu, bD, bJ = bufs[k % 2]
        with torch.cuda.stream(stream):
            if k >= 2:
                stream.wait_event(done_copy[k % 2])
            bu.copy_(hu, non_blocking=True)
            d.assemble_defect_jacobian(bu, bD, bJ, stream=stream)
            done_asm[k % 2].record(stream)
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(done_asm[k % 2])
            hD.copy_(bD, non_blocking=True)
            hJ.copy_(bJ, non_blocking=True)
            done_copy[k % 2].record(copy_stream)
    stream.wait_stream(copy_stream)
    o1.record(stream)
    o1.synchronize()
    e2e_ov_ms = o0.elapsed_time(o1) / ov_steps
    del bufs

    # kernel launches of one step of each mode (counted by the profiler interface, after the timed region)
    launches64 = launches32 = {"ours": None, "skipped": True}
    if not args.no_launch_count:
        with torch.cuda.stream(stream):
            count_launches(step64)   # the first profiling session can miss the first launches
            launches64 = count_launches(step64)
            launches32 = count_launches(step32)

    # roofline of the dominant kernel (the fused FP64 defect + Jacobian pass): algorithmic bytes =
    # Jacobian values and defect written once + u, coordinates, connectivity, block map read once
    in_bytes = tu.numel() * 8 + X.size * 8 + C.size * 4 + n_el * 64 * 4
    alg_bytes = nnzb * b * b * 8 + tu.numel() * 8 + in_bytes
    achieved = alg_bytes / (ms64 * 1e-3) / 1e9
    jac32_ms = sum(tjac32) / len(tjac32)
    alg32 = nnzb * b * b * 4 + in_bytes
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    prof = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            prof = json.load(f)
    except OSError:
        pass
    traffic = prof.get("defect_jacobian_f64_bytes_per_assembly")
    # FP64-pipe roofline of the fused pass: FP64 instructions per element (ncu instruction mix,
    # profiles/) x elements over this run's time, against one warp instruction per 16 cycles per SM
    fp64_pipe = None
    if prof.get("fp64_inst_per_element"):
        props = torch.cuda.get_device_properties(dev)
        sm_mhz = 2070.0   # maximum SM clock of GB300 (the clock samples of this run are in "clocks")
        peak_wi = props.multi_processor_count * sm_mhz * 1e6 / 16.0
        ach_wi = prof["fp64_inst_per_element"] * n_el / 32.0 / (ms64 * 1e-3)
        fp64_pipe = {"achieved_warp_inst_per_s": ach_wi, "peak_warp_inst_per_s": peak_wi, "frac": ach_wi / peak_wi,
                     "fp64_inst_per_element": prof["fp64_inst_per_element"], "sm_mhz": sm_mhz,
                     "source": "FP64 instruction count per element from ncu (profiles/k_defect_jacobian_hex_fp64.md)"}
    traffic32 = prof.get("jacobian_f32_bytes_per_assembly")
    # the colour launches of one assembly (the rooflines' figures are per launch)
    n_launch = int(d.pattern_info().get("n_colors", prof.get("launches_per_assembly", 8)))

    cpu, check = None, None
    if rank == 0:
        # the oracle's full-size assembly: the CPU baseline (timed) and the parity check of this run
        nthreads = os.cpu_count() or 1
        v, o, Dref, Jref = cpu_baseline_run(roid, X, C, U, nthreads)
        if world == 1 and not args.no_cpu_baseline:
            cpu = {"value": v, "unit": "elems/s", "cores": nthreads, "kind": "port",
                   "sample": f"full {N_CELLS}^3 mesh, one defect + Jacobian assembly (oracle, OpenMP over colours)"}
        check = oracle_check(o, d, Dref, Jref, hD.numpy(), hJ.numpy(), J32f)
        check["oracle_err_jacobian_f32_kernel"] = rel_err(J32.cpu().numpy(), Jref)
        check["pass"] = bool(check["pass"] and check["oracle_err_jacobian_f32_kernel"] <= 2e-5)
        del o, Dref, Jref

    if rank == 0:
        line = {
            "metric": "assembly elems/s", "value": value, "unit": "elems/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded solenoidal state)",
            "config": config_dict({"step": "one FP64 defect + Jacobian assembly (nsfv1_assemble_defect_jacobian, one pass)",
                                   "separate_calls_ms": {"defect": sum(tdef64) / len(tdef64), "jacobian": sum(tjac64) / len(tjac64)},
                                   "assembly_cta_threads": asm_threads,
                                   "autotune_ms": dict(zip(("32", "64", "128"), [round(x, 3) for x in asm_ms])),
                                   "oracle_check": check,
                                   "fp32_jacobian_mode": {"value": world * n_el / (ms32 * 1e-3), "ms_per_step": ms32,
                                                          "step": "FP64 defect + FP32 Jacobian (nsfv1_assemble_defect_jacobian with FP32 values: per colour the FP64 defect kernel, then the lane-per-corner FP32 Jacobian kernel)",
                                                          "jacobian_only_ms": jac32_ms,
                                                          "roofline": {"bound": "hbm", "kernel": "FP32 Jacobian assembly alone (k_jacobian_lanes, one lane per element corner)",
                                                                       "achieved": alg32 / (jac32_ms * 1e-3) / 1e9, "peak": peak,
                                                                       "unit": "GB/s", "frac": alg32 / (jac32_ms * 1e-3) / 1e9 / peak,
                                                                       "algorithmic_bytes": alg32 / n_launch,
                                                                       "traffic": traffic32 / n_launch if traffic32 else None,
                                                                       "per": f"launch (one colour; {n_launch} per assembly, the time of the assembly / {n_launch})",
                                                                       "traffic_source": prof.get("source_f32")}}}),
            "e2e": {"value": world * n_el / (e2e_ms * 1e-3), "unit": "elems/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                    "overlapped": {"value": world * n_el / (e2e_ov_ms * 1e-3), "ms_per_step": e2e_ov_ms, "steps": ov_steps,
                                   "note": "consecutive host-buffer steps: step k's device-to-host copies overlap step k+1's "
                                           "upload and assembly (copy stream, two device buffer sets)"}},
            "roofline": {"bound": "hbm", "kernel": "fused FP64 defect + Jacobian assembly (one launch per colour)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic / n_launch if traffic else None, "traffic_source": prof.get("source_f64"),
                         "algorithmic_bytes": alg_bytes / n_launch,
                         "per": f"launch (one colour; {n_launch} per assembly, the time of the assembly / {n_launch})",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                         "fp64_pipe": fp64_pipe,
                         "note": "FP64-pipe bound (GB300: 2 FP64 lanes per clock per SM); HBM traffic runs underneath"},
            "cpu_baseline": cpu,
            "gpu_launches": (launches64["ours"] * args.steps) if launches64.get("ours") is not None else None,
            "gpu_launches_per_step": {"f64": launches64, "f32_mode": launches32},
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---- solve workloads (batched cavities, learned warm start) ---------------------

def cavity_draws(n, seed):
    """(Re, lid) draws of the learned workload: Re ~ logU[10, 1000], lid ~ U[0.5, 2]."""
    import numpy as np

    from plugin_navierstokes_gb300 import mesh

    r = mesh.uniform(seed, 2 * n).reshape(n, 2)
    return np.exp(np.log(10.0) + r[:, 0] * (np.log(1000.0) - np.log(10.0))), 0.5 + 1.5 * r[:, 1]


def _oracle_solves(N, Re, lid, budget_s=20.0, nthreads=1):
    """The oracle's Newton (block-Jacobi BiCGStab; OpenMP over element colours with
    nthreads > 1) on cavities of the list, in order, until the time budget is spent:
    (solves/s, solves, seconds)."""
    import numpy as np

    import oracle
    from plugin_navierstokes_gb300 import mesh

    done, t0 = 0, time.perf_counter()
    for n, re, u0 in zip(N, Re, lid):
        roid, X, C = mesh.structured_quads(int(n))
        dofs, vals = mesh.cavity_dirichlet(X, float(u0))
        o = oracle.Oracle(2)
        o.set_kinematic_viscosity(float(u0) / float(re))
        o.set_upwind("full")
        o.set_stabilization("flow")
        o.set_mesh(roid, X, C)
        o.set_dirichlet(dofs, vals)
        o.newton(np.zeros(X.shape[0] * 3), rtol=1e-8, maxit=100, lin_rtol=1e-3, lin_maxit=20000, nthreads=nthreads)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return done / el, done, el


# Newton options of the fast (mixed) path: the reference's exact-Jacobian
# factor 1 (set_exact_jacobian, navier_stokes_base.h:194-196) and Eisenstat-
# Walker linear tolerances up to 0.3; the plain path keeps the reference's
# defaults (factor 0) and a fixed linear tolerance of 1e-3.
FAST_EXACT, FAST_FORCING = 1.0, 0.3


def run_solves(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    from plugin_navierstokes_gb300 import mesh

    if args.workload == "batched":
        N, Re, lid = mesh.draw_cavity_params(256, seed=3)
        N, Re, lid = N[:args.instances], Re[:args.instances], lid[:args.instances]
        wl = "256 lid-driven cavities, N ~ U{32,48,64,96,128,192,256}, Re ~ logU[10,1000], lid ~ U[0.5,2] (seed 3), full upwind + FLOW"
    else:
        Re, lid = cavity_draws(256, 5)
        N = np.full(256, 128)
        wl = "256 held-out lid-driven cavities on 128^2 quads, Re ~ logU[10,1000], lid ~ U[0.5,2] (seed 5), full upwind + FLOW; " \
             "warm start trained on 2048 solves (seed 4)"
    if args.impl == "reference":
        if rank != 0:
            return 0
        # bounded sample: the draws of the batch on 32^2 meshes (the smallest size of the batched workload)
        v, k, el = _oracle_solves(np.full(len(N), 32), np.asarray(Re), np.asarray(lid), budget_s=20.0)
        line = {"impl": "reference", "metric": "solves/s to rel defect 1e-8", "value": v, "unit": "solves/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / k, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": {"workload": wl},
                "cpu_baseline": {"value": v, "unit": "solves/s", "cores": 1, "kind": "port",
                                 "sample": f"first {k} (Re, lid) draws on 32^2 meshes, serial oracle Newton"},
                "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    total_inst = len(N)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        # instance sharding: every rank solves its own cost-balanced share
        from plugin_navierstokes_gb300.sharding import shard_instances

        mine = shard_instances((np.asarray(N) + 1) ** 2, world)[rank]
        N, Re, lid = np.asarray(N)[mine], np.asarray(Re)[mine], np.asarray(lid)[mine]
    from plugin_navierstokes_gb300 import build
    from plugin_navierstokes_gb300.warm_start import CavityBatch, CoordinateMLP, generate_training_set

    build.build()
    extra = {}
    model = None
    learned = args.workload == "learned" or args.warm_start == "learned"
    if learned:
        t0 = time.perf_counter()
        tRe, tlid = cavity_draws(2048, 4)
        coords, targets, cond, tres = generate_training_set(tRe, tlid, N=128, batch=256, cluster_size=16)
        tgen = time.perf_counter() - t0
        # one slot holds a whole instance: the capacity covers the largest mesh of the batch
        model = CoordinateMLP(max_points=max(65536, int((np.max(N) + 1) ** 2)), max_slots=64, seed=4)
        t0 = time.perf_counter()
        hist = model.train(coords, targets, cond, steps=6000, slots=64, points_per_slot=1024, lr=2e-3, lr_final=2e-5, seed=4)
        torch.cuda.synchronize()
        extra["training"] = {"solves": 2048, "converged": int(sum(r["status"] == 0 for r in tres)), "generate_s": round(tgen, 2),
                             "train_steps": 6000, "train_s": round(time.perf_counter() - t0, 2), "final_loss": float(hist[-20:].mean())}
        del coords, targets, cond
    cb_fast = CavityBatch(N, Re, lid, exact_jacobian=FAST_EXACT)
    cb_plain = CavityBatch(N, Re, lid)
    n_inst = cb_fast.n_inst

    def setting(cb, prec, init, forcing):
        tune = cb.autotune(prec, forcing_max=forcing)
        return {"cb": cb, "prec": prec, "init": init, "forcing": forcing, "tune": tune}

    def solve_once(st):
        cb = st["cb"]
        cb.cluster_size, cb.smooth_steps, cb.coarse_steps = st["tune"]["cluster_size"], st["tune"]["smooth_steps"], st["tune"]["coarse_steps"]
        u = cb.zeros()
        if st["init"] == "learned":
            cb.predict(model, u)
        res = cb.solve(u, st["prec"], zero_fallback=st["init"] == "learned", forcing_max=st["forcing"])
        return u, res

    def timed(st, k):
        ts, res = [], None
        for _ in range(k):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            u, res = solve_once(st)
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return ts, res

    stats = lambda r: {"converged": int(sum(x["status"] == 0 for x in r)), "newton_its_mean": float(np.mean([x["iterations"] for x in r])),
                       "newton_its_max": int(max(x["iterations"] for x in r)),
                       "linear_its_mean": float(np.mean([x["linear_iterations"] for x in r]))}
    # learned workload (uniform 128^2): warm start + FP32 Jacobian + exact Jacobian + adaptive
    # tolerances; the uneven batch: FP32 Jacobian with the reference's Newton options, from the warm
    # start with --warm-start learned (the exact-Jacobian variant costs more on its 192^2 and 256^2
    # instances, see the ablations)
    if args.workload == "learned":
        main = setting(cb_fast, "f32", "learned", FAST_FORCING)
    else:
        main = setting(cb_plain, "f32", "learned" if learned else "zero", 0.0)
    if learned and args.workload == "batched":
        wl += "; main path from the warm start of the network trained on 2048 solves of 128^2 cavities (seed 4)"
    for _ in range(args.warmup):
        solve_once(main)
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(local) as clk:
        ts, res = timed(main, args.steps)
    main_stats = main["cb"].disc.batch_stats()   # step work and line-search time of the last timed main solve
    sec = sum(ts) / len(ts)
    if world > 1:
        t = torch.tensor([sec], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        sec = float(t.item())
    value = total_inst / sec
    extra["main"] = dict(stats(res), jacobian="f32", init=main["init"], exact_jacobian=main["cb"].exact_jacobian,
                         forcing_max=main["forcing"], **main["tune"])
    # the plain FP64 method from zero, and ablations, on the same instances (one warm-up and one timed solve each)
    ablations = [("plain_f64", setting(cb_plain, "f64", "zero", 0.0)),
                 ("f64_exact_forcing", setting(cb_fast, "f64", "zero", FAST_FORCING))]
    if not learned:
        ablations += [("f32_exact_forcing", setting(cb_fast, "f32", "zero", FAST_FORCING))]
    else:
        ablations += [("f32_plain_newton", setting(cb_plain, "f32", "zero", 0.0))]
        ablations += [("f32_exact_forcing_zero_init", setting(cb_fast, "f32", "zero", FAST_FORCING))]
        if args.workload == "learned":
            ablations += [("learned_f32_plain_newton", setting(cb_plain, "f32", "learned", 0.0))]
        else:
            ablations += [("learned_f32_exact_forcing", setting(cb_fast, "f32", "learned", FAST_FORCING))]
        ablations += [("learned_f64_exact_forcing", setting(cb_fast, "f64", "learned", FAST_FORCING)),
                      ("learned_f64_plain_newton", setting(cb_plain, "f64", "learned", 0.0))]
    for name, st in ablations:
        solve_once(st)
        t1, r1 = timed(st, 1)
        extra[name] = dict(stats(r1), solves_per_s=n_inst / t1[0], **st["tune"])
    extra["speedup_vs_plain_f64"] = (n_inst / sec) / extra["plain_f64"]["solves_per_s"]
    best64 = max((v["solves_per_s"], k) for k, v in extra.items() if isinstance(v, dict) and k.startswith(("plain_f64", "f64_")))
    extra["speedup_vs_best_f64"] = {"value": (n_inst / sec) / best64[0], "best_f64_path": best64[1]}

    # roofline of the step work (Jacobians on all levels, block inverses, the persistent GMRES) of one
    # timed main solve: algorithmic bytes = per instance, per GMRES iteration, the fine matrix and the
    # V-cycle's level matrices (pre- and post-smoothing sweeps and a residual per level, the level
    # matrices summing to 4/3 of the fine one), 16 basis vectors of Gram-Schmidt and the SpMV vectors;
    # plus per Newton step the Jacobians written once
    vt = 4 if main["prec"] == "f32" else 8
    nb = (np.asarray(N) * 3 + 1) ** 2
    nn = (np.asarray(N) + 1) ** 2
    its = np.array([r["linear_iterations"] for r in res], dtype=np.float64)
    newt = np.array([r["iterations"] for r in res], dtype=np.float64)
    jb = nb * (9 * vt + 4)
    per_it = jb * (1.0 + (2 * main["tune"]["smooth_steps"] + 1) * 4.0 / 3.0) + 18 * nn * 3 * vt
    alg = float(np.sum(its * per_it) + np.sum(newt * jb * 4.0 / 3.0))
    st = main_stats
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    ach = alg / (st["step_work_ms"] * 1e-3) / 1e9 if st["step_work_ms"] > 0 else None
    roofline = {"bound": "hbm", "kernel": "batched Newton step work (level Jacobians, block inverses, persistent GMRES)",
                "achieved": ach, "peak": peak, "unit": "GB/s", "frac": (ach / peak) if ach else None, "traffic": None,
                "algorithmic_bytes": alg, "step_work_ms": st["step_work_ms"], "line_search_ms": st["line_search_ms"],
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                "note": "matrices of small instances stay in L2, so DRAM traffic is below the algorithmic bytes"}

    # FP64-oracle defect of every instance's final iterate (rank 0, one solve of the main path)
    u, res = solve_once(main)
    U = u.cpu().numpy()
    if rank == 0 and not args.no_cpu_baseline:
        import oracle

        worst = 0.0
        offs = main["cb"].node_offsets
        for i in range(n_inst):
            roid, X, C = mesh.structured_quads(int(N[i]))
            dofs, vals = mesh.cavity_dirichlet(X, float(lid[i]))
            o = oracle.Oracle(2)
            o.set_kinematic_viscosity(float(lid[i]) / float(Re[i]))
            o.set_upwind("full")
            o.set_stabilization("flow")
            o.set_mesh(roid, X, C)
            o.set_dirichlet(dofs, vals)
            D, _ = o.assemble(U[offs[i] * 3:offs[i + 1] * 3], jacobian=False, nthreads=os.cpu_count() or 1)
            x0 = np.zeros(X.shape[0] * 3)
            x0[dofs] = vals
            D0, _ = o.assemble(x0, jacobian=False, nthreads=os.cpu_count() or 1)
            worst = max(worst, float(np.linalg.norm(D) / np.linalg.norm(D0)))
        extra["oracle_rel_defect_max"] = worst

    # e2e through the public API with host buffers: H2D of the initial iterate, D2H of the solutions
    cb = main["cb"]
    hu0 = torch.zeros(cb.n_nodes * 3, dtype=torch.float64).pin_memory()
    hu = torch.empty_like(hu0).pin_memory()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ud = hu0.to(dev, non_blocking=True)
    if learned:
        cb.predict(model, ud)
    cb.cluster_size, cb.smooth_steps, cb.coarse_steps = main["tune"]["cluster_size"], main["tune"]["smooth_steps"], main["tune"]["coarse_steps"]
    cb.solve(ud, "f32", zero_fallback=learned, forcing_max=main["forcing"])
    hu.copy_(ud, non_blocking=True)
    e1.record()
    e1.synchronize()
    e2e_s = e0.elapsed_time(e1) * 1e-3

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # bounded sample of the same instances: the batch's own (N, Re, lid) draws, smallest meshes first,
        # until 30 s are spent (the CPU's solves/s is therefore an upper bound for the whole batch)
        nthreads = os.cpu_count() or 1
        order = np.argsort(np.asarray(N), kind="stable")
        v, k, el = _oracle_solves(np.asarray(N)[order], np.asarray(Re)[order], np.asarray(lid)[order], budget_s=30.0, nthreads=nthreads)
        sizes = sorted(Counter(int(x) for x in np.asarray(N)[order][:k]).items())
        cpu = {"value": v, "unit": "solves/s", "cores": nthreads, "kind": "port",
               "sample": f"{k} of the batch's instances, smallest first (sizes {sizes}), oracle Newton with block-Jacobi "
                         f"BiCGStab, OpenMP over colours, {el:.1f} s"}
    if rank == 0:
        line = {"metric": "solves/s to rel defect 1e-8", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * sec, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64 defect / f32 jacobian", "data": "synthetic (seeded cavity draws)",
                "config": {"workload": wl, "instances": total_inst, "l2": "inputs larger than L2 (" + str(cb.n_nodes) + " nodes)",
                           "target": "||d_i|| <= 1e-8 ||d_i(zero iterate)|| per instance", **extra},
                "e2e": {"value": n_inst * world / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": hu0.numel() * 8,
                        "d2h_bytes_per_step": hu.numel() * 8},
                "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": None, "clocks": clk.summary()}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# Newton tolerance of each backward-Euler step: full upwinding makes the defect
# only piecewise smooth, and the Newton iteration stalls at an upwind kink (near
# 2e-7 relative from rest, near 1e-9 absolute later), in FP64 as well, so each
# step stops at 1e-6 relative to its initial defect or at 1e-5 of the first
# step's initial defect, whichever comes first.
RTOL_STEP = 1e-6
ATOL_FRACTION = 1e-5


def _transient_cpu_sample(nu, dt, nthreads):
    """The oracle's first backward-Euler step (Newton + block-Jacobi BiCGStab) on a 128^2 grid
    of the transient workload's construction; returns (seconds, triangles, Newton result)."""
    import numpy as np

    import oracle
    from plugin_navierstokes_gb300 import mesh

    rs, rX, rC = mesh.jittered_triangles(128, seed=2)
    rd, rv = mesh.cavity_dirichlet(rX, 1.0)
    o = oracle.Oracle(2)
    o.set_kinematic_viscosity(nu)
    o.set_upwind("full")
    o.set_stabilization("fields")
    o.set_mesh(rs, rX, rC)
    o.set_dirichlet(rd, rv)
    U0 = np.zeros(rX.shape[0] * 3)
    U0[rd] = rv
    t0 = time.perf_counter()
    _, st = o.newton(U0.copy(), U_old=U0, dt=dt, rtol=1e-8, lin_rtol=1e-4, lin_maxit=20000, nthreads=nthreads)
    return time.perf_counter() - t0, int(rC.shape[0]), st


def run_transient(args):
    import numpy as np
    import torch

    from plugin_navierstokes_gb300 import NavierStokesFV1, build, mesh

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    n_cells, n_steps, dt, nu = args.cells if args.cells != 64 else 1024, args.time_steps, 0.01, 0.001
    wl = (f"{n_cells}^2 jittered grid (+-0.2h, seed 2) split into {2 * n_cells * n_cells} triangles, backward Euler dt={dt} x {n_steps}, "
          f"nu={nu}, full upwind + FIELDS, lid-driven cavity walls")
    roid, X, C = mesh.jittered_triangles(n_cells, seed=2)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)
    nthreads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return 0
        # bounded sample: the first time step on a 128^2 grid of the same construction, scaled by elements
        el, tri, _ = _transient_cpu_sample(nu, dt, nthreads)
        v = (tri / C.shape[0]) / el
        line = {"impl": "reference", "metric": "time steps/s", "value": v, "unit": "steps/s", "n_gpus": args.gpus, "steps": 1,
                "warmup": 0, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": wl},
                "cpu_baseline": {"value": v, "unit": "steps/s", "cores": nthreads, "kind": "port",
                                 "sample": f"first time step on the 128^2 grid of the same construction ({el:.1f} s, oracle Newton, "
                                           f"OpenMP assembly), scaled by elements"},
                "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    build.build()
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(nu)
    d.set_upwind("full")
    d.set_stabilization("fields")
    d.set_mesh(roid, X, C)
    d.set_dirichlet(dofs, vals)
    n = X.shape[0] * 3
    u0 = torch.zeros(n, dtype=torch.float64, device=dev)
    u0[torch.from_numpy(dofs.astype(np.int64)).to(dev)] = torch.from_numpy(vals).to(dev)

    D0 = torch.empty_like(u0)
    d.assemble_defect(u0, D0, u0, dt)
    atol = ATOL_FRACTION * float(D0.norm().item())

    def step(u, prec):
        uo = u.clone()
        return d.newton_solve(u, uo, dt=dt, rtol=RTOL_STEP, atol=atol, lin_rtol=1e-4, lin_max_iter=5000, jacobian_prec=prec,
                              linear_solver="bicgstab")

    def march(prec, k):
        u = u0.clone()
        its, lin, times = [], [], []
        for _ in range(k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = step(u, prec)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
            its.append(r["iterations"])
            lin.append(r["linear_iterations"])
        return u, its, lin, times

    n_warm = min(max(args.warmup, 3), n_steps)
    # the warm-up steps run under the profiler interface: kernel launches per Krylov iteration
    launch = None
    march("f32", n_warm)
    if not args.no_launch_count:
        wres = {}

        def one_step():
            wres["r"] = march("f32", 1)

        count_launches(one_step)   # the first profiling session can miss the first launches
        launch = count_launches(one_step)
        launch["steps"] = 1
        launch["linear_its"] = int(sum(wres["r"][2]))
        launch["newton_its"] = int(sum(wres["r"][1]))
    with ClockSampler(local) as clk:
        u32, its32, lin32, t32 = march("f32", n_steps)
    u64, its64, lin64, t64 = march("f64", n_steps)
    # the mixed run's final state against the all-FP64 run
    rel_diff = float(((u32 - u64).norm() / u64.norm()).item())
    sec = sum(t32)
    value = n_steps / sec
    # e2e: host iterate in, 20 steps, host solution out
    hu = u0.cpu().pin_memory()
    hout = torch.empty_like(hu).pin_memory()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    u = hu.to(dev, non_blocking=True)
    for _ in range(n_steps):
        step(u, "f32")
    hout.copy_(u, non_blocking=True)
    e1.record()
    e1.synchronize()
    e2e = n_steps / (e0.elapsed_time(e1) * 1e-3)

    # full-size parity at the second time step's first Newton iterate (u = u_old = the state after the
    # first step, where the defect is dt A(u), not the cancellation left at a converged iterate): FP64
    # defect, FP64 and FP32 Jacobians, pattern and colouring against the FP64 oracle
    u1 = u0.clone()
    step(u1, "f32")
    u0 = u1.clone()
    info = d.pattern_info()
    nnzb = int(info["nnz_blocks"])
    Dg = torch.empty_like(u1)
    J64 = torch.empty(nnzb * 9, dtype=torch.float64, device=dev)
    J32 = torch.empty(nnzb * 9, dtype=torch.float32, device=dev)
    d.assemble_defect(u1, Dg, u0, dt)
    d.assemble_jacobian(u1, J64, u0, dt)
    d.assemble_jacobian(u1, J32, u0, dt)
    torch.cuda.synchronize()
    check = None
    if not args.no_cpu_baseline:
        import oracle

        o = oracle.Oracle(2)
        o.set_kinematic_viscosity(nu)
        o.set_upwind("full")
        o.set_stabilization("fields")
        o.set_mesh(roid, X, C)
        o.set_dirichlet(dofs, vals)
        Dref, Jref = o.assemble(u1.cpu().numpy(), U_old=u0.cpu().numpy(), dt=dt, nthreads=nthreads)
        check = oracle_check(o, d, Dref, Jref, Dg.cpu().numpy(), J64.cpu().numpy(), J32.cpu().numpy())
        check["state"] = "first Newton iterate of the second time step (u = u_old = the first step's solution)"
        del Jref, o
    del J64
    # the dominant kernel: the FP32-matrix x FP64-vector block SpMV of BiCGStab (x split into
    # float pairs by the update kernel that produces it), timed alone
    x = u1.clone()
    xs = d.split_vector(x)
    y = torch.empty_like(x)
    for _ in range(3):
        d.bsr_mv_split(J32, xs, y)
    torch.cuda.synchronize()
    k_mv = 50
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(k_mv):
        d.bsr_mv_split(J32, xs, y)
    e1.record()
    e1.synchronize()
    mv_s = e0.elapsed_time(e1) * 1e-3 / k_mv
    nrows = X.shape[0]
    mv_bytes = nnzb * (9 * 4 + 4) + (nrows + 1) * 4 + 2 * n * 8
    peak, peak_src = measured_peak()
    prof = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            prof = json.load(f)
    except OSError:
        pass
    mv_traffic = prof.get("spmv_tri1024_f32_bytes") if n_cells == 1024 else None
    roofline = {"bound": "hbm", "kernel": "k_bsr_mv_split<3, 4> (FP32 Jacobian x FP64 vector given as float pairs, the BiCGStab SpMV)",
                "achieved": mv_bytes / mv_s / 1e9, "peak": peak, "unit": "GB/s", "frac": mv_bytes / mv_s / 1e9 / peak,
                "traffic": mv_traffic, "traffic_source": prof.get("source_spmv") if mv_traffic else None,
                "algorithmic_bytes": mv_bytes, "us_per_launch": mv_s * 1e6, "peak_source": peak_src,
                "note": "algorithmic bytes = FP32 blocks + column indices + row pointers + x read (8 B per entry, as a float pair) + y written"}
    cpu = None
    if not args.no_cpu_baseline:
        el, tri, _ = _transient_cpu_sample(nu, dt, nthreads)
        cv = (tri / C.shape[0]) / el
        cpu = {"value": cv, "unit": "steps/s", "cores": nthreads, "kind": "port",
               "sample": f"first time step on the 128^2 grid of the same construction ({el:.1f} s, oracle Newton, OpenMP assembly), "
                         f"scaled by elements"}
    gpu_launches = None
    if launch and launch.get("ours") and launch["linear_its"]:
        # launches scale with the Krylov iterations; the timed march's count from the warm-up's rate
        gpu_launches = int(round(launch["ours"] * sum(lin32) / launch["linear_its"]))
    line = {"metric": "time steps/s", "value": value, "unit": "steps/s", "n_gpus": 1, "steps": n_steps, "warmup": n_warm,
            "ms_per_step": 1e3 * sec / n_steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 defect / f32 jacobian", "data": "synthetic (seeded jittered grid)",
            "config": {"workload": wl, "triangles": int(C.shape[0]), "nodes": int(X.shape[0]),
                       "l2": "inputs larger than L2",
                       "mixed": {"newton_its": its32, "linear_its": lin32, "seconds": sec},
                       "all_f64": {"newton_its": its64, "linear_its": lin64, "seconds": sum(t64), "steps_per_s": n_steps / sum(t64)},
                       "final_state_rel_diff_vs_all_f64": rel_diff, "oracle_check": check},
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": hu.numel() * 8 / n_steps,
                    "d2h_bytes_per_step": hout.numel() * 8 / n_steps},
            "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": gpu_launches,
            "gpu_launches_measured": launch, "clocks": clk.summary()}
    if launch:
        line["gpu_launches_note"] = "the first time step profiled (untimed), scaled to the timed steps by Krylov iterations"
    print(json.dumps(line))
    return 0


def run_cavity(args):
    """The plain method on one 64^2 cavity: single-instance FP64 Newton with block-Jacobi
    BiCGStab (the reference's solver setup restated), and the batched solver on the same
    single instance (multigrid-preconditioned GMRES); the CPU oracle Newton beside it."""
    import numpy as np
    import torch

    from plugin_navierstokes_gb300 import NavierStokesFV1, build, mesh

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    n, nu = 64, 0.01
    wl = f"{n}^2 lid-driven cavity (quads), nu={nu}, lid 1, full upwind + FLOW, zero initial guess, Newton to rel defect 1e-8"
    roid, X, C = mesh.structured_quads(n)
    dofs, vals = mesh.cavity_dirichlet(X, 1.0)

    def oracle_solve():
        import oracle

        o = oracle.Oracle(2)
        o.set_kinematic_viscosity(nu)
        o.set_upwind("full")
        o.set_stabilization("flow")
        o.set_mesh(roid, X, C)
        o.set_dirichlet(dofs, vals)
        t0 = time.perf_counter()
        U, st = o.newton(np.zeros(X.shape[0] * 3), rtol=1e-8, maxit=100, lin_rtol=1e-3, lin_maxit=20000)
        return time.perf_counter() - t0, st

    if args.impl == "reference":
        if rank != 0:
            return 0
        el, st = oracle_solve()
        line = {"impl": "reference", "metric": "solves/s to rel defect 1e-8", "value": 1.0 / el, "unit": "solves/s", "n_gpus": args.gpus,
                "steps": 1, "warmup": 0, "ms_per_step": 1e3 * el, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": {"workload": wl, "newton_its": st["iterations"]},
                "cpu_baseline": {"value": 1.0 / el, "unit": "solves/s", "cores": 1, "kind": "port", "sample": "one full solve, serial oracle"},
                "e2e": {"value": 1.0 / el, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    build.build()
    d = NavierStokesFV1("u,v,p", "Inner")
    d.set_kinematic_viscosity(nu)
    d.set_upwind("full")
    d.set_stabilization("flow")
    d.set_mesh(roid, X, C)
    d.set_dirichlet(dofs, vals)
    nn = X.shape[0] * 3

    def single():
        u = torch.zeros(nn, dtype=torch.float64, device=dev)
        return d.newton_solve(u, rtol=1e-8, lin_rtol=1e-3, lin_max_iter=5000, jacobian_prec="f64", linear_solver="bicgstab")

    def timed(fn, k):
        ts, r = [], None
        for _ in range(k):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return sum(ts) / len(ts), r

    for _ in range(args.warmup):
        single()
    with ClockSampler(local) as clk:
        sec, r = timed(single, args.steps)
    # the batched solver on the single instance (multigrid GMRES, one persistent launch per step)
    from plugin_navierstokes_gb300.warm_start import CavityBatch

    cb = CavityBatch([n], [1.0 / nu], [1.0])
    cb.cluster_size = 16

    def batched(prec):
        u = cb.zeros()
        return cb.solve(u, prec, defect_reference="initial")

    batched("f64")
    sec_b64, rb64 = timed(lambda: batched("f64"), args.steps)
    batched("f32")
    sec_b32, rb32 = timed(lambda: batched("f32"), args.steps)
    # e2e: host zero iterate in, solution out, through the public API
    hu = torch.zeros(nn, dtype=torch.float64).pin_memory()
    ho = torch.empty_like(hu).pin_memory()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    u = hu.to(dev, non_blocking=True)
    ub = cb.zeros()
    ub.copy_(u)
    cb.solve(ub, "f64", defect_reference="initial")
    ho.copy_(ub, non_blocking=True)
    e1.record()
    e1.synchronize()
    e2e = 1.0 / (e0.elapsed_time(e1) * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:
        el, st = oracle_solve()
        cpu = {"value": 1.0 / el, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"one full solve, serial oracle Newton ({st['iterations']} steps, {el:.1f} s)"}
    # value: the plain method (FP64 Jacobian) through the multigrid-preconditioned solver; the
    # block-Jacobi BiCGStab Newton and the FP32-Jacobian variant beside it
    line = {"metric": "solves/s to rel defect 1e-8", "value": 1.0 / sec_b64, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec_b64, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": {"workload": wl, "solver": "Newton + GMRES(30) with the geometric V-cycle",
                                                           "newton_its": rb64[0]["iterations"], "linear_its": rb64[0]["linear_iterations"],
                                                           "bicgstab_block_jacobi_f64": {"solves_per_s": 1.0 / sec, "newton_its": r["iterations"],
                                                                                         "linear_its": r["linear_iterations"]},
                                                           "fp32_jacobian": {"solves_per_s": 1.0 / sec_b32, "newton_its": rb32[0]["iterations"]}},
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": hu.numel() * 8, "d2h_bytes_per_step": ho.numel() * 8},
            "roofline": None, "cpu_baseline": cpu, "gpu_launches": None, "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
