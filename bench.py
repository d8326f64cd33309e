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

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
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
    d = {"workload": f"FV1 defect+Jacobian assembly, {N_CELLS}^3 hexahedra (274625 nodes, b=4), "
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


def cpu_baseline_run(roid, X, C, U, nthreads, steps=1):
    """The oracle (scalar C++ restatement of the reference path) on the host cores."""
    import oracle

    o = oracle.Oracle(3)
    o.set_kinematic_viscosity(NU)
    o.set_upwind(UPWIND)
    o.set_stabilization(STAB)
    o.set_mesh(roid, X, C)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.assemble(U, defect=True, jacobian=True, nthreads=nthreads)
    dt = (time.perf_counter() - t0) / steps
    return C.shape[0] / dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    roid, X, C, U = workload()
    nthreads = os.cpu_count() or 1
    cpu_baseline_run(roid, X, C, U, nthreads, steps=1)  # warm (page-in)
    vals = []
    for _ in range(max(args.warmup, 0)):
        cpu_baseline_run(roid, X, C, U, nthreads, steps=1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline_run(roid, X, C, U, nthreads, steps=1))
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
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
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

    def step(J):
        d.assemble_defect(tu, D, stream=stream)
        d.assemble_jacobian(tu, J, stream=stream)

    ev = lambda: torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step(J64)
            step(J32)
    torch.cuda.synchronize()

    def timed(J, k):
        """per-step device times (ms) of defect, jacobian, total; L2 flushed before each step"""
        tdef, tjac = [], []
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0, e1, e2 = ev(), ev(), ev()
                e0.record(stream)
                d.assemble_defect(tu, D, stream=stream)
                e1.record(stream)
                d.assemble_jacobian(tu, J, stream=stream)
                e2.record(stream)
            e2.synchronize()
            tdef.append(e0.elapsed_time(e1))
            tjac.append(e1.elapsed_time(e2))
        return tdef, tjac

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        tdef64, tjac64 = timed(J64, args.steps)
        tdef32, tjac32 = timed(J32, args.steps)
    torch.cuda.synchronize()
    ms64 = (sum(tdef64) + sum(tjac64)) / args.steps
    ms32 = (sum(tdef32) + sum(tjac32)) / args.steps
    if world > 1:
        t = torch.tensor([ms64, ms32], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms64, ms32 = t.tolist()
    value = world * n_el / (ms64 * 1e-3)

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
            d.assemble_defect(du, D, stream=stream)
            d.assemble_jacobian(du, J64, stream=stream)
            hD.copy_(D, non_blocking=True)
            hJ.copy_(J64, non_blocking=True)
            e1.record(stream)
            e1.synchronize()
            if it > 0:
                e2e_times.append(e0.elapsed_time(e1))
    e2e_ms = sum(e2e_times) / len(e2e_times)
    h2d = hu.numel() * 8
    d2h = (hD.numel() + hJ.numel()) * 8

    # roofline of the dominant kernel (the FP64 Jacobian assembly): algorithmic bytes =
    # Jacobian values written once + u, coordinates, connectivity, block map read once
    jac_ms = sum(tjac64) / args.steps
    alg_bytes = nnzb * b * b * 8 + tu.numel() * 8 + X.size * 8 + C.size * 4 + n_el * 64 * 4
    achieved = alg_bytes / (jac_ms * 1e-3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get("jacobian_f64_bytes_per_assembly")
    except OSError:
        pass

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v = cpu_baseline_run(roid, X, C, U, nthreads, steps=1)
        cpu = {"value": v, "unit": "elems/s", "cores": nthreads, "kind": "port",
               "sample": f"full {N_CELLS}^3 mesh, one defect + Jacobian assembly (oracle, OpenMP over colours)"}

    if rank == 0:
        line = {
            "metric": "assembly elems/s", "value": value, "unit": "elems/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded solenoidal state)",
            "config": config_dict({"defect_ms": sum(tdef64) / args.steps, "jacobian_ms": jac_ms,
                                   "fp32_jacobian_mode": {"value": world * n_el / (ms32 * 1e-3), "ms_per_step": ms32,
                                                          "defect_ms": sum(tdef32) / args.steps,
                                                          "jacobian_ms": sum(tjac32) / args.steps}}),
            "e2e": {"value": world * n_el / (e2e_ms * 1e-3), "unit": "elems/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "kernel": "FP64 Jacobian assembly (8 colour launches)", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "algorithmic_bytes": alg_bytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "gpu_launches": 16 * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
