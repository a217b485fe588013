"""Benchmark of the GB300 finite-element path.

Workload (one "step" = one full linear-elastic solve):
  3D box 1000 x 100 x 100 mm, organised HEXA8 400 x 40 x 40 (640,000 elements,
  674,081 nodes, 2,022,243 DOF, 158,254,569 CSR entries), E = 210000 MPa,
  nu = 0.3, clamped at x = 0, traction -1 MPa in z on the x = 1000 face.
  Step = FP64 element assembly into the CSR values + FP32 copy + Neumann load
  + Dirichlet state + mixed-precision PCG (FP32 SpMV / block-Jacobi / vectors,
  FP64 dots and reliable-update residuals) to relative residual 1e-10.

Prints one JSON line.  ``value`` (solves/s) is measured with inputs resident
in HBM; ``e2e`` goes through the public ``Simulations.Elastic`` API with the
per-step boundary conditions uploaded from pinned host memory and the
displacement read back.  ``--impl reference`` times the CPU oracle (a numpy /
scipy restatement of the reference's path) on a bounded sample of the same
workload.
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

METRIC = "solves/s (HEXA8 2.02M-DOF elastic solve, mixed precision, rel residual 1e-10)"
UNIT = "solves/s"
NX, NY, NZ = 400, 40, 40
L, H, W = 1000.0, 100.0, 100.0
RTOL = 1e-10
# CPU sample: same box aspect, material and boundary conditions
SAMPLE = (80, 8, 8)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, nargs=3, default=None, help="override nx ny nz (testing)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


# --------------------------------------------------------------------------
# CPU oracle sample (reference arm and cpu_baseline)
# --------------------------------------------------------------------------

def cpu_sample(nx, ny, nz):
    """Oracle assembly + SuperLU solve of a small box with the same aspect; returns (seconds, dof)."""
    import numpy as np

    from easyfea_gb300 import mesh as gmesh
    from oracle.simulate import OracleMesh, elastic_solve

    m = gmesh.Mesh_Hexa8_Box(L, H, W, nx, ny, nz)
    om = OracleMesh.from_mesh(m)
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    right = m.Nodes_Conditions(lambda x, y, z: x == L)
    t0 = time.perf_counter()
    u, K, b = elastic_solve(om, 210000.0, 0.3, False, 1.0, [(left, [0.0, 0.0, 0.0], ["x", "y", "z"])],
                            [(right, [-1.0], ["z"])])
    dt = time.perf_counter() - t0
    assert np.isfinite(u).all()
    return dt, u.size


def cpu_threads():
    try:
        from threadpoolctl import threadpool_info

        return max([i.get("num_threads", 1) for i in threadpool_info()] + [1])
    except Exception:
        return 1


def dof_of(nx, ny, nz):
    return 3 * (nx + 1) * (ny + 1) * (nz + 1)


def cpu_baseline_value(steps=1):
    times = []
    for _ in range(steps):
        dt, dof = cpu_sample(*SAMPLE)
        times.append(dt)
    t = statistics.median(times)
    # linear extrapolation of DOF/s to the full workload (favours the CPU:
    # a direct solve's cost grows faster than linearly with the DOF count)
    value = (dof / t) / dof_of(NX, NY, NZ)
    return value, t, dof


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_sample(*SAMPLE)
    times = []
    for _ in range(args.steps):
        dt, dof = cpu_sample(*SAMPLE)
        times.append(dt)
    total = sum(times)
    value = (dof * args.steps / total) / dof_of(NX, NY, NZ)
    sample = (f"oracle (numpy/scipy restatement of EasyFEA's path: einsum element matrices, bincount "
              f"assembly, SuperLU spsolve) on HEXA8 {SAMPLE[0]}x{SAMPLE[1]}x{SAMPLE[2]} box ({dof} DOF, same "
              f"aspect/material/BCs), {total / args.steps:.2f} s per solve; value = DOF/s / 2,022,243 DOF "
              f"(linear extrapolation, favours the CPU)")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 / value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"hexa8_box_{NX}x{NY}x{NZ}_elastic_solve", "dof": dof_of(NX, NY, NZ)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# clocks sampler
# --------------------------------------------------------------------------

class Clocks:
    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[3 + i]
                          and "Not" not in s[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------

def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    from easyfea_gb300 import Models, _lib
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300 import simulations as Simulations

    nx, ny, nz = args.size or (NX, NY, NZ)
    m = gmesh.Mesh_Hexa8_Box(L, H, W, nx, ny, nz)
    mat = Models.Elastic.Isotropic(3, E=210000.0, v=0.3, planeStress=False)
    simu = Simulations.Elastic(m, mat)
    simu.precision = "mixed"
    simu.rtol = RTOL
    left = m.Nodes_Conditions(lambda x, y, z: x == 0)
    right = m.Nodes_Conditions(lambda x, y, z: x == L)
    t0 = time.perf_counter()
    dm = simu.dmesh  # node graph + slot ranks: once per mesh
    torch.cuda.synchronize()
    t_graph = time.perf_counter() - t0
    simu.add_dirichlet(left, [0.0, 0.0, 0.0], ["x", "y", "z"])
    simu.add_surfLoad(right, [-1.0], ["z"])
    lib = _lib.load()
    N = 3 * m.Nn

    def step():
        simu.Need_Update()  # re-assemble every step
        return simu.Solve_device()

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    lib.gfea_profile_enable(1)
    import ctypes

    _ms, _n = ctypes.c_double(), ctypes.c_longlong()
    lib.gfea_profile_read(ctypes.byref(_ms), ctypes.byref(_n))  # reset
    launches0 = lib.gfea_launch_count()
    iters = []
    with Clocks(local) as clk:
        evs[0].record(st)
        for k in range(args.steps):
            step()
            iters.append(simu.last_solve.iterations)
            evs[k + 1].record(st)
        torch.cuda.synchronize()
    launches = lib.gfea_launch_count() - launches0
    lib.gfea_profile_read(ctypes.byref(_ms), ctypes.byref(_n))
    lib.gfea_profile_enable(0)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    info = simu.last_solve
    u = simu.u_device

    # dominant kernel: PCG direction + SpMV (FP32 values, node-block CSR)
    nnz = dm.nnz(3)
    spmv_bytes = nnz * 4 + dm.n_pairs * 4 + (m.Nn + 1) * 4 + N * 4 * 4 + N
    avg_ms = _ms.value / max(_n.value, 1)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    achieved = spmv_bytes / (avg_ms * 1e-3) / 1e9 if _n.value else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tr = json.load(open(tpath)).get("dir_spmv_f32_hexa8_400x40x40")
        traffic = tr if tr else None

    # e2e through the public API: boundary conditions up, displacement down
    pinned_known = torch.zeros(N, dtype=torch.uint8).pin_memory()
    e2e_ms = []
    h2d = d2h = 0
    for k in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        simu.Bc_Init()
        simu.add_dirichlet(left, [0.0, 0.0, 0.0], ["x", "y", "z"])
        simu.add_surfLoad(right, [-1.0], ["z"])
        simu.Need_Update()
        u_host = simu.Solve()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        h2d = N * 1 + N * 8 + m.Nn * 1 + right.size * 8 + left.size * 0
        d2h = N * 8
    del pinned_known

    value = world * args.steps / (total_ms / 1e3)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {
            "workload": f"hexa8_box_{nx}x{ny}x{nz}_elastic_solve",
            "dof": N, "elements": m.Ne, "csr_nnz": nnz, "rtol": RTOL,
            "precision": "FP64 assembly; FP32 SpMV/block-Jacobi/vectors; FP64 dots, scalars, reliable-update residuals",
            "pcg_iterations": iters, "final_rel_residual": info.rel_residual,
            "reliable_updates": info.refinements,
            "graph_setup_s": t_graph,
            "l2": "inputs larger than L2 (FP32 CSR values 0.63 GB, FP64 1.27 GB per step)",
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "dof_per_s": value * N,
        "gpu_launches": int(launches),
        "roofline": {
            "kernel": "dir_spmv_kernel<3,32,float> (PCG direction update + masked SpMV)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": traffic,
            "bytes_per_launch": spmv_bytes,
            "avg_launch_ms": avg_ms,
            "launches": int(_n.value),
            "peak_source": peak_src,
        },
        "e2e": {"value": 1000.0 / statistics.median(e2e_ms), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, t, dof = cpu_baseline_value(2)
        line["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": cpu_threads(), "kind": "port",
            "sample": f"oracle on HEXA8 {SAMPLE[0]}x{SAMPLE[1]}x{SAMPLE[2]} box ({dof} DOF), {t:.2f} s per solve, "
                      f"DOF/s linearly extrapolated to 2,022,243 DOF",
        }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    assert u is not None and np.isfinite(u_host).all()


if __name__ == "__main__":
    main()
