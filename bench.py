#!/usr/bin/env python
"""Benchmark: ms per pressure projection at 256^3 (the c2 workload).

One step = one pressure projection of SIMCOFlow's projection step on the 256^3
cut-cell sphere + gas-bubble column (density ratio 1000): GFM coefficients,
operator and right-hand side, the multigrid-preconditioned CG solve to
relative residual 1e-8, the pressure scatter, the velocity correction and the
boundary conditions.  ``value`` is the device time per projection of the
mixed solver with the inputs resident in HBM: an FP32 V-cycle (FP32 storage
and arithmetic), CG vectors and operator in double-float (FP32 pairs, about
48 significand bits), CG dot products formed from per-cell FP64 products and
summed in FP64, and an FP64 true residual (iterative refinement) and FP64
coarsest-grid solve.  The same projection with the FP64 solver (FP64 V-cycle
and CG) is timed beside it.  ``e2e`` is the drop-in call ``scf_update_puvw``
with the reference's host arrays in page-locked memory (host->device copy of
every input and device->host copy of u, v, w, p and the BC planes inside the
timed region).  After the timed regions the line adds both arms' pressure and
velocity errors against the oracle's FP64 solve to 1e-13, and the other named
configurations: c0 (64^3) and c1 (128^3) in FP64 to 1e-10 with their errors,
the c3 adjoint gradient (128^3) against central differences, and the c4 wave
tank's 20 warm-started calls in both precisions.

``--impl reference`` times the CPU path (the oracle's restatement of the
reference path, multigrid-preconditioned CG with OpenMP on all host cores).

Multi-GPU: the path runs on one GPU per projection (the reference builds the
whole system on every rank), so ``--gpus N`` runs N independent replicas.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "ms/projection & HBM GB/s at 256^3: mixed vs FP64 GPU solve at rel res 1e-8"
FALLBACK_HBM_GBS = 6800.0


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def allreduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return out
        out["samples"] = len(rows)
        out["sm_mhz"] = statistics.median(r[0] for r in rows)
        out["sm_max_mhz"] = max(r[1] for r in rows)
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = set()
        for r in rows:
            for name, val in zip(names, r[2:]):
                if val.lower() == "active":
                    reasons.add(name)
        out["reasons"] = sorted(reasons)
        return out


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            for k in ("hbm_gbs", "hbm_GBs", "copy_gbs"):
                if k in d:
                    return float(d[k]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch at
# 256^3, from ncu captures at 192^3 scaled by the number of cells
# (x 16777216/7077888): the fine-level FP32 Chebyshev step, 213.5 MB for a
# first pre-smoothing step (profiles/k_cheb_step_f32_c2_192.md), and the
# TMA-staged two-step kernel, 184.1 + 43.8 MB for the first pre-smoothing
# pair (profiles/k_cheb_pair_c2_192.md)
SMOOTH_TRAFFIC_256 = {
    "smooth": {"bytes": 213.5e6 * 16777216 / 7077888,
               "note": "first pre-smoothing step (32 B/cell algorithmic), ncu at 192^3 scaled by cells"},
    "smooth2": {"bytes": (184.1e6 + 43.8e6) * 16777216 / 7077888,
                "note": "first pre-smoothing pair (32 B/cell algorithmic for two steps), ncu at 192^3 "
                        "(16 k-planes per block there, 32 at 256^3) scaled by cells"},
}


def smoother_traffic(n_cells: int, kind: str = "smooth"):
    if n_cells != 16777216:
        return None
    return SMOOTH_TRAFFIC_256.get(kind)


def make_workload(name: str, seed: int, n=None):
    from simcoflow3d_gb300 import workloads as W
    return W.config(name, seed=seed, n=n)


def pin_arrays(lib, w):
    """Pins the workload's host arrays in place (cudaHostRegister)."""
    pinned = []
    for a in w.arrays.values():
        if a.nbytes and lib.scf_host_register(a.ctypes.data, a.nbytes) == 0:
            pinned.append(a)
    return pinned


def pinned_like(a):
    """A Fortran-ordered copy of ``a`` (FP64 or int32) in page-locked host
    memory allocated as such (cudaHostAlloc through torch)."""
    import numpy as np
    import torch
    tdt = {np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32}[a.dtype]
    buf = torch.empty(max(a.size, 1), dtype=tdt, pin_memory=True).numpy()[:a.size]
    out = buf.reshape(a.shape, order="F")
    if not (out.flags.f_contiguous and out.ctypes.data == buf.ctypes.data):
        raise RuntimeError("pinned buffer is not Fortran-contiguous")
    out[...] = a
    return out


def pinned_workload(w):
    """A copy of workload ``w`` whose every array lives in page-locked host
    memory allocated once (cudaHostAlloc), the way a caller that keeps its
    fields pinned for the whole run would hold them."""
    import dataclasses
    p = dataclasses.replace(w)
    p.arrays = {k: (pinned_like(v) if v.nbytes else v.copy(order="F")) for k, v in w.arrays.items()}
    p.meta = dict(w.meta)
    return p


def numa_report(arrays, gpu_index: int):
    """Where the host buffers' pages live (/proc/self/numa_maps), the GPU's
    NUMA affinity and the kernel's NUMA balancing switch."""
    out = {"buffer_pages_by_node": {}, "gpu_numa_node": None, "numa_balancing": None, "host_nodes": None}
    try:
        maps = []
        for line in open("/proc/self/numa_maps"):
            f = line.split()
            maps.append((int(f[0], 16), f))
        maps.sort()
        import bisect
        starts = [m[0] for m in maps]
        seen = set()
        for a in arrays:
            i = bisect.bisect_right(starts, a.ctypes.data) - 1
            if i < 0 or i in seen:
                continue
            seen.add(i)
            for tok in maps[i][1]:
                if tok[:1] == "N" and "=" in tok:
                    k, v = tok.split("=")
                    out["buffer_pages_by_node"][k] = out["buffer_pages_by_node"].get(k, 0) + int(v)
    except Exception as e:      # not Linux, or no numa_maps
        out["buffer_pages_by_node"] = f"unavailable: {e}"
    try:
        out["numa_balancing"] = int(open("/proc/sys/kernel/numa_balancing").read())
    except Exception:
        pass
    try:
        out["host_nodes"] = sorted(n for n in os.listdir("/sys/devices/system/node") if n.startswith("node"))
        bus = subprocess.run(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout.strip().lower()
        if bus:
            dom, rest = bus.split(":", 1)
            path = "/sys/bus/pci/devices/%s:%s/numa_node" % (dom[-4:], rest)
            if os.path.exists(path):
                out["gpu_numa_node"] = int(open(path).read())
    except Exception:
        pass
    return out


def unpin(lib, arrs):
    for a in arrs:
        lib.scf_host_unregister(a.ctypes.data)


def time_device(proj, steps, warmup, live_kernel_timing=0):
    """W untimed + K timed device-resident projections; returns (list of ms, stats).
    With live_kernel_timing = n > 0 the fine-level kernels of the last n timed
    projections are bracketed by CUDA events on the context's stream
    (Projection.kernel_timing).  Each bracketed launch costs a few microseconds
    of graph replay, so only a sample of the timed steps carries them."""
    for _ in range(warmup):
        proj.run()
    ms, launches, last = [], 0, None
    for s in range(steps):
        if live_kernel_timing and s == steps - min(live_kernel_timing, steps):
            proj.kernel_timing(True)
        st = proj.run()
        ms.append(st["ms_total"])
        launches += st["gpu_launches"]
        last = st
    return ms, launches, last


def cpu_projection_ms(w, threads: int, tol: float = 1e-8):
    """One projection on the host cores with the oracle's restatement."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O
    t0 = time.perf_counter()
    pc = O.pocoef(w)
    b = O.rhs(w, pc)
    x, st = O.gmg_solve(w, pc, b, precision=0, rel_tol=tol, degree=3)
    pp = O.scatter(w, x)
    O.correct(w, pc, pp)
    return (time.perf_counter() - t0) * 1e3, st


def projection_config(args, w, ws: int) -> dict:
    """The ``config`` of the projection line, the same in both arms."""
    return {
        "workload": f"{args.config}: {w.imax}x{w.jmax}x{w.kmax} cut-cell sphere r=0.15 at (0.5,0.5,0.3) + gas "
                    "bubble r=0.1 at (0.5,0.5,0.65) in a water column, rho ratio 1000, all-Neumann p, "
                    f"rel res {args.tol:g}" if args.config == "c2" else f"{args.config} at {w.imax}x{w.jmax}x{w.kmax}",
        "grid": [w.imax, w.jmax, w.kmax],
        "rel_tol": args.tol,
        "l2": "inputs larger than L2 (about 3.5 GB resident per projection)",
        "parallelism": f"replicas x{ws}",
    }


def oracle_errors(w, ref, pp, uvw):
    """Pressure (the solve's Pp) and corrected-velocity errors of one device
    projection against the oracle's FP64 solve to 1e-13 (relative L2; the
    pressure mean-aligned for all-Neumann systems)."""
    from oracle import oracle as O
    return {"err_p_vs_oracle": float("%.3e" % O.pressure_error(w, pp, ref["pp"], ref["singular"])),
            "err_u_vs_oracle": float("%.3e" % O.velocity_error(uvw, (ref["u"], ref["v"], ref["w"])))}


def fp64_config_leg(name: str, args, device: int):
    """c0 (64^3, no solid) or c1 (128^3, with the sphere): the plain FP64
    projection to relative residual 1e-10, device-resident (W untimed + K
    timed), its errors against the oracle's FP64 solve to 1e-13, and the
    oracle's CPU projection to 1e-10 at the same size on all host cores."""
    import numpy as np
    from simcoflow3d_gb300 import capi
    from simcoflow3d_gb300.projection import Projection
    from oracle import oracle as O
    w = make_workload(name, args.seed, None)
    proj = Projection.for_workload(w, precision=capi.SCF_PREC_FP64, rel_tol=1e-10, device=device)
    proj.stage(w)
    ms, launches, st = time_device(proj, args.steps, args.warmup)
    u, v, ww, _, _, su = proj.update_puvw(w, want_bc=False)
    p = np.zeros(w.shape_g, order="F")      # the solve's pressure Pp
    proj.fetch(pp=p)
    proj.close()
    out = {"grid": [w.imax, w.jmax, w.kmax], "precision": "fp64", "rel_tol": 1e-10,
           "ms_per_projection": round(statistics.mean(ms), 4), "iterations": st["iterations"],
           "rel_residual": st["rel_residual"], "gpu_launches": launches}
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    ref = O.project(w, rel_tol=1e-13)
    out.update(oracle_errors(w, ref, p, (u, v, ww)))
    del ref
    cpu_ms, cpu_st = cpu_projection_ms(w, threads, tol=1e-10)
    out["cpu_oracle"] = {"ms_per_projection": round(cpu_ms, 2), "cores": threads,
                         "iterations": cpu_st["iterations"], "kind": "port"}
    return out


def adjoint_leg(args, device: int, directions: int = 32, eps: float = 1e-6):
    """c3 (128^3, the c1 geometry, FP64): the loss J = sum over cut cells of
    p n_z WlLh + 1/2 ||D u||^2 and its adjoint gradient with respect to u*
    and the cell densities.  Times the forward (projection to 1e-12 + loss)
    and the backward (one adjoint solve to 1e-10 + gradient kernels) as the
    library's host calls, W untimed + K timed; then checks the gradient on
    `directions` seeded random directions each for (u*, v*, w*) and for rho
    against central finite differences with step eps.  The error is
    relative to the directional derivatives over the set of directions."""
    import numpy as np
    from simcoflow3d_gb300 import workloads as W
    from simcoflow3d_gb300.autograd import ProjectionLoss
    from oracle import adjoint as AD
    w = make_workload("c3", args.seed, None)
    g = W.pressure_force_weights(w)
    rho = AD.phase_density(w)
    R = ProjectionLoss(w, g=g, device=device)
    a = w.arrays
    us, vs, ws = a["u_star"], a["v_star"], a["w_star"]
    fwd, bwd = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        J, _, sf = R.forward(us, vs, ws, rho)
        t1 = time.perf_counter()
        (gu, gv, gw, grho), sb = R.backward()
        t2 = time.perf_counter()
        if i >= args.warmup:
            fwd.append((t1 - t0) * 1e3)
            bwd.append((t2 - t1) * 1e3)
    rng = np.random.default_rng(args.seed)
    fd_u, an_u, fd_r, an_r = [], [], [], []
    for _ in range(directions):
        d = [np.asfortranarray(rng.normal(size=w.shape_g)) for _ in range(3)]
        jp = R.forward(us + eps * d[0], vs + eps * d[1], ws + eps * d[2], rho)[0]
        jm = R.forward(us - eps * d[0], vs - eps * d[1], ws - eps * d[2], rho)[0]
        fd_u.append((jp - jm) / (2 * eps))
        an_u.append(float(np.sum(gu * d[0]) + np.sum(gv * d[1]) + np.sum(gw * d[2])))
    for _ in range(directions):
        dr = np.asfortranarray(rng.normal(size=w.shape_g) * rho)
        jp = R.forward(us, vs, ws, rho + eps * dr)[0]
        jm = R.forward(us, vs, ws, rho - eps * dr)[0]
        fd_r.append((jp - jm) / (2 * eps))
        an_r.append(float(np.sum(grho * dr)))
    R.proj.close()
    err = lambda fd, an: float("%.3e" % (np.linalg.norm(np.array(fd) - np.array(an)) / np.linalg.norm(an)))
    return {"grid": [w.imax, w.jmax, w.kmax], "precision": "fp64",
            "ms_forward": round(statistics.mean(fwd), 3), "ms_backward": round(statistics.mean(bwd), 3),
            "forward_iterations": sf["iterations"], "adjoint_iterations": sb["iterations"],
            "fd_directions": directions, "fd_eps": eps,
            "grad_rel_err_u_star": err(fd_u, an_u), "grad_rel_err_rho": err(fd_r, an_r),
            "timing": "host calls (inputs copied in, gradients copied out), W untimed + K timed"}


def run_reference(args):
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    if rank != 0:
        barrier(dist)
        return 0
    if args.config == "clsvof":
        n = args.n or 256
        ms = []
        for i in range(args.warmup + args.steps):
            t, _ = clsvof_cpu_ms(n)
            if i >= args.warmup:
                ms.append(t)
            if args.max_cpu_s and sum(ms) / 1e3 * 64 ** 3 / n ** 3 > args.max_cpu_s and len(ms) >= 1:
                break
        v = statistics.mean(ms)
        line = {
            "impl": "reference", "metric": "ms per Clsvof_Scheme step at %d^3 (6 sub-steps x 3 split sweeps, wall "
                                           "planes, reconstruction, redistancing)" % n,
            "value": round(v, 3), "unit": "ms/step", "n_gpus": ws, "steps": len(ms), "warmup": args.warmup,
            "ms_per_step": round(v, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic: the 3-D deformation test of the reference's AdvectionTest at t = 0",
            "config": {"workload": "CLSVOF transport: liquid sphere r=0.15 at (0.35,0.35,0.35) in the %d^3 unit "
                                   "cube, LeVeque deformation field, CFL 0.15" % n, "grid": [n, n, n]},
            "cpu_baseline": {"value": round(v, 3), "unit": "ms/step", "cores": 1, "kind": "port",
                             "sample": "each step one oracle Clsvof_Scheme step at 64^3 (the reference test's own "
                                       "grid), scaled by the cell count to %d^3" % n},
            "e2e": {"value": round(v, 3), "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        barrier(dist)
        return 0
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    # warm-up steps (untimed) run the same path on a 32^3 grid of the same
    # configuration: the CPU port has nothing to warm but its threads and
    # caches, and the K timed full-size steps alone take minutes
    wsmall = make_workload(args.config, args.seed, 32)
    for _ in range(args.warmup):
        cpu_projection_ms(wsmall, threads, tol=args.tol)
    w = make_workload(args.config, args.seed, args.n)
    ms = []
    for i in range(args.steps):
        t, st = cpu_projection_ms(w, threads, tol=args.tol)
        ms.append(t)
        if args.max_cpu_s and sum(ms) / 1e3 > args.max_cpu_s and len(ms) < args.steps:
            break
    v = statistics.mean(ms)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "ms/projection",
        "n_gpus": ws, "steps": len(ms), "warmup": args.warmup, "ms_per_step": round(v, 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded u*, cut-cell sphere + gas bubble)",
        "config": projection_config(args, w, ws),
        "cpu_baseline": {"value": round(v, 3), "unit": "ms/projection", "cores": threads, "kind": "port",
                         "sample": "full projection per step (oracle restatement: coefficients, rhs, "
                                   "FP64 MG-PCG to %g, scatter, correction); warm-ups on a 32^3 grid" % args.tol},
        "e2e": {"value": round(v, 3), "unit": "ms/projection", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "iterations": st.get("iterations"),
        "steps_requested": args.steps,
        "max_cpu_s": args.max_cpu_s,
        "capped": len(ms) < args.steps,
    }
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def run_ours(args):
    import numpy as np
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    from simcoflow3d_gb300 import capi
    from simcoflow3d_gb300.projection import Projection, load_library
    lib = load_library()
    w = make_workload(args.config, args.seed + rank, args.n)
    pinned = pin_arrays(lib, w)

    # device-resident timing: mixed (value) and FP64 (comparison)
    results = {}
    precs = (("mixed", capi.SCF_PREC_MIXED), ("fp64", capi.SCF_PREC_FP64))
    # Each arm runs at its fastest Chebyshev degree on this workload (sweep of
    # degrees 2-5 at 256^3): 4 for the FP32 V-cycle (8 CG iterations), 2 for
    # the FP64 one (12).
    degree = {"mixed": 4, "fp64": 2}
    if args.only:
        # profiling captures: one precision, device-resident loop only
        name, prec = [x for x in precs if x[0] == args.only][0]
        proj = Projection.for_workload(w, precision=prec, rel_tol=args.tol, device=local,
                                       smoother_degree=degree[name])
        proj.stage(w)
        ms, launches, st = time_device(proj, args.steps, args.warmup)
        print(json.dumps({"only": name, "ms_per_projection": statistics.mean(ms), "stats": st}), flush=True)
        unpin(lib, pinned)
        return 0
    for name, prec in precs:
        proj = Projection.for_workload(w, precision=prec, rel_tol=args.tol, device=local,
                                       smoother_degree=degree[name])
        proj.stage(w)
        barrier(dist)
        if name == "mixed":
            with ClockSampler(local) as cs:
                ms, launches, st = time_device(proj, args.steps, args.warmup,
                                               live_kernel_timing=max(1, args.steps // 5))
            clocks = cs.summary()
        else:
            ms, launches, st = time_device(proj, args.steps, args.warmup)
        total = allreduce_max(dist, sum(ms))
        results[name] = {"ms": ms, "total": total, "launches": launches, "stats": st, "proj": proj}

    # dominant-kernel roofline on the mixed context (fine-level smoother),
    # from the launches of the timed projections themselves
    mixed = results["mixed"]["proj"]
    live = {}
    classes = {"smooth": capi.SCF_K_SMOOTH, "smooth2": capi.SCF_K_SMOOTH2, "spmv": capi.SCF_K_SPMV,
               "restrict": capi.SCF_K_RESTRICT, "prolong": capi.SCF_K_PROLONG, "cg_update": capi.SCF_K_CGUPDATE}
    for name, kc in classes.items():
        tot, nl, by = mixed.kernel_timing_read(kc)
        live[name] = {"launches": nl, "ms_per_launch": round(tot / max(nl, 1), 5), "ms_total": round(tot, 4),
                      "GB/s": round(by * nl / (tot * 1e-3) / 1e9, 1) if tot > 0 else None,
                      "bytes_per_launch": by}
    mixed.kernel_timing(False)
    # the roofline's kernel: the fine-level smoother class with the most device time
    kind = "smooth2" if live["smooth2"]["ms_total"] > live["smooth"]["ms_total"] else "smooth"
    k_nl, k_bytes = live[kind]["launches"], live[kind]["bytes_per_launch"]
    k_ms = live[kind]["ms_per_launch"]
    iso_ms, _ = mixed.time_kernel(classes[kind], reps=50)
    peak, peak_kind = measured_peaks()
    achieved = k_bytes / (k_ms * 1e-3) / 1e9
    trf = smoother_traffic(w.imax * w.jmax * w.kmax, kind)
    k_name = {"smooth": "k_cheb_step<float> (fine-level Chebyshev step)",
              "smooth2": "k_cheb_pair (two fused fine-level Chebyshev steps)"}[kind]

    # the FP64 arm's fields of one drop-in call and its pressure Pp, for its
    # errors against the oracle (computed after every timed region)
    u64, v64, w64, _, _, _ = results["fp64"]["proj"].update_puvw(w, want_bc=False)
    p64 = np.zeros(w.shape_g, order="F")
    results["fp64"]["proj"].fetch(pp=p64)
    results["fp64"]["proj"].close()     # only the mixed context stays on the device
    # end to end through the drop-in call: every input and output array in
    # page-locked host memory allocated once, outside the timed region
    unpin(lib, pinned)
    pinned = []
    wh = pinned_workload(w)
    a = wh.arrays
    tv_keys = ("tvar_u", "tvar_v", "tvar_w", "tvar_p")
    tv = [pinned_like(a[k]) for k in tv_keys]
    in_bytes = sum(x.nbytes for x in a.values())
    numa = numa_report(list(a.values()) + tv, local)
    bc_struct, bc = capi.new_bc_out(w.imax, w.jmax, w.kmax)
    bc = [[pinned_like(x) for x in row] for row in bc]
    e2e_ms, lib_ms, h2d_ms, d2h_ms = [], [], [], []
    e2e_stats = None
    gc.collect()
    gc.disable()   # no collector pauses inside the timed host calls (as timeit does)
    for i in range(args.warmup + args.steps):
        for t, k in zip(tv, tv_keys):
            t[...] = a[k]
        barrier(dist) if i == args.warmup else None
        t0 = time.perf_counter()
        u, v, ww, p, _, st = mixed.update_puvw(wh, tvar=tv, want_bc=True, bc_out=bc)
        dt = (time.perf_counter() - t0) * 1e3
        if i >= args.warmup:
            e2e_ms.append(dt)
            lib_ms.append(st["ms_total"])
            h2d_ms.append(st["ms_h2d"])
            d2h_ms.append(st["ms_d2h"])
            e2e_stats = st
    gc.enable()
    e2e_total = allreduce_max(dist, sum(e2e_ms))
    mixed_out = [x.copy(order="F") for x in (u, v, ww)] + [np.zeros(w.shape_g, order="F")]
    mixed.fetch(pp=mixed_out[3])
    mixed.close()
    del wh, tv, bc

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu_ms, cpu_st = cpu_projection_ms(w, threads)
        cpu = {"value": round(cpu_ms, 3), "unit": "ms/projection", "cores": threads, "kind": "port",
               "sample": "one full 256^3 projection (oracle restatement: coefficients, rhs, FP64 MG-PCG to "
                         f"1e-8 in {cpu_st['iterations']} iterations, scatter, correction), OpenMP"}

    # errors of both arms against the oracle's FP64 solve to 1e-13, and the
    # other named configurations (c0, c1 in FP64; the c3 adjoint; the c4
    # warm-started sequence in both precisions): all after the timed regions
    errors, configs = {}, {}
    if rank == 0 and ws == 1 and not args.no_oracle:
        from oracle import oracle as O
        os.environ["OMP_NUM_THREADS"] = str(os.cpu_count() or 1)
        ref = O.project(w, rel_tol=1e-13)
        errors["mixed"] = oracle_errors(w, ref, mixed_out[3], mixed_out[:3])
        errors["fp64"] = oracle_errors(w, ref, p64, (u64, v64, w64))
        errors["oracle"] = {"rel_tol": 1e-13, "iterations": ref["stats"]["iterations"],
                            "residual_in_reference_matrix": ref["stats"]["csr_relres"]}
        del ref
    del mixed_out, u64, v64, w64, p64
    if rank == 0 and ws == 1 and not args.no_configs and args.config == "c2" and args.n is None:
        for name in ("c0", "c1"):
            configs[name] = fp64_config_leg(name, args, local)
        configs["c3_adjoint"] = adjoint_leg(args, local)
        w4 = make_workload("c4", args.seed, None)
        configs["c4_sequence"] = {"grid": [w4.imax, w4.jmax, w4.kmax], "rel_tol": args.tol,
                                  "arms": sequence_arms(w4, 20, args.tol, args.seed, device=local)}
        del w4

    if rank != 0:
        barrier(dist)
        return 0
    nproj = ws * args.steps
    value = results["mixed"]["total"] / nproj
    fp64 = results["fp64"]["total"] / nproj
    smx, s64 = results["mixed"]["stats"], results["fp64"]["stats"]
    line = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "ms/projection",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(value, 4),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 V-cycle, double-float CG vectors, f64 CG dots / true residual / coarsest solve",
        "data": "synthetic (seeded u*, cut-cell sphere + gas bubble)",
        "config": projection_config(args, w, ws),
        "fp64": {"ms_per_projection": round(fp64, 4), "iterations": s64["iterations"],
                 "smoother_degree": degree["fp64"],
                 "rel_residual": s64["rel_residual"], **errors.get("fp64", {})},
        "mixed": {"iterations": smx["iterations"], "rel_residual": smx["rel_residual"],
                  **errors.get("mixed", {}),
                  "smoother_degree": degree["mixed"],
                  "ms_steps": [round(x, 3) for x in results["mixed"]["ms"]],
                  "ms_assemble": round(smx["ms_assemble"], 3), "ms_solve": round(smx["ms_solve"], 3),
                  "ms_correct": round(smx["ms_correct"], 3)},
        "speedup_mixed_vs_fp64": round(fp64 / value, 3),
        "e2e": {"value": round(e2e_total / nproj, 4), "unit": "ms/projection",
                "h2d_bytes_per_step": int(e2e_stats["bytes_h2d"]),
                "d2h_bytes_per_step": int(e2e_stats["bytes_d2h"]),
                "ms_h2d": round(e2e_stats["ms_h2d"], 3), "ms_d2h": round(e2e_stats["ms_d2h"], 3),
                "ms_min": round(min(e2e_ms), 3), "ms_median": round(statistics.median(e2e_ms), 3),
                "ms_max": round(max(e2e_ms), 3), "ms_steps": [round(x, 2) for x in e2e_ms],
                "ms_steps_in_library": [round(x, 2) for x in lib_ms],
                "ms_h2d_steps": [round(x, 2) for x in h2d_ms],
                "ms_d2h_steps": [round(x, 2) for x in d2h_ms],
                "h2d_GBps_median": round(e2e_stats["bytes_h2d"] / (statistics.median(h2d_ms) * 1e-3) / 1e9, 1),
                "spread": round((max(e2e_ms) - min(e2e_ms)) / statistics.median(e2e_ms), 3),
                "host_memory": "every input and output in page-locked memory allocated once (cudaHostAlloc), "
                               "%.2f GB of inputs" % (in_bytes / 1e9),
                "numa": numa},
        "roofline": {"bound": "hbm", "kernel": k_name,
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_launch": k_bytes, "ms_per_launch": k_ms, "launches_timed": k_nl,
                     "timing": "CUDA events around each fine-level launch of the last %d timed projections"
                               % max(1, args.steps // 5),
                     "ms_per_launch_isolated": round(iso_ms, 5),
                     "traffic": round(trf["bytes"]) if trf else None,
                     "traffic_note": trf["note"] if trf else None,
                     # a pair launch does the work of two one-step launches
                     "one_step_equivalent_gbs": round(2 * achieved, 1) if kind == "smooth2" else None},
        "kernels_live": live,
        "oracle_solve": errors.get("oracle"),
        "configs": configs or None,
        "clocks": clocks,
        "gpu_launches": results["mixed"]["launches"],
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def sequence_arms(w, calls: int, tol: float, seed: int, device: int = 0):
    """A sequence of warm-started projections on a fixed geometry: each call
    gets a freshly seeded prediction, staged outside the timed region, and
    starts from the previous call's pressure (call 0 cold).  Both precisions,
    each at its fastest Chebyshev degree on the z-stretched wave tank (sweep
    3-8): 8 for the FP32 line-block V-cycle, 6 for the FP64 one.  The first
    pass over the calls warms the context up; the second is timed."""
    from simcoflow3d_gb300 import capi, workloads as W
    from simcoflow3d_gb300.projection import Projection
    preds = W.PredictionSequence(w, seed=seed + 1)
    degree = {"mixed": 8, "fp64": 6}
    out = []
    for name, prec in (("mixed", capi.SCF_PREC_MIXED), ("fp64", capi.SCF_PREC_FP64)):
        proj = Projection.for_workload(w, precision=prec, rel_tol=tol, smoother_degree=degree[name], device=device)
        for timed in (False, True):
            ms, its, res = [], [], []
            for c in range(calls):
                proj.set_opts(warm_start=0 if c == 0 else 1)
                proj.stage(w, pred=preds(c))
                st = proj.run()
                ms.append(st["ms_total"])
                its.append(st["iterations"])
                res.append(st["rel_residual"])
        out.append({"precision": name, "smoother_degree": degree[name], "calls": len(ms),
                    "ms_per_call": round(statistics.mean(ms), 3), "ms_min": round(min(ms), 3),
                    "ms_max": round(max(ms), 3), "iterations": its, "max_rel_residual": max(res)})
        proj.close()
    return out


def run_sequence(args):
    """The warm-started sequence (default: the 512x256x256 wave tank); one
    JSON line per precision."""
    w = make_workload(args.config, args.seed, args.n)
    for arm in sequence_arms(w, args.sequence, args.tol, args.seed):
        arm.update({"sequence": args.config, "grid": [w.imax, w.jmax, w.kmax], "rel_tol": args.tol,
                    "bcp_flag": list(w.bcp_flag)})
        print(json.dumps(arm), flush=True)
    return 0


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# k_geo_faces on the PCell family, from the ncu capture summarised in
# profiles/k_geo_faces_geometry_c2_128.md at 128^3, scaled to 256^3 by cells.
GEO_FACES_TRAFFIC_128 = 132.545e6 + 222.457e6


def run_geometry(args):
    """The cut-cell geometry preprocessing (GridPreprocess +
    DefineMomentumExchangeCell + NumberExternalCell x4) on the P/U/V/W cells of
    the c2 geometry: device-resident time, the host-array call end to end,
    the face kernel's live roofline and the oracle on the host cores.  One
    JSON line."""
    import numpy as np
    from simcoflow3d_gb300 import geometry as GM
    from simcoflow3d_gb300.projection import load_library
    n = args.n or 256
    g = GM.geometry_inputs("c2", n=n, seed=args.seed)
    lib = load_library()
    gp = GM.GridPreprocess(g.imax, g.jmax, g.kmax)
    gp.stage(g)
    for _ in range(args.warmup):
        gp.run()
    with ClockSampler(0) as cs:
        runs = [gp.run() for _ in range(args.steps)]
    clocks = cs.summary()
    ms = [r["ms_device"] for r in runs]
    ms_faces = [r["ms_faces"] / 4 for r in runs]
    by_faces = runs[-1]["bytes_faces"] / 4
    # end to end through scf_grid_preprocess with page-locked host arrays
    pinned = []
    for fam in g.fams.values():
        for a in fam.arrays.values():
            if a is not None and a.nbytes and lib.scf_host_register(a.ctypes.data, a.nbytes) == 0:
                pinned.append(a)
    e2e = [gp(g) for _ in range(max(3, args.steps // 4))]
    unpin(lib, pinned)
    peak, peak_kind = measured_peaks()
    achieved = by_faces / (statistics.mean(ms_faces) * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        os.environ["OMP_NUM_THREADS"] = str(threads)
        from oracle import oracle as O
        t0 = time.perf_counter()
        O.grid_preprocess(g)
        cpu = {"value": round((time.perf_counter() - t0) * 1e3, 1), "unit": "ms/call", "cores": threads,
               "kind": "port", "sample": "one full call at %d^3 (oracle restatement of the four families' "
                                        "GridPreprocess, DefineMomentumExchangeCell, NumberExternalCell), OpenMP" % n}
    cells = g.imax * g.jmax * g.kmax
    trf = None
    if GEO_FACES_TRAFFIC_128 is not None:
        trf = GEO_FACES_TRAFFIC_128 * cells / 128 ** 3
    line = {
        "metric": "ms per cut-cell geometry preprocessing call at %d^3 (GridPreprocess + "
                  "DefineMomentumExchangeCell + NumberExternalCell x4, P/U/V/W cells)" % n,
        "value": round(statistics.mean(ms), 4), "unit": "ms/call", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(ms), 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (solid sphere level set, normals and fluid fractions of each family on its own "
                "staggered grid; in/out arrays seeded)",
        "config": {"workload": "geometry of c2: %d^3 unit cube, solid sphere r=0.15 at (0.5,0.5,0.3), "
                               "liquid bubble r=0.1 at (0.5,0.5,0.65)" % n,
                   "grid": [g.imax, g.jmax, g.kmax],
                   "l2": "inputs larger than L2 (%.1f GB on the device)" % (e2e[-1]["bytes_h2d"] / 1e9)},
        "exact_faces": runs[-1]["exact_faces"],
        "e2e": {"value": round(statistics.mean(r["ms_total"] for r in e2e), 3), "unit": "ms/call",
                "h2d_bytes_per_step": int(e2e[-1]["bytes_h2d"]), "d2h_bytes_per_step": int(e2e[-1]["bytes_d2h"]),
                "ms_h2d": round(statistics.mean(r["ms_h2d"] for r in e2e), 3),
                "ms_d2h": round(statistics.mean(r["ms_d2h"] for r in e2e), 3),
                "inputs_pinned_fraction": round(sum(a.nbytes for a in pinned) /
                                                max(1, sum(a.nbytes for f in g.fams.values()
                                                           for a in f.arrays.values() if a is not None)), 4)},
        "roofline": {"bound": "hbm", "kernel": "k_geo_faces (CellGeoCal faces of one family)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "bytes_per_launch": by_faces,
                     "ms_per_launch": round(statistics.mean(ms_faces), 5), "launches_timed": 4 * args.steps,
                     "timing": "CUDA events around each face-kernel launch of the timed calls",
                     "traffic": round(trf) if trf else None},
        "clocks": clocks,
        "gpu_launches": sum(r["gpu_launches"] for r in runs),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


# Algorithmic bytes per cell of one BiCGStab iteration's passes in FP32
# (s = 4): U reads r, p, v, writes p (4 s); P reads p, r0 and the six
# couplings, writes v (9 s); S reads r, v and the couplings, writes t (9 s);
# X reads x, r, r0, p, v, t, writes x, r (8 s).
BCG_BYTES_F32 = {"U": 16, "P": 36, "S": 36, "X": 32}


def run_predictor(args):
    """The implicit solves of the momentum predictor (SetMatrix + SetVectors
    + solve + DeltaGetValues for u, v, w, then the tail of PredictingUVW) on
    the c2 geometry at 256^3 with dam-break viscosity (Rey = 300): device
    time with the inputs resident (FP32 BiCGStab inside FP64 refinement, and
    FP64 BiCGStab), the host-array call end to end, the live roofline of the
    largest BiCGStab kernel, and the oracle on the host cores.  One JSON line."""
    import numpy as np
    from simcoflow3d_gb300 import capi, geometry as GM, predictor as PR
    from simcoflow3d_gb300.projection import load_library
    geo = args.pred_geometry
    n = args.n or 256
    g = GM.geometry_inputs(geo, n=n, seed=args.seed)
    GM.GridPreprocess(g.imax, g.jmax, g.kmax)(g)
    inp = PR.momentum_inputs(g, seed=args.seed)
    lib = load_library()
    ps = PR.PredictSolves(g.imax, g.jmax, g.kmax)
    ps.stage(inp)
    tol = 1e-10   # the reference's PCG tolerance (PredictUVW.f90:830)
    opts = PR.default_opts(precision=capi.SCF_PREC_MIXED, rel_tol=tol)
    for _ in range(args.warmup):
        ps.run(opts)
    with ClockSampler(0) as cs:
        runs = [ps.run(opts) for _ in range(args.steps)]
    clocks = cs.summary()
    topts = PR.default_opts(precision=capi.SCF_PREC_MIXED, rel_tol=tol)
    topts.kernel_timing = 1
    timed = [ps.run(topts) for _ in range(2)]
    o64 = PR.default_opts(precision=capi.SCF_PREC_FP64, rel_tol=tol)
    runs64 = [ps.run(o64) for _ in range(3)]
    # end to end through scf_predict_solves with page-locked host arrays
    pred, dpo = PR.new_outputs(inp)
    pinned = []
    for arr in [a for c in inp.comps for a in list(c.arrays.values()) + c.bc_var] + pred + dpo:
        if arr.nbytes and lib.scf_host_register(arr.ctypes.data, arr.nbytes) == 0:
            pinned.append(arr)
    e2e = [ps(inp, opts, pred, dpo)[2] for _ in range(max(3, args.steps // 4))]
    unpin(lib, pinned)
    cells = g.imax * g.jmax * g.kmax
    it = sum(t["timed_iterations"] for t in timed)
    kms = {k: sum(t["ms_kernels"][q] for t in timed) / it for q, k in enumerate(("U", "P", "S", "X"))}
    kb = {k: BCG_BYTES_F32[k] * cells for k in kms}
    top = max(("P", "S"), key=lambda k: kms[k])
    achieved = kb[top] / (kms[top] * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        os.environ["OMP_NUM_THREADS"] = str(threads)
        from oracle import oracle as O
        o_cpu = PR.default_opts(rel_tol=tol)
        t0 = time.perf_counter()
        A, b, _ = O.mom_system(inp, o_cpu, 0)
        x, its, _ = O.csr_bicgstab(A, b, tol=tol)
        sec = time.perf_counter() - t0
        cpu = {"value": round(3 * sec * 1e3, 1), "unit": "ms/call", "cores": threads, "kind": "port",
               "sample": "the u system at %dx%dx%d (oracle SetMatrix + SetVectors, then Jacobi BiCGStab with OpenMP "
                         "to the same tolerance, %d iterations) timed once, times 3 components"
                         % (g.imax, g.jmax, g.kmax, its)}
    ms = [r["ms_total"] for r in runs]
    line = {
        "metric": "ms per momentum-predictor solve call at %dx%dx%d (SetMatrix + SetVectors + solve + "
                  "DeltaGetValues for u, v, w, Dp ghosts and predictor BCs)" % (g.imax, g.jmax, g.kmax),
        "value": round(statistics.mean(ms), 3), "unit": "ms/call", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(ms), 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 BiCGStab inside f64 refinement; f64 rows and Dp",
        "data": "synthetic (%s cut-cell geometry from GridPreprocess; viscous conductances from the apertures and "
                "the liquid fraction, Rey = 300; cut-face terms, wall friction and fluxes seeded)" % geo,
        "config": {"workload": ("momentum systems of c2: %d^3 unit cube, solid sphere, liquid bubble" % n
                                if geo == "c2" else
                                "momentum systems of c4: %dx%dx%d wave tank on [0,4]x[0,1]x[0,1], z-stretched "
                                "(ratio 1.02), vertical cylinder" % (g.imax, g.jmax, g.kmax))
                               + ", dt = 1e-3, Rey = 300, rel. tol 1e-10",
                   "grid": [g.imax, g.jmax, g.kmax],
                   "l2": "inputs larger than L2 (%.1f GB staged)" % (e2e[-1]["bytes_h2d"] / 1e9)},
        "iterations": runs[-1]["iterations"], "rounds": runs[-1]["rounds"],
        "rel_residual": runs[-1]["rel_residual"],
        "ms_assemble": round(statistics.mean(r["ms_assemble"] for r in runs), 3),
        "ms_solve": round(statistics.mean(r["ms_solve"] for r in runs), 3),
        "ms_tail": round(statistics.mean(r["ms_tail"] for r in runs), 3),
        "fp64": {"value": round(statistics.mean(r["ms_total"] for r in runs64), 3), "unit": "ms/call",
                 "iterations": runs64[-1]["iterations"], "ms_solve": round(statistics.mean(r["ms_solve"] for r in runs64), 3)},
        "e2e": {"value": round(statistics.mean(r["ms_total"] for r in e2e), 3), "unit": "ms/call",
                "h2d_bytes_per_step": int(e2e[-1]["bytes_h2d"]), "d2h_bytes_per_step": int(e2e[-1]["bytes_d2h"]),
                "ms_h2d": round(statistics.mean(r["ms_h2d"] for r in e2e), 3),
                "ms_d2h": round(statistics.mean(r["ms_d2h"] for r in e2e), 3)},
        "roofline": {"bound": "hbm",
                     "kernel": {"P": "k_bcg_p<float> (v = A p, r0.v)", "S": "k_bcg_s<float> (t = A s, t.s, t.t)"}[top]
                               + ", 16-cell column segments",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "bytes_per_launch": kb[top],
                     "ms_per_launch": round(kms[top], 5), "launches_timed": it,
                     "passes": {k: {"ms_per_launch": round(kms[k], 5), "bytes_per_launch": kb[k],
                                    "GB/s": round(kb[k] / (kms[k] * 1e-3) / 1e9, 1)} for k in kms},
                     "timing": "CUDA events around each stencil kernel of the BiCGStab iterations of 2 calls",
                     "traffic": None},
        "clocks": clocks,
        "gpu_launches": sum(r["gpu_launches"] for r in runs),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def clsvof_workload(n: int):
    """The 3-D deformation test of the reference's src/Test/AdvectionTest at
    t = 0 on an n^3 unit cube: a liquid sphere r = 0.15 at (0.35, 0.35, 0.35)
    (phiL its signed distance, vofL the cut of each cell by the sphere's
    tangent plane), u = 2 sin^2(pi x) sin(2 pi y) sin(2 pi z) and its v, w
    partners at the cell centres (zero in the ghosts), the fluid normals of
    a sphere about (1000, 1000, 1000), Dirichlet zero walls, dt from CFL 0.15
    capped at 0.15 h / 0.2 (AdvectionTest.f90:180-212)."""
    import numpy as np
    from simcoflow3d_gb300 import workloads as W
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    cg = (np.arange(n + 2) - 0.5) * h
    centres = tuple(np.asfortranarray(a) for a in np.meshgrid(c, c, c, indexing="ij"))
    spacings = tuple(np.full((n, n, n), h, order="F") for _ in range(3))
    X, Y, Z = np.meshgrid(cg, cg, cg, indexing="ij")
    dx, dy, dz = X - 0.35, Y - 0.35, Z - 0.35
    r = np.sqrt(dx * dx + dy * dy + dz * dz)
    phi = np.asfortranarray(r - 0.15)
    rn = np.maximum(r, 1e-300)
    nx, ny, nz = dx / rn, dy / rn, dz / rn
    s = phi + 0.5 * h * (np.abs(nx) + np.abs(ny) + np.abs(nz))
    vof = 1.0 - W.volume_fraction_calc(h, h, h, nx, ny, nz, s) / h ** 3
    vof = np.asfortranarray(np.where(vof <= 1e-14, 0.0, np.where(vof >= 1 - 1e-14, 1.0, vof)))
    inner = (slice(1, -1),) * 3
    vel = [np.zeros((n + 2,) * 3, order="F") for _ in range(3)]
    sx, sy, sz = np.sin(np.pi * X), np.sin(np.pi * Y), np.sin(np.pi * Z)
    s2x, s2y, s2z = np.sin(2 * np.pi * X), np.sin(2 * np.pi * Y), np.sin(2 * np.pi * Z)
    vel[0][inner] = (2.0 * sx * sx * s2y * s2z)[inner]
    vel[1][inner] = (-s2x * sy * sy * s2z)[inner]
    vel[2][inner] = (-s2x * s2y * sz * sz)[inner]
    fx, fy, fz = X - 1000.0, Y - 1000.0, Z - 1000.0
    fr = np.sqrt(fx * fx + fy * fy + fz * fz)
    fn = [np.zeros((n + 2,) * 3, order="F") for _ in range(3)]
    for q, f in enumerate((fx, fy, fz)):
        fn[q][inner] = (f / fr)[inner]
    vmax = max(np.abs(v).max() for v in vel)
    dt = min(0.15 * h / (vmax + 1e-30), 0.15 * h / 0.2)
    state = {"vofl": vof, "phil": phi}
    for key in ("nxl", "nyl", "nzl"):
        state[key] = np.zeros((n + 2,) * 3, order="F")
    shapes = [(n, n)] * 6
    lvs_bc = [np.zeros(sh, order="F") for sh in shapes]
    bc_vel = [np.zeros((n, n), order="F") for _ in range(3)]
    flags = dict(lvs_flag=(0,) * 6, lvs_const=(0.0,) * 6, vof_flag=(0,) * 6, vof_const=(0.0,) * 6)
    return centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags


# algorithmic bytes per interior cell of one launch: the fields a kernel must
# read and write once (neighbours come from cache)
CLSVOF_BYTES = {"sweep_first": 40, "sweep_later": 56, "reconstruct": 40}


def clsvof_cpu_ms(n_full: int, sample_n: int = 64):
    """The oracle's Clsvof_Scheme step on the same test at sample_n^3 (the
    reference test's own size), scaled to n_full^3 by the cell count."""
    from oracle import oracle as O
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags = clsvof_workload(sample_n)
    t0 = time.perf_counter()
    O.clsvof_scheme(centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, **flags)
    sec = time.perf_counter() - t0
    return sec * 1e3 * (n_full / sample_n) ** 3, sec


def run_clsvof(args):
    """One Clsvof_Scheme step (six sub-steps of three split sweeps, the wall
    planes, the reconstruction and the redistancing) on the reference's
    3-D deformation test scaled to 256^3: device time with the state
    resident, the host-array call end to end, the live roofline of the
    heaviest kernel kind, and the oracle on the host cores.  One JSON line."""
    import numpy as np
    from simcoflow3d_gb300.projection import load_library
    from simcoflow3d_gb300.transport import ClsvofScheme
    n = args.n or 256
    centres, spacings, state, vel, fn, bc_vel, lvs_bc, dt, flags = clsvof_workload(n)
    lib = load_library()
    sch = ClsvofScheme(n, n, n, lib=lib)
    work = {k: v.copy(order="F") for k, v in state.items()}
    planes = [p.copy(order="F") for p in lvs_bc]
    sch.stage(centres, spacings, work, vel, fn, bc_vel, planes, dt, **flags)
    for _ in range(args.warmup):
        sch.run(1)
    with ClockSampler(0) as cs:
        runs = [sch.run(1) for _ in range(args.steps)]
    clocks = cs.summary()
    sch.set_timing(True)
    timed = [sch.run(1) for _ in range(2)]
    sch.set_timing(False)
    # end to end through scf_clsvof_step with page-locked host arrays
    e_state = {k: v.copy(order="F") for k, v in state.items()}
    e_planes = [p.copy(order="F") for p in lvs_bc]
    pinned = []
    for arr in list(e_state.values()) + e_planes + list(centres) + list(spacings) + vel + fn + bc_vel:
        if arr.nbytes and lib.scf_host_register(arr.ctypes.data, arr.nbytes) == 0:
            pinned.append(arr)
    e2e = [sch(centres, spacings, e_state, vel, fn, bc_vel, e_planes, dt, **flags)[1]
           for _ in range(max(3, args.steps // 4))]
    unpin(lib, pinned)
    sch.close()
    cells = n ** 3
    kinds = ("reconstruct", "sweep", "walls", "redistance")
    kms = {k: sum(t["ms_kernels"][q] for t in timed) / len(timed) for q, k in enumerate(kinds)}
    # per step: 18 sweeps (6 first, 12 later) and 24 reconstructions
    sweep_bytes = 6 * cells * (CLSVOF_BYTES["sweep_first"] + 2 * CLSVOF_BYTES["sweep_later"])
    rec_bytes = 24 * cells * CLSVOF_BYTES["reconstruct"]
    top = max(("sweep", "reconstruct"), key=lambda k: kms[k])
    tb = {"sweep": sweep_bytes, "reconstruct": rec_bytes}[top]
    launches = {"sweep": 18, "reconstruct": 24}[top]
    achieved = tb / (kms[top] * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    cpu = None
    if not args.no_cpu:
        ms_cpu, sec = clsvof_cpu_ms(n)
        cpu = {"value": round(ms_cpu, 1), "unit": "ms/step", "cores": 1, "kind": "port",
               "sample": "one oracle Clsvof_Scheme step of the same test at 64^3 (the reference test's own grid), "
                         "%.2f s, scaled by the cell count to %d^3" % (sec, n)}
    ms = [r["ms_run"] for r in runs]
    line = {
        "metric": "ms per Clsvof_Scheme step at %d^3 (6 sub-steps x 3 split sweeps, wall planes, reconstruction, "
                  "redistancing)" % n,
        "value": round(statistics.mean(ms), 3), "unit": "ms/step", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(ms), 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: the 3-D deformation test of the reference's AdvectionTest at t = 0",
        "config": {"workload": "CLSVOF transport: liquid sphere r=0.15 at (0.35,0.35,0.35) in the %d^3 unit cube, "
                               "LeVeque deformation field, CFL 0.15, dt = %.3e" % (n, dt),
                   "grid": [n, n, n],
                   "l2": "inputs larger than L2 (%.1f GB staged)" % (e2e[-1]["bytes_h2d"] / 1e9)},
        "e2e": {"value": round(statistics.mean(r["ms_total"] for r in e2e), 3), "unit": "ms/step",
                "h2d_bytes_per_step": int(e2e[-1]["bytes_h2d"]), "d2h_bytes_per_step": int(e2e[-1]["bytes_d2h"]),
                "ms_h2d": round(statistics.mean(r["ms_h2d"] for r in e2e), 3),
                "ms_d2h": round(statistics.mean(r["ms_d2h"] for r in e2e), 3)},
        "roofline": {"bound": "hbm", "kernel": {"sweep": "k_sweep", "reconstruct": "k_reconstruct"}[top],
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind, "bytes_per_launch": tb // launches,
                     "ms_per_launch": round(kms[top] / launches, 5),
                     "kinds_ms_per_step": {k: round(v, 4) for k, v in kms.items()},
                     "timing": "CUDA events around every kernel of 2 steps", "traffic": None},
        "clocks": clocks,
        "gpu_launches": sum(r["gpu_launches"] for r in runs),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_output(args):
    """PrintResultVTK's snapshot of a c2 projection (p, u, v, w, phiL, phi,
    vofL, vof at 256^3) written by scf_write_vtr from the projection
    context's device arrays (the solid level set from the host), against the
    oracle's numpy writer from host arrays.  One JSON line."""
    import numpy as np
    from simcoflow3d_gb300 import output as OUT
    from simcoflow3d_gb300.projection import Projection
    w = make_workload("c2", args.seed, args.n)
    proj = Projection.for_workload(w, precision=1, rel_tol=args.tol, smoother_degree=4)
    u, v, ww, pp, _, _ = proj.update_puvw(w)
    dev = proj.device_fields()
    a = w.arrays
    phi = np.zeros(w.shape_g, order="F")
    phi[1:-1, 1:-1, 1:-1] = a["pcell_phi"]
    dx, dy, dz = a["pgrid_dx"][:, 0, 0], a["pgrid_dy"][0, :, 0], a["pgrid_dz"][0, 0, :]
    axes = (np.cumsum(dx) - dx / 2, dx, np.cumsum(dy) - dy / 2, dy, np.cumsum(dz) - dz / 2, dz)
    names = OUT.PRINT_RESULT_VTK_FIELDS
    fields = [(names[0], dev["p"]), (names[1], dev["u"]), (names[2], dev["v"]), (names[3], dev["w"]),
              (names[4], dev["phil"]), (names[5], phi), (names[6], dev["vofl"]), (names[7], dev["vof"])]
    shape = (w.imax, w.jmax, w.kmax)
    d = tempfile.mkdtemp(prefix="scf_vtr_")
    path = os.path.join(d, "PCell_3D.vtr")
    for _ in range(args.warmup):
        OUT.write_vtr(path, shape, axes, fields)
    runs = [OUT.write_vtr(path, shape, axes, fields) for _ in range(args.steps)]
    nbytes = runs[-1]["bytes_file"]
    cpu = None
    if not args.no_cpu:
        from oracle import vtr as V
        host = [(names[0], pp), (names[1], u), (names[2], v), (names[3], ww), (names[4], a["phil"]),
                (names[5], phi), (names[6], a["vofl"]), (names[7], a["vof"])]
        t0 = time.perf_counter()
        V.write_vtr(path + ".ref", shape, axes, host)
        cpu = {"value": round((time.perf_counter() - t0) * 1e3, 1), "unit": "ms/snapshot", "cores": 1,
               "kind": "port", "sample": "one 256^3 snapshot of the 8 fields from host arrays (numpy restatement)"}
        same = open(path, "rb").read() == open(path + ".ref", "rb").read()
        os.unlink(path + ".ref")
    else:
        same = None
    os.unlink(path)
    os.rmdir(d)
    mean = lambda k: statistics.mean(r[k] for r in runs)
    n = w.imax * w.jmax * w.kmax
    peak, peak_kind = measured_peaks()
    conv_ms = mean("ms_convert") / 8
    by = 12.0 * n     # one FP64 read and one FP32 write per cell and field
    line = {
        "metric": "ms per PrintResultVTK snapshot (8 fields, 256^3) from device-resident fields to a .vtr file",
        "value": round(mean("ms_total"), 3), "unit": "ms/snapshot", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(mean("ms_total"), 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64->f32", "data": "a c2 projection's fields (synthetic)",
        "config": {"workload": "c2 256^3 snapshot: p, u, v, w, phiL, phi, vofL, vof", "file_bytes": nbytes,
                   "file_system": "tempfile.gettempdir() of the box"},
        "breakdown_ms": {"convert": round(mean("ms_convert"), 3), "d2h": round(mean("ms_d2h"), 3),
                         "write": round(mean("ms_write"), 3)},
        "roofline": {"bound": "hbm", "kernel": "k_gather_f32 (gather + FP32 rounding of one field)",
                     "achieved": round(by / (conv_ms * 1e-3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(by / (conv_ms * 1e-3) / 1e9 / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_launch": by, "ms_per_launch": round(conv_ms, 5),
                     "timing": "CUDA events around each conversion launch"},
        "identical_to_oracle": same,
        "gpu_launches": sum(r["gpu_launches"] for r in runs),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2",
                    help="c0..c4; geometry (the cut-cell geometry preprocessing of the c2 geometry); output "
                         "(a PrintResultVTK snapshot of a c2 projection); predictor (the momentum predictor's "
                         "implicit solves on the c2 geometry); clsvof (one Clsvof_Scheme step of the "
                         "reference's 3-D deformation test at 256^3)")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--n", type=int, default=None, help="smaller grid (profiling captures only)")
    ap.add_argument("--sequence", type=int, default=0,
                    help="time N warm-started calls with fresh predictions (e.g. --config c4 --sequence 20)")
    ap.add_argument("--only", choices=["mixed", "fp64"], default=None,
                    help="time one precision device-resident only (profiling captures)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-oracle", action="store_true",
                    help="skip the errors against the oracle's FP64 solve (c2 line)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the c0, c1, c3 and c4-sequence legs of the default line")
    ap.add_argument("--pred-geometry", choices=["c2", "c4"], default="c2",
                    help="geometry of --config predictor (c4: the z-stretched wave tank, 512x256x256)")
    ap.add_argument("--max-cpu-s", type=float, default=330.0,
                    help="stop the reference arm's timed steps after this many s (recorded in its line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.sequence:
        return run_sequence(args)
    if args.config == "geometry":
        return run_geometry(args)
    if args.config == "output":
        return run_output(args)
    if args.config == "predictor":
        return run_predictor(args)
    if args.config == "clsvof":
        return run_clsvof(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
