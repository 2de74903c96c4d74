"""Benchmark: solves/s to a 1e-8 relative residual, learned preconditioner vs plain BiCGStab.

Default workload (``--workload learned3d``): the 3D 27-point nodal system at
257x129x257 nodes (stratified background times a seeded log-normal(0.1) cell
factor, divergence right-hand side).  The learned preconditioner -- the
background (spectral) solve of the horizontally averaged operator corrected by
a 6-layer BF16 network trained on the GPU with the library's own kernels --
runs inside flexible GMRES with FP64 refinement; one step = the background
solve's set-up from the step's coefficients + one solve, 256 MB L2 flush
before every step.  The same JSON line carries the plain double-float
BiCGStab arm (1 warm-up + 1 timed step: one plain solve takes tens of
seconds), the background-solve-only arm, the end-to-end rate from host
memory, the network's roofline and the CPU baseline.

``--workload solve2d``: the 2049x1025 standalone 9-point solve (plain
double-float BiCGStab on the GPU, ``--precision df64`` default; ``fp64``:
the reference algorithm in FP64; ``mixed``: FP32 inner solves in FP64
refinement), 64 seeds resident in HBM.  ``--workload ensemble``: the
48-member ensemble in one persistent launch per round.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--workload ...]

Prints one JSON line (rank 0).  Under torchrun (N > 1) each rank solves its
own system (independent replicas, weak scaling) and the time is the max over
ranks.  ``--impl reference`` times the reference algorithm on the host cores
(the CPU restatement of the reference path: NumPy stencil + plain FP64
BiCGStab) on the same configuration.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY = 2049, 1025
TOL = 1e-8
MAXIT = 30000
METRIC = "solves/s to 1e-8 residual: learned-precond vs plain BiCGStab, 1 GB300"
# DRAM bytes read + written by one launch of a roofline kernel, from one ncu capture
# each (the summaries in profiles/ give the commands); per launch, like `achieved`
STENCIL3D_TRAFFIC = 211.3e6     # k_stencil3d<float, APPLY>, 257x129x257 nodes
STENCIL2D_TRAFFIC = 134.4e6     # k_stencil2d<dfloat, PDIR>, 2049x1025 nodes
CONV_TRAFFIC = 107.1e6          # k_conv3d_tc<32, 32>, one hidden layer at 257x129x257 nodes (2x2x2 blocked)
# k_batch_bicgstab<dfloat, 64, 8>: 16.95 GB read + written by a 20-iteration launch of the
# 48-member ensemble, whose algorithmic bytes are 20 x 4,327,728 nodes x 200 B = 17.31 GB
ENSEMBLE_TRAFFIC_RATIO = 16.951e9 / 17.311e9
WORKLOAD = "2D nodal Helmholtz 9-point solve, 2049x1025 nodes, pseudo-incompressible, rtol 1e-8, 64 seeds"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seeds", type=int, default=64)
    ap.add_argument("--precision", default="df64", choices=["fp64", "mixed", "df64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="learned3d",
                    choices=["solve2d", "ensemble", "learned3d", "step3d", "step2d", "ensemble_steps"])
    ap.add_argument("--nz", type=int, default=257)
    ap.add_argument("--train-steps", type=int, default=1000)
    ap.add_argument("--skip", type=float, default=0.9)
    ap.add_argument("--no-subresults", action="store_true",
                    help="learned3d: skip the 2D solve and ensemble measurements carried in the same line")
    return ap.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled during the timed region:
    NVML through ctypes every 5 ms (the device matched by the CUDA device's UUID),
    else nvidia-smi every 200 ms.  Only samples taken between start() and stop() count;
    reading these values changes no setting of the GPU."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits (nvml.h): SW power cap, HW slowdown, SW thermal, HW thermal, HW power brake
    BITS = ((0x4, "sw_power_cap"), (0x8, "hw_slowdown"), (0x20, "sw_thermal_slowdown"),
            (0x40, "hw_thermal_slowdown"), (0x80, "hw_power_brake_slowdown"))
    PERIOD_S = 0.005

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.nvml = None
        self.stop_evt = threading.Event()

    def _nvml_handle(self):
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        try:
            import torch
            u = str(torch.cuda.get_device_properties(self.index).uuid)
            u = u if u.startswith("GPU-") else "GPU-" + u
            if lib.nvmlDeviceGetHandleByUUID(u.encode(), ctypes.byref(h)) == 0:
                return lib, h
        except Exception:
            pass
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) == 0:
            return lib, h
        return None

    def _nvml_loop(self):
        lib, h = self.nvml
        sm, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_r = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop_evt.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0 and \
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 and get_r(h, ctypes.byref(rs)) == 0:
                self.rows.append((float(sm.value), float(mx.value), int(rs.value)))
            self.stop_evt.wait(self.PERIOD_S)

    def start(self):
        try:
            self.nvml = self._nvml_handle()
        except OSError:
            self.nvml = None
        if self.nvml is not None:
            self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.nvml is not None:
            self.stop_evt.set()
            self.thread.join(timeout=5)
            sm = [r[0] for r in self.rows]
            reasons = {name for r in self.rows for bit, name in self.BITS if r[2] & bit}
            return {"sm_mhz": statistics.median(sm) if sm else None,
                    "sm_max_mhz": max(r[1] for r in self.rows) if self.rows else None,
                    "reasons": sorted(reasons), "samples": len(sm), "source": "nvml, 5 ms"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# --------------------------------------------------------------------------
# CPU side (reference algorithm restated; bounded sample)
# --------------------------------------------------------------------------
def cpu_sample(w_np, iters_per_solve, seconds):
    """Time the FP64 NumPy/SciPy restatement of the reference solve on this host.

    Runs scipy BiCGStab with the oracle's vectorised lap2D_gather_new for a
    bounded number of iterations and converts the time per iteration to
    solves/s with the iteration count of one full FP64 solve.
    """
    import scipy.sparse.linalg as spla
    from oracle import nodal2d as n2
    op = w_np
    n = op["nx"] * op["ny"]
    mv = lambda v: n2.lap2d_gather(v, op)
    t0 = time.perf_counter()
    mv(op["b"])
    t_mv = time.perf_counter() - t0
    it = max(3, int(seconds / (2.2 * t_mv)))
    A = spla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    cnt = [0]
    t0 = time.perf_counter()
    spla.bicgstab(A, op["b"], rtol=1e-30, atol=0.0, maxiter=it, callback=lambda xk: cnt.__setitem__(0, cnt[0] + 1))
    dt = time.perf_counter() - t0
    per_iter = dt / max(cnt[0], 1)
    return 1.0 / (per_iter * iters_per_solve), per_iter, cnt[0], dt


def _to_np(w):
    import torch
    out = {}
    for k, v in w.items():
        if isinstance(v, torch.Tensor):
            out[k] = v.cpu().numpy()
        elif isinstance(v, tuple):
            out[k] = tuple(None if t is None else t.cpu().numpy() for t in v)
        else:
            out[k] = v
    nc = (out["nx"] + 1) * (out["ny"] + 1)
    cxx, cyy, cxy, cyx = out["cor"]
    z = np.zeros(nc)
    out["cor"] = (cxx, cyy, z if cxy is None else cxy, z if cyx is None else cyx)
    out["hcenter"] = np.zeros(out["nx"] * out["ny"]) if out["hcenter"] is None else out["hcenter"]
    return out


def run_reference(args):
    """``--impl reference``: the reference algorithm on the host cores."""
    ws, rank, local = _dist()
    if ws > 1 and rank != 0:
        return
    from oracle import cases
    w = cases.stratified_2d(seed=0, inx=NX, iny=NY)
    w_np = dict(w["op"])
    w_np["b"] = w["b"]
    # iterations of one full FP64 solve: measured once on a smaller grid of the
    # same construction and scaled with the grid size (BiCGStab iterations on
    # this operator grow linearly with the node count per dimension)
    from oracle.krylov import bicgstab_legacy
    ws_small = cases.stratified_2d(seed=0, inx=257, iny=129)
    _, info, it_small = bicgstab_legacy(ws_small["op"], ws_small["b"], TOL, MAXIT)
    iters_est = it_small * (NX - 1) / 256.0
    vals = []
    t_all0 = time.perf_counter()
    for s in range(args.warmup + args.steps):
        v, per_iter, n_it, dt = cpu_sample(w_np, iters_est, max(2.0, args.cpu_seconds / 4))
        if s >= args.warmup:
            vals.append(v)
    wall = time.perf_counter() - t_all0
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": solve2d_config(args, _dist()[0], args.seeds),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": 1, "kind": "port",
                             "sample": "NumPy lap2D_gather_new restatement + scipy bicgstab (FP64), "
                                       "bounded iteration samples on seed 0; solves/s = 1/(s per iteration x "
                                       "%.0f iterations per solve, from a 257x129 solve scaled by grid size)"
                                       % iters_est},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU side
# --------------------------------------------------------------------------
def run_gpu(args):
    global NX, NY
    NX, NY = args.nx, args.ny
    import torch
    from pybella_gb300 import linalg, workloads, _lib

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    line = solve2d_line(args, dev, local, rank, world, dist, args.steps, args.warmup, max(1, args.seeds), args.steps,
                        want_cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def solve2d_line(args, dev, local, rank, world, dist, steps, warmup, nseeds, e2e_steps, want_cpu):
    """The 2049x1025 standalone solve measured over ``steps`` solves of ``nseeds``
    resident systems; returns the JSON line (dict)."""
    import torch
    from pybella_gb300 import linalg, workloads, _lib
    from pybella_gb300 import replicas
    systems = [workloads.stratified_2d(seed=sd, nx=NX, ny=NY, device=dev) for sd in replicas.seeds_for_rank(rank, nseeds)]
    ws = _lib.Workspace(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    xbuf = torch.empty(NX * NY, dtype=torch.float64, device=dev)

    def step(i, stats):
        w = systems[i % nseeds]
        flush.fill_(float(i))
        A = linalg.NodalHelmholtz2D(w["hplusx"], w["hplusy"], w["hcenter"], w["cor"], w["diag_inv"],
                                    NX, NY, w["dx"], w["dy"], w["x_wall"], w["y_wall"], ws=ws)
        x, st = A.solve(w["b"], tol=TOL, maxiter=MAXIT, precision=args.precision, out=xbuf)
        stats.append(st)

    warm = []
    for i in range(warmup):
        step(i, warm)
    # one FP64 solve of the first system: iteration count of the scipy-path algorithm
    w0 = systems[0]
    A0 = linalg.NodalHelmholtz2D(w0["hplusx"], w0["hplusy"], w0["hcenter"], w0["cor"], w0["diag_inv"],
                                 NX, NY, w0["dx"], w0["dy"], w0["x_wall"], w0["y_wall"], ws=ws)
    _, st64 = A0.solve(w0["b"], tol=TOL, maxiter=MAXIT, precision="fp64")

    ws.profile(True)
    launches0 = ws.launches
    clocks = ClockSampler(local)
    clocks.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ev0.record()
    stats = []
    for i in range(steps):
        step(warmup + i, stats)
    ev1.record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = ws.launches - launches0
    kt = {k: ws.kernel_time(k) for k in range(4)}
    ws.profile(False)
    ms = replicas.max_over_ranks(ms, device=dev)
    total_solves = steps * world
    value = replicas.aggregate_rate(steps, world, ms / 1000.0)

    # ---- end to end through the drop-in API with host buffers ----
    host = [] if args.no_e2e or e2e_steps == 0 else [_to_np(systems[i % nseeds]) for i in range(min(nseeds, 4))]
    e2e_stats = []
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    for i in range(e2e_steps if host else 0):
        h = host[i % len(host)]
        A = linalg.NodalHelmholtz2D(h["hplusx"], h["hplusy"], h["hcenter"], h["cor"], h["diag_inv"],
                                    NX, NY, h["dx"], h["dy"], h["x_wall"], h["y_wall"], ws=ws)
        x, info = linalg.bicgstab(linalg.LinearOperator(A.shape, A), h["b"], tol=TOL, maxiter=MAXIT,
                                  precision=args.precision)
        e2e_stats.append(info)
    torch.cuda.synchronize()
    te = time.perf_counter() - te0
    if dist is not None:
        t = torch.tensor([te], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        te = float(t.item())
    e2e_value = e2e_steps * world / te if host else None
    nnode = NX * NY
    ncell = (NX + 1) * (NY + 1)
    h2d = 8 * (4 * ncell + 2 * nnode) + 8 * nnode   # hplusx, hplusy, cxx, cyy, diag_inv, hcenter, b
    d2h = 8 * nnode

    # ---- roofline of the dominant kernel (p-direction stencil, FP32) ----
    peak, peak_kind = _peaks()
    names = {0: "stencil_pdir", 1: "stencil_sdir", 2: "vector_update", 3: "resid_fp64"}
    share = {names[k]: kt[k][0] for k in kt}
    tot_k = sum(share.values()) or 1.0
    pd_ms, pd_n = kt[0]
    # algorithmic bytes per launch of the p-direction stencil: r, p_old, v_old, r^
    # read, p_new, v_new written, diag_inv (7 node words) + Axx, Ayy (2 cell words)
    word = 4.0 if args.precision == "mixed" else 8.0
    alg_bytes = word * (7 * nnode + 2 * ncell)
    achieved = alg_bytes / (pd_ms / pd_n / 1000.0) / 1e9 if pd_n else None
    iters = [s["iterations"] for s in stats]

    # ---- the same systems with the background-solve preconditioner (set up per step) ----
    from pybella_gb300.spectral import BackgroundSolve
    bg_stats = []
    bg_holder = []

    def bg_step(i):
        w = systems[i % nseeds]
        flush.fill_(float(i))
        A = linalg.NodalHelmholtz2D(w["hplusx"], w["hplusy"], w["hcenter"], w["cor"], w["diag_inv"],
                                    NX, NY, w["dx"], w["dy"], w["x_wall"], w["y_wall"], ws=ws)
        # the background solve re-derived from this step's coefficients (made once, updated in place)
        if not bg_holder:
            bg_holder.append(BackgroundSolve(A))
        bg = bg_holder[0].update(A)
        x, st = A.solve(w["b"], tol=TOL, maxiter=MAXIT, preconditioner=bg, out=xbuf)
        bg_stats.append(st)

    for i in range(warmup):
        bg_step(i)
    bg_stats.clear()
    torch.cuda.synchronize()
    eb0, eb1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    eb0.record()
    for i in range(steps):
        bg_step(warmup + i)
    eb1.record()
    torch.cuda.synchronize()
    bg_ms = eb0.elapsed_time(eb1) / steps

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "mixed": "f32+f64", "df64": "f32x2 (double-float)"}[args.precision],
        "data": "synthetic",
        "config": solve2d_config(args, world, nseeds),
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "path": "pybella_gb300.linalg.bicgstab on NumPy operands"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": STENCIL2D_TRAFFIC if args.precision == "df64" else None,
                     "traffic_source": "ncu dram bytes read + written of one launch "
                                       "(profiles/stencil2d_df64_pdir_2049x1025_ncu.md)",
                     "kernel": "k_stencil2d<%s, PDIR>" % {"fp64": "double", "mixed": "float", "df64": "dfloat"}[args.precision],
                     "peak_source": peak_kind,
                     "alg_bytes_per_launch": alg_bytes},
        "clocks": clk,
        "solver": {"iterations_mean": float(np.mean(iters)), "outer_mean": float(np.mean([s["outer"] for s in stats])),
                   "relres_max": max(s["relres"] for s in stats), "status": sorted(set(s["status"] for s in stats)),
                   "fp64_path_iterations": st64["iterations"], "fp64_path_relres": st64["relres"],
                   "e2e_info": sorted(set(e2e_stats))},
        "background": {"solves_per_s": 1000.0 / bg_ms, "ms": bg_ms,
                       "iterations_mean": float(np.mean([q["iterations"] for q in bg_stats])),
                       "relres_max": max(q["relres"] for q in bg_stats),
                       "fallback": max(q["fallback"] for q in bg_stats),
                       "over_value": (1000.0 / bg_ms) / value,
                       "what": "background-solve preconditioned flexible BiCGStab, same systems, set-up per step"},
        "kernel_ms_share": {k: v / tot_k for k, v in share.items()},
        "kernel_ms_per_launch": {names[k]: (kt[k][0] / kt[k][1] if kt[k][1] else None) for k in kt},
        "wall_s": wall,
    }
    if want_cpu:
        w_np = _to_np(systems[0])
        v, per_iter, n_it, dt = cpu_sample(w_np, st64["iterations"], args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": "%d FP64 BiCGStab iterations (NumPy lap2D_gather_new restatement + scipy) "
                                          "on seed 0 in %.1f s; solves/s = 1/(%.3f s/iter x %d iterations of the "
                                          "FP64 solve)" % (n_it, dt, per_iter, st64["iterations"])}
    return line


# --------------------------------------------------------------------------
# ensemble: 48 rising-bubble members' solves in one persistent launch
# --------------------------------------------------------------------------
ENS_WORKLOAD = ("ensemble of 48 rising-bubble projection solves (16 each at 160x80, 320x160, 640x320 cells), "
                "BiCGStab rtol 1e-10 (FP64 true residual), one persistent launch per round")


def _cpu_iter_seconds(w_np, iters=20):
    """Seconds per FP64 BiCGStab iteration of the NumPy/SciPy restatement on this host (bounded sample)."""
    import scipy.sparse.linalg as spla
    from oracle import nodal2d as n2
    n = w_np["nx"] * w_np["ny"]
    A = spla.LinearOperator((n, n), matvec=lambda v: n2.lap2d_gather(v, w_np), dtype=np.float64)
    cnt = [0]
    t0 = time.perf_counter()
    spla.bicgstab(A, w_np["b"], rtol=1e-30, atol=0.0, maxiter=iters, callback=lambda xk: cnt.__setitem__(0, cnt[0] + 1))
    return (time.perf_counter() - t0) / max(cnt[0], 1)


def run_ensemble(args):
    import torch
    from pybella_gb300 import ensemble, workloads
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    line = ensemble_line(args, dev, local, rank, world, dist, args.steps, args.warmup, args.steps,
                         want_cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def ensemble_line(args, dev, local, rank, world, dist, steps, warmup, e2e_steps, want_cpu):
    """One round of the 48 members' solves per step in one persistent launch; returns the JSON line (dict)."""
    import torch
    from pybella_gb300 import ensemble, workloads
    members = workloads.rising_bubble_ensemble(seed=17 + rank, device=dev)
    ops = [workloads.operator_2d(w) for w in members]
    bs = [w["b"] for w in members]
    xs = [torch.zeros_like(b) for b in bs]
    prec = "fp64" if args.precision == "fp64" else "df64"
    choice, tune_ms = ensemble.autotune(ops, bs, probe_iters=20, precision=prec)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for i in range(warmup):
        ensemble.solve_ensemble(ops, bs, tol=1e-10, maxiter=20000, out=xs, precision=prec)
    clocks = ClockSampler(local)
    clocks.start()
    if dist is not None:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kms = []
    stats = None
    torch.cuda.synchronize()
    ev0.record()
    for i in range(steps):
        flush.fill_(float(i))
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k0.record()
        _, stats = ensemble.solve_ensemble(ops, bs, tol=1e-10, maxiter=20000, out=xs, precision=prec)
        k1.record()
        kms.append((k0, k1))
    ev1.record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    step_ms = [a.elapsed_time(b) for a, b in kms]
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = steps * world * len(ops) / (ms / 1000.0)
    # end to end: host operands -> device, one round, solutions back to the host
    def _np(v):
        if isinstance(v, torch.Tensor):
            return v.cpu().numpy()
        if isinstance(v, tuple):
            return tuple(_np(t) for t in v)
        return v
    host = [{k: _np(v) for k, v in w.items()} for w in members]
    te0 = time.perf_counter()
    h2d = d2h = 0
    for i in range(e2e_steps):
        ops_e = [workloads.operator_2d(h, ws=op.ws) for h, op in zip(host, ops)]
        xs_e, _ = ensemble.solve_ensemble(ops_e, [h["b"] for h in host], tol=1e-10, maxiter=20000, precision=prec)
        out = [x.cpu().numpy() for x in xs_e]
    torch.cuda.synchronize()
    te = time.perf_counter() - te0
    # the same round as 48 separate single solves (the per-member path), for comparison
    ops_s = [workloads.operator_2d(w, ws=op.ws) for w, op in zip(members, ops)]
    for op, b in zip(ops_s, bs):
        op.solve(b, tol=1e-10, maxiter=20000, precision=prec)
    torch.cuda.synchronize()
    ts0 = time.perf_counter()
    for op, b in zip(ops_s, bs):
        op.solve(b, tol=1e-10, maxiter=20000, precision=prec)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - ts0
    for h in host:
        nn, nc = h["nx"] * h["ny"], (h["nx"] + 1) * (h["ny"] + 1)
        h2d += 8 * (4 * nc + 2 * nn)
        d2h += 8 * nn
    # roofline: FP64 words per node and iteration (two 5-word matvecs + 15-word vector chain)
    peak, peak_kind = _peaks()
    alg = sum(200.0 * op.n * st["iterations"] for op, st in zip(ops, stats))
    achieved = alg / (statistics.median(step_ms) / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32x2 (double-float) + f64 refinement",
        "data": "synthetic",
        "config": {"workload": ENS_WORKLOAD, "members": len(ops), "unknowns": int(sum(op.n for op in ops)),
                   "precision": prec,
                   "rtol": 1e-10, "launch_config": ensemble.configs()[choice], "autotune_ms": tune_ms,
                   "l2": "flushed (256 MB write) before every round",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e_steps * world * len(ops) / te if e2e_steps else None, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "path": "pybella_gb300.ensemble.solve_ensemble on NumPy operands"},
        "gpu_launches": steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": alg * ENSEMBLE_TRAFFIC_RATIO,
                     "traffic_source": "ncu dram bytes read + written of one 20-iteration launch of the same 48 "
                                       "members, 0.979 of its algorithmic bytes, scaled to this round by member "
                                       "iterations x nodes",
                     "kernel": "k_batch_bicgstab (whole round, one launch)",
                     "peak_source": peak_kind, "alg_bytes_per_launch": alg},
        "clocks": clk,
        "solver": {"iterations": [st["iterations"] for st in stats], "status": sorted(set(st["status"] for st in stats)),
                   "relres_max": max(st["relres"] for st in stats),
                   "refinement_rounds": [st["fallback"] for st in stats]},
        "sequential_single_solves": {"solves_per_s": len(ops) / seq_s, "round_s": seq_s,
                                     "path": "NodalHelmholtz2D.solve per member, precision %s" % prec},
    }
    if want_cpu:
        per_grid = {}
        est = 0.0
        for w, op, st in zip(host, ops, stats):
            key = (w["nx"], w["ny"])
            if key not in per_grid:
                w_np = dict(w)
                nc = (w["nx"] + 1) * (w["ny"] + 1)
                w_np["cor"] = (w["cor"][0], w["cor"][1], np.zeros(nc), np.zeros(nc))
                w_np["hcenter"] = np.zeros(w["nx"] * w["ny"])
                per_grid[key] = _cpu_iter_seconds(w_np, iters=40)
            est += per_grid[key] * st["iterations"]
        line["cpu_baseline"] = {"value": len(ops) / est, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": "40 FP64 BiCGStab iterations per grid size (NumPy lap2D_gather_new "
                                          "restatement + scipy); a round = sum over members of s/iteration x the "
                                          "member's iterations"}
    return line


# --------------------------------------------------------------------------
# learned preconditioner vs plain BiCGStab on the 3D 27-point problem
# --------------------------------------------------------------------------
LEARNED3D = ("3D 27-point nodal solve %s nodes, stratified x log-normal(0.1) cells, rtol 1e-8: learned "
             "preconditioner (background solve + trained network, flexible GMRES) vs plain double-float BiCGStab")


def _peaks_tensor():
    """(HBM GB/s, sustained BF16 TFLOP/s, source) from MEASURED_PEAKS.json."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops_sustained"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1700.0, "fallback"


def cpu_sample_3d(op, seconds):
    """Seconds per plain FP64 BiCGStab iteration of the oracle's C restatement
    (lap3D + scipy's BiCGStab loop, OpenMP over all host threads) on the full 3D
    grid: bounded runs of a few iterations until ``seconds`` have passed.
    Returns ``(seconds per iteration, iterations timed, threads)``."""
    from oracle import cbuild
    b = np.random.default_rng(0).standard_normal(op["nx"] * op["ny"] * op["nz"])
    cbuild.bicgstab3d(op, b, 1e-30, 1)                       # first touch, thread start-up
    t0 = time.perf_counter()
    k = 0
    while k < 3 or time.perf_counter() - t0 < seconds:
        _, _, it, _ = cbuild.bicgstab3d(op, b, 1e-30, 5)
        k += it
    return (time.perf_counter() - t0) / k, k, cbuild.threads()


def plain_iterations_fit(seed, shape, grids=((33, 17, 33), (65, 33, 65), (129, 65, 129))):
    """Iterations of plain FP64 BiCGStab to rtol 1e-8 on ``shape``, from full solves
    of the same construction (same seed) on smaller grids with the C restatement,
    fitted as log(iterations) = a + alpha log(nx - 1) and evaluated at ``shape``
    (plain BiCGStab on this operator needs about h^-alpha iterations; its slow
    modes are the smooth and hourglass-modulated ones).  Returns
    ``(estimate, {grid: iterations}, alpha, seconds)``."""
    from oracle import cases, cbuild
    t0 = time.perf_counter()
    pts = {}
    for g in grids:
        w = cases.stratified_3d(seed, *g)
        _, info, it, _ = cbuild.bicgstab3d(w["op"], w["b"], TOL, 400000)
        pts["x".join(map(str, g))] = it
    xs = np.log(np.array([g[0] - 1.0 for g in grids]))
    ys = np.log(np.array(list(pts.values()), dtype=np.float64))
    alpha, a = np.polyfit(xs, ys, 1)
    est = float(np.exp(a + alpha * np.log(shape[0] - 1.0)))
    return est, pts, float(alpha), time.perf_counter() - t0


def fp64_oracle_errors(A, b, xs, shape):
    """Relative L2 error of each solution in ``xs`` against a tightly converged FP64
    solution of the same system (true FP64 residual <= 1e-13: background-
    preconditioned solve with FP64 refinement), computed outside the timed region.
    The pressure is determined only up to the operator's null space (constants and
    the hourglass families, about nx + ny + nz modes), which no physical quantity
    sees, so it is compared through its cell gradients -- the 4-edge differences
    the momentum correction applies (rhou, rhov, rhow)."""
    import torch
    from pybella_gb300.spectral import BackgroundSolve
    bg = BackgroundSolve(A)
    xs_ref, st = A.solve(b, tol=1e-13, maxiter=5000, preconditioner=bg, method="bicgstab", max_outer=60)
    bg.close()

    def grads(x):
        p = x.reshape(shape)
        gx = p[1:] - p[:-1]
        gy = p[:, 1:] - p[:, :-1]
        gz = p[:, :, 1:] - p[:, :, :-1]
        return (gx[:, 1:, 1:] + gx[:, :-1, 1:] + gx[:, 1:, :-1] + gx[:, :-1, :-1],
                gy[1:, :, 1:] + gy[:-1, :, 1:] + gy[1:, :, :-1] + gy[:-1, :, :-1],
                gz[1:, 1:] + gz[:-1, 1:] + gz[1:, :-1] + gz[:-1, :-1])
    rel = lambda a_, b_: float(torch.linalg.norm(a_ - b_) / torch.linalg.norm(b_))
    gref = grads(xs_ref)
    out = {"reference_solution": {"relres": st["relres"], "iterations": st["iterations"], "status": st["status"],
                                  "what": "FP64 true residual <= 1e-13, background-preconditioned, FP64 refinement"}}
    for name, x in xs.items():
        g = grads(x)
        out[name] = {"grad_x_rhou": rel(g[0], gref[0]), "grad_y_rhov": rel(g[1], gref[1]),
                     "grad_z_rhow": rel(g[2], gref[2])}
    return out


def learned3d_config(shape):
    """The ``config`` of the 3D solve workload: identical in both arms."""
    return {"workload": LEARNED3D % "x".join(map(str, shape)), "nodes": list(shape), "rtol": TOL,
            "system_seed": 7}


def run_learned3d(args):
    import torch
    import warnings
    from pybella_gb300 import learned, workloads, _lib, replicas
    from pybella_gb300.linalg import NodalHelmholtz3D
    from pybella_gb300.spectral import BackgroundSolve
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    shape = (args.nx, args.ny, args.nz)
    # training (not timed; every rank trains the same network from the same seeds):
    # pairs from the background-preconditioned solver's own iterates on seeds
    # 1, 2, 3, 5, Adam on the library's kernels
    t0 = time.perf_counter()
    params, losses = learned.train_preconditioner(shape=shape, background=True, skip=args.skip,
                                                  steps=args.train_steps, npairs=4000)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    w = workloads.stratified_3d(7 + 1000 * rank, *shape)          # each replica its own system
    ws = _lib.Workspace(local)
    A = learned.operator_3d(w, ws=ws)
    net = learned.CNN(shape, block=2, mode="linear", skip=args.skip)
    net.set_params(params)
    b = w["b"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    kw_learned = dict(method="fgmres", restart=30)
    bg_launches = [0]
    xs = {k: torch.zeros(A.n, dtype=torch.float64, device=dev)
          for k in ("plain", "background", "background_fgmres", "learned")}

    bg_keep = BackgroundSolve(A)                     # made once; every step re-derives it in place

    def step(name):
        if name == "plain":
            return A.solve(b, tol=TOL, maxiter=200000, precision="df64", out=xs[name])[1]
        l0 = bg_keep.launches()
        bg = bg_keep.update(A)                       # from this step's coefficients
        pc = bg if name.startswith("background") else learned.LearnedPreconditioner(bg, net, "post")
        kw = dict(method="bicgstab") if name == "background" else kw_learned
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            st = A.solve(b, tol=TOL, maxiter=20000, preconditioner=pc, out=xs[name], **kw)[1]
        bg_launches[0] += bg.launches() - l0
        return st

    def timed(name, nw, ns, sample_clocks=False):
        for _ in range(nw):
            step(name)
        clocks = ClockSampler(local) if sample_clocks else None
        if clocks:
            clocks.start()
        l0, n0, b0 = ws.launches, net.launches, bg_launches[0]
        if dist is not None:
            dist.barrier()
        tot, sts = 0.0, []
        for _ in range(ns):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            sts.append(step(name))
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        if dist is not None:
            dist.barrier()
        launches = (ws.launches - l0) + (net.launches - n0) + (bg_launches[0] - b0)
        clk = clocks.stop() if clocks else None
        return {"ms": tot / ns, "stats": sts, "launches": launches, "clocks": clk}

    # the headline: learned-preconditioned solves, every rank, max over ranks
    L = timed("learned", args.warmup, args.steps, sample_clocks=True)
    ms_max = replicas.max_over_ranks(L["ms"] * args.steps, device=dev)
    value = replicas.aggregate_rate(args.steps, world, ms_max / 1000.0)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    B = timed("background", args.warmup, args.steps)
    BF = timed("background_fgmres", args.warmup, args.steps)
    P = timed("plain", 1, 1)                         # one plain solve takes tens of seconds
    # end to end through the public API: operator planes and b from pinned host
    # memory, device operator and background set-up, solve, x back to the host
    host = {k: w[k].detach().cpu().pin_memory() for k in ("hplusx", "hplusy", "hplusz", "diag_inv", "b")}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    e2e_ms = []
    ws_e2e = _lib.Workspace(local)
    bg_e2e = []                                      # one background solve per grid, as a time loop keeps it
    xh = torch.empty(A.n, dtype=torch.float64, pin_memory=True)   # the caller's pinned result buffer
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Ah = NodalHelmholtz3D(host["hplusx"], host["hplusy"], host["hplusz"], None, host["diag_inv"], *shape,
                              w["dx"], w["dy"], w["dz"], walls=w["walls"], ws=ws_e2e)
        if not bg_e2e:                               # made in the first (warm-up) call
            bg_e2e.append(BackgroundSolve(Ah))
        bg = bg_e2e[0].update(Ah)                    # from this call's coefficients
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            x, _ = Ah.solve(host["b"], tol=TOL, maxiter=20000,
                            preconditioner=learned.LearnedPreconditioner(bg, net, "post"), **kw_learned)
        xh.copy_(x)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1000.0)
        del Ah
    for b_ in bg_e2e:
        b_.close()
    # the learned solve's kernels: network application and background solve, timed alone
    bg = BackgroundSolve(A)
    r32 = torch.randn(A.n, device=dev)
    y32 = torch.empty_like(r32)

    def ev_ms(f, k=10):
        for _ in range(3):
            f()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(k):
            f()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    cnn_ms = ev_ms(lambda: net.forward(r32, shape, scale=1.0, out=y32))
    bg_ms = ev_ms(lambda: bg.apply(r32, out=y32))
    # the FGMRES iteration's FP32 matvec (k_stencil3d<float, APPLY>), back to back:
    # its 204 MB working set is larger than L2.  Algorithmic bytes: x, y, diag_inv
    # per node, the three axis coefficients per cell, 4 bytes each.
    st_ms = ev_ms(lambda: A.matvec_f32(r32), k=20)
    ncell = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    st_bytes = A.n * 3 * 4 + ncell * 3 * 4
    nv = learned.net_voxels(shape, 2)
    cnn_flops = nv * 2 * 27 * (8 * 32 + 4 * 32 * 32 + 32 * 8)      # 8 sub-node channels in and out
    napp = L["stats"][-1]["iterations"]
    hbm, tpeak, pkind = _peaks_tensor()
    ach = cnn_flops / (cnn_ms / 1000.0) / 1e12
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        from oracle import cases
        wc = cases.stratified_3d(7, *shape)
        per_it, k, nthr = cpu_sample_3d(wc["op"], args.cpu_seconds)
        cpu = {"value": 1.0 / (per_it * P["stats"][-1]["iterations"]), "unit": "solves/s", "cores": nthr,
               "kind": "port",
               "sample": "%d iterations of plain FP64 BiCGStab (the oracle's C restatement of lap3D and scipy's "
                         "loop, OpenMP on %d host threads) on the full grid, %.1f ms each, times the %d iterations "
                         "the GPU's plain BiCGStab (scipy's control flow in double-float arithmetic) took on this "
                         "system in this run: extrapolated; the count of this ill-conditioned iteration depends on "
                         "rounding (the reference arm fits FP64 solves on smaller grids instead)"
                         % (k, nthr, per_it * 1e3, P["stats"][-1]["iterations"])}
    stats = lambda R: {"solves_per_s": 1000.0 / R["ms"], "ms": R["ms"], "iterations": R["stats"][-1]["iterations"],
                       "outer": R["stats"][-1]["outer"], "relres": R["stats"][-1]["relres"],
                       "fallback": R["stats"][-1]["fallback"], "status": R["stats"][-1]["status"]}
    oracle_err = fp64_oracle_errors(A, b, xs, shape)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 network + f32 inner / f64 refinement", "data": "synthetic",
        "config": learned3d_config(shape),
        "setup": {"network": "6 layers 3x3x3, 32 channels, 2x2x2-blocked grid, linear, identity path %.2f"
                             % args.skip,
                  "train_steps": args.train_steps, "train_s": train_s, "final_loss": losses[-1][1],
                  "parallelism": "replicas" if world > 1 else "single GPU",
                  "plain_steps": "1 warm-up + 1 timed (one plain solve takes tens of seconds)",
                  "l2": "256 MB L2 flush before every step; operator planes %.0f MB" % (A.n * 8 * 6 / 1e6)},
        "fp64_oracle_err": oracle_err,
        "plain": stats(P), "background": stats(B), "background_fgmres": stats(BF), "learned": stats(L),
        "learned_over_plain": P["ms"] / L["ms"], "background_over_plain": P["ms"] / B["ms"],
        "network_gain_over_background": B["ms"] / L["ms"],
        "network_gain_over_background_fgmres": {"time": BF["ms"] / L["ms"],
                                                "iterations": BF["stats"][-1]["iterations"]
                                                / max(L["stats"][-1]["iterations"], 1),
                                                "what": "the same flexible GMRES with the background solve alone"},
        "e2e": ({"value": 1000.0 / statistics.median(e2e_ms), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                 "d2h_bytes_per_step": A.n * 8,
                 "path": "NodalHelmholtz3D from pinned host planes, BackgroundSolve.update, solve(preconditioner="
                         "LearnedPreconditioner, method='fgmres'), x into a pinned host buffer; median of the "
                         "timed calls"}
                if e2e_ms else None),
        "gpu_launches": L["launches"],
        "roofline": {"bound": "tensor", "achieved": ach, "peak": tpeak, "unit": "TFLOP/s", "frac": ach / tpeak,
                     "traffic": CONV_TRAFFIC,
                     "traffic_source": "ncu dram bytes read + written of one hidden-layer launch (one of the "
                                       "six; profiles/conv3d_tc_ws_bf16_257x129x257_ncu.md)",
                     "kernel": "k_conv3d_tc x6 (one network application)",
                     "peak_source": pkind + " bf16 sustained", "flops_per_launch": cnn_flops,
                     "ms_per_application": cnn_ms, "applications_per_solve": napp,
                     "background_apply_ms": bg_ms},
        "stencil_roofline": {"bound": "hbm", "kernel": "k_stencil3d<float, APPLY> (the FP32 matvec of each "
                                                      "FGMRES iteration)",
                             "achieved": st_bytes / (st_ms / 1000.0) / 1e9, "peak": hbm, "unit": "GB/s",
                             "frac": st_bytes / (st_ms / 1000.0) / 1e9 / hbm, "us_per_launch": st_ms * 1000.0,
                             "alg_bytes_per_launch": st_bytes, "traffic": STENCIL3D_TRAFFIC,
                             "traffic_source": "ncu dram bytes read + written of one launch at this size "
                                               "(profiles/stencil3d_f32_apply_257x129x257_ncu.md)"},
        "clocks": L["clocks"],
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if world == 1 and not args.no_subresults:
        # the other measured configurations, in the same run: the 2049x1025 standalone
        # solve over its 64 seeds, and one ensemble round of 48 members per step
        del A, net, xs, bg
        torch.cuda.empty_cache()
        line["solve2d"] = solve2d_line(args, dev, local, 0, 1, None, 64, 2, 64, 4, want_cpu=False)
        line["ensemble"] = ensemble_line(args, dev, local, 0, 1, None, 5, 2, 2, want_cpu=False)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference_3d(args):
    """``--impl reference`` for the 3D workload: plain FP64 BiCGStab -- the
    reference's solve, scipy's bicgstab on lap3D -- as the oracle's C restatement
    on all the host cores.  A full solve takes tens of thousands of iterations
    (tens of minutes on the host), so each step times a bounded sample of
    iterations on the full grid and the iterations per solve come from full
    solves on smaller grids of the same construction, fitted over the grid size
    (stated in the line as an extrapolation)."""
    world, rank, local = _dist()
    if world > 1 and rank != 0:
        return
    from oracle import cases
    shape = (args.nx, args.ny, args.nz)
    t_all0 = time.perf_counter()
    iters, pts, alpha, fit_s = plain_iterations_fit(7, shape)
    wc = cases.stratified_3d(7, *shape)
    vals, per = [], []
    for s_ in range(args.warmup + args.steps):
        per_it, k, nthr = cpu_sample_3d(wc["op"], max(1.0, args.cpu_seconds / 8))
        if s_ >= args.warmup:
            vals.append(1.0 / (per_it * iters))
            per.append(per_it)
    value = float(np.mean(vals))
    sample = ("plain FP64 BiCGStab (the oracle's C restatement of lap3D and scipy's loop) on %d host threads: "
              "%.1f ms per iteration on the full grid (bounded samples), times %.0f iterations per solve "
              "extrapolated from full solves of the same system construction on smaller grids %s (fit "
              "iterations ~ (nx-1)^%.2f)" % (nthr, 1e3 * float(np.mean(per)), iters, pts, alpha))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": learned3d_config(shape),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthr, "kind": "port", "sample": sample},
            "extrapolated": {"iterations_per_solve": iters, "fit_points": pts, "alpha": alpha, "fit_s": fit_s,
                             "what": "solves/s = 1 / (measured s per iteration x fitted iterations per solve); "
                                     "no full solve runs in this line"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_all0}
    print(json.dumps(line), flush=True)


def _cpu_step2d_sample(seconds):
    """Steps/s of the oracle's 2D time step (NumPy restatement of time_update.do,
    pinned to the reference) on the 160x80-cell rising bubble, one host thread."""
    from oracle import advection2d as adv, cases, step2d
    grid, prm, Sol, p2, hn, hc, sf = cases.rising_bubble()
    S0c = np.broadcast_to(hc["S0"][None, :], grid.elem_sc).copy()
    flux = adv.new_flux(grid)
    t0, k = time.perf_counter(), 0
    while k < 1 or time.perf_counter() - t0 < seconds:
        Sol = step2d.time_step(Sol, p2, flux, k, 0.02169, grid, prm, hn, hc, S0c, sf)
        k += 1
    return k / (time.perf_counter() - t0), k


def run_step2d(args):
    """``--workload step2d``: whole 2D time steps of the rising bubble (160x80
    cells, tol 1e-10, fixed dt = 21.69 s as the reference's 'CFLfixed' first steps)
    with the state resident on the GPU (DeviceStep2D: advection, explicit and
    implicit projection halves, double-float solves); value = steps/s.  The CPU
    baseline is the oracle's step (the reference's algorithm restated in NumPy)."""
    import torch
    from pybella_gb300 import workloads
    from pybella_gb300.time_update import DeviceStep2D
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    st = workloads.bubble_2d_state()
    run = DeviceStep2D(st["Sol"], st["mpv"], st["elem"], st["node"], st["ud"], st["th"], device=local)
    dt = 21.69 / st["ud"].t_ref
    for k in range(args.warmup):
        run.step(k, dt, precision=args.precision)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = ClockSampler(local)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.steps):
        run.step(args.warmup + k, dt, precision=args.precision)
    e1.record()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            v, k = _cpu_step2d_sample(args.cpu_seconds)
            cpu = {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                   "sample": "%d steps of the oracle's time step on the same state" % k}
        its = [s_["iterations"] for s_ in run.stats[-2 * args.steps:]]
        print(json.dumps({"metric": "2D time steps/s (rising bubble 160x80, projections to 1e-10)",
                          "value": world * 1000.0 / ms, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64 state, %s solves" % args.precision, "data": "synthetic",
                          "config": step2d_config(world),
                          "solve_iterations": its, "clocks": clocks, "cpu_baseline": cpu,
                          "gpu_launches": None}), flush=True)


ENS_STEPS_WORKLOAD = ("ensemble time steps: 48 rising-bubble members (16 each at 160x80, 320x160, 640x320 cells, "
                      "amplitude N(2 K, 0.2 K), centre N(0, 200 m)), each step's two projections of all members "
                      "solved in one persistent launch (rtol 1e-10)")


def solve2d_config(args, world, nseeds):
    """config of the 2049x1025 standalone-solve lines (both arms)."""
    return {"workload": WORKLOAD, "nx": NX, "ny": NY, "rtol": TOL, "precision": args.precision,
            "l2": "GPU arm: flushed (256 MB write) before every step; CPU arm: host-resident inputs",
            "seeds": nseeds, "parallelism": "replicas" if world > 1 else "single"}


def step2d_config(world):
    """config of the 2D time-step lines (both arms, so the driver sees the same config)."""
    return {"workload": "2D time step, rising bubble 160x80 cells",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "state of 1 MB, L2-resident (a launch-bound workload)"}


def ens_steps_config(world):
    """config of the ensemble time-step lines (both arms): 16 members on each grid."""
    from pybella_gb300.workloads import ENSEMBLE_GRIDS
    nodes = [(cx + 1, cy + 1) for cx, cy in ENSEMBLE_GRIDS]
    return {"workload": ENS_STEPS_WORKLOAD, "members": 16 * len(nodes),
            "unknowns": int(sum(16 * nx * ny for nx, ny in nodes)),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "state of %.0f MB resident (larger than L2 across the ensemble)"
                  % (sum(16 * 6 * 8 * (nx + 3) * (ny + 3) for nx, ny in nodes) / 1e6)}


def ensemble_steps_line(args, local, rank, world, nsteps, warmup, want_cpu):
    """``nsteps`` time steps of the 48-member ensemble with the state resident on the
    GPU (EnsembleStep2D); returns the JSON line (dict)."""
    import torch
    from pybella_gb300 import workloads
    from pybella_gb300.time_update import DeviceStep2D, EnsembleStep2D
    states = workloads.bubble_ensemble_states(seed=17 + rank)
    members = [DeviceStep2D(st["Sol"], st["mpv"], st["elem"], st["node"], st["ud"], st["th"], device=local)
               for st in states]
    prec = "fp64" if args.precision == "fp64" else "df64"
    E = EnsembleStep2D(members, precision=prec)
    step = 0
    for _ in range(warmup):
        E.step(step, E.time_steps(step, t_ref=1000.0))
        step += 1
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    nstat0 = len(E.stats)
    for _ in range(nsteps):
        E.step(step, E.time_steps(step, t_ref=1000.0))
        step += 1
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    nmem = len(members)
    stats = E.stats[nstat0:]
    iters = np.array([[st["iterations"] for st in rnd] for rnd in stats], dtype=np.float64)
    status = sorted(set(st["status"] for rnd in stats for st in rnd))
    status_counts = {}
    for rnd in stats:
        for st in rnd:
            status_counts[str(st["status"])] = status_counts.get(str(st["status"]), 0) + 1
    finished_alone = sum(1 for rnd in stats for st in rnd if st["fallback"] >= 256)
    relres_max = max(st["relres"] for rnd in stats for st in rnd)
    sizes = np.array([int(m.adv.inx) * int(m.adv.iny) for m in members], dtype=np.float64)
    # algorithmic bytes of the batched solves: 25 words per node and iteration (two
    # 5-word matvecs and the 15-word vector chain), 8 bytes each (FP64 or FP32 pair)
    alg = float((iters * sizes[None, :]).sum() * 25 * 8)
    peak, peak_kind = _peaks()
    line = {
        "metric": "ensemble time steps: projection solves/s (48 uneven members, batched)",
        "value": 2.0 * nmem * nsteps / (ms / 1000.0), "unit": "solves/s", "n_gpus": world, "steps": nsteps,
        "warmup": warmup, "ms_per_step": ms / nsteps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 state, %s solves" % prec, "data": "synthetic",
        "config": ens_steps_config(world),
        "member_steps_per_s": nmem * nsteps / (ms / 1000.0),
        "solver": {"iterations_mean_per_grid": {
            "%dx%d" % (int(m.adv.inx) - 1, int(m.adv.iny) - 1): float(iters[:, k].mean())
            for k, m in enumerate(members) if k % 16 == 0},
            "status": status, "status_counts": status_counts, "relres_max": relres_max,
            "finished_alone": finished_alone, "solves": int(iters.size)},
        "roofline": {"bound": "hbm", "achieved": alg / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / (ms / 1000.0) / 1e9 / peak, "traffic": None,
                     "kernel": "whole ensemble step (k_batch_bicgstab dominates)", "peak_source": peak_kind,
                     "what": "algorithmic bytes of the batched solves / step time (the step's other kernels "
                             "count as time, not bytes)"},
        "clocks": clk, "wall_s": wall, "gpu_launches": None,
    }
    if want_cpu:
        v, k = _cpu_step2d_sample(args.cpu_seconds)
        it_small = float(iters[:, :16].mean())
        work = float((iters.mean(axis=0) * sizes).sum()) / (it_small * sizes[0])
        line["cpu_baseline"] = {"value": 2.0 * v / work, "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": "%d steps of the oracle's time step on the 160x80 member (%.2f steps/s), "
                                          "scaled to the whole ensemble by nodes x solver iterations (%.1f x one "
                                          "160x80 member): extrapolated" % (k, v, work)}
    return line


def run_ensemble_steps(args):
    import torch
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    line = ensemble_steps_line(args, local, rank, world, args.steps, args.warmup,
                               want_cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if world > 1:
        t = torch.tensor([line["ms_per_step"]], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        line["ms_per_step"] = float(t.item())
        line["value"] = world * 2.0 * line["config"]["members"] / (line["ms_per_step"] / 1000.0)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_step3d(args):
    """``--workload step3d``: whole 3D time steps of the warm bubble (advection,
    explicit and implicit projection halves, background-preconditioned solves to
    1e-10) with the state resident on the GPU; value = steps/s.  Replicas under
    torchrun.  The reference cannot run a 3D step, so there is no CPU arm."""
    import torch
    from types import SimpleNamespace as NS
    from pybella_gb300 import workloads
    from pybella_gb300.time_update import DeviceStep3D
    world, rank, local = _dist()
    torch.cuda.set_device(local)
    nx, ny, nz = args.nx, args.ny, args.nz
    st = workloads.bubble_3d_state(nx, ny, nz, seed=11 + rank)
    run = DeviceStep3D(st["Sol"], st["mpv"], st["elem"], st["node"], st["ud"], st["th"], device=local,
                       preconditioner="background")
    dt = 0.02169
    for k in range(args.warmup):
        run.step(k, dt)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = ClockSampler(local)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.steps):
        run.step(args.warmup + k, dt)
    e1.record()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    if rank == 0:
        its = [s_["iterations"] for s_ in run.stats[-2 * args.steps:]]
        print(json.dumps({"metric": "3D time steps/s (warm bubble, projections to 1e-10)", "value": world * 1000.0 / ms,
                          "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64 state, f32/f64 solves", "data": "synthetic",
                          "config": {"workload": "3D time step %dx%dx%d nodes, rising-bubble background, "
                                                 "background-preconditioned projections" % (nx, ny, nz),
                                     "parallelism": "replicas" if world > 1 else "single GPU",
                                     "l2": "state of %.1f GB resident, larger than L2" % (
                                         6 * 8 * (nx + 2) * (ny + 2) * (nz + 2) / 1e9)},
                          "solve_iterations": its, "clocks": clocks, "cpu_baseline": None,
                          "gpu_launches": None}), flush=True)


def main():
    args = _args()
    if args.workload in ("learned3d", "step3d") and args.nx == NX and args.ny == NY:
        args.nx, args.ny = 257, 129
    if args.impl == "reference":
        if args.workload == "step2d":
            if _dist()[1] == 0:
                v, k = _cpu_step2d_sample(args.cpu_seconds)
                print(json.dumps({"impl": "reference", "metric": "2D time steps/s (rising bubble 160x80, "
                                  "projections to 1e-10)", "value": v, "unit": "steps/s", "n_gpus": 1,
                                  "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                                  "config": step2d_config(_dist()[0]),
                                  "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                                                   "sample": "%d steps of the oracle's time step" % k},
                                  "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}))
            return
        if args.workload == "ensemble_steps":
            if _dist()[1] == 0:
                v, k = _cpu_step2d_sample(args.cpu_seconds)
                # work of one ensemble step in 160x80 member-steps: nodes x solver iterations,
                # the iterations growing with the grid's linear size (231 / 460 / 950 measured)
                from pybella_gb300.workloads import ENSEMBLE_GRIDS
                work = 16.0 * sum((cx * cy) / (160.0 * 80.0) * (cx / 160.0) for cx, cy in ENSEMBLE_GRIDS)
                ref = 96.0 * v / work
                print(json.dumps({"impl": "reference", "metric": "ensemble time steps: projection solves/s "
                                  "(48 uneven members, batched)", "value": ref, "unit": "solves/s",
                                  "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                                  "config": ens_steps_config(_dist()[0]),
                                  "cpu_baseline": {"value": ref, "unit": "solves/s", "cores": 1,
                                                   "kind": "port",
                                                   "sample": "%d steps of the oracle's time step on a 160x80 member, "
                                                             "members run one after another (__main__.py:223-254); "
                                                             "one ensemble step is %.0f such steps (nodes x "
                                                             "iterations): extrapolated" % (k, work)},
                                  "e2e": {"value": ref, "unit": "solves/s",
                                          "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
            return
        if args.workload == "step3d":
            if _dist()[1] == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference's 3D time step cannot run "
                                  "(second_projection.py:183-203 use diag_inv and p2 unassigned)"}))
            return
        if args.workload == "learned3d":
            run_reference_3d(args)
        else:
            run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "learned3d":
        run_learned3d(args)
    elif args.workload == "step3d":
        run_step3d(args)
    elif args.workload == "step2d":
        run_step2d(args)
    elif args.workload == "ensemble_steps":
        run_ensemble_steps(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
