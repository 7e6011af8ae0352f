"""Throughput benchmark of the fused GB300 MHD step.

Workload (the configuration the headline metric is quoted on): 2D
Kelvin-Helmholtz shear layer, 4096 x 2048 interior cells, x periodic, y
zero-gradient walls, HLLD + minmod + GLM + TVD-RK2, CFL 0.4, FP64.  One step =
one full TVD-RK2 step (two fused stage kernels) over the whole grid.  The
state (605 MB) is larger than L2 (129 MB), so no L2 flush is needed between
steps.  Synthetic seeded initial data (no external dataset exists).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  --impl reference times the reference's own
CPU code on all host cores: its 2D_KH driver, translated mechanically from the
Fortran to C with its OpenMP directives (oracle/ref.py), at this grid from the
same seeded state; where that translation is absent, the C restatement of the
reference's path (the oracle port, OpenMP).  Multi-GPU runs are independent
replicas, one per GPU ("replicas only": the path has no exchange once one GPU
holds a grid).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY = 4096, 2048
WORKLOAD = "kh2d_4096x2048_hlld_minmod_glm_tvdrk2"


def headline_config(ws: int) -> dict:
    """The workload both arms (this library and the reference) run, in the same
    words: KH 4096x2048, HLLD + minmod + GLM + TVD-RK2, CFL 0.4, FP64."""
    return {"workload": WORKLOAD, "nx": NX, "ny": NY, "precision": "fp64", "cfl": 0.4,
            "l2": "state 605 MB > 129 MB L2: no flush needed", "parallelism": f"replicas{ws}"}


# Algorithmic cost of one 2D cell-update (both RK stages, GLM, CFL) is read
# from profiles/flops_kh2d.txt (flop-counting build of the oracle on this
# workload: add/sub/mul/div/sqrt/exp = 1 flop, min/max/abs/sign/compare = 0).
BYTES_PER_CELL_UPDATE_2D = 45 * 8  # stage 1: read U, write U1; stage 2: read U, U1, write U


def _load_flops(name: str = "flops_kh2d.txt"):
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        m = re.search(r"flops_per_cell_update:\s*([0-9.]+)", open(p).read())
        if m:
            return float(m.group(1))
    return 2100.0  # estimate until the counting build has run


def _load_flops_split(name: str):
    """(total, face-flux part, rest, u2v part of the rest) flops per cell-update
    from a profiles/ flop count: the face part (limiters, face fixes, Riemann
    solver, resistive face terms) is what the FP32-mixed kernels compute in
    FP32, the rest (u2v, CFL, GLM, RK update) their FP64 residual, except the
    u2v part, which they run in FP32 in cells whose internal energy is at least
    the kinetic plus magnetic energy."""
    p = os.path.join(ROOT, "profiles", name)
    txt = open(p).read()
    get = lambda k: float(re.search(k + r":\s*([0-9.]+)", txt).group(1))  # noqa: E731
    return (get("flops_per_cell_update"), get("face_flux_flops_per_cell_update"), get("rest_flops_per_cell_update"),
            get("u2v_flops_per_cell_update"))


def _u2v_fp64_share(states) -> float:
    """Share of the cells whose primitives the FP32-mixed kernels recover in
    FP64 (E < rho v^2 + B^2: the internal energy below the kinetic plus
    magnetic energy), over conserved states (9, ...) on the device."""
    n = low = 0
    for U in states:
        U = U.reshape(9, -1)
        rv2 = (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]) / U[4]
        B2 = U[5] * U[5] + U[6] * U[6] + U[7] * U[7]
        low += int((U[3] < rv2 + B2).sum())
        n += U.shape[1]
    return low / max(n, 1)


def _mixed_roofline(cells_per_s: float, split, fp64_peak_gflops: float, fp32_peak_gflops: float,
                    hbm_peak_gbs: float, bytes_per_cu: float = BYTES_PER_CELL_UPDATE_2D, u2v_fp64_share: float = 1.0):
    """Roofline of an FP32-mixed run: the time per cell-update is bounded by
    the slowest of its FP64 residual flops at the FP64 peak, its FP32 flops
    (face work, and the u2v of the cells recovered in FP32: 1 - u2v_fp64_share
    of them) at the FP32 peak and its bytes at the HBM peak.  `achieved`/`frac`
    are those of the binding resource (the FP64 residual on GB300, whose FP64
    pipe is 1/64 of its FP32 rate); `roof_frac` = roof time / measured time."""
    _, face, rest, u2v = split
    rest, face = rest - u2v * (1.0 - u2v_fp64_share), face + u2v * (1.0 - u2v_fp64_share)
    t64 = rest / (fp64_peak_gflops * 1e9)
    t32 = face / (fp32_peak_gflops * 1e9)
    tb = bytes_per_cu / (hbm_peak_gbs * 1e9)
    parts = {"fp64": (rest, fp64_peak_gflops / 1e3, t64, "TFLOP/s"), "fp32": (face, fp32_peak_gflops / 1e3, t32,
                                                                               "TFLOP/s"),
             "hbm": (bytes_per_cu, hbm_peak_gbs, tb, "GB/s")}
    bound = max(parts, key=lambda k: parts[k][2])
    out = {"bound": bound}
    for k, (per_cu, peak, troof, unit) in parts.items():
        ach = per_cu * cells_per_s / (1e12 if unit == "TFLOP/s" else 1e9)
        out[k] = {"per_cell_update": per_cu, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak}
    out["achieved"], out["peak"], out["unit"], out["frac"] = (out[bound]["achieved"], out[bound]["peak"],
                                                              out[bound]["unit"], out[bound]["frac"])
    out["roof_frac"] = max(t64, t32, tb) * cells_per_s
    out["u2v_fp64_share"] = u2v_fp64_share
    return out


def _fp64_roofline(cells_per_s: float, flops_cu: float, fp64_peak_gflops: float, hbm_peak_gbs: float,
                   bytes_per_cu: float = BYTES_PER_CELL_UPDATE_2D):
    ach = flops_cu * cells_per_s / 1e12
    hbm = bytes_per_cu * cells_per_s / 1e9
    return {"bound": "fp64", "achieved": ach, "peak": fp64_peak_gflops / 1e3, "unit": "TFLOP/s",
            "frac": ach / (fp64_peak_gflops / 1e3), "flops_per_cell_update": flops_cu,
            "hbm": {"achieved": hbm, "peak": hbm_peak_gbs, "unit": "GB/s", "frac": hbm / hbm_peak_gbs}}


def _errors(a, b):
    """Per-variable error of state a against b ((9, ...) numpy arrays or torch
    tensors; tensors are reduced on their device): scaled L1
    (openmhd_gb300.metrics.scaled_l1), relative L1 against each variable's own
    norm, and the max norm; plus the largest own-norm error over the variables
    that hold at least 1e-4 of their physical scale."""
    import numpy as np
    import torch

    from openmhd_gb300.metrics import VAR_NAMES

    if isinstance(a, np.ndarray):
        a, b = torch.from_numpy(np.ascontiguousarray(a)), torch.from_numpy(np.ascontiguousarray(b))
    a = a.reshape(9, -1)
    b = b.reshape(9, -1)
    num = torch.stack([(a[v] - b[v]).abs().sum() for v in range(9)])
    li = torch.stack([(a[v] - b[v]).abs().max() for v in range(9)])
    norm = torch.stack([b[v].abs().sum() for v in range(9)])
    m = torch.sqrt((2.0 * b[4] * b[3]).abs()).sum()
    B = torch.sqrt(b[5] * b[5] + b[6] * b[6] + b[7] * b[7]).sum()
    scale = torch.stack([m, m, m, norm[3], norm[4], B, B, B, B])
    num, li, norm, scale = (x.double().cpu().numpy() for x in (num, li, norm, scale))
    floor = max(scale.max(), 1e-300) * 1e-12
    sc = num / np.maximum(scale, floor)
    own = np.where(norm > 0, num / np.where(norm > 0, norm, 1.0), num)
    sig = norm >= 1e-4 * scale
    return {"scaled_l1": dict(zip(VAR_NAMES, map(float, sc))),
            "own_norm_rel_l1": dict(zip(VAR_NAMES, map(float, own))),
            "linf": dict(zip(VAR_NAMES, map(float, li))),
            "max_scaled_l1": float(sc.max()),
            "max_own_norm_rel_l1_significant": float(own[sig].max()) if sig.any() else 0.0,
            "max_own_norm_var": VAR_NAMES[int(np.argmax(np.where(sig, own, -1.0)))] if sig.any() else None,
            "significant_vars": [v for v, g in zip(VAR_NAMES, sig) if g]}


def _load_traffic(name: str):
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(p).read())
        if m:
            return float(m.group(1))
    return None


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id: str | None):
        self.dev = device_id
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.dev:
            cmd += ["-i", self.dev]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate(per_rank_seconds: list[float], cells_per_rank: int, steps: int) -> tuple[float, float]:
    """Whole-job throughput of independent replicas: all ranks' cell-updates
    divided by the slowest rank's time (max over ranks)."""
    t = max(per_rank_seconds)
    return len(per_rank_seconds) * cells_per_rank * steps / t, t


def cpu_baseline(steps_budget_s: float = 12.0, omp: bool = True, nx: int = NX, ny: int = NY, min_steps: int = 5):
    """Oracle (C restatement of the reference's serial path) on the host cores,
    same KH workload: at least `min_steps` timed steps, then more until about
    `steps_budget_s` of CPU time has passed (at most 50)."""
    from oracle import oracle
    from openmhd_gb300 import kelvin_helmholtz

    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cfg, model = kelvin_helmholtz(nx, ny, precision="fp64")
    g = oracle.Grid.from_solver_config(cfg, omp=omp)
    g.model(model.kind, amp=model.amp, bx0=model.bx0, pert=model.pert, seed=model.seed)
    g.step(1)  # warm-up (page-in)
    done, t0 = 0, time.perf_counter()
    while True:
        g.step(1)
        done += 1
        el = time.perf_counter() - t0
        if (el >= steps_budget_s and done >= min_steps) or done >= 50:
            break
    cells = (nx * ny)
    return {"value": cells * done / el, "unit": "cell-updates/s", "cores": int(os.environ["OMP_NUM_THREADS"]) if omp else 1,
            "kind": "port", "sample": f"{done} steps of KH {nx}x{ny} after 1 warm-up step ({el:.1f} s)"}, el / done


def _omp_threads(n: int) -> None:
    """Set the OpenMP thread count of this process's OpenMP runtime (shared by
    the oracle's and the reference translation's libraries)."""
    import ctypes as C

    try:
        C.CDLL("libgomp.so.1").omp_set_num_threads(int(n))
    except OSError:
        pass


def reference_cpu(threads: int, budget_s: float = 12.0, nx: int = NX, ny: int = NY):
    """The reference's own CPU implementation on the host cores: its 2D_KH
    driver (2D_KH/main.f90 with u2v, limiter, flux_solver, rk, glm_ss2, set_dt
    and its bc.f90 walls), translated mechanically to C with the reference's
    OpenMP directives (oracle/ref.py), at the configuration's grid, started
    from the configuration's seeded KH state instead of 2D_KH/model.f90.  The
    reference assumes dy = dx, so its y spacing is the x spacing here: the same
    work per cell-update on a squeezed domain.  Timed as the difference of two
    runs of the driver (2 and 2 + K steps: the first two steps, which touch the
    work arrays first, cancel).  Returns None when the translation is absent."""
    from oracle import oracle, ref

    if not ref.buildable():
        return None
    ref.build("2D_KH")
    from openmhd_gb300 import kelvin_helmholtz

    cfg, model = kelvin_helmholtz(nx, ny, precision="fp64")
    g = oracle.Grid.from_solver_config(cfg)
    g.model(model.kind, amp=model.amp, bx0=model.bx0, pert=model.pert, seed=model.seed)
    ref.set_initial_2d("2D_KH", g.U, g.x, g.y, cfg.dx)
    del g
    _omp_threads(threads)
    run = dict(ix=cfg.ix, jx=cfg.jx, tend=1e30, dtout=1e30, cfl=cfg.cfl, lm_type=1, flux_type=3, time_type=0)

    def timed(nsteps):
        t0 = time.perf_counter()
        st, _ = ref.run_main("2D_KH", loop_max=nsteps + 1, **run)
        if st:
            raise RuntimeError(f"the reference driver stopped (line {st})")
        return time.perf_counter() - t0

    t2 = timed(2)
    t3 = timed(3)
    per_step = max(t3 - t2, 1e-9)
    k = int(min(30, max(3, budget_s / per_step)))
    tk = timed(2 + k)
    el = tk - t2
    ref.set_initial_2d("2D_KH")
    _omp_threads(os.cpu_count() or 1)
    return {"value": nx * ny * k / el, "unit": "cell-updates/s", "cores": threads, "kind": "reference",
            "sample": f"{k} steps of the reference's 2D_KH driver (translated to C, OpenMP, {threads} threads) at "
                      f"{nx}x{ny} from the configuration's KH state, after 2 warm-up steps ({el:.1f} s)"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    base = reference_cpu(cores, budget_s=min(60.0, max(8.0, 4.0 * args.steps)))
    if base is None:  # no translation of the reference here: the oracle port on all cores
        base, _ = cpu_baseline(steps_budget_s=min(60.0, max(8.0, 4.0 * args.steps)))
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": base["value"], "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(ws),
        "note": "the reference is Fortran (no compiler here or on the box): its own source translated "
                "mechanically to C (oracle/ref.py), OpenMP, timed on rank 0; else the C restatement",
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _leg(fn, *a):
    """One of the further legs of the bench line.  A leg that raises is
    reported under its own key as {"error": ...}; the headline figures, measured
    before it, still print."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- any failure of a leg is reported, not hidden
        return {"error": f"{type(e).__name__}: {e}"}


def run_ours(args):
    import numpy as np
    import torch

    from openmhd_gb300 import Solver, kelvin_helmholtz
    from openmhd_gb300 import _lib

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    props = torch.cuda.get_device_properties(dev)
    uuid = None
    try:
        uuid = "GPU-" + str(props.uuid)
    except Exception:
        pass

    cfg, model = kelvin_helmholtz(NX, NY, precision="fp64")
    cells = cfg.interior_cells
    s = Solver(cfg).init_model(model)
    s.step(args.warmup)
    s.sync()

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed FP64 run ----
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(uuid) as clk:
        e0.record(s.stream)
        s.step(args.steps)
        e1.record(s.stream)
        e1.synchronize()
    info = s.sync()
    if info.status != 0 or info.steps != args.warmup + args.steps:
        raise RuntimeError(f"solver failed: status {info.status} steps {info.steps}")
    t_fp64 = e0.elapsed_time(e1) / 1e3
    barrier()
    if ws > 1:
        import torch.distributed as dist

        tt = torch.tensor([t_fp64], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_fp64 = float(tt.item())
    value = ws * cells * args.steps / t_fp64
    U64 = s.get_state_numpy()
    div_b = _div_b_max(s.U, cfg.dx, cfg.dy)

    # ---- FP32-mixed on the same workload (same warm-up + steps) ----
    cfgm, _ = kelvin_helmholtz(NX, NY, precision="mixed")
    m = Solver(cfgm).init_model(model)
    m.step(args.warmup)
    m.sync()
    barrier()
    e0.record(m.stream)
    m.step(args.steps)
    e1.record(m.stream)
    e1.synchronize()
    im = m.sync()
    t_mx = e0.elapsed_time(e1) / 1e3
    Um = m.get_state_numpy()
    mixed_err = _errors(Um[:, 1:-1, 1:-1], U64[:, 1:-1, 1:-1])
    mixed_share = _u2v_fp64_share([m.U[:, 1:-1, 1:-1]])
    del m

    # ---- end to end through the C ABI with host buffers ----
    lib = _lib.load()
    h = s._h
    host = torch.empty(cfg.shape, dtype=torch.float64).pin_memory()
    host.copy_(torch.from_numpy(U64))
    nbytes = host.numel() * 8
    ke2e = max(3, min(args.steps, 20))
    # one call per step: host state in, one step, host state out
    # (omhd_solver_step_host; page-locked buffer, so the upload and the first
    # dt share one pass and the step writes its result straight to the buffer)
    if lib.omhd_solver_step_host(h, host.data_ptr(), host.data_ptr(), 0.0, 1):
        raise RuntimeError("e2e call failed")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke2e):
        if lib.omhd_solver_step_host(h, host.data_ptr(), host.data_ptr(), 0.0, 1):
            raise RuntimeError("e2e call failed")
    t_e2e = time.perf_counter() - t0
    # the same through the separate put_state / step / get_state copies
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke2e):
        st1 = lib.omhd_solver_put_state(h, host.data_ptr(), 0.0)
        st2 = lib.omhd_solver_step(h, 1)
        st3 = lib.omhd_solver_get_state(h, host.data_ptr())
        if st1 or st2 or st3:
            raise RuntimeError("e2e call failed")
    t_e2e_copies = time.perf_counter() - t0
    e2e = {"value": ws * cells * ke2e / t_e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "steps": ke2e,
           "path": "omhd_solver_step_host(host pinned U in / out, 1 step)",
           "copies_path_value": ws * cells * ke2e / t_e2e_copies,
           "copies_path": "omhd_solver_put_state + omhd_solver_step(1) + omhd_solver_get_state, same buffer"}

    peaks, peak_src = _peaks()
    flops_cu = _load_flops()
    fp64_peak = _fp64_peak_gflops(lib)
    fp32_peak = _fp32_peak_gflops(lib)
    launch_s = t_fp64 / (2 * args.steps)  # two stage launches per step, nothing else in the region
    ach_tflops = flops_cu * cells / 2 / launch_s / 1e12
    hbm_gbs = BYTES_PER_CELL_UPDATE_2D * cells / (t_fp64 / args.steps) / 1e9
    roofline = {
        "bound": "fp64", "achieved": ach_tflops, "peak": fp64_peak / 1e3, "unit": "TFLOP/s",
        "frac": ach_tflops / (fp64_peak / 1e3),
        "traffic": _load_traffic("stage2d_fp64_kh4096x2048.md"),
        "peak_source": "DFMA burst throughput measured in this run (omhd_probe_fp64_peak: register "
                       "operands, best of five launches; nominal 1.25 TFLOP/s); MEASURED_PEAKS.json has no "
                       "FP64 entry",
        "flops_per_cell_update": flops_cu,
        "kernel": "omhd::v_fp64::k_stage2d_pipe<HLLD,tape-capable,3 producer warps>",
        "hbm": {"achieved": hbm_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": hbm_gbs / peaks.get("hbm_gbs", 1.0), "peak_source": peak_src,
                "bytes_per_cell_update": BYTES_PER_CELL_UPDATE_2D},
    }
    line = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_fp64 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded KH initial state)",
        "config": headline_config(ws),
        "roofline": roofline,
        "gpu_launches": 2 * args.steps,
        "max_div_b": div_b,
        "e2e": e2e,
        "clocks": clk.summary(),
        "mixed": {"value": ws * cells * args.steps / t_mx, "speedup_vs_fp64": t_fp64 / t_mx,
                  "roofline": _mixed_roofline(cells * args.steps / t_mx, _load_flops_split("flops_kh2d.txt"),
                                              fp64_peak, fp32_peak, peaks.get("hbm_gbs", 6800.0),
                                              u2v_fp64_share=mixed_share),
                  "error_vs_fp64": mixed_err, "status": im.status,
                  "steps_compared": args.warmup + args.steps},
        "peaks_in_run": {"fp64_gflops": fp64_peak, "fp32_gflops": fp32_peak,
                         "source": "omhd_probe_fp64_peak / omhd_probe_fp32_peak (FMA chains in registers, best "
                                   "of five launches); HBM from MEASURED_PEAKS.json"},
    }
    if not args.no_batched:
        line["batched"] = _leg(run_batched, args, fp64_peak, fp32_peak)
    if not args.no_adjoint:
        line["adjoint"] = _leg(run_adjoint, args)
    if not args.no_3d:
        line["harris3d"] = _leg(run_3d, args, fp64_peak, fp32_peak)
    if not args.no_sq:
        line["ot4096sq"] = _leg(run_sq4096, args, fp64_peak)
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        base = _leg(lambda: reference_cpu(cores, budget_s=10.0))
        if base is None or "error" in base:  # the oracle port, where the translation is absent
            if base is not None:
                line["reference_cpu_error"] = base["error"]
            base = _leg(lambda: cpu_baseline(steps_budget_s=10.0)[0])
            if "error" not in base:  # the same oracle on one core, beside the all-core figure
                base["serial"] = _leg(lambda: cpu_baseline(steps_budget_s=4.0, omp=False)[0])
        else:  # the reference on one core, and the oracle port beside it
            base["serial"] = _leg(lambda: reference_cpu(1, budget_s=12.0))
            base["port"] = _leg(lambda: cpu_baseline(steps_budget_s=6.0)[0])
        line["cpu_baseline"] = base
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def _member_summary(i: int, own_vars: list, cfgs: list, models: list) -> dict:
    """Which ensemble member, model, grid (with ghosts) and variable an error
    figure belongs to."""
    return {"member": i, "var": own_vars[i],
            "model": {0: "orszag_tang", 1: "kelvin_helmholtz"}.get(models[i].kind, str(models[i].kind)),
            "ix": cfgs[i].ix, "jx": cfgs[i].jx}


def run_batched(args, fp64_peak: float = float("nan"), fp32_peak: float = float("nan")):
    """128-member ensemble (seeded sizes in {128..1024}^2, half OT, half KH),
    FP32-mixed, one persistent batched kernel per RK stage, autotuned tiling,
    K steps replayed as one CUDA graph.  Every member runs 500 steps in all;
    the per-member error is against the same ensemble run in FP64 for the
    same 500 steps, whose K-step time (its own autotuned tiling, stream
    launches) is the FP64 batched throughput."""
    import numpy as np
    import torch

    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(128, seed=0, precision="mixed")
    ens = Ensemble(cfgs).init_models(models)
    kind, cps, ms_tune = ens.autotune(steps=2)
    tuned_steps = 0  # the autotuner restores the ensemble state after timing each candidate
    ens.step_graph(args.steps, replays=1)  # capture + first replay (warm)
    before = ens.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ens.stream)
    ens.step_graph(args.steps, replays=1)
    e1.record(ens.stream)
    e1.synchronize()
    infos = ens.sync()
    t = e0.elapsed_time(e1) / 1e3
    # cell-updates actually made: a member that reaches its end time stops
    # (its tiles are skipped), so only the steps each member took count
    cells_m = [c.interior_cells for c in cfgs]
    updates = sum(n * (a.steps - b.steps) for n, a, b in zip(cells_m, infos, before))
    active = sum(1 for a, b in zip(infos, before) if a.steps - b.steps == args.steps)
    # every member runs BATCH_STEPS steps in all; the error is taken there
    rest = BATCH_STEPS - tuned_steps - 2 * args.steps
    if rest > 0:
        ens.step(rest)
        infos = ens.sync()
    total_steps = max(BATCH_STEPS, tuned_steps + 2 * args.steps)
    cfg64, _ = batched_problem_set(128, seed=0, precision="fp64")
    ref = Ensemble(cfg64).init_models(models)
    kind64, cps64, _ = ref.autotune(steps=2)  # the FP64 ensemble's own best tiling
    ref.step(3)
    before64 = ref.sync()
    e0.record(ref.stream)
    ref.step(args.steps)
    e1.record(ref.stream)
    e1.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3
    updates64 = sum(n * (a.steps - b.steps) for n, a, b in zip(cells_m, ref.sync(), before64))
    ref.step(total_steps - 3 - args.steps)
    ref.sync()
    errs, owns, own_vars, lis = [], [], [], []
    low = cnt = 0.0
    for i in range(len(cfgs)):
        Ui = ens.member_state(i)[:, 1:-1, 1:-1]
        low += _u2v_fp64_share([Ui]) * Ui[0].size
        cnt += Ui[0].size
        e = _errors(Ui, ref.member_state(i)[:, 1:-1, 1:-1])
        errs.append(e["max_scaled_l1"])
        owns.append(e["max_own_norm_rel_l1_significant"])
        own_vars.append(e["max_own_norm_var"])
        lis.append(max(e["linf"].values()))
    del ref
    batch_share = low / max(cnt, 1.0)
    peaks, _ = _peaks()
    split = _load_flops_split("flops_ensemble2d.txt")
    return {"value": updates / t, "unit": "cell-updates/s", "members": len(cfgs),
            "roofline": _mixed_roofline(updates / t, split, fp64_peak, fp32_peak, peaks.get("hbm_gbs", 6800.0),
                                        u2v_fp64_share=batch_share),
            "fp64_roofline": _fp64_roofline(updates64 / t64, split[0], fp64_peak, peaks.get("hbm_gbs", 6800.0)),
            "max_member_own_norm_rel_l1_vs_fp64": max(owns),
            "median_member_own_norm_rel_l1_vs_fp64": float(np.median(owns)),
            "members_own_norm_within_1e-6": int(sum(o <= 1e-6 for o in owns)),
            "worst_member_own_norm": _member_summary(int(np.argmax(owns)), own_vars, cfgs, models),
            "members_scaled_within_1e-6": int(sum(x <= 1e-6 for x in errs)),
            "max_member_linf_vs_fp64": max(lis),
            "members_stepping_throughout": active,
            "fp64_batched_value": updates64 / t64, "speedup_vs_fp64_batched": (updates / t) / (updates64 / t64),
            "fp64_tile": ["32x8", "32x4", "16x16", "64x4", "16x8"][kind64], "fp64_ctas_per_sm": cps64,
            "cells": ens.cells, "precision": "mixed", "tile_kind": kind, "ctas_per_sm": cps,
            "tile": ["32x8", "32x4", "16x16", "64x4", "16x8"][kind], "ms_per_step": 1e3 * t / args.steps,
            "steps_compared": total_steps, "max_member_scaled_l1_vs_fp64": max(errs),
            "worst_member": int(np.argmax(errs)),
            "median_member_scaled_l1_vs_fp64": float(np.median(errs)),
            "dt_range": [min(x.dt for x in infos), max(x.dt for x in infos)]}


def run_sq4096(args, fp64_peak_gflops: float):
    """Orszag-Tang 4096 x 4096 (HLLD + MC + GLM + TVD-RK2, periodic), FP64: the
    square grid the FP64 roofline target is stated on.  Throughput and the
    fraction of the FP64 DFMA peak from the flop count of this workload
    (profiles/flops_ot2d_4096x4096.txt); the state (1.21 GB) is larger than L2."""
    import torch

    from openmhd_gb300 import Solver, orszag_tang

    steps = max(3, min(args.steps, 20))
    warm = 3
    cfg, model = orszag_tang(4096, precision="fp64")
    s = Solver(cfg).init_model(model)
    s.step(warm)
    s.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s.stream)
    s.step(steps)
    e1.record(s.stream)
    e1.synchronize()
    info = s.sync()
    t = e0.elapsed_time(e1) / 1e3
    cells = cfg.interior_cells
    flops_cu = _load_flops("flops_ot2d_4096x4096.txt")
    ach = flops_cu * cells * steps / t / 1e12
    out = {"workload": "ot2d_4096x4096_hlld_mc_glm_tvdrk2", "steps": steps, "warmup": warm,
           "value": cells * steps / t, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / steps,
           "status": info.status, "steps_done": info.steps,
           "roofline": {"bound": "fp64", "achieved": ach, "peak": fp64_peak_gflops / 1e3, "unit": "TFLOP/s",
                        "frac": ach / (fp64_peak_gflops / 1e3), "flops_per_cell_update": flops_cu,
                        "timing": "whole step (both stage launches and the step planning)"}}
    del s
    torch.cuda.empty_cache()
    return out


H3_NX, H3_NY, H3_NZ = 512, 256, 512


def _div_b_max(U, dx, dy, dz=None):
    """max |div B| over the interior, centred differences (the reference's
    diagnostic form; GLM keeps it bounded rather than zero)."""
    if U.dim() == 3:
        d = (U[5, 1:-1, 2:] - U[5, 1:-1, :-2]) / (2 * dx) + (U[6, 2:, 1:-1] - U[6, :-2, 1:-1]) / (2 * dy)
    else:
        d = ((U[5, 1:-1, 1:-1, 2:] - U[5, 1:-1, 1:-1, :-2]) / (2 * dx)
             + (U[6, 1:-1, 2:, 1:-1] - U[6, 1:-1, :-2, 1:-1]) / (2 * dy)
             + (U[7, 2:, 1:-1, 1:-1] - U[7, :-2, 1:-1, 1:-1]) / (2 * dz))
    return float(d.abs().max())


def run_3d(args, fp64_peak: float = float("nan"), fp32_peak: float = float("nan")):
    """3D resistive Harris sheet 512 x 256 x 512 (x, y periodic, z conducting
    walls, HLLD + MC + GLM + resistive fluxes), FP64 and FP32-mixed on the
    same steps: cell-updates/s, HBM GB/s against the 360 B per cell-update of
    the fused two-stage design, and the mixed path's error against FP64."""
    import torch

    from openmhd_gb300 import Solver, harris3d

    steps = max(3, min(args.steps, 20))
    warm = 2
    out = {"workload": f"harris3d_{H3_NX}x{H3_NY}x{H3_NZ}_hlld_mc_glm_resistive_tvdrk2", "steps": steps,
           "warmup": warm}
    states = {}
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    peaks, peak_src = _peaks()
    for prec in ("fp64", "mixed"):
        cfg, model = harris3d(H3_NX, H3_NY, H3_NZ, precision=prec)
        s = Solver(cfg).init_model(model)
        s.step(warm)
        s.sync()
        torch.cuda.synchronize()
        e0.record(s.stream)
        s.step(steps)
        e1.record(s.stream)
        e1.synchronize()
        info = s.sync()
        t = e0.elapsed_time(e1) / 1e3
        cells = cfg.interior_cells
        gbs = BYTES_PER_CELL_UPDATE_2D * cells * steps / t / 1e9
        out[prec] = {"value": cells * steps / t, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / steps,
                     "hbm_gbs_algorithmic": gbs, "hbm_frac": gbs / peaks.get("hbm_gbs", 1.0),
                     "hbm_peak_source": peak_src, "status": info.status, "launches_per_step": 2}
        split = _load_flops_split("flops_harris3d.txt")
        if prec == "fp64":
            out[prec]["max_div_b"] = _div_b_max(s.U, cfg.dx, cfg.dy, cfg.dz)
            out[prec]["roofline"] = _fp64_roofline(cells * steps / t, split[0], fp64_peak, peaks.get("hbm_gbs", 6800.0))
        else:
            out[prec]["roofline"] = _mixed_roofline(cells * steps / t, split, fp64_peak, fp32_peak,
                                                    peaks.get("hbm_gbs", 6800.0),
                                                    u2v_fp64_share=_u2v_fp64_share([s.U[:, 1:-1, 1:-1, 1:-1]]))
        states[prec] = s
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["mixed"]["error_vs_fp64"] = _errors(states["mixed"].U[:, 1:-1, 1:-1, 1:-1], states["fp64"].U[:, 1:-1, 1:-1, 1:-1])
    out["mixed"]["steps_compared"] = warm + steps
    del states
    torch.cuda.empty_cache()
    return out


ADJ_NX, ADJ_NY, ADJ_STEPS, ADJ_EVERY = 512, 256, 400, 20
BATCH_STEPS = 500  # steps every ensemble member runs (the error is taken there)


def run_adjoint(args, ndir: int = 16, eps: float = 1e-6):
    """Gradient through time: KH 512 x 256 FP64, 400 TVD-RK2 steps (HLLD +
    minmod + GLM), J = sum By^2 at the final time, dJ/dvy0 over the full
    interior vy0 field through the hand-written adjoint kernels behind a
    torch.autograd.Function, checkpoint every 20 steps.  Reports forward and
    backward time, the time of one adjoint step against one forward step,
    device memory, and central finite differences of J (eps = 1e-6) along
    seeded random directions."""
    import numpy as np
    import torch

    from openmhd_gb300 import Solver, kelvin_helmholtz
    from openmhd_gb300.adjoint import AdjointRun, Evolve, kh_state

    cfg, model = kelvin_helmholtz(ADJ_NX, ADJ_NY, precision="fp64")
    s = Solver(cfg).init_model(model)
    base = s.U.clone()
    torch.cuda.synchronize()
    run = AdjointRun(cfg, ADJ_STEPS, ADJ_EVERY)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(stream, fn):
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    # plain forward: the fused solver alone (warm once)
    s.step(3)
    s.sync()
    s.put_state(base)
    t_fwd = timed(s.stream, lambda: s.step(ADJ_STEPS))
    s.sync()

    def objective(vy):
        UN = Evolve.apply(kh_state(base, vy), run)
        return (UN[6, 1:-1, 1:-1] ** 2).sum()

    vy0 = (base[1, 1:-1, 1:-1] / base[4, 1:-1, 1:-1]).clone()
    vy = vy0.clone().requires_grad_(True)
    J = objective(vy)  # warm-up forward + backward
    J.backward()
    torch.cuda.reset_peak_memory_stats()
    vy = vy0.clone().requires_grad_(True)
    U0 = kh_state(base, vy)
    UN_holder = {}
    t_fwd_ck = timed(run.stream, lambda: UN_holder.update(UN=Evolve.apply(U0, run)))
    J = (UN_holder["UN"][6, 1:-1, 1:-1] ** 2).sum()
    t_bwd = timed(run.stream, lambda: J.backward())
    run.sync()
    grad = vy.grad.detach().clone()
    peak_torch = torch.cuda.max_memory_allocated()

    # one adjoint step against one forward step, on stored stage inputs
    s.put_state(base)
    s.step(5)
    s.sync()
    Un = s.U.clone()
    s.step(1)
    s.sync()
    U1 = s.U1.clone()
    log3 = torch.tensor(run.step_log()[5], dtype=torch.float64, device="cuda")
    lam = torch.randn(cfg.shape, dtype=torch.float64, device="cuda")
    lam_out = torch.empty_like(lam)
    reps = 50
    run.step_vjp(Un, U1, log3, lam.clone(), lam_out)
    t_vjp = timed(run.stream, lambda: [run.step_vjp(Un, U1, log3, lam, lam_out) for _ in range(reps)]) / reps
    t_step = timed(s.stream, lambda: s.step(reps)) / reps

    # central finite differences (eps = 1e-6) along seeded random directions
    # of the full vy0 field.  The scheme is piecewise smooth: limiter
    # selections and HLLD branches switch at kinks, and KH's uniform far
    # field (rho, p, Bx exactly constant) sits on minmod kinks that any +-eps
    # straddles, so plain differences of J are not derivatives there.  The
    # check therefore differences the forward with the base run's decisions
    # frozen (record once, replay +-eps): the smooth map the adjoint is the
    # derivative of.  Plain differences are reported beside it.
    gen = torch.Generator(device="cuda").manual_seed(1234)
    with torch.no_grad():
        run.record(kh_state(base, vy0))

        def frozen(v):
            return float((run.replay(kh_state(base, v))[6, 1:-1, 1:-1] ** 2).sum())

        frozen_err, plain_err, samples = [], [], []
        for k in range(ndir):
            d = torch.randn(tuple(vy0.shape), dtype=torch.float64, device="cuda", generator=gen)
            ad = float((grad * d).sum())
            fdf = (frozen(vy0 + eps * d) - frozen(vy0 - eps * d)) / (2 * eps)
            fdp = (float(objective(vy0 + eps * d)) - float(objective(vy0 - eps * d))) / (2 * eps)
            frozen_err.append(abs(fdf - ad) / max(abs(fdf), 1e-300))
            plain_err.append(abs(fdp - ad) / max(abs(fdp), 1e-300))
            if k < 3:
                samples.append({"adjoint": ad, "fd_frozen": fdf, "fd_plain": fdp})
        # step-size sweep on the first directions: rounding noise of the
        # 400-step trajectories falls as 1/eps, truncation grows as eps^2
        gen2 = torch.Generator(device="cuda").manual_seed(1234)
        sweep = {}
        for k in range(4):
            d = torch.randn(tuple(vy0.shape), dtype=torch.float64, device="cuda", generator=gen2)
            ad = float((grad * d).sum())
            for e in (1e-4, 1e-5, 1e-6, 1e-7):
                fdf = (frozen(vy0 + e * d) - frozen(vy0 - e * d)) / (2 * e)
                sweep.setdefault(f"{e:g}", []).append(abs(fdf - ad) / max(abs(fdf), 1e-300))
    run.sync()
    fd_report = {"eps": eps, "directions": ndir, "direction_kind": "seeded N(0,1) per interior cell",
                 "eps_sweep_max_rel_err_4dirs": {k: max(v) for k, v in sweep.items()},
                 "max_rel_err": max(frozen_err), "median_rel_err": float(np.median(frozen_err)),
                 "kind": "frozen decisions (omhd_adjoint_record / omhd_adjoint_replay)",
                 "plain_fd_max_rel_err": max(plain_err), "plain_fd_median_rel_err": float(np.median(plain_err)),
                 "samples": samples}
    return {
        "workload": f"kh2d_{ADJ_NX}x{ADJ_NY}_fp64_{ADJ_STEPS}steps_adjoint_J=sum(By^2)_d/dvy0",
        "steps": ADJ_STEPS, "checkpoint_every": ADJ_EVERY, "J": float(J.detach()),
        "forward_s": t_fwd, "forward_with_checkpoints_s": t_fwd_ck, "backward_s": t_bwd,
        "backward_over_forward": t_bwd / t_fwd,
        "adjoint_step_ms": 1e3 * t_vjp, "forward_step_ms": 1e3 * t_step,
        "adjoint_step_over_forward_step": t_vjp / t_step,
        "adjoint_launches_per_step": 6,
        "device_bytes_adjoint_handle": run.memory_bytes, "device_bytes_torch_peak": int(peak_torch),
        "state_bytes": 9 * cfg.ix * cfg.jx * 8,
        "fd": fd_report,
        "grad_norm": float(grad.norm()),
    }


def run_accuracy(args):
    """Error of the FP32-mixed path against the FP64 path over long runs (not
    a throughput measurement): KH 4096 x 2048 (HLLD + minmod + GLM) for
    --accuracy-steps steps (the configuration's 2000 by default) and the
    resistive Harris sheet 512 x 256 x 512 (HLLD + MC + GLM) for
    --accuracy-steps-3d steps, both solvers from the same initial state; the
    per-variable scaled L1, own-norm relative L1 and max-norm errors at a few
    step counts along the way, computed on the device."""
    import torch

    from openmhd_gb300 import Solver, harris3d, kelvin_helmholtz

    def curve(make, total, marks, pair=("fp64", "mixed")):
        cfg64, model = make(pair[0])
        cfgmx, _ = make(pair[1])
        a = Solver(cfg64).init_model(model)
        b = Solver(cfgmx).init_model(model)
        sl = (slice(None),) + (slice(1, -1),) * (a.U.dim() - 1)
        out, done = [], 0
        for mk in marks:
            if mk > total:
                break
            a.step(mk - done)
            b.step(mk - done)
            ia, ib = a.sync(), b.sync()
            done = mk
            if ia.status or ib.status:
                out.append({"steps": mk, "status": [ia.status, ib.status]})
                break
            e = _errors(b.U[sl], a.U[sl])
            e.update({"steps": mk, "t_fp64": ia.t, "t_mixed": ib.t})
            out.append(e)
        del a, b
        torch.cuda.empty_cache()
        return out

    marks2 = sorted({10, 100, 500, 1000, args.accuracy_steps})
    marks3 = sorted({10, 100, 300, max(args.accuracy_steps_3d, 1)})
    kh = lambda p: kelvin_helmholtz(NX, NY, precision=p)  # noqa: E731
    h3 = lambda p: harris3d(H3_NX, H3_NY, H3_NZ, precision=p)  # noqa: E731
    res = {"accuracy": {"kh2d_4096x2048": curve(kh, args.accuracy_steps, marks2)}}
    if args.accuracy_steps_3d > 0:  # 0 skips the 3D run
        res["accuracy"]["harris3d_512x256x512"] = curve(h3, args.accuracy_steps_3d, marks3)
    if args.accuracy_control:
        # control: the FP64 build against the FP64 build without multiply-add
        # contraction, i.e. how far round-off alone (1e-16 per operation) is
        # carried by the flow over the same steps
        res["accuracy"]["control_kh2d_fp64_vs_fp64_parity"] = curve(kh, args.accuracy_steps, marks2,
                                                                    ("fp64_parity", "fp64"))
        if args.accuracy_steps_3d > 0:
            res["accuracy"]["control_harris3d_fp64_vs_fp64_parity"] = curve(
                h3, min(args.accuracy_steps_3d, 300), sorted({10, 100, 300}), ("fp64_parity", "fp64"))
    res["accuracy"]["ensemble_worst_members"] = _ensemble_worst_members(curve, args.accuracy_control)
    print(json.dumps(res), flush=True)
    return 0


def _ensemble_worst_members(curve, control: bool, nworst: int = 3):
    """The batched configuration's members with the largest FP32-mixed error
    against FP64 after its 500 steps (both ensembles in one batched launch per
    stage with the autotuned tiling, as the bench's batched leg runs them),
    then each of those members alone: its error curve, and with control=True
    the same member in FP64 against FP64 without multiply-add contraction
    (round-off growth)."""
    import numpy as np
    import torch

    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(128, seed=0, precision="mixed")
    cfg64, _ = batched_problem_set(128, seed=0, precision="fp64")
    mx = Ensemble(cfgs).init_models(models)
    r64 = Ensemble(cfg64).init_models(models)
    kind, cps, _ = mx.autotune(steps=2)  # the tiling the batched leg runs (the tuner restores the state)
    r64.set_tiling(kind, cps)
    mx.step(BATCH_STEPS)
    r64.step(BATCH_STEPS)
    mx.sync()
    r64.sync()
    errs = [_errors(mx.member_state(i)[:, 1:-1, 1:-1], r64.member_state(i)[:, 1:-1, 1:-1])["max_scaled_l1"]
            for i in range(len(cfgs))]
    del mx, r64
    torch.cuda.empty_cache()
    out = []
    marks = sorted({10, 100, BATCH_STEPS})
    for i in [int(k) for k in np.argsort(errs)[::-1][:nworst]]:
        make = lambda p, i=i: (batched_problem_set(128, seed=0, precision=p)[0][i], models[i])  # noqa: E731
        c = cfgs[i]
        m = models[i]
        rec = {"member": i, "grid": [c.ix - 2, c.jx - 2],
               "model": ["orszag_tang", "kelvin_helmholtz", "harris"][m.kind],
               "model_params": {"amp": m.amp, "bx0": m.bx0, "phase_x": m.phase_x, "phase_y": m.phase_y},
               "ensemble_max_scaled_l1": errs[i], "mixed_vs_fp64": curve(make, BATCH_STEPS, marks)}
        if control:
            rec["control_fp64_vs_fp64_parity"] = curve(make, BATCH_STEPS, marks, ("fp64_parity", "fp64"))
        out.append(rec)
    return out


def _fp64_peak_gflops(lib) -> float:
    import ctypes as C

    g = C.c_double()
    if lib.omhd_probe_fp64_peak(C.byref(g)) != 0:
        return float("nan")
    return g.value


def _fp32_peak_gflops(lib) -> float:
    import ctypes as C

    g = C.c_double()
    if lib.omhd_probe_fp32_peak(C.byref(g)) != 0:
        return float("nan")
    return g.value


def run_profile(args):
    """Small fixed run for profiler captures: --nx x --ny KH grid, one
    precision, warm-up + steps stage launches and nothing else."""
    import torch

    from openmhd_gb300 import Solver, harris3d, kelvin_helmholtz

    if args.pipelined_3d or args.one_role_2d:
        from openmhd_gb300 import _lib

        if args.pipelined_3d:
            _lib.load().omhd_set_3d_pipeline(1)
        if args.one_role_2d:
            _lib.load().omhd_set_2d_pipeline(0)
    if args.nz:
        cfg, model = harris3d(args.nx, args.ny, args.nz, precision=args.precision)
    else:
        cfg, model = kelvin_helmholtz(args.nx, args.ny, precision=args.precision)
    s = Solver(cfg).init_model(model)
    s.step(args.warmup)
    s.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s.stream)
    s.step(args.steps)
    e1.record(s.stream)
    info = s.sync()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    print(json.dumps({"profile": True, "nx": args.nx, "ny": args.ny, "nz": args.nz, "precision": args.precision,
                      "ms_per_step": ms, "cell_updates_per_s": cfg.interior_cells / (ms / 1e3),
                      "status": info.status, "steps": info.steps}), flush=True)
    return 0 if info.status == 0 else 1


def run_profile_adjoint(args):
    """Small fixed adjoint run for profiler captures: KH --nx x --ny, --steps
    steps (checkpoint every step), one forward and one backward."""
    import torch

    from openmhd_gb300 import Solver, kelvin_helmholtz
    from openmhd_gb300.adjoint import AdjointRun

    cfg, model = kelvin_helmholtz(args.nx, args.ny, precision="fp64")
    base = Solver(cfg).init_model(model).U.clone()
    run = AdjointRun(cfg, args.steps, 1)
    UN = run.forward(base)
    g = torch.zeros_like(UN)
    g[6] = 2 * UN[6]
    gU0 = run.backward(g)
    run.sync()
    print(json.dumps({"profile": "adjoint", "nx": args.nx, "ny": args.ny, "steps": args.steps,
                      "grad_norm": float(gU0.norm())}), flush=True)
    return 0


def run_profile_batched(args):
    """Small fixed ensemble run for profiler captures: 16 members, sides
    {256..512}, --precision (fp64 or mixed), --steps steps with the 32x8 tiling,
    2 CTAs per SM for FP32-mixed, 1 for FP64."""
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    prec = "mixed" if args.precision == "mixed" else "fp64"
    cfgs, models = batched_problem_set(16, seed=1, precision=prec, sides=[256, 320, 384, 448, 512])
    ens = Ensemble(cfgs).init_models(models)
    ens.set_tiling(0, 2 if prec == "mixed" else 1)
    ens.step(args.steps)
    infos = ens.sync()
    print(json.dumps({"profile": "batched", "precision": prec, "members": len(cfgs), "cells": ens.cells,
                      "steps": args.steps, "status": max(i.status for i in infos)}), flush=True)
    return 0


def run_profile_routines(args):
    """Small fixed run of the routine-level drop-in kernels for profiler
    captures: u2v, limiter (x, every variable of V) and flux_solver (x, HLLD)
    on an Orszag-Tang state of --nx x --ny cells held on the device, --steps
    times."""
    import torch

    from openmhd_gb300 import Solver, orszag_tang, routines

    cfg, model = orszag_tang(args.nx, args.ny, precision="fp64")
    U = Solver(cfg).init_model(model).U.clone()
    V = torch.empty((4,) + tuple(U.shape[1:]), dtype=torch.float64, device="cuda")
    VL = torch.empty_like(U)
    VR = torch.empty_like(U)
    F = torch.empty_like(U)
    for _ in range(args.steps):
        routines.u2v(U, V)
        for v in range(4):
            routines.limiter(V[v], VL[v], VR[v], 1, 2)
        for v in range(4, 9):
            routines.limiter(U[v], VL[v], VR[v], 1, 2)
        routines.flux_solver(F, VL, VR, 1.0, 1, 3)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "routines", "nx": args.nx, "ny": args.ny, "steps": args.steps}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-3d", action="store_true")
    ap.add_argument("--no-sq", action="store_true", help="skip the Orszag-Tang 4096x4096 FP64 leg")
    ap.add_argument("--adjoint-only", action="store_true", help="run the adjoint leg alone")
    ap.add_argument("--profile", action="store_true", help="small fixed run for profiler captures")
    ap.add_argument("--profile-adjoint", action="store_true", help="small adjoint run for profiler captures")
    ap.add_argument("--profile-batched", action="store_true", help="small ensemble run for profiler captures")
    ap.add_argument("--profile-routines", action="store_true",
                    help="routine-level drop-in kernels (u2v, limiter, flux_solver) for profiler captures")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--nz", type=int, default=0)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_parity", "mixed"])
    ap.add_argument("--pipelined-3d", action="store_true",
                    help="with --profile: the warp-specialised FP64 3D stage kernel instead of the one-role one")
    ap.add_argument("--one-role-2d", action="store_true",
                    help="with --profile: the one-role 2D stage kernels instead of the warp-specialised ones")
    ap.add_argument("--accuracy", action="store_true",
                    help="long-run error of the FP32-mixed path against FP64 (KH 2D and Harris 3D)")
    ap.add_argument("--accuracy-steps", type=int, default=2000)
    ap.add_argument("--accuracy-steps-3d", type=int, default=1000, help="0 skips the 3D run")
    ap.add_argument("--accuracy-control", action="store_true",
                    help="with --accuracy: also FP64 against FP64 without contraction (round-off growth)")
    args = ap.parse_args()
    if args.accuracy:
        from openmhd_gb300.build import build

        build()
        return run_accuracy(args)
    if args.profile or args.profile_adjoint or args.profile_batched or args.profile_routines:
        from openmhd_gb300.build import build

        build()
        if args.profile_adjoint:
            return run_profile_adjoint(args)
        if args.profile_batched:
            return run_profile_batched(args)
        if args.profile_routines:
            return run_profile_routines(args)
        return run_profile(args)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    from openmhd_gb300.build import build
    from oracle import oracle

    build()
    if args.adjoint_only:
        print(json.dumps({"adjoint": run_adjoint(args)}), flush=True)
        return 0
    oracle.build()
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
