"""Host-side mirror of the reference's driver loop (2D_basic/main.f90:56-188)
over the fused GB300 step, plus the problem setups used by this project.

A `Solver` owns one omhd_solver handle.  Its state and stage buffers are
torch float64 CUDA tensors bound to the handle, shaped (9, jx, ix) in 2D and
(9, kx, jx, ix) in 3D: exactly the reference's column-major U(ix,jx[,kx],var)
in memory.  Work runs on the solver's own CUDA stream, and nothing in a step
synchronises with the host.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

from . import _lib

OMHD_BAD_ARG = 4  # omhd_status_t
OMHD_TIMEOUT = 5
OMHD_CUDA_ERR = 6
OMHD_NOT_SUPPORTED = 7
OMHD_IO_ERR = 8
LIMITERS = {"flat": 0, "minmod": 1, "mc": 2, "vanleer": 3, "koren": 4}
FLUXES = {"llf": 0, "hll": 1, "hllc": 2, "hlld": 3, "lhlld": 4}
PRECISIONS = {"fp64": 0, "fp64_parity": 1, "mixed": 2}
ETA = {"none": 0, "recon2d": 1, "harris_xz": 2}

# variable slots (param.h:6-15), 1-based as in the reference
MX, MY, MZ, EN, RO, BX, BY, BZ, PS = range(1, 10)
VAR_NAMES = ["mx", "my", "mz", "en", "ro", "bx", "by", "bz", "ps"]


def flip(*slots: int) -> int:
    """Sign-flip mask for mirror boundaries (bit = 1-based variable slot - 1)."""
    m = 0
    for s in slots:
        m |= 1 << (s - 1)
    return m


class OmhdError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        super().__init__(f"openmhd_gb300 status {code}: {message}")
        self.code = code


@dataclass
class SolverConfig:
    nd: int
    ix: int
    jx: int
    kx: int = 1
    dx: float = 1.0
    dy: float = 1.0
    dz: float = 1.0
    x0: float = 0.0
    y0: float = 0.0
    z0: float = 0.0
    cfl: float = 0.4
    gamma: float = 5.0 / 3.0
    limiter: str = "minmod"
    flux: str = "hlld"
    time: str = "tvdrk2"
    eta: str = "none"
    bc_kind: tuple = (0, 0, 0, 0, 0, 0)
    bc_flip: tuple = (0, 0, 0, 0, 0, 0)
    precision: str = "fp64"
    tend: float = 0.0

    def to_c(self) -> _lib.Config:
        c = _lib.Config()
        c.nd, c.ix, c.jx, c.kx = self.nd, self.ix, self.jx, self.kx
        c.dx, c.dy, c.dz = self.dx, self.dy, self.dz
        c.x0, c.y0, c.z0 = self.x0, self.y0, self.z0
        c.cfl, c.gamma = self.cfl, self.gamma
        c.lm_type = LIMITERS[self.limiter]
        c.flux_type = FLUXES[self.flux]
        c.time_type = 0 if self.time == "tvdrk2" else 1
        c.eta_kind = ETA[self.eta]
        for q in range(6):
            c.bc_kind[q] = int(self.bc_kind[q])
            c.bc_flip[q] = int(self.bc_flip[q])
        c.precision = PRECISIONS[self.precision]
        c.tend = self.tend
        return c

    @property
    def shape(self) -> tuple:
        return (9, self.jx, self.ix) if self.nd == 2 else (9, self.kx, self.jx, self.ix)

    @property
    def interior_cells(self) -> int:
        n = (self.ix - 2) * (self.jx - 2)
        return n * (self.kx - 2) if self.nd == 3 else n


@dataclass
class ModelSpec:
    kind: int = 0          # 0 Orszag-Tang, 1 KH shear layer, 2 Harris sheet
    amp: float = 1.0
    bx0: float = 0.0
    phase_x: float = 0.0
    phase_y: float = 0.0
    beta: float = 0.2
    pert: float = 0.0
    seed: int = 0

    def to_c(self) -> _lib.Model:
        m = _lib.Model()
        m.kind, m.amp, m.bx0 = self.kind, self.amp, self.bx0
        m.phase_x, m.phase_y, m.beta, m.pert, m.seed = self.phase_x, self.phase_y, self.beta, self.pert, self.seed
        return m


# ---------------------------------------------------------------------------
# problem setups
# ---------------------------------------------------------------------------
def orszag_tang(nx: int = 256, ny: int | None = None, precision: str = "fp64", limiter: str = "mc",
                flux: str = "hlld", cfl: float = 0.4, tend: float = math.pi, amp: float = 1.0,
                phase_x: float = 0.0, phase_y: float = 0.0):
    """Orszag-Tang vortex on [0,2pi]^2, periodic (2D_basic/model.f90:34-50)."""
    ny = nx if ny is None else ny
    two_pi = 2 * (4.0 * math.atan(1.0))
    cfg = SolverConfig(nd=2, ix=nx + 2, jx=ny + 2, dx=two_pi / nx, dy=two_pi / ny, x0=0.0, y0=0.0,
                       cfl=cfl, limiter=limiter, flux=flux, precision=precision, tend=tend)
    if nx == ny:
        cfg.dy = cfg.dx  # the reference derives y spacing from dx (model.f90:19-28)
    return cfg, ModelSpec(kind=0, amp=amp, phase_x=phase_x, phase_y=phase_y)


def kelvin_helmholtz(nx: int = 4096, ny: int = 2048, precision: str = "fp64", limiter: str = "minmod",
                     flux: str = "hlld", cfl: float = 0.4, tend: float = 0.0, shear: float = 0.5,
                     bx0: float = 0.2, pert: float = 0.01, seed: int = 0):
    """KH shear layer: x in [0,40) periodic, y in [-20,20] with zero-gradient
    walls; rho=1, p=0.5, vx=shear*tanh(y), Bx=bx0, vy=pert*exp(-y^2)*r(x,y)."""
    Lx, Ly = 40.0, 40.0
    cfg = SolverConfig(nd=2, ix=nx + 2, jx=ny + 2, dx=Lx / nx, dy=Ly / ny, x0=0.0, y0=-20.0, cfl=cfl,
                       limiter=limiter, flux=flux, precision=precision, tend=tend,
                       bc_kind=(0, 0, 1, 1, 0, 0), bc_flip=(0, 0, 0, 0, 0, 0))
    if nx == ny:
        cfg.dy = cfg.dx
    return cfg, ModelSpec(kind=1, amp=shear, bx0=bx0, pert=pert, seed=seed)


def harris3d(nx: int = 512, ny: int = 256, nz: int = 512, precision: str = "fp64", limiter: str = "mc",
             flux: str = "hlld", cfl: float = 0.4, tend: float = 0.0, beta: float = 0.2, amp: float = 2.0e-3,
             seed: int = 0):
    """3D resistive Harris sheet: x in [-100,100], y in [-50,50] periodic, z in
    [-100,100] conducting walls (mz, Bz flip); eta = 1e-3 + exp(-(x^2+z^2)/4)/60."""
    dx, dy, dz = 200.0 / nx, 100.0 / ny, 200.0 / nz
    cfg = SolverConfig(nd=3, ix=nx + 2, jx=ny + 2, kx=nz + 2, dx=dx, dy=dy, dz=dz, x0=-100.0, y0=-50.0,
                       z0=-100.0, cfl=cfl, limiter=limiter, flux=flux, precision=precision, tend=tend,
                       eta="harris_xz", bc_kind=(0, 0, 0, 0, 1, 1),
                       bc_flip=(0, 0, 0, 0, flip(MZ, BZ), flip(MZ, BZ)))
    if dy == dx:
        cfg.dy = cfg.dx
    if dz == dx:
        cfg.dz = cfg.dx
    return cfg, ModelSpec(kind=2, beta=beta, amp=amp, seed=seed)


def reconnection2d(nx: int = 2000, ny: int = 500, precision: str = "fp64", limiter: str = "minmod",
                   flux: str = "hlld", cfl: float = 0.35, tend: float = 0.0, beta: float = 0.2, b1: float = 0.03):
    """2D resistive reconnection (2D_reconnection/model.f90, bc.f90, flux_resistive.f90):
    the quarter domain x in [0,200], y >= 0 with dy = dx, Harris sheet
    rho = 1 + cosh(y)^-2/beta, Bx = tanh(y) plus an X-point perturbation of
    amplitude b1, and the reference's symmetry walls (bc_for_U): west/east flip
    mx, mz, By, psi; south flips my, mz, Bx, psi; north flips my, By."""
    dx = 200.0 / nx
    lr = flip(MX, MZ, BY, PS)
    cfg = SolverConfig(nd=2, ix=nx + 2, jx=ny + 2, dx=dx, dy=dx, x0=0.0, y0=0.0, cfl=cfl, limiter=limiter,
                       flux=flux, precision=precision, tend=tend, eta="recon2d", bc_kind=(1, 1, 1, 1, 0, 0),
                       bc_flip=(lr, lr, flip(MY, MZ, BX, PS), flip(MY, BY), 0, 0))
    return cfg, ModelSpec(kind=3, beta=beta, amp=b1)


def brio_wu(nx: int = 300, precision: str = "fp64", limiter: str = "minmod", flux: str = "hlld", cfl: float = 0.8,
            tend: float = 0.2):
    """Brio-Wu MHD shock tube (1D_basic/model.f90, the active states) on
    x in [-0.5, 0.5] with zero-gradient ends, run as a strip of two periodic
    rows of the 2D step."""
    dx = 1.0 / nx
    cfg = SolverConfig(nd=2, ix=nx + 2, jx=4, dx=dx, dy=dx, x0=-0.5, y0=0.0, cfl=cfl, limiter=limiter, flux=flux,
                       precision=precision, tend=tend, bc_kind=(1, 1, 0, 0, 0, 0), bc_flip=(0,) * 6)
    return cfg, ModelSpec(kind=4)


def field_loop3d(nx: int = 100, ny: int = 100, nz: int = 200, precision: str = "fp64", limiter: str = "minmod",
                 flux: str = "hlld", cfl: float = 0.3, tend: float = 1.01, amp: float = 0.001):
    """3D field-loop advection (3D_basic/model.f90): a cylindrical A-profile
    loop, v = (1, 1, 2), on x in [-0.5, 0.5], y from -0.5, z from -1, periodic."""
    dx = 1.0 / nx
    cfg = SolverConfig(nd=3, ix=nx + 2, jx=ny + 2, kx=nz + 2, dx=dx, dy=dx, dz=dx, x0=-0.5, y0=-0.5, z0=-1.0,
                       cfl=cfl, limiter=limiter, flux=flux, precision=precision, tend=tend)
    return cfg, ModelSpec(kind=5, amp=amp)


# ---------------------------------------------------------------------------
# solver
# ---------------------------------------------------------------------------
class Solver:
    """Fused TVD-RK2 stepping of one grid on the current CUDA device."""

    def __init__(self, cfg: SolverConfig, stream=None):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("openmhd_gb300.Solver needs a CUDA device")
        self.cfg = cfg
        self.lib = _lib.load()
        self._h = C.c_void_p()
        ccfg = cfg.to_c()
        st = self.lib.omhd_solver_create(C.byref(ccfg), C.byref(self._h))
        if st:
            raise OmhdError(st, "omhd_solver_create rejected the configuration")
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.U = torch.empty(cfg.shape, dtype=torch.float64, device="cuda")
        self.U1 = torch.empty(cfg.shape, dtype=torch.float64, device="cuda")
        self._check(self.lib.omhd_solver_bind(self._h, self.U.data_ptr(), self.U1.data_ptr()))
        self._check(self.lib.omhd_solver_set_stream(self._h, C.c_void_p(self.stream.cuda_stream)))

    def _check(self, st: int):
        if st:
            info = _lib.ErrorInfo()
            self.lib.omhd_solver_last_error(self._h, C.byref(info))
            raise OmhdError(st, info.message.decode(errors="replace"))

    def close(self):
        if self._h:
            self.lib.omhd_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state --
    def init_model(self, m: ModelSpec):
        import torch

        torch.cuda.current_stream().synchronize()
        mc = m.to_c()
        self._check(self.lib.omhd_solver_init_model(self._h, C.byref(mc)))
        torch.cuda.current_stream().wait_stream(self.stream)  # U is read on the caller's stream next
        return self

    def put_state(self, U, t: float = 0.0):
        """Load a full state (numpy array or torch tensor, any device)."""
        import numpy as np
        import torch

        if isinstance(U, np.ndarray):
            a = np.ascontiguousarray(U, dtype=np.float64).reshape(self.cfg.shape)
            self._check(self.lib.omhd_solver_put_state(self._h, a.ctypes.data, float(t)))
            self.sync()
        else:
            src = U.to(dtype=torch.float64).contiguous().reshape(self.cfg.shape)
            torch.cuda.current_stream().synchronize()
            self._check(self.lib.omhd_solver_put_state(self._h, src.data_ptr(), float(t)))
            self.sync()
        return self

    def step_host(self, U_in, U_out=None, t: float = 0.0, n: int = 1) -> int:
        """Host state in, `n` steps, host state out, in one call
        (omhd_solver_step_host): U_in / U_out are CPU torch tensors or numpy
        arrays of the state's shape (float64, contiguous); U_in None continues
        from the device state, U_out None writes back into U_in.  Page-locked
        tensors (pin_memory) take the fused upload and the direct write of the
        result.  Returns the device error code (0: no error)."""
        import torch

        def ptr(a):
            if a is None:
                return None
            if isinstance(a, torch.Tensor):
                if a.device.type != "cpu" or a.dtype != torch.float64 or not a.is_contiguous():
                    raise ValueError("step_host takes contiguous float64 CPU tensors")
                return a.data_ptr()
            if a.dtype.str != "<f8" or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("step_host takes contiguous float64 arrays")
            return a.ctypes.data

        if U_out is None:
            U_out = U_in
        if U_out is None:
            raise ValueError("step_host needs an output buffer")
        for a in (U_in, U_out):
            if a is not None and tuple(a.shape) != tuple(self.cfg.shape):
                raise ValueError(f"state shape {tuple(a.shape)} != {tuple(self.cfg.shape)}")
        self.stream.wait_stream(torch.cuda.current_stream())
        st = self.lib.omhd_solver_step_host(self._h, ptr(U_in), ptr(U_out), float(t), int(n))
        if st in (OMHD_BAD_ARG, OMHD_CUDA_ERR):
            self._check(st)
        torch.cuda.current_stream().wait_stream(self.stream)
        return st

    def state(self):
        """The bound state tensor (valid after sync())."""
        return self.U

    def get_state_numpy(self):
        import numpy as np

        out = np.empty(self.cfg.shape, dtype=np.float64)
        self._check(self.lib.omhd_solver_get_state(self._h, out.ctypes.data))
        return out

    def coords(self):
        import numpy as np

        x = np.empty(self.cfg.ix)
        y = np.empty(self.cfg.jx)
        z = np.empty(self.cfg.kx)
        self.lib.omhd_solver_coords(self._h, x.ctypes.data, y.ctypes.data, z.ctypes.data)
        return x, y, z

    # -- snapshot files (fileio.f90 layout) --
    def write_snapshot(self, path: str):
        """State, primitives, coordinates and t in the reference's field file format."""
        self._check(self.lib.omhd_solver_write(self._h, str(path).encode()))
        return self

    def read_snapshot(self, path: str):
        """Restart from a field file (its t becomes the solver's time)."""
        self._check(self.lib.omhd_solver_read(self._h, str(path).encode()))
        return self

    # -- stepping --
    def step(self, n: int = 1):
        import torch

        self.stream.wait_stream(torch.cuda.current_stream())  # the caller may have written U
        self._check(self.lib.omhd_solver_step(self._h, int(n)))
        torch.cuda.current_stream().wait_stream(self.stream)
        return self

    def step_graph(self, n: int, replays: int = 1):
        self._check(self.lib.omhd_solver_step_graph(self._h, int(n), int(replays)))
        return self

    def sync(self) -> _lib.StepInfo:
        info = _lib.StepInfo()
        st = self.lib.omhd_solver_sync(self._h, C.byref(info))
        if st:
            self._check(st)
        return info

    def set_tend(self, tend: float):
        """Set the end time; steps stop on the device at the first t >= tend."""
        self._check(self.lib.omhd_solver_set_tend(self._h, float(tend)))
        return self

    def run_until(self, tend: float, batch: int = 64):
        """Advance until the first t >= tend (main.f90:73).  Steps are enqueued
        in batches; kernels turn themselves off once t >= tend, so the step
        count matches the reference's loop exactly."""
        self.set_tend(tend)
        last = -1
        while True:
            self.step(batch)
            info = self.sync()  # raises on a device-reported failure
            if info.done:
                return info
            if info.steps == last:
                raise OmhdError(OMHD_TIMEOUT, "run_until made no progress")
            last = info.steps

    def run_with_output(self, tend: float, dtout: float, outdir: str = "data", batch: int = 64,
                        n_start: int = 0) -> list:
        """The reference driver's time loop with snapshot output (2D_basic/main.f90:36-75):
        a field file `outdir/field-NNNNN.dat` at the start and then at the first
        t >= t_output, t_output starting at t0 - dt0/3 (dt0: the first CFL step)
        and advancing by dtout per file, until the first t >= tend.  Between
        files the steps run on the device without host synchronisation; as in
        the reference, at most one file is written per step.  `n_start` restarts
        as the reference's MPI driver does (2D_basic/mainp.f90:85-118): n_start > 0
        reads file n_start and continues with file n_start + 1 at t + dtout;
        n_start < 0 first looks for the newest file from floor(tend/dtout) down.
        Returns the written paths."""
        return run_with_output(self, tend, dtout, outdir, batch, n_start)

    @property
    def launches_per_step(self) -> int:
        return int(self.lib.omhd_solver_launches_per_step(self._h))


def snapshot_path(outdir: str, n: int) -> str:
    """File name of snapshot n (the reference's 'data/field-',i5.5,'.dat' format, mainp.f90:277)."""
    import os

    return os.path.join(outdir, "field-%05d.dat" % n)


def run_with_output(solver, tend: float, dtout: float, outdir: str = "data", batch: int = 64,
                    n_start: int = 0) -> list:
    """Output cadence of the reference's main loop (2D_basic/main.f90:41-75) over
    a solver's sync / set_tend / step / run_until / write_snapshot /
    read_snapshot calls.

    The reference writes, at the top of each loop iteration, one file if
    t >= t_output (then t_output += dtout), stops if t >= tend, and otherwise
    takes one step; t_output starts at -dt/3 with dt the first CFL step, and
    a first dt above dtout stops the run (main.f90:44-47).  Here the steps
    between two files are enqueued with the device-side end time set to the
    next output time, so the files fall on the same steps.

    Restart (2D_basic/mainp.f90:85-118): with n_start < 0 the newest existing
    file is searched from k = floor(tend/dtout) down to 0 (n_start = 0, a
    fresh start, if there is none); with n_start > 0 file n_start is read (its
    t becomes the solver's time), the next file is n_start + 1 and the next
    output time t + dtout, so the restart file itself is not written again."""
    import math
    import os

    info = solver.sync()
    t, dt0 = info.t, info.dt
    if dt0 > dtout:
        raise ValueError(f"error: {dt0} > {dtout} (the first dt exceeds the output interval)")
    os.makedirs(outdir, exist_ok=True)
    if n_start < 0:
        n_start = 0
        for k in range(math.floor(tend / dtout), -1, -1):
            if os.path.isfile(snapshot_path(outdir, k)):
                n_start = k
                break
    if n_start == 0:
        t_output = t - dt0 / 3.0
        n_output = 0
    else:
        solver.read_snapshot(snapshot_path(outdir, n_start))
        t = solver.sync().t
        n_output = n_start + 1
        t_output = t + dtout
    paths = []
    while True:
        if t >= t_output:
            path = snapshot_path(outdir, n_output)
            solver.write_snapshot(path)
            paths.append(path)
            n_output += 1
            t_output += dtout
        if t >= tend:
            break
        target = min(t_output, tend)
        if t >= target:  # the next output time has already passed: one step, as the reference's loop
            solver.set_tend(tend)
            solver.step(1)
            info = solver.sync()
        else:
            info = solver.run_until(target, batch=batch)
        t = info.t
    solver.set_tend(tend)
    return paths
