"""xcore_gb300 -- Python host side of the GB300 drop-in for xcore.jl's time-step path.

This module mirrors the reference's host-facing API (aelligp/xcore.jl, pure
Julia) over the C ABI of ``libxcore_gb300.so`` (include/xcore_gb300.h):

* ``Parameters`` / ``Grid`` / ``compute_scales`` restate the host-side scalar
  setup (src/parameters.jl:12-89, src/grid.jl:311-334, src/scales.jl:85-185);
* ``State`` owns one device context holding FluidState + PhaseState +
  NoiseState + StepResidual with the reference's field names and sizes, and
  exposes the reference's mutating functions as methods: ``phsevo``
  (phsevo!), ``fluidmech`` (fluidmech!), ``noise`` (noise!), ``update``
  (update!), ``update_phase_velocities``, ``store_previous``, ``store_noise``,
  ``snapshot``, ``update_dt``, ``compute_resnorm``, ``initialize``, ``step``;
* module functions ``advect`` / ``advect_with_flux`` / ``diffus`` /
  ``diffus_with_flux`` / ``fill_ghosts`` take device arrays (torch CUDA
  tensors) exactly as the reference kernels take arrays.

Arrays cross the boundary column-major with z the leading dimension, like the
Julia matrices.  Host arrays here are numpy arrays indexed ``[z, x]``.
There is no CPU fallback: the library must be built (``build()``) and a CUDA
device present, otherwise calls raise.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libxcore_gb300.so")

XC_OK, XC_BAD_ARG, XC_NOT_CONVERGED, XC_NAN, XC_TIMEOUT, XC_CUDA, XC_NO_DEVICE = range(7)
SCHEMES = {"centr": 0, "upwd1": 1, "quick": 2, "fromm": 3, "weno3": 4, "weno5": 5, "tvdim": 6}
BCS = {"periodic": 0, "closed": 1}
TINTS = {"be1im": 0, "bd2im": 1, "cn2si": 2, "bd2si": 3}
SOLVERS = {"fgmres64": 0, "mixed": 1}
EPS = float(np.finfo(np.float64).eps)


class XcoreError(RuntimeError):
    """A non-OK status from the library, with its message."""

    def __init__(self, status, msg):
        super().__init__(f"xcore_gb300 status {status}: {msg}")
        self.status = status


class NotConverged(XcoreError):
    """A Stokes solve stopped at its iteration cap above its tolerance.  For a
    whole time step the step was still completed; ``info`` then holds its
    statistics (as ``State.step`` returns them)."""

    info = None


class _Params(ctypes.Structure):
    _fields_ = [("Nz", ctypes.c_int), ("Nx", ctypes.c_int), ("h", ctypes.c_double), ("D", ctypes.c_double),
                ("rhom0", ctypes.c_double), ("rhox0", ctypes.c_double), ("d0", ctypes.c_double),
                ("g0", ctypes.c_double), ("etam0", ctypes.c_double), ("etax0", ctypes.c_double),
                ("AA", ctypes.c_double * 4), ("BB", ctypes.c_double * 4), ("CC", ctypes.c_double * 4),
                ("Xi", ctypes.c_double), ("Ptop", ctypes.c_double), ("alpha", ctypes.c_double),
                ("gamma", ctypes.c_double), ("CFL", ctypes.c_double), ("dtmax", ctypes.c_double),
                ("etacntr", ctypes.c_double), ("open_sgr", ctypes.c_int),
                ("L0", ctypes.c_double), ("l0", ctypes.c_double), ("L0h", ctypes.c_double),
                ("l0h", ctypes.c_double), ("D0", ctypes.c_double), ("txi0", ctypes.c_double),
                ("G0", ctypes.c_double), ("bnd_w", ctypes.c_double), ("dt0", ctypes.c_double),
                ("ADVN", ctypes.c_int), ("TINT", ctypes.c_int), ("xBC", ctypes.c_int), ("zBC", ctypes.c_int),
                ("sds", ctypes.c_int), ("top_cnv", ctypes.c_int), ("bot_cnv", ctypes.c_int),
                ("open_cnv", ctypes.c_int), ("weno_weights", ctypes.c_int)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("rtol", ctypes.c_double), ("maxit", ctypes.c_int),
                ("restart", ctypes.c_int), ("inner_rtol", ctypes.c_double), ("inner_maxit", ctypes.c_int),
                ("smooth_sweeps", ctypes.c_int), ("omega_velocity", ctypes.c_double),
                ("schur_mass", ctypes.c_double), ("schur_full_diagonal", ctypes.c_int),
                ("coarse_cells", ctypes.c_int), ("coarse_sweeps", ctypes.c_int), ("small_cells", ctypes.c_int),
                ("pressure_sweeps", ctypes.c_int), ("inner_gs_passes", ctypes.c_int),
                ("serial_launch", ctypes.c_int), ("coarse_viscosity_mean", ctypes.c_int),
                ("tiled_sweep", ctypes.c_int), ("post_sweeps", ctypes.c_int), ("outer_solver", ctypes.c_int),
                ("fused_pressure_cells", ctypes.c_int),
                ("stage_small_levels", ctypes.c_int),
                ("jacobi_coarse", ctypes.c_int), ("row_block_sweep", ctypes.c_int), ("learned", ctypes.c_int),
                ("device_givens", ctypes.c_int), ("cluster_cells", ctypes.c_int)]

    @classmethod
    def make(cls, solver="fgmres64", rtol=1e-10, maxit=500, restart=30, inner_rtol=1e-4, inner_maxit=60,
             smooth_sweeps=0, omega_velocity=0.0, schur_mass=0.0, schur_full_diagonal=False,
             coarse_cells=0, coarse_sweeps=0, small_cells=0, pressure_sweeps=0, inner_gs_passes=0,
             serial_launch=False, coarse_viscosity_mean=0, tiled_sweep=False, post_sweeps=0, outer_solver=0,
             fused_pressure_cells=0, stage_small_levels=False,
             jacobi_coarse=False, row_block_sweep=False, learned=0, device_givens=False,
             cluster_cells=0):
        return cls(SOLVERS[solver], float(rtol), int(maxit), int(restart), float(inner_rtol), int(inner_maxit),
                   int(smooth_sweeps), float(omega_velocity), float(schur_mass), int(bool(schur_full_diagonal)),
                   int(coarse_cells), int(coarse_sweeps), int(small_cells), int(pressure_sweeps),
                   int(inner_gs_passes), int(bool(serial_launch)), int(coarse_viscosity_mean),
                   int(bool(tiled_sweep)), int(post_sweeps), int(outer_solver),
                   int(fused_pressure_cells), int(bool(stage_small_levels)),
                   int(bool(jacobi_coarse)), int(bool(row_block_sweep)), int(learned), int(bool(device_givens)),
                   int(cluster_cells))


class SolverStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("refinements", ctypes.c_int), ("rel_residual", ctypes.c_double),
                ("converged", ctypes.c_int), ("seconds", ctypes.c_double), ("learned_fallbacks", ctypes.c_int),
                ("device_givens_steps", ctypes.c_int)]


MAX_SWEEPS = 64


class StepStats(ctypes.Structure):
    _fields_ = [("resnorm", ctypes.c_double * MAX_SWEEPS), ("resnorm0", ctypes.c_double),
                ("sweeps", ctypes.c_int), ("solver_iterations", ctypes.c_int),
                ("solver_rel_residual", ctypes.c_double), ("dt_next", ctypes.c_double),
                ("unconverged_solves", ctypes.c_int), ("picard_converged", ctypes.c_int)]

    def as_dict(self):
        return dict(resnorm=list(self.resnorm[:self.sweeps]), resnorm0=self.resnorm0, sweeps=self.sweeps,
                    solver_iterations=self.solver_iterations, solver_rel_residual=self.solver_rel_residual,
                    dt_next=self.dt_next, unconverged_solves=self.unconverged_solves,
                    picard_converged=bool(self.picard_converged))


_lib = None


def lib():
    """Load libxcore_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: run xcore_gb300.build() first (no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        D6 = ctypes.POINTER(ctypes.c_double)
        sig = {
            "xc_ctx_create": (ip, [ctypes.POINTER(_Params), ctypes.POINTER(vp)]),
            "xc_ctx_destroy": (ip, [vp]),
            "xc_field_count": (ip, []),
            "xc_field_name": (ctypes.c_char_p, [ip]),
            "xc_field_id": (ip, [ctypes.c_char_p]),
            "xc_field_shape": (ip, [vp, ip, ctypes.POINTER(ip), ctypes.POINTER(ip), ctypes.POINTER(ip)]),
            "xc_field_device_ptr": (ip, [vp, ip, ctypes.POINTER(vp)]),
            "xc_field_bind": (ip, [vp, ip, vp]),
            "xc_field_upload": (ip, [vp, ip, vp]),
            "xc_field_download": (ip, [vp, ip, vp]),
            "xc_synchronize": (ip, [vp]),
            "xc_store_previous": (ip, [vp]),
            "xc_store_noise": (ip, [vp]),
            "xc_snapshot": (ip, [vp]),
            "xc_phsevo": (ip, [vp, ip, D6, dp, dp]),
            "xc_fluidmech": (ip, [vp, D6, dp, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolverStats)]),
            "xc_fluidmech_mms": (ip, [vp, vp, vp, vp, vp, vp, vp, D6, dp, ctypes.POINTER(SolverOpts),
                                      ctypes.POINTER(SolverStats)]),
            "xc_noise": (ip, [vp, dp, ip, vp, vp]),
            "xc_update_phase_velocities": (ip, [vp]),
            "xc_update": (ip, [vp]),
            "xc_update_dt": (ip, [vp, dp, D6]),
            "xc_resnorm": (ip, [vp, dp, D6]),
            "xc_conservation_sums": (ip, [vp, D6]),
            "xc_history_stats": (ip, [vp, D6]),
            "xc_initialize": (ip, [vp, vp, vp, vp]),
            "xc_step": (ip, [vp, ip, dp, ip, vp, vp, ctypes.POINTER(SolverOpts), ctypes.POINTER(StepStats)]),
            "xc_step_converge": (ip, [vp, ip, dp, dp, dp, ip, vp, vp, ctypes.POINTER(SolverOpts),
                                      ctypes.POINTER(StepStats)]),
            "xc_print_step_stats": (ip, [vp, D6]),
            "xc_ensemble_create": (ip, [ctypes.POINTER(vp), ip, ip, ctypes.POINTER(vp)]),
            "xc_ensemble_destroy": (ip, [vp]),
            "xc_ensemble_step": (ip, [vp, ctypes.POINTER(ip), D6, ip, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                      ctypes.POINTER(SolverOpts), ctypes.POINTER(StepStats)]),
            "xc_fill_ghosts": (ip, [vp, ip, ip, ip, ip, ip, vp]),
            "xc_advect": (ip, [vp, vp, vp, vp, ip, ip, dp, ip, vp]),
            "xc_advect_with_flux": (ip, [vp, vp, vp, vp, vp, vp, ip, ip, dp, ip, ip, ip, vp]),
            "xc_advect_centered_with_flux": (ip, [vp, vp, vp, vp, vp, vp, ip, ip, dp, ip, ip, ip, vp]),
            "xc_diffus": (ip, [vp, vp, vp, ip, ip, dp, vp]),
            "xc_diffus_with_flux": (ip, [vp, vp, vp, vp, vp, ip, ip, dp, ip, ip, vp]),
            "xc_time_coefs": (ip, [ip, ip, D6]),
            "xc_stream": (vp, [vp]),
            "xc_launch_count": (ctypes.c_longlong, []),
            "xc_bench_kernel": (ip, [vp, ip, ip, D6]),
            "xc_update_dt_noalloc": (ip, [vp, vp, vp, vp, vp, ip, ip, dp, dp, dp, dp, vp, vp]),
            "xc_nn_conv3x3": (ip, [vp, vp, vp, vp, vp, ip, ip, ip, ip, ip, ip, vp]),
            "xc_nn_conv3x3_wgrad": (ip, [vp, vp, vp, ip, ip, ip, ip, ip, vp]),
            "xc_nn_create": (ip, [ip, ip, ip, ip, ip, ctypes.c_ulonglong, ctypes.POINTER(vp)]),
            "xc_nn_destroy": (ip, [vp]),
            "xc_nn_param_count": (ctypes.c_longlong, [vp]),
            "xc_nn_layout": (ip, [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                  ctypes.POINTER(ip)]),
            "xc_nn_get_params": (ip, [vp, vp]),
            "xc_nn_set_params": (ip, [vp, vp]),
            "xc_nn_get_grads": (ip, [vp, vp]),
            "xc_nn_forward": (ip, [vp, vp, vp, vp]),
            "xc_nn_loss_grad": (ip, [vp, vp, vp, ctypes.POINTER(ctypes.c_float), vp]),
            "xc_nn_train_step": (ip, [vp, vp, vp, ctypes.c_float, ctypes.POINTER(ctypes.c_float), vp]),
            "xc_set_learned_preconditioner": (ip, [vp, vp, ctypes.c_longlong]),
            "xc_learned_sample": (ip, [vp, vp, ip, vp, vp, dp, ip, ctypes.POINTER(ip)]),
            "xc_stokes_apply_scaled": (ip, [vp, vp, vp]),
            "xc_last_error": (ctypes.c_char_p, []),
            "xc_version": (ctypes.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status):
    if status != XC_OK:
        msg = lib().xc_last_error().decode()
        if status == XC_NOT_CONVERGED:
            raise NotConverged(status, msg)
        raise XcoreError(status, msg)


def build(force: bool = False) -> str:
    """Compile the CUDA sources in-tree (nvcc, sm_103a) and return the .so path."""
    from importlib import util
    spec = util.spec_from_file_location("_xcore_gb300_build", os.path.join(_HERE, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def field_names():
    L = lib()
    return [L.xc_field_name(i).decode() for i in range(L.xc_field_count())]


# What save_checkpoint writes (src/restart.jl:53-83): every array field of
# FluidState (src/state.jl:74-122; its solver cache is rebuilt on load) and of
# PhaseState (src/state.jl:165-258), and the time-evolving NoiseState fields
# of noise_dynamic_fields (src/restart.jl:25-28).  The noise RNG stays with the
# caller: the library takes each step's white-noise draws as inputs.
CHECKPOINT_GROUPS = {
    "fluid": ("W", "U", "P", "eta", "etaco", "rho", "rhow", "rhou", "Drho", "rhoo", "rhooo", "drhodt",
              "drhodto", "drhodtoo", "MFS", "rhoWo", "rhoWoo", "rhoUo", "rhoUoo"),
    "phase": ("x", "m", "X", "M", "Xo", "Xoo", "Mo", "Moo", "chi", "mu", "hasx", "hasm", "chiw", "muw", "chiu",
              "muu", "x_w", "m_w", "x_u", "m_u", "Drhom", "Drhox", "Pl", "Pt", "etamix", "etae", "ke", "kx",
              "etat", "etas", "etasw", "ks", "V", "Div_V", "exx", "ezz", "exz", "eII", "vx", "vm", "txx", "tzz",
              "txz", "tII", "fReL", "ReL", "ReD", "Ra", "fRel", "Rel", "Red", "Rc", "Wx", "Wm", "Ux", "Um", "wx",
              "wm", "bndtaperw", "bndshape", "advn_X", "advn_M", "advn_rho", "qx_advn_X", "qz_advn_X",
              "qx_advn_M", "qz_advn_M", "qx_dffn_X", "qz_dffn_X", "qx_dffn_M", "qz_dffn_M", "dffn_X", "Gx",
              "dXdt", "dXdto", "dXdtoo"),
    "noise": ("psie", "psix", "psis", "psieo", "psixo", "psiso", "re", "rs", "xiew", "xieu", "xixw", "xixu",
              "xisw", "xisu", "xie", "xix", "xis"),
}


# ---------------------------------------------------------------------------
# host-side scalar setup (restated from the reference)
# ---------------------------------------------------------------------------


@dataclass
class Parameters:
    """Parameters{Float64} fields the path reads (src/parameters.jl:12-89)."""
    D: float = 10.0
    N: int = 100
    L: float = 10.0
    x0: float = EPS
    dxr: float = 0.1
    rhom0: float = 2700.0
    rhox0: float = 3200.0
    d0: float = 0.01
    g0: float = 10.0
    etam0: float = 10.0
    etax0: float = 1e18
    AA: tuple = ((0.72, 0.19), (0.81, 0.20))
    BB: tuple = ((0.63, 0.37), (0.999, 0.001))
    CC: tuple = ((2.09, 0.09), (0.37, 1.45))
    L0: float = 0.1
    l0: float = 0.1
    Da: float = 0.01
    Xi: float = 0.5
    Ptop: float = 1e5
    open_sgr: bool = False
    TINT: str = "bd2im"
    ADVN: str = "weno5"
    CFL: float = 0.5
    alpha: float = 0.9
    gamma: float = 1e-3
    dtmax: float = 1e32
    etacntr: float = 1e8


@dataclass
class Grid:
    """src/grid.jl:311-334."""
    Nx: int
    Nz: int
    h: float
    D: float
    L: float

    @classmethod
    def from_params(cls, p: Parameters) -> "Grid":
        h = p.D / p.N
        return cls(Nx=max(1, int(round(p.L / h))), Nz=p.N, h=h, D=p.D, L=p.L)


def compute_scales(p: Parameters, g: Grid, tol: float = 1e-9, maxiter: int = 200) -> dict:
    """The scales the path reads, from the fixed point of src/scales.jl:85-185."""
    D, d0, x0, Da, h = p.D, p.d0, p.x0, p.Da, g.h
    rho0, Drho0, eta0, g0 = p.rhom0, p.rhox0 - p.rhom0, p.etam0, p.g0
    D0 = D / 10
    L0, l0 = p.L0, p.l0
    L0h, l0h = (L0 + h) / 2, (l0 + h) / 2
    bnd_w = l0 / 2 + D / 100
    chi0, Dchi0 = (Da, Da / 10) if Da > 0 else (x0, x0 / 10)
    W0 = Dchi0 * Drho0 * g0 * (D0 * D0) / eta0
    w0 = Drho0 * g0 * (d0 * d0) / eta0
    W0t = math.sqrt(Dchi0 * Drho0 * g0 * (D0 * D0 * D0) / ((L0 * L0) * rho0))
    W0i = math.sqrt(Dchi0 * Drho0 * g0 * D / rho0)
    Ri2 = (W0i / W0t) ** 2
    fReL0 = 1 - math.exp(-(W0 * L0 / (eta0 / rho0)))
    for _ in range(maxiter):
        W0p, w0p = W0, w0
        fReL0 = 1 - math.exp(-(W0 * L0 / (eta0 / rho0)))
        fRel0 = 1 - math.exp(-(w0 * l0 / (eta0 / rho0)))
        W0 = (math.sqrt(4 / Ri2 * Dchi0 * Drho0 * g0 * rho0 * fReL0 * (L0 * L0) * D0 + eta0 * eta0) - eta0) \
            * D0 / (2 * fReL0 * (L0 * L0) * rho0 / Ri2)
        w0 = (math.sqrt(4 * Drho0 * g0 * rho0 * fRel0 * l0 * (d0 * d0) + eta0 * eta0) - eta0) / (2 * fRel0 * l0 * rho0)
        if abs(W0 - W0p) / W0 + abs(w0 - w0p) / w0 <= tol:
            break
    ke0 = (W0 / D0) * (L0 * L0)
    ks0 = w0 * l0
    kx0 = ks0 + fReL0 * ke0
    tW0, tw0, tk0, ti0 = D / W0, D / w0, (D * D) / kx0, D / W0i
    t0 = 1.0 / (1 / (ti0 + tW0) + 1 / tw0 + 1 / tk0)
    return dict(D0=D0, L0=L0, L0h=L0h, l0=l0, l0h=l0h, bnd_w=bnd_w, W0=W0, w0=w0, kx0=kx0,
                txi0=p.rhox0 * (d0 * d0) / 18 / eta0, t0=t0,
                dt0=min((h / 2) * (h / 2) / kx0, (h / 2) / (W0 + w0)), G0=Da * rho0 / t0 * D / D0)


def time_coefs(TINT: str, step: int):
    """time_coefs(Float64, TINT, step) through the library (src/timing.jl:18-36)."""
    out = (ctypes.c_double * 6)()
    _check(lib().xc_time_coefs(TINTS[TINT], int(step), out))
    return tuple(out)


# ---------------------------------------------------------------------------
# device state
# ---------------------------------------------------------------------------


def _host(arr, shape, dtype=np.float64):
    a = np.asarray(arr, dtype=dtype)
    if a.shape != tuple(shape):
        raise ValueError(f"expected shape {tuple(shape)}, got {a.shape}")
    return np.asfortranarray(a)


class State:
    """FluidState + PhaseState + NoiseState + StepResidual resident on the GPU."""

    def __init__(self, par: Parameters, grid: Grid | None = None, scales: dict | None = None,
                 xBC="periodic", zBC="closed", sds=-1, top_cnv=1, bot_cnv=1, open_cnv=False,
                 weno_weights=0):
        self.par = par
        self.grid = grid or Grid.from_params(par)
        self.scales = scales or compute_scales(par, self.grid)
        g, s = self.grid, self.scales
        P = _Params()
        P.Nz, P.Nx, P.h, P.D = g.Nz, g.Nx, g.h, g.D
        for k in ("rhom0", "rhox0", "d0", "g0", "etam0", "etax0", "Xi", "Ptop", "alpha", "gamma", "CFL",
                  "dtmax", "etacntr"):
            setattr(P, k, float(getattr(par, k)))
        for k in ("AA", "BB", "CC"):
            m = getattr(par, k)
            getattr(P, k)[:] = [m[0][0], m[0][1], m[1][0], m[1][1]]
        P.open_sgr = int(bool(par.open_sgr))
        for k in ("L0", "l0", "L0h", "l0h", "D0", "txi0", "G0", "bnd_w", "dt0"):
            setattr(P, k, float(s[k]))
        P.ADVN, P.TINT = SCHEMES[par.ADVN], TINTS[par.TINT]
        P.xBC, P.zBC = BCS[xBC], BCS[zBC]
        P.sds, P.top_cnv, P.bot_cnv, P.open_cnv = int(sds), int(top_cnv), int(bot_cnv), int(bool(open_cnv))
        P.weno_weights = int(weno_weights)
        self._p = P
        h = ctypes.c_void_p()
        _check(lib().xc_ctx_create(ctypes.byref(P), ctypes.byref(h)))
        self._h = h
        self._ids = {n: i for i, n in enumerate(field_names())}
        # StepResidual.resnorm0 (src/diagnose.jl:23, 1.0 at construction):
        # compute_resnorm raises it, nothing else touches it
        self.resnorm0 = 1.0

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().xc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields ------------------------------------------------------------
    def shape(self, name):
        r, c, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().xc_field_shape(self._h, self._ids[name], ctypes.byref(r), ctypes.byref(c), ctypes.byref(e)))
        return (r.value, c.value), e.value

    def __getitem__(self, name):
        shp, eb = self.shape(name)
        out = np.empty(shp, dtype=np.float64 if eb == 8 else np.uint8, order="F")
        _check(lib().xc_field_download(self._h, self._ids[name], out.ctypes.data))
        return np.ascontiguousarray(out) if eb == 8 else out.astype(bool)

    def __setitem__(self, name, value):
        shp, eb = self.shape(name)
        a = _host(value, shp, np.float64 if eb == 8 else np.uint8)
        _check(lib().xc_field_upload(self._h, self._ids[name], a.ctypes.data))

    def device_ptr(self, name) -> int:
        p = ctypes.c_void_p()
        _check(lib().xc_field_device_ptr(self._h, self._ids[name], ctypes.byref(p)))
        return p.value

    def bind(self, name, tensor):
        """Work in place on a caller's CUDA tensor for field `name` (zero
        copy): a contiguous tensor of shape (cols, rows) -- the field's
        column-major bytes -- and its dtype (float64; uint8/bool for hasx,
        hasm).  None unbinds.  The tensor must outlive the binding."""
        if tensor is None:
            _check(lib().xc_field_bind(self._h, self._ids[name], None))
            return
        (rows, cols), eb = self.shape(name)
        if tuple(tensor.shape) != (cols, rows) or tensor.element_size() != eb or not tensor.is_contiguous():
            raise ValueError(f"{name}: need a contiguous ({cols}, {rows}) tensor of {eb}-byte elements")
        _check(lib().xc_field_bind(self._h, self._ids[name], ctypes.c_void_p(tensor.data_ptr())))

    def synchronize(self):
        _check(lib().xc_synchronize(self._h))

    def stream_handle(self) -> int:
        """The context's cudaStream_t (for events recorded by the caller)."""
        return lib().xc_stream(self._h)

    def bench_kernel(self, which: int, iters: int = 20):
        """CUDA-event timing of one kernel on the current state:
        (ms per launch, algorithmic bytes, algorithmic flops, units)."""
        out = (ctypes.c_double * 4)()
        _check(lib().xc_bench_kernel(self._h, int(which), int(iters), out))
        return tuple(out)


    # -- the reference's functions ------------------------------------------
    def store_previous(self):
        """store_previous!(fluid, phase) -- src/store.jl:13-30."""
        _check(lib().xc_store_previous(self._h))

    def store_noise(self):
        """store_noise!(ns) -- src/noise.jl:115-120."""
        _check(lib().xc_store_noise(self._h))

    def snapshot(self):
        """snapshot!(res, phase, fluid) -- src/diagnose.jl:42-49."""
        _check(lib().xc_snapshot(self._h))

    def phsevo(self, coefs, dt, ADVN=None, alpha=None):
        """phsevo!(phase, fluid, grid, par, scales; ADVN, a1..b3, dt, alpha) -- src/phsevo.jl:164-214."""
        c6 = (ctypes.c_double * 6)(*coefs)
        scheme = -1 if ADVN is None else SCHEMES[ADVN]
        _check(lib().xc_phsevo(self._h, scheme, c6, float(dt), float(self.par.alpha if alpha is None else alpha)))

    def fluidmech(self, coefs, dt, solver="fgmres64", rtol=1e-10, maxit=500, restart=30,
                  inner_rtol=1e-4, inner_maxit=60, mms=None, **knobs):
        """fluidmech!(fluid, grid, par; phase, ..., dt, a1..b3) -- src/fluidmech.jl:71-534.

        The sparse LU of the reference is replaced by an iterative solve;
        returns its statistics.  ``mms`` = dict of src_W/src_U/src_P/W_exact/
        U_exact/P_exact host arrays selects the manufactured-solution branch."""
        c6 = (ctypes.c_double * 6)(*coefs)
        o = SolverOpts.make(solver, rtol, maxit, restart, inner_rtol, inner_maxit, **knobs)
        st = SolverStats()
        if mms is None:
            status = lib().xc_fluidmech(self._h, c6, float(dt), ctypes.byref(o), ctypes.byref(st))
        else:
            g = self.grid
            arrs = [_host(mms[k], shp) for k, shp in (
                ("src_W", (g.Nz + 1, g.Nx + 2)), ("src_U", (g.Nz + 2, g.Nx + 1)), ("src_P", (g.Nz + 2, g.Nx + 2)),
                ("W_exact", (g.Nz + 1, g.Nx + 2)), ("U_exact", (g.Nz + 2, g.Nx + 1)),
                ("P_exact", (g.Nz + 2, g.Nx + 2)))]
            status = lib().xc_fluidmech_mms(self._h, *[a.ctypes.data for a in arrs], c6, float(dt),
                                            ctypes.byref(o), ctypes.byref(st))
        _check(status)
        return {k: getattr(st, k) for k, _ in SolverStats._fields_}

    def noise(self, dt, first_iter=True, re=None, rs=None):
        """noise!(ns, phase, grid, par, scales, dt; first_iter) -- src/noise.jl:138-239.
        re/rs replace the reference's randn! draw on the first sweep."""
        g = self.grid
        a = _host(re, (g.Nz, g.Nx)) if re is not None else None
        b = _host(rs, (g.Nz, g.Nx)) if rs is not None else None
        _check(lib().xc_noise(self._h, float(dt), int(bool(first_iter)),
                              a.ctypes.data if a is not None else None, b.ctypes.data if b is not None else None))

    def update_phase_velocities(self):
        """update_phase_velocities!(phase, fluid, ns, grid, par) -- src/store.jl:80-105."""
        _check(lib().xc_update_phase_velocities(self._h))

    def update(self):
        """update!(phase, fluid, grid, par, scales) -- src/update.jl:525-538."""
        _check(lib().xc_update(self._h))

    def update_dt(self, dt_prev):
        """update_dt(phase, fluid, grid, par, dt_prev) -- src/update.jl:494-502."""
        out = ctypes.c_double()
        _check(lib().xc_update_dt(self._h, float(dt_prev), ctypes.byref(out)))
        return out.value

    def compute_resnorm(self, dt):
        """compute_resnorm(res, phase, fluid, dt) -- src/diagnose.jl:57-71:
        (resnorm, res_mass, res_mmnt) against the last snapshot; raises
        ``self.resnorm0`` to resnorm + 1e-32 when it is below resnorm."""
        out = (ctypes.c_double * 3)()
        _check(lib().xc_resnorm(self._h, float(dt), out))
        if self.resnorm0 < out[0]:
            self.resnorm0 = out[0] + 1e-32
        return tuple(out)

    def conservation_sums(self):
        """FP64 sums of record_history! -- src/history.jl:121-145."""
        out = (ctypes.c_double * 12)()
        _check(lib().xc_conservation_sums(self._h, out))
        keys = ("sumB", "sumM", "sumX", "sumGx", "top_aX", "bot_aX", "top_aM", "bot_aM", "top_dX", "bot_dX",
                "top_dM", "bot_dM")
        return dict(zip(keys, out))

    HISTORY_KEYS = (["x_min", "x_mean", "x_max", "x_std"]
                    + [f"{f}_{s}" for f in ("V", "vx", "vm", "xie", "xix", "xis") for s in ("min", "rms", "max")]
                    + [f"{f}_{s}" for f in ("Ra", "Rc", "ReD", "Red", "ks", "ke", "kx", "eta", "etamix", "etae",
                                            "etas", "etat") for s in ("min", "gm", "max")])

    def history_stats(self):
        """Field statistics of record_history! -- src/history.jl:183-222."""
        out = (ctypes.c_double * 58)()
        _check(lib().xc_history_stats(self._h, out))
        return dict(zip(self.HISTORY_KEYS, out))

    PRINT_KEYS = (["m_min", "m_mean", "m_max"]
                  + [f"{f}_{s}" for f in ("rho", "V", "vx", "vm", "xie", "xix", "xis") for s in ("min", "gm", "max")])

    def print_step_stats(self):
        """The statistics print_step! adds to record_history!'s, on the raw
        fields -- src/diagnose.jl:92-182."""
        out = (ctypes.c_double * 24)()
        _check(lib().xc_print_step_stats(self._h, out))
        return dict(zip(self.PRINT_KEYS, out))

    # ---- checkpoints -------------------------------------------------------
    def checkpoint(self):
        """The device state as save_checkpoint groups it (src/restart.jl:53-83):
        {"fluid/<name>", "phase/<name>", "noise/<name>": host array}."""
        out = {}
        for group, names in CHECKPOINT_GROUPS.items():
            for n in names:
                out[f"{group}/{n}"] = self[n]
        return out

    def restore(self, ckpt):
        """Upload every field of a checkpoint dict (load_checkpoint!,
        src/restart.jl:94-127); sizes must match this context's grid."""
        for group, names in CHECKPOINT_GROUPS.items():
            for n in names:
                self[n] = ckpt[f"{group}/{n}"]

    def save_checkpoint(self, path, time, dt, step):
        """Write the checkpoint with the reference's dataset names and the
        meta/time, meta/dt, meta/step scalars to an .npz file (no HDF5
        writer is available to Python here; the Julia binding writes the
        reference's JLD2 file through xcore.save_checkpoint)."""
        d = self.checkpoint()
        d.update({"meta/time": np.float64(time), "meta/dt": np.float64(dt), "meta/step": np.int64(step)})
        with open(path, "wb") as f:
            np.savez(f, **d)

    def load_checkpoint(self, path):
        """Read a file written by save_checkpoint into this context; returns
        (time, dt, step) to resume the time loop."""
        with np.load(path) as z:
            self.restore({k: z[k] for k in z.files})
            return float(z["meta/time"]), float(z["meta/dt"]), int(z["meta/step"])

    def initialize(self, x_init, re, rs):
        """Fresh-start initialize! -- src/run.jl:71-140 (x_init replaces the
        seeded perturbation, re/rs the first noise draw)."""
        g = self.grid
        x = _host(x_init, (g.Nz, g.Nx))
        a, b = _host(re, (g.Nz, g.Nx)), _host(rs, (g.Nz, g.Nx))
        _check(lib().xc_initialize(self._h, x.ctypes.data, a.ctypes.data, b.ctypes.data))

    def _draws(self, re, rs):
        g = self.grid
        a = _host(re, (g.Nz, g.Nx)) if re is not None else None
        b = _host(rs, (g.Nz, g.Nx)) if rs is not None else None
        return a, b, (a.ctypes.data if a is not None else None), (b.ctypes.data if b is not None else None)

    @staticmethod
    def _step_result(status, st):
        """The step's statistics; a non-converged Stokes solve raises
        NotConverged carrying them (the step itself was completed)."""
        info = st.as_dict()
        if status == XC_NOT_CONVERGED:
            err = NotConverged(status, lib().xc_last_error().decode())
            err.info = info
            raise err
        _check(status)
        return info

    def step(self, step, dt, re=None, rs=None, sweeps=3, solver="fgmres64", rtol=1e-10, maxit=500,
             restart=30, inner_rtol=1e-4, inner_maxit=60, **knobs):
        """One outer step of run! (src/run.jl:204-274) with `sweeps` Picard
        sweeps (the reference's loop with maxit = sweeps, rtol = atol = 0)."""
        a, b, pa, pb = self._draws(re, rs)
        o = SolverOpts.make(solver, rtol, maxit, restart, inner_rtol, inner_maxit, **knobs)
        st = StepStats()
        status = lib().xc_step(self._h, int(step), float(dt), int(sweeps), pa, pb, ctypes.byref(o),
                               ctypes.byref(st))
        return self._step_result(status, st)

    def step_converge(self, step, dt, re=None, rs=None, picard_rtol=1e-4, picard_atol=1e-9, picard_maxit=15,
                      solver="fgmres64", rtol=1e-10, maxit=500, restart=30, inner_rtol=1e-4, inner_maxit=60,
                      **knobs):
        """One outer step of run! with the reference's own Picard loop
        (src/run.jl:220-250): at least 3 sweeps, then on while
        resnorm/resnorm0 >= picard_rtol and resnorm >= picard_atol and fewer
        than picard_maxit sweeps ran (par.rtol, par.atol, par.maxit,
        src/parameters.jl:76-78)."""
        a, b, pa, pb = self._draws(re, rs)
        o = SolverOpts.make(solver, rtol, maxit, restart, inner_rtol, inner_maxit, **knobs)
        st = StepStats()
        status = lib().xc_step_converge(self._h, int(step), float(dt), float(picard_rtol), float(picard_atol),
                                        int(picard_maxit), pa, pb, ctypes.byref(o), ctypes.byref(st))
        return self._step_result(status, st)


class Ensemble:
    """Independent instances -- grid sizes, parameters and noise seeds may all
    differ -- advanced together on one GPU, each member a ``State`` with its
    own device context and CUDA stream.  Two drivers, both leaving every
    member bit-identical to the same instance stepped alone:

    * ``graphs=False``: one host thread per member runs ``State.step`` (ctypes
      releases the GIL for each library call), so the kernels of different
      members overlap on the GPU where one small instance alone would leave
      it idle between launches;
    * ``graphs=True``: one ``xc_ensemble_step`` call per time step, in which
      every explicit stage of a Picard sweep is one CUDA graph launch holding
      all members' kernels of that stage, and the Stokes solves run on
      ``threads`` host threads of the library (default one per member).  Only
      the fixed-sweep step (``sweeps``) is available this way."""

    def __init__(self, members, threads=None, graphs=False):
        self.members = list(members)
        self.graphs = bool(graphs)
        self._pool = None
        self._h = None
        if self.graphs:
            n = len(self.members)
            arr = (ctypes.c_void_p * n)(*[m._h.value for m in self.members])
            h = ctypes.c_void_p()
            _check(lib().xc_ensemble_create(arr, n, int(threads or 0), ctypes.byref(h)))
            self._h = h
        else:
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(max_workers=threads or max(1, len(self.members)))

    def step(self, steps, dts, draws, **solver):
        """One time step of every member: ``steps[i]``, ``dts[i]`` and the
        noise draws ``draws[i] = (re, rs)`` of member i (either may be None:
        the device draws are kept); ``solver`` as for ``State.step``.  Returns
        the members' step statistics in order."""
        if not self.graphs:
            futs = [self._pool.submit(m.step, steps[i], dts[i], draws[i][0], draws[i][1], **solver)
                    for i, m in enumerate(self.members)]
            return [f.result() for f in futs]
        n = len(self.members)
        kw = dict(solver)
        sweeps = int(kw.pop("sweeps", 3))
        o = SolverOpts.make(kw.pop("solver", "fgmres64"), kw.pop("rtol", 1e-10), kw.pop("maxit", 500),
                            kw.pop("restart", 30), kw.pop("inner_rtol", 1e-4), kw.pop("inner_maxit", 60), **kw)
        host = [m._draws(re, rs) for m, (re, rs) in zip(self.members, draws)]   # kept alive for the call
        re_p = (ctypes.c_void_p * n)(*[h[2] for h in host])
        rs_p = (ctypes.c_void_p * n)(*[h[3] for h in host])
        st = (StepStats * n)()
        status = lib().xc_ensemble_step(self._h, (ctypes.c_int * n)(*[int(k) for k in steps]),
                                        (ctypes.c_double * n)(*[float(d) for d in dts]), sweeps, re_p, rs_p,
                                        ctypes.byref(o), st)
        infos = [s.as_dict() for s in st]
        if status == XC_NOT_CONVERGED:
            err = NotConverged(status, lib().xc_last_error().decode())
            err.info = infos
            raise err
        _check(status)
        return infos

    def close(self):
        """Release the ensemble and close its members."""
        if self._h is not None:
            lib().xc_ensemble_destroy(self._h)
            self._h = None
        if self._pool is not None:
            self._pool.shutdown()
        for m in self.members:
            m.close()

    def __del__(self):
        # the library's ensemble (streams, events, host threads); the members
        # close themselves
        try:
            if self._h is not None:
                lib().xc_ensemble_destroy(self._h)
                self._h = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
# stencil-level functions on device arrays (torch CUDA tensors laid out
# column-major: a (rows, cols) Julia matrix is a contiguous torch tensor of
# shape (cols, rows))
# ---------------------------------------------------------------------------


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    return ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)


def fill_ghosts(f, halo, zBC="closed", xBC="periodic", stream=None):
    """fill_ghosts!(f, halo; zBC, xBC) -- src/kernels/ghosts.jl:18-51."""
    Nx, Nz = f.shape[0] - 2 * halo, f.shape[1] - 2 * halo
    _check(lib().xc_fill_ghosts(_ptr(f), Nz, Nx, halo, BCS[zBC], BCS[xBC], _stream(stream)))


def advect(adv, f_halo, u, w, h, scheme, stream=None):
    """advect!(adv, f_halo, u, w, h, scheme) -- src/kernels/advect.jl:374-425."""
    Nx, Nz = adv.shape
    _check(lib().xc_advect(_ptr(adv), _ptr(f_halo), _ptr(u), _ptr(w), Nz, Nx, float(h), SCHEMES[scheme],
                           _stream(stream)))


def advect_with_flux(adv, qx, qz, f_halo, u, w, h, scheme, xBC="periodic", zBC="closed", stream=None):
    """advect_with_flux! -- src/kernels/advect.jl:717-798."""
    Nx, Nz = adv.shape
    _check(lib().xc_advect_with_flux(_ptr(adv), _ptr(qx), _ptr(qz), _ptr(f_halo), _ptr(u), _ptr(w), Nz, Nx,
                                     float(h), SCHEMES[scheme], BCS[xBC], BCS[zBC], _stream(stream)))


def advect_centered_with_flux(adv, qx, qz, f, u, w, h, scheme, xBC="periodic", zBC="closed", stream=None):
    """advect_centered_with_flux! -- src/phsevo.jl:90-128 (qx/qz may be None)."""
    Nx, Nz = adv.shape
    _check(lib().xc_advect_centered_with_flux(_ptr(adv), _ptr(qx) if qx is not None else None,
                                              _ptr(qz) if qz is not None else None, _ptr(f), _ptr(u), _ptr(w),
                                              Nz, Nx, float(h), SCHEMES[scheme], BCS[xBC], BCS[zBC],
                                              _stream(stream)))


def diffus(dff, f_halo, k_halo, h, stream=None):
    """diffus!(dff, f_halo, k_halo, h) -- src/kernels/diffus.jl:109-121."""
    Nx, Nz = dff.shape
    _check(lib().xc_diffus(_ptr(dff), _ptr(f_halo), _ptr(k_halo), Nz, Nx, float(h), _stream(stream)))


def diffus_with_flux(dff, qx, qz, f_halo, k_halo, h, xBC="periodic", zBC="closed", stream=None):
    """diffus_with_flux! -- src/kernels/diffus.jl:169-211."""
    Nx, Nz = dff.shape
    _check(lib().xc_diffus_with_flux(_ptr(dff), _ptr(qx), _ptr(qz), _ptr(f_halo), _ptr(k_halo), Nz, Nx,
                                     float(h), BCS[xBC], BCS[zBC], _stream(stream)))


def launch_count() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(lib().xc_launch_count())
