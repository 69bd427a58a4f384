"""CPU oracle for the xcore.jl per-timestep hot path -- TEST INFRASTRUCTURE ONLY.

This module is a numpy restatement of the reference algorithm (aelligp/xcore.jl,
pure Julia).  It exists to CHECK the GB300 library: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it, and never as the thing measured or shipped.

Parity status.  The reference is Julia and Julia is not installed here, so no
reference-run golden vectors exist.  This restatement is pinned by the
reference's own known-answer tests, re-implemented in ``tests/test_oracle_pins.py``:
exact ghost-fill values (test/test_stencils.jl:37-56), time_coefs tuples
(test/test_run.jl:5-25), the store_previous! shift chain (test/test_run.jl:27-46),
rheology against the naive permission-weight reference at rtol 1e-12
(test/test_update.jl:8-47), advection / diffusion / strain-rate / MMS-Stokes
convergence orders (test/test_advect.jl, test/test_diffus.jl,
test/test_update.jl:49-94, test/test_mms.jl) and resnorm == 0 with no change
(test/test_diagnose.jl:52-63).  Per-field VALUES beyond those are therefore
"parity partially pinned": they follow the reference's operation order line by
line, but Julia's own reduction order (pairwise / SIMD sums, BLAS nrm2), its
libm (exp, pow) and its third-party dependencies cannot be reproduced bit for
bit without Julia.

Third-party dependencies of the reference that are absent here:
  * FFTW (FFTW.jl, Project.toml:11, compat "1"; no Manifest, so unpinned) --
    call sites src/noise.jl:100-101 (fftfreq) and 254-256 (fft/ifft).  Its
    published algorithm is the exact DFT; numpy's pocketfft stands in.
  * UMFPACK (SuiteSparse via Julia's SparseArrays stdlib, unpinned) -- call
    sites src/fluidmech.jl:513,516,522.  scipy's SuperLU (splu) stands in; the
    two agree to about cond(LL)*eps, not bitwise.
  * Random.MersenneTwister + randn! (src/noise.jl:155-156, src/run.jl:99) --
    not reproducible without Julia, so white-noise draws and the initial
    perturbation are INPUTS here, fed identically to the oracle and the GPU.

Conventions: every field is a float64 numpy array indexed [z, x] (the
reference's column-major Julia matrices, z the leading dimension), with exactly
the reference's sizes (src/state.jl:101-122, 218-258; src/noise.jl:82-92).
Index comments use 0-based numpy indices.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EPS = float(np.finfo(np.float64).eps)
SQRT_EPS = math.sqrt(EPS)


def jl_max(a, b):
    """Julia's ``max`` of Float64 values, elementwise with broadcasting: NaN
    if either argument is NaN, and -0.0 < +0.0, so max(0.0, -0.0) is +0.0
    in either order (numpy's maximum returns its second argument for two
    zeros)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    r = np.where(a > b, a, np.where(b > a, b, np.where(np.signbit(a), b, a)))
    return np.where(np.isnan(a) | np.isnan(b), a + b, r)


def jl_min(a, b):
    """Julia's ``min`` of Float64 values (NaN propagates; min(0.0, -0.0) is
    -0.0 in either order)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    r = np.where(a < b, a, np.where(b < a, b, np.where(np.signbit(a), a, b)))
    return np.where(np.isnan(a) | np.isnan(b), a + b, r)


def jl_maximum(a) -> float:
    """Julia's ``maximum`` of a Float64 array: NaN if any element is NaN
    (numpy's max agrees), and +0.0 when the largest value is a zero and any
    zero is +0.0 (numpy may return either zero)."""
    a = np.asarray(a, dtype=np.float64)
    m = float(a.max())
    if m == 0.0:
        return 0.0 if (~np.signbit(a[a == 0.0])).any() else -0.0
    return m


def jl_minimum(a) -> float:
    """Julia's ``minimum`` of a Float64 array (NaN propagates; -0.0 when the
    smallest value is a zero and any zero is -0.0)."""
    a = np.asarray(a, dtype=np.float64)
    m = float(a.min())
    if m == 0.0:
        return -0.0 if np.signbit(a[a == 0.0]).any() else 0.0
    return m


# ---------------------------------------------------------------------------
# parameters, grid, scales  (src/parameters.jl:12-89, src/grid.jl:311-334,
#                            src/scales.jl:85-185)
# ---------------------------------------------------------------------------


@dataclass
class Params:
    """Subset of ``Parameters{Float64}`` (src/parameters.jl:12-89) the path reads."""
    D: float = 10.0
    N: int = 100
    L: float = 10.0
    x0: float = EPS
    dxr: float = 0.1
    dxg: float = 0.0
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
    rtol: float = 1e-4
    atol: float = 1e-9
    maxit: int = 15
    alpha: float = 0.9
    gamma: float = 1e-3
    dtmax: float = 1e32
    etacntr: float = 1e8


def julia_round(x: float) -> int:
    """Julia ``round(Int, x)``: round half to even (Python's ``round`` does the same)."""
    return int(round(x))


@dataclass
class Grid:
    """src/grid.jl:311-334."""
    Nx: int
    Nz: int
    h: float
    D: float
    L: float


def make_grid(p: Params) -> Grid:
    h = p.D / p.N
    Nx = max(1, julia_round(p.L / h))
    return Grid(Nx=Nx, Nz=p.N, h=h, D=p.D, L=p.L)


def compute_scales(p: Params, g: Grid, tol: float = 1e-9, maxiter: int = 200) -> dict:
    """Fixed point of src/scales.jl:85-185 in Float64 (host scalars)."""
    D, d0, x0, Da = p.D, p.d0, p.x0, p.Da
    rhom0, rhox0, etam0, g0, Xi, h = p.rhom0, p.rhox0, p.etam0, p.g0, p.Xi, g.h
    h0 = h
    D0 = D / 10
    L0 = p.L0
    L0h = (L0 + h0) / 2
    l0 = p.l0
    l0h = (l0 + h0) / 2
    bnd_w = l0 / 2 + D / 100
    rho0 = rhom0
    Drho0 = rhox0 - rhom0
    if Da > 0:
        chi0, Dchi0 = Da, Da / 10
    else:
        chi0, Dchi0 = x0, x0 / 10
    eta0 = etam0
    W0l = Dchi0 * Drho0 * g0 * (D0 * D0) / eta0
    w0l = Drho0 * g0 * (d0 * d0) / eta0
    w0t = math.sqrt(Drho0 * g0 * (d0 * d0) / (l0 * rho0))
    W0t = math.sqrt(Dchi0 * Drho0 * g0 * (D0 * D0 * D0) / ((L0 * L0) * rho0))
    W0i = math.sqrt(Dchi0 * Drho0 * g0 * D / rho0)
    Ri0 = W0i / W0t
    W0, w0 = W0l, w0l
    ReL0 = W0 * L0 / (eta0 / rho0)
    Rel0 = w0 * l0 / (eta0 / rho0)
    fReL0 = 1 - math.exp(-ReL0)
    fRel0 = 1 - math.exp(-Rel0)
    for _ in range(maxiter):
        W0prv, w0prv = W0, w0
        ReL0 = W0 * L0 / (eta0 / rho0)
        Rel0 = w0 * l0 / (eta0 / rho0)
        fReL0 = 1 - math.exp(-ReL0)
        fRel0 = 1 - math.exp(-Rel0)
        Ri2 = Ri0 * Ri0
        W0 = (math.sqrt(4 / Ri2 * Dchi0 * Drho0 * g0 * rho0 * fReL0 * (L0 * L0) * D0 + eta0 * eta0) - eta0) \
            * D0 / (2 * fReL0 * (L0 * L0) * rho0 / Ri2)
        w0 = (math.sqrt(4 * Drho0 * g0 * rho0 * fRel0 * l0 * (d0 * d0) + eta0 * eta0) - eta0) \
            / (2 * fRel0 * l0 * rho0)
        res = abs(W0 - W0prv) / W0 + abs(w0 - w0prv) / w0
        if res <= tol:
            break
    eII0 = W0 / D0
    ke0 = eII0 * (L0 * L0)
    ks0 = w0 * l0
    kx0 = ks0 + fReL0 * ke0
    tW0 = D / W0
    tw0 = D / w0
    tk0 = (D * D) / kx0
    ti0 = D / W0i
    txi0 = rhox0 * (d0 * d0) / 18 / eta0
    t0 = 1.0 / (1 / (ti0 + tW0) + 1 / tw0 + 1 / tk0)
    dt0 = min((h0 / 2) * (h0 / 2) / kx0, (h0 / 2) / (W0 + w0))
    G0 = Da * rho0 / t0 * D / D0
    return dict(h0=h0, D0=D0, d0=d0, L0=L0, L0h=L0h, l0=l0, l0h=l0h, bnd_w=bnd_w,
                rho0=rho0, Drho0=Drho0, chi0=chi0, Dchi0=Dchi0, eta0=eta0, W0=W0, w0=w0,
                ReL0=ReL0, Rel0=Rel0, fReL0=fReL0, fRel0=fRel0, ke0=ke0, ks0=ks0, kx0=kx0,
                txi0=txi0, t0=t0, dt0=dt0, G0=G0, Ri0=Ri0, W0l=W0l)


def time_coefs(TINT: str, step: int):
    """src/timing.jl:18-36."""
    if TINT.endswith("im"):
        if TINT == "be1im" or step <= 2:
            return (1.0, 1.0, 0.0, 1.0, 0.0, 0.0)
        if TINT == "bd2im":
            return (1.5, 2.0, -0.5, 1.0, 0.0, 0.0)
    elif TINT.endswith("si"):
        if step == 1:
            return (1.0, 1.0, 0.0, 1.0, 0.0, 0.0)
        if TINT == "cn2si" or step == 2:
            return (1.0, 1.0, 0.0, 0.5, 0.5, 0.0)
        if TINT == "bd2si":
            return (1.5, 2.0, -0.5, 0.75, 0.5, -0.25)
    raise ValueError(f"time_coefs: unsupported TINT scheme {TINT}")


def icx_of(Nx: int, xBC: str) -> np.ndarray:
    """Ghost index vector [Nx; 1:Nx; 1] (periodic) or [1; 1:Nx; Nx], 0-based."""
    mid = np.arange(Nx)
    return np.concatenate(([Nx - 1], mid, [0])) if xBC == "periodic" else np.concatenate(([0], mid, [Nx - 1]))


def icz_of(Nz: int, zBC: str) -> np.ndarray:
    mid = np.arange(Nz)
    return np.concatenate(([Nz - 1], mid, [0])) if zBC == "periodic" else np.concatenate(([0], mid, [Nz - 1]))


# ---------------------------------------------------------------------------
# halo fill  (src/kernels/ghosts.jl:18-64)
# ---------------------------------------------------------------------------


def fill_ghosts(f: np.ndarray, halo: int, zBC: str = "closed", xBC: str = "periodic") -> np.ndarray:
    Nzt, Nxt = f.shape
    Nz, Nx = Nzt - 2 * halo, Nxt - 2 * halo
    assert Nz >= 1 and Nx >= 1
    if xBC == "periodic":
        f[:, 0:halo] = f[:, Nx:Nx + halo]
        f[:, Nx + halo:Nxt] = f[:, halo:2 * halo]
    elif xBC == "closed":
        for k in range(halo):
            f[:, k] = f[:, halo]
            f[:, Nx + halo + k] = f[:, Nx + halo - 1]
    else:
        raise ValueError(f"fill_ghosts: unsupported xBC = {xBC}")
    if zBC == "periodic":
        f[0:halo, :] = f[Nz:Nz + halo, :]
        f[Nz + halo:Nzt, :] = f[halo:2 * halo, :]
    elif zBC == "closed":
        for k in range(halo):
            f[k, :] = f[halo, :]
            f[Nz + halo + k, :] = f[Nz + halo - 1, :]
    else:
        raise ValueError(f"fill_ghosts: unsupported zBC = {zBC}")
    return f


def embed_halo(f: np.ndarray, halo: int, zBC: str, xBC: str) -> np.ndarray:
    """advect_centered!/diffus_centered! halo preparation (src/phsevo.jl:26-30)."""
    fh = np.zeros((f.shape[0] + 2 * halo, f.shape[1] + 2 * halo))
    fh[halo:halo + f.shape[0], halo:halo + f.shape[1]] = f
    return fill_ghosts(fh, halo, zBC=zBC, xBC=xBC)


# ---------------------------------------------------------------------------
# advection  (src/kernels/advect.jl)
# ---------------------------------------------------------------------------

SCHEME_HALO = {"centr": 1, "upwd1": 1, "quick": 2, "fromm": 2, "weno3": 2, "weno5": 3, "tvdim": 2}


def scheme_halo(scheme: str) -> int:
    """src/kernels/advect.jl:346-355."""
    if scheme not in SCHEME_HALO:
        raise ValueError(f"scheme_halo: unsupported scheme = :{scheme}")
    return SCHEME_HALO[scheme]


def weno5_poly(fmm, fm, fc, fp, fpp, eps_val):
    """Jiang-Shu face value, src/kernels/advect.jl:35-53 (same operation order)."""
    sixth = 1.0 / 6.0
    quarter = 0.25
    c1312 = 13.0 / 12.0
    p1 = sixth * ((2.0 * fmm - 7.0 * fm) + 11.0 * fc)
    p2 = sixth * ((-fm + 5.0 * fc) + 2.0 * fp)
    p3 = sixth * ((2.0 * fc + 5.0 * fp) - fpp)
    t = (fmm - 2.0 * fm) + fc
    s = (fmm - 4.0 * fm) + 3.0 * fc
    b1 = c1312 * (t * t) + quarter * (s * s)
    t = (fm - 2.0 * fc) + fp
    s = fm - fp
    b2 = c1312 * (t * t) + quarter * (s * s)
    t = (fc - 2.0 * fp) + fpp
    s = (3.0 * fc - 4.0 * fp) + fpp
    b3 = c1312 * (t * t) + quarter * (s * s)
    e1 = b1 + eps_val
    e2 = b2 + eps_val
    e3 = b3 + eps_val
    w1 = 0.1 / (e1 * e1)
    w2 = 0.6 / (e2 * e2)
    w3 = 0.3 / (e3 * e3)
    return ((w1 * p1 + w2 * p2) + w3 * p3) / ((w1 + w2) + w3)


def weno3_poly(fm, fc, fp, eps_val):
    """src/kernels/advect.jl:216-229."""
    half = 0.5
    p1 = half * (fc + fp)
    p2 = half * (3.0 * fc - fm)
    d1 = fp - fc
    d2 = fc - fm
    w1 = (1.0 / 3.0) / (d1 * d1 + eps_val)
    w2 = (2.0 / 3.0) / (d2 * d2 + eps_val)
    return (w1 * p1 + w2 * p2) / (w1 + w2)


def tvd_flux(fm, fc, fp, vm, vp):
    """Superbee-limited face value, src/kernels/advect.jl:275-283."""
    num = vm * (fc - fm)
    den = vp * (fp - fc)
    R = num / (den + np.copysign(EPS, den))
    lim = jl_max(0.0, jl_max(jl_min(1.0, 2.0 * R), jl_min(2.0, R)))
    return fc + (0.5 * lim) * (fp - fc)


def _split(v):
    a = np.abs(v)
    return (v + a) * 0.5, (v - a) * 0.5


def _face_values(s0, s1, s2, s3, s4, s5, scheme):
    """Left-biased (pos) and right-biased (neg) face values at the face between
    cells s2 and s3, from the six cells s0..s5 around it.  These are the per-face
    formulas of the flux kernels, src/kernels/advect.jl:444-637, which equal the
    divergence kernels' face values bitwise (advect.jl:428-432)."""
    if scheme == "centr":
        return None
    if scheme == "upwd1":
        return s2, s3
    if scheme == "quick":
        sixth = 1.0 / 6.0
        return sixth * ((2.0 * s3 + 5.0 * s2) - s1), sixth * ((2.0 * s2 + 5.0 * s3) - s4)
    if scheme == "fromm":
        return s2 + 0.25 * (s3 - s1), s3 + 0.25 * (s2 - s4)
    if scheme == "weno3":
        return weno3_poly(s1, s2, s3, 1e-6), weno3_poly(s4, s3, s2, 1e-6)
    if scheme == "weno5":
        return weno5_poly(s0, s1, s2, s3, s4, EPS), weno5_poly(s5, s4, s3, s2, s1, EPS)
    raise ValueError(scheme)


def _pad_velocity_tvd(u, w, xBC, zBC):
    """TVD velocity padding, src/phsevo.jl:34-53."""
    Nz, Nxp1 = u.shape
    Nx = Nxp1 - 1
    u_pad = np.empty((Nz, Nx + 3))
    w_pad = np.empty((w.shape[0] + 2, w.shape[1]))
    Nzw = w.shape[0] - 1
    u_pad[:, 1:Nx + 2] = u
    w_pad[1:Nzw + 2, :] = w
    if xBC == "periodic":
        u_pad[:, 0] = u[:, Nx - 1]
        u_pad[:, Nx + 2] = u[:, 1]
    else:
        u_pad[:, 0] = u[:, 0]
        u_pad[:, Nx + 2] = u[:, Nx]
    if zBC == "periodic":
        w_pad[0, :] = w[Nzw - 1, :]
        w_pad[Nzw + 2, :] = w[1, :]
    else:
        w_pad[0, :] = w[0, :]
        w_pad[Nzw + 2, :] = w[Nzw, :]
    return u_pad, w_pad


def advect_fluxes(fh, u, w, scheme, g):
    """Interior face fluxes qx_int (Nz, Nx+1) and qz_int (Nz+1, Nx) from a halo'd
    field fh (halo g).  For tvdim, u/w are the padded velocities.
    src/kernels/advect.jl:444-695."""
    Nz, Nx = fh.shape[0] - 2 * g, fh.shape[1] - 2 * g
    # x-faces: face ix (0..Nx) sits between cells ix-1 and ix, i.e. halo'd
    # columns g+ix-1 and g+ix.
    rows = slice(g, g + Nz)

    def colx(off):
        return fh[rows, g + off: g + off + Nx + 1]

    def rowz(off):
        return fh[g + off: g + off + Nz + 1, g:g + Nx]

    if scheme == "centr":
        qx = u * (colx(-1) + colx(0)) * 0.5
        qz = w * (rowz(-1) + rowz(0)) * 0.5
        return qx, qz
    if scheme == "tvdim":
        # x: fppos = tvd(f[ix-2], f[ix-1], f[ix], upos[face ix-1], upos[face ix])
        ul = u[:, 0:Nx + 1]
        uc = u[:, 1:Nx + 2]
        ur = u[:, 2:Nx + 3]
        ulpos, _ = _split(ul)
        ucpos, ucneg = _split(uc)
        _, urneg = _split(ur)
        fppos = tvd_flux(colx(-2), colx(-1), colx(0), ulpos, ucpos)
        fpneg = tvd_flux(colx(1), colx(0), colx(-1), urneg, ucneg)
        qx = ucpos * fppos + ucneg * fpneg
        wt = w[0:Nz + 1, :]
        wc = w[1:Nz + 2, :]
        wb = w[2:Nz + 3, :]
        wtpos, _ = _split(wt)
        wcpos, wcneg = _split(wc)
        _, wbneg = _split(wb)
        fppos = tvd_flux(rowz(-2), rowz(-1), rowz(0), wtpos, wcpos)
        fpneg = tvd_flux(rowz(1), rowz(0), rowz(-1), wbneg, wcneg)
        qz = wcpos * fppos + wcneg * fpneg
        return qx, qz
    h3 = g >= 3
    pos, neg = _face_values(colx(-3) if h3 else None, colx(-2) if g >= 2 else None, colx(-1), colx(0),
                            colx(1) if g >= 2 else None, colx(2) if h3 else None, scheme)
    upos, uneg = _split(u)
    qx = upos * pos + uneg * neg
    pos, neg = _face_values(rowz(-3) if h3 else None, rowz(-2) if g >= 2 else None, rowz(-1), rowz(0),
                            rowz(1) if g >= 2 else None, rowz(2) if h3 else None, scheme)
    wpos, wneg = _split(w)
    qz = wpos * pos + wneg * neg
    return qx, qz


def divergence(qx, qz, invh):
    """adv = (qxr - qxl + qzb - qzt) * invh, src/kernels/advect.jl:94."""
    return (((qx[:, 1:] - qx[:, :-1]) + qz[1:, :]) - qz[:-1, :]) * invh


def advect_centered(f, u, w, h, scheme, xBC="periodic", zBC="closed"):
    """advect_centered! (src/phsevo.jl:21-59) -> adv (Nz, Nx)."""
    g = scheme_halo(scheme)
    fh = embed_halo(f, g, zBC, xBC)
    if scheme == "tvdim":
        u, w = _pad_velocity_tvd(u, w, xBC, zBC)
    qx, qz = advect_fluxes(fh, u, w, scheme, g)
    return divergence(qx, qz, 1.0 / h)


def pad_face_fluxes(qx_int, qz_int, xBC, zBC):
    """MATLAB-sized flux arrays with boundary fills, src/kernels/advect.jl:779-795."""
    Nz, Nxp1 = qx_int.shape
    Nx = Nxp1 - 1
    qx = np.zeros((Nz + 2, Nx + 1))
    qz = np.zeros((Nz + 1, Nx + 2))
    qx[1:Nz + 1, :] = qx_int
    qz[:, 1:Nx + 1] = qz_int
    if xBC == "periodic" and Nx > 1:
        qz[:, 0] = qz[:, Nx]
        qz[:, Nx + 1] = qz[:, 1]
    else:
        qz[:, 0] = qz[:, 1]
        qz[:, Nx + 1] = qz[:, Nx]
    if zBC == "periodic" and Nz > 1:
        qx[0, :] = qx[Nz, :]
        qx[Nz + 1, :] = qx[1, :]
    else:
        qx[0, :] = qx[1, :]
        qx[Nz + 1, :] = qx[Nz, :]
    return qx, qz


def advect_centered_with_flux(f, u, w, h, scheme, xBC="periodic", zBC="closed"):
    """advect_centered_with_flux! (src/phsevo.jl:90-128) -> (adv, qx, qz)."""
    g = scheme_halo(scheme)
    fh = embed_halo(f, g, zBC, xBC)
    if scheme == "tvdim":
        u, w = _pad_velocity_tvd(u, w, xBC, zBC)
    qxi, qzi = advect_fluxes(fh, u, w, scheme, g)
    adv = divergence(qxi, qzi, 1.0 / h)
    qx, qz = pad_face_fluxes(qxi, qzi, xBC, zBC)
    return adv, qx, qz


# ---------------------------------------------------------------------------
# diffusion  (src/kernels/diffus.jl)
# ---------------------------------------------------------------------------


def diffus_halo(fh, kh, h):
    """_diffus_kernel! (src/kernels/diffus.jl:9-31) on halo-1 inputs."""
    invh = 1.0 / h
    invh2 = invh * invh
    fc = fh[1:-1, 1:-1]
    kc = kh[1:-1, 1:-1]
    fxr = (kh[1:-1, 2:] + kc) * (fh[1:-1, 2:] - fc)
    fxl = (kc + kh[1:-1, :-2]) * (fc - fh[1:-1, :-2])
    fzb = (kh[2:, 1:-1] + kc) * (fh[2:, 1:-1] - fc)
    fzt = (kc + kh[:-2, 1:-1]) * (fc - fh[:-2, 1:-1])
    return (0.5 * invh2) * (((fxr - fxl) + fzb) - fzt)


def diffus_centered_with_flux(f, k, h, xBC="periodic", zBC="closed"):
    """diffus_centered_with_flux! (src/phsevo.jl:135-149, src/kernels/diffus.jl:105-147)."""
    fh = embed_halo(f, 1, zBC, xBC)
    kh = embed_halo(k, 1, zBC, xBC)
    dff = diffus_halo(fh, kh, h)
    invh = 1.0 / h
    Nz, Nx = f.shape
    fL = fh[1:Nz + 1, 0:Nx + 1]
    fR = fh[1:Nz + 1, 1:Nx + 2]
    kL = kh[1:Nz + 1, 0:Nx + 1]
    kR = kh[1:Nz + 1, 1:Nx + 2]
    qxi = ((-(kL + kR)) * 0.5 * (fR - fL)) * invh
    fT = fh[0:Nz + 1, 1:Nx + 1]
    fB = fh[1:Nz + 2, 1:Nx + 1]
    kT = kh[0:Nz + 1, 1:Nx + 1]
    kB = kh[1:Nz + 2, 1:Nx + 1]
    qzi = ((-(kT + kB)) * 0.5 * (fB - fT)) * invh
    qx, qz = pad_face_fluxes(qxi, qzi, xBC, zBC)
    return dff, qx, qz


# ---------------------------------------------------------------------------
# state containers  (src/state.jl, src/noise.jl)
# ---------------------------------------------------------------------------

def field_shapes(Nz: int, Nx: int) -> dict:
    """Sizes of every FluidState / PhaseState / NoiseState field on the path."""
    c = (Nz, Nx)
    zf = (Nz + 1, Nx)
    xf = (Nz, Nx + 1)
    wf = (Nz + 1, Nx + 2)
    uf = (Nz + 2, Nx + 1)
    co = (Nz + 1, Nx + 1)
    qx = (Nz + 2, Nx + 1)
    qz = (Nz + 1, Nx + 2)
    s = {}
    # FluidState (src/state.jl:101-122)
    s.update(W=wf, U=uf, P=(Nz + 2, Nx + 2), eta=c, etaco=co, rho=c, rhow=zf, rhou=xf, Drho=zf,
             rhoo=c, rhooo=c, drhodt=c, drhodto=c, drhodtoo=c, MFS=c,
             rhoWo=zf, rhoWoo=zf, rhoUo=xf, rhoUoo=xf)
    # PhaseState (src/state.jl:218-258)
    s.update(x=c, m=c, X=c, M=c, Xo=c, Xoo=c, Mo=c, Moo=c, chi=c, mu=c, hasx=c, hasm=c,
             chiw=wf, muw=wf, chiu=uf, muu=uf, x_w=zf, m_w=zf, x_u=xf, m_u=xf,
             Drhom=zf, Drhox=zf, Pl=c, Pt=c, etamix=c, etae=c, ke=c, kx=c,
             etat=c, etas=c, etasw=zf, ks=c, V=c, Div_V=c, exx=c, ezz=c, exz=co, eII=c,
             vx=c, vm=c, txx=c, tzz=c, txz=co, tII=c, fReL=c, ReL=c, ReD=c, Ra=c,
             fRel=c, Rel=c, Red=c, Rc=c, Wx=wf, Wm=wf, Ux=uf, Um=uf, wx=wf, wm=wf,
             bndtaperw=wf, bndshape=c, advn_X=c, advn_M=c, advn_rho=c,
             qx_advn_X=qx, qz_advn_X=qz, qx_advn_M=qx, qz_advn_M=qz,
             qx_dffn_X=qx, qz_dffn_X=qz, qx_dffn_M=qx, qz_dffn_M=qz,
             dffn_X=c, Gx=c, dXdt=c, dXdto=c, dXdtoo=c)
    # NoiseState (src/noise.jl:82-92)
    s.update(psie=c, psix=c, psis=c, psieo=c, psixo=c, psiso=c, re=c, rs=c,
             xiew=wf, xieu=uf, xixw=wf, xixu=uf, xisw=wf, xisu=uf, xie=c, xix=c, xis=c)
    return s


class State:
    """All path fields as numpy float64 arrays (hasx/hasm as float 0/1)."""

    def __init__(self, Nz: int, Nx: int):
        self.Nz, self.Nx = Nz, Nx
        for k, shp in field_shapes(Nz, Nx).items():
            setattr(self, k, np.zeros(shp))

    def copy(self) -> "State":
        s = State.__new__(State)
        s.__dict__ = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()}
        return s


# ---------------------------------------------------------------------------
# phsevo!  (src/phsevo.jl:164-214)
# ---------------------------------------------------------------------------


def phsevo(st: State, grid: Grid, par: Params, sc: dict, ADVN, coefs, dt, alpha=None,
           xBC="periodic", zBC="closed"):
    a1, a2, a3, b1, b2, b3 = coefs
    alpha = par.alpha if alpha is None else alpha
    h = grid.h
    Wx_face = st.Wx[:, 1:-1]
    Wm_face = st.Wm[:, 1:-1]
    Ux_face = st.Ux[1:-1, :]
    Um_face = st.Um[1:-1, :]
    st.advn_X, st.qx_advn_X, st.qz_advn_X = advect_centered_with_flux(st.X, Ux_face, Wx_face, h, ADVN, xBC, zBC)
    st.advn_M, st.qx_advn_M, st.qz_advn_M = advect_centered_with_flux(st.M, Um_face, Wm_face, h, ADVN, xBC, zBC)
    st.advn_rho = st.advn_X + st.advn_M
    Xkx = st.X * st.kx
    st.dffn_X, st.qx_dffn_X, st.qz_dffn_X = diffus_centered_with_flux(st.chi, Xkx, h, xBC, zBC)
    st.Gx = (sc["G0"] * (1.0 - st.x)) * st.bndshape
    st.dXdt = (-st.advn_X + st.dffn_X) + st.Gx
    res_X = ((a1 * st.X - a2 * st.Xo) - a3 * st.Xoo) - (((b1 * st.dXdt + b2 * st.dXdto) + b3 * st.dXdtoo) * dt)
    upd_X = ((-alpha) * res_X) / a1
    X = st.X + upd_X
    lo = st.rho * EPS
    hi = st.rho * (1.0 - EPS)
    X = np.where(X > hi, hi, np.where(X < lo, lo, X))
    st.X = X
    st.M = st.rho - st.X
    st.x = st.X / st.rho
    st.m = st.M / st.rho


# ---------------------------------------------------------------------------
# store.jl  (src/store.jl:13-105)
# ---------------------------------------------------------------------------


def store_previous(st: State):
    """src/store.jl:13-30."""
    st.Xoo = st.Xo.copy(); st.Xo = st.X.copy()
    st.Moo = st.Mo.copy(); st.Mo = st.M.copy()
    st.dXdtoo = st.dXdto.copy(); st.dXdto = st.dXdt.copy()
    st.rhooo = st.rhoo.copy(); st.rhoo = st.rho.copy()
    st.drhodtoo = st.drhodto.copy(); st.drhodto = st.drhodt.copy()
    st.rhoWoo = st.rhoWo.copy(); st.rhoWo = st.rhow * st.W[:, 1:-1]
    st.rhoUoo = st.rhoUo.copy(); st.rhoUo = st.rhou * st.U[1:-1, :]


def store_noise(st: State):
    """src/noise.jl:115-120."""
    st.psieo = st.psie.copy(); st.psixo = st.psix.copy(); st.psiso = st.psis.copy()


def update_segregation_speed(st: State, grid: Grid, par: Params, xBC="periodic"):
    """src/store.jl:47-68."""
    icx = icx_of(grid.Nx, xBC)
    st.wx[:, 1:-1] = (((par.d0 * par.d0) / st.etasw) * st.Drhox) * par.g0
    st.wx = st.wx * st.bndtaperw
    st.wx[:, 0] = st.wx[:, -2]
    st.wx[:, -1] = st.wx[:, 1]
    x_w_ext = st.x_w[:, icx]
    m_w_ext = st.m_w[:, icx]
    st.wm = ((-x_w_ext) / jl_max(m_w_ext, EPS)) * st.wx


def update_phase_velocities(st: State, grid: Grid, par: Params, xBC="periodic", zBC="closed"):
    """src/store.jl:80-105."""
    update_segregation_speed(st, grid, par, xBC)
    icx = icx_of(grid.Nx, xBC)
    icz = icz_of(grid.Nz, zBC)
    x_w_ext = st.x_w[:, icx]
    m_w_ext = st.m_w[:, icx]
    x_u_ext = st.x_u[icz, :]
    m_u_ext = st.m_u[icz, :]
    st.Wx = ((st.W + st.wx) + (st.xisw + st.xixw)) + st.xiew
    st.Ux = (st.U + (st.xisu + st.xixu)) + st.xieu
    st.Wm = ((st.W + st.wm) - ((x_w_ext / jl_max(m_w_ext, EPS)) * (st.xisw + st.xixw))) + st.xiew
    st.Um = (st.U + (((-x_u_ext) / jl_max(m_u_ext, EPS)) * (st.xisu + st.xixu))) + st.xieu


# ---------------------------------------------------------------------------
# update!  (src/update.jl)
# ---------------------------------------------------------------------------


def rowmean_seq(A):
    """``mean(A, dims=2)``: Julia reduces the non-leading dimension column by
    column (sequential), then divides by the count."""
    acc = np.zeros(A.shape[0])
    for i in range(A.shape[1]):
        acc = acc + A[:, i]
    return acc / A.shape[1]


def update_volume_fractions(st: State, par: Params):
    """compute_volfrac_kernel! (src/update.jl:18-35)."""
    x, m = st.x, st.m
    rho = 1.0 / (m / par.rhom0 + x / par.rhox0)
    st.rho = rho
    chi_raw = (x * rho) / par.rhox0
    mu_raw = (m * rho) / par.rhom0
    lo, hi = EPS, 1.0 - EPS
    st.chi = np.where(chi_raw > hi, hi, np.where(chi_raw < lo, lo, chi_raw))
    st.mu = np.where(mu_raw > hi, hi, np.where(mu_raw < lo, lo, mu_raw))
    st.hasx = (x >= SQRT_EPS).astype(np.float64)
    st.hasm = (m >= SQRT_EPS).astype(np.float64)


def update_interpolations(st: State, grid: Grid, par: Params, xBC="periodic", zBC="closed"):
    """src/update.jl:73-107."""
    icx = icx_of(grid.Nx, xBC)
    icz = icz_of(grid.Nz, zBC)
    st.rhow = (st.rho[icz[:-1], :] + st.rho[icz[1:], :]) / 2.0
    st.rhou = (st.rho[:, icx[:-1]] + st.rho[:, icx[1:]]) / 2.0
    rhoref = rowmean_seq(st.rhow)
    st.Drho = st.rhow - rhoref[:, None]
    st.Drhom = par.rhom0 - st.rhow
    st.Drhox = par.rhox0 - st.rhow
    st.chiw = (st.chi[icz[:-1]][:, icx] + st.chi[icz[1:]][:, icx]) / 2.0
    st.muw = (st.mu[icz[:-1]][:, icx] + st.mu[icz[1:]][:, icx]) / 2.0
    st.chiu = (st.chi[icz][:, icx[:-1]] + st.chi[icz][:, icx[1:]]) / 2.0
    st.muu = (st.mu[icz][:, icx[:-1]] + st.mu[icz][:, icx[1:]]) / 2.0
    st.x_w = (st.x[icz[:-1], :] + st.x[icz[1:], :]) / 2.0
    st.m_w = (st.m[icz[:-1], :] + st.m[icz[1:], :]) / 2.0
    st.x_u = (st.x[:, icx[:-1]] + st.x[:, icx[1:]]) / 2.0
    st.m_u = (st.m[:, icx[:-1]] + st.m[:, icx[1:]]) / 2.0


def update_pressure(st: State, grid: Grid, par: Params):
    """src/update.jl:119-136 (z-scan of the row-mean face density)."""
    Nz, h = grid.Nz, grid.h
    rhoref = rowmean_seq(st.rhow)
    col = np.empty(Nz)
    col[0] = ((rhoref[0] * par.g0) * h) / 2.0 + par.Ptop
    for j in range(1, Nz):
        col[j] = col[j - 1] + (rhoref[j] * par.g0) * h
    st.Pl = np.repeat(col[:, None], grid.Nx, axis=1)
    st.Pt = jl_max(par.Ptop / 100.0, st.Pl + st.P[1:-1, 1:-1])


def rheology(chi, mu, par: Params):
    """compute_rheology_kernel! (src/update.jl:144-177)."""
    (A11, A12), (A21, A22) = par.AA
    (B11, B12), (B21, B22) = par.BB
    (C11, C12), (C21, C22) = par.CC
    f1, f2 = chi, mu
    s11 = np.power(f1 / B11, 1.0 / C11)
    s12 = np.power(f2 / B12, 1.0 / C12)
    s21 = np.power(f1 / B21, 1.0 / C21)
    s22 = np.power(f2 / B22, 1.0 / C22)
    n1 = s11 + s12
    n2 = s21 + s22
    Sf11, Sf12 = s11 / n1, s12 / n1
    Sf21, Sf22 = s21 / n2, s22 / n2
    a1 = A11 * Sf11 + A12 * Sf12
    a2 = A21 * Sf21 + A22 * Sf22
    Xf11 = a1 * f1 + (1.0 - a1) * Sf11
    Xf12 = a1 * f2 + (1.0 - a1) * Sf12
    Xf21 = a2 * f1 + (1.0 - a2) * Sf21
    Xf22 = a2 * f2 + (1.0 - a2) * Sf22
    ex, em = par.etax0, par.etam0
    thtv1 = np.power(ex / ex, Xf11) * np.power(em / ex, Xf12)
    thtv2 = np.power(ex / em, Xf21) * np.power(em / em, Xf22)
    etaf1 = ex * thtv1
    etaf2 = em * thtv2
    return f1 * etaf1 + f2 * etaf2


def update_kinematics(st: State, grid: Grid):
    """src/update.jl:202-280."""
    invh = 1.0 / grid.h
    W, U = st.W, st.U
    Ux_c = (U[1:-1, 1:] - U[1:-1, :-1]) * invh
    Wz_c = (W[1:, 1:-1] - W[:-1, 1:-1]) * invh
    div = Ux_c + Wz_c
    st.Div_V = div
    st.exx = Ux_c - div / 3.0
    st.ezz = Wz_c - div / 3.0
    dUdz = (U[1:, :] - U[:-1, :]) * invh
    dWdx = (W[:, 1:] - W[:, :-1]) * invh
    st.exz = (dUdz + dWdx) / 2.0
    e = st.exz
    exz_sq = (((e[:-1, :-1] * e[:-1, :-1] + e[1:, :-1] * e[1:, :-1]) + e[:-1, 1:] * e[:-1, 1:])
              + e[1:, 1:] * e[1:, 1:]) / 4.0
    st.eII = np.sqrt((EPS + (st.exx * st.exx + st.ezz * st.ezz) / 2.0) + exz_sq)
    wc = (W[:-1, 1:-1] + W[1:, 1:-1]) / 2.0
    uc = (U[1:-1, :-1] + U[1:-1, 1:]) / 2.0
    st.V = np.sqrt(wc * wc + uc * uc)
    t = (st.wx[:-1, 1:-1] + st.wx[1:, 1:-1]) / 2.0
    st.vx = np.sqrt(t * t + EPS)
    t = (st.wm[:-1, 1:-1] + st.wm[1:, 1:-1]) / 2.0
    st.vm = np.sqrt(t * t + EPS)


def corner_eta(eta, xBC="periodic", zBC="closed"):
    """compute_corner_eta! (src/update.jl:411-426)."""
    Nz, Nx = eta.shape
    icx = icx_of(Nx, xBC)
    icz = icz_of(Nz, zBC)
    e00 = eta[icz[:-1]][:, icx[:-1]]
    e10 = eta[icz[1:]][:, icx[:-1]]
    e01 = eta[icz[:-1]][:, icx[1:]]
    e11 = eta[icz[1:]][:, icx[1:]]
    return np.power(((e00 * e10) * e01) * e11, 0.25)


def update_viscosity(st: State, grid: Grid, par: Params, sc: dict):
    """src/update.jl:286-343."""
    eta_prev = st.eta.copy()
    L0 = sc["L0"]
    ke = (st.eII * L0) * L0
    ReL = (st.V * L0) / (st.etamix / st.rho)
    fReL = 1.0 - np.exp(-ReL)
    etae = (fReL * ke) * st.rho
    etai = st.etamix + etae
    st.etae, st.ke, st.kx, st.ReL, st.fReL = etae, ke, ke.copy(), ReL, fReL
    emax = jl_minimum(etai) * par.etacntr
    eta = 1.0 / (1.0 / emax + 1.0 / etai)
    st.eta = 0.5 * eta + 0.5 * eta_prev
    st.ReD = (st.V * sc["D0"]) / (st.eta / st.rho)
    st.etaco = corner_eta(st.eta, "periodic", "closed")


def update_segregation_viscosity(st: State, par: Params, sc: dict, zBC="closed"):
    """src/update.jl:345-409."""
    etas_prev = st.etas.copy()
    l0 = sc["l0"]
    vx, rho, etamix = st.vx, st.rho, st.etamix
    Rel = ((vx * l0) * rho) / etamix
    fRel = 1.0 - np.exp(-Rel)
    ks = vx * l0
    etat = (fRel * ks) * rho
    etasi = etamix + etat
    st.Rel, st.fRel, st.ks, st.etat = Rel, fRel, ks, etat
    st.kx = ks + st.fReL * st.ke
    st.Rc = st.V / jl_max(vx, EPS)
    emax = jl_minimum(etasi) * par.etacntr
    etas = 1.0 / (1.0 / emax + 1.0 / etasi)
    st.etas = 0.5 * etas + 0.5 * etas_prev
    st.Red = (vx * par.d0) / (st.etas / rho)
    icz = icz_of(st.Nz, zBC)
    st.etasw = np.sqrt(st.etas[icz[:-1], :] * st.etas[icz[1:], :])


def update_stresses(st: State, sc: dict):
    """src/update.jl:432-476."""
    st.txz = st.etaco * st.exz
    st.txx = st.eta * st.exx
    st.tzz = st.eta * st.ezz
    t = st.txz
    txz_sq = (((t[:-1, :-1] * t[:-1, :-1] + t[1:, :-1] * t[1:, :-1]) + t[:-1, 1:] * t[:-1, 1:])
              + t[1:, 1:] * t[1:, 1:]) / 4.0
    st.tII = np.sqrt((EPS + (st.txx * st.txx + st.tzz * st.tzz) / 2.0) + txz_sq)
    st.Ra = (st.V * sc["D0"]) / st.kx


def update(st: State, grid: Grid, par: Params, sc: dict, xBC="periodic", zBC="closed"):
    """update! (src/update.jl:525-538)."""
    update_volume_fractions(st, par)
    update_interpolations(st, grid, par, xBC, zBC)
    update_pressure(st, grid, par)
    st.etamix = rheology(st.chi, st.mu, par)
    update_kinematics(st, grid)
    update_viscosity(st, grid, par, sc)
    update_segregation_viscosity(st, par, sc, zBC)
    update_stresses(st, sc)


def jmax(*v):
    """Julia's max of Float64 scalars, max(max(a, b), c)...: NaN if any
    argument is NaN (Python's builtin max keeps or drops a NaN depending on
    argument order)."""
    r = v[0]
    for x in v[1:]:
        r = jl_max(r, x)
    return float(r)


def jmin(*v):
    """Julia's min of Float64 scalars (NaN propagates)."""
    r = v[0]
    for x in v[1:]:
        r = jl_min(r, x)
    return float(r)


def update_dt(st: State, grid: Grid, par: Params, dt_prev: float) -> float:
    """src/update.jl:494-502, with Julia's maximum / max / min (NaN
    propagates, -0.0 < +0.0)."""
    h = grid.h
    dtk = (h / 2.0) * (h / 2.0) / jl_maximum(st.kx)
    vmax = jmax(jl_maximum(np.abs(st.Wx)), jl_maximum(np.abs(st.Wm)), jl_maximum(np.abs(st.Ux)),
                jl_maximum(np.abs(st.Um))) + EPS
    dta = (h / 2.0) / vmax
    return jmin(1.5 * dt_prev, jmin(dtk, par.CFL * dta), par.dtmax)


# ---------------------------------------------------------------------------
# noise!  (src/noise.jl)
# ---------------------------------------------------------------------------


def noise_pads(grid: Grid, sc: dict):
    """padL0 / padl0 of the NoiseState constructor (src/noise.jl:69-70)."""
    padL0 = 4 * math.ceil(sc["L0h"] / grid.h)
    padl0 = 4 * math.ceil(sc["l0h"] / grid.h)
    return padL0, padl0


def make_gaussian_filter(Nz_pad: int, Nx: int, h: float, sigma: float) -> np.ndarray:
    """_make_gaussian_filter (src/noise.jl:98-107): exp(-sigma^2 (kz^2 + kx^2))
    with kz = 2*pi*fftfreq(Nz_pad, 1/h) (AbstractFFTs Frequencies arithmetic)."""
    def freqs(n):
        nn = (n + 1) >> 1
        mult = 2 * math.pi * ((1.0 / h) / n)
        k = np.array([(i if i < nn else i - n) for i in range(n)], dtype=np.float64)
        return k * mult
    kz = freqs(Nz_pad)
    kx = freqs(Nx)
    return np.exp(-(sigma * sigma) * (kz[:, None] * kz[:, None] + kx[None, :] * kx[None, :]))


def std1(a):
    """Julia ``std`` (corrected, two-pass)."""
    m = a.mean()
    d = a - m
    return math.sqrt(float((d * d).sum()) / (a.size - 1))


def fft_filter(psi, Gk, pad):
    """compute_fft_filter (src/noise.jl:244-270)."""
    Nz, Nx = psi.shape
    halfpad = pad // 2
    pp = np.zeros((Nz + pad, Nx), dtype=np.complex128)
    pp[halfpad:halfpad + Nz, :] = psi
    pp = np.fft.fft2(pp)
    pp = pp * Gk
    pp = np.fft.ifft2(pp)
    flt = pp[halfpad:halfpad + Nz, :].real.copy()
    raw_std = std1(psi)
    raw_mean = float(psi.mean())
    flt_std = std1(flt)
    flt_mean = float(flt.mean())
    if flt_std > EPS:
        flt = (((flt - flt_mean) * raw_std) / flt_std) + raw_mean
    return flt


class NoiseStatic:
    """Precomputed pieces of NoiseState (src/noise.jl:61-93)."""

    def __init__(self, grid: Grid, sc: dict):
        self.padL0, self.padl0 = noise_pads(grid, sc)
        self.Gkpe = make_gaussian_filter(grid.Nz + self.padL0, grid.Nx, grid.h, sc["L0h"])
        self.Gkps = make_gaussian_filter(grid.Nz + self.padl0, grid.Nx, grid.h, sc["l0h"])


def noise(st: State, grid: Grid, par: Params, sc: dict, ns: NoiseStatic, dt: float,
          first_iter: bool, re=None, rs=None):
    """noise! (src/noise.jl:138-239).  White noise ``re``/``rs`` is supplied by
    the caller on the first sweep (it replaces ``randn!(ns.rng, ...)``)."""
    Nz, Nx = grid.Nz, grid.Nx
    icz = icz_of(Nz, "closed")
    icx = icx_of(Nx, "periodic")
    Xi, L0h, l0h, h, txi0 = par.Xi, sc["L0h"], sc["l0h"], grid.h, sc["txi0"]
    if first_iter:
        st.re = np.array(re, dtype=np.float64, copy=True)
        st.rs = np.array(rs, dtype=np.float64, copy=True)
    taue = L0h / (2.0 * (st.V + EPS))
    taus = l0h / (2.0 * (st.vx + EPS))
    St = txi0 / (taue + EPS)
    sge = Xi * np.sqrt(jl_max(0.0, (st.fReL * st.ke) / taue))
    sgx = Xi * np.sqrt(jl_max(0.0, ((((st.chi * st.fReL) * st.ke) / taue) * St) / (1.0 + St * St)))
    sgs = Xi * np.sqrt(jl_max(0.0, (st.chi * st.ks) / taus))
    taue = 1.0 / (1.0 / taue + 1.0 / (1e2 * dt)) + dt
    taus = 1.0 / (1.0 / taus + 1.0 / (1e2 * dt)) + dt
    Fte = np.exp((-dt) / taue)
    Fts = np.exp((-dt) / taus)
    fL = 2.0 / math.sqrt(1.0 - math.exp(-(h * h) / (2 * (L0h * L0h))))
    fl = 2.0 / math.sqrt(1.0 - math.exp(-(h * h) / (2 * (l0h * l0h))))
    ae = np.sqrt(jl_max(0.0, 1.0 - Fte * Fte))
    as_ = np.sqrt(jl_max(0.0, 1.0 - Fts * Fts))
    st.psie = Fte * st.psieo + ((ae * sge) * fL) * st.re
    st.psix = Fte * st.psixo + ((ae * sgx) * fL) * st.re
    st.psis = Fts * st.psiso + ((as_ * sgs) * fl) * st.rs
    pe = fft_filter(st.psie, ns.Gkpe, ns.padL0)
    px = fft_filter(st.psix, ns.Gkpe, ns.padL0)
    ps = fft_filter(st.psis, ns.Gkps, ns.padl0)
    pe_ext = pe[icz][:, icx]
    psiec = (((pe_ext[:-1, :-1] + pe_ext[:-1, 1:]) + pe_ext[1:, :-1]) + pe_ext[1:, 1:]) / 4.0
    xieu_int = psiec[1:, :] - psiec[:-1, :]
    xiew_int = -(psiec[:, 1:] - psiec[:, :-1])
    st.xieu = xieu_int[icz, :]
    st.xiew = xiew_int[:, icx]
    xtaperw = (1.0 - np.exp((-st.chiw) / 1e-4)) * (1.0 - np.exp((-jl_max(0.0, st.muw - 0.4)) / 0.05))
    xtaperu = (1.0 - np.exp((-st.chiu) / 1e-4)) * (1.0 - np.exp((-jl_max(0.0, st.muu - 0.4)) / 0.05))
    px_ext = px[icz][:, icx]
    ps_ext = ps[icz][:, icx]
    st.xixu = (-(px_ext[:, 1:] - px_ext[:, :-1])) * xtaperu
    st.xixw = (-(px_ext[1:, :] - px_ext[:-1, :])) * xtaperw
    st.xisu = (-(ps_ext[:, 1:] - ps_ext[:, :-1])) * xtaperu
    st.xisw = (-(ps_ext[1:, :] - ps_ext[:-1, :])) * xtaperw

    def speed(aw, au):
        wz = (aw[:-1, 1:-1] + aw[1:, 1:-1]) / 2.0
        wx = (au[1:-1, :-1] + au[1:-1, 1:]) / 2.0
        return np.sqrt(wz * wz + wx * wx)
    st.xis = speed(st.xisw, st.xisu)
    st.xix = speed(st.xixw, st.xixu)
    st.xie = speed(st.xiew, st.xieu)
    return dict(pe=pe, px=px, ps=ps)


# ---------------------------------------------------------------------------
# fluidmech!  (src/fluidmech.jl:71-534)
# ---------------------------------------------------------------------------


@dataclass
class Bnchm:
    """BnchmData (src/state.jl:131-134)."""
    src_W: np.ndarray
    src_U: np.ndarray
    src_P: np.ndarray
    W_exact: np.ndarray
    U_exact: np.ndarray
    P_exact: np.ndarray


def mfs_update(st: State, par: Params, coefs, dt):
    """MFS correction, src/fluidmech.jl:115-126 (mutates drhodt, MFS)."""
    a1, a2, a3, b1, b2, b3 = coefs
    st.drhodt = -st.advn_rho
    res_rho = ((a1 * st.rho - a2 * st.rhoo) - a3 * st.rhooo) / dt \
        - ((b1 * st.drhodt + b2 * st.drhodto) + b3 * st.drhodtoo)
    st.MFS = st.MFS - par.alpha * res_rho


def assemble_stokes(st: State, grid: Grid, par: Params, coefs, dt, bn: Bnchm | None = None,
                    sds=-1, top_cnv=1, bot_cnv=1, open_cnv=False, xBC="periodic", zBC="closed"):
    """Triplets of LL = [KV GG; DM KP] and the dense RHS RR, exactly as
    src/fluidmech.jl:130-493 builds them.  Returns (I, J, V, RR, n) with 0-based
    indices; duplicates are summed by the caller.  Unknown order: vec(W),
    vec(U), vec(P), column-major (MapW/MapU/MapP, fluidmech.jl:95-100)."""
    a1, a2, a3 = coefs[0], coefs[1], coefs[2]
    bnchm = bn is not None
    Nz, Nx, h = grid.Nz, grid.Nx, grid.h
    g0, gamma = par.g0, par.gamma
    invh = 1.0 / h
    invh2 = invh * invh
    NP = (Nz + 2) * (Nx + 2)
    NW = (Nz + 1) * (Nx + 2)
    NU = (Nz + 2) * (Nx + 1)
    n = NW + NU + NP

    def MapW(j, i):
        return np.asarray(j) + np.asarray(i) * (Nz + 1)

    def MapU(j, i):
        return NW + np.asarray(j) + np.asarray(i) * (Nz + 2)

    def MapP(j, i):
        return NW + NU + np.asarray(j) + np.asarray(i) * (Nz + 2)

    W, U, P = st.W, st.U, st.P
    eta, etaco, rho, rhow, rhou, Drho = st.eta, st.etaco, st.rho, st.rhow, st.rhou, st.Drho
    MFS = st.MFS
    MFSmean = float(MFS.mean())
    II, JJ, VV = [], [], []
    RR = np.zeros(n)

    def addm(imat, jmat, vmat):
        """Append matrices of equal shape in column-major (vec) order."""
        imat = np.asarray(imat)
        II.append(imat.ravel(order="F"))
        JJ.append(np.broadcast_to(np.asarray(jmat), imat.shape).ravel(order="F"))
        VV.append(np.broadcast_to(np.asarray(vmat, dtype=np.float64), imat.shape).ravel(order="F"))

    jz = np.arange(Nz + 1)[:, None]
    # W ghost columns: W[:,1] + sds W[:,end-1] = 0 ; W[:,end] + sds W[:,2] = 0
    addm(MapW(jz, 0), MapW(jz, 0), 1.0)
    addm(MapW(jz, 0), MapW(jz, Nx), float(sds))
    addm(MapW(jz, Nx + 1), MapW(jz, Nx + 1), 1.0)
    addm(MapW(jz, Nx + 1), MapW(jz, 1), float(sds))
    ix = np.arange(1, Nx + 1)[None, :]
    # top W = 0
    addm(MapW(0, ix), MapW(0, ix), 1.0)
    # bottom
    oc = 1.0 if open_cnv else 0.0
    rho1 = rhow[Nz, :][None, :]
    rho2 = rhow[Nz - 1, :][None, :]
    rho3 = rhou[Nz - 1, 1:][None, :]
    rho4 = rhou[Nz - 1, :-1][None, :]
    ib = MapW(Nz, ix)
    addm(ib, ib, rho1 * invh)
    addm(ib, MapW(Nz - 1, ix), -oc * rho2 * invh)
    addm(ib, MapU(Nz, np.arange(1, Nx + 1)[None, :]), oc * rho3 * invh)
    addm(ib, MapU(Nz, np.arange(0, Nx)[None, :]), -oc * rho4 * invh)
    mfbg_bot = MFSmean * grid.D / h
    RR[ib.ravel()] = (oc * MFS[Nz - 1, :] + (1.0 - oc) * mfbg_bot)
    # interior W: rows j = 1..Nz-1 (0-based), cols i = 1..Nx
    J = np.arange(1, Nz)[:, None]
    I = np.arange(1, Nx + 1)[None, :]
    ii = MapW(J, I)
    EtaC1 = etaco[1:Nz, 0:Nx]
    EtaC2 = etaco[1:Nz, 1:Nx + 1]
    EtaP1 = eta[0:Nz - 1, :]
    EtaP2 = eta[1:Nz, :]
    addm(ii, ii, a1 * rhow[1:Nz, :] / dt)
    addm(ii, ii, (2.0 / 3.0) * (EtaP1 + EtaP2) * invh2 + 0.5 * (EtaC1 + EtaC2) * invh2)
    addm(ii, MapW(J - 1, I), -(2.0 / 3.0) * EtaP1 * invh2)
    addm(ii, MapW(J + 1, I), -(2.0 / 3.0) * EtaP2 * invh2)
    addm(ii, MapW(J, I - 1), -0.5 * EtaC1 * invh2)
    addm(ii, MapW(J, I + 1), -0.5 * EtaC2 * invh2)
    if not bnchm:
        ddz_rho = (rho[1:, :] - rho[:-1, :]) * invh
        addm(ii, ii, ddz_rho * g0 * dt)
    addm(ii, MapU(J, I - 1), -(0.5 * EtaC1 - (1.0 / 3.0) * EtaP1) * invh2)
    addm(ii, MapU(J + 1, I - 1), +(0.5 * EtaC1 - (1.0 / 3.0) * EtaP2) * invh2)
    addm(ii, MapU(J, I), +(0.5 * EtaC2 - (1.0 / 3.0) * EtaP1) * invh2)
    addm(ii, MapU(J + 1, I), -(0.5 * EtaC2 - (1.0 / 3.0) * EtaP2) * invh2)
    f_mz = rhow[1:Nz, :] * W[1:Nz, 1:Nx + 1]
    u_mz = (U[1:Nz, :] + U[2:Nz + 1, :]) / 2.0
    w_mz = (W[0:Nz, 1:Nx + 1] + W[1:Nz + 1, 1:Nx + 1]) / 2.0
    advn_mz = advect_centered(f_mz, u_mz, w_mz, h, par.ADVN, xBC, zBC)
    rr = (Drho[1:Nz, :] * g0 + (a2 * st.rhoWo[1:Nz, :] + a3 * st.rhoWoo[1:Nz, :]) / dt) - advn_mz
    if bnchm:
        rr = rr + bn.src_W[1:Nz, 1:Nx + 1]
    RR[ii.ravel(order="F")] = rr.ravel(order="F")

    # U equations
    ia = np.arange(Nx + 1)[None, :]
    addm(MapU(0, ia), MapU(0, ia), 1.0)
    addm(MapU(0, ia), MapU(1, ia), float(top_cnv))
    addm(MapU(Nz + 1, ia), MapU(Nz + 1, ia), 1.0)
    addm(MapU(Nz + 1, ia), MapU(Nz, ia), float(bot_cnv))
    icx = np.concatenate(([Nx - 1], np.arange(Nx), [0]))          # [Nx; 1:Nx; 1]
    ifx = np.concatenate(([Nx - 1], np.arange(Nx + 1), [1]))      # [Nx; 1:Nx+1; 2]
    J = np.arange(1, Nz + 1)[:, None]
    I = np.arange(Nx + 1)[None, :]
    ii = MapU(J, I)
    EtaC1 = etaco[0:Nz, :]
    EtaC2 = etaco[1:Nz + 1, :]
    EtaP1 = eta[:, icx[:-1]]
    EtaP2 = eta[:, icx[1:]]
    addm(ii, ii, (a1 + gamma) * rhou / dt)
    addm(ii, ii, (2.0 / 3.0) * (EtaP1 + EtaP2) * invh2 + 0.5 * (EtaC1 + EtaC2) * invh2)
    addm(ii, MapU(J, ifx[None, 0:Nx + 1]), -(2.0 / 3.0) * EtaP1 * invh2)
    addm(ii, MapU(J, ifx[None, 2:Nx + 3]), -(2.0 / 3.0) * EtaP2 * invh2)
    addm(ii, MapU(J - 1, ifx[None, 1:Nx + 2]), -0.5 * EtaC1 * invh2)
    addm(ii, MapU(J + 1, ifx[None, 1:Nx + 2]), -0.5 * EtaC2 * invh2)
    if not bnchm:
        ddx_rho = (rho[:, icx[1:]] - rho[:, icx[:-1]]) * invh
        addm(ii, ii, ddx_rho * g0 * dt)
    addm(ii, MapW(J - 1, I), -(0.5 * EtaC1 - (1.0 / 3.0) * EtaP1) * invh2)
    addm(ii, MapW(J - 1, I + 1), +(0.5 * EtaC1 - (1.0 / 3.0) * EtaP2) * invh2)
    addm(ii, MapW(J, I), +(0.5 * EtaC2 - (1.0 / 3.0) * EtaP1) * invh2)
    addm(ii, MapW(J, I + 1), -(0.5 * EtaC2 - (1.0 / 3.0) * EtaP2) * invh2)
    u_mx = (U[1:Nz + 1, ifx[:-1]] + U[1:Nz + 1, ifx[1:]]) / 2.0
    w_mx = (W[:, :-1] + W[:, 1:]) / 2.0
    f_mx = rhou * U[1:Nz + 1, :]
    advn_mx = advect_centered(f_mx, u_mx, w_mx, h, par.ADVN, xBC, zBC)
    col_avg = (advn_mx[:, 0] + advn_mx[:, -1]) / 2.0
    advn_mx[:, 0] = col_avg
    advn_mx[:, -1] = col_avg
    rr = (a2 * st.rhoUo + a3 * st.rhoUoo) / dt - advn_mx
    if bnchm:
        rr = rr + bn.src_U[1:Nz + 1, :]
    RR[ii.ravel(order="F")] = rr.ravel(order="F")

    # GG (gradient)
    J = np.arange(1, Nz)[:, None]
    I = np.arange(1, Nx + 1)[None, :]
    addm(MapW(J, I), MapP(J, I), -invh)
    addm(MapW(J, I), MapP(J + 1, I), +invh)
    J = np.arange(1, Nz + 1)[:, None]
    I = np.arange(Nx + 1)[None, :]
    addm(MapU(J, I), MapP(J, I), -invh)
    addm(MapU(J, I), MapP(J, I + 1), +invh)

    # DM (rho-weighted divergence), interior P rows j = 1..Nz, i = 1..Nx
    J = np.arange(1, Nz + 1)[:, None]
    I = np.arange(1, Nx + 1)[None, :]
    ip = MapP(J, I)
    addm(ip, MapU(J, I - 1), -rhou[:, 0:Nx] * invh)
    addm(ip, MapU(J, I), +rhou[:, 1:Nx + 1] * invh)
    addm(ip, MapW(J - 1, I), -rhow[0:Nz, :] * invh)
    addm(ip, MapW(J, I), +rhow[1:Nz + 1, :] * invh)
    # KP ghost rows
    ia = np.arange(Nx + 2)[None, :]
    addm(MapP(0, ia), MapP(0, ia), 1.0)
    addm(MapP(0, ia), MapP(1, ia), -1.0)
    addm(MapP(Nz + 1, ia), MapP(Nz + 1, ia), 1.0)
    addm(MapP(Nz + 1, ia), MapP(Nz, ia), -1.0)
    J = np.arange(1, Nz + 1)[:, None]
    addm(MapP(J, 0), MapP(J, 0), 1.0)
    addm(MapP(J, 0), MapP(J, Nx), -1.0)
    addm(MapP(J, Nx + 1), MapP(J, Nx + 1), 1.0)
    addm(MapP(J, Nx + 1), MapP(J, 1), -1.0)

    RR[MapP(np.arange(1, Nz + 1)[:, None], np.arange(1, Nx + 1)[None, :]).ravel(order="F")] = \
        (MFS + (bn.src_P[1:Nz + 1, 1:Nx + 1] if bnchm else 0.0)).ravel(order="F")

    Iall = np.concatenate(II)
    Jall = np.concatenate(JJ)
    Vall = np.concatenate(VV)
    zero_rows = []
    unit_diag = []
    if bnchm:
        nzp = julia_round((Nz + 2) * 3 / 8) - 1
        nxp = julia_round((Nx + 2) / 2) - 1
        np0 = int(MapP(nzp, nxp))
        zero_rows.append(np0)
        unit_diag.append(np0)
        RR[np0] = bn.P_exact[nzp, nxp]
        nzu = julia_round((Nz + 2) / 2) - 1
        nxu = julia_round((Nx + 2) / 2) - 1
        nu0 = int(MapU(nzu, nxu))
        zero_rows.append(nu0)
        unit_diag.append(nu0)
        RR[nu0] = bn.U_exact[nzu, nxu]
        keep = ~np.isin(Iall, zero_rows)
    else:
        if open_cnv:
            pins = [int(MapP(Nz, i)) for i in range(Nx + 2)]
        else:
            pins = [int(MapP(julia_round(Nz / 2) - 1, julia_round(Nx / 2) - 1))]
        # pin: zero the KP row (it only holds the pre-added zero diagonal for an
        # interior pin), set the diagonal to one; DM row is kept.
        pmask = np.isin(Iall, pins) & (Jall >= NW + NU)
        keep = ~pmask
        unit_diag.extend(pins)
    Iall, Jall, Vall = Iall[keep], Jall[keep], Vall[keep]
    Iall = np.concatenate((Iall, np.array(unit_diag, dtype=Iall.dtype)))
    Jall = np.concatenate((Jall, np.array(unit_diag, dtype=Jall.dtype)))
    Vall = np.concatenate((Vall, np.ones(len(unit_diag))))
    return Iall, Jall, Vall, RR, (NW, NU, NP)


def stokes_matrix(st, grid, par, coefs, dt, bn=None, **bc):
    """Assembled scipy CSC matrix LL, RHS RR and block sizes."""
    import scipy.sparse as sp
    I, J, V, RR, blocks = assemble_stokes(st, grid, par, coefs, dt, bn, **bc)
    n = len(RR)
    LL = sp.coo_matrix((V, (I, J)), shape=(n, n)).tocsc()
    LL.sum_duplicates()
    return LL, RR, blocks


def stokes_scaling(LL, st, blocks):
    """scl = 1/(sqrt|diag LL| + [0; sqrt(eta/rho) on interior P, 1 on ghost P])
    (src/fluidmech.jl:496-501)."""
    NW, NU, NP = blocks
    Nz, Nx = st.Nz, st.Nx
    diagLL = np.abs(LL.diagonal())
    scl_p = np.ones((Nz + 2, Nx + 2))
    scl_p[1:-1, 1:-1] = st.rho / st.eta
    extra = np.concatenate((np.zeros(NW + NU), np.sqrt(1.0 / scl_p.ravel(order="F"))))
    return 1.0 / (np.sqrt(diagLL) + extra)


def fluidmech(st: State, grid: Grid, par: Params, coefs, dt, bn: Bnchm | None = None,
              sds=-1, top_cnv=1, bot_cnv=1, open_cnv=False, xBC="periodic", zBC="closed",
              return_system=False):
    """fluidmech! (src/fluidmech.jl:71-534).  The sparse direct solve uses
    scipy's SuperLU in place of UMFPACK."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    if bn is None:
        mfs_update(st, par, coefs, dt)
    LL, RR, blocks = stokes_matrix(st, grid, par, coefs, dt, bn, sds=sds, top_cnv=top_cnv,
                                   bot_cnv=bot_cnv, open_cnv=open_cnv, xBC=xBC, zBC=zBC)
    NW, NU, NP = blocks
    scl = stokes_scaling(LL, st, blocks)
    SCL = sp.diags(scl)
    SOL = np.concatenate((st.W.ravel(order="F"), st.U.ravel(order="F"), st.P.ravel(order="F")))
    FF = scl * (LL @ SOL - RR)
    LLs = (SCL @ LL @ SCL).tocsc()
    lu = spla.splu(LLs)
    UPD = scl * lu.solve(FF)
    Nz, Nx = grid.Nz, grid.Nx
    st.W = st.W - UPD[:NW].reshape((Nz + 1, Nx + 2), order="F")
    st.U = st.U - UPD[NW:NW + NU].reshape((Nz + 2, Nx + 1), order="F")
    st.P = st.P - UPD[NW + NU:].reshape((Nz + 2, Nx + 2), order="F")
    if return_system:
        return LL, RR, blocks
    return None


# ---------------------------------------------------------------------------
# residual norms and conservation sums  (src/diagnose.jl:42-71, src/history.jl:122-145)
# ---------------------------------------------------------------------------


def snapshot(st: State, res: dict | None = None) -> dict:
    """snapshot! (src/diagnose.jl:42-49): the StepResidual's buffers as a dict.
    Given a StepResidual ``res`` (a dict from an earlier call), its buffers
    are replaced and its ``resnorm0`` kept, as snapshot! leaves that field
    alone; a fresh one starts with resnorm0 = 1.0 (diagnose.jl:26-33)."""
    out = res if res is not None else {"resnorm0": 1.0}
    out.update(W=st.W.copy(), U=st.U.copy(), P=st.P.copy(), X=st.X.copy(), MFS=st.MFS.copy())
    return out


def resnorm(st: State, snap: dict, dt: float):
    """compute_resnorm (src/diagnose.jl:57-71) -> (resnorm, res_mass, res_mmnt);
    raises the StepResidual's resnorm0 to resnorm + 1e-32 when it is below
    resnorm (diagnose.jl:67-69)."""
    nrm = np.linalg.norm
    ep = EPS
    nrho = float(nrm(st.rho))
    res_mass = nrm(st.X - snap["X"]) / (nrho + ep) + nrm(st.MFS - snap["MFS"]) / (nrho / dt + ep)
    res_mmnt = (nrm(st.W - snap["W"]) / (nrm(st.W) + ep) + nrm(st.U - snap["U"]) / (nrm(st.U) + ep)
                + nrm(st.P - snap["P"]) / (nrm(st.P) + ep))
    r = float(res_mass + res_mmnt)
    if "resnorm0" in snap and snap["resnorm0"] < r:
        snap["resnorm0"] = r + 1e-32
    return r, float(res_mass), float(res_mmnt)


def conservation_sums(st: State, grid: Grid) -> dict:
    """FP64 mass sums and boundary-flux line integrals of record_history!
    (src/history.jl:121-145)."""
    h = grid.h
    h2 = h * h
    out = dict(sumB=float(st.rho.sum()) * h2 + EPS, sumM=float(st.M.sum()) * h2 + EPS,
               sumX=float(st.X.sum()) * h2 + EPS, sumGx=float(st.Gx.sum()) * h2)
    for name, arr in (("aX", st.qz_advn_X), ("aM", st.qz_advn_M), ("dX", st.qz_dffn_X), ("dM", st.qz_dffn_M)):
        out["top_" + name] = float(arr[0, 1:-1].sum()) * h
        out["bot_" + name] = float(arr[-1, 1:-1].sum()) * h
    return out


def print_step_stats(st: State) -> dict:
    """The statistics print_step! prints beyond record_history!'s
    (src/diagnose.jl:92-182) on the raw fields, with
    _gm(A) = exp(sum(log(max(A, 1e-300))) / length(A)) (diagnose.jl:10)."""
    out = {"m_min": jl_minimum(st.m), "m_mean": float(st.m.mean()), "m_max": jl_maximum(st.m)}
    for f in ("rho", "V", "vx", "vm", "xie", "xix", "xis"):
        a = getattr(st, f)
        out[f + "_min"] = jl_minimum(a)
        out[f + "_gm"] = math.exp(float(np.log(jl_max(a, 1e-300)).sum()) / a.size)
        out[f + "_max"] = jl_maximum(a)
    return out


def history_stats(st: State) -> dict:
    """Field statistics pushed by record_history! (src/history.jl:183-222), with
    _rms = sqrt(mean(x^2)) and _geomean = exp(mean(log(max(x, eps)))) (history.jl:8-9)."""
    out = {"x_min": jl_minimum(st.x), "x_mean": float(st.x.mean()), "x_max": jl_maximum(st.x),
           "x_std": std1(st.x)}
    for f in ("V", "vx", "vm", "xie", "xix", "xis"):
        a = getattr(st, f)
        out[f + "_min"], out[f + "_max"] = jl_minimum(a), jl_maximum(a)
        out[f + "_rms"] = math.sqrt(float((a * a).mean()))
    for f in ("Ra", "Rc", "ReD", "Red", "ks", "ke", "kx", "eta", "etamix", "etae", "etas", "etat"):
        a = getattr(st, f)
        out[f + "_min"] = jl_minimum(a)
        out[f + "_gm"] = math.exp(float(np.log(jl_max(a, EPS)).mean()))
        out[f + "_max"] = jl_maximum(a)
    return out


# ---------------------------------------------------------------------------
# initialize! and run!  (src/run.jl:24-140, 167-277)
# ---------------------------------------------------------------------------


def compute_bndtaperw(grid: Grid, par: Params, sc: dict) -> np.ndarray:
    """src/run.jl:24-35."""
    Nz1, Nx2 = grid.Nz + 1, grid.Nx + 2
    osgr = 1.0 if par.open_sgr else 0.0
    z = np.arange(Nz1, dtype=np.float64) * grid.h
    col = 1.0 - (np.exp(-z / sc["l0h"]) + np.exp(-(grid.D - z) / sc["l0h"])) * (1.0 - osgr)
    return np.repeat(col[:, None], Nx2, axis=1)


def compute_bndshape(grid: Grid, sc: dict) -> np.ndarray:
    """src/run.jl:47-55."""
    zc = (np.arange(1, grid.Nz + 1, dtype=np.float64) - 0.5) * grid.h
    col = np.exp((-zc + grid.h / 2.0) / sc["bnd_w"])
    return np.repeat(col[:, None], grid.Nx, axis=1)


def initialize(grid: Grid, par: Params, sc: dict, ns: NoiseStatic, x_init: np.ndarray,
               re: np.ndarray, rs: np.ndarray, xBC="periodic", zBC="closed") -> State:
    """Fresh-start initialize! (src/run.jl:71-140) with the initial crystal
    fraction supplied as an array (it replaces the MersenneTwister draw of
    run.jl:98-108) and the first white-noise draw supplied too."""
    st = State(grid.Nz, grid.Nx)
    st.bndtaperw = compute_bndtaperw(grid, par, sc)
    st.bndshape = compute_bndshape(grid, sc)
    st.x = np.array(x_init, dtype=np.float64, copy=True)
    st.m = 1.0 - st.x
    st.eta[:] = par.etam0
    st.etaco[:] = par.etam0
    st.etas[:] = par.etam0
    update(st, grid, par, sc, xBC, zBC)
    st.X = st.rho * st.x
    st.M = st.rho * st.m
    noise(st, grid, par, sc, ns, sc["dt0"], True, re, rs)
    update_phase_velocities(st, grid, par, xBC, zBC)
    st.Xo = st.X.copy(); st.Xoo = st.X.copy()
    st.Mo = st.M.copy(); st.Moo = st.M.copy()
    st.rhoo = st.rho.copy(); st.rhooo = st.rho.copy()
    store_noise(st)
    return st


def picard_sweep(st, grid, par, sc, ns, coefs, dt, it, re, rs, ADVN=None, xBC="periodic", zBC="closed",
                 stokes=None):
    """One pass of the run! Picard loop body (src/run.jl:224-245)."""
    snap = snapshot(st)
    phsevo(st, grid, par, sc, ADVN or par.ADVN, coefs, dt, xBC=xBC, zBC=zBC)
    if stokes is None:
        fluidmech(st, grid, par, coefs, dt, xBC=xBC, zBC=zBC)
    else:
        stokes(st, coefs, dt)
    noise(st, grid, par, sc, ns, dt, it <= 1, re, rs)
    update_phase_velocities(st, grid, par, xBC, zBC)
    update(st, grid, par, sc, xBC, zBC)
    return resnorm(st, snap, dt)


def timestep_converge(st, grid, par, sc, ns, step, dt, re, rs, rtol=1e-4, atol=1e-9, maxit=15,
                      xBC="periodic", zBC="closed", stokes=None):
    """One outer step of run! with its own Picard loop (src/run.jl:204-274,
    the while-condition of 220-222 and the resnorm0 rule of 246-249); returns
    (dt_next, [resnorms], resnorm0)."""
    coefs = time_coefs(par.TINT, step)
    store_previous(st)
    store_noise(st)
    resnorm, resnorm0, it = 1.0, 1.0, 0
    norms = []
    while (resnorm / resnorm0 >= rtol and resnorm >= atol and it < maxit) or it < 3:
        it += 1
        resnorm = picard_sweep(st, grid, par, sc, ns, coefs, dt, it, re, rs, xBC=xBC, zBC=zBC, stokes=stokes)[0]
        norms.append(resnorm)
        if it == 1 or resnorm > resnorm0:
            resnorm0 = resnorm + 1e-32
        if math.isnan(resnorm):
            raise FloatingPointError(f"Solver diverged with NaN at iter {it}")
    return update_dt(st, grid, par, dt), norms, resnorm0


def timestep(st, grid, par, sc, ns, step, dt, re, rs, sweeps=3, xBC="periodic", zBC="closed",
             stokes=None, on_sweep=None):
    """One outer step of run! (src/run.jl:204-274) with a fixed number of Picard
    sweeps (maxit = sweeps, rtol = atol = 0); returns (dt_next, [resnorms])."""
    coefs = time_coefs(par.TINT, step)
    store_previous(st)
    store_noise(st)
    norms = []
    for it in range(1, sweeps + 1):
        norms.append(picard_sweep(st, grid, par, sc, ns, coefs, dt, it, re, rs, xBC=xBC, zBC=zBC,
                                  stokes=stokes))
        if on_sweep is not None:
            on_sweep(it, st)
    return update_dt(st, grid, par, dt), norms
