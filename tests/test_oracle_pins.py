"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates one reference test (file:line in its docstring) against the
numpy restatement in ``oracle/xcore_oracle.py``.  CPU only."""
import math

import numpy as np
import pytest

import xcore_oracle as O
from mms import mms_sources


def _cosine_setup(N, halo):
    L = 2 * math.pi
    h = L / N
    xc = (np.arange(1, N + 1) - 0.5) * h
    XX, ZZ = np.meshgrid(xc, xc, indexing="xy")
    f = np.cos(XX) * np.cos(ZZ)
    fh = O.embed_halo(f, halo, "periodic", "periodic")
    return h, XX, ZZ, f, fh


@pytest.mark.parametrize("scheme,orders", [("centr", (1.9, 1.9)), ("weno5", (4.0, 3.5))])
def test_advect_convergence(scheme, orders):
    """test/test_advect.jl:1-78: div(v f) on cos(x)cos(z), (U0, W0) = (0.7, -0.3)."""
    U0, W0 = 0.7, -0.3
    g = O.scheme_halo(scheme)
    errs = []
    for N in (32, 64, 128):
        h, XX, ZZ, f, fh = _cosine_setup(N, g)
        u = np.full((N, N + 1), U0)
        w = np.full((N + 1, N), W0)
        qx, qz = O.advect_fluxes(fh, u, w, scheme, g)
        adv = O.divergence(qx, qz, 1.0 / h)
        exact = -U0 * np.sin(XX) * np.cos(ZZ) + W0 * np.cos(XX) * (-np.sin(ZZ))
        errs.append(math.sqrt(((adv - exact) ** 2).sum() / (N * N)))
    assert math.log2(errs[0] / errs[1]) > orders[0]
    assert math.log2(errs[1] / errs[2]) > orders[1]


def test_diffus_convergence():
    """test/test_diffus.jl:1-35: diffus! ~ Laplacian of sin(x)sin(z), order > 1.9."""
    errs = []
    for N in (32, 64, 128):
        L = 2 * math.pi
        h = L / N
        xc = (np.arange(1, N + 1) - 0.5) * h
        XX, ZZ = np.meshgrid(xc, xc, indexing="xy")
        f = np.sin(XX) * np.sin(ZZ)
        fh = O.embed_halo(f, 1, "periodic", "periodic")
        kh = O.embed_halo(np.ones((N, N)), 1, "periodic", "periodic")
        dff = O.diffus_halo(fh, kh, h)
        errs.append(math.sqrt(((dff - (-2.0 * f)) ** 2).sum() / (N * N)))
    assert math.log2(errs[0] / errs[1]) > 1.9
    assert math.log2(errs[1] / errs[2]) > 1.9


def test_fill_ghosts_exact():
    """test/test_stencils.jl:37-56: periodic-x / closed-z ghost values."""
    f = np.arange(1, 17, dtype=float).reshape(4, 4)
    fh = O.embed_halo(f, 1, "closed", "periodic")
    assert np.array_equal(fh[1:5, 0], fh[1:5, 4])
    assert np.array_equal(fh[1:5, -1], fh[1:5, 1])
    assert np.array_equal(fh[0, 1:5], fh[1, 1:5])
    assert np.array_equal(fh[-1, 1:5], fh[-2, 1:5])


def test_time_coefs():
    """test/test_run.jl:5-25."""
    assert O.time_coefs("bd2im", 1) == (1.0, 1.0, 0.0, 1.0, 0.0, 0.0)
    assert O.time_coefs("bd2im", 2) == (1.0, 1.0, 0.0, 1.0, 0.0, 0.0)
    assert O.time_coefs("bd2im", 3) == (1.5, 2.0, -0.5, 1.0, 0.0, 0.0)
    assert O.time_coefs("bd2si", 1) == (1.0, 1.0, 0.0, 1.0, 0.0, 0.0)
    assert O.time_coefs("bd2si", 2) == (1.0, 1.0, 0.0, 0.5, 0.5, 0.0)
    assert O.time_coefs("bd2si", 3) == (1.5, 2.0, -0.5, 0.75, 0.5, -0.25)
    with pytest.raises(ValueError):
        O.time_coefs("bogus", 1)


def _naive_rheology(chi, mu, par):
    """compute_rheology_reference of test/test_update.jl:8-28."""
    f = (chi, mu)
    AA, BB, CC = np.array(par.AA), np.array(par.BB), np.array(par.CC)
    Sf = np.array([[(f[j] / BB[i, j]) ** (1.0 / CC[i, j]) for j in range(2)] for i in range(2)])
    Sf = Sf / Sf.sum(axis=1, keepdims=True)
    Xf = np.empty((2, 2))
    for i in range(2):
        a = AA[i, 0] * Sf[i, 0] + AA[i, 1] * Sf[i, 1]
        Xf[i, 0] = a * f[0] + (1 - a) * Sf[i, 0]
        Xf[i, 1] = a * f[1] + (1 - a) * Sf[i, 1]
    kv = (par.etax0, par.etam0)
    thtv = [(kv[0] / kv[i]) ** Xf[i, 0] * (kv[1] / kv[i]) ** Xf[i, 1] for i in range(2)]
    etaf = (kv[0] * thtv[0], kv[1] * thtv[1])
    return chi * etaf[0] + mu * etaf[1]


@pytest.mark.parametrize("chi,mu", [(0.3, 0.7), (0.5, 0.5), (0.1, 0.9), (0.9, 0.1)])
def test_rheology_matches_naive(chi, mu):
    """test/test_update.jl:30-47 (rtol 1e-12 in Float64)."""
    par = O.Params()
    got = O.rheology(np.array([[chi]]), np.array([[mu]]), par)[0, 0]
    assert got == pytest.approx(_naive_rheology(chi, mu, par), rel=1e-12)


def test_kinematics_convergence():
    """test/test_update.jl:49-94: strain-rate order > 1.8 and Div V ~ 0."""
    errs_exx, errs_ezz, errs_div = [], [], []
    for N in (16, 32, 64):
        L = 2 * math.pi
        h = L / N
        par = O.Params(D=L, N=N, L=L)
        g = O.make_grid(par)
        st = O.State(g.Nz, g.Nx)
        j = np.arange(N + 1)[:, None]
        i = np.arange(N + 2)[None, :]
        st.W = np.sin(j * h) * np.cos((i - 0.5) * h)
        j = np.arange(N + 2)[:, None]
        i = np.arange(N + 1)[None, :]
        st.U = -np.cos((j - 0.5) * h) * np.sin(i * h)
        O.update_kinematics(st, g)
        c = (np.arange(1, N + 1) - 0.5) * h
        ex = -np.cos(c)[:, None] * np.cos(c)[None, :]
        errs_exx.append(np.linalg.norm(st.exx - ex) / np.linalg.norm(ex))
        errs_ezz.append(np.linalg.norm(st.ezz + ex) / np.linalg.norm(ex))
        errs_div.append(np.linalg.norm(st.Div_V))
    for e in (errs_exx, errs_ezz):
        assert math.log2(e[0] / e[1]) > 1.8
        assert math.log2(e[1] / e[2]) > 1.8
    assert errs_div[-1] < 1e-10


def _mms_state(N):
    L = 10.0
    m = mms_sources(N, L)
    par = O.Params(D=L, N=N, L=L, etam0=1e3, g0=10.0, rhom0=2700, rhox0=3200, d0=1e-2,
                   Da=0.0, Xi=0.0, gamma=0.0)
    g = O.make_grid(par)
    st = O.State(g.Nz, g.Nx)
    for k in ("eta", "etaco", "rho", "rhow", "rhou", "Drho", "MFS"):
        setattr(st, k, m[k].copy())
    bn = O.Bnchm(m["src_W"], m["src_U"], m["src_P"], m["W_exact"], m["U_exact"], m["P_exact"])
    return par, g, st, bn, m


def test_mms_stokes_convergence():
    """test/test_mms.jl:4-71: W, U, P second order (> 1.8) at N = 32, 64, 128."""
    errs = {"W": [], "U": [], "P": []}
    for N in (32, 64, 128):
        par, g, st, bn, m = _mms_state(N)
        O.fluidmech(st, g, par, (1.0, 1.0, 0.0, 1.0, 0.0, 0.0), 1e32, bn=bn, sds=-1, top_cnv=-1, bot_cnv=-1)
        for k in errs:
            errs[k].append(np.linalg.norm(getattr(st, k) - m[k + "_exact"]) / np.linalg.norm(m[k + "_exact"]))
    for k, e in errs.items():
        assert math.log2(e[0] / e[1]) > 1.8, (k, e)
        assert math.log2(e[1] / e[2]) > 1.8, (k, e)


def _small_run(N=16, seed=3):
    par = O.Params(D=10.0, N=N, L=10.0, etam0=10.0, x0=0.05, dxr=0.1, Da=0.0, TINT="bd2im",
                   ADVN="weno5", alpha=0.5)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(seed)
    rp = rng.standard_normal((g.Nz, g.Nx))
    rp = (rp - rp.mean()) / rp.std(ddof=1)
    x0 = par.x0 * (1 + par.dxr * rp)
    st = O.initialize(g, par, sc, ns, x0, rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx)))
    return par, g, sc, ns, st, rng


def test_store_previous_chain():
    """test/test_run.jl:27-46."""
    par, g, sc, ns, st, _ = _small_run(N=8)
    st.X[0, 0] = 7.0
    O.store_previous(st)
    assert st.Xo[0, 0] == 7.0
    st.X[0, 0] = 9.0
    O.store_previous(st)
    assert st.Xo[0, 0] == 9.0 and st.Xoo[0, 0] == 7.0


def test_resnorm_zero_without_change():
    """test/test_diagnose.jl:52-63."""
    par, g, sc, ns, st, _ = _small_run(N=8)
    snap = O.snapshot(st)
    assert O.resnorm(st, snap, sc["dt0"]) == (0.0, 0.0, 0.0)


def test_noise_draw_reused_and_finite():
    """test/test_noise.jl:61-92: first sweep takes the draw, later sweeps reuse it."""
    par, g, sc, ns, st, rng = _small_run(N=16)
    re, rs = rng.standard_normal((16, 16)), rng.standard_normal((16, 16))
    O.noise(st, g, par, sc, ns, sc["dt0"], True, re, rs)
    re1 = st.re.copy()
    O.noise(st, g, par, sc, ns, sc["dt0"], False, None, None)
    assert np.array_equal(st.re, re1)
    for k in ("xie", "xix", "xis"):
        v = getattr(st, k)
        assert np.all(np.isfinite(v)) and np.all(v >= 0)


def test_run_five_steps_finite():
    """test/test_run.jl:48-73: 5 WENO5 steps at N = 16 stay finite, 0 < x < 1."""
    par, g, sc, ns, st, rng = _small_run(N=16)
    dt = sc["dt0"]
    for step in range(1, 6):
        dt, _ = O.timestep(st, g, par, sc, ns, step, dt, rng.standard_normal((16, 16)),
                           rng.standard_normal((16, 16)))
    assert math.isfinite(dt) and dt > 0
    assert np.all(np.isfinite(st.x)) and np.all(st.x > 0) and np.all(st.x < 1)
    for k in ("W", "U", "P", "eta", "etamix"):
        assert np.all(np.isfinite(getattr(st, k)))
    assert np.all(st.eta > 0) and np.all(st.etamix > 0)


def test_fft_filter_is_the_exact_dft_filter():
    """The numpy FFT that stands in for FFTW (src/noise.jl:254-256) against a
    direct O(n^2) DFT of the same padded field: same filtered field to 1e-12."""
    rng = np.random.default_rng(1)
    Nz, Nx, pad, h, sig = 12, 10, 4, 0.1, 0.15
    psi = rng.standard_normal((Nz, Nx))
    Gk = O.make_gaussian_filter(Nz + pad, Nx, h, sig)
    got = O.fft_filter(psi, Gk, pad)
    nz = Nz + pad
    Fz = np.exp(-2j * np.pi * np.outer(np.arange(nz), np.arange(nz)) / nz)
    Fx = np.exp(-2j * np.pi * np.outer(np.arange(Nx), np.arange(Nx)) / Nx)
    pp = np.zeros((nz, Nx), complex)
    pp[pad // 2:pad // 2 + Nz] = psi
    spec = Fz @ pp @ Fx.T
    back = (np.conj(Fz) @ (spec * Gk) @ np.conj(Fx).T) / (nz * Nx)
    flt = back[pad // 2:pad // 2 + Nz].real
    flt = (flt - flt.mean()) * O.std1(psi) / O.std1(flt) + psi.mean()
    assert np.allclose(got, flt, rtol=1e-12, atol=1e-12 * np.abs(flt).max())
    # the re-standardisation keeps mean and corrected std (src/noise.jl:261-267)
    assert got.mean() == pytest.approx(psi.mean(), abs=1e-12)
    assert O.std1(got) == pytest.approx(O.std1(psi), rel=1e-12)


def test_advect_flux_divergence_identity():
    """advect.jl:428-432: adv is bitwise the divergence of the emitted face
    fluxes, for every scheme."""
    rng = np.random.default_rng(2)
    Nz, Nx, h = 9, 11, 0.3
    f = rng.random((Nz, Nx))
    u = rng.standard_normal((Nz, Nx + 1))
    w = rng.standard_normal((Nz + 1, Nx))
    for scheme in O.SCHEME_HALO:
        adv, qx, qz = O.advect_centered_with_flux(f, u, w, h, scheme)
        adv2 = O.divergence(qx[1:-1, :], qz[:, 1:-1], 1.0 / h)
        assert np.array_equal(adv, adv2)
        assert np.all(np.isfinite(adv))


def _literal_cell_kernel(fh, u, w, h, scheme, g):
    """The reference's per-cell divergence kernels written out literally
    (src/kernels/advect.jl:57-96 WENO5, 130-170 QUICK): four face values per
    direction computed from the cell's own stencil."""
    Nz, Nx = fh.shape[0] - 2 * g, fh.shape[1] - 2 * g

    def F(dz, dx):
        return fh[g + dz:g + dz + Nz, g + dx:g + dx + Nx]
    invh, half = 1.0 / h, 0.5
    fc = F(0, 0)
    if scheme == "weno5":
        P = lambda a, b, c, d, e: O.weno5_poly(a, b, c, d, e, O.EPS)
        fxppos = P(F(0, -2), F(0, -1), fc, F(0, 1), F(0, 2))
        fxpneg = P(F(0, 3), F(0, 2), F(0, 1), fc, F(0, -1))
        fxmpos = P(F(0, -3), F(0, -2), F(0, -1), fc, F(0, 1))
        fxmneg = P(F(0, 2), F(0, 1), fc, F(0, -1), F(0, -2))
        fzppos = P(F(-2, 0), F(-1, 0), fc, F(1, 0), F(2, 0))
        fzpneg = P(F(3, 0), F(2, 0), F(1, 0), fc, F(-1, 0))
        fzmpos = P(F(-3, 0), F(-2, 0), F(-1, 0), fc, F(1, 0))
        fzmneg = P(F(2, 0), F(1, 0), fc, F(-1, 0), F(-2, 0))
    else:
        s = 1.0 / 6.0
        fxppos = s * ((2 * F(0, 1) + 5 * fc) - F(0, -1))
        fxpneg = s * ((2 * fc + 5 * F(0, 1)) - F(0, 2))
        fxmpos = s * ((2 * fc + 5 * F(0, -1)) - F(0, -2))
        fxmneg = s * ((2 * F(0, -1) + 5 * fc) - F(0, 1))
        fzppos = s * ((2 * F(1, 0) + 5 * fc) - F(-1, 0))
        fzpneg = s * ((2 * fc + 5 * F(1, 0)) - F(2, 0))
        fzmpos = s * ((2 * fc + 5 * F(-1, 0)) - F(-2, 0))
        fzmneg = s * ((2 * F(-1, 0) + 5 * fc) - F(1, 0))
    ul, ur = u[:, :-1], u[:, 1:]
    wt, wb = w[:-1, :], w[1:, :]
    sp = lambda v: ((v + np.abs(v)) * half, (v - np.abs(v)) * half)
    (ulp, uln), (urp, urn), (wtp, wtn), (wbp, wbn) = sp(ul), sp(ur), sp(wt), sp(wb)
    qxr = urp * fxppos + urn * fxpneg
    qxl = ulp * fxmpos + uln * fxmneg
    qzb = wbp * fzppos + wbn * fzpneg
    qzt = wtp * fzmpos + wtn * fzmneg
    return (((qxr - qxl) + qzb) - qzt) * invh


@pytest.mark.parametrize("scheme", ["weno5", "quick"])
def test_flux_form_equals_literal_cell_kernel(scheme):
    """The oracle's flux-difference form reproduces the reference's per-cell
    kernel bit for bit (the identity advect.jl:428-432 states)."""
    rng = np.random.default_rng(5)
    Nz, Nx, h = 13, 10, 0.25
    g = O.scheme_halo(scheme)
    f = rng.random((Nz, Nx)) * 3 + rng.standard_normal((Nz, Nx)) ** 3
    fh = O.embed_halo(f, g, "closed", "periodic")
    u = rng.standard_normal((Nz, Nx + 1))
    w = rng.standard_normal((Nz + 1, Nx))
    qx, qz = O.advect_fluxes(fh, u, w, scheme, g)
    assert np.array_equal(O.divergence(qx, qz, 1.0 / h), _literal_cell_kernel(fh, u, w, h, scheme, g))


def test_grid_sizes_and_ghost_maps():
    """test/test_grid.jl:1-29: sizes, spacing and the ghost index vectors
    (0-based here: Julia's icx = [Nx; 1:Nx; 1] is [Nx-1, 0..Nx-1, 0])."""
    g = O.make_grid(O.Params(D=10.0, N=100, L=10.0))
    assert (g.Nz, g.Nx, g.h) == (100, 100, 0.1)
    icx, icz = O.icx_of(g.Nx, "periodic"), O.icz_of(g.Nz, "closed")
    assert icx[0] == g.Nx - 1 and icx[-1] == 0 and len(icx) == g.Nx + 2
    assert icz[0] == 0 and icz[-1] == g.Nz - 1
    assert O.make_grid(O.Params(D=10.0, N=50, L=15.0)).Nx == 75


def test_scales_fixed_point_and_ordering():
    """test/test_scales.jl:1-30: the convection speed is the fixed point of its
    defining relation to 1e-12, and the derived scales have the stated signs
    and ranges; the package's host restatement gives the same numbers."""
    import xcore_gb300 as xc
    par = O.Params(D=10.0, N=200, L=15.0, d0=1e-2, etam0=1e1, rhom0=2700, rhox0=3200, g0=10.0, L0=10.0 / 100,
                   l0=1e-2 * 10, Da=0.01, Xi=0.5, x0=float(np.finfo(np.float64).eps))
    g = O.make_grid(par)
    s = O.compute_scales(par, g)
    Ri2 = s["Ri0"] ** 2
    W0 = (math.sqrt(4 / Ri2 * s["Dchi0"] * s["Drho0"] * par.g0 * s["rho0"] * s["fReL0"] * s["L0"] ** 2 * s["D0"]
                    + s["eta0"] ** 2) - s["eta0"]) * s["D0"] / (2 * s["fReL0"] * s["L0"] ** 2 * s["rho0"] / Ri2)
    assert W0 == pytest.approx(s["W0"], rel=1e-12)
    assert s["W0l"] > 0 and s["W0"] > 0 and s["w0"] > 0
    assert 0 < s["fReL0"] <= 1 and 0 < s["fRel0"] <= 1
    pp = xc.Parameters(**{k: getattr(par, k) for k in xc.Parameters.__dataclass_fields__ if hasattr(par, k)})
    ps = xc.compute_scales(pp, xc.Grid(Nx=g.Nx, Nz=g.Nz, h=g.h, D=g.D, L=g.L))
    common = [k for k in ps if k in s]
    assert len(common) >= 10
    for k in common:
        assert ps[k] == pytest.approx(s[k], rel=1e-14), k


def test_resnorm_positive_after_change():
    """test/test_diagnose.jl:65-78: after a field changes, compute_resnorm is
    positive."""
    par = O.Params(D=10.0, N=16, L=10.0, x0=0.05, Da=0.0)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(3)
    x0 = np.clip(rng.uniform(0.02, 0.1, (g.Nz, g.Nx)), 0, 1)
    st = O.initialize(g, par, sc, ns, x0, rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx)))
    snap = O.snapshot(st)
    st.X = st.X * 1.01
    assert O.resnorm(st, snap, sc["dt0"])[0] > 0


def test_resnorm_raises_resnorm0_when_the_residual_rises():
    """test/test_diagnose.jl:80-91: with resnorm0 = 1e-10, a change of W makes
    compute_resnorm set resnorm0 to resnorm + 1e-32; snapshot! keeps it."""
    par, g, sc, ns, st, _ = _small_run(N=8)
    res = O.snapshot(st)
    assert res["resnorm0"] == 1.0
    res["resnorm0"] = 1e-10
    res = O.snapshot(st, res)
    assert res["resnorm0"] == 1e-10
    st.W = st.W + 1.0
    rn = O.resnorm(st, res, sc["dt0"])[0]
    assert rn > 1e-10
    assert res["resnorm0"] == pytest.approx(rn + 1e-32)
    # a smaller residual leaves it where it is
    res = O.snapshot(st, res)
    st.W = st.W + 1e-6
    O.resnorm(st, res, sc["dt0"])
    assert res["resnorm0"] == pytest.approx(rn + 1e-32)


def _noise_setup(N=16, seed=42):
    """test/test_noise.jl:8-19: Parameters(D = 10, N, L = 10, etam0 = 10,
    x0 = 0.1, Da = 0, Xi = 0.5) after initialize! (the initial draw supplied)."""
    par = O.Params(D=10.0, N=N, L=10.0, etam0=10.0, x0=0.1, Da=0.0, Xi=0.5)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(seed)
    rp = rng.standard_normal((g.Nz, g.Nx))
    rp = (rp - rp.mean()) / rp.std(ddof=1)
    x0 = par.x0 * (1 + par.dxr * rp)
    st = O.initialize(g, par, sc, ns, x0, rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx)))
    return par, g, sc, ns, st, rng


def test_store_noise_snapshots_potentials():
    """test/test_noise.jl:44-59."""
    par, g, sc, ns, st, rng = _noise_setup()
    st.psie[:] = 1.0
    st.psix[:] = 2.0
    st.psis[:] = 3.0
    O.store_noise(st)
    assert np.all(st.psieo == 1.0) and np.all(st.psixo == 2.0) and np.all(st.psiso == 3.0)
    st.psie[:] = 7.0
    O.store_noise(st)
    assert np.all(st.psieo == 7.0)


def test_noise_speeds_and_fluxes_finite_over_sweeps():
    """test/test_noise.jl:61-76: three noise! calls, the first drawing; the
    speed magnitudes are finite and non-negative, the fluxes finite."""
    par, g, sc, ns, st, rng = _noise_setup()
    for it in range(3):
        first = it == 0
        re = rng.standard_normal((g.Nz, g.Nx)) if first else None
        rs = rng.standard_normal((g.Nz, g.Nx)) if first else None
        O.noise(st, g, par, sc, ns, sc["dt0"], first, re, rs)
    for k in ("xie", "xix", "xis"):
        v = getattr(st, k)
        assert np.all(np.isfinite(v)) and np.all(v >= 0), k
    for k in ("xiew", "xieu", "xixw", "xixu"):
        assert np.all(np.isfinite(getattr(st, k))), k


def test_noise_from_zero_potential_finite():
    """test/test_noise.jl:94-110 (N = 24): psie = psieo = 0 and a fresh draw."""
    par, g, sc, ns, st, rng = _noise_setup(N=24)
    O.store_noise(st)
    st.psie[:] = 0.0
    st.psieo[:] = 0.0
    O.noise(st, g, par, sc, ns, sc["dt0"], True, rng.standard_normal((g.Nz, g.Nx)),
            rng.standard_normal((g.Nz, g.Nx)))
    assert np.all(np.isfinite(st.xie)) and np.all(np.isfinite(st.xiew))


def test_update_end_to_end_smoke():
    """test/test_update.jl:96-131: update! on a smooth x perturbation with a
    weak W seed keeps rho, etamix, eta positive and finite, eII, tII >= 0."""
    par = O.Params(D=10.0, N=32, L=10.0, etam0=10.0, x0=0.1)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    st = O.State(g.Nz, g.Nx)
    j = np.arange(1, g.Nz + 1)[:, None]
    i = np.arange(1, g.Nx + 1)[None, :]
    zg = (j - 0.5) * g.h / g.D
    xg = (i - 0.5) * g.h / g.L
    st.x = 0.1 + 0.05 * np.sin(2 * math.pi * zg) * np.cos(2 * math.pi * xg)
    st.m = 1.0 - st.x
    st.eta[:] = par.etam0
    st.etaco[:] = par.etam0
    nW = st.W.shape[0]
    st.W = np.repeat(1e-3 * np.sin(np.arange(nW) * 2 * math.pi / nW)[:, None], st.W.shape[1], axis=1)
    O.update(st, g, par, sc)
    for k, positive in (("rho", True), ("etamix", True), ("eta", True), ("eII", False), ("tII", False)):
        v = getattr(st, k)
        assert np.all(np.isfinite(v)), k
        assert np.all(v > 0) if positive else np.all(v >= 0), k
    assert st.chi.shape == (g.Nz, g.Nx) and st.etamix.shape == (g.Nz, g.Nx)
    assert st.exz.shape == (g.Nz + 1, g.Nx + 1)


def test_history_stats_ordering_and_finite():
    """test/test_history.jl:50-73 on the initialized N = 8 state of
    test/test_history.jl:6-16: min <= mean <= max for x, min <= rms <= max
    (+ sqrt(eps)) for V and vx, every recorded value finite."""
    par = O.Params(D=10.0, N=8, L=10.0, etam0=10.0, x0=0.1, Da=0.0)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(5)
    rp = rng.standard_normal((g.Nz, g.Nx))
    rp = (rp - rp.mean()) / rp.std(ddof=1)
    st = O.initialize(g, par, sc, ns, par.x0 * (1 + par.dxr * rp), rng.standard_normal((g.Nz, g.Nx)),
                      rng.standard_normal((g.Nz, g.Nx)))
    h = O.history_stats(st)
    tol = math.sqrt(np.finfo(np.float64).eps)
    assert h["x_min"] <= h["x_mean"] <= h["x_max"]
    assert h["V_min"] <= h["V_rms"] <= h["V_max"] + tol
    assert h["vx_min"] <= h["vx_rms"] <= h["vx_max"] + tol
    assert all(math.isfinite(v) for v in h.values())
    assert all(math.isfinite(v) for v in O.conservation_sums(st, g).values())


def test_snapshot_copies_primary_fields():
    """test/test_diagnose.jl:34-50: snapshot! copies W, U, X into its own
    buffers; changing a field afterwards leaves the snapshot unchanged."""
    par, g, sc, ns, st, rng = _small_run(N=8)
    st.W[1, 1] = 42.0
    st.U[2, 1] = -7.0
    st.X[0, 0] = 0.3
    snap = O.snapshot(st)
    assert snap["W"][1, 1] == 42.0 and snap["U"][2, 1] == -7.0 and snap["X"][0, 0] == 0.3
    st.W[1, 1] = 0.0
    assert snap["W"][1, 1] == 42.0


# src/parameters.jl:14-86, the defaults of Parameters{Float64}() the path reads
REFERENCE_DEFAULTS = dict(
    D=10.0, N=100, L=10.0, x0=float(np.finfo(np.float64).eps), dxr=0.1, dxg=0.0, rhom0=2700.0, rhox0=3200.0,
    d0=0.01, g0=10.0, etam0=10.0, etax0=1e18, AA=((0.72, 0.19), (0.81, 0.20)), BB=((0.63, 0.37), (0.999, 0.001)),
    CC=((2.09, 0.09), (0.37, 1.45)), L0=0.1, l0=0.1, Da=0.01, Xi=0.5, Ptop=1e5, open_sgr=False, TINT="bd2im",
    ADVN="weno5", CFL=0.5, rtol=1e-4, atol=1e-9, maxit=15, alpha=0.9, gamma=1e-3, dtmax=1e32, etacntr=1e8)


def test_parameter_defaults_match_the_reference():
    """test/test_parameters.jl:1-6 (D = 10, N = 100, ADVN = :weno5) and every
    other default the path reads, for the oracle's Params and the library's
    Python Parameters alike."""
    import xcore_gb300 as xc
    for cls in (O.Params, xc.Parameters):
        p = cls()
        for k, v in REFERENCE_DEFAULTS.items():
            if hasattr(p, k):
                assert getattr(p, k) == v, (cls.__name__, k)
    p = O.Params()
    assert all(hasattr(p, k) for k in REFERENCE_DEFAULTS), "the oracle carries every default"
