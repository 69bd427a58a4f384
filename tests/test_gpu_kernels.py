"""GPU parity of the time-step kernels against the CPU oracle, through the C ABI.

Bitwise where the path is pure +,-,*,/ and sqrt (stencils, phsevo!, store,
phase velocities, kinematics, interpolations); normwise relative error
<= 1e-12 per field (the reference tolerance for stencils and noise) where CUDA's
exp / pow enter (rheology, viscosity, noise)."""
import numpy as np
import pytest

import xcore_oracle as O
from gpu_helpers import (assert_fields, device_state, realistic_state, rel_err)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import xcore_gb300 as xc  # noqa: E402

SCHEMES = list(O.SCHEME_HALO)


def _dev(a):
    """numpy [z, x] -> contiguous CUDA tensor holding the column-major bytes."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda()


def _host(t):
    return t.cpu().numpy().T


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("shape", [(37, 45), (64, 32), (5, 7)])
@pytest.mark.parametrize("bcs", [("periodic", "closed"), ("closed", "periodic"), ("periodic", "periodic")])
def test_advect_centered_with_flux_bitwise(scheme, shape, bcs):
    Nz, Nx = shape
    xBC, zBC = bcs
    g = O.scheme_halo(scheme)
    if Nz < g or Nx < g:
        pytest.skip("grid smaller than halo")
    rng = np.random.default_rng(Nz * 100 + Nx + g)
    f = rng.random((Nz, Nx)) * 2 + rng.standard_normal((Nz, Nx)) ** 3
    u = rng.standard_normal((Nz, Nx + 1))
    w = rng.standard_normal((Nz + 1, Nx))
    h = 0.37
    adv, qx, qz = O.advect_centered_with_flux(f, u, w, h, scheme, xBC, zBC)
    d_adv = torch.zeros((Nx, Nz), dtype=torch.float64, device="cuda")
    d_qx = torch.zeros((Nx + 1, Nz + 2), dtype=torch.float64, device="cuda")
    d_qz = torch.zeros((Nx + 2, Nz + 1), dtype=torch.float64, device="cuda")
    xc.advect_centered_with_flux(d_adv, d_qx, d_qz, _dev(f), _dev(u), _dev(w), h, scheme, xBC, zBC)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_adv), adv)
    np.testing.assert_array_equal(_host(d_qx), qx)
    np.testing.assert_array_equal(_host(d_qz), qz)


@pytest.mark.parametrize("scheme", ["weno5", "quick", "tvdim", "centr"])
def test_advect_halo_input_bitwise(scheme):
    """advect! / advect_with_flux! on a caller-filled halo (advect.jl:374, 717)."""
    Nz, Nx = 33, 29
    g = O.scheme_halo(scheme)
    rng = np.random.default_rng(11)
    f = rng.random((Nz, Nx))
    u = rng.standard_normal((Nz, Nx + 1))
    w = rng.standard_normal((Nz + 1, Nx))
    fh = O.embed_halo(f, g, "closed", "periodic")
    uu, ww = (O._pad_velocity_tvd(u, w, "periodic", "closed") if scheme == "tvdim" else (u, w))
    adv, qx, qz = O.advect_centered_with_flux(f, u, w, 0.2, scheme)
    d_adv = torch.zeros((Nx, Nz), dtype=torch.float64, device="cuda")
    xc.advect(d_adv, _dev(fh), _dev(uu), _dev(ww), 0.2, scheme)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_adv), adv)
    d_qx = torch.zeros((Nx + 1, Nz + 2), dtype=torch.float64, device="cuda")
    d_qz = torch.zeros((Nx + 2, Nz + 1), dtype=torch.float64, device="cuda")
    xc.advect_with_flux(d_adv, d_qx, d_qz, _dev(fh), _dev(uu), _dev(ww), 0.2, scheme)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_qx), qx)
    np.testing.assert_array_equal(_host(d_qz), qz)


def test_diffus_and_ghosts_bitwise():
    Nz, Nx = 41, 23
    rng = np.random.default_rng(3)
    f = rng.random((Nz, Nx))
    k = rng.random((Nz, Nx)) + 0.5
    dff, qx, qz = O.diffus_centered_with_flux(f, k, 0.3)
    fh = np.zeros((Nz + 2, Nx + 2))
    fh[1:-1, 1:-1] = f
    kh = np.zeros((Nz + 2, Nx + 2))
    kh[1:-1, 1:-1] = k
    d_fh, d_kh = _dev(fh), _dev(kh)
    xc.fill_ghosts(d_fh, 1)
    xc.fill_ghosts(d_kh, 1)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_fh), O.embed_halo(f, 1, "closed", "periodic"))
    d_dff = torch.zeros((Nx, Nz), dtype=torch.float64, device="cuda")
    d_qx = torch.zeros((Nx + 1, Nz + 2), dtype=torch.float64, device="cuda")
    d_qz = torch.zeros((Nx + 2, Nz + 1), dtype=torch.float64, device="cuda")
    xc.diffus_with_flux(d_dff, d_qx, d_qz, d_fh, d_kh, 0.3)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_dff), dff)
    np.testing.assert_array_equal(_host(d_qx), qx)
    np.testing.assert_array_equal(_host(d_qz), qz)
    xc.diffus(d_dff, d_fh, d_kh, 0.3)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d_dff), dff)


def test_ghosts_halo3_both_closed():
    Nz, Nx, g = 9, 6, 3
    f = np.random.default_rng(1).random((Nz, Nx))
    fh = np.zeros((Nz + 2 * g, Nx + 2 * g))
    fh[g:-g, g:-g] = f
    d = _dev(fh)
    xc.fill_ghosts(d, g, zBC="closed", xBC="closed")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_host(d), O.embed_halo(f, g, "closed", "closed"))


@pytest.mark.parametrize("scheme", ["weno5", "quick"])
def test_phsevo_bitwise(scheme):
    par, g, sc, ns, st, dt, rng = realistic_state(ADVN=scheme)
    ds = device_state(par, g, sc, st)
    coefs = O.time_coefs("bd2im", 3)
    O.phsevo(st, g, par, sc, scheme, coefs, dt)
    ds.phsevo(coefs, dt, ADVN=scheme)
    assert_fields(ds, st, ["advn_X", "advn_M", "advn_rho", "dffn_X", "qx_advn_X", "qz_advn_X",
                           "qx_advn_M", "qz_advn_M", "qx_dffn_X", "qz_dffn_X", "Gx", "dXdt", "X", "M",
                           "x", "m"], exact=True)


@pytest.mark.parametrize("ADVN", ["weno5", "weno3"])
def test_phsevo_weno5_one_division_weights(ADVN):
    """weno_weights = 1: WENO5's nonlinear weights over a common denominator,
    one division per reconstruction; within 1e-12 of the reference's form
    (and WENO3, which it does not touch, still bit for bit)."""
    par, g, sc, ns, st, dt, rng = realistic_state(N=40, Nx=36, ADVN=ADVN)
    ds = device_state(par, g, sc, st, weno_weights=1)
    coefs = O.time_coefs("bd2im", 3)
    O.phsevo(st, g, par, sc, ADVN, coefs, dt)
    ds.phsevo(coefs, dt, ADVN=ADVN)
    names = ["advn_X", "advn_M", "qx_advn_X", "qz_advn_X", "qx_advn_M", "qz_advn_M", "Gx", "dXdt", "X", "M",
             "x", "m"]
    assert_fields(ds, st, names, exact=ADVN == "weno3", tol=1e-12)
    ds.close()


def test_store_and_phase_velocities_bitwise():
    par, g, sc, ns, st, dt, rng = realistic_state()
    ds = device_state(par, g, sc, st)
    O.store_previous(st)
    ds.store_previous()
    assert_fields(ds, st, ["Xo", "Xoo", "Mo", "Moo", "dXdto", "dXdtoo", "rhoo", "rhooo", "drhodto",
                           "drhodtoo", "rhoWo", "rhoWoo", "rhoUo", "rhoUoo"], exact=True)
    O.update_phase_velocities(st, g, par)
    ds.update_phase_velocities()
    assert_fields(ds, st, ["wx", "wm", "Wx", "Wm", "Ux", "Um"], exact=True)


def test_update_parity():
    par, g, sc, ns, st, dt, rng = realistic_state()
    ds = device_state(par, g, sc, st)
    O.update(st, g, par, sc)
    ds.update()
    exact = ["rho", "chi", "mu", "rhow", "rhou", "Drho", "Drhom", "Drhox", "chiw", "muw", "chiu", "muu",
             "x_w", "m_w", "x_u", "m_u", "Pl", "Pt", "exx", "ezz", "exz", "Div_V", "eII", "V", "vx", "vm"]
    assert_fields(ds, st, exact, exact=True)
    assert np.array_equal(ds["hasx"], st.hasx.astype(bool)) and np.array_equal(ds["hasm"], st.hasm.astype(bool))
    assert_fields(ds, st, ["etamix", "etae", "ke", "kx", "ReL", "fReL", "eta", "ReD", "etaco", "Rel", "fRel",
                           "ks", "etat", "etas", "Red", "etasw", "Rc", "txz", "txx", "tzz", "tII", "Ra"],
                  tol=1e-12)


@pytest.mark.parametrize("first", [True, False])
def test_noise_parity(first):
    par, g, sc, ns, st, dt, rng = realistic_state()
    ds = device_state(par, g, sc, st)
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    ds["re"], ds["rs"] = st.re, st.rs
    O.noise(st, g, par, sc, ns, dt, first, re, rs)
    ds.noise(dt, first, re if first else None, rs if first else None)
    assert_fields(ds, st, ["re", "rs"], exact=True)
    assert_fields(ds, st, ["psie", "psix", "psis", "xiew", "xieu", "xixw", "xixu", "xisw", "xisu",
                           "xie", "xix", "xis"], tol=1e-12)


@pytest.mark.parametrize("shape", [(100, 100), (64, 96), (30, 17)])
def test_noise_filter_sizes(shape):
    """The separable FFT filter at non-power-of-two and power-of-two sizes."""
    N, Nx = shape
    par, g, sc, ns, st, dt, rng = realistic_state(N=N, Nx=Nx, steps=0)
    ds = device_state(par, g, sc, st)
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    O.noise(st, g, par, sc, ns, dt, True, re, rs)
    ds.noise(dt, True, re, rs)
    assert_fields(ds, st, ["xiew", "xieu", "xixw", "xixu", "xisw", "xisu", "xie", "xix", "xis"], tol=1e-12)


def test_dt_resnorm_sums():
    par, g, sc, ns, st, dt, rng = realistic_state()
    ds = device_state(par, g, sc, st)
    assert ds.update_dt(dt) == O.update_dt(st, g, par, dt)
    snap = O.snapshot(st)
    ds.snapshot()
    assert ds.compute_resnorm(dt) == (0.0, 0.0, 0.0)
    st.X = st.X * 1.001
    st.W = st.W + 1e-3
    ds["X"], ds["W"] = st.X, st.W
    got = ds.compute_resnorm(dt)
    ref = O.resnorm(st, snap, dt)
    np.testing.assert_allclose(got, ref, rtol=1e-12)
    # compute_resnorm's resnorm0 rule as the oracle's StepResidual has it
    # (test/test_diagnose.jl:80-91)
    res = O.snapshot(st)
    ds.snapshot()
    res["resnorm0"] = ds.resnorm0 = 1e-10
    st.W = st.W + 1.0
    ds["W"] = st.W
    rn = ds.compute_resnorm(dt)[0]
    assert rn == pytest.approx(O.resnorm(st, res, dt)[0], rel=1e-12)
    assert ds.resnorm0 == pytest.approx(rn + 1e-32) and res["resnorm0"] == pytest.approx(ds.resnorm0, rel=1e-12)
    s = ds.conservation_sums()
    r = O.conservation_sums(st, g)
    for k, v in r.items():
        assert s[k] == pytest.approx(v, rel=1e-12, abs=1e-12 * max(1.0, abs(r["sumB"]))), k


def test_initialize_parity():
    par = None
    from gpu_helpers import oracle_params
    par = oracle_params(32, 24)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    rng = np.random.default_rng(5)
    x0 = rng.uniform(0.02, 0.1, (g.Nz, g.Nx))
    re, rs = rng.standard_normal((g.Nz, g.Nx)), rng.standard_normal((g.Nz, g.Nx))
    st = O.initialize(g, par, sc, ns, x0, re, rs)
    ds = device_state(par, g, sc)
    ds.initialize(x0, re, rs)
    assert_fields(ds, st, ["x", "m", "X", "M", "rho", "chi", "mu", "Xo", "Xoo", "rhoo", "bndshape", "bndtaperw",
                           "eta", "etaco", "etas", "Wx", "Wm", "Ux", "Um", "psie", "psieo", "xie"], tol=1e-12)


def test_bad_arguments_fail_loudly():
    """Arguments the host side rejects before any launch (advect.jl:354,421)."""
    d = torch.zeros((8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(KeyError):
        xc.advect(d, d, d, d, 0.1, "bogus")
    r = xc.lib().xc_advect(xc._ptr(d), xc._ptr(d), xc._ptr(d), xc._ptr(d), 8, 8, 0.1, 42, None)
    assert r == xc.XC_BAD_ARG and b"scheme" in xc.lib().xc_last_error()
    r = xc.lib().xc_fill_ghosts(xc._ptr(d), 2, 2, 3, 0, 0, None)
    assert r == xc.XC_BAD_ARG
    with pytest.raises(xc.XcoreError):
        xc.State(xc.Parameters(N=2))
