"""Manufactured Stokes solution used by the MMS convergence tests.

Restates the manufactured fields and their hand-derived Stokes residuals that
the reference's test helper builds (test/mms_sources.jl:36-145): the same
sinusoidal forms, coefficients and staggered evaluation grids."""
import numpy as np


def mms_sources(N: int, L: float):
    h = L / N
    aW, aU, aP = 5e-5, 4e-5, -3e3
    eta0, aeta = 1e3, -9e2
    rho0, arho = 3e3, -5e1
    asrc, rhoref, g0 = -1e3, 3e3, 10.0
    k = 4.0 * np.pi / L
    x = -h / 2 + np.arange(N + 2) * h
    z = -h / 2 + np.arange(N + 2) * h
    xu = (x[:-1] + x[1:]) / 2
    zw = (z[:-1] + z[1:]) / 2

    def grid(zs, xs):
        return np.meshgrid(zs, xs, indexing="ij")

    C = lambda X, Z: np.cos(k * X) * np.sin(k * Z)
    S = lambda X, Z: np.sin(k * X) * np.cos(k * Z)
    CC = lambda X, Z: np.cos(k * X) * np.cos(k * Z)
    SS = lambda X, Z: np.sin(k * X) * np.sin(k * Z)
    a_exx = (2 * aU - aW) / 3
    a_ezz = (2 * aW - aU) / 3
    a_exz = -(aW + aU) / 2

    def fields(X, Z):
        eta = eta0 + aeta * C(X, Z)
        rho = rho0 + arho * C(X, Z)
        exx = k * CC(X, Z) * a_exx
        ezz = k * CC(X, Z) * a_ezz
        exz = k * SS(X, Z) * a_exz
        eta_x = -aeta * k * SS(X, Z)
        eta_z = aeta * k * CC(X, Z)
        exx_x = -k * k * S(X, Z) * a_exx
        exx_z = -k * k * C(X, Z) * a_exx
        ezz_x = -k * k * S(X, Z) * a_ezz
        ezz_z = -k * k * C(X, Z) * a_ezz
        exz_x = k * k * C(X, Z) * a_exz
        exz_z = k * k * S(X, Z) * a_exz
        dx_txx = eta_x * exx + eta * exx_x
        dz_tzz = eta_z * ezz + eta * ezz_z
        dx_txz = eta_x * exz + eta * exz_x
        dz_txz = eta_z * exz + eta * exz_z
        Px = -aP * k * S(X, Z)
        Pz = -aP * k * C(X, Z)
        res_W = -(dz_tzz + dx_txz) + Pz - (rho - rhoref) * g0
        res_U = -(dx_txx + dz_txz) + Px
        Wv = aW * C(X, Z)
        Uv = aU * S(X, Z)
        rho_z = arho * k * CC(X, Z)
        rho_x = -arho * k * SS(X, Z)
        res_P = rho_z * Wv + rho * (aW * k * CC(X, Z)) + rho_x * Uv + rho * (aU * k * CC(X, Z)) - asrc * C(X, Z)
        return dict(W=Wv, U=Uv, P=aP * CC(X, Z), eta=eta, rho=rho, res_W=res_W, res_U=res_U, res_P=res_P,
                    src=asrc * C(X, Z))

    Zw, Xw = grid(zw, x)
    Zu, Xu = grid(z, xu)
    Zp, Xp = grid(z, x)
    Zc, Xc = grid(zw, xu)
    fw, fu, fp, fc = fields(Xw, Zw), fields(Xu, Zu), fields(Xp, Zp), fields(Xc, Zc)
    rhow = fw["rho"][:, 1:-1]
    out = dict(W_exact=fw["W"], U_exact=fu["U"], P_exact=fp["P"],
               src_W=fw["res_W"], src_U=fu["res_U"], src_P=fp["res_P"],
               eta=fp["eta"][1:-1, 1:-1], etaco=fc["eta"], rho=fp["rho"][1:-1, 1:-1],
               rhow=rhow, rhou=fu["rho"][1:-1, :], MFS=fp["src"][1:-1, 1:-1])
    out["Drho"] = rhow - rhow.mean(axis=1, keepdims=True)
    return out
