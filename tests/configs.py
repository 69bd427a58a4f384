"""The workloads of the parity and bench configurations, built the same way by
the fixture generator (tests/golden/make_configs.py), the GPU tests and the
CPU oracle.

The reference has no temperature field and its viscosity is the
permission-weight mixture capped by etacntr (src/update.jl:144-177, 330-335),
so each configuration maps onto the reference's own inputs:

* box100: 100 x 100 box (D = L = 10), x0 = 0.05, Da = 0, dxr = 0, L0 = l0 = 3h,
  etacntr 1e2, WENO5, BD2; the initial crystal fraction is
  x = 0.05 (1 + 1e-3 G2 * xi), xi ~ N(0, 1) from seed 0 and G2 a Gaussian
  smoothing over 2 cells (periodic in x, mirrored in z), in place of the
  reference's MersenneTwister perturbation (src/run.jl:98-108);
* box400: 400 x 400, x ~ U[0.02, 0.10] (seed 1), etacntr 1e3, WENO5 or QUICK;
* lognormal: N x N, x ~ lognormal (median 0.1, sigma 0.5) clipped to [0, 0.4],
  etacntr 1e4, WENO5.

White-noise draws come from numpy's default_rng(seed + 1000) as two
standard-normal (N, N) arrays per step (the reference draws them with
randn!(ns.rng, ...), noise.jl:154-157, which cannot be reproduced without
Julia); the same arrays feed the oracle and the GPU.
"""
import numpy as np

import xcore_oracle as O

# fields whose digest is compared per step
DIGEST_FIELDS = ("X", "M", "x", "W", "U", "P", "eta", "MFS", "psie", "xie", "Wx", "Ux", "kx", "rho")
N_SAMPLES = 64


def params(cfg, N=None, scheme="weno5"):
    N = N or {"box100": 100, "box400": 400, "lognormal": 256}[cfg]
    D = 10.0
    h = D / N
    etacntr = {"box100": 1e2, "box400": 1e3, "lognormal": 1e4}[cfg]
    x0 = {"box100": 0.05, "box400": 0.06, "lognormal": 0.1}[cfg]
    return O.Params(D=D, N=N, L=D, etam0=10.0, x0=x0, Da=0.0, dxr=0.0, L0=3 * h, l0=3 * h, etacntr=etacntr,
                    ADVN=scheme, TINT="bd2im")


def smooth2(a):
    """Gaussian smoothing over 2 cells: separable kernel exp(-k^2 / (2 * 2^2)),
    |k| <= 6, normalised; periodic along x (axis 1), mirrored along z (axis 0)."""
    k = np.arange(-6, 7, dtype=np.float64)
    w = np.exp(-(k * k) / 8.0)
    w /= w.sum()
    Nz, Nx = a.shape
    out = np.zeros_like(a)
    for t, wt in zip(k.astype(int), w):
        out += wt * np.roll(a, t, axis=1)
    a2 = out
    out = np.zeros_like(a)
    zi = np.arange(Nz)
    for t, wt in zip(k.astype(int), w):
        j = zi + t
        j = np.where(j < 0, -j - 1, j)
        j = np.where(j >= Nz, 2 * Nz - 1 - j, j)
        out += wt * a2[j, :]
    return out


def initial_x(cfg, N):
    if cfg == "box100":
        xi = np.random.default_rng(0).standard_normal((N, N))
        return 0.05 * (1.0 + 1e-3 * smooth2(xi))
    if cfg == "box400":
        return np.random.default_rng(1).uniform(0.02, 0.10, (N, N))
    rng = np.random.default_rng(2)
    return np.clip(np.exp(np.log(0.1) + 0.5 * rng.standard_normal((N, N))), 0.0, 0.4)


class Draws:
    """Per-step white-noise draws (re, rs) of a configuration."""

    def __init__(self, cfg, N):
        self.rng = np.random.default_rng({"box100": 1000, "box400": 1001, "lognormal": 1002}[cfg])
        self.N = N

    def next(self):
        return self.rng.standard_normal((self.N, self.N)), self.rng.standard_normal((self.N, self.N))


def setup(cfg, N=None, scheme="weno5"):
    """(par, grid, scales, noise statics, initial x, draws, initial draw)."""
    par = params(cfg, N, scheme)
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    x0 = initial_x(cfg, g.Nz)
    draws = Draws(cfg, g.Nz)
    return par, g, sc, ns, x0, draws, draws.next()


def sample_index(shape, n=N_SAMPLES):
    """Fixed sample positions (flat, column-major) of a field of this shape."""
    size = shape[0] * shape[1]
    return np.random.default_rng(12345 + size).choice(size, size=min(n, size), replace=False)


def digest(a):
    """[L2 norm, sum, sum of |a|, min, max, values at the fixed sample positions]."""
    a = np.asarray(a, dtype=np.float64)
    flat = a.ravel(order="F")
    return np.concatenate(([np.linalg.norm(flat), flat.sum(), np.abs(flat).sum(), flat.min(), flat.max()],
                           flat[sample_index(a.shape)]))


def digest_error(got, ref):
    """Largest relative deviation between two digests: the norm and the sum of
    |a| against themselves, the sum against the sum of |a|, and the extremes
    and samples against the field's largest magnitude."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    tiny = 1e-300
    amax = max(abs(ref[3]), abs(ref[4]), tiny)
    errs = [abs(got[0] - ref[0]) / max(ref[0], tiny),
            abs(got[1] - ref[1]) / max(ref[2], tiny),
            abs(got[2] - ref[2]) / max(ref[2], tiny),
            float(np.max(np.abs(got[3:] - ref[3:]))) / amax]
    return float(max(errs))
