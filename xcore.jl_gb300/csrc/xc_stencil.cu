// Advection and diffusion stencils, halo fill and phsevo! on the GPU.
//
// Reference: src/kernels/advect.jl, src/kernels/diffus.jl, src/kernels/ghosts.jl,
// src/phsevo.jl.  The reference evaluates every face value twice (once for each
// neighbouring cell, advect.jl:57-96) and then a third time in the per-face
// flux kernels (advect.jl:603-637).  Those three evaluations are bitwise
// identical (advect.jl:428-432), so here each CTA computes every face flux of
// its tile ONCE into shared memory and takes the cell divergence from there,
// in the reference's operation order: adv = (qxr - qxl + qzb - qzt) * invh.
// Compiled with -fmad=false so no multiply-add is contracted (Julia does not
// contract either); with identical inputs the results are bitwise equal to
// the reference arithmetic.
#include "xc_internal.cuh"

namespace {

constexpr int TZ = 32;        // tile rows (z, contiguous in memory)
constexpr int TX = 16;        // tile columns (x)
constexpr int NT = 256;       // threads per CTA

// ---------------------------------------------------------------------------
// face reconstructions (advect.jl:35-53, 216-229, 275-283)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double weno5_poly(double fmm, double fm, double fc, double fp,
                                             double fpp) {
  const double sixth = 1.0 / 6.0, quarter = 0.25, c1312 = 13.0 / 12.0;
  const double eps_val = XC_EPS;
  double p1 = sixth * ((2.0 * fmm - 7.0 * fm) + 11.0 * fc);
  double p2 = sixth * ((-fm + 5.0 * fc) + 2.0 * fp);
  double p3 = sixth * ((2.0 * fc + 5.0 * fp) - fpp);
  double t = (fmm - 2.0 * fm) + fc, s = (fmm - 4.0 * fm) + 3.0 * fc;
  double b1 = c1312 * (t * t) + quarter * (s * s);
  t = (fm - 2.0 * fc) + fp;
  s = fm - fp;
  double b2 = c1312 * (t * t) + quarter * (s * s);
  t = (fc - 2.0 * fp) + fpp;
  s = (3.0 * fc - 4.0 * fp) + fpp;
  double b3 = c1312 * (t * t) + quarter * (s * s);
  double e1 = b1 + eps_val, e2 = b2 + eps_val, e3 = b3 + eps_val;
  double w1 = 0.1 / (e1 * e1);
  double w2 = 0.6 / (e2 * e2);
  double w3 = 0.3 / (e3 * e3);
  return ((w1 * p1 + w2 * p2) + w3 * p3) / ((w1 + w2) + w3);
}

// The same reconstruction with the weights over a common denominator: with
// q_k = (eps + b_k)^2 the weights d_k / q_k are proportional to
// n_1 = d_1 q_2 q_3, n_2 = d_2 q_1 q_3, n_3 = d_3 q_1 q_2, so the weighted
// mean needs one division instead of four (an FP64 division costs about ten
// times a multiply on this GPU).  Each q_k lies in [eps^2, (eps + b_k)^2]:
// the products stay normal and finite for fields below about 1e70.  The
// polynomials and smoothness indicators use fused multiply-adds (about 60
// FP64 instructions per reconstruction instead of 78; within a few ulps).
__device__ __forceinline__ double weno5_poly_onediv(double fmm, double fm, double fc, double fp,
                                                    double fpp) {
  const double sixth = 1.0 / 6.0, quarter = 0.25, c1312 = 13.0 / 12.0;
  const double eps_val = XC_EPS;
  const double p1 = sixth * __fma_rn(11.0, fc, __fma_rn(-7.0, fm, 2.0 * fmm));
  const double p2 = sixth * __fma_rn(2.0, fp, __fma_rn(5.0, fc, -fm));
  const double p3 = sixth * (__fma_rn(2.0, fc, 5.0 * fp) - fpp);
  double t = __fma_rn(-2.0, fm, fmm) + fc, s = __fma_rn(3.0, fc, __fma_rn(-4.0, fm, fmm));
  const double b1 = __fma_rn(c1312 * t, t, quarter * (s * s));
  t = __fma_rn(-2.0, fc, fm) + fp;
  s = fm - fp;
  const double b2 = __fma_rn(c1312 * t, t, quarter * (s * s));
  t = __fma_rn(-2.0, fp, fc) + fpp;
  s = __fma_rn(3.0, fc, -4.0 * fp) + fpp;
  const double b3 = __fma_rn(c1312 * t, t, quarter * (s * s));
  const double e1 = b1 + eps_val, e2 = b2 + eps_val, e3 = b3 + eps_val;
  const double q1 = e1 * e1, q2 = e2 * e2, q3 = e3 * e3;
  const double n1 = 0.1 * (q2 * q3), n2 = 0.6 * (q1 * q3), n3 = 0.3 * (q1 * q2);
  return __fma_rn(n1, p1, __fma_rn(n2, p2, n3 * p3)) / ((n1 + n2) + n3);
}

__device__ __forceinline__ double weno3_poly(double fm, double fc, double fp) {
  const double half = 0.5, eps_val = 1e-6;
  double p1 = half * (fc + fp);
  double p2 = half * (3.0 * fc - fm);
  double d1 = fp - fc, d2 = fc - fm;
  double w1 = (1.0 / 3.0) / (d1 * d1 + eps_val);
  double w2 = (2.0 / 3.0) / (d2 * d2 + eps_val);
  return (w1 * p1 + w2 * p2) / (w1 + w2);
}

__device__ __forceinline__ double tvd_flux(double fm, double fc, double fp, double vm, double vp) {
  double num = vm * (fc - fm);
  double den = vp * (fp - fc);
  double R = num / (den + copysign(XC_EPS, den));
  double l = jmax(0.0, jmax(jmin(1.0, 2.0 * R), jmin(2.0, R)));
  return fc + (0.5 * l) * (fp - fc);
}

__device__ __forceinline__ double vpos(double v) { return (v + fabs(v)) * 0.5; }
__device__ __forceinline__ double vneg(double v) { return (v - fabs(v)) * 0.5; }

// Flux through the face between cells s2 and s3 of the six-cell window
// s0..s5, with face velocity v (and the neighbouring faces' vl, vr for TVD).
// Per-face formulas of advect.jl:444-695.
template <int S>
__device__ __forceinline__ double face_flux(double s0, double s1, double s2, double s3, double s4,
                                            double s5, double v, double vl, double vr) {
  if (S == XC_CENTR) {
    return v * (s2 + s3) * 0.5;
  } else if (S == XC_UPWD1) {
    return vpos(v) * s2 + vneg(v) * s3;
  } else if (S == XC_QUICK) {
    const double sixth = 1.0 / 6.0;
    double pos = sixth * ((2.0 * s3 + 5.0 * s2) - s1);
    double neg = sixth * ((2.0 * s2 + 5.0 * s3) - s4);
    return vpos(v) * pos + vneg(v) * neg;
  } else if (S == XC_FROMM) {
    double pos = s2 + 0.25 * (s3 - s1);
    double neg = s3 + 0.25 * (s2 - s4);
    return vpos(v) * pos + vneg(v) * neg;
  } else if (S == XC_WENO3 || S == XC_WENO5 || S == kWeno5OneDiv) {
    // vpos(v) pos + vneg(v) neg has one weight exactly zero: only the upwind
    // reconstruction is evaluated.  The dropped term is (+0) x (finite) = +-0,
    // which changes no value (at most the sign of a zero result); v = +-0
    // gives 0 and a NaN v stays NaN, as in the full formula.
    // The mirrored stencil is selected first, so a warp with faces of both
    // signs still evaluates one polynomial per face.
    const bool up = v > 0.0;
    const double a0 = up ? s0 : s5, a1 = up ? s1 : s4, a2 = up ? s2 : s3, a3 = up ? s3 : s2,
                 a4 = up ? s4 : s1;
    const double p = S == XC_WENO5        ? weno5_poly(a0, a1, a2, a3, a4)
                     : S == kWeno5OneDiv ? weno5_poly_onediv(a0, a1, a2, a3, a4)
                                         : weno3_poly(a1, a2, a3);
    if (up) return vpos(v) * p;
    if (v < 0.0) return vneg(v) * p;
    return v * 0.0;
  } else {  // XC_TVDIM
    double cpos = vpos(v), cneg = vneg(v);
    double pos = tvd_flux(s1, s2, s3, vpos(vl), cpos);
    double neg = tvd_flux(s4, s3, s2, vneg(vr), cneg);
    return cpos * pos + cneg * neg;
  }
}

template <int S> struct Halo {
  static constexpr int G = (S == XC_WENO5 || S == kWeno5OneDiv) ? 3 : (S == XC_CENTR || S == XC_UPWD1) ? 1 : 2;
};

__device__ __forceinline__ int map_bc(int k, int n, int bc) {
  if (bc == XC_PERIODIC) {
    k %= n;
    return k < 0 ? k + n : k;
  }
  return k < 0 ? 0 : (k >= n ? n - 1 : k);
}

// velocity at face index k (0..n) of an axis with n cells, extended by one
// face on each side for TVD exactly as the reference pads u/w (phsevo.jl:34-53)
__device__ __forceinline__ int map_face(int k, int n, int bc) {
  if (k >= 0 && k <= n) return k;
  if (bc == XC_PERIODIC) return k < 0 ? k + n : k - n;
  return k < 0 ? 0 : n;
}

// ---------------------------------------------------------------------------
// advection tile kernel
// f: interior (Nz, Nx) field read through the BC map, or (HALOD) the caller's
// halo'd (Nz+2G, Nx+2G) array.  u (Nz, Nx+1) x-face velocities, w (Nz+1, Nx)
// z-face velocities (for HALOD tvdim: the padded (Nz, Nx+3) / (Nz+3, Nx)).
// Outputs (any may be null): adv (Nz, Nx), qx_int (Nz, Nx+1), qz_int (Nz+1, Nx).
// ---------------------------------------------------------------------------
template <int S, bool HALOD>
__global__ void __launch_bounds__(NT) advect_tile_kernel(
    const double* __restrict__ f, int ldf, int Nz, int Nx, int xBC, int zBC,
    CView u, CView w, double invh, DView adv, DView qx, DView qz) {
  XC_PDL_WAIT();
  constexpr int G = Halo<S>::G;
  constexpr int HZ = TZ + 2 * G, HX = TX + 2 * G;
  __shared__ double sf[HX][HZ];
  __shared__ double sqx[TX + 1][TZ];
  __shared__ double sqz[TX][TZ + 1];
  const int j0 = blockIdx.x * TZ, i0 = blockIdx.y * TX;
  const int tid = threadIdx.x;

  for (int idx = tid; idx < HZ * HX; idx += NT) {
    int jj = idx % HZ, ii = idx / HZ;
    int j = j0 - G + jj, i = i0 - G + ii;
    double v = 0.0;
    if (HALOD) {
      int hj = j + G, hi = i + G;
      if (hj < Nz + 2 * G && hi < Nx + 2 * G) v = f[(size_t)hi * ldf + hj];
    } else {
      v = f[(size_t)map_bc(i, Nx, xBC) * ldf + map_bc(j, Nz, zBC)];
    }
    sf[ii][jj] = v;
  }
  __syncthreads();

  // x-faces: rows j0..j0+TZ-1, faces i0..i0+TX
  for (int idx = tid; idx < TZ * (TX + 1); idx += NT) {
    int jj = idx % TZ, ii = idx / TZ;
    int j = j0 + jj, i = i0 + ii;
    double q = 0.0;
    if (j < Nz && i <= Nx) {
      double uv = AT(u, j, HALOD && S == XC_TVDIM ? i + 1 : i);
      double ul = 0.0, ur = 0.0;
      if (S == XC_TVDIM) {
        if (HALOD) {
          ul = AT(u, j, i);
          ur = AT(u, j, i + 2);
        } else {
          ul = AT(u, j, map_face(i - 1, Nx, xBC));
          ur = AT(u, j, map_face(i + 1, Nx, xBC));
        }
      }
      // face i sits between cells i-1 and i -> tile columns ii+G-1 and ii+G
      const int c = ii + G, r = jj + G;
      double s0 = (G >= 3) ? sf[c - 3][r] : 0.0;
      double s1 = (G >= 2) ? sf[c - 2][r] : 0.0;
      double s4 = (G >= 2) ? sf[c + 1][r] : 0.0;
      double s5 = (G >= 3) ? sf[c + 2][r] : 0.0;
      q = face_flux<S>(s0, s1, sf[c - 1][r], sf[c][r], s4, s5, uv, ul, ur);
      if (qx.p && (ii < TX || i == Nx)) AT(qx, j, i) = q;
    }
    sqx[ii][jj] = q;
  }
  // z-faces: faces j0..j0+TZ, columns i0..i0+TX-1
  for (int idx = tid; idx < (TZ + 1) * TX; idx += NT) {
    int jj = idx % (TZ + 1), ii = idx / (TZ + 1);
    int j = j0 + jj, i = i0 + ii;
    double q = 0.0;
    if (j <= Nz && i < Nx) {
      double wv = AT(w, HALOD && S == XC_TVDIM ? j + 1 : j, i);
      double wt = 0.0, wb = 0.0;
      if (S == XC_TVDIM) {
        if (HALOD) {
          wt = AT(w, j, i);
          wb = AT(w, j + 2, i);
        } else {
          wt = AT(w, map_face(j - 1, Nz, zBC), i);
          wb = AT(w, map_face(j + 1, Nz, zBC), i);
        }
      }
      const int c = ii + G, r = jj + G;
      double s0 = (G >= 3) ? sf[c][r - 3] : 0.0;
      double s1 = (G >= 2) ? sf[c][r - 2] : 0.0;
      double s4 = (G >= 2) ? sf[c][r + 1] : 0.0;
      double s5 = (G >= 3) ? sf[c][r + 2] : 0.0;
      q = face_flux<S>(s0, s1, sf[c][r - 1], sf[c][r], s4, s5, wv, wt, wb);
      if (qz.p && (jj < TZ || j == Nz)) AT(qz, j, i) = q;
    }
    sqz[ii][jj] = q;
  }
  if (!adv.p) return;
  __syncthreads();
  for (int idx = tid; idx < TZ * TX; idx += NT) {
    int jj = idx % TZ, ii = idx / TZ;
    int j = j0 + jj, i = i0 + ii;
    if (j < Nz && i < Nx)
      AT(adv, j, i) = (((sqx[ii + 1][jj] - sqx[ii][jj]) + sqz[ii][jj + 1]) - sqz[ii][jj]) * invh;
  }
}

// ---------------------------------------------------------------------------
// diffusion tile kernel (diffus.jl:9-31, 68-91); k = k1 (* k2 when given)
// ---------------------------------------------------------------------------
template <bool HALOD>
__global__ void __launch_bounds__(NT) diffus_tile_kernel(
    const double* __restrict__ f, const double* __restrict__ k1, const double* __restrict__ k2,
    int ld, int Nz, int Nx, int xBC, int zBC, double invh, DView dff, DView qx, DView qz) {
  XC_PDL_WAIT();
  constexpr int G = 1;
  constexpr int HZ = TZ + 2 * G, HX = TX + 2 * G;
  __shared__ double sf[HX][HZ];
  __shared__ double sk[HX][HZ];
  const int j0 = blockIdx.x * TZ, i0 = blockIdx.y * TX;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < HZ * HX; idx += NT) {
    int jj = idx % HZ, ii = idx / HZ;
    int j = j0 - G + jj, i = i0 - G + ii;
    double fv = 0.0, kv = 0.0;
    if (HALOD) {
      int hj = j + G, hi = i + G;
      if (hj < Nz + 2 && hi < Nx + 2) {
        size_t o = (size_t)hi * ld + hj;
        fv = f[o];
        kv = k1[o];
        if (k2) kv = kv * k2[o];
      }
    } else {
      size_t o = (size_t)map_bc(i, Nx, xBC) * ld + map_bc(j, Nz, zBC);
      fv = f[o];
      kv = k1[o];
      if (k2) kv = kv * k2[o];
    }
    sf[ii][jj] = fv;
    sk[ii][jj] = kv;
  }
  __syncthreads();
  const double half = 0.5;
  const double invh2 = invh * invh;
  if (dff.p) {
    for (int idx = tid; idx < TZ * TX; idx += NT) {
      int jj = idx % TZ, ii = idx / TZ;
      int j = j0 + jj, i = i0 + ii;
      if (j < Nz && i < Nx) {
        int c = ii + 1, r = jj + 1;
        double fc = sf[c][r], kc = sk[c][r];
        double fxr = (sk[c + 1][r] + kc) * (sf[c + 1][r] - fc);
        double fxl = (kc + sk[c - 1][r]) * (fc - sf[c - 1][r]);
        double fzb = (sk[c][r + 1] + kc) * (sf[c][r + 1] - fc);
        double fzt = (kc + sk[c][r - 1]) * (fc - sf[c][r - 1]);
        AT(dff, j, i) = (half * invh2) * (((fxr - fxl) + fzb) - fzt);
      }
    }
  }
  if (qx.p) {
    for (int idx = tid; idx < TZ * (TX + 1); idx += NT) {
      int jj = idx % TZ, ii = idx / TZ;
      int j = j0 + jj, i = i0 + ii;
      if (j < Nz && i <= Nx && (ii < TX || i == Nx)) {
        int c = ii + 1, r = jj + 1;
        double fL = sf[c - 1][r], fR = sf[c][r], kL = sk[c - 1][r], kR = sk[c][r];
        AT(qx, j, i) = (((-(kL + kR)) * half) * (fR - fL)) * invh;
      }
    }
  }
  if (qz.p) {
    for (int idx = tid; idx < (TZ + 1) * TX; idx += NT) {
      int jj = idx % (TZ + 1), ii = idx / (TZ + 1);
      int j = j0 + jj, i = i0 + ii;
      if (j <= Nz && i < Nx && (jj < TZ || j == Nz)) {
        int c = ii + 1, r = jj + 1;
        double fT = sf[c][r - 1], fB = sf[c][r], kT = sk[c][r - 1], kB = sk[c][r];
        AT(qz, j, i) = (((-(kT + kB)) * half) * (fB - fT)) * invh;
      }
    }
  }
}

// MATLAB-sized boundary rows/cols of the face-flux arrays (advect.jl:779-795,
// diffus.jl:194-208): qz cols 0 / Nx+1 and qx rows 0 / Nz+1.
__global__ void pad_fluxes_kernel(DView qx, DView qz, int Nz, int Nx, int xBC, int zBC) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Nz + 1) {   // qz (Nz+1, Nx+2)
    if (xBC == XC_PERIODIC && Nx > 1) {
      AT(qz, t, 0) = AT(qz, t, Nx);
      AT(qz, t, Nx + 1) = AT(qz, t, 1);
    } else {
      AT(qz, t, 0) = AT(qz, t, 1);
      AT(qz, t, Nx + 1) = AT(qz, t, Nx);
    }
  }
  if (t < Nx + 1) {   // qx (Nz+2, Nx+1)
    if (zBC == XC_PERIODIC && Nz > 1) {
      AT(qx, 0, t) = AT(qx, Nz, t);
      AT(qx, Nz + 1, t) = AT(qx, 1, t);
    } else {
      AT(qx, 0, t) = AT(qx, 1, t);
      AT(qx, Nz + 1, t) = AT(qx, Nz, t);
    }
  }
}

// ghost ring of a halo'd array (ghosts.jl:18-51; for N >= halo the x-then-z
// fill equals reading the BC-mapped interior cell, corners included)
__global__ void fill_ghosts_kernel(double* f, int Nz, int Nx, int g, int zBC, int xBC) {
  XC_PDL_WAIT();
  const int rows = Nz + 2 * g, cols = Nx + 2 * g;
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)rows * cols) return;
  int hj = (int)(t % rows), hi = (int)(t / rows);
  int j = hj - g, i = hi - g;
  if (j >= 0 && j < Nz && i >= 0 && i < Nx) return;
  int sj = map_bc(j, Nz, zBC) + g, si = map_bc(i, Nx, xBC) + g;
  f[(size_t)hi * rows + hj] = f[(size_t)si * rows + sj];
}

// phsevo! tail (phsevo.jl:189, 197-211), one thread per cell
__global__ void phsevo_tail_kernel(int Nz, int Nx, double a1, double a2, double a3, double b1,
                                   double b2, double b3, double dt, double alpha, double G0,
                                   DView X, CView Xo, CView Xoo, DView M, DView x, DView m,
                                   CView rho, CView advn_X, CView advn_M, DView advn_rho,
                                   CView dffn_X, CView bndshape, DView Gx, DView dXdt,
                                   CView dXdto, CView dXdtoo) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    double aX = AT(advn_X, j, i);
    AT(advn_rho, j, i) = aX + AT(advn_M, j, i);
    double gx = (G0 * (1.0 - AT(x, j, i))) * AT(bndshape, j, i);
    AT(Gx, j, i) = gx;
    double dxdt = (-aX + AT(dffn_X, j, i)) + gx;
    AT(dXdt, j, i) = dxdt;
    double Xc = AT(X, j, i);
    double res = ((a1 * Xc - a2 * AT(Xo, j, i)) - a3 * AT(Xoo, j, i)) -
                 (((b1 * dxdt + b2 * AT(dXdto, j, i)) + b3 * AT(dXdtoo, j, i)) * dt);
    double upd = ((-alpha) * res) / a1;
    double Xn = Xc + upd;
    double r = AT(rho, j, i);
    double lo = r * XC_EPS, hi = r * (1.0 - XC_EPS);
    Xn = Xn > hi ? hi : (Xn < lo ? lo : Xn);
    AT(X, j, i) = Xn;
    double Mn = r - Xn;
    AT(M, j, i) = Mn;
    AT(x, j, i) = Xn / r;
    AT(m, j, i) = Mn / r;
  });
}

template <int S>
int launch_advect(const double* f, int ldf, bool halod, int Nz, int Nx, int xBC, int zBC, CView u,
                  CView w, double invh, DView adv, DView qx, DView qz, cudaStream_t s) {
  // the last tile of each axis also writes the closing face (index Nz / Nx)
  dim3 grid((Nz + TZ - 1) / TZ, (Nx + TX - 1) / TX);
  if (halod) {
    xc_launch(advect_tile_kernel<S, true>, grid, NT, 0, s, f, ldf, Nz, Nx, xBC, zBC, u, w, invh, adv, qx, qz);
  } else {
    xc_launch(advect_tile_kernel<S, false>, grid, NT, 0, s, f, ldf, Nz, Nx, xBC, zBC, u, w, invh, adv, qx, qz);
  }
  XC_LAUNCH_CHECK();
  return XC_OK;
}

}  // namespace

int scheme_halo(int scheme) {
  switch (scheme) {
    case XC_CENTR: case XC_UPWD1: return 1;
    case XC_QUICK: case XC_FROMM: case XC_WENO3: case XC_TVDIM: return 2;
    case XC_WENO5: case kWeno5OneDiv: return 3;
    default: return -1;
  }
}

int stencil_advect_flux(const double* f, int ldf, bool halod, int Nz, int Nx, int scheme, int xBC,
                        int zBC, CView u, CView w, double h, DView adv, DView qx_int,
                        DView qz_int, cudaStream_t s) {
  int g = scheme_halo(scheme);
  if (g < 0) { xc_set_error("advect: unsupported scheme %d", scheme); return XC_BAD_ARG; }
  if (Nz < g || Nx < g) {
    xc_set_error("advect: grid %dx%d smaller than the scheme halo %d", Nz, Nx, g);
    return XC_BAD_ARG;
  }
  double invh = 1.0 / h;
  switch (scheme) {
    case XC_CENTR: return launch_advect<XC_CENTR>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case XC_UPWD1: return launch_advect<XC_UPWD1>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case XC_QUICK: return launch_advect<XC_QUICK>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case XC_FROMM: return launch_advect<XC_FROMM>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case XC_WENO3: return launch_advect<XC_WENO3>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case XC_WENO5: return launch_advect<XC_WENO5>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    case kWeno5OneDiv:
      return launch_advect<kWeno5OneDiv>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
    default: return launch_advect<XC_TVDIM>(f, ldf, halod, Nz, Nx, xBC, zBC, u, w, invh, adv, qx_int, qz_int, s);
  }
}

static int diffus_launch(const double* f, const double* k1, const double* k2, int ld, bool halod,
                         int Nz, int Nx, int xBC, int zBC, double h, DView dff, DView qx, DView qz,
                         cudaStream_t s) {
  dim3 grid((Nz + TZ - 1) / TZ, (Nx + TX - 1) / TX);
  double invh = 1.0 / h;
  if (halod) {
    xc_launch(diffus_tile_kernel<true>, grid, NT, 0, s, f, k1, k2, ld, Nz, Nx, xBC, zBC, invh, dff, qx, qz);
  } else {
    xc_launch(diffus_tile_kernel<false>, grid, NT, 0, s, f, k1, k2, ld, Nz, Nx, xBC, zBC, invh, dff, qx, qz);
  }
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int stencil_diffus_flux(const double* f, const double* k, int ld, bool halod, int Nz, int Nx,
                        int xBC, int zBC, double h, DView dff, DView qx_int, DView qz_int,
                        cudaStream_t s) {
  return diffus_launch(f, k, nullptr, ld, halod, Nz, Nx, xBC, zBC, h, dff, qx_int, qz_int, s);
}

int pad_face_fluxes(DView qx, DView qz, int Nz, int Nx, int xBC, int zBC, cudaStream_t s) {
  int n = (Nz > Nx ? Nz : Nx) + 1;
  xc_launch(pad_fluxes_kernel, (n + 255) / 256, 256, 0, s, qx, qz, Nz, Nx, xBC, zBC);
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// phsevo! (src/phsevo.jl:164-214)
int phsevo_impl(xc_ctx* c, int scheme, const double coefs[6], double dt, double alpha) {
  const int Nz = c->Nz, Nx = c->Nx, xBC = c->p.xBC, zBC = c->p.zBC;
  const double h = c->p.h;
  cudaStream_t s = c->stream;
  // face-velocity views: Wx[:, 2:end-1] (Nz+1, Nx), Ux[2:end-1, :] (Nz, Nx+1)
  DView Wx = F(c, FLD_Wx), Wm = F(c, FLD_Wm), Ux = F(c, FLD_Ux), Um = F(c, FLD_Um);
  CView Wx_face{Wx.p + Wx.ld, Wx.ld}, Wm_face{Wm.p + Wm.ld, Wm.ld};
  CView Ux_face{Ux.p + 1, Ux.ld}, Um_face{Um.p + 1, Um.ld};
  auto qx_int = [&](int id) { DView q = F(c, id); return DView{q.p + 1, q.ld}; };
  auto qz_int = [&](int id) { DView q = F(c, id); return DView{q.p + q.ld, q.ld}; };
  DView X = F(c, FLD_X), M = F(c, FLD_M);
  scheme = advect_scheme(scheme, c->p);
  XC_TRY(stencil_advect_flux(X.p, X.ld, false, Nz, Nx, scheme, xBC, zBC, Ux_face, Wx_face, h,
                             F(c, FLD_advn_X), qx_int(FLD_qx_advn_X), qz_int(FLD_qz_advn_X), s));
  XC_TRY(stencil_advect_flux(M.p, M.ld, false, Nz, Nx, scheme, xBC, zBC, Um_face, Wm_face, h,
                             F(c, FLD_advn_M), qx_int(FLD_qx_advn_M), qz_int(FLD_qz_advn_M), s));
  // diffusion of chi with k = X .* kx (phsevo.jl:192-194)
  XC_TRY(diffus_launch(F(c, FLD_chi).p, X.p, F(c, FLD_kx).p, Nz, false, Nz, Nx, xBC, zBC, h,
                       F(c, FLD_dffn_X), qx_int(FLD_qx_dffn_X), qz_int(FLD_qz_dffn_X), s));
  XC_TRY(pad_face_fluxes(F(c, FLD_qx_advn_X), F(c, FLD_qz_advn_X), Nz, Nx, xBC, zBC, s));
  XC_TRY(pad_face_fluxes(F(c, FLD_qx_advn_M), F(c, FLD_qz_advn_M), Nz, Nx, xBC, zBC, s));
  XC_TRY(pad_face_fluxes(F(c, FLD_qx_dffn_X), F(c, FLD_qz_dffn_X), Nz, Nx, xBC, zBC, s));
  dim3 blk(32, 8);
  xc_launch(phsevo_tail_kernel, dim3(persistent_grid((const void*)phsevo_tail_kernel, Nz, Nx)), blk, 0, s, Nz, Nx,
      coefs[0], coefs[1], coefs[2], coefs[3],
      coefs[4], coefs[5], dt, alpha, c->p.G0,
      X, CF(c, FLD_Xo), CF(c, FLD_Xoo), M, F(c, FLD_x), F(c, FLD_m), CF(c, FLD_rho),
      CF(c, FLD_advn_X), CF(c, FLD_advn_M), F(c, FLD_advn_rho), CF(c, FLD_dffn_X),
      CF(c, FLD_bndshape), F(c, FLD_Gx), F(c, FLD_dXdt), CF(c, FLD_dXdto), CF(c, FLD_dXdtoo));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// ---------------------------------------------------------------------------
// C ABI: stencil-level entry points on caller device pointers
// ---------------------------------------------------------------------------
static bool bc_ok(int b) { return b == XC_PERIODIC || b == XC_CLOSED; }

extern "C" int xc_fill_ghosts(double* f, int Nz, int Nx, int halo, int zBC, int xBC, void* stream) {
  if (!f || Nz < halo || Nx < halo || halo < 1 || !bc_ok(zBC) || !bc_ok(xBC)) {
    xc_set_error("xc_fill_ghosts: bad arguments (Nz=%d Nx=%d halo=%d)", Nz, Nx, halo);
    return XC_BAD_ARG;
  }
  long long n = (long long)(Nz + 2 * halo) * (Nx + 2 * halo);
  xc_launch(fill_ghosts_kernel, (unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream, f, Nz, Nx, halo, zBC, xBC);
  XC_LAUNCH_CHECK();
  return XC_OK;
}

extern "C" int xc_advect(double* adv, const double* f_halo, const double* u, const double* w,
                         int Nz, int Nx, double h, int scheme, void* stream) {
  int g = scheme <= XC_TVDIM ? scheme_halo(scheme) : -1;   // the public scheme codes
  if (!adv || !f_halo || !u || !w || g < 0 || Nz < g || Nx < g) {
    xc_set_error("xc_advect: bad arguments (scheme=%d Nz=%d Nx=%d)", scheme, Nz, Nx);
    return XC_BAD_ARG;
  }
  CView uv{u, Nz}, wv{w, scheme == XC_TVDIM ? Nz + 3 : Nz + 1};
  return stencil_advect_flux(f_halo, Nz + 2 * g, true, Nz, Nx, scheme, XC_PERIODIC, XC_CLOSED, uv,
                             wv, h, DView{adv, Nz}, DView{nullptr, 0}, DView{nullptr, 0},
                             (cudaStream_t)stream);
}

extern "C" int xc_advect_with_flux(double* adv, double* qx, double* qz, const double* f_halo,
                                   const double* u, const double* w, int Nz, int Nx, double h,
                                   int scheme, int xBC, int zBC, void* stream) {
  int g = scheme <= XC_TVDIM ? scheme_halo(scheme) : -1;   // the public scheme codes
  if (!adv || !qx || !qz || !f_halo || !u || !w || g < 0 || Nz < g || Nx < g || !bc_ok(xBC) ||
      !bc_ok(zBC)) {
    xc_set_error("xc_advect_with_flux: bad arguments (scheme=%d Nz=%d Nx=%d)", scheme, Nz, Nx);
    return XC_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CView uv{u, Nz}, wv{w, scheme == XC_TVDIM ? Nz + 3 : Nz + 1};
  DView qxv{qx, Nz + 2}, qzv{qz, Nz + 1};
  XC_TRY(stencil_advect_flux(f_halo, Nz + 2 * g, true, Nz, Nx, scheme, xBC, zBC, uv, wv, h,
                             DView{adv, Nz}, DView{qx + 1, Nz + 2}, DView{qz + (Nz + 1), Nz + 1}, s));
  return pad_face_fluxes(qxv, qzv, Nz, Nx, xBC, zBC, s);
}

extern "C" int xc_advect_centered_with_flux(double* adv, double* qx, double* qz, const double* f,
                                            const double* u, const double* w, int Nz, int Nx,
                                            double h, int scheme, int xBC, int zBC, void* stream) {
  int g = scheme <= XC_TVDIM ? scheme_halo(scheme) : -1;   // the public scheme codes
  if (!adv || !f || !u || !w || g < 0 || Nz < g || Nx < g || !bc_ok(xBC) || !bc_ok(zBC) ||
      ((qx == nullptr) != (qz == nullptr))) {
    xc_set_error("xc_advect_centered_with_flux: bad arguments (scheme=%d Nz=%d Nx=%d)", scheme, Nz, Nx);
    return XC_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CView uv{u, Nz}, wv{w, Nz + 1};
  DView qxi{qx ? qx + 1 : nullptr, Nz + 2}, qzi{qz ? qz + (Nz + 1) : nullptr, Nz + 1};
  XC_TRY(stencil_advect_flux(f, Nz, false, Nz, Nx, scheme, xBC, zBC, uv, wv, h, DView{adv, Nz},
                             qxi, qzi, s));
  if (qx) return pad_face_fluxes(DView{qx, Nz + 2}, DView{qz, Nz + 1}, Nz, Nx, xBC, zBC, s);
  return XC_OK;
}

extern "C" int xc_diffus(double* dff, const double* f_halo, const double* k_halo, int Nz, int Nx,
                         double h, void* stream) {
  if (!dff || !f_halo || !k_halo || Nz < 1 || Nx < 1) {
    xc_set_error("xc_diffus: bad arguments");
    return XC_BAD_ARG;
  }
  return diffus_launch(f_halo, k_halo, nullptr, Nz + 2, true, Nz, Nx, XC_PERIODIC, XC_CLOSED, h,
                       DView{dff, Nz}, DView{nullptr, 0}, DView{nullptr, 0}, (cudaStream_t)stream);
}

extern "C" int xc_diffus_with_flux(double* dff, double* qx, double* qz, const double* f_halo,
                                   const double* k_halo, int Nz, int Nx, double h, int xBC,
                                   int zBC, void* stream) {
  if (!dff || !qx || !qz || !f_halo || !k_halo || Nz < 1 || Nx < 1 || !bc_ok(xBC) || !bc_ok(zBC)) {
    xc_set_error("xc_diffus_with_flux: bad arguments");
    return XC_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  XC_TRY(diffus_launch(f_halo, k_halo, nullptr, Nz + 2, true, Nz, Nx, xBC, zBC, h, DView{dff, Nz},
                       DView{qx + 1, Nz + 2}, DView{qz + (Nz + 1), Nz + 1}, s));
  return pad_face_fluxes(DView{qx, Nz + 2}, DView{qz, Nz + 1}, Nz, Nx, xBC, zBC, s);
}
