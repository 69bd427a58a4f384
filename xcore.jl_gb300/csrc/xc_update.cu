// Constitutive update!, store_previous!, update_phase_velocities!, update_dt,
// compute_resnorm and the FP64 conservation sums on the GPU.
//
// Reference: src/update.jl, src/store.jl, src/diagnose.jl:42-71,
// src/history.jl:121-145.  Each kernel keeps the reference's per-element
// operation order; compiled with -fmad=false.  exp / pow are CUDA's, so
// results agree with the reference arithmetic to a few ulp (the reference's
// own libm differs from any other libm by as much).
#include <cmath>

#include "xc_internal.cuh"

namespace {

__device__ __forceinline__ int icz_at(int j, int Nz, int zBC) {   // icz[j], j = 0..Nz+1
  if (j == 0) return zBC == XC_PERIODIC ? Nz - 1 : 0;
  if (j == Nz + 1) return zBC == XC_PERIODIC ? 0 : Nz - 1;
  return j - 1;
}
__device__ __forceinline__ int icx_at(int i, int Nx, int xBC) {   // icx[i], i = 0..Nx+1
  if (i == 0) return xBC == XC_PERIODIC ? Nx - 1 : 0;
  if (i == Nx + 1) return xBC == XC_PERIODIC ? 0 : Nx - 1;
  return i - 1;
}
__device__ __forceinline__ double clampd(double x, double lo, double hi) {
  return x > hi ? hi : (x < lo ? lo : x);
}

struct Rheo {
  double A11, A12, A21, A22, lB11, lB12, lB21, lB22, iC11, iC12, iC21, iC22, ex, em;   // lB = log(B)
  double lmx, lxm;   // log(em / ex), log(ex / em)
};

// compute_volfrac_kernel! (update.jl:18-35) fused with compute_rheology_kernel!
// (update.jl:144-177), one thread per cell
__global__ void volfrac_rheology_kernel(int Nz, int Nx, double rhom0, double rhox0, Rheo r,
                                        CView x, CView m, DView rho, DView chi, DView mu,
                                        uint8_t* hasx, uint8_t* hasm, DView etamix) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    double xc = AT(x, j, i), mc = AT(m, j, i);
    double rh = 1.0 / (mc / rhom0 + xc / rhox0);
    AT(rho, j, i) = rh;
    double f1 = clampd((xc * rh) / rhox0, XC_EPS, 1.0 - XC_EPS);
    double f2 = clampd((mc * rh) / rhom0, XC_EPS, 1.0 - XC_EPS);
    AT(chi, j, i) = f1;
    AT(mu, j, i) = f2;
    size_t o = (size_t)i * Nz + j;
    hasx[o] = xc >= XC_SQRT_EPS;
    hasm[o] = mc >= XC_SQRT_EPS;
    // The powers of update.jl:153-171 as exp(y log x): pow carries its log in
    // extra precision, which costs about twice the FP64 work; the relative error
    // of exp(y log x) is |y log x| eps, below 2e-14 for these operands (f >= eps,
    // 1/C and the fractions Xf of order one), far inside the 1e-12 bound of
    // these fields.  log(f / B) as log f - log B (log B once on the host) and
    // the two normalisations as one reciprocal each: two logarithms and two
    // divisions per cell instead of four and eight, with an absolute error of
    // the exponent of a few eps |log f|.
    const double lf1 = log(f1), lf2 = log(f2);
    double s11 = exp(r.iC11 * (lf1 - r.lB11)), s12 = exp(r.iC12 * (lf2 - r.lB12));
    double s21 = exp(r.iC21 * (lf1 - r.lB21)), s22 = exp(r.iC22 * (lf2 - r.lB22));
    const double in1 = 1.0 / (s11 + s12), in2 = 1.0 / (s21 + s22);
    double Sf11 = s11 * in1, Sf12 = s12 * in1, Sf21 = s21 * in2, Sf22 = s22 * in2;
    double a1 = r.A11 * Sf11 + r.A12 * Sf12;
    double a2 = r.A21 * Sf21 + r.A22 * Sf22;
    double Xf11 = a1 * f1 + (1.0 - a1) * Sf11;
    double Xf12 = a1 * f2 + (1.0 - a1) * Sf12;
    double Xf21 = a2 * f1 + (1.0 - a2) * Sf21;
    double Xf22 = a2 * f2 + (1.0 - a2) * Sf22;
    // update.jl:170-171 multiply by pow(ex/ex, Xf11) and pow(em/em, Xf22): with
    // positive finite ex, em those are pow(1, y) = 1 exactly, and x * 1 = x, so
    // the two FP64 pow calls are left out without changing a bit
    double thtv1 = exp(Xf12 * r.lmx);
    double thtv2 = exp(Xf21 * r.lxm);
    double etaf1 = r.ex * thtv1, etaf2 = r.em * thtv2;
    AT(etamix, j, i) = f1 * etaf1 + f2 * etaf2;
  });
}

// update_interpolations! (update.jl:73-107) without the row mean; one thread
// per (j, i) of the (Nz+2, Nx+2) bounding box
__global__ void interp_kernel(int Nz, int Nx, int xBC, int zBC, double rhom0, double rhox0,
                              CView rho, CView chi, CView mu, CView x, CView m, DView rhow,
                              DView rhou, DView Drhom, DView Drhox, DView chiw, DView muw,
                              DView chiu, DView muu, DView x_w, DView m_w, DView x_u,
                              DView m_u) {
  XC_PDL_WAIT();
  for_tiles(Nz + 2, Nx + 2, [&](int j, int i) {
    if (j > Nz + 1 || i > Nx + 1) return;
    if (j <= Nz && i < Nx) {   // (Nz+1, Nx)
      int a = icz_at(j, Nz, zBC), b = icz_at(j + 1, Nz, zBC);
      double rw = (AT(rho, a, i) + AT(rho, b, i)) / 2.0;
      AT(rhow, j, i) = rw;
      AT(Drhom, j, i) = rhom0 - rw;
      AT(Drhox, j, i) = rhox0 - rw;
      AT(x_w, j, i) = (AT(x, a, i) + AT(x, b, i)) / 2.0;
      AT(m_w, j, i) = (AT(m, a, i) + AT(m, b, i)) / 2.0;
    }
    if (j < Nz && i <= Nx) {   // (Nz, Nx+1)
      int a = icx_at(i, Nx, xBC), b = icx_at(i + 1, Nx, xBC);
      AT(rhou, j, i) = (AT(rho, j, a) + AT(rho, j, b)) / 2.0;
      AT(x_u, j, i) = (AT(x, j, a) + AT(x, j, b)) / 2.0;
      AT(m_u, j, i) = (AT(m, j, a) + AT(m, j, b)) / 2.0;
    }
    if (j <= Nz) {             // (Nz+1, Nx+2)
      int a = icz_at(j, Nz, zBC), b = icz_at(j + 1, Nz, zBC), ci = icx_at(i, Nx, xBC);
      AT(chiw, j, i) = (AT(chi, a, ci) + AT(chi, b, ci)) / 2.0;
      AT(muw, j, i) = (AT(mu, a, ci) + AT(mu, b, ci)) / 2.0;
    }
    if (i <= Nx) {             // (Nz+2, Nx+1)
      int cj = icz_at(j, Nz, zBC), a = icx_at(i, Nx, xBC), b = icx_at(i + 1, Nx, xBC);
      AT(chiu, j, i) = (AT(chi, cj, a) + AT(chi, cj, b)) / 2.0;
      AT(muu, j, i) = (AT(mu, cj, a) + AT(mu, cj, b)) / 2.0;
    }
  });
}

// mean(rhow, dims=2) (sequential over columns, as Julia reduces a
// non-leading dimension) and, below, the lithostatic z-scan of
// update_pressure! (update.jl:119-131); rhoref and Pl_col go to scratch.
// One thread per row j sums the row in column order; the columns are loaded
// 16 at a time ahead of the additions, so the order (and the bits) of the sum
// stay sequential while many loads are in flight.
// mean(rhow, dims = 2) in Julia's order: for each row, the columns added one
// after another from the left.  A block of 256 threads takes 32 rows: all its
// threads load 32 x kRowTile tiles (coalesced, many loads in flight) into
// shared memory, then one warp -- a thread per row -- adds them in column
// order.  Same additions as a thread walking its row alone.
constexpr int kRowTile = 128;
__global__ void __launch_bounds__(256) rowmean_kernel(int Nz, int Nx, CView rhow, double* rhoref) {
  XC_PDL_WAIT();
  __shared__ double tile[kRowTile][33];
  const int j0 = blockIdx.x * 32;
  const int r = threadIdx.x & 31, cw = threadIdx.x >> 5;   // row in the block, column phase
  const int j = j0 + r;
  double acc = 0.0;
  for (int i0 = 0; i0 < Nx; i0 += kRowTile) {
    for (int c = cw; c < kRowTile; c += 8) {
      const int i = i0 + c;
      tile[c][r] = (j <= Nz && i < Nx) ? AT(rhow, j, i) : 0.0;
    }
    __syncthreads();
    if (cw == 0) {
      const int n = Nx - i0 < kRowTile ? Nx - i0 : kRowTile;
      for (int c = 0; c < n; ++c) acc = acc + tile[c][r];
    }
    __syncthreads();
  }
  if (cw == 0 && j <= Nz) rhoref[j] = acc / (double)Nx;
}

// the column of Pl (update.jl:123-131): the terms (rhoref[j] g0) h of all
// rows formed by the block into shared memory, then added in row order by one
// thread (the reference's loop), in chunks of kScanChunk rows
constexpr int kScanChunk = 4096;
__global__ void __launch_bounds__(256) pressure_scan_kernel(int Nz, double g0, double h, double Ptop,
                                                            const double* rhoref, double* plcol) {
  XC_PDL_WAIT();
  __shared__ double q[kScanChunk];
  double p = 0.0;
  for (int j0 = 0; j0 < Nz; j0 += kScanChunk) {
    const int n = Nz - j0 < kScanChunk ? Nz - j0 : kScanChunk;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const int j = j0 + k;
      q[k] = j == 0 ? ((rhoref[0] * g0) * h) / 2.0 + Ptop : (rhoref[j] * g0) * h;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < n; ++k) {
        p = (j0 + k == 0) ? q[0] : p + q[k];
        q[k] = p;
      }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) plcol[j0 + k] = q[k];
    __syncthreads();
  }
}

// Drho = rhow - rhoref (update.jl:86-87); Pl, Pt (update.jl:132-134)
__global__ void drho_pressure_kernel(int Nz, int Nx, double Ptop, const double* rhoref,
                                     const double* plcol, CView rhow, DView Drho, CView P,
                                     DView Pl, DView Pt) {
  XC_PDL_WAIT();
  for_tiles(Nz + 1, Nx, [&](int j, int i) {
    if (j > Nz || i >= Nx) return;
    AT(Drho, j, i) = AT(rhow, j, i) - rhoref[j];
    if (j < Nz) {
      double pl = plcol[j];
      AT(Pl, j, i) = pl;
      AT(Pt, j, i) = jmax(Ptop / 100.0, pl + AT(P, j + 1, i + 1));
    }
  });
}

__device__ __forceinline__ double exz_at(CView W, CView U, int j, int i, double invh) {
  double dUdz = (AT(U, j + 1, i) - AT(U, j, i)) * invh;
  double dWdx = (AT(W, j, i + 1) - AT(W, j, i)) * invh;
  return (dUdz + dWdx) / 2.0;
}

// update_kinematics! (update.jl:202-280): exz on corners, the rest on cells
__global__ void kinematics_kernel(int Nz, int Nx, double invh, CView W, CView U, CView wx,
                                  CView wm, DView exz, DView exx, DView ezz, DView Div_V,
                                  DView eII, DView V, DView vx, DView vm) {
  XC_PDL_WAIT();
  for_tiles(Nz + 1, Nx + 1, [&](int j, int i) {
    if (j > Nz || i > Nx) return;
    AT(exz, j, i) = exz_at(W, U, j, i, invh);
    if (j >= Nz || i >= Nx) return;
    double Ux_c = (AT(U, j + 1, i + 1) - AT(U, j + 1, i)) * invh;
    double Wz_c = (AT(W, j + 1, i + 1) - AT(W, j, i + 1)) * invh;
    double div = Ux_c + Wz_c;
    AT(Div_V, j, i) = div;
    double ex = Ux_c - div / 3.0, ez = Wz_c - div / 3.0;
    AT(exx, j, i) = ex;
    AT(ezz, j, i) = ez;
    double e1 = exz_at(W, U, j, i, invh), e2 = exz_at(W, U, j + 1, i, invh);
    double e3 = exz_at(W, U, j, i + 1, invh), e4 = exz_at(W, U, j + 1, i + 1, invh);
    double exz_sq = (((e1 * e1 + e2 * e2) + e3 * e3) + e4 * e4) / 4.0;
    AT(eII, j, i) = sqrt((XC_EPS + (ex * ex + ez * ez) / 2.0) + exz_sq);
    double wc = (AT(W, j, i + 1) + AT(W, j + 1, i + 1)) / 2.0;
    double uc = (AT(U, j + 1, i) + AT(U, j + 1, i + 1)) / 2.0;
    AT(V, j, i) = sqrt(wc * wc + uc * uc);
    double t = (AT(wx, j, i + 1) + AT(wx, j + 1, i + 1)) / 2.0;
    AT(vx, j, i) = sqrt(t * t + XC_EPS);
    t = (AT(wm, j, i + 1) + AT(wm, j + 1, i + 1)) / 2.0;
    AT(vm, j, i) = sqrt(t * t + XC_EPS);
  });
}

// compute_viscblend_kernel! (update.jl:286-308); etai -> scratch
__global__ void viscblend_kernel(int Nz, int Nx, double L0, CView etamix, CView eII, CView rho,
                                 CView V, DView etai, DView etae, DView ke, DView kx, DView ReL,
                                 DView fReL) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    double r = AT(rho, j, i), em = AT(etamix, j, i);
    double k = (AT(eII, j, i) * L0) * L0;
    double Re = ((AT(V, j, i) * L0) * r) / em;   // (V L0) / (em / r) with one division (1e-12 fields)
    double f = 1.0 - exp(-Re);
    double ee = (f * k) * r;
    AT(etai, j, i) = em + ee;
    AT(etae, j, i) = ee;
    AT(ke, j, i) = k;
    AT(kx, j, i) = k;
    AT(ReL, j, i) = Re;
    AT(fReL, j, i) = f;
  });
}

// contrast cap + Picard blend of eta (update.jl:331-337) fused with
// compute_segvisc_kernel! (update.jl:345-370); etasi -> scratch
__global__ void blend_segvisc_kernel(int Nz, int Nx, const double* min_etai, double etacntr,
                                     double D0, double l0, CView etai, DView eta, CView V,
                                     CView rho, DView ReD, CView vx, CView etamix, CView ke,
                                     CView fReL, DView Rel, DView fRel, DView ks, DView etat,
                                     DView etasi, DView kx, DView Rc) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    // The harmonic cap 1 / (1/emax + 1/etai) as emax etai / (emax + etai) and
    // (v D0) / (en / r) as (v D0) r / en: one FP64 division each instead of
    // three and two (a division costs about ten FP64 instructions on this GPU;
    // these fields carry the 1e-12 tolerance)
    double emax = (*min_etai) * etacntr;
    const double ei = AT(etai, j, i);
    double e = (emax * ei) / (emax + ei);
    double en = 0.5 * e + 0.5 * AT(eta, j, i);
    AT(eta, j, i) = en;
    double r = AT(rho, j, i), v = AT(V, j, i);
    AT(ReD, j, i) = ((v * D0) * r) / en;
    double vxc = AT(vx, j, i), em = AT(etamix, j, i);
    double Re = ((vxc * l0) * r) / em;
    double f = 1.0 - exp(-Re);
    double k = vxc * l0;
    double et = (f * k) * r;
    AT(etasi, j, i) = em + et;
    AT(Rel, j, i) = Re;
    AT(fRel, j, i) = f;
    AT(ks, j, i) = k;
    AT(etat, j, i) = et;
    AT(kx, j, i) = k + AT(fReL, j, i) * AT(ke, j, i);
    AT(Rc, j, i) = v / jmax(vxc, XC_EPS);
  });
}

// cap + blend of etas and Red (update.jl:396-402)
__global__ void etas_blend_kernel(int Nz, int Nx, const double* min_etasi, double etacntr,
                                  double d0, CView etasi, DView etas, CView vx, CView rho,
                                  DView Red) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    // one division each, as in blend_segvisc_kernel
    double emax = (*min_etasi) * etacntr;
    const double ei = AT(etasi, j, i);
    double e = (emax * ei) / (emax + ei);
    double en = 0.5 * e + 0.5 * AT(etas, j, i);
    AT(etas, j, i) = en;
    AT(Red, j, i) = ((AT(vx, j, i) * d0) * AT(rho, j, i)) / en;
  });
}

// compute_corner_eta! (update.jl:411-426, always periodic x / closed z as
// update_viscosity! calls it, update.jl:341) and etasw (update.jl:405-407)
__global__ void corner_eta_etasw_kernel(int Nz, int Nx, int zBC, CView eta, DView etaco,
                                        CView etas, DView etasw) {
  XC_PDL_WAIT();
  for_tiles(Nz + 1, Nx + 1, [&](int j, int i) {
    if (j > Nz || i > Nx) return;
    int a = icz_at(j, Nz, XC_CLOSED), b = icz_at(j + 1, Nz, XC_CLOSED);
    int c = icx_at(i, Nx, XC_PERIODIC), d = icx_at(i + 1, Nx, XC_PERIODIC);
    double e00 = AT(eta, a, c), e10 = AT(eta, b, c), e01 = AT(eta, a, d), e11 = AT(eta, b, d);
    // the fourth root as two correctly rounded square roots: within one ulp,
    // as pow is, at a fraction of pow's FP64 work
    AT(etaco, j, i) = sqrt(sqrt(((e00 * e10) * e01) * e11));
    if (i < Nx) {
      int p = icz_at(j, Nz, zBC), q = icz_at(j + 1, Nz, zBC);
      AT(etasw, j, i) = sqrt(AT(etas, p, i) * AT(etas, q, i));
    }
  });
}

// update_stresses! (update.jl:432-476)
__global__ void stress_kernel(int Nz, int Nx, double D0, CView etaco, CView exz, DView txz,
                              CView eta, CView exx, CView ezz, DView txx, DView tzz, DView tII,
                              CView V, CView kx, DView Ra) {
  XC_PDL_WAIT();
  for_tiles(Nz + 1, Nx + 1, [&](int j, int i) {
    if (j > Nz || i > Nx) return;
    AT(txz, j, i) = AT(etaco, j, i) * AT(exz, j, i);
    if (j >= Nz || i >= Nx) return;
    double e = AT(eta, j, i);
    double tx = e * AT(exx, j, i), tz = e * AT(ezz, j, i);
    AT(txx, j, i) = tx;
    AT(tzz, j, i) = tz;
    double t1 = AT(etaco, j, i) * AT(exz, j, i), t2 = AT(etaco, j + 1, i) * AT(exz, j + 1, i);
    double t3 = AT(etaco, j, i + 1) * AT(exz, j, i + 1);
    double t4 = AT(etaco, j + 1, i + 1) * AT(exz, j + 1, i + 1);
    double txz_sq = (((t1 * t1 + t2 * t2) + t3 * t3) + t4 * t4) / 4.0;
    AT(tII, j, i) = sqrt((XC_EPS + (tx * tx + tz * tz) / 2.0) + txz_sq);
    AT(Ra, j, i) = (AT(V, j, i) * D0) / AT(kx, j, i);
  });
}

// update_segregation_speed! + update_phase_velocities! (store.jl:47-105),
// one thread per (j, i) of the (Nz+2, Nx+2) bounding box
__global__ void phase_velocities_kernel(int Nz, int Nx, int xBC, int zBC, double d0, double g0,
                                        CView etasw, CView Drhox, CView bndtaperw, CView x_w,
                                        CView m_w, CView x_u, CView m_u, CView W, CView U,
                                        CView xisw, CView xixw, CView xiew, CView xisu,
                                        CView xixu, CView xieu, DView wx, DView wm, DView Wx,
                                        DView Wm, DView Ux, DView Um) {
  XC_PDL_WAIT();
  for_tiles(Nz + 2, Nx + 2, [&](int j, int i) {
    if (j > Nz + 1 || i > Nx + 1) return;
    if (j <= Nz) {   // W-shaped (Nz+1, Nx+2)
      // the ghost columns copy the tapered interior columns periodically
      // (store.jl:272-273 applies the copy for every xBC)
      int is = (i == 0) ? Nx : (i == Nx + 1 ? 1 : i);
      double w = (((d0 * d0) / AT(etasw, j, is - 1)) * AT(Drhox, j, is - 1)) * g0;
      w = w * AT(bndtaperw, j, is);
      AT(wx, j, i) = w;
      int ci = icx_at(i, Nx, xBC);
      double xe = AT(x_w, j, ci), me = jmax(AT(m_w, j, ci), XC_EPS);
      double wmv = ((-xe) / me) * w;
      AT(wm, j, i) = wmv;
      double sx = AT(xisw, j, i) + AT(xixw, j, i);
      double Wv = AT(W, j, i), xe_w = AT(xiew, j, i);
      AT(Wx, j, i) = ((Wv + w) + sx) + xe_w;
      AT(Wm, j, i) = ((Wv + wmv) - ((xe / me) * sx)) + xe_w;
    }
    if (i <= Nx) {   // U-shaped (Nz+2, Nx+1)
      int cj = icz_at(j, Nz, zBC);
      double xe = AT(x_u, cj, i), me = jmax(AT(m_u, cj, i), XC_EPS);
      double sx = AT(xisu, j, i) + AT(xixu, j, i);
      double Uv = AT(U, j, i), xe_u = AT(xieu, j, i);
      AT(Ux, j, i) = (Uv + sx) + xe_u;
      AT(Um, j, i) = (Uv + (((-xe) / me) * sx)) + xe_u;
    }
  });
}

// store_previous! (store.jl:13-30)
__global__ void store_previous_kernel(int Nz, int Nx, DView X, DView Xo, DView Xoo, DView M,
                                      DView Mo, DView Moo, DView dXdt, DView dXdto, DView dXdtoo,
                                      DView rho, DView rhoo, DView rhooo, DView drhodt,
                                      DView drhodto, DView drhodtoo, CView rhow, CView W,
                                      DView rhoWo, DView rhoWoo, CView rhou, CView U,
                                      DView rhoUo, DView rhoUoo) {
  XC_PDL_WAIT();
  for_tiles(Nz + 1, Nx + 1, [&](int j, int i) {
    if (j > Nz || i > Nx) return;
    if (j < Nz && i < Nx) {
      AT(Xoo, j, i) = AT(Xo, j, i); AT(Xo, j, i) = AT(X, j, i);
      AT(Moo, j, i) = AT(Mo, j, i); AT(Mo, j, i) = AT(M, j, i);
      AT(dXdtoo, j, i) = AT(dXdto, j, i); AT(dXdto, j, i) = AT(dXdt, j, i);
      AT(rhooo, j, i) = AT(rhoo, j, i); AT(rhoo, j, i) = AT(rho, j, i);
      AT(drhodtoo, j, i) = AT(drhodto, j, i); AT(drhodto, j, i) = AT(drhodt, j, i);
    }
    if (i < Nx) {    // (Nz+1, Nx)
      AT(rhoWoo, j, i) = AT(rhoWo, j, i);
      AT(rhoWo, j, i) = AT(rhow, j, i) * AT(W, j, i + 1);
    }
    if (j < Nz) {    // (Nz, Nx+1)
      AT(rhoUoo, j, i) = AT(rhoUo, j, i);
      AT(rhoUo, j, i) = AT(rhou, j, i) * AT(U, j + 1, i);
    }
  });
}

}  // namespace

// ---------------------------------------------------------------------------

int update_impl(xc_ctx* c) {
  const int Nz = c->Nz, Nx = c->Nx;
  const xc_params& p = c->p;
  cudaStream_t s = c->stream;
  dim3 blk(32, 8);
  Rheo r{p.AA[0], p.AA[1], p.AA[2], p.AA[3], std::log(p.BB[0]), std::log(p.BB[1]), std::log(p.BB[2]),
         std::log(p.BB[3]),
         1.0 / p.CC[0], 1.0 / p.CC[1], 1.0 / p.CC[2], 1.0 / p.CC[3], p.etax0, p.etam0,
         std::log(p.etam0 / p.etax0), std::log(p.etax0 / p.etam0)};
  xc_launch(volfrac_rheology_kernel, dim3(persistent_grid((const void*)volfrac_rheology_kernel, Nz, Nx)), blk, 0, s,
      Nz, Nx, p.rhom0, p.rhox0, r, CF(c, FLD_x),
      CF(c, FLD_m), F(c, FLD_rho), F(c, FLD_chi),
      F(c, FLD_mu), (uint8_t*)c->field[FLD_hasx], (uint8_t*)c->field[FLD_hasm], F(c, FLD_etamix));
  XC_LAUNCH_CHECK();
  xc_launch(interp_kernel, dim3(persistent_grid((const void*)interp_kernel, Nz + 2, Nx + 2)), blk, 0, s, Nz, Nx,
      p.xBC, p.zBC, p.rhom0, p.rhox0,
      CF(c, FLD_rho), CF(c, FLD_chi), CF(c, FLD_mu),
      CF(c, FLD_x), CF(c, FLD_m), F(c, FLD_rhow), F(c, FLD_rhou), F(c, FLD_Drhom),
      F(c, FLD_Drhox), F(c, FLD_chiw), F(c, FLD_muw), F(c, FLD_chiu), F(c, FLD_muu),
      F(c, FLD_x_w), F(c, FLD_m_w), F(c, FLD_x_u), F(c, FLD_m_u));
  XC_LAUNCH_CHECK();
  // update_pressure! (update.jl:111-138): the row means of rhow and the z
  // prefix sum are chains of dependent FP64 additions in the reference's
  // order (latency-bound, a few warps); nothing else of update! reads their
  // results (Drho, Pl, Pt), so they run on the side stream beside the
  // kinematics-to-stress kernels and are joined at the end
  double* rhoref = c->tmp[6];
  double* plcol = c->tmp[6] + (Nz + 8);
  cudaStream_t side = c->side;
  XC_CUDA_TRY(cudaEventRecord(c->ev_fork, s));
  XC_CUDA_TRY(cudaStreamWaitEvent(side, c->ev_fork, 0));
  xc_launch(rowmean_kernel, (Nz + 1 + 31) / 32, 256, 0, side, Nz, Nx, CF(c, FLD_rhow), rhoref);
  xc_launch(pressure_scan_kernel, 1, 256, 0, side, Nz, p.g0, p.h, p.Ptop, rhoref, plcol);
  XC_LAUNCH_CHECK();
  xc_launch(drho_pressure_kernel, dim3(persistent_grid((const void*)drho_pressure_kernel, Nz + 1, Nx)), blk, 0,
      side, Nz, Nx, p.Ptop, rhoref, plcol,
      CF(c, FLD_rhow), F(c, FLD_Drho), CF(c, FLD_P), F(c, FLD_Pl),
      F(c, FLD_Pt));
  XC_LAUNCH_CHECK();
  XC_CUDA_TRY(cudaEventRecord(c->ev_join, side));
  const double invh = 1.0 / p.h;
  xc_launch(kinematics_kernel, dim3(persistent_grid((const void*)kinematics_kernel, Nz + 1, Nx + 1)), blk, 0, s, Nz,
      Nx, invh, CF(c, FLD_W), CF(c, FLD_U),
      CF(c, FLD_wx), CF(c, FLD_wm), F(c, FLD_exz),
      F(c, FLD_exx), F(c, FLD_ezz), F(c, FLD_Div_V), F(c, FLD_eII), F(c, FLD_V), F(c, FLD_vx),
      F(c, FLD_vm));
  XC_LAUNCH_CHECK();
  DView etai{c->tmp[0], Nz}, etasi{c->tmp[1], Nz};
  xc_launch(viscblend_kernel, dim3(persistent_grid((const void*)viscblend_kernel, Nz, Nx)), blk, 0, s, Nz, Nx, p.L0,
      CF(c, FLD_etamix), CF(c, FLD_eII),
      CF(c, FLD_rho), CF(c, FLD_V), etai,
      F(c, FLD_etae), F(c, FLD_ke), F(c, FLD_kx), F(c, FLD_ReL), F(c, FLD_fReL));
  XC_LAUNCH_CHECK();
  XC_TRY(reduce_view(c, RED_MIN, CView{etai.p, Nz}, CView{nullptr, 0}, Nz, Nx, SC_EMAX_ETA));
  xc_launch(blend_segvisc_kernel, dim3(persistent_grid((const void*)blend_segvisc_kernel, Nz, Nx)), blk, 0, s, Nz, Nx,
      c->dscal + SC_EMAX_ETA, p.etacntr, p.D0, p.l0, CView{etai.p, Nz}, F(c, FLD_eta),
      CF(c, FLD_V), CF(c, FLD_rho), F(c, FLD_ReD), CF(c, FLD_vx), CF(c, FLD_etamix),
      CF(c, FLD_ke), CF(c, FLD_fReL), F(c, FLD_Rel), F(c, FLD_fRel), F(c, FLD_ks),
      F(c, FLD_etat), etasi, F(c, FLD_kx), F(c, FLD_Rc));
  XC_LAUNCH_CHECK();
  XC_TRY(reduce_view(c, RED_MIN, CView{etasi.p, Nz}, CView{nullptr, 0}, Nz, Nx, SC_EMAX_ETAS));
  xc_launch(etas_blend_kernel, dim3(persistent_grid((const void*)etas_blend_kernel, Nz, Nx)), blk, 0, s, Nz, Nx,
      c->dscal + SC_EMAX_ETAS, p.etacntr, p.d0, CView{etasi.p, Nz}, F(c, FLD_etas),
      CF(c, FLD_vx), CF(c, FLD_rho), F(c, FLD_Red));
  XC_LAUNCH_CHECK();
  xc_launch(corner_eta_etasw_kernel, dim3(persistent_grid((const void*)corner_eta_etasw_kernel, Nz + 1, Nx + 1)),
      blk, 0, s, Nz, Nx, p.zBC, CF(c, FLD_eta),
      F(c, FLD_etaco), CF(c, FLD_etas), F(c, FLD_etasw));
  XC_LAUNCH_CHECK();
  xc_launch(stress_kernel, dim3(persistent_grid((const void*)stress_kernel, Nz + 1, Nx + 1)), blk, 0, s, Nz, Nx,
      p.D0, CF(c, FLD_etaco), CF(c, FLD_exz),
      F(c, FLD_txz), CF(c, FLD_eta),
      CF(c, FLD_exx), CF(c, FLD_ezz), F(c, FLD_txx), F(c, FLD_tzz), F(c, FLD_tII), CF(c, FLD_V),
      CF(c, FLD_kx), F(c, FLD_Ra));
  XC_LAUNCH_CHECK();
  XC_CUDA_TRY(cudaStreamWaitEvent(s, c->ev_join, 0));   // update_pressure! on the side stream
  return XC_OK;
}

int phase_velocities_impl(xc_ctx* c) {
  const int Nz = c->Nz, Nx = c->Nx;
  dim3 blk(32, 8);
  xc_launch(phase_velocities_kernel, dim3(persistent_grid((const void*)phase_velocities_kernel, Nz + 2, Nx + 2)),
      blk, 0,
      c->stream, Nz, Nx, c->p.xBC, c->p.zBC, c->p.d0, c->p.g0, CF(c, FLD_etasw), CF(c, FLD_Drhox),
      CF(c, FLD_bndtaperw), CF(c, FLD_x_w), CF(c, FLD_m_w), CF(c, FLD_x_u), CF(c, FLD_m_u),
      CF(c, FLD_W), CF(c, FLD_U), CF(c, FLD_xisw), CF(c, FLD_xixw), CF(c, FLD_xiew),
      CF(c, FLD_xisu), CF(c, FLD_xixu), CF(c, FLD_xieu), F(c, FLD_wx), F(c, FLD_wm),
      F(c, FLD_Wx), F(c, FLD_Wm), F(c, FLD_Ux), F(c, FLD_Um));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int store_previous_impl(xc_ctx* c) {
  const int Nz = c->Nz, Nx = c->Nx;
  dim3 blk(32, 8);
  xc_launch(store_previous_kernel, dim3(persistent_grid((const void*)store_previous_kernel, Nz + 1, Nx + 1)), blk,
      0, c->stream, Nz, Nx, F(c, FLD_X), F(c,
      FLD_Xo), F(c, FLD_Xoo), F(c, FLD_M), F(c, FLD_Mo), F(c, FLD_Moo),
      F(c, FLD_dXdt), F(c, FLD_dXdto), F(c, FLD_dXdtoo), F(c, FLD_rho), F(c, FLD_rhoo),
      F(c, FLD_rhooo), F(c, FLD_drhodt), F(c, FLD_drhodto), F(c, FLD_drhodtoo), CF(c, FLD_rhow),
      CF(c, FLD_W), F(c, FLD_rhoWo), F(c, FLD_rhoWoo), CF(c, FLD_rhou), CF(c, FLD_U),
      F(c, FLD_rhoUo), F(c, FLD_rhoUoo));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

static int copy_field(xc_ctx* c, int dst, int src) {
  size_t n = (size_t)c->shape[src].rows * c->shape[src].cols * c->elem[src];
  XC_CUDA_TRY(cudaMemcpyAsync(c->field[dst], c->field[src], n, cudaMemcpyDeviceToDevice, c->stream));
  return XC_OK;
}

int store_noise_impl(xc_ctx* c) {
  XC_TRY(copy_field(c, FLD_psieo, FLD_psie));
  XC_TRY(copy_field(c, FLD_psixo, FLD_psix));
  return copy_field(c, FLD_psiso, FLD_psis);
}

int snapshot_impl(xc_ctx* c) {
  XC_TRY(copy_field(c, FLD_res_Wo, FLD_W));
  XC_TRY(copy_field(c, FLD_res_Uo, FLD_U));
  XC_TRY(copy_field(c, FLD_res_Po, FLD_P));
  XC_TRY(copy_field(c, FLD_res_Xo, FLD_X));
  return copy_field(c, FLD_res_MFSo, FLD_MFS);
}

static inline CView whole(xc_ctx* c, int id) { return CF(c, id); }
static const CView kNone{nullptr, 0};

int update_dt_reduce(xc_ctx* c, cudaStream_t s) {
  const int Nz = c->Nz, Nx = c->Nx;
  double* d = c->dscal + SC_DT;
  const RedJob jobs[5] = {
      red_job(RED_MAX, whole(c, FLD_kx), kNone, nullptr, Nz, Nx, d + 0),
      red_job(RED_MAXABS, whole(c, FLD_Wx), kNone, nullptr, Nz + 1, Nx + 2, d + 1),
      red_job(RED_MAXABS, whole(c, FLD_Wm), kNone, nullptr, Nz + 1, Nx + 2, d + 2),
      red_job(RED_MAXABS, whole(c, FLD_Ux), kNone, nullptr, Nz + 2, Nx + 1, d + 3),
      red_job(RED_MAXABS, whole(c, FLD_Um), kNone, nullptr, Nz + 2, Nx + 1, d + 4)};
  return reduce_batch(c, jobs, 5, s ? s : c->stream);
}

int update_dt_impl(xc_ctx* c, double dt_prev, double* dt_out) {
  XC_TRY(update_dt_reduce(c));
  XC_TRY(fetch_scalars(c, SC_DT, 5));
  update_dt_finish(c, dt_prev, dt_out);
  return XC_OK;
}

void update_dt_finish(const xc_ctx* c, double dt_prev, double* dt_out) {
  const double* m = c->hscal + SC_DT;
  const double h = c->p.h;
  // Julia's min / max (a NaN speed or diffusivity gives a NaN step)
  double dtk = (h / 2.0) * (h / 2.0) / m[0];
  double vmax = jmax(jmax(jmax(m[1], m[2]), m[3]), m[4]) + XC_EPS;
  double dta = (h / 2.0) / vmax;
  *dt_out = jmin(jmin(1.5 * dt_prev, jmin(dtk, c->p.CFL * dta)), c->p.dtmax);
}

int resnorm_reduce(xc_ctx* c, cudaStream_t s) {
  const int Nz = c->Nz, Nx = c->Nx;
  double* d = c->dscal + SC_RESNORM;
  const RedJob jobs[9] = {
      red_job(RED_SUMSQ, whole(c, FLD_rho), kNone, nullptr, Nz, Nx, d + 0),
      red_job(RED_SUMSQDIFF, whole(c, FLD_X), whole(c, FLD_res_Xo), nullptr, Nz, Nx, d + 1),
      red_job(RED_SUMSQDIFF, whole(c, FLD_MFS), whole(c, FLD_res_MFSo), nullptr, Nz, Nx, d + 2),
      red_job(RED_SUMSQDIFF, whole(c, FLD_W), whole(c, FLD_res_Wo), nullptr, Nz + 1, Nx + 2, d + 3),
      red_job(RED_SUMSQ, whole(c, FLD_W), kNone, nullptr, Nz + 1, Nx + 2, d + 4),
      red_job(RED_SUMSQDIFF, whole(c, FLD_U), whole(c, FLD_res_Uo), nullptr, Nz + 2, Nx + 1, d + 5),
      red_job(RED_SUMSQ, whole(c, FLD_U), kNone, nullptr, Nz + 2, Nx + 1, d + 6),
      red_job(RED_SUMSQDIFF, whole(c, FLD_P), whole(c, FLD_res_Po), nullptr, Nz + 2, Nx + 2, d + 7),
      red_job(RED_SUMSQ, whole(c, FLD_P), kNone, nullptr, Nz + 2, Nx + 2, d + 8)};
  return reduce_batch(c, jobs, 9, s ? s : c->stream);
}

int resnorm_impl(xc_ctx* c, double dt, double out[3]) {
  XC_TRY(resnorm_reduce(c));
  XC_TRY(fetch_scalars(c, SC_RESNORM, 9));
  resnorm_finish(c, dt, out);
  return XC_OK;
}

void resnorm_finish(const xc_ctx* c, double dt, double out[3]) {
  const double* q = c->hscal + SC_RESNORM;
  const double ep = XC_EPS;
  double nrho = std::sqrt(q[0]);
  double res_mass = std::sqrt(q[1]) / (nrho + ep) + std::sqrt(q[2]) / (nrho / dt + ep);
  double res_mmnt = (std::sqrt(q[3]) / (std::sqrt(q[4]) + ep) + std::sqrt(q[5]) / (std::sqrt(q[6]) + ep)) +
                    std::sqrt(q[7]) / (std::sqrt(q[8]) + ep);
  out[0] = res_mass + res_mmnt;
  out[1] = res_mass;
  out[2] = res_mmnt;
}

int sums_impl(xc_ctx* c, double out[12]) {
  const int Nz = c->Nz, Nx = c->Nx;
  const int b = SC_SUMS;
  double* d = c->dscal + b;
  RedJob jobs[12];
  const int whole_f[4] = {FLD_rho, FLD_M, FLD_X, FLD_Gx};
  for (int k = 0; k < 4; ++k) jobs[k] = red_job(RED_SUM, whole(c, whole_f[k]), kNone, nullptr, Nz, Nx, d + k);
  const int fl[4] = {FLD_qz_advn_X, FLD_qz_advn_M, FLD_qz_dffn_X, FLD_qz_dffn_M};
  for (int k = 0; k < 4; ++k) {
    CView q = CF(c, fl[k]);
    CView top{q.p + q.ld, q.ld};                 // row 0, columns 1..Nx
    CView bot{q.p + q.ld + Nz, q.ld};            // row Nz, columns 1..Nx
    jobs[4 + 2 * k] = red_job(RED_SUM, top, kNone, nullptr, 1, Nx, d + 4 + 2 * k);
    jobs[5 + 2 * k] = red_job(RED_SUM, bot, kNone, nullptr, 1, Nx, d + 5 + 2 * k);
  }
  XC_TRY(reduce_batch(c, jobs, 12, c->stream));
  XC_TRY(fetch_scalars(c, b, 12));
  const double* q = c->hscal + b;
  const double h = c->p.h, h2 = h * h;
  out[0] = q[0] * h2 + XC_EPS;
  out[1] = q[1] * h2 + XC_EPS;
  out[2] = q[2] * h2 + XC_EPS;
  out[3] = q[3] * h2;
  for (int k = 4; k < 12; ++k) out[k] = q[k] * h;
  return XC_OK;
}

// Per-step statistics of record_history! (src/history.jl:183-222):
// x: min, mean, max, std; V, vx, vm, xie, xix, xis: min, rms, max;
// Ra, Rc, ReD, Red, ks, ke, kx, eta, etamix, etae, etas, etat: min, geomean, max
// (_rms = sqrt(mean(x^2)), _geomean = exp(mean(log(max(x, eps))))).
int history_impl(xc_ctx* c, double out[58]) {
  const int Nz = c->Nz, Nx = c->Nx;
  const double n = (double)Nz * (double)Nx;
  cudaStream_t s = c->stream;
  double* d = c->tmp[7];    // 64 device scalars
  const CView none{nullptr, 0};
  RedJob jobs[58];
  int k = 0;
  CView x = CF(c, FLD_x);
  jobs[k] = red_job(RED_MIN, x, none, nullptr, Nz, Nx, d + k); ++k;
  jobs[k] = red_job(RED_SUM, x, none, nullptr, Nz, Nx, d + k, n); ++k;
  jobs[k] = red_job(RED_MAX, x, none, nullptr, Nz, Nx, d + k); ++k;
  ++k;   // d[3]: sum (x - mean)^2, after the mean (second batch)
  const int rms_f[6] = {FLD_V, FLD_vx, FLD_vm, FLD_xie, FLD_xix, FLD_xis};
  for (int q = 0; q < 6; ++q) {
    CView f = CF(c, rms_f[q]);
    jobs[k] = red_job(RED_MIN, f, none, nullptr, Nz, Nx, d + k); ++k;
    jobs[k] = red_job(RED_SUMSQ, f, none, nullptr, Nz, Nx, d + k, n); ++k;
    jobs[k] = red_job(RED_MAX, f, none, nullptr, Nz, Nx, d + k); ++k;
  }
  const int gm_f[12] = {FLD_Ra, FLD_Rc, FLD_ReD, FLD_Red, FLD_ks, FLD_ke, FLD_kx, FLD_eta, FLD_etamix,
                        FLD_etae, FLD_etas, FLD_etat};
  for (int q = 0; q < 12; ++q) {
    CView f = CF(c, gm_f[q]);
    jobs[k] = red_job(RED_MIN, f, none, nullptr, Nz, Nx, d + k); ++k;
    jobs[k] = red_job(RED_SUMLOG, f, none, nullptr, Nz, Nx, d + k, n); ++k;
    jobs[k] = red_job(RED_MAX, f, none, nullptr, Nz, Nx, d + k); ++k;
  }
  // first batch: everything but the std; the mean of x lands in d[1]
  RedJob first[57];
  int nf = 0;
  for (int q = 0; q < 58; ++q)
    if (q != 3) first[nf++] = jobs[q];
  XC_TRY(reduce_batch(c, first, nf, s));
  const RedJob dev = red_job(RED_SUM, x, none, d + 1, Nz, Nx, d + 3);
  XC_TRY(reduce_batch(c, &dev, 1, s));
  XC_CUDA_TRY(cudaMemcpyAsync(out, d, sizeof(double) * 58, cudaMemcpyDeviceToHost, s));
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  out[3] = std::sqrt(out[3] / (n - 1.0));
  for (int q = 0; q < 6; ++q) out[4 + 3 * q + 1] = std::sqrt(out[4 + 3 * q + 1]);
  for (int q = 0; q < 12; ++q) out[22 + 3 * q + 1] = std::exp(out[22 + 3 * q + 1]);
  return XC_OK;
}

// The statistics print_step! prints beyond record_history!'s
// (src/diagnose.jl:92-182), each on the raw field (the reference divides by a
// scale before printing; min, max and geomean commute with that division):
// m: min, mean, max; rho: min, geomean, max; V, vx, vm, xie, xix, xis: min,
// geomean, max -- with _gm(A) = exp(sum(log(max(A, 1e-300))) / length(A))
// (diagnose.jl:10).
int print_stats_impl(xc_ctx* c, double out[24]) {
  const int Nz = c->Nz, Nx = c->Nx;
  const double n = (double)Nz * (double)Nx;
  cudaStream_t s = c->stream;
  double* d = c->tmp[7];
  const CView none{nullptr, 0};
  RedJob jobs[24];
  int k = 0;
  CView m = CF(c, FLD_m);
  jobs[k] = red_job(RED_MIN, m, none, nullptr, Nz, Nx, d + k); ++k;
  jobs[k] = red_job(RED_SUM, m, none, nullptr, Nz, Nx, d + k, n); ++k;
  jobs[k] = red_job(RED_MAX, m, none, nullptr, Nz, Nx, d + k); ++k;
  const int gm_f[7] = {FLD_rho, FLD_V, FLD_vx, FLD_vm, FLD_xie, FLD_xix, FLD_xis};
  for (int q = 0; q < 7; ++q) {
    CView f = CF(c, gm_f[q]);
    jobs[k] = red_job(RED_MIN, f, none, nullptr, Nz, Nx, d + k); ++k;
    jobs[k] = red_job(RED_SUMLOG, f, none, nullptr, Nz, Nx, d + k, n);
    jobs[k].floor = 1e-300;
    ++k;
    jobs[k] = red_job(RED_MAX, f, none, nullptr, Nz, Nx, d + k); ++k;
  }
  XC_TRY(reduce_batch(c, jobs, k, s));
  XC_CUDA_TRY(cudaMemcpyAsync(out, d, sizeof(double) * 24, cudaMemcpyDeviceToHost, s));
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  for (int q = 0; q < 7; ++q) out[3 + 3 * q + 1] = std::exp(out[3 + 3 * q + 1]);
  return XC_OK;
}
