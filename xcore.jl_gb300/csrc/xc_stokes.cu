// fluidmech! on the GPU: the staggered-grid Stokes saddle-point system of
// src/fluidmech.jl:71-534, solved matrix-free.
//
// The reference assembles LL = [KV GG; DM KP] from triplets, scales it with
// scl = 1/(sqrt|diag LL| + [0; sqrt(eta/rho)]) and factorises SCL*LL*SCL with
// UMFPACK; one call is mathematically SOL <- LL^{-1} RR.  Here the same LL
// (every row of fluidmech.jl:145-488, incl. the periodic W ghost columns, the
// top/bottom U rows, the P ghost ring and the pressure pin) is applied as a
// stencil, the right-hand side RR (fluidmech.jl:111-127, 236-246, 310-323,
// 446-459, with the WENO5/QUICK momentum advection of the current W, U) is
// assembled on the device, and the scaled system is solved by FGMRES with a
// block upper-triangular preconditioner
//     [A  B]^-1            z_p = S~^-1 r_p,   z_v = A~^-1 (r_v - B z_p)
//     [0  S]
// where A~^-1 is one V-cycle of a geometric multigrid for the velocity block
// (re-discretised coarse operators from averaged eta / etaco / rho, damped
// Jacobi smoothing, bilinear transfers) and S~^-1 one V-cycle of a
// cell-centred multigrid for S = -DM diag(A)^-1 GG, a variable-coefficient
// pressure Laplacian with the pin (plus an optional eta/rho mass term).
// Mixed precision: the same Krylov/multigrid machinery in FP32 inside FP64
// iterative refinement on the FP64 residual.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <cstring>
#include <type_traits>
#include <utility>
#include <vector>

#include "xc_internal.cuh"
#include "xc_nn.cuh"

namespace {

// Every kernel of this unit begins with XC_PDL_WAIT() (xc_internal.cuh), so the
// solver's graph-captured launches may be issued with programmatic
// serialization.

// programmatic launches on (the default) or off for the solves of this thread
thread_local bool g_xc_pdl = true;
#define PDL_ON g_xc_pdl

template <typename... KArgs, typename... Args>
void pdl_smem(bool on, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = on ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
  xc_count_launch();
}
template <typename... KArgs, typename... Args>
void pdl(bool on, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args&&... args) {
  pdl_smem(on, kernel, grid, block, 0, s, std::forward<Args>(args)...);
}

constexpr int kMaxLevels = 12;
constexpr int kMaxRestart = 64;

struct Geo {          // one grid level
  int Nz, Nx, NW, NU, NP;
  double h, invh;
  float invhf, ih2f;  // FP32 1/h and 1/h^2, rounded once here: FP32 kernels do no FP64 arithmetic
};

Geo make_geo(int Nz, int Nx, double h) {
  Geo g;
  g.Nz = Nz; g.Nx = Nx; g.h = h; g.invh = 1.0 / h;
  g.invhf = (float)g.invh;
  g.ih2f = (float)(g.invh * g.invh);
  g.NW = (Nz + 1) * (Nx + 2);
  g.NU = (Nz + 2) * (Nx + 1);
  g.NP = (Nz + 2) * (Nx + 2);
  return g;
}

// row-local scalars of the operator
struct OpConst {
  double a1, gamma, dt, g0;
  double idt;          // 1 / dt (the coefficient kernels multiply instead of dividing per row)
  int sds, top_cnv, bot_cnv;
  int sailor;          // 0 in MMS mode (fluidmech.jl:218, 293)
  int pin_p;           // flat P index (0..NP-1) of the pressure pin
  int mms;             // 1: MMS pins (P row and U row are identity rows)
  int pin_u;           // flat U index of the MMS velocity pin
  int open_cnv;        // 1: open bottom (fluidmech.jl:169-190, 426-429, 478-487)
};

// ---------------------------------------------------------------------------
// coefficient planes of the velocity block (physical, unscaled), one level.
// W row planes: 0 diag, 1 W(j-1,i), 2 W(j+1,i), 3 W(j,i-1), 4 W(j,i+1),
//               5 U(j,i-1), 6 U(j+1,i-1), 7 U(j,i), 8 U(j+1,i)
// U row planes: 0 diag, 1 U(j,il), 2 U(j,ir), 3 U(j-1,i), 4 U(j+1,i),
//               5 W(j-1,i), 6 W(j-1,i+1), 7 W(j,i), 8 W(j,i+1)
// Plane 9 holds the inertial part a1*rho/dt of the diagonal alone (without the
// drunken-sailor term, which can make it negative at large dt).
// (fluidmech.jl:194-233, 270-307)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void vel_coef_kernel(Geo g, OpConst k, const double* __restrict__ eta,
                                const double* __restrict__ etaco, const double* __restrict__ rho,
                                const double* __restrict__ rhow, const double* __restrict__ rhou,
                                T* cw, T* cu) {
  XC_PDL_WAIT();
  const int Nz = g.Nz, Nx = g.Nx;
  const double invh = g.invh, invh2 = invh * invh;
  // 32-bit row indices (a level's unknowns are checked below 2^31 at setup):
  // a 64-bit integer division per row cost more than the coefficients
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double c23 = 2.0 / 3.0, c13 = 1.0 / 3.0;
  if (t < g.NW) {
    int j = t % (Nz + 1), i = t / (Nz + 1);
    double c[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (i == 0 || i == Nx + 1 || j == 0) {
      c[0] = 1.0;
    } else if (j == Nz) {
      // bottom row: closed (W = MFSmean D / h) or open, a continuity row
      // rho1 W(Nz) - rho2 W(Nz-1) + rho3 U(Nz, i) - rho4 U(Nz, i-1) (fluidmech.jl:169-190)
      c[0] = rhow[(size_t)(i - 1) * (Nz + 1) + Nz] * invh;
      if (k.open_cnv) {
        c[1] = -rhow[(size_t)(i - 1) * (Nz + 1) + Nz - 1] * invh;
        c[7] = +rhou[(size_t)i * Nz + Nz - 1] * invh;
        c[5] = -rhou[(size_t)(i - 1) * Nz + Nz - 1] * invh;
      }
    } else {
      double C1 = etaco[(size_t)(i - 1) * (Nz + 1) + j], C2 = etaco[(size_t)i * (Nz + 1) + j];
      double P1 = eta[(size_t)(i - 1) * Nz + (j - 1)], P2 = eta[(size_t)(i - 1) * Nz + j];
      double iner = k.a1 * rhow[(size_t)(i - 1) * (Nz + 1) + j] * k.idt;
      double d = iner + (c23 * (P1 + P2) * invh2 + 0.5 * (C1 + C2) * invh2);
      double sail = 0.0;
      if (k.sailor) {
        double dz = (rho[(size_t)(i - 1) * Nz + j] - rho[(size_t)(i - 1) * Nz + j - 1]) * invh;
        sail = dz * k.g0 * k.dt;
        d = d + sail;
      }
      c[0] = d;
      c[1] = -c23 * P1 * invh2;
      c[2] = -c23 * P2 * invh2;
      c[3] = -0.5 * C1 * invh2;
      c[4] = -0.5 * C2 * invh2;
      c[5] = -(0.5 * C1 - c13 * P1) * invh2;
      c[6] = +(0.5 * C1 - c13 * P2) * invh2;
      c[7] = +(0.5 * C2 - c13 * P1) * invh2;
      c[8] = -(0.5 * C2 - c13 * P2) * invh2;
      c[9] = iner;
    }
    for (int q = 0; q < 10; ++q) cw[(size_t)q * g.NW + t] = (T)c[q];
    return;
  }
  t -= g.NW;
  if (t < g.NU) {
    int j = (int)(t % (Nz + 2)), i = (int)(t / (Nz + 2));
    double c[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (j == 0 || j == Nz + 1 || (k.mms && (int)t == k.pin_u)) {
      c[0] = 1.0;
    } else {
      int ia = (i == 0) ? Nx - 1 : i - 1;       // icx[i]
      int ib = (i == Nx) ? 0 : i;               // icx[i+1]
      double C1 = etaco[(size_t)i * (Nz + 1) + j - 1], C2 = etaco[(size_t)i * (Nz + 1) + j];
      double P1 = eta[(size_t)ia * Nz + j - 1], P2 = eta[(size_t)ib * Nz + j - 1];
      double iner = (k.a1 + k.gamma) * rhou[(size_t)i * Nz + j - 1] * k.idt;
      double d = iner + (c23 * (P1 + P2) * invh2 + 0.5 * (C1 + C2) * invh2);
      double sail = 0.0;
      if (k.sailor) {
        double dx = (rho[(size_t)ib * Nz + j - 1] - rho[(size_t)ia * Nz + j - 1]) * invh;
        sail = dx * k.g0 * k.dt;
        d = d + sail;
      }
      c[0] = d;
      c[1] = -c23 * P1 * invh2;
      c[2] = -c23 * P2 * invh2;
      c[3] = -0.5 * C1 * invh2;
      c[4] = -0.5 * C2 * invh2;
      c[5] = -(0.5 * C1 - c13 * P1) * invh2;
      c[6] = +(0.5 * C1 - c13 * P2) * invh2;
      c[7] = +(0.5 * C2 - c13 * P1) * invh2;
      c[8] = -(0.5 * C2 - c13 * P2) * invh2;
      c[9] = iner;
    }
    for (int q = 0; q < 10; ++q) cu[(size_t)q * g.NU + t] = (T)c[q];
  }
}

// ---------------------------------------------------------------------------
// Velocity-block coefficients of one level, as the kernels see them.  The
// FP64 hierarchy (whose operator defines the residual the solve converges on)
// reads the ten planes above.  The FP32 hierarchy (preconditioner and inner
// operator) rebuilds the nine stencil weights of a row from FP32 copies of
// eta and etaco plus one precomputed diagonal term per row: 16 bytes per cell
// from HBM instead of 80, the rest is arithmetic the FP32 pipes have to spare.
// ---------------------------------------------------------------------------
template <typename T>
struct VOp {
  const T* cw;      // planes (FP64 hierarchy)
  const T* cu;
  const T* eta;     // FP32 hierarchy: cell viscosity (Nz, Nx)
  const T* etaco;   //   corner viscosity (Nz+1, Nx+1)
  const T* dw;      //   W rows: inertia + drunken-sailor term; bottom row: its diagonal
  const T* du;      //   U rows: inertia + drunken-sailor term
  const T* dbot;    //   open bottom: the W(Nz-1), U(Nz, i-1), U(Nz, i) weights of the bottom W row,
                    //   three per column
};
template <typename T>
constexpr bool kFly = std::is_same<T, float>::value;
// 1/h and 1/h^2 of a level in T (the same values as converting the FP64 ones)
template <typename T>
__host__ __device__ __forceinline__ T geo_invh(const Geo& g) {
  if constexpr (kFly<T>) return g.invhf;
  else return g.invh;
}
template <typename T>
__host__ __device__ __forceinline__ T geo_ih2(const Geo& g) {
  if constexpr (kFly<T>) return g.ih2f;
  else return g.invh * g.invh;
}

// smoother update r / d: the FP32 preconditioner takes the fast approximate
// division (2 ulp; d is a positive diagonal far inside its range), FP64 the
// IEEE one
template <typename T>
__device__ __forceinline__ T sdiv(T r, T d) {
  if constexpr (kFly<T>) return __fdividef(r, d);
  else return r / d;
}
// rounded products and sums the compiler may not contract into FMAs: the
// pressure multigrid forms the same values in its fused and split kernels,
// whose inlined contexts would otherwise contract differently
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b) {
  if constexpr (kFly<T>) return __fmul_rn(a, b);
  else return __dmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b) {
  if constexpr (kFly<T>) return __fadd_rn(a, b);
  else return __dadd_rn(a, b);
}

// dw / du and the FP32 viscosity copies of one level (terms as vel_coef_kernel)
template <typename T>
__global__ void fly_coef_kernel(Geo g, OpConst k, const double* __restrict__ eta,
                                const double* __restrict__ etaco, const double* __restrict__ rho,
                                const double* __restrict__ rhow, const double* __restrict__ rhou,
                                T* feta, T* fetaco, T* dw, T* du, T* dbot) {
  XC_PDL_WAIT();
  const int Nz = g.Nz, Nx = g.Nx;
  const double invh = g.invh;
  int t = blockIdx.x * blockDim.x + threadIdx.x;   // 32-bit row indices, as vel_coef_kernel
  if (t < Nz * Nx) feta[t] = (T)eta[t];
  if (t < (Nz + 1) * (Nx + 1)) fetaco[t] = (T)etaco[t];
  if (t < g.NW) {
    int j = t % (Nz + 1), i = t / (Nz + 1);
    double v = 1.0;
    if (i >= 1 && i <= Nx && j == Nz) {
      v = rhow[(size_t)(i - 1) * (Nz + 1) + Nz] * invh;
    } else if (i >= 1 && i <= Nx && j >= 1 && j < Nz) {
      v = k.a1 * rhow[(size_t)(i - 1) * (Nz + 1) + j] * k.idt;
      if (k.sailor) v += (rho[(size_t)(i - 1) * Nz + j] - rho[(size_t)(i - 1) * Nz + j - 1]) * invh * k.g0 * k.dt;
    }
    dw[t] = (T)v;
    if (k.open_cnv && j == Nz && i >= 1 && i <= Nx) {
      dbot[3 * i + 0] = (T)(-rhow[(size_t)(i - 1) * (Nz + 1) + Nz - 1] * invh);
      dbot[3 * i + 1] = (T)(-rhou[(size_t)(i - 1) * Nz + Nz - 1] * invh);
      dbot[3 * i + 2] = (T)(+rhou[(size_t)i * Nz + Nz - 1] * invh);
    }
  }
  if (t < g.NU) {
    int j = (int)(t % (Nz + 2)), i = (int)(t / (Nz + 2));
    double v = 1.0;
    if (j >= 1 && j <= Nz) {
      int ia = (i == 0) ? Nx - 1 : i - 1, ib = (i == Nx) ? 0 : i;
      v = (k.a1 + k.gamma) * rhou[(size_t)i * Nz + j - 1] * k.idt;
      if (k.sailor) v += (rho[(size_t)ib * Nz + j - 1] - rho[(size_t)ia * Nz + j - 1]) * invh * k.g0 * k.dt;
    }
    du[t] = (T)v;
  }
}

// the nine weights of an interior row from its two corner (C) and two cell (P)
// viscosities (fluidmech.jl:194-233 for W rows, 270-307 for U rows)
template <typename T>
struct RowW { T d, c1, c2, c3, c4, c5, c6, c7, c8; };
template <typename T>
__device__ __forceinline__ RowW<T> fly_row(T C1, T C2, T P1, T P2, T extra, T ih2) {
  const T c23 = (T)(2.0 / 3.0), c13 = (T)(1.0 / 3.0), hf = (T)0.5;
  RowW<T> w;
  w.d = extra + (c23 * (P1 + P2) * ih2 + hf * (C1 + C2) * ih2);
  w.c1 = -c23 * P1 * ih2;
  w.c2 = -c23 * P2 * ih2;
  w.c3 = -hf * C1 * ih2;
  w.c4 = -hf * C2 * ih2;
  w.c5 = -(hf * C1 - c13 * P1) * ih2;
  w.c6 = +(hf * C1 - c13 * P2) * ih2;
  w.c7 = +(hf * C2 - c13 * P1) * ih2;
  w.c8 = -(hf * C2 - c13 * P2) * ih2;
  return w;
}
template <typename T>
__device__ __forceinline__ RowW<T> plane_row(const T* __restrict__ c, size_t N, long long t) {
  RowW<T> w;
  w.d = c[t]; w.c1 = c[N + t]; w.c2 = c[2 * N + t]; w.c3 = c[3 * N + t]; w.c4 = c[4 * N + t];
  w.c5 = c[5 * N + t]; w.c6 = c[6 * N + t]; w.c7 = c[7 * N + t]; w.c8 = c[8 * N + t];
  return w;
}
// weights of interior W row t = (j, i) and interior U row u = (j, i).  Index
// arithmetic is 32-bit (a level holds fewer than 2^31 unknowns) and each
// neighbour is an offset from one base pointer.
template <typename T>
__device__ __forceinline__ RowW<T> w_row(const Geo& g, const VOp<T>& op, long long t, int j, int i) {
  if constexpr (kFly<T>) {
    const int Nz = g.Nz;
    const T* pc = op.etaco + ((i - 1) * (Nz + 1) + j);    // corners (j, i-1), (j, i)
    const T* pe = op.eta + ((i - 1) * Nz + j - 1);        // cells (j-1, i-1), (j, i-1)
    return fly_row<T>(pc[0], pc[Nz + 1], pe[0], pe[1], op.dw[t], geo_ih2<T>(g));
  } else {
    return plane_row<T>(op.cw, (size_t)g.NW, t);
  }
}
template <typename T>
__device__ __forceinline__ RowW<T> u_row(const Geo& g, const VOp<T>& op, long long u, int j, int i) {
  if constexpr (kFly<T>) {
    const int Nz = g.Nz, Nx = g.Nx;
    const int ia = (i == 0) ? Nx - 1 : i - 1, ib = (i == Nx) ? 0 : i;
    const T* pc = op.etaco + (i * (Nz + 1) + j - 1);      // corners (j-1, i), (j, i)
    return fly_row<T>(pc[0], pc[1], op.eta[ia * Nz + j - 1], op.eta[ib * Nz + j - 1], op.du[u],
                      geo_ih2<T>(g));
  } else {
    return plane_row<T>(op.cu, (size_t)g.NU, u);
  }
}
// W row t = (j, i) and U row u = (j, i) of A x, with the row's diagonal in *dg
// (boundary rows: their exact-row value).  FULL adds the pressure gradient GG p
// of the fine level (fluidmech.jl:343-356).
template <typename T, bool FULL>
__device__ __forceinline__ T vel_row_w(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xw,
                                       const T* xu, const T* xp, long long t, int j, int i, T* dg) {
  const int Nz = g.Nz, Nx = g.Nx, lw = Nz + 1, lu = Nz + 2;
  if (i == 0) { *dg = (T)1; return xw[t] + (T)k.sds * xw[(size_t)Nx * lw + j]; }
  if (i == Nx + 1) { *dg = (T)1; return xw[t] + (T)k.sds * xw[(size_t)1 * lw + j]; }
  if (j == 0 || j == Nz) {
    T d;
    if constexpr (kFly<T>) d = j == 0 ? (T)1 : op.dw[t];
    else d = op.cw[t];
    *dg = d;
    if (j == Nz && k.open_cnv) {   // open bottom: the continuity-like row, no pressure gradient
      T c1, c5, c7;
      if constexpr (kFly<T>) {
        c1 = op.dbot[3 * i]; c5 = op.dbot[3 * i + 1]; c7 = op.dbot[3 * i + 2];
      } else {
        c1 = op.cw[g.NW + t]; c5 = op.cw[5 * (size_t)g.NW + t]; c7 = op.cw[7 * (size_t)g.NW + t];
      }
      T s = d * xw[t];
      s += c1 * xw[t - 1];
      s += c5 * xu[(i - 1) * lu + j];
      s += c7 * xu[i * lu + j];
      return s;
    }
    return d * xw[t];
  }
  const RowW<T> c = w_row<T>(g, op, t, j, i);
  *dg = c.d;
  const T* pw = xw + t;                          // W(j, i)
  const T* pu = xu + ((i - 1) * lu + j);         // U(j, i-1)
  T s = c.d * pw[0];
  s += c.c1 * pw[-1];
  s += c.c2 * pw[1];
  s += c.c3 * pw[-lw];
  s += c.c4 * pw[lw];
  s += c.c5 * pu[0];
  s += c.c6 * pu[1];
  s += c.c7 * pu[lu];
  s += c.c8 * pu[lu + 1];
  if (FULL) {
    const T* pp = xp + (i * lu + j);
    s += geo_invh<T>(g) * (pp[1] - pp[0]);
  }
  return s;
}
template <typename T, bool FULL>
__device__ __forceinline__ T vel_row_u(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xw,
                                       const T* xu, const T* xp, long long u, int j, int i, T* dg) {
  const int Nz = g.Nz, Nx = g.Nx, lw = Nz + 1, lu = Nz + 2;
  if (j == 0) { *dg = (T)1; return xu[u] + (T)k.top_cnv * xu[u + 1]; }
  if (j == Nz + 1) { *dg = (T)1; return xu[u] + (T)k.bot_cnv * xu[u - 1]; }
  if (k.mms && (int)u == k.pin_u) { *dg = (T)1; return xu[u]; }
  const int il = (i == 0) ? Nx - 1 : i - 1, ir = (i == Nx) ? 1 : i + 1;
  const RowW<T> c = u_row<T>(g, op, u, j, i);
  *dg = c.d;
  const T* pu = xu + u;                          // U(j, i)
  const T* pw = xw + (i * lw + j - 1);           // W(j-1, i)
  T s = c.d * pu[0];
  s += c.c1 * xu[il * lu + j];
  s += c.c2 * xu[ir * lu + j];
  s += c.c3 * pu[-1];
  s += c.c4 * pu[1];
  s += c.c5 * pw[0];
  s += c.c6 * pw[lw];
  s += c.c7 * pw[1];
  s += c.c8 * pw[lw + 1];
  if (FULL) {
    const T* pp = xp + (i * lu + j);
    s += geo_invh<T>(g) * (pp[lu] - pp[0]);
  }
  return s;
}
// diagonal alone (the first Jacobi sweep from zero needs nothing else)
template <typename T>
__device__ __forceinline__ T vel_diag_w(const Geo& g, const VOp<T>& op, long long t, int j, int i) {
  if (i == 0 || i == g.Nx + 1 || j == 0) return (T)1;
  if constexpr (kFly<T>) return j == g.Nz ? op.dw[t] : w_row<T>(g, op, t, j, i).d;
  else return op.cw[t];
}
template <typename T>
__device__ __forceinline__ T vel_diag_u(const Geo& g, const OpConst& k, const VOp<T>& op, long long u, int j,
                                        int i) {
  if (j == 0 || j == g.Nz + 1 || (k.mms && (int)u == k.pin_u)) return (T)1;
  if constexpr (kFly<T>) return u_row<T>(g, op, u, j, i).d;
  else return op.cu[u];
}
// diagonal of velocity row t (flat index over W then U rows)
template <typename T>
__device__ __forceinline__ T vel_diag(const Geo& g, const OpConst& k, const VOp<T>& op, long long t) {
  if (t < g.NW) return vel_diag_w<T>(g, op, t, (int)(t % (g.Nz + 1)), (int)(t / (g.Nz + 1)));
  const long long u = t - g.NW;
  return vel_diag_u<T>(g, k, op, u, (int)(u % (g.Nz + 2)), (int)(u / (g.Nz + 2)));
}
// inertial part of the diagonal of interior U row u
template <typename T>
__device__ __forceinline__ T vel_inertia_u(const Geo& g, const VOp<T>& op, long long u) {
  if constexpr (kFly<T>) return op.du[u];
  else return op.cu[9 * (size_t)g.NU + u];
}

// y = A x over all velocity rows of a level (ghost / boundary rows included);
// if b != null: y = b - A x.  With FULL (fine level): adds the pressure
// gradient GG p (fluidmech.jl:343-356).  The unknowns are not __restrict__:
// the one-CTA multigrid kernels read them after other threads of the CTA wrote
// them, which the read-only load path does not see.
template <typename T, bool FULL>
__device__ __forceinline__ T vel_row(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xw, const T* xu,
                                     const T* xp, long long t) {
  T d;
  if (t < g.NW)
    return vel_row_w<T, FULL>(g, k, op, xw, xu, xp, t, (int)(t % (g.Nz + 1)), (int)(t / (g.Nz + 1)), &d);
  const long long u = t - g.NW;
  return vel_row_u<T, FULL>(g, k, op, xw, xu, xp, u, (int)(u % (g.Nz + 2)), (int)(u / (g.Nz + 2)), &d);
}

// pressure rows of LL: ghost ring, pin, rho-weighted divergence (fluidmech.jl:367-488)
template <typename T>
__device__ __forceinline__ T p_row(const Geo& g, const OpConst& k, const T* __restrict__ cp,
                                   const T* __restrict__ xw, const T* __restrict__ xu,
                                   const T* __restrict__ xp, int t, int j, int i) {
  const int Nz = g.Nz, Nx = g.Nx, lp = Nz + 2, lw = Nz + 1;
  if (j == 0) return xp[t] - xp[t + 1];
  if (j == Nz + 1) return xp[t] - xp[t - 1];
  // open bottom: the whole last interior row of P is pinned like the single
  // interior cell otherwise (its KP row becomes the identity, DM stays), and
  // its two ghost-column cells become P = 0 rows (fluidmech.jl:426-429, 478-487)
  const bool open_row = k.open_cnv && j == Nz;
  if (i == 0) return open_row ? xp[t] : xp[t] - xp[(size_t)Nx * lp + j];
  if (i == Nx + 1) return open_row ? xp[t] : xp[t] - xp[(size_t)1 * lp + j];
  if (k.mms && t == k.pin_p) return xp[t];
  const size_t NP = g.NP;
  T s = cp[t] * xu[(size_t)(i - 1) * lp + j] + cp[NP + t] * xu[(size_t)i * lp + j] +
        cp[2 * NP + t] * xw[(size_t)i * lw + j - 1] + cp[3 * NP + t] * xw[(size_t)i * lw + j];
  if (t == k.pin_p || open_row) s += xp[t];
  return s;
}

// DM coefficients of the interior P rows (fluidmech.jl:373-386)
__global__ void p_coef_kernel(Geo g, const double* __restrict__ rhow, const double* __restrict__ rhou,
                              double* cp) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.NP) return;
  const int Nz = g.Nz, Nx = g.Nx, lp = Nz + 2;
  int j = t % lp, i = t / lp;
  double c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  if (j >= 1 && j <= Nz && i >= 1 && i <= Nx) {
    c0 = -rhou[(size_t)(i - 1) * Nz + j - 1] * g.invh;
    c1 = +rhou[(size_t)i * Nz + j - 1] * g.invh;
    c2 = -rhow[(size_t)(i - 1) * (Nz + 1) + j - 1] * g.invh;
    c3 = +rhow[(size_t)(i - 1) * (Nz + 1) + j] * g.invh;
  }
  cp[t] = c0; cp[g.NP + t] = c1; cp[2 * g.NP + t] = c2; cp[3 * g.NP + t] = c3;
}

// y = S o (LL (S o v)) on the whole unknown vector; t must hold S o v.
// If b != null: y = b - S o (LL t).  Thread (j, i) of the 2-D grid takes the
// W, U and P rows at (j, i).
template <typename T>
__global__ void __launch_bounds__(256) stokes_apply_kernel(Geo g, OpConst k, VOp<T> op, const T* __restrict__ cp,
                                                           const T* __restrict__ scl, const T* __restrict__ tv,
                                                           const T* __restrict__ b, T* y) {
  XC_PDL_WAIT();
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int i = blockIdx.y * 8 + threadIdx.y;
  const int Nz = g.Nz, Nx = g.Nx;
  if (j > Nz + 1 || i > Nx + 1) return;
  const T* xw = tv;
  const T* xu = tv + g.NW;
  const T* xp = tv + g.NW + g.NU;
  T d;
  if (j <= Nz) {
    const long long t = (long long)i * (Nz + 1) + j;
    const T v = vel_row_w<T, true>(g, k, op, xw, xu, xp, t, j, i, &d) * scl[t];
    y[t] = b ? b[t] - v : v;
  }
  if (i <= Nx) {
    const long long u = (long long)i * (Nz + 2) + j, t = g.NW + u;
    const T v = vel_row_u<T, true>(g, k, op, xw, xu, xp, u, j, i, &d) * scl[t];
    y[t] = b ? b[t] - v : v;
  }
  {
    const int pt = i * (Nz + 2) + j;
    const long long t = (long long)g.NW + g.NU + pt;
    const T v = p_row<T>(g, k, cp, xw, xu, xp, pt, j, i) * scl[t];
    y[t] = b ? b[t] - v : v;
  }
}

template <typename T>
__global__ void mul_kernel(long long n, const T* __restrict__ a, const T* __restrict__ b, T* out) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = a[t] * b[t];
}
template <typename T>
__global__ void div_kernel(long long n, const T* __restrict__ a, const T* __restrict__ b, T* out) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = a[t] / b[t];
}
template <typename A, typename B>
__global__ void convert_kernel(long long n, const A* __restrict__ a, B* out) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) out[t] = (B)a[t];
}
// x += s o dy (FP64 refinement update)
template <typename T>
__global__ void refine_update_kernel(long long n, const T* __restrict__ dy, const double* __restrict__ scl,
                                     double* x) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) x[t] += scl[t] * (double)dy[t];
}

// ---------------------------------------------------------------------------
// velocity multigrid
// ---------------------------------------------------------------------------
// Each multigrid operation is a per-unknown body (`*_at`, index t) used both by
// a grid-wide kernel and by the one-CTA kernels of the small levels.
// one velocity row of a Jacobi sweep (MODE 0: first sweep from zero, 1: sweep)
// or of the residual (MODE 2): out = xi + w D^-1 (b - A xi), resp. b - A xi;
// ghost / boundary rows are relaxed exactly (w = 1)
template <typename T, int MODE>
__device__ __forceinline__ void vel_update_w(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xi,
                                             const T* b, T* out, T omega, long long t, int j, int i,
                                             const T* dscl = nullptr) {
  const bool exact = i == 0 || i == g.Nx + 1 || j == 0 || j == g.Nz;
  if (MODE == 0) {
    out[t] = sdiv<T>((exact ? (T)1 : omega) * b[t], vel_diag_w<T>(g, op, t, j, i));
    return;
  }
  T d;
  const T ax = vel_row_w<T, false>(g, k, op, xi, xi + g.NW, nullptr, t, j, i, &d);
  if (MODE == 2) out[t] = b[t] - ax;
  else if (MODE == 3) out[t] = (xi[t] + sdiv<T>((exact ? (T)1 : omega) * (b[t] - ax), d)) / dscl[t];
  else out[t] = xi[t] + sdiv<T>((exact ? (T)1 : omega) * (b[t] - ax), d);
}
template <typename T, int MODE>
__device__ __forceinline__ void vel_update_u(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xi,
                                             const T* b, T* out, T omega, long long u, int j, int i,
                                             const T* dscl = nullptr) {
  const bool exact = j == 0 || j == g.Nz + 1 || (k.mms && (int)u == k.pin_u);
  const long long t = g.NW + u;
  if (MODE == 0) {
    out[t] = sdiv<T>((exact ? (T)1 : omega) * b[t], vel_diag_u<T>(g, k, op, u, j, i));
    return;
  }
  T d;
  const T ax = vel_row_u<T, false>(g, k, op, xi, xi + g.NW, nullptr, u, j, i, &d);
  if (MODE == 2) out[t] = b[t] - ax;
  else if (MODE == 3) out[t] = (xi[t] + sdiv<T>((exact ? (T)1 : omega) * (b[t] - ax), d)) / dscl[t];
  else out[t] = xi[t] + sdiv<T>((exact ? (T)1 : omega) * (b[t] - ax), d);
}
// a level's rows on a 2-D grid: thread (j, i) takes W row (j, i) and U row
// (j, i) -- no index division, and the two rows share viscosity loads.
// MODE 3 is a sweep whose result is written divided by dscl (the last sweep
// of the fine level, returning the preconditioned vector in scaled form).
template <typename T, int MODE>
__global__ void __launch_bounds__(256) vel_sweep2d_kernel(Geo g, OpConst k, VOp<T> op, const T* __restrict__ xi,
                                                          const T* __restrict__ b, T* out, T omega,
                                                          const T* __restrict__ dscl) {
  XC_PDL_WAIT();
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int i = blockIdx.y * 8 + threadIdx.y;
  if (j <= g.Nz && i <= g.Nx + 1)
    vel_update_w<T, MODE>(g, k, op, xi, b, out, omega, (long long)i * (g.Nz + 1) + j, j, i, dscl);
  if (j <= g.Nz + 1 && i <= g.Nx)
    vel_update_u<T, MODE>(g, k, op, xi, b, out, omega, (long long)i * (g.Nz + 2) + j, j, i, dscl);
}


// FP32 sweep (all MODEs of vel_sweep2d_kernel) with each thread taking kRB
// consecutive rows along z of one column i, W and U rows alike.  Threads whose
// rows are all interior (W rows 1..Nz-1, U rows 1..Nz, columns 1..Nx-1, no
// MMS pin) take a path without any boundary classification or periodic wrap,
// and vertically adjacent rows share their loads: the W rows' lower corner
// and cell viscosities are the next row's upper ones, the U rows reuse the W
// rows' corner and cell values of the same column, and the unknowns of the
// column are loaded once for both row kinds.  Per row the weights and the
// products are those of vel_update_w / vel_update_u in the same order.  Other
// threads run those per-row bodies.
constexpr int kRB = 4;

template <int MODE>
__device__ __forceinline__ void rb_store(float* out, long long t, float xc, float bt, float ax, float d,
                                         float omega, const float* dscl) {
  if (MODE == 2) out[t] = bt - ax;
  else if (MODE == 3) out[t] = (xc + sdiv<float>(omega * (bt - ax), d)) / dscl[t];
  else out[t] = xc + sdiv<float>(omega * (bt - ax), d);
}

template <int MODE>
__global__ void __launch_bounds__(256) vel_sweep_rb_kernel(Geo g, OpConst k, VOp<float> op,
                                                          const float* __restrict__ xi,
                                                          const float* __restrict__ b, float* out, float omega,
                                                          const float* __restrict__ dscl) {
  XC_PDL_WAIT();
  const int j0 = (blockIdx.x * 32 + threadIdx.x) * kRB;
  const int i = blockIdx.y * 8 + threadIdx.y;
  const int Nz = g.Nz, Nx = g.Nx, lw = Nz + 1, lu = Nz + 2;
  const bool interior = !k.mms && j0 >= 1 && j0 + kRB - 1 <= Nz - 1 && i >= 1 && i <= Nx - 1;
  if (!interior) {
#pragma unroll
    for (int r = 0; r < kRB; ++r) {
      const int j = j0 + r;
      if (j <= Nz && i <= Nx + 1)
        vel_update_w<float, MODE>(g, k, op, xi, b, out, omega, (long long)i * lw + j, j, i, dscl);
      if (j <= Nz + 1 && i <= Nx)
        vel_update_u<float, MODE>(g, k, op, xi, b, out, omega, (long long)i * lu + j, j, i, dscl);
    }
    return;
  }
  const float ih2 = g.ih2f;
  const float* xw = xi;
  const float* xu = xi + g.NW;
  // viscosities: corners of columns i-1 (W rows' C1) and i (W rows' C2, U
  // rows' C1 / C2) at z = j0-1 .. j0+kRB-1; cells of columns i-1 and i at
  // z = j0-1 .. j0+kRB-1
  float ca[kRB + 1], cb[kRB + 1], pa[kRB + 1], pb[kRB + 1];
#pragma unroll
  for (int r = 0; r <= kRB; ++r) {
    ca[r] = op.etaco[(i - 1) * lw + j0 - 1 + r];
    cb[r] = op.etaco[i * lw + j0 - 1 + r];
    pa[r] = op.eta[(i - 1) * Nz + j0 - 1 + r];
    pb[r] = op.eta[i * Nz + j0 - 1 + r];
  }
  // W rows (j, i), j = j0 + r: C1 = corner (j, i-1), C2 = corner (j, i),
  // P1 = cell (j-1, i-1), P2 = cell (j, i-1)
  {
    const long long t0 = (long long)i * lw + j0;
    const float* pw = xw + t0;
    const float* pu = xu + ((i - 1) * lu + j0);
#pragma unroll
    for (int r = 0; r < kRB; ++r) {
      const long long t = t0 + r;
      const RowW<float> c = fly_row<float>(ca[r + 1], cb[r + 1], pa[r], pa[r + 1], op.dw[t], ih2);
      if (MODE == 0) {
        out[t] = sdiv<float>(omega * b[t], c.d);
        continue;
      }
      float sum = c.d * pw[r];
      sum += c.c1 * pw[r - 1];
      sum += c.c2 * pw[r + 1];
      sum += c.c3 * pw[r - lw];
      sum += c.c4 * pw[r + lw];
      sum += c.c5 * pu[r];
      sum += c.c6 * pu[r + 1];
      sum += c.c7 * pu[r + lu];
      sum += c.c8 * pu[r + lu + 1];
      rb_store<MODE>(out, t, pw[r], b[t], sum, c.d, omega, dscl);
    }
  }
  // U rows (j, i): C1 = corner (j-1, i), C2 = corner (j, i), P1 = cell (j-1,
  // i-1), P2 = cell (j-1, i); no periodic wrap for 1 <= i <= Nx-1
  {
    const long long u0 = (long long)i * lu + j0;
    const float* pu = xu + u0;
    const float* pw = xw + (i * lw + j0 - 1);
#pragma unroll
    for (int r = 0; r < kRB; ++r) {
      const long long u = u0 + r;
      const RowW<float> c = fly_row<float>(cb[r], cb[r + 1], pa[r], pb[r], op.du[u], ih2);
      if (MODE == 0) {
        out[g.NW + u] = sdiv<float>(omega * b[g.NW + u], c.d);
        continue;
      }
      float sum = c.d * pu[r];
      sum += c.c1 * pu[r - lu];
      sum += c.c2 * pu[r + lu];
      sum += c.c3 * pu[r - 1];
      sum += c.c4 * pu[r + 1];
      sum += c.c5 * pw[r];
      sum += c.c6 * pw[r + lw];
      sum += c.c7 * pw[r + 1];
      sum += c.c8 * pw[r + lw + 1];
      rb_store<MODE>(out, g.NW + u, pu[r], b[g.NW + u], sum, c.d, omega, dscl);
    }
  }
}

inline dim3 grid_rb(const Geo& g) {
  return dim3((unsigned)((g.Nz + 2 + 32 * kRB - 1) / (32 * kRB)), (unsigned)((g.Nx + 2 + 7) / 8));
}

// FP32 sweep (MODE 1, 2, 3 of vel_sweep2d_kernel) of a block from shared
// memory.  A 32 x 8 block stages the W and U unknowns and the cell and corner
// viscosities of its rows with a one-row and one-column halo (34 x 10 each)
// once; every row then reads its nine neighbours and four viscosities from
// there, so the per-row address arithmetic and the repeated L1 traffic of
// vel_sweep2d_kernel are gone.  Blocks at the periodic seam (i0 = 0 or
// i0 + 8 > Nx), whose stencils wrap to the far side, take the per-row path.
// The operations and their order are those of vel_update_w / vel_update_u.
// Measured at 1024^2 it is 5% slower than the per-row kernel (L1 already
// serves the neighbours there, and the tile barrier costs latency hiding), so
// the solver uses it only when asked (xc_solver_opts.tiled_sweep).
constexpr int kTJ = 32, kTI = 8;

template <int MODE>
__device__ __forceinline__ void sweep_store(float* out, long long t, float xc, float bt, float ax, float d,
                                            bool exact, float omega, const float* dscl) {
  if (MODE == 2) out[t] = bt - ax;
  else if (MODE == 3) out[t] = (xc + sdiv<float>((exact ? 1.f : omega) * (bt - ax), d)) / dscl[t];
  else out[t] = xc + sdiv<float>((exact ? 1.f : omega) * (bt - ax), d);
}

template <int MODE>
__global__ void __launch_bounds__(kTJ * kTI) vel_sweep_tiled_kernel(Geo g, OpConst k, VOp<float> op,
                                                                    const float* __restrict__ xi,
                                                                    const float* __restrict__ b, float* out,
                                                                    float omega, const float* __restrict__ dscl) {
  XC_PDL_WAIT();
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j0 = blockIdx.x * kTJ, i0 = blockIdx.y * kTI;
  const int j = j0 + tx, i = i0 + ty;
  const int Nz = g.Nz, Nx = g.Nx, lw = Nz + 1, lu = Nz + 2;
  if (i0 < 1 || i0 + kTI > Nx || (k.open_cnv && j0 <= Nz && Nz < j0 + kTJ)) {
    if (j <= Nz && i <= Nx + 1) vel_update_w<float, MODE>(g, k, op, xi, b, out, omega, (long long)i * lw + j, j, i, dscl);
    if (j <= Nz + 1 && i <= Nx) vel_update_u<float, MODE>(g, k, op, xi, b, out, omega, (long long)i * lu + j, j, i, dscl);
    return;
  }
  __shared__ float sW[kTI + 2][kTJ + 2], sU[kTI + 2][kTJ + 2], sE[kTI + 2][kTJ + 2], sC[kTI + 2][kTJ + 2];
  const float* xw = xi;
  const float* xu = xi + g.NW;
  for (int q = ty * kTJ + tx; q < (kTI + 2) * (kTJ + 2); q += kTJ * kTI) {
    const int ii = q / (kTJ + 2), jj = q % (kTJ + 2);
    const int gi = i0 - 1 + ii, gj = j0 - 1 + jj;    // gi in [0, Nx]: inside every array's columns
    sW[ii][jj] = (gj >= 0 && gj <= Nz) ? xw[gi * lw + gj] : 0.f;
    sU[ii][jj] = (gj >= 0 && gj <= Nz + 1) ? xu[gi * lu + gj] : 0.f;
    sE[ii][jj] = (gj >= 0 && gj < Nz && gi < Nx) ? op.eta[gi * Nz + gj] : 0.f;
    sC[ii][jj] = (gj >= 0 && gj <= Nz) ? op.etaco[gi * (Nz + 1) + gj] : 0.f;
  }
  __syncthreads();
  const float ih2 = g.ih2f;
  const int a = ty + 1, c = tx + 1;    // this thread's (i, j) in the tiles
  if (j <= Nz) {                       // W row (j, i), 1 <= i <= Nx here
    const long long t = (long long)i * lw + j;
    const bool exact = j == 0 || j == Nz;
    float ax, d;
    if (exact) {
      d = j == 0 ? 1.f : op.dw[t];
      ax = d * sW[a][c];
    } else {
      const RowW<float> w = fly_row<float>(sC[a - 1][c], sC[a][c], sE[a - 1][c - 1], sE[a - 1][c], op.dw[t], ih2);
      d = w.d;
      float s = w.d * sW[a][c];
      s += w.c1 * sW[a][c - 1];
      s += w.c2 * sW[a][c + 1];
      s += w.c3 * sW[a - 1][c];
      s += w.c4 * sW[a + 1][c];
      s += w.c5 * sU[a - 1][c];
      s += w.c6 * sU[a - 1][c + 1];
      s += w.c7 * sU[a][c];
      s += w.c8 * sU[a][c + 1];
      ax = s;
    }
    sweep_store<MODE>(out, t, sW[a][c], b[t], ax, d, exact, omega, dscl);
  }
  if (j <= Nz + 1) {                   // U row (j, i), 1 <= i <= Nx - 1 here
    const long long u = (long long)i * lu + j, t = g.NW + u;
    const bool exact = j == 0 || j == Nz + 1 || (k.mms && (int)u == k.pin_u);
    float ax, d = 1.f;
    if (j == 0) ax = sU[a][c] + (float)k.top_cnv * sU[a][c + 1];
    else if (j == Nz + 1) ax = sU[a][c] + (float)k.bot_cnv * sU[a][c - 1];
    else if (exact) ax = sU[a][c];
    else {
      const RowW<float> w = fly_row<float>(sC[a][c - 1], sC[a][c], sE[a - 1][c - 1], sE[a][c - 1], op.du[u], ih2);
      d = w.d;
      float s = w.d * sU[a][c];
      s += w.c1 * sU[a - 1][c];
      s += w.c2 * sU[a + 1][c];
      s += w.c3 * sU[a][c - 1];
      s += w.c4 * sU[a][c + 1];
      s += w.c5 * sW[a][c - 1];
      s += w.c6 * sW[a + 1][c - 1];
      s += w.c7 * sW[a][c];
      s += w.c8 * sW[a + 1][c];
      ax = s;
    }
    sweep_store<MODE>(out, t, sU[a][c], b[t], ax, d, exact, omega, dscl);
  }
}

// damped Jacobi: xo = xi + w D^-1 (b - A xi); ghost / boundary rows exact
template <typename T>
__device__ __forceinline__ void vel_jacobi_at(const Geo& g, const OpConst& k, const VOp<T>& op, const T* xi,
                                              const T* b, T* xo, T omega, int zero_init, long long t) {
  // flat index over W then U rows; levels stay below 2^31 unknowns
  const int tt = (int)t;
  if (tt < g.NW) {
    const int j = tt % (g.Nz + 1), i = tt / (g.Nz + 1);
    if (zero_init) vel_update_w<T, 0>(g, k, op, xi, b, xo, omega, t, j, i);
    else vel_update_w<T, 1>(g, k, op, xi, b, xo, omega, t, j, i);
  } else {
    const int u = tt - g.NW, j = u % (g.Nz + 2), i = u / (g.Nz + 2);
    if (zero_init) vel_update_u<T, 0>(g, k, op, xi, b, xo, omega, u, j, i);
    else vel_update_u<T, 1>(g, k, op, xi, b, xo, omega, u, j, i);
  }
}
template <typename T>
__device__ __forceinline__ void vel_residual_at(const Geo& g, const OpConst& k, const VOp<T>& op, const T* x,
                                                const T* b, T* r, long long t) {
  const int tt = (int)t;
  if (tt < g.NW) {
    vel_update_w<T, 2>(g, k, op, x, b, r, (T)0, t, tt % (g.Nz + 1), tt / (g.Nz + 1));
  } else {
    const int u = tt - g.NW;
    vel_update_u<T, 2>(g, k, op, x, b, r, (T)0, u, u % (g.Nz + 2), u / (g.Nz + 2));
  }
}

// restriction of the interior-row residual (full weighting / 4 of the
// bilinear prolongation); coarse ghost / boundary rows get zero.  W row
// (J, Ic) and U row (Jr, I) of the coarse level.
template <typename T>
__device__ __forceinline__ T vel_restrict_w(const Geo& f, const Geo& c, const T* rw, int J, int Ic) {
  const int lwf = f.Nz + 1;
  T acc = 0;
  if (J >= 1 && J <= c.Nz - 1 && Ic >= 1 && Ic <= c.Nx) {
    const int I = Ic - 1;
    const int ixs[4] = {2 * I - 1, 2 * I, 2 * I + 1, 2 * I + 2};
    const T wx[4] = {(T)0.25, (T)0.75, (T)0.75, (T)0.25};
    for (int dj = -1; dj <= 1; ++dj) {
      const T wz = dj == 0 ? (T)1 : (T)0.5;
      const int j = 2 * J + dj;
      for (int q = 0; q < 4; ++q) {
        int ix = ixs[q];
        ix = ix < 0 ? ix + f.Nx : (ix >= f.Nx ? ix - f.Nx : ix);
        acc += wz * wx[q] * rw[(ix + 1) * lwf + j];
      }
    }
    acc *= (T)0.25;
  }
  return acc;
}
template <typename T>
__device__ __forceinline__ T vel_restrict_u(const Geo& f, const Geo& c, const T* ru, int Jr, int I) {
  const int luf = f.Nz + 2;
  T acc = 0;
  if (Jr >= 1 && Jr <= c.Nz) {
    const int Jc = Jr - 1;
    const int jzs[4] = {2 * Jc - 1, 2 * Jc, 2 * Jc + 1, 2 * Jc + 2};
    const T wz[4] = {(T)0.25, (T)0.75, (T)0.75, (T)0.25};
    for (int q = 0; q < 4; ++q) {
      const int jz = jzs[q];
      if (jz < 0 || jz >= f.Nz) continue;
      for (int di = -1; di <= 1; ++di) {
        const int i = 2 * I + di;
        if (i < 0 || i > f.Nx) continue;
        const T wx = di == 0 ? (T)1 : (T)0.5;
        acc += wz[q] * wx * ru[i * luf + jz + 1];
      }
    }
    acc *= (T)0.25;
  }
  return acc;
}
// flat index over the coarse W then U rows (levels stay below 2^31 unknowns)
template <typename T>
__device__ __forceinline__ void vel_restrict_at(const Geo& f, const Geo& c, const T* r, T* bc, long long t) {
  const int tt = (int)t;
  if (tt < c.NW) {
    bc[t] = vel_restrict_w<T>(f, c, r, tt % (c.Nz + 1), tt / (c.Nz + 1));
  } else {
    const int u = tt - c.NW;
    bc[t] = vel_restrict_u<T>(f, c, r + f.NW, u % (c.Nz + 2), u / (c.Nz + 2));
  }
}
// 2-D grid over the coarse row positions (grid2 of the coarse level)
template <typename T>
__global__ void __launch_bounds__(256) vel_restrict2d_kernel(Geo f, Geo c, const T* __restrict__ r, T* bc) {
  XC_PDL_WAIT();
  const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
  if (j <= c.Nz && i <= c.Nx + 1) bc[i * (c.Nz + 1) + j] = vel_restrict_w<T>(f, c, r, j, i);
  if (j <= c.Nz + 1 && i <= c.Nx) bc[c.NW + i * (c.Nz + 2) + j] = vel_restrict_u<T>(f, c, r + f.NW, j, i);
}

// x_f += P x_c (bilinear; ghost rows of U follow the reflection rule): the
// correction of fine W row (j, i) and fine U row (j, i)
template <typename T>
__device__ __forceinline__ T vel_prolong_w(const Geo& f, const Geo& c, const T* cw, int j, int i) {
  const int lwc = c.Nz + 1;
  int ix = (i - 1) % f.Nx;
  if (ix < 0) ix += f.Nx;
  const int I0 = ix / 2;
  const int In = (ix % 2 == 0) ? (I0 - 1 + c.Nx) % c.Nx : (I0 + 1) % c.Nx;
  T v = 0;
  const int J0 = j / 2;
  const int nz = (j % 2 == 0) ? 1 : 2;
  for (int q = 0; q < nz; ++q) {
    const int J = J0 + q;
    const T wz = nz == 1 ? (T)1 : (T)0.5;
    v += wz * ((T)0.75 * cw[(I0 + 1) * lwc + J] + (T)0.25 * cw[(In + 1) * lwc + J]);
  }
  return v;
}
template <typename T>
__device__ __forceinline__ T vel_prolong_u(const Geo& f, const Geo& c, const OpConst& k, const T* cu, int j, int i) {
  const int luc = c.Nz + 2;
  auto interior = [&](int jj) -> T {
    const int jz = jj - 1, J0 = jz / 2;
    const int Jn = (jz % 2 == 0) ? J0 : J0 + 2;     // coarse row of the 1/4 neighbour (full layout)
    T v = 0;
    const int nx = (i % 2 == 0) ? 1 : 2;
    const int I0 = (i % 2 == 0) ? i / 2 : (i - 1) / 2;
    for (int q = 0; q < nx; ++q) {
      const T wx = nx == 1 ? (T)1 : (T)0.5;
      const int I = I0 + q;
      v += wx * ((T)0.75 * cu[I * luc + J0 + 1] + (T)0.25 * cu[I * luc + Jn]);
    }
    return v;
  };
  if (j == 0) return -(T)k.top_cnv * interior(1);
  if (j == f.Nz + 1) return -(T)k.bot_cnv * interior(f.Nz);
  return interior(j);
}
template <typename T>
__device__ __forceinline__ void vel_prolong_at(const Geo& f, const Geo& c, const OpConst& k, const T* xc, T* xf,
                                               long long t) {
  const int tt = (int)t;
  if (tt < f.NW) {
    xf[t] += vel_prolong_w<T>(f, c, xc, tt % (f.Nz + 1), tt / (f.Nz + 1));
  } else {
    const int u = tt - f.NW;
    xf[t] += vel_prolong_u<T>(f, c, k, xc + c.NW, u % (f.Nz + 2), u / (f.Nz + 2));
  }
}
// 2-D grid over the fine row positions (grid2 of the fine level)
template <typename T>
__global__ void __launch_bounds__(256) vel_prolong2d_kernel(Geo f, Geo c, OpConst k, const T* __restrict__ xc,
                                                            T* xf) {
  XC_PDL_WAIT();
  const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
  if (j <= f.Nz && i <= f.Nx + 1) xf[i * (f.Nz + 1) + j] += vel_prolong_w<T>(f, c, xc, j, i);
  if (j <= f.Nz + 1 && i <= f.Nx) xf[f.NW + i * (f.Nz + 2) + j] += vel_prolong_u<T>(f, c, k, xc + c.NW, j, i);
}

// coarse coefficient fields: eta (avg4), etaco (injection), rho (avg4),
// rhow / rhou (avg of the two fine faces of the coarse face)
__global__ void coarsen_fields_kernel(int Nzc, int Nxc, const double* __restrict__ eta,
                                      const double* __restrict__ etaco, const double* __restrict__ rho,
                                      const double* __restrict__ rhow, const double* __restrict__ rhou,
                                      double* etac, double* etacoc, double* rhoc, double* rhowc,
                                      double* rhouc, int mean) {
  XC_PDL_WAIT();
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  const int Nz = 2 * Nzc;
  if (J > Nzc || I > Nxc) return;
  etacoc[(size_t)I * (Nzc + 1) + J] = etaco[(size_t)(2 * I) * (Nz + 1) + 2 * J];
  if (I < Nxc) {
    rhowc[(size_t)I * (Nzc + 1) + J] = 0.5 * (rhow[(size_t)(2 * I) * (Nz + 1) + 2 * J] +
                                              rhow[(size_t)(2 * I + 1) * (Nz + 1) + 2 * J]);
  }
  if (J < Nzc) {
    rhouc[(size_t)I * Nzc + J] = 0.5 * (rhou[(size_t)(2 * I) * Nz + 2 * J] + rhou[(size_t)(2 * I) * Nz + 2 * J + 1]);
  }
  if (J < Nzc && I < Nxc) {
    size_t a = (size_t)(2 * I) * Nz + 2 * J, b = (size_t)(2 * I + 1) * Nz + 2 * J;
    if (mean == 1)        // geometric
      etac[(size_t)I * Nzc + J] = exp(0.25 * (log(eta[a]) + log(eta[a + 1]) + log(eta[b]) + log(eta[b + 1])));
    else if (mean == 2)   // harmonic
      etac[(size_t)I * Nzc + J] = 4.0 / (1.0 / eta[a] + 1.0 / eta[a + 1] + 1.0 / eta[b] + 1.0 / eta[b + 1]);
    else
      etac[(size_t)I * Nzc + J] = 0.25 * (eta[a] + eta[a + 1] + eta[b] + eta[b + 1]);
    rhoc[(size_t)I * Nzc + J] = 0.25 * (rho[a] + rho[a + 1] + rho[b] + rho[b + 1]);
  }
}

// sum of v over the CTA (all threads get it); red holds 32 doubles
__device__ __forceinline__ double cta_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0;
  for (int q = 0; q < nw; ++q) s += red[q];
  return s;
}

__device__ __forceinline__ double cta_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double m = 0;
  for (int q = 0; q < nw; ++q) m = fmax(m, red[q]);
  return m;
}

// ---- direct solve of a small coarsest level -------------------------------
// A coarsest level of at most kDenseMax unknowns is solved with its inverse:
// the dense matrix is formed once per solve by applying the level's rows to
// unit vectors (kDenseBatch at a time), inverted by Gauss-Jordan elimination
// with partial pivoting in the hierarchy's precision, and each V-cycle's
// coarse solve becomes one matrix-vector product by one CTA instead of tens of
// CTA-wide Jacobi sweeps.  ok = 0 (the sweeps are used instead) on a pivot
// below 1e-6 (FP32) or 1e-12 (FP64) of the largest entry, or where the
// velocity level has the unlifted uniform-U mode.
constexpr int kDenseMax = 64;
constexpr int kDenseBatch = 16;

// In-place inverse of the n x n row-major matrix M in shared memory, in the
// working precision R of the hierarchy (the coarse matrix is far from
// singular wherever ok stays 1; the FP64 pipe would make an FP64 inversion of
// the FP32 hierarchy's matrix several times slower).  Per column k, warp 0
// finds the pivot, swaps it into row k, scales that row and saves column k;
// then every thread eliminates: two CTA barriers per column.
template <typename R>
__device__ void gj_invert_cta(R* M, int n, int* piv, int* ok, R* fcol, double* red) {
  double amax = 0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) amax = fmax(amax, (double)fabs(M[e]));
  amax = cta_max(amax, red);
  const double thr = (std::is_same<R, float>::value ? 1e-6 : 1e-12) * amax;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      R best = (R)-1;
      int bi = k;
      for (int i = k + lane; i < n; i += 32) {
        const R v = fabs(M[i * n + k]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const R ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        piv[k] = bi;
        if (!((double)best > thr)) *ok = 0;
      }
      if (bi != k)
        for (int c = lane; c < n; c += 32) {
          const R t = M[k * n + c];
          M[k * n + c] = M[bi * n + c];
          M[bi * n + c] = t;
        }
      __syncwarp();
      const R pv = M[k * n + k];
      __syncwarp();
      // row k scaled, its pivot entry becoming 1 / pv; column k of the others saved
      for (int c = lane; c < n; c += 32) M[k * n + c] = (c == k ? (R)1 : M[k * n + c]) / pv;
      for (int i = lane; i < n; i += 32) fcol[i] = M[i * n + k];
    }
    __syncthreads();
    // thread (row group, column): column c = tid mod 64 of rows tid / 64,
    // + blockDim / 64, ... (n <= 64; no index division per entry, the pivot
    // row's entry of the column read once); the same update of each entry
    {
      const int c = threadIdx.x & 63, rs = blockDim.x >> 6;
      if (c < n) {
        const R mk = M[k * n + c];
        for (int i = threadIdx.x >> 6; i < n; i += rs)
          if (i != k) M[i * n + c] = (c == k ? (R)0 : M[i * n + c]) - fcol[i] * mk;
      }
    }
    __syncthreads();
  }
  // A^-1 = (P A)^-1 P: the row interchanges undone as column interchanges,
  // last first, each thread on its own rows
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = n - 1; k >= 0; --k) {
      const int p = piv[k];
      if (p != k) {
        const R t = M[i * n + k];
        M[i * n + k] = M[i * n + p];
        M[i * n + p] = t;
      }
    }
  __syncthreads();
}

// x = inv b by one CTA (a warp per row); ends with a barrier
template <typename T>
__device__ void dense_apply_cta(const T* __restrict__ inv, int n, const T* b, T* x) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = warp; r < n; r += nw) {
    T acc = 0;
    for (int c = lane; c < n; c += 32) acc += inv[r * n + c] * b[c];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[r] = acc;
  }
  __syncthreads();
}

// many damped-Jacobi sweeps on the coarsest velocity level, by one whole CTA.
// With free slip at top and bottom (top_cnv = bot_cnv = -1) and periodic x, a
// uniform U shift is a null mode of the viscous rows; where inertia does not
// lift it (the inertia-free limit of the manufactured solution) the sweeps
// would let that mode grow with the sweep count, so it is removed from the
// coarse correction and left to the pinned fine level and the Krylov method.
template <typename T>
__device__ void vel_coarse_cta(const Geo& g, const OpConst& k, const VOp<T>& op, T* x, T* x2, const T* b,
                               int sweeps, T omega, const T* inv = nullptr, const int* inv_ok = nullptr) {
  const long long n = (long long)g.NW + g.NU;
  if (inv && *inv_ok) {
    dense_apply_cta<T>(inv, (int)n, b, x);
    return;
  }
  for (long long t = threadIdx.x; t < n; t += blockDim.x) x[t] = 0;
  __syncthreads();
  T* a = x;
  T* o = x2;
  for (int s = 0; s < sweeps; ++s) {
    for (long long t = threadIdx.x; t < n; t += blockDim.x) vel_jacobi_at<T>(g, k, op, a, b, o, omega, 0, t);
    __syncthreads();
    T* tmp = a; a = o; o = tmp;
  }
  if (a != x)
    for (long long t = threadIdx.x; t < n; t += blockDim.x) x[t] = a[t];
  __syncthreads();
  if (k.top_cnv == -1 && k.bot_cnv == -1 && !k.mms) {
    __shared__ double red[32];
    double si = 0, sd = 0, sx = 0;
    for (long long u = threadIdx.x; u < g.NU; u += blockDim.x) {
      int j = (int)(u % (g.Nz + 2));
      if (j >= 1 && j <= g.Nz) {
        si += (double)vel_inertia_u<T>(g, op, u);
        sd += (double)vel_diag<T>(g, k, op, g.NW + u);
      }
      sx += (double)x[g.NW + u];
    }
    si = cta_sum(si, red);
    sd = cta_sum(sd, red);
    sx = cta_sum(sx, red);
    if (si <= 1e-6 * sd) {
      const T m = (T)(sx / (double)g.NU);
      for (long long u = threadIdx.x; u < g.NU; u += blockDim.x) x[g.NW + u] -= m;
    }
    __syncthreads();
  }
}
template <typename T>
__global__ void vel_coarse_kernel(Geo g, OpConst k, VOp<T> op, T* x, T* x2, const T* __restrict__ b, int sweeps,
                                  T omega, const T* inv, const int* inv_ok) {
  XC_PDL_WAIT();
  vel_coarse_cta<T>(g, k, op, x, x2, b, sweeps, omega, inv, inv_ok);
}

// the inverse of the coarsest velocity level (NW + NU <= kDenseMax), one CTA
template <typename T>
__global__ void __launch_bounds__(256) vel_dense_inv_kernel(Geo g, OpConst k, VOp<T> op, T* inv, int* ok) {
  XC_PDL_WAIT();
  __shared__ T M[kDenseMax * kDenseMax];
  __shared__ T xb[kDenseBatch][kDenseMax];
  __shared__ T fcol[kDenseMax];
  __shared__ double red[32];
  __shared__ int piv[kDenseMax];
  __shared__ int sok;
  const int n = g.NW + g.NU;
  if (threadIdx.x == 0) sok = 1;
  for (int c0 = 0; c0 < n; c0 += kDenseBatch) {
    for (int e = threadIdx.x; e < kDenseBatch * kDenseMax; e += blockDim.x) {
      const int bq = e / kDenseMax, r = e - bq * kDenseMax;
      xb[bq][r] = (T)(r == c0 + bq ? 1 : 0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kDenseBatch * n; e += blockDim.x) {
      const int bq = e / n, r = e - bq * n, c = c0 + bq;
      if (c >= n) continue;
      const T* xv = xb[bq];
      T d, v;
      if (r < g.NW) {
        v = vel_row_w<T, false>(g, k, op, xv, xv + g.NW, nullptr, r, r % (g.Nz + 1), r / (g.Nz + 1), &d);
      } else {
        const int u = r - g.NW;
        v = vel_row_u<T, false>(g, k, op, xv, xv + g.NW, nullptr, u, u % (g.Nz + 2), u / (g.Nz + 2), &d);
      }
      M[r * n + c] = v;
    }
    __syncthreads();
  }
  if (k.top_cnv == -1 && k.bot_cnv == -1 && !k.mms) {
    double si = 0, sd = 0;
    for (int u = threadIdx.x; u < g.NU; u += blockDim.x) {
      const int j = u % (g.Nz + 2);
      if (j >= 1 && j <= g.Nz) {
        si += (double)vel_inertia_u<T>(g, op, u);
        sd += (double)vel_diag<T>(g, k, op, g.NW + u);
      }
    }
    si = cta_sum(si, red);
    sd = cta_sum(sd, red);
    if (threadIdx.x == 0 && si <= 1e-6 * sd) sok = 0;
  }
  __syncthreads();
  gj_invert_cta<T>(M, n, piv, &sok, fcol, red);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) inv[e] = M[e];
  if (threadIdx.x == 0) *ok = sok;
}

// ---------------------------------------------------------------------------
// pressure (Schur) multigrid on interior cells: periodic x, no flux in z
// (L p)_c = sum_faces k_f (p_c - p_n) + dpin p_pin
// kx[j,i]: face left of cell (j,i) (periodic); kz[j,i]: face above (kz[0]=kz[Nz]=0)
// ---------------------------------------------------------------------------
// (L p)(j, i) with p(j', i') supplied by pv -- a stored array or values formed
// on the fly by the fused kernels below; one body, so both give the same bits
template <typename T, typename PV>
__device__ __forceinline__ T p_apply_fn(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz,
                                        int pin, T dpin, PV pv, int j, int i, T* diag) {
  size_t c = (size_t)i * Nz + j;
  int il = i == 0 ? Nx - 1 : i - 1, ir = i == Nx - 1 ? 0 : i + 1;
  T kl = kx[c], kr = kx[(size_t)ir * Nz + j];
  T kt = kz[(size_t)i * (Nz + 1) + j], kb = kz[(size_t)i * (Nz + 1) + j + 1];
  T pc = pv(j, i);
  T s = add_rn<T>(mul_rn<T>(kl, pc - pv(j, il)), mul_rn<T>(kr, pc - pv(j, ir)));
  if (j > 0) s = add_rn<T>(s, mul_rn<T>(kt, pc - pv(j - 1, i)));
  if (j < Nz - 1) s = add_rn<T>(s, mul_rn<T>(kb, pc - pv(j + 1, i)));
  T d = kl + kr + (j > 0 ? kt : (T)0) + (j < Nz - 1 ? kb : (T)0);
  if ((int)c == pin) { s = add_rn<T>(s, mul_rn<T>(dpin, pc)); d += dpin; }
  *diag = d;
  return s;
}
template <typename T>
__device__ __forceinline__ T p_apply_at(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz,
                                        int pin, T dpin, const T* p, int j, int i, T* diag) {
  return p_apply_fn<T>(Nz, Nx, kx, kz, pin, dpin, [=](int jj, int ii) { return p[(size_t)ii * Nz + jj]; }, j, i,
                       diag);
}
// the first Jacobi sweep from zero at one cell: omega b / d
template <typename T>
__device__ __forceinline__ T p_jacobi0_val(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz,
                                           int pin, T dpin, const T* b, T omega, int j, int i) {
  T d;
  p_apply_fn<T>(Nz, Nx, kx, kz, pin, dpin, [](int, int) { return (T)0; }, j, i, &d);   // only the diagonal
  return d > (T)0 ? sdiv<T>(omega * b[(size_t)i * Nz + j], d) : (T)0;
}

template <typename T>
__device__ __forceinline__ void p_jacobi_at(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz,
                                            int pin, T dpin, const T* xi, const T* b, T* xo, T omega,
                                            int zero_init, int t) {
  int j = t % Nz, i = t / Nz;
  T d;
  if (zero_init) {
    xo[t] = p_jacobi0_val<T>(Nz, Nx, kx, kz, pin, dpin, b, omega, j, i);
    return;
  }
  T ax = p_apply_at<T>(Nz, Nx, kx, kz, pin, dpin, xi, j, i, &d);
  xo[t] = d > (T)0 ? xi[t] + sdiv<T>(omega * (b[t] - ax), d) : (T)0;
}
template <typename T>
__global__ void p_jacobi_kernel(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin,
                                T dpin, const T* __restrict__ xi, const T* __restrict__ b, T* xo, T omega,
                                int zero_init) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Nz * Nx) return;
  p_jacobi_at<T>(Nz, Nx, kx, kz, pin, dpin, xi, b, xo, omega, zero_init, t);
}

template <typename T>
__device__ __forceinline__ void p_residual_at(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz,
                                              int pin, T dpin, const T* x, const T* b, T* r, int t) {
  T d;
  r[t] = b[t] - p_apply_at<T>(Nz, Nx, kx, kz, pin, dpin, x, t % Nz, t / Nz, &d);
}
template <typename T>
__global__ void p_residual_kernel(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin,
                                  T dpin, const T* __restrict__ x, const T* __restrict__ b, T* r) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Nz * Nx) return;
  p_residual_at<T>(Nz, Nx, kx, kz, pin, dpin, x, b, r, t);
}

template <typename T>
__device__ __forceinline__ void p_restrict_at(int Nzc, int Nxc, const T* r, T* bc, int t) {
  int J = t % Nzc, I = t / Nzc;
  const int Nz = 2 * Nzc;
  size_t a = (size_t)(2 * I) * Nz + 2 * J, b = (size_t)(2 * I + 1) * Nz + 2 * J;
  bc[t] = (T)0.25 * (r[a] + r[a + 1] + r[b] + r[b + 1]);
}
template <typename T>
__global__ void p_restrict_kernel(int Nzc, int Nxc, const T* __restrict__ r, T* bc) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Nzc * Nxc) return;
  p_restrict_at<T>(Nzc, Nxc, r, bc, t);
}

// bilinear prolongation of the coarse correction to fine cell (j, i)
template <typename T>
__device__ __forceinline__ T p_prolong_val(int Nzc, int Nxc, const T* xc, int j, int i) {
  int J = j / 2, I = i / 2;
  int Jn = (j % 2 == 0) ? (J > 0 ? J - 1 : 0) : (J < Nzc - 1 ? J + 1 : Nzc - 1);
  int In = (i % 2 == 0) ? (I - 1 + Nxc) % Nxc : (I + 1) % Nxc;
  T v = add_rn<T>(add_rn<T>(add_rn<T>(mul_rn<T>((T)9, xc[(size_t)I * Nzc + J]), mul_rn<T>((T)3, xc[(size_t)I * Nzc + Jn])),
                            mul_rn<T>((T)3, xc[(size_t)In * Nzc + J])),
                  xc[(size_t)In * Nzc + Jn]);
  return mul_rn<T>(v, (T)0.0625);
}
template <typename T>
__device__ __forceinline__ void p_prolong_at(int Nzc, int Nxc, const T* xc, T* xf, int t) {
  const int Nz = 2 * Nzc;
  xf[t] = add_rn<T>(xf[t], p_prolong_val<T>(Nzc, Nxc, xc, t % Nz, t / Nz));
}
template <typename T>
__global__ void p_prolong_kernel(int Nzc, int Nxc, const T* __restrict__ xc, T* xf) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * Nzc * Nxc) return;
  p_prolong_at<T>(Nzc, Nxc, xc, xf, t);
}

// Fused descent of one pressure level (one thread per coarse cell): the
// residual b - L x of its four fine cells, restricted.  zero_init: x is the
// first Jacobi sweep from zero, formed on the fly at the cells the stencils
// read and stored at the thread's own four cells (pre-smoothing of one sweep).
// Same values as p_jacobi (from zero) + p_residual + p_restrict.
template <typename T>
__global__ void p_down_kernel(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin, T dpin,
                              T* x, const T* __restrict__ b, T* bc, T omega, int zero_init) {
  XC_PDL_WAIT();
  const int Nzc = Nz / 2, Nxc = Nx / 2;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Nzc * Nxc) return;
  const int J = t % Nzc, I = t / Nzc;
  T r[4];
  for (int q = 0; q < 4; ++q) {
    const int j = 2 * J + (q & 1), i = 2 * I + (q >> 1);
    T d;
    T ax;
    if (zero_init)
      ax = p_apply_fn<T>(Nz, Nx, kx, kz, pin, dpin,
                         [=](int jj, int ii) { return p_jacobi0_val<T>(Nz, Nx, kx, kz, pin, dpin, b, omega, jj, ii); },
                         j, i, &d);
    else
      ax = p_apply_at<T>(Nz, Nx, kx, kz, pin, dpin, x, j, i, &d);
    r[q] = b[(size_t)i * Nz + j] - ax;
  }
  if (zero_init)
    for (int q = 0; q < 4; ++q) {
      const int j = 2 * J + (q & 1), i = 2 * I + (q >> 1);
      x[(size_t)i * Nz + j] = p_jacobi0_val<T>(Nz, Nx, kx, kz, pin, dpin, b, omega, j, i);
    }
  // p_restrict_at's order: (2J, 2I), (2J+1, 2I), (2J, 2I+1), (2J+1, 2I+1)
  bc[t] = (T)0.25 * (r[0] + r[1] + r[2] + r[3]);
}

// Fused ascent (one thread per fine cell): the first post-smoothing Jacobi
// sweep of x + P xc, the coarse correction added on the fly at the cells the
// stencil reads; xo != x.  Same values as p_prolong + p_jacobi.
template <typename T>
__global__ void p_up_kernel(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin, T dpin,
                            const T* __restrict__ xc, const T* __restrict__ x, const T* __restrict__ b, T* xo,
                            T omega) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Nz * Nx) return;
  const int Nzc = Nz / 2, Nxc = Nx / 2;
  const int j = t % Nz, i = t / Nz;
  auto xv = [=](int jj, int ii) {
    return add_rn<T>(x[(size_t)ii * Nz + jj], p_prolong_val<T>(Nzc, Nxc, xc, jj, ii));
  };
  T d;
  T ax = p_apply_fn<T>(Nz, Nx, kx, kz, pin, dpin, xv, j, i, &d);
  xo[t] = d > (T)0 ? xv(j, i) + sdiv<T>(omega * (b[t] - ax), d) : (T)0;
}

template <typename T>
__global__ void p_coarsen_kernel(int Nzc, int Nxc, const T* __restrict__ kx, const T* __restrict__ kz,
                                 T* kxc, T* kzc) {
  XC_PDL_WAIT();
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  const int Nz = 2 * Nzc;
  if (J > Nzc || I >= Nxc) return;
  if (J < Nzc)
    kxc[(size_t)I * Nzc + J] = (kx[(size_t)(2 * I) * Nz + 2 * J] + kx[(size_t)(2 * I) * Nz + 2 * J + 1]) / (T)8;
  kzc[(size_t)I * (Nzc + 1) + J] = (kz[(size_t)(2 * I) * (Nz + 1) + 2 * J] +
                                    kz[(size_t)(2 * I + 1) * (Nz + 1) + 2 * J]) / (T)8;
}

template <typename T>
__device__ void p_coarse_cta(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin,
                             T dpin, T* x, T* x2, const T* b, int sweeps, T omega, const T* inv = nullptr,
                             const int* inv_ok = nullptr) {
  const int n = Nz * Nx;
  if (inv && *inv_ok) {
    dense_apply_cta<T>(inv, n, b, x);
    return;
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) x[t] = 0;
  __syncthreads();
  T* a = x;
  T* o = x2;
  for (int s = 0; s < sweeps; ++s) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      T d;
      T ax = p_apply_at<T>(Nz, Nx, kx, kz, pin, dpin, a, t % Nz, t / Nz, &d);
      o[t] = d > (T)0 ? a[t] + sdiv<T>(omega * (b[t] - ax), d) : (T)0;
    }
    __syncthreads();
    T* tmp = a; a = o; o = tmp;
  }
  if (a != x)
    for (int t = threadIdx.x; t < n; t += blockDim.x) x[t] = a[t];
  __syncthreads();
}
template <typename T>
__global__ void p_coarse_kernel(int Nz, int Nx, const T* __restrict__ kx, const T* __restrict__ kz, int pin,
                                T dpin, T* x, T* x2, const T* __restrict__ b, int sweeps, T omega, const T* inv,
                                const int* inv_ok) {
  XC_PDL_WAIT();
  p_coarse_cta<T>(Nz, Nx, kx, kz, pin, dpin, x, x2, b, sweeps, omega, inv, inv_ok);
}

// the inverse of the coarsest pressure level (Nz Nx <= kDenseMax), one CTA
template <typename T>
__global__ void __launch_bounds__(256) p_dense_inv_kernel(int Nz, int Nx, const T* __restrict__ kx,
                                                           const T* __restrict__ kz, int pin, T dpin, T* inv, int* ok) {
  XC_PDL_WAIT();
  __shared__ T M[kDenseMax * kDenseMax];
  __shared__ T xb[kDenseBatch][kDenseMax];
  __shared__ T fcol[kDenseMax];
  __shared__ double red[32];
  __shared__ int piv[kDenseMax];
  __shared__ int sok;
  const int n = Nz * Nx;
  if (threadIdx.x == 0) sok = 1;
  for (int c0 = 0; c0 < n; c0 += kDenseBatch) {
    for (int e = threadIdx.x; e < kDenseBatch * kDenseMax; e += blockDim.x) {
      const int bq = e / kDenseMax, r = e - bq * kDenseMax;
      xb[bq][r] = (T)(r == c0 + bq ? 1 : 0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kDenseBatch * n; e += blockDim.x) {
      const int bq = e / n, r = e - bq * n, c = c0 + bq;
      if (c >= n) continue;
      T d;
      M[r * n + c] = p_apply_at<T>(Nz, Nx, kx, kz, pin, dpin, xb[bq], r % Nz, r / Nz, &d);
    }
    __syncthreads();
  }
  gj_invert_cta<T>(M, n, piv, &sok, fcol, red);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) inv[e] = M[e];
  if (threadIdx.x == 0) *ok = sok;
}

// ---------------------------------------------------------------------------
// Small levels in one CTA.  A level of a few hundred cells is a few hundred
// unknowns, and each phase of its V-cycle (a smoothing sweep, the residual,
// the restriction, the prolongation) is bound by launch latency, not by
// bandwidth.  These kernels run the V-cycle from level l0 down to the coarsest
// level lc and back up inside one CTA, with CTA barriers between the phases;
// the level data stays in L1/L2.  Measured at 1024^2 against one launch per
// phase: handing the levels up to 16x16 to one CTA saves 3% of the solve; up
// to 64x64 it costs 6% (one CTA then streams too many rows per phase).
// ---------------------------------------------------------------------------
template <typename T>
struct VelLevels {
  Geo g[kMaxLevels];
  VOp<T> op[kMaxLevels];
  T* x[kMaxLevels];
  T* x2[kMaxLevels];
  T* b[kMaxLevels];
  T* r[kMaxLevels];
};

// `sweeps` damped-Jacobi sweeps (the first from zero when from_zero), x holds the result
template <typename T>
__device__ void vel_smooth_cta(const Geo& g, const OpConst& k, const VOp<T>& op, T* x, T* x2, const T* b, T om,
                               int sweeps, bool from_zero) {
  const long long n = (long long)g.NW + g.NU;
  T* a = x;
  T* o = x2;
  int q = 0;
  if (from_zero) {
    for (long long t = threadIdx.x; t < n; t += blockDim.x) vel_jacobi_at<T>(g, k, op, x, b, x, om, 1, t);
    __syncthreads();
    q = 1;
  }
  for (; q < sweeps; ++q) {
    for (long long t = threadIdx.x; t < n; t += blockDim.x) vel_jacobi_at<T>(g, k, op, a, b, o, om, 0, t);
    __syncthreads();
    T* tmp = a; a = o; o = tmp;
  }
  if (a != x) {
    for (long long t = threadIdx.x; t < n; t += blockDim.x) x[t] = a[t];
    __syncthreads();
  }
}

// the MMS pins (k.mms) belong to level 0 only
__host__ __device__ __forceinline__ OpConst level_const(const OpConst& k, int l) {
  OpConst c = k;
  if (l > 0) c.mms = 0;
  return c;
}

// Shared-memory staging of the one-CTA V-cycles.  The small levels are a few
// hundred unknowns each, and every sweep of them is a chain of dependent loads
// separated by CTA barriers: from shared memory instead of L2 each sweep costs
// a fraction of the latency.  Arrays are carved in a fixed order, each rounded
// up to 16 bytes; the host sizes the dynamic allocation with the same counts.
template <typename T>
__host__ __device__ __forceinline__ long long smem_round(long long c) {
  constexpr long long q = 16 / sizeof(T);
  return (c + q - 1) / q * q;
}
template <typename T>
__host__ __device__ inline long long vel_stage_elems(const Geo* gs, int l0, int lc) {
  long long e = 0;
  for (int q = l0; q <= lc; ++q) {
    const Geo& g = gs[q];
    if (kFly<T>)
      e += smem_round<T>((long long)g.Nz * g.Nx) + smem_round<T>((long long)(g.Nz + 1) * (g.Nx + 1)) +
           smem_round<T>(g.NW) + smem_round<T>(g.NU) + smem_round<T>(3LL * (g.Nx + 2));
    else
      e += smem_round<T>(10LL * g.NW) + smem_round<T>(10LL * g.NU);
    e += 4 * smem_round<T>((long long)g.NW + g.NU);
  }
  return e;
}
template <typename T>
__device__ __forceinline__ void cta_copy(T* dst, const T* src, long long n) {
  for (long long t = threadIdx.x; t < n; t += blockDim.x) dst[t] = src[t];
}
constexpr size_t kStageMaxBytes = 160 * 1024;

// the V-cycle of levels l0..lc (lc the coarsest) by one CTA: nu sweeps
// before and after each coarse correction, the coarsest solved directly
template <typename T>
__device__ void vel_vcycle_cta(const VelLevels<T>& L, const OpConst& kf, int l0, int lc, int nu, T om, int csweeps,
                               const T* inv, const int* inv_ok) {
  for (int l = l0; l < lc; ++l) {
    const OpConst k = level_const(kf, l);
    const Geo& g = L.g[l];
    const Geo& c = L.g[l + 1];
    vel_smooth_cta<T>(g, k, L.op[l], L.x[l], L.x2[l], L.b[l], om, nu, true);
    const long long n = (long long)g.NW + g.NU;
    for (long long t = threadIdx.x; t < n; t += blockDim.x)
      vel_residual_at<T>(g, k, L.op[l], L.x[l], L.b[l], L.r[l], t);
    __syncthreads();
    const long long nc = (long long)c.NW + c.NU;
    for (long long t = threadIdx.x; t < nc; t += blockDim.x) vel_restrict_at<T>(g, c, L.r[l], L.b[l + 1], t);
    __syncthreads();
  }
  vel_coarse_cta<T>(L.g[lc], level_const(kf, lc), L.op[lc], L.x[lc], L.x2[lc], L.b[lc], csweeps, om, inv, inv_ok);
  for (int l = lc - 1; l >= l0; --l) {
    const OpConst k = level_const(kf, l);
    const Geo& g = L.g[l];
    const long long n = (long long)g.NW + g.NU;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) vel_prolong_at<T>(g, L.g[l + 1], k, L.x[l + 1], L.x[l], t);
    __syncthreads();
    vel_smooth_cta<T>(g, k, L.op[l], L.x[l], L.x2[l], L.b[l], om, nu, false);
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) vel_vcycle_small_kernel(VelLevels<T> Lg, OpConst kf, int l0, int lc, int nu,
                                                                T om, int csweeps, int staged, const T* inv,
                                                                const int* inv_ok) {
  XC_PDL_WAIT();
  extern __shared__ __align__(16) unsigned char xc_stage[];
  __shared__ VelLevels<T> L;
  if (threadIdx.x == 0) {
    T* p = reinterpret_cast<T*>(xc_stage);
    for (int q = l0; q <= lc; ++q) {
      const Geo& g = Lg.g[q];
      L.g[q] = g; L.op[q] = Lg.op[q];
      L.x[q] = Lg.x[q]; L.x2[q] = Lg.x2[q]; L.b[q] = Lg.b[q]; L.r[q] = Lg.r[q];
      if (!staged) continue;
      if constexpr (kFly<T>) {
        L.op[q].eta = p; p += smem_round<T>((long long)g.Nz * g.Nx);
        L.op[q].etaco = p; p += smem_round<T>((long long)(g.Nz + 1) * (g.Nx + 1));
        L.op[q].dw = p; p += smem_round<T>(g.NW);
        L.op[q].du = p; p += smem_round<T>(g.NU);
        L.op[q].dbot = p; p += smem_round<T>(3LL * (g.Nx + 2));
      } else {
        L.op[q].cw = p; p += smem_round<T>(10LL * g.NW);
        L.op[q].cu = p; p += smem_round<T>(10LL * g.NU);
      }
      const long long nvv = (long long)g.NW + g.NU;
      L.x[q] = p; p += smem_round<T>(nvv);
      L.x2[q] = p; p += smem_round<T>(nvv);
      L.b[q] = p; p += smem_round<T>(nvv);
      L.r[q] = p; p += smem_round<T>(nvv);
    }
  }
  __syncthreads();
  if (staged) {
    for (int q = l0; q <= lc; ++q) {
      const Geo& g = L.g[q];
      if constexpr (kFly<T>) {
        cta_copy<T>(const_cast<T*>(L.op[q].eta), Lg.op[q].eta, (long long)g.Nz * g.Nx);
        cta_copy<T>(const_cast<T*>(L.op[q].etaco), Lg.op[q].etaco, (long long)(g.Nz + 1) * (g.Nx + 1));
        cta_copy<T>(const_cast<T*>(L.op[q].dw), Lg.op[q].dw, g.NW);
        cta_copy<T>(const_cast<T*>(L.op[q].du), Lg.op[q].du, g.NU);
        cta_copy<T>(const_cast<T*>(L.op[q].dbot), Lg.op[q].dbot, 3LL * (g.Nx + 2));
      } else {
        cta_copy<T>(const_cast<T*>(L.op[q].cw), Lg.op[q].cw, 10LL * g.NW);
        cta_copy<T>(const_cast<T*>(L.op[q].cu), Lg.op[q].cu, 10LL * g.NU);
      }
    }
    cta_copy<T>(L.b[l0], Lg.b[l0], (long long)L.g[l0].NW + L.g[l0].NU);
    __syncthreads();
  }
  vel_vcycle_cta<T>(L, kf, l0, lc, nu, om, csweeps, inv, inv_ok);
  if (staged) cta_copy<T>(Lg.x[l0], L.x[l0], (long long)L.g[l0].NW + L.g[l0].NU);
}


// ---- thread-block-cluster V-cycle of the middle levels ---------------------
// Levels of up to a few ten thousand cells are too small to fill the GPU and
// each of their operations costs a launch; one cluster of CTAs (16 where the
// GPU allows, else 8) runs all of them in one launch, the CTAs dividing each
// level's unknowns and meeting at cluster barriers between the operations
// (the barrier's release / acquire makes every global-memory write before it
// visible to the whole cluster after it).  The operations are the per-unknown
// bodies of the separate launches, so the results are the same.  The levels
// below the one-CTA size are then handled by CTA 0 alone, as the one-CTA
// kernel would.  Every loop bound is uniform across the cluster and no thread
// leaves early, so every thread reaches every barrier.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank_u32() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size_u32() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

// vel_smooth_cta over the cluster (unknowns t0, t0 + ts, ...)
template <typename T>
__device__ void vel_smooth_cluster(const Geo& g, const OpConst& k, const VOp<T>& op, T* x, T* x2, const T* b, T om,
                                   int sweeps, bool from_zero, long long t0, long long ts) {
  const long long n = (long long)g.NW + g.NU;
  T* a = x;
  T* o = x2;
  int q = 0;
  if (from_zero) {
    for (long long t = t0; t < n; t += ts) vel_jacobi_at<T>(g, k, op, x, b, x, om, 1, t);
    cluster_barrier();
    q = 1;
  }
  for (; q < sweeps; ++q) {
    for (long long t = t0; t < n; t += ts) vel_jacobi_at<T>(g, k, op, a, b, o, om, 0, t);
    cluster_barrier();
    T* tmp = a; a = o; o = tmp;
  }
  if (a != x) {
    for (long long t = t0; t < n; t += ts) x[t] = a[t];
    cluster_barrier();
  }
}

// levels l0..ls-1 over the cluster (nu sweeps before, nu_post after each
// coarse correction, as the per-level launches do), ls..lc by CTA 0
template <typename T>
__global__ void __launch_bounds__(1024) vel_vcycle_cluster_kernel(VelLevels<T> Lg, OpConst kf, int l0, int ls, int lc,
                                                                  int nu, int nu_post, T om, int csweeps,
                                                                  const T* inv, const int* inv_ok) {
  XC_PDL_WAIT();
  __shared__ VelLevels<T> L;
  if (threadIdx.x == 0) L = Lg;
  __syncthreads();
  const unsigned rank = cluster_rank_u32();
  const long long t0 = (long long)rank * blockDim.x + threadIdx.x;
  const long long ts = (long long)cluster_size_u32() * blockDim.x;
  for (int l = l0; l < ls; ++l) {
    const OpConst k = level_const(kf, l);
    const Geo& g = L.g[l];
    const Geo& c = L.g[l + 1];
    vel_smooth_cluster<T>(g, k, L.op[l], L.x[l], L.x2[l], L.b[l], om, nu, true, t0, ts);
    const long long n = (long long)g.NW + g.NU;
    for (long long t = t0; t < n; t += ts) vel_residual_at<T>(g, k, L.op[l], L.x[l], L.b[l], L.r[l], t);
    cluster_barrier();
    const long long nc = (long long)c.NW + c.NU;
    for (long long t = t0; t < nc; t += ts) vel_restrict_at<T>(g, c, L.r[l], L.b[l + 1], t);
    cluster_barrier();
  }
  if (rank == 0) vel_vcycle_cta<T>(L, kf, ls, lc, nu, om, csweeps, inv, inv_ok);
  cluster_barrier();
  for (int l = ls - 1; l >= l0; --l) {
    const OpConst k = level_const(kf, l);
    const Geo& g = L.g[l];
    const long long n = (long long)g.NW + g.NU;
    for (long long t = t0; t < n; t += ts) vel_prolong_at<T>(g, L.g[l + 1], k, L.x[l + 1], L.x[l], t);
    cluster_barrier();
    vel_smooth_cluster<T>(g, k, L.op[l], L.x[l], L.x2[l], L.b[l], om, nu_post, false, t0, ts);
  }
}

template <typename T>
struct PLevels {
  int Nz[kMaxLevels], Nx[kMaxLevels], pin[kMaxLevels];
  T dpin[kMaxLevels];
  const T* kx[kMaxLevels];
  const T* kz[kMaxLevels];
  T* x[kMaxLevels];
  T* x2[kMaxLevels];
  T* b[kMaxLevels];
  T* r[kMaxLevels];
};

template <typename T>
__device__ void p_smooth_cta(const PLevels<T>& L, int l, T om, int sweeps, bool from_zero) {
  const int Nz = L.Nz[l], Nx = L.Nx[l], n = Nz * Nx;
  T* x = L.x[l];
  T* a = x;
  T* o = L.x2[l];
  int q = 0;
  if (from_zero) {
    for (int t = threadIdx.x; t < n; t += blockDim.x)
      p_jacobi_at<T>(Nz, Nx, L.kx[l], L.kz[l], L.pin[l], L.dpin[l], x, L.b[l], x, om, 1, t);
    __syncthreads();
    q = 1;
  }
  for (; q < sweeps; ++q) {
    for (int t = threadIdx.x; t < n; t += blockDim.x)
      p_jacobi_at<T>(Nz, Nx, L.kx[l], L.kz[l], L.pin[l], L.dpin[l], a, L.b[l], o, om, 0, t);
    __syncthreads();
    T* tmp = a; a = o; o = tmp;
  }
  if (a != x) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) x[t] = a[t];
    __syncthreads();
  }
}

template <typename T>
__host__ __device__ inline long long p_stage_elems(const int* Nzs, const int* Nxs, int l0, int lc) {
  long long e = 0;
  for (int q = l0; q <= lc; ++q) {
    const long long n = (long long)Nzs[q] * Nxs[q];
    e += 5 * smem_round<T>(n) + smem_round<T>((long long)(Nzs[q] + 1) * Nxs[q]);
  }
  return e;
}
template <typename T>
__global__ void __launch_bounds__(1024) p_vcycle_small_kernel(PLevels<T> Lg, int l0, int lc, int nu, T om,
                                                              int csweeps, int staged, const T* inv,
                                                              const int* inv_ok) {
  XC_PDL_WAIT();
  extern __shared__ __align__(16) unsigned char xc_stage[];
  __shared__ PLevels<T> L;
  if (threadIdx.x == 0) {
    T* p = reinterpret_cast<T*>(xc_stage);
    for (int q = l0; q <= lc; ++q) {
      L.Nz[q] = Lg.Nz[q]; L.Nx[q] = Lg.Nx[q]; L.pin[q] = Lg.pin[q]; L.dpin[q] = Lg.dpin[q];
      L.kx[q] = Lg.kx[q]; L.kz[q] = Lg.kz[q];
      L.x[q] = Lg.x[q]; L.x2[q] = Lg.x2[q]; L.b[q] = Lg.b[q]; L.r[q] = Lg.r[q];
      if (!staged) continue;
      const long long n = (long long)Lg.Nz[q] * Lg.Nx[q];
      L.kx[q] = p; p += smem_round<T>(n);
      L.kz[q] = p; p += smem_round<T>((long long)(Lg.Nz[q] + 1) * Lg.Nx[q]);
      L.x[q] = p; p += smem_round<T>(n);
      L.x2[q] = p; p += smem_round<T>(n);
      L.b[q] = p; p += smem_round<T>(n);
      L.r[q] = p; p += smem_round<T>(n);
    }
  }
  __syncthreads();
  if (staged) {
    for (int q = l0; q <= lc; ++q) {
      cta_copy<T>(const_cast<T*>(L.kx[q]), Lg.kx[q], (long long)L.Nz[q] * L.Nx[q]);
      cta_copy<T>(const_cast<T*>(L.kz[q]), Lg.kz[q], (long long)(L.Nz[q] + 1) * L.Nx[q]);
    }
    cta_copy<T>(L.b[l0], Lg.b[l0], (long long)L.Nz[l0] * L.Nx[l0]);
    __syncthreads();
  }
  for (int l = l0; l < lc; ++l) {
    const int Nz = L.Nz[l], Nx = L.Nx[l], n = Nz * Nx;
    p_smooth_cta<T>(L, l, om, nu, true);
    for (int t = threadIdx.x; t < n; t += blockDim.x)
      p_residual_at<T>(Nz, Nx, L.kx[l], L.kz[l], L.pin[l], L.dpin[l], L.x[l], L.b[l], L.r[l], t);
    __syncthreads();
    const int nc = L.Nz[l + 1] * L.Nx[l + 1];
    for (int t = threadIdx.x; t < nc; t += blockDim.x) p_restrict_at<T>(L.Nz[l + 1], L.Nx[l + 1], L.r[l], L.b[l + 1], t);
    __syncthreads();
  }
  p_coarse_cta<T>(L.Nz[lc], L.Nx[lc], L.kx[lc], L.kz[lc], L.pin[lc], L.dpin[lc], L.x[lc], L.x2[lc], L.b[lc],
                  csweeps, om, inv, inv_ok);
  for (int l = lc - 1; l >= l0; --l) {
    const int n = L.Nz[l] * L.Nx[l];
    for (int t = threadIdx.x; t < n; t += blockDim.x) p_prolong_at<T>(L.Nz[l + 1], L.Nx[l + 1], L.x[l + 1], L.x[l], t);
    __syncthreads();
    p_smooth_cta<T>(L, l, om, nu, false);
  }
  if (staged) cta_copy<T>(Lg.x[l0], L.x[l0], (long long)L.Nz[l0] * L.Nx[l0]);
}

// fine-level pressure coefficients from the velocity diagonal (plane 0: full,
// plane 9: inertia only) -- k = rho_face / (h^2 A_ff)
template <typename T>
__global__ void p_kcoef_kernel(Geo g, const double* __restrict__ rhow, const double* __restrict__ rhou,
                               const double* __restrict__ cw, const double* __restrict__ cu, int plane, T* kx,
                               T* kz, T* kr) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Nz = g.Nz, Nx = g.Nx;
  const double ih2 = g.invh * g.invh;
  // k = rho_face / (h^2 a) with a the chosen diagonal; 0 where the inertial
  // diagonal is negligible against the full one (a Stokes limit, e.g. MMS)
  auto kval = [&](double rho_f, double a, double full) -> T {
    if (!(a > 1e-12 * fabs(full))) return (T)0;
    return (T)(rho_f * ih2 / a);
  };
  if (t < Nz * Nx) {
    int j = t % Nz, i = t / Nz;
    // face left of cell (j,i) is U(j+1, i)
    size_t o = (size_t)i * (Nz + 2) + j + 1;
    kx[t] = kval(rhou[(size_t)i * Nz + j], (double)cu[(size_t)plane * g.NU + o], (double)cu[o]);
    if (i == Nx - 1) {    // right face of the last column is U(j+1, Nx)
      size_t orr = (size_t)Nx * (Nz + 2) + j + 1;
      kr[j] = kval(rhou[(size_t)Nx * Nz + j], (double)cu[(size_t)plane * g.NU + orr], (double)cu[orr]);
    }
  }
  if (t < (Nz + 1) * Nx) {
    int j = t % (Nz + 1), i = t / (Nz + 1);
    T v = 0;
    if (j >= 1 && j <= Nz - 1) {
      size_t o = (size_t)(i + 1) * (Nz + 1) + j;
      v = kval(rhow[(size_t)i * (Nz + 1) + j], (double)cw[(size_t)plane * g.NW + o], (double)cw[o]);
    }
    kz[t] = v;
  }
}

// pressure part of the preconditioner, before / after the interior solve:
// ghost elimination of the residual (P ghost rows P_g - P_n = r_g) and the
// ghost values of the result (P_g = r_g + P_neighbour, fluidmech.jl:403-417).
// The physical pressure residual r = v_p / scl_p is formed where it is read
// (no r array, no separate division pass), and the interior cells, ghost
// columns and ghost rows are written by one launch: a ghost entry recomputes
// the interior or ghost-column value it copies with the same operations (the
// ghost rows of columns 0 and Nx+1 read ghost-column values).
template <typename T>
__global__ void p_gather_fused_kernel(Geo g, const T* __restrict__ kx, const T* __restrict__ kr,
                                      const T* __restrict__ vp, const T* __restrict__ sp, T* rin) {
  XC_PDL_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Nz = g.Nz, Nx = g.Nx, lp = Nz + 2;
  if (t >= Nz * Nx) return;
  int j = t % Nz, i = t / Nz;
  const size_t o = (size_t)(i + 1) * lp + j + 1;
  T v = vp[o] / sp[o];
  if (i == 0) v += kx[j] * (vp[j + 1] / sp[j + 1]);
  if (i == Nx - 1) {
    const size_t q = (size_t)(Nx + 1) * lp + j + 1;
    v += kr[j] * (vp[q] / sp[q]);
  }
  rin[t] = v;
}

template <typename T>
__global__ void p_scatter_fused_kernel(Geo g, const T* __restrict__ z, const T* __restrict__ vp,
                                       const T* __restrict__ sp, const T* __restrict__ etarho, T cmass,
                                       int open_bottom, T* zp) {
  XC_PDL_WAIT();
  const int Nz = g.Nz, Nx = g.Nx, lp = Nz + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lp * (Nx + 2)) return;
  const int j = t % lp, i = t / lp;
  auto r = [&](int jj, int ii) {
    const size_t o = (size_t)ii * lp + jj;
    return vp[o] / sp[o];
  };
  auto zint = [&](int jj, int ii) {   // interior cell (1..Nz, 1..Nx)
    const int c = (ii - 1) * Nz + (jj - 1);
    return z[c] + cmass * etarho[c] * r(jj, ii);
  };
  auto zcol = [&](int jj, int ii) {   // ghost column ii = 0 or Nx+1, rows 1..Nz
    if (open_bottom && jj == Nz) return r(jj, ii);   // P = 0 rows of the open bottom
    return r(jj, ii) + zint(jj, ii == 0 ? Nx : 1);
  };
  T out;
  const bool col_in = i >= 1 && i <= Nx;
  if (j >= 1 && j <= Nz) out = col_in ? zint(j, i) : zcol(j, i);
  else if (j == 0) out = r(0, i) + (col_in ? zint(1, i) : zcol(1, i));
  else out = r(Nz + 1, i) + (col_in ? zint(Nz, i) : zcol(Nz, i));
  zp[t] = out;
}

// velocity right-hand side of the preconditioner: rv = S^-1 v - GG z_p on the
// interior velocity rows (fluidmech.jl:343-356), S^-1 v elsewhere -- the
// unscaling of the residual fused with the gradient of the pressure part
template <typename T>
__global__ void sub_grad_kernel(Geo g, const T* __restrict__ zp, const T* __restrict__ v,
                                const T* __restrict__ scl, T* rv) {
  XC_PDL_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Nz = g.Nz, Nx = g.Nx, lw = Nz + 1, lu = Nz + 2;
  if (t >= g.NW + g.NU) return;
  T r = v[t] / scl[t];
  if (t < g.NW) {
    const int j = t % lw, i = t / lw;
    if (j >= 1 && j <= Nz - 1 && i >= 1 && i <= Nx) r -= geo_invh<T>(g) * (zp[i * lu + j + 1] - zp[i * lu + j]);
  } else {
    const int u = t - g.NW, j = u % lu, i = u / lu;
    if (j >= 1 && j <= Nz) r -= geo_invh<T>(g) * (zp[(i + 1) * lu + j] - zp[i * lu + j]);
  }
  rv[t] = r;
}

// ---------------------------------------------------------------------------
// Krylov vector kernels
// ---------------------------------------------------------------------------
constexpr int KB = 256;
constexpr int KGMAX = 8 * kNumSMs;   // partial-sum slots: at most 8 CTAs of 256 threads per SM

// partial dot products of w with V[0..m) -> part[blk * m + k], m <= MAXK.
// One pass: w is read once, every thread keeps m running sums in the working
// precision T (FP32 for the inner solver -- FP64 arithmetic is 58x slower on
// GB300), then warps and the CTA combine them in FP64.  MAXK (8, 16, 32) is
// picked by the host so that few accumulators keep the occupancy high; the
// grid-stride loop takes two elements per step for more loads in flight.
// EXACT: m == MAXK (instantiated for 1..8 basis vectors), so no accumulator
// slot is predicated off -- a predicated-off FP64 FMA still takes an issue
// slot on GB300's narrow FP64 pipe; otherwise m <= MAXK
template <typename T, int MAXK, bool EXACT = false>
__global__ void __launch_bounds__(KB) multidot_kernel(long long n, int m, const T* __restrict__ V, long long ldv,
                                                      const T* __restrict__ w, double* part) {
  XC_PDL_WAIT();
  __shared__ double sh[KB / 32][MAXK];
  T acc[MAXK];
#pragma unroll
  for (int k = 0; k < MAXK; ++k) acc[k] = (T)0;
  const long long stride = (long long)gridDim.x * KB;
  long long t = blockIdx.x * (long long)KB + threadIdx.x;
  for (; t + stride < n; t += 2 * stride) {
    const T w0 = w[t], w1 = w[t + stride];
#pragma unroll
    for (int k = 0; k < MAXK; ++k)
      if (EXACT || k < m) {
        const T* vk = V + (size_t)k * ldv;
        acc[k] += vk[t] * w0;
        acc[k] += vk[t + stride] * w1;
      }
  }
  if (t < n) {
    const T w0 = w[t];
#pragma unroll
    for (int k = 0; k < MAXK; ++k)
      if (EXACT || k < m) acc[k] += V[(size_t)k * ldv + t] * w0;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the warp's 32 partial sums are added in the working precision (in FP64
  // each would cost a conversion and five additions on the narrow FP64 pipe
  // per thread); warps and CTAs are combined in FP64
#pragma unroll
  for (int k = 0; k < MAXK; ++k) {
    if (EXACT || k < m) {
      T v = acc[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) sh[warp][k] = (double)v;
    }
  }
  __syncthreads();
  if (threadIdx.x < m) {
    double s = 0;
    for (int q = 0; q < KB / 32; ++q) s += sh[q][threadIdx.x];
    part[(size_t)blockIdx.x * m + threadIdx.x] = s;
  }
}
__global__ void multidot_final_kernel(int m, int nb, const double* __restrict__ part, double* out) {
  XC_PDL_WAIT();
  int k = blockIdx.x;
  __shared__ double sh[KB];
  double acc = 0;
  for (int b = threadIdx.x; b < nb; b += KB) acc += part[(size_t)b * m + k];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = KB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[k] = sh[0];
}
// ||v||^2 from one partial column -> *nrm2, and 1/||v|| (1 for a zero norm) -> *inv
__global__ void norm_final_kernel(int nb, const double* __restrict__ part, double* nrm2, double* inv) {
  XC_PDL_WAIT();
  __shared__ double sh[KB];
  double acc = 0;
  for (int b = threadIdx.x; b < nb; b += KB) acc += part[b];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = KB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *nrm2 = sh[0];
    *inv = sh[0] > 0.0 ? 1.0 / sqrt(sh[0]) : 1.0;
  }
}
// w -= sum_k h[k] V[k] and ||w||^2 in the same pass: per-CTA partial sums
// (working precision per thread and warp, FP64 across warps) to part[blk],
// combined by norm_final_kernel.  Grid-stride over a grid of at most KGMAX
// CTAs, so the partials fit the multi-dot scratch.
template <typename T>
__global__ void __launch_bounds__(KB) multiaxpy_norm_kernel(long long n, int m, const T* __restrict__ V,
                                                            long long ldv, const double* __restrict__ h, T* w,
                                                            double* part) {
  XC_PDL_WAIT();
  __shared__ T hs[32];
  __shared__ double sh[KB / 32];
  if (threadIdx.x < m) hs[threadIdx.x] = (T)h[threadIdx.x];
  __syncthreads();
  T acc = (T)0;
  const long long stride = (long long)gridDim.x * KB;
  for (long long t = blockIdx.x * (long long)KB + threadIdx.x; t < n; t += stride) {
    T s = w[t];
    const T* vk = V + t;
    for (int k = 0; k < m; ++k, vk += ldv) s -= hs[k] * *vk;
    w[t] = s;
    acc += s * s;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = sh[0];
    for (int q = 1; q < KB / 32; ++q) r += sh[q];
    part[blockIdx.x] = r;
  }
}
// w -= sum_k h[k] V[k]
template <typename T>
__global__ void multiaxpy_kernel(long long n, int m, const T* __restrict__ V, long long ldv,
                                 const double* __restrict__ h, T* w) {
  XC_PDL_WAIT();
  __shared__ T hs[32];
  if (threadIdx.x < m) hs[threadIdx.x] = (T)h[threadIdx.x];
  __syncthreads();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  T s = w[t];
  const T* vk = V + t;
  for (int k = 0; k < m; ++k, vk += ldv) s -= hs[k] * *vk;
  w[t] = s;
}
// sum_k y[k] zk[k * ldz] with four independent partial sums, so the loads of
// four basis vectors are in flight at once (a single running sum over a
// runtime-length loop issued them one after another)
template <typename T>
__device__ __forceinline__ T combine_sum(const T* ys, int m, const T* zk, long long ldz) {
  T a0 = (T)0, a1 = (T)0, a2 = (T)0, a3 = (T)0;
  int k = 0;
  for (; k + 4 <= m; k += 4, zk += 4 * ldz) {
    a0 += ys[k] * zk[0];
    a1 += ys[k + 1] * zk[ldz];
    a2 += ys[k + 2] * zk[2 * ldz];
    a3 += ys[k + 3] * zk[3 * ldz];
  }
  for (; k < m; ++k, zk += ldz) a0 += ys[k] * *zk;
  return (a0 + a1) + (a2 + a3);
}
// x += sum_k y[k] Z[k], or with dscl: x += (sum_k y[k] Z[k]) / dscl (the
// basis held in physical variables, Z[k] = S z_k of the scaled system)
template <typename T>
__global__ void combine_kernel(long long n, int m, const T* __restrict__ Z, long long ldz,
                               const double* __restrict__ y, T* x, const T* __restrict__ dscl) {
  XC_PDL_WAIT();
  __shared__ T ys[64];
  if (threadIdx.x < m) ys[threadIdx.x] = (T)y[threadIdx.x];
  __syncthreads();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const T* zk = Z + t;
  if (dscl) {
    x[t] += combine_sum<T>(ys, m, zk, ldz) / dscl[t];
    return;
  }
  T s = x[t];
  for (int k = 0; k < m; ++k, zk += ldz) s += ys[k] * *zk;
  x[t] = s;
}
// v = w * inv with a scale factor computed once elsewhere (a per-CTA FP64
// reciprocal in front of a barrier stalls every CTA of the grid).  The factor
// is converted to T once per CTA: a conversion from FP64 issues on GB300's
// narrow FP64 pipe, and one per element made these FP32 kernels FP64-bound.
template <typename T>
__global__ void scale_kernel(long long n, const double* __restrict__ inv, const T* __restrict__ w, T* v) {
  XC_PDL_WAIT();
  __shared__ T f;
  if (threadIdx.x == 0) f = (T)__ldg(inv);
  __syncthreads();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) v[t] = w[t] * f;
}
// v *= inv (inv = 1/||v|| from norm_final_kernel; 1 on a zero norm, which the
// host reports as breakdown)
template <typename T>
__global__ void normalize_kernel(long long n, const double* __restrict__ inv, T* v) {
  XC_PDL_WAIT();
  __shared__ T f;
  if (threadIdx.x == 0) f = (T)__ldg(inv);
  __syncthreads();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) v[t] = v[t] * f;
}

// ---------------------------------------------------------------------------
// RHS assembly
// ---------------------------------------------------------------------------
// momentum-advection inputs (fluidmech.jl:236-240, 310-314)
__global__ void mom_prep_kernel(int Nz, int Nx, CView W, CView U, CView rhow, CView rhou, double* fz,
                                double* uz, double* wz, double* fx, double* ux, double* wxm) {
  XC_PDL_WAIT();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  // z-momentum grid (Nz-1, Nx): f (Nz-1, Nx), u (Nz-1, Nx+1), w (Nz, Nx)
  if (j < Nz - 1 && i < Nx) fz[(size_t)i * (Nz - 1) + j] = AT(rhow, j + 1, i) * AT(W, j + 1, i + 1);
  if (j < Nz - 1 && i <= Nx) uz[(size_t)i * (Nz - 1) + j] = (AT(U, j + 1, i) + AT(U, j + 2, i)) / 2.0;
  if (j < Nz && i < Nx) wz[(size_t)i * Nz + j] = (AT(W, j, i + 1) + AT(W, j + 1, i + 1)) / 2.0;
  // x-momentum grid (Nz, Nx+1): f (Nz, Nx+1), u (Nz, Nx+2) with ifx, w (Nz+1, Nx+1)
  if (j < Nz && i <= Nx) fx[(size_t)i * Nz + j] = AT(rhou, j, i) * AT(U, j + 1, i);
  if (j < Nz && i <= Nx + 1) {
    int a = (i == 0) ? Nx - 1 : i - 1;          // ifx[i]
    int b = (i == Nx + 1) ? 1 : i;              // ifx[i+1]
    ux[(size_t)i * Nz + j] = (AT(U, j + 1, a) + AT(U, j + 1, b)) / 2.0;
  }
  if (j <= Nz && i <= Nx) wxm[(size_t)i * (Nz + 1) + j] = (AT(W, j, i) + AT(W, j, i + 1)) / 2.0;
}

struct RhsArgs {
  double a1, a2, a3, dt, g0, D, h, oc;
  double idt;   // 1 / dt
  int mms;
  int pin_p, pin_u;
};

__global__ void rhs_kernel(Geo g, RhsArgs a, CView Drho, CView rhoWo, CView rhoWoo, CView rhoUo, CView rhoUoo,
                           CView MFS, const double* __restrict__ advz, const double* __restrict__ advx,
                           const double* __restrict__ mfs_mean, const double* __restrict__ src_w,
                           const double* __restrict__ src_u, const double* __restrict__ src_p,
                           double pin_p_val, double pin_u_val, double* RR) {
  XC_PDL_WAIT();
  // 32-bit indices (the unknown count is checked below 2^31 at setup) and
  // the division by dt as a product with 1/dt: a 64-bit integer division and
  // an FP64 division per row were most of this kernel's time on GB300.  RR
  // is the solve's right-hand side only, so a last-bit difference in it is
  // far inside the solver's tolerance.
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int Nz = g.Nz, Nx = g.Nx;
  const int n = g.NW + g.NU + g.NP;
  if (t >= n) return;
  double v = 0.0;
  if (t < g.NW) {
    const int j = t % (Nz + 1), i = t / (Nz + 1);
    if (i >= 1 && i <= Nx) {
      if (j == Nz) {
        double mfbg = (*mfs_mean) * a.D / a.h;
        v = a.oc * AT(MFS, Nz - 1, i - 1) + (1.0 - a.oc) * mfbg;
      } else if (j >= 1) {
        v = (AT(Drho, j, i - 1) * a.g0 + (a.a2 * AT(rhoWo, j, i - 1) + a.a3 * AT(rhoWoo, j, i - 1)) * a.idt) -
            advz[(size_t)(i - 1) * (Nz - 1) + j - 1];
        if (a.mms) v = v + src_w[t];
      }
    }
  } else if (t < g.NW + g.NU) {
    const int u = t - g.NW;
    const int j = u % (Nz + 2), i = u / (Nz + 2);
    if (j >= 1 && j <= Nz) {
      double ad;
      if (i == 0 || i == Nx) ad = (advx[(size_t)j - 1] + advx[(size_t)Nx * Nz + j - 1]) / 2.0;
      else ad = advx[(size_t)i * Nz + j - 1];
      v = (a.a2 * AT(rhoUo, j - 1, i) + a.a3 * AT(rhoUoo, j - 1, i)) * a.idt - ad;
      if (a.mms) v = v + src_u[u];
      if (a.mms && u == a.pin_u) v = pin_u_val;
    }
  } else {
    const int p = t - g.NW - g.NU;
    const int j = p % (Nz + 2), i = p / (Nz + 2);
    if (j >= 1 && j <= Nz && i >= 1 && i <= Nx) {
      v = AT(MFS, j - 1, i - 1);
      if (a.mms) v = v + src_p[p];
    }
    if (a.mms && p == a.pin_p) v = pin_p_val;
  }
  RR[t] = v;
}

// MFS update (fluidmech.jl:115-126); explicit round-to-nearest intrinsics keep
// every product and sum separately rounded (no FMA contraction) so the state
// field MFS matches the reference arithmetic bit for bit
__global__ void mfs_kernel(int Nz, int Nx, double a1, double a2, double a3, double b1, double b2, double b3,
                           double dt, double alpha, CView rho, CView rhoo, CView rhooo, CView advn_rho,
                           DView drhodt, CView drhodto, CView drhodtoo, DView MFS) {
  XC_PDL_WAIT();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (j >= Nz || i >= Nx) return;
  double d = -AT(advn_rho, j, i);
  AT(drhodt, j, i) = d;
  double lhs = __dsub_rn(__dsub_rn(__dmul_rn(a1, AT(rho, j, i)), __dmul_rn(a2, AT(rhoo, j, i))),
                         __dmul_rn(a3, AT(rhooo, j, i)));
  double rhs = __dadd_rn(__dadd_rn(__dmul_rn(b1, d), __dmul_rn(b2, AT(drhodto, j, i))),
                         __dmul_rn(b3, AT(drhodtoo, j, i)));
  double res = __dsub_rn(__ddiv_rn(lhs, dt), rhs);
  AT(MFS, j, i) = __dsub_rn(AT(MFS, j, i), __dmul_rn(alpha, res));
}

// scl = 1 / (sqrt|diag LL| + extra) (fluidmech.jl:496-501)
__global__ void scl_kernel(Geo g, OpConst k, const double* __restrict__ cw, const double* __restrict__ cu,
                           CView rho, CView eta, double* scl, double* etarho) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = (long long)g.NW + g.NU + g.NP;
  if (t >= n) return;
  // scl = 1 / (sqrt|d| + sqrt(eta / rho)) (fluidmech.jl:496-501), with
  // sqrt(eta / rho) only on the pressure rows.  The velocity rows and the
  // interior pressure rows (d = 0) take one reciprocal square root, the
  // pressure rows one division: the scaling only conditions the solve, so
  // rounding differences in it move the solution by far less than the
  // solve's tolerance, and FP64 division and square root are slow here.
  double s;
  if (t < g.NW) s = rsqrt(fabs(cw[t]));
  else if (t < (long long)g.NW + g.NU) s = rsqrt(fabs(cu[t - g.NW]));
  else {
    const int p = (int)(t - g.NW - g.NU);
    const int j = p % (g.Nz + 2), i = p / (g.Nz + 2);
    const bool interior = j >= 1 && j <= g.Nz && i >= 1 && i <= g.Nx;
    double d = interior ? 0.0 : 1.0;
    if (p == k.pin_p || (k.open_cnv && j == g.Nz)) d = 1.0;
    const double er = interior ? AT(eta, j - 1, i - 1) / AT(rho, j - 1, i - 1) : 1.0;   // eta / rho
    if (interior) etarho[(size_t)(i - 1) * g.Nz + j - 1] = er;
    s = d == 0.0 ? rsqrt(er) : 1.0 / (sqrt(d) + sqrt(er));
  }
  scl[t] = s;
}

// write the solution back (x is the physical unknown vector)
__global__ void unpack_kernel(Geo g, const double* __restrict__ x, DView W, DView U, DView P) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < g.NW) { W.p[t] = x[t]; return; }
  t -= g.NW;
  if (t < g.NU) { U.p[t] = x[g.NW + t]; return; }
  t -= g.NU;
  if (t < g.NP) P.p[t] = x[g.NW + g.NU + t];
}
__global__ void pack_kernel(Geo g, CView W, CView U, CView P, double* x) {
  XC_PDL_WAIT();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < g.NW) { x[t] = W.p[t]; return; }
  t -= g.NW;
  if (t < g.NU) { x[g.NW + t] = U.p[t]; return; }
  t -= g.NU;
  if (t < g.NP) x[g.NW + g.NU + t] = P.p[t];
}

inline unsigned nblk(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }
// 2-D launch over the (Nz + 2) x (Nx + 2) row positions of a level
inline dim3 blk2() { return dim3(32, 8); }
inline dim3 grid2(const Geo& g) { return dim3((unsigned)((g.Nz + 2 + 31) / 32), (unsigned)((g.Nx + 2 + 7) / 8)); }

}  // namespace

namespace {

struct SolveCfg {
  double omega_v = 0.7, omega_p = 0.8;
  int nu = 1;              // velocity pre-smoothing sweeps (and both on the one-CTA levels)
  int nu_post = 2;         // velocity post-smoothing sweeps on the large levels
  int coarse_sweeps = 0;   // 0: 4 * (Nz + Nx) of the coarsest level, at least 32
  int coarse_cells = 16;   // a velocity level of at most this many cells (pressure: a quarter) is
                           // solved by Jacobi sweeps
  int small_cells = 256;   // levels of at most this many cells run in one CTA
  int nu_p = 2;            // pressure smoothing sweeps before and after each coarse correction
  int gs_passes = 2;       // classical Gram-Schmidt passes per Arnoldi step
  bool pdl = true;         // programmatic dependent launch inside the captured graphs
  bool tiled = false;      // FP32 sweeps from shared-memory tiles (opt-in, measured slower)
  // Schur approximation (Cahouet-Chabard): S^-1 ~ L_in^-1 + cmass * eta/rho with
  // L_in = DM diag(a1 rho/dt)^-1 GG (kplane 9); kplane 0 builds L from the full
  // velocity diagonal instead (cmass then defaults to 0)
  double cmass = 0.5;
  int kplane = 9;
  // pressure levels of at most this many cells use the fused descent /
  // ascent kernels, larger ones one launch per operation (none by default:
  // measured no faster at any level size, programmatic launch already hides
  // the launches they save, and 1% slower on the fine levels)
  long long pfuse_cells = 0;
  // one-CTA levels staged in shared memory (off by default: measured 1.5%
  // slower at 1024^2 -- the small levels' sweeps are bound by instruction
  // latency on one SM, and their L1-resident loads gain nothing from it)
  bool stage_small = false;
  // coarsest levels of at most kDenseMax unknowns solved by their inverse
  bool direct_coarse = true;
  // FP32 inner solves: 0 multigrid preconditioner, 1 the learned network in
  // its place, 2 the network applied to what the multigrid V-cycle leaves
  int learned = 0;
  // FP32 velocity sweeps with four rows along z per thread (vel_sweep_rb_kernel;
  // opt-in: measured 20% slower at 1024^2 than one row per thread)
  bool row_block = false;
  // the Hessenberg least-squares problem of FGMRES on the device (conditional
  // graphs) instead of on the host with one synchronisation per Arnoldi step
  bool device_givens = false;
  // velocity levels of more than small_cells and at most this many cells
  // (below the finest) run in one thread-block-cluster launch (0: none;
  // opt-in: measured no faster than the programmatic per-level launches)
  long long cluster_cells = 0;
};

// The least-squares problem of (F)GMRES(m) on the device: the Hessenberg
// columns, their Givens rotations, the rotated right-hand side g and the
// iteration counters.  Written by one thread at the end of every Arnoldi
// step, so the host needs no synchronisation between steps.
struct KrylovDev {
  double Hm[(kMaxRestart + 1) * kMaxRestart];   // column j at Hm[j * (kMaxRestart + 1)]
  double cs[kMaxRestart], sn[kMaxRestart], gv[kMaxRestart + 1], yv[kMaxRestart];
  double bnorm, stop, relres;
  int its, maxit, kk, done, bad;
};
// what the host reads between steps (pinned, mapped into the device's
// address space; written by the same thread after each step)
struct KrylovStatus {
  double relres;
  int its, kk, done, bad;
};

}  // namespace

// ---------------------------------------------------------------------------
// host-side solver state
// ---------------------------------------------------------------------------
template <typename T>
struct Hier {
  int nv, np_lv;               // velocity and pressure level counts
  Geo vg[kMaxLevels];
  T* cw[kMaxLevels];           // coefficient planes (FP64 hierarchy only)
  T* cu[kMaxLevels];
  T* feta[kMaxLevels];         // FP32 hierarchy: the VOp fields
  T* fetaco[kMaxLevels];
  T* fdw[kMaxLevels];
  T* fdu[kMaxLevels];
  T* fdbot[kMaxLevels];        //   open-bottom row weights, 3 per column
  T* vx[kMaxLevels];
  T* vx2[kMaxLevels];
  T* vb[kMaxLevels];
  T* vr[kMaxLevels];
  int pNz[kMaxLevels], pNx[kMaxLevels], ppin[kMaxLevels];
  T pdpin[kMaxLevels];
  T* kx[kMaxLevels];
  T* kz[kMaxLevels];
  T* px[kMaxLevels];
  T* px2[kMaxLevels];
  T* pb[kMaxLevels];
  T* pr[kMaxLevels];
  T* kr;          // right-face coefficient of the last column (fine level)
  // dense inverses of the coarsest velocity and pressure levels (direct
  // coarse solves) and their validity flags dok[0], dok[1] (device)
  T* vinv;
  T* pinv;
  int* dok;
  bool vdirect, pdirect;
  T* cp;          // DM coefficient planes (fine level)
  T* scl;         // scaling vector
  T* etarho;      // eta/rho on interior cells
  // Krylov
  int m;
  T* V;
  T* Z;
  T* w;
  T* t;
  T* y;           // current iterate (scaled unknowns)
  T* rv;          // preconditioner scratch (velocity part, physical)
  T* rin;         // interior pressure rhs
  // captured graphs per Arnoldi index for two configuration keys (the
  // learned preconditioner and its multigrid fallback alternate within one
  // solve); the least recently used set is rebuilt when a third key appears
  cudaGraphExec_t gexec[2][kMaxRestart];
  long long gnodes[2][kMaxRestart];
  unsigned long long gkey[2];
  int glast;
  // the same steps as conditional graphs (a gate kernel, then the step and
  // its Givens update only while the solve has not stopped), per key set;
  // cnodes = kernels of the gate and of the body
  cudaGraphExec_t cexec[2][kMaxRestart];
  long long cnodes[2][kMaxRestart][2];
  KrylovDev* kd;
  KrylovStatus* ks_host;
  KrylovStatus* ks_dev;
  cudaEvent_t kev[2];
  bool cond_broken;   // building a conditional graph failed: host Givens from then on
};

struct StokesWork {
  Geo g;
  bool ok;
  Hier<double> d;
  Hier<float> f;
  bool f_alloc;
  // coarse coefficient fields (double), per velocity level >= 1
  double *eta[kMaxLevels], *etaco[kMaxLevels], *rho[kMaxLevels], *rhow[kMaxLevels], *rhou[kMaxLevels];
  OpConst last_k;   // operator constants of the last solve (instrumentation)
  bool have_k;
  double* RR;
  double* x;      // physical solution (double)
  double* r;      // scaled residual (double)
  double* part;   // multidot partials
  double* hdev;   // device small vectors (2 * kMaxRestart + 8)
  double* hhost;  // pinned host mirror
  // momentum advection scratch
  double *fz, *uz, *wz, *fx, *ux, *wx, *advz, *advx;
  double *srcw, *srcu, *srcp;
  cudaEvent_t ev0, ev1;
  // learned preconditioner: the network sized for this grid, its input
  // [Nz][Nx][4] (W, U, P components of the vector, log10(eta / etam0)), the
  // log-viscosity channel of the current solve and the hybrid's residual
  xc_nn* net;
  float* nn_in;
  float* nn_logeta;
  float* nn_r;          // 2 n: the V-cycle's residual and A times the network's direction
  float* nn_z;          // n: the network's direction
  double* nn_xprev;     // n: the iterate before a learned refinement pass (restored if the pass fails)
  double* nn_dv;        // 2 n: training samples' V-cycle result and its residual
  bool last_fp64_mg;    // the last solve set up the FP64 multigrid
  SolveCfg last_cfg;
  long long dev_steps;  // Arnoldi steps of the current solve with the least-squares update on the device
};

namespace {

template <typename T>
int alloc_hier(StokesWork* w, Hier<T>& H, int m) {
  const Geo& g = w->g;
  H.m = m;
  const long long n = (long long)g.NW + g.NU + g.NP;
  // velocity levels
  int Nz = g.Nz, Nx = g.Nx;
  double h = g.h;
  H.nv = 0;
  while (H.nv < kMaxLevels) {
    Geo lg = make_geo(Nz, Nx, h);
    H.vg[H.nv] = lg;
    long long nvv = (long long)lg.NW + lg.NU;
    if (kFly<T>) {
      XC_CUDA_TRY(cudaMalloc(&H.feta[H.nv], sizeof(T) * lg.Nz * lg.Nx));
      XC_CUDA_TRY(cudaMalloc(&H.fetaco[H.nv], sizeof(T) * (lg.Nz + 1) * (lg.Nx + 1)));
      XC_CUDA_TRY(cudaMalloc(&H.fdw[H.nv], sizeof(T) * lg.NW));
      XC_CUDA_TRY(cudaMalloc(&H.fdu[H.nv], sizeof(T) * lg.NU));
      XC_CUDA_TRY(cudaMalloc(&H.fdbot[H.nv], sizeof(T) * 3 * (lg.Nx + 2)));
    } else {
      XC_CUDA_TRY(cudaMalloc(&H.cw[H.nv], sizeof(T) * 10 * lg.NW));
      XC_CUDA_TRY(cudaMalloc(&H.cu[H.nv], sizeof(T) * 10 * lg.NU));
    }
    XC_CUDA_TRY(cudaMalloc(&H.vx[H.nv], sizeof(T) * nvv));
    XC_CUDA_TRY(cudaMalloc(&H.vx2[H.nv], sizeof(T) * nvv));
    XC_CUDA_TRY(cudaMalloc(&H.vb[H.nv], sizeof(T) * nvv));
    XC_CUDA_TRY(cudaMalloc(&H.vr[H.nv], sizeof(T) * nvv));
    H.nv++;
    if (Nz % 2 || Nx % 2 || Nz / 2 < 4 || Nx / 2 < 4) break;
    Nz /= 2; Nx /= 2; h *= 2;
  }
  XC_CUDA_TRY(cudaMalloc(&H.vinv, sizeof(T) * kDenseMax * kDenseMax));
  XC_CUDA_TRY(cudaMalloc(&H.pinv, sizeof(T) * kDenseMax * kDenseMax));
  XC_CUDA_TRY(cudaMalloc(&H.dok, sizeof(int) * 2));
  XC_CUDA_TRY(cudaMemset(H.dok, 0, sizeof(int) * 2));
  // pressure levels
  Nz = g.Nz; Nx = g.Nx;
  int pz = (int)std::nearbyint(g.Nz / 2.0) - 2, px = (int)std::nearbyint(g.Nx / 2.0) - 2;
  H.np_lv = 0;
  while (H.np_lv < kMaxLevels) {
    int L = H.np_lv;
    H.pNz[L] = Nz; H.pNx[L] = Nx; H.ppin[L] = px * Nz + pz;
    XC_CUDA_TRY(cudaMalloc(&H.kx[L], sizeof(T) * Nz * Nx));
    XC_CUDA_TRY(cudaMalloc(&H.kz[L], sizeof(T) * (Nz + 1) * Nx));
    XC_CUDA_TRY(cudaMalloc(&H.px[L], sizeof(T) * Nz * Nx));
    XC_CUDA_TRY(cudaMalloc(&H.px2[L], sizeof(T) * Nz * Nx));
    XC_CUDA_TRY(cudaMalloc(&H.pb[L], sizeof(T) * Nz * Nx));
    XC_CUDA_TRY(cudaMalloc(&H.pr[L], sizeof(T) * Nz * Nx));
    H.np_lv++;
    if (Nz % 2 || Nx % 2 || Nz / 2 < 2 || Nx / 2 < 2) break;
    Nz /= 2; Nx /= 2; pz /= 2; px /= 2;
  }
  XC_CUDA_TRY(cudaMalloc(&H.kr, sizeof(T) * g.Nz));
  XC_CUDA_TRY(cudaMalloc(&H.cp, sizeof(T) * 4 * g.NP));
  XC_CUDA_TRY(cudaMalloc(&H.scl, sizeof(T) * n));
  XC_CUDA_TRY(cudaMalloc(&H.etarho, sizeof(T) * g.Nz * g.Nx));
  XC_CUDA_TRY(cudaMalloc(&H.V, sizeof(T) * n * (m + 1)));
  XC_CUDA_TRY(cudaMalloc(&H.Z, sizeof(T) * n * m));
  XC_CUDA_TRY(cudaMalloc(&H.w, sizeof(T) * n));
  XC_CUDA_TRY(cudaMalloc(&H.t, sizeof(T) * n));
  XC_CUDA_TRY(cudaMalloc(&H.y, sizeof(T) * n));
  XC_CUDA_TRY(cudaMalloc(&H.rv, sizeof(T) * (g.NW + g.NU)));
  XC_CUDA_TRY(cudaMalloc(&H.rin, sizeof(T) * g.Nz * g.Nx));
  XC_CUDA_TRY(cudaMalloc(&H.kd, sizeof(KrylovDev)));
  XC_CUDA_TRY(cudaMemset(H.kd, 0, sizeof(KrylovDev)));
  XC_CUDA_TRY(cudaHostAlloc(&H.ks_host, sizeof(KrylovStatus), cudaHostAllocMapped));
  std::memset(H.ks_host, 0, sizeof(KrylovStatus));
  XC_CUDA_TRY(cudaHostGetDevicePointer((void**)&H.ks_dev, H.ks_host, 0));
  for (int q = 0; q < 2; ++q) XC_CUDA_TRY(cudaEventCreateWithFlags(&H.kev[q], cudaEventDisableTiming));
  return XC_OK;
}

template <typename T>
void free_hier(Hier<T>& H) {
  for (int e = 0; e < 2; ++e)
    for (int q = 0; q < kMaxRestart; ++q) {
      if (H.gexec[e][q]) { cudaGraphExecDestroy(H.gexec[e][q]); H.gexec[e][q] = nullptr; }
      if (H.cexec[e][q]) { cudaGraphExecDestroy(H.cexec[e][q]); H.cexec[e][q] = nullptr; }
    }
  cudaFree(H.kd);
  if (H.ks_host) cudaFreeHost(H.ks_host);
  for (int q = 0; q < 2; ++q)
    if (H.kev[q]) cudaEventDestroy(H.kev[q]);
  for (int l = 0; l < H.nv; ++l) {
    cudaFree(H.cw[l]); cudaFree(H.cu[l]); cudaFree(H.vx[l]); cudaFree(H.vx2[l]); cudaFree(H.vb[l]); cudaFree(H.vr[l]);
    cudaFree(H.feta[l]); cudaFree(H.fetaco[l]); cudaFree(H.fdw[l]); cudaFree(H.fdu[l]); cudaFree(H.fdbot[l]);
  }
  for (int l = 0; l < H.np_lv; ++l) {
    cudaFree(H.kx[l]); cudaFree(H.kz[l]); cudaFree(H.px[l]); cudaFree(H.px2[l]); cudaFree(H.pb[l]); cudaFree(H.pr[l]);
  }
  cudaFree(H.kr); cudaFree(H.cp); cudaFree(H.scl); cudaFree(H.etarho); cudaFree(H.V); cudaFree(H.Z);
  cudaFree(H.w); cudaFree(H.t); cudaFree(H.y); cudaFree(H.rv); cudaFree(H.rin);
  cudaFree(H.vinv); cudaFree(H.pinv); cudaFree(H.dok);
  H.nv = H.np_lv = 0;
}

template <typename T>
VOp<T> vop(const Hier<T>& H, int l) {
  VOp<T> o;
  o.cw = H.cw[l]; o.cu = H.cu[l];
  o.eta = H.feta[l]; o.etaco = H.fetaco[l]; o.dw = H.fdw[l]; o.du = H.fdu[l]; o.dbot = H.fdbot[l];
  return o;
}



// Jacobi sweeps on a coarsest level of Nz x Nx cells: a few times the grid's
// diameter, enough for the smoothing to reach across the level
static int coarse_sweeps(const SolveCfg& cfg, int Nz, int Nx) {
  if (cfg.coarse_sweeps > 0) return cfg.coarse_sweeps;
  return 4 * (Nz + Nx) > 32 ? 4 * (Nz + Nx) : 32;
}

template <typename T>
static bool vel_coarsest(const Hier<T>& H, const SolveCfg& cfg, int l) {
  return l == H.nv - 1 || (long long)H.vg[l].Nz * H.vg[l].Nx <= cfg.coarse_cells;
}
template <typename T>
static bool p_coarsest(const Hier<T>& H, const SolveCfg& cfg, int l) {
  return l == H.np_lv - 1 || 4LL * H.pNz[l] * H.pNx[l] <= cfg.coarse_cells;
}

// one CTA runs the coarsest level; fewer threads make each sweep's barrier cheaper
static int coarse_threads(long long n) { return n > 512 ? 1024 : (n > 128 ? 256 : 128); }

// ---- velocity V-cycle on level l: solve A x = vb[l] approximately (x := vx[l])
// one velocity sweep (MODE of vel_sweep2d_kernel) of level g: the FP32
// hierarchy takes the shared-memory tiled kernel for the sweeps that read
// neighbours
template <typename T, int MODE>
void launch_sweep(const SolveCfg& cfg, const Geo& g, const OpConst& k, const VOp<T>& op, const T* xi, const T* b,
                  T* out, T om, const T* dscl, cudaStream_t s) {
  if constexpr (kFly<T>) {
    if (MODE != 0 && cfg.tiled) {
      pdl(PDL_ON, vel_sweep_tiled_kernel<MODE>, grid2(g), blk2(), s, g, k, op, xi, b, out, om, dscl);
      return;
    }
    if (cfg.row_block) {
      pdl(PDL_ON, vel_sweep_rb_kernel<MODE>, grid_rb(g), blk2(), s, g, k, op, xi, b, out, om, dscl);
      return;
    }
  }
  pdl(PDL_ON, vel_sweep2d_kernel<T, MODE>, grid2(g), blk2(), s, g, k, op, xi, b, out, om, dscl);
}

// CTAs per cluster of the cluster V-cycle (16 where the device schedules
// clusters of 16 CTAs of 1024 threads, else 8; 0: clusters unavailable),
// per precision, found once per process
int g_vcluster[2] = {-1, -1};
std::mutex g_vcluster_mu;
template <typename T>
int vel_cluster_size() {
  const int p = std::is_same<T, float>::value ? 0 : 1;
  std::lock_guard<std::mutex> lock(g_vcluster_mu);
  if (g_vcluster[p] >= 0) return g_vcluster[p];
  int best = 0;
  cudaFuncSetAttribute(vel_vcycle_cluster_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  for (int cs : {16, 8}) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(cs);
    lc.blockDim = dim3(1024);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, vel_vcycle_cluster_kernel<T>, &lc) == cudaSuccess &&
        nclusters >= 1) {
      best = cs;
      break;
    }
  }
  cudaGetLastError();
  g_vcluster[p] = best;
  return best;
}

template <typename T>
int vcycle_vel(Hier<T>& H, const OpConst& kf, const SolveCfg& cfg, int l, cudaStream_t s, T* final_out = nullptr,
               const T* final_scl = nullptr, bool* final_done = nullptr) {
  const Geo& g = H.vg[l];
  const long long n = (long long)g.NW + g.NU;
  const T om = (T)cfg.omega_v;
  const OpConst k = level_const(kf, l);
  const long long cells = (long long)g.Nz * g.Nx;
  if (l > 0 && cfg.cluster_cells > 0 && cells <= cfg.cluster_cells && cells > cfg.small_cells &&
      !vel_coarsest(H, cfg, l)) {
    const int cs = vel_cluster_size<T>();
    if (cs > 0) {
      int ls = l;
      while (!vel_coarsest(H, cfg, ls) && (long long)H.vg[ls].Nz * H.vg[ls].Nx > cfg.small_cells) ++ls;
      int lc = ls;
      while (!vel_coarsest(H, cfg, lc)) ++lc;
      VelLevels<T> L;
      for (int q = 0; q <= lc; ++q) {
        L.g[q] = H.vg[q]; L.op[q] = vop(H, q);
        L.x[q] = H.vx[q]; L.x2[q] = H.vx2[q]; L.b[q] = H.vb[q]; L.r[q] = H.vr[q];
      }
      cudaLaunchConfig_t lcfg = {};
      lcfg.gridDim = dim3(cs);
      lcfg.blockDim = dim3(1024);
      lcfg.stream = s;
      cudaLaunchAttribute at[2];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = cs;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      at[1].val.programmaticStreamSerializationAllowed = 1;
      lcfg.attrs = at;
      lcfg.numAttrs = PDL_ON ? 2 : 1;
      XC_CUDA_TRY(cudaLaunchKernelEx(&lcfg, vel_vcycle_cluster_kernel<T>, L, kf, l, ls, lc, cfg.nu, cfg.nu_post, om,
                                     coarse_sweeps(cfg, H.vg[lc].Nz, H.vg[lc].Nx),
                                     (const T*)(H.vdirect ? H.vinv : nullptr), (const int*)H.dok));
      xc_count_launch();
      XC_LAUNCH_CHECK();
      return XC_OK;
    }
  }
  if (!vel_coarsest(H, cfg, l) && (long long)g.Nz * g.Nx <= cfg.small_cells) {
    int lc = l;
    while (!vel_coarsest(H, cfg, lc)) ++lc;
    VelLevels<T> L;
    for (int q = 0; q <= lc; ++q) {
      L.g[q] = H.vg[q]; L.op[q] = vop(H, q);
      L.x[q] = H.vx[q]; L.x2[q] = H.vx2[q]; L.b[q] = H.vb[q]; L.r[q] = H.vr[q];
    }
    const size_t bytes = sizeof(T) * (size_t)vel_stage_elems<T>(H.vg, l, lc);
    const int staged = cfg.stage_small && bytes <= kStageMaxBytes;
    pdl_smem(PDL_ON, vel_vcycle_small_kernel<T>, 1, coarse_threads(n), staged ? bytes : 0, s, L, kf, l, lc, cfg.nu,
             om, coarse_sweeps(cfg, H.vg[lc].Nz, H.vg[lc].Nx), staged, H.vdirect ? H.vinv : nullptr, H.dok);
    XC_LAUNCH_CHECK();
    return XC_OK;
  }
  if (vel_coarsest(H, cfg, l)) {
    pdl(PDL_ON, vel_coarse_kernel<T>, 1, coarse_threads(n), s, g, k, vop(H, l), H.vx[l], H.vx2[l], H.vb[l],
                                                        coarse_sweeps(cfg, g.Nz, g.Nx), om,
                                                        (const T*)(H.vdirect ? H.vinv : nullptr), (const int*)H.dok);
    XC_LAUNCH_CHECK();
    return XC_OK;
  }
  // pre-smoothing (first sweep from zero, into the buffer that makes the last
  // sweep land in vx)
  const VOp<T> op = vop(H, l);
  const T* no = nullptr;
  T* a = (cfg.nu - 1) % 2 ? H.vx2[l] : H.vx[l];
  T* o = (cfg.nu - 1) % 2 ? H.vx[l] : H.vx2[l];
  launch_sweep<T, 0>(cfg, g, k, op, a, H.vb[l], a, om, no, s);
  for (int q = 1; q < cfg.nu; ++q) {
    launch_sweep<T, 1>(cfg, g, k, op, a, H.vb[l], o, om, no, s);
    T* tmp = a; a = o; o = tmp;
  }
  launch_sweep<T, 2>(cfg, g, k, op, H.vx[l], H.vb[l], H.vr[l], om, no, s);
  const Geo& c = H.vg[l + 1];
  pdl(PDL_ON, vel_restrict2d_kernel<T>, grid2(c), blk2(), s, g, c, H.vr[l], H.vb[l + 1]);
  XC_LAUNCH_CHECK();
  XC_TRY(vcycle_vel<T>(H, kf, cfg, l + 1, s));
  pdl(PDL_ON, vel_prolong2d_kernel<T>, grid2(g), blk2(), s, g, c, k, H.vx[l + 1], H.vx[l]);
  a = H.vx[l];
  o = H.vx2[l];
  const int npost = cfg.nu_post;
  for (int q = 0; q < npost; ++q) {
    if (final_out && q == npost - 1) {   // last sweep of the fine level straight into the output
      if (final_scl) launch_sweep<T, 3>(cfg, g, k, op, a, H.vb[l], final_out, om, final_scl, s);   // scaled
      else launch_sweep<T, 1>(cfg, g, k, op, a, H.vb[l], final_out, om, final_scl, s);           // physical
      *final_done = true;
      XC_LAUNCH_CHECK();
      return XC_OK;
    }
    launch_sweep<T, 1>(cfg, g, k, op, a, H.vb[l], o, om, no, s);
    T* tmp = a; a = o; o = tmp;
  }
  if (a != H.vx[l]) XC_CUDA_TRY(cudaMemcpyAsync(H.vx[l], a, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// ---- pressure V-cycle on level l: solve L x = pb[l] approximately; *res is
// the buffer holding x (px[l] or px2[l]: the sweeps alternate between the two
// and no copy is made)
template <typename T>
int vcycle_p(Hier<T>& H, const SolveCfg& cfg, int l, cudaStream_t s, T** res) {
  const int Nz = H.pNz[l], Nx = H.pNx[l], n = Nz * Nx;
  const T om = (T)cfg.omega_p;
  *res = H.px[l];
  if (!p_coarsest(H, cfg, l) && (long long)n <= cfg.small_cells) {
    int lc = l;
    while (!p_coarsest(H, cfg, lc)) ++lc;
    PLevels<T> L;
    for (int q = 0; q <= lc; ++q) {
      L.Nz[q] = H.pNz[q]; L.Nx[q] = H.pNx[q]; L.pin[q] = H.ppin[q]; L.dpin[q] = H.pdpin[q];
      L.kx[q] = H.kx[q]; L.kz[q] = H.kz[q];
      L.x[q] = H.px[q]; L.x2[q] = H.px2[q]; L.b[q] = H.pb[q]; L.r[q] = H.pr[q];
    }
    const size_t bytes = sizeof(T) * (size_t)p_stage_elems<T>(H.pNz, H.pNx, l, lc);
    const int staged = cfg.stage_small && bytes <= kStageMaxBytes;
    pdl_smem(PDL_ON, p_vcycle_small_kernel<T>, 1, coarse_threads(n), staged ? bytes : 0, s, L, l, lc, cfg.nu_p, om,
             coarse_sweeps(cfg, H.pNz[lc], H.pNx[lc]), staged, H.pdirect ? H.pinv : nullptr, H.dok + 1);
    XC_LAUNCH_CHECK();
    return XC_OK;
  }
  if (p_coarsest(H, cfg, l)) {
    pdl(PDL_ON, p_coarse_kernel<T>, 1, coarse_threads(n), s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], H.px[l],
                                                      H.px2[l], H.pb[l], coarse_sweeps(cfg, Nz, Nx), om,
                                                      (const T*)(H.pdirect ? H.pinv : nullptr), (const int*)(H.dok + 1));
    XC_LAUNCH_CHECK();
    return XC_OK;
  }
  const int Nzc = H.pNz[l + 1], Nxc = H.pNx[l + 1];
  T* ec = nullptr;
  if ((long long)n > cfg.pfuse_cells) {
    // one launch per operation (same values as the fused path below)
    pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], H.px[l], H.pb[l],
                                               H.px[l], om, 1);
    T* a = H.px[l];
    T* o = H.px2[l];
    for (int q = 1; q < cfg.nu_p; ++q) {
      pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l], o,
                                                 om, 0);
      T* tmp = a; a = o; o = tmp;
    }
    pdl(PDL_ON, p_residual_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l],
                                                 H.pr[l]);
    pdl(PDL_ON, p_restrict_kernel<T>, nblk(Nzc * Nxc), 256, s, Nzc, Nxc, H.pr[l], H.pb[l + 1]);
    XC_LAUNCH_CHECK();
    XC_TRY(vcycle_p<T>(H, cfg, l + 1, s, &ec));
    pdl(PDL_ON, p_prolong_kernel<T>, nblk(n), 256, s, Nzc, Nxc, ec, a);
    for (int q = 0; q < cfg.nu_p; ++q) {
      pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l], o,
                                                 om, 0);
      T* tmp = a; a = o; o = tmp;
    }
    *res = a;
    XC_LAUNCH_CHECK();
    return XC_OK;
  }
  // pre-smoothing: with one sweep, the sweep from zero, the residual and the
  // restriction are one launch; otherwise the last of them fuses the last two
  T* a = H.px[l];
  T* o = H.px2[l];
  if (cfg.nu_p > 1) {
    pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l], a,
                                               om, 1);
    for (int q = 1; q < cfg.nu_p; ++q) {
      pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l], o,
                                                 om, 0);
      T* tmp = a; a = o; o = tmp;
    }
  }
  pdl(PDL_ON, p_down_kernel<T>, nblk(Nzc * Nxc), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l],
                                             H.pb[l + 1], om, cfg.nu_p > 1 ? 0 : 1);
  XC_LAUNCH_CHECK();
  XC_TRY(vcycle_p<T>(H, cfg, l + 1, s, &ec));
  // post-smoothing: the first sweep takes the prolongation along
  pdl(PDL_ON, p_up_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], ec, a, H.pb[l], o, om);
  { T* tmp = a; a = o; o = tmp; }
  for (int q = 1; q < cfg.nu_p; ++q) {
    pdl(PDL_ON, p_jacobi_kernel<T>, nblk(n), 256, s, Nz, Nx, H.kx[l], H.kz[l], H.ppin[l], H.pdpin[l], a, H.pb[l], o,
                                               om, 0);
    T* tmp = a; a = o; o = tmp;
  }
  *res = a;
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// out = M^-1 v for the scaled system: out = S^-1 M_phys (S^-1 v)
// phys_out: out = M_phys (S^-1 v) in physical variables, without the final
// S^-1 (the caller applies the operator to it directly)
template <typename T>
int precond(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, const T* v, T* out,
            cudaStream_t s, bool phys_out = false) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  const long long nvv = (long long)g.NW + g.NU;
  // physical residual r = S^-1 v: pressure part into rp here, velocity part
  // into vb[0] by sub_grad_kernel below
  // pressure: interior solve with ghost elimination
  pdl(PDL_ON, p_gather_fused_kernel<T>, nblk(g.Nz * g.Nx), 256, s, g, (const T*)H.kx[0], (const T*)H.kr,
      v + nvv, (const T*)(H.scl + nvv), H.pb[0]);
  XC_LAUNCH_CHECK();
  T* px0 = nullptr;
  XC_TRY(vcycle_p<T>(H, cfg, 0, s, &px0));
  T* zp = out + nvv;   // physical z_p written directly into out, rescaled below
  pdl(PDL_ON, p_scatter_fused_kernel<T>, nblk(g.NP), 256, s, g, (const T*)px0, v + nvv, (const T*)(H.scl + nvv),
      (const T*)H.etarho, (T)cfg.cmass, k.open_cnv, zp);
  // velocity: rhs r_v - GG z_p, one V-cycle
  pdl(PDL_ON, sub_grad_kernel<T>, nblk(nvv), 256, s, g, zp, v, H.scl, H.vb[0]);
  XC_LAUNCH_CHECK();
  bool done = false;
  XC_TRY(vcycle_vel<T>(H, k, cfg, 0, s, out, phys_out ? nullptr : H.scl, &done));
  if (!done) {
    if (phys_out) XC_CUDA_TRY(cudaMemcpyAsync(out, H.vx[0], sizeof(T) * nvv, cudaMemcpyDeviceToDevice, s));
    else pdl(PDL_ON, div_kernel<T>, nblk(nvv), 256, s, nvv, H.vx[0], H.scl, out);
  }
  if (!phys_out) pdl(PDL_ON, div_kernel<T>, nblk(g.NP), 256, s, g.NP, zp, H.scl + nvv, zp);
  XC_LAUNCH_CHECK();
  (void)n;
  return XC_OK;
}

// y_out = S o LL (S o v)  (or b - that when b != null)
template <typename T>
int apply_scaled(StokesWork* w, Hier<T>& H, const OpConst& k, const T* v, const T* b, T* y, cudaStream_t s) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  pdl(PDL_ON, mul_kernel<T>, nblk(n), 256, s, n, v, H.scl, H.t);
  pdl(PDL_ON, stokes_apply_kernel<T>, grid2(g), blk2(), s, g, k, vop(H, 0), H.cp, H.scl, H.t, b, y);
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// Grid of each multidot variant: one wave of as many CTAs as its register use
// lets an SM hold (more accumulators, fewer CTAs), queried once per process.
int g_md_grid[2][3];   // [FP32, FP64][8, 16, 32 accumulators]
std::once_flag g_md_once;
void md_grid_init() {
  int dev = 0, sms = kNumSMs;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto grid = [&](const void* fn) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, KB, 0) != cudaSuccess || b < 1) b = 1;
    return std::min(std::min(b, 8) * sms, KGMAX);
  };
  g_md_grid[0][0] = grid((const void*)multidot_kernel<float, 8>);
  g_md_grid[0][1] = grid((const void*)multidot_kernel<float, 16>);
  g_md_grid[0][2] = grid((const void*)multidot_kernel<float, 32>);
  g_md_grid[1][0] = grid((const void*)multidot_kernel<double, 8>);
  g_md_grid[1][1] = grid((const void*)multidot_kernel<double, 16>);
  g_md_grid[1][2] = grid((const void*)multidot_kernel<double, 32>);
}

// partial dots of wv with V[0..m), accumulator count chosen from m; returns
// the number of partial rows written
template <typename T>
int launch_multidot(long long n, int m, const T* V, long long ldv, const T* wv, double* part, cudaStream_t s) {
  const int* gr = g_md_grid[std::is_same<T, float>::value ? 0 : 1];
  int nb;
  nb = gr[0];
  switch (m) {
    case 1: pdl(PDL_ON, multidot_kernel<T, 1, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 2: pdl(PDL_ON, multidot_kernel<T, 2, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 3: pdl(PDL_ON, multidot_kernel<T, 3, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 4: pdl(PDL_ON, multidot_kernel<T, 4, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 5: pdl(PDL_ON, multidot_kernel<T, 5, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 6: pdl(PDL_ON, multidot_kernel<T, 6, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 7: pdl(PDL_ON, multidot_kernel<T, 7, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    case 8: pdl(PDL_ON, multidot_kernel<T, 8, true>, nb, KB, s, n, m, V, ldv, wv, part); return nb;
    default: break;
  }
  if (m <= 16) pdl(PDL_ON, multidot_kernel<T, 16>, (nb = gr[1]), KB, s, n, m, V, ldv, wv, part);
  else pdl(PDL_ON, multidot_kernel<T, 32>, (nb = gr[2]), KB, s, n, m, V, ldv, wv, part);
  return nb;
}

// ||v||^2 -> hdev[slot] (device), deterministic; 1/||v|| -> hdev[6]
template <typename T>
int dot_self(StokesWork* w, Hier<T>& H, const T* v, long long n, int slot, cudaStream_t s) {
  const int nb = launch_multidot<T>(n, 1, v, n, v, w->part, s);
  pdl(PDL_ON, norm_final_kernel, 1, KB, s, nb, w->part, w->hdev + slot, w->hdev + 6);
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// ---------------------------------------------------------------------------
// learned preconditioner glue.  The network sees the grid's Nz x Nx cells as
// an image (row j = z, column i = x) with four channels: the vector's W
// component on the top face of the cell W(j, i+1), its U component on the
// left face U(j+1, i), its P component P(j+1, i+1), and log10(eta / etam0).
// Its three output channels give the correction on the interior unknowns
// (W rows 1..Nz-1, U columns 0..Nx-1, interior P); every boundary, ghost and
// duplicated-periodic unknown keeps the vector's own value (their scaled rows
// are near identity).
// ---------------------------------------------------------------------------
__global__ void nn_logeta_kernel(int Nz, int Nx, const double* __restrict__ eta, double etam0, float* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)Nz * Nx) return;
  const int j = (int)(t / Nx), i = (int)(t % Nx);
  out[t] = (float)log10(eta[(size_t)i * Nz + j] / etam0);
}

// network input of a vector v: its components times scale (times 1/||v||
// from the device when inv_norm is given).  Vectors of unit norm enter with
// scale sqrt(Nz Nx), i.e. at O(1) per pixel.
template <typename V>
__global__ void nn_pack_kernel(Geo g, const V* __restrict__ v, const float* __restrict__ logeta,
                               const double* __restrict__ inv_norm, float scale, float* in, int channels) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)g.Nz * g.Nx) return;
  const int j = (int)(t / g.Nx), i = (int)(t % g.Nx);
  const float sc = (inv_norm ? (float)*inv_norm : 1.0f) * scale;
  float* o = in + t * channels;
  o[0] = sc * (float)v[(size_t)(i + 1) * (g.Nz + 1) + j];
  o[1] = sc * (float)v[(size_t)g.NW + (size_t)i * (g.Nz + 2) + j + 1];
  o[2] = sc * (float)v[(size_t)g.NW + g.NU + (size_t)(i + 1) * (g.Nz + 2) + j + 1];
  if (channels > 3) o[3] = logeta[t];
}

// image pixel and channel of unknown t, or -1 for the unknowns the network
// does not correct
__device__ __forceinline__ long long nn_pixel(const Geo& g, long long t, int* ch) {
  if (t < g.NW) {
    const int i = (int)(t / (g.Nz + 1)), j = (int)(t % (g.Nz + 1));
    *ch = 0;
    return (j >= 1 && j <= g.Nz - 1 && i >= 1 && i <= g.Nx) ? (long long)j * g.Nx + (i - 1) : -1;
  }
  t -= g.NW;
  if (t < g.NU) {
    const int i = (int)(t / (g.Nz + 2)), j = (int)(t % (g.Nz + 2));
    *ch = 1;
    return (j >= 1 && j <= g.Nz && i <= g.Nx - 1) ? (long long)(j - 1) * g.Nx + i : -1;
  }
  t -= g.NU;
  const int i = (int)(t / (g.Nz + 2)), j = (int)(t % (g.Nz + 2));
  *ch = 2;
  return (j >= 1 && j <= g.Nz && i >= 1 && i <= g.Nx) ? (long long)(j - 1) * g.Nx + (i - 1) : -1;
}

// z = network output on the interior unknowns and `outside` elsewhere (zero
// when outside is null)
__global__ void nn_unpack_kernel(Geo g, const float* __restrict__ o16, const float* __restrict__ outside,
                                 float* z) {
  const long long n = (long long)g.NW + g.NU + g.NP;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  int ch = 0;
  const long long p = nn_pixel(g, t, &ch);
  z[t] = p >= 0 ? o16[p * 16 + ch] : (outside ? outside[t] : 0.0f);
}

// z += alpha n with alpha = dots[0] / dots[1], the least-squares step of n
// against the residual r it targets (|r|^2 = *rnorm2).  The step is taken
// only when it removes at least a tenth of |r|^2: a direction the network
// gets wrong is then left out instead of adding a large, nearly A-null
// component that the FP32 Krylov basis could not resolve.
__global__ void nn_axpy_kernel(long long n, const double* __restrict__ dots, const double* __restrict__ rnorm2,
                               const float* __restrict__ nz, float* z) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double num = dots[0], den = dots[1];
  const bool take = den > 0.0 && num * num >= 0.1 * (*rnorm2) * den;
  const float alpha = take ? (float)(num / den) : 0.0f;
  z[t] += alpha * nz[t];
}

// the training target: a scaled FP64 solution y on the interior unknowns,
// [Nz][Nx][3] in the input's pixel layout
__global__ void nn_target_kernel(Geo g, const double* __restrict__ y, float* out) {
  const long long n = (long long)g.NW + g.NU + g.NP;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  int ch = 0;
  const long long p = nn_pixel(g, t, &ch);
  if (p >= 0) out[p * 3 + ch] = (float)y[t];
}

// z = M v for the configured preconditioner
template <typename T>
int apply_precond(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, const T* v, T* out,
                  cudaStream_t s, bool phys_out = false) {
  if constexpr (std::is_same<T, float>::value) {
    if (cfg.learned != 0) {
      const Geo& g = w->g;
      const long long n = (long long)g.NW + g.NU + g.NP;
      const long long npx = (long long)g.Nz * g.Nx;
      const float unit = sqrtf((float)npx);
      if (cfg.learned == 1) {
        // the network in place of the V-cycle (the Krylov vector has unit
        // norm; FGMRES is indifferent to the scale of each z)
        nn_pack_kernel<float><<<nblk(npx), 256, 0, s>>>(g, v, w->nn_logeta, nullptr, unit, w->nn_in, 4);
        xc_count_launch();
        XC_TRY(nn_forward_async(w->net, w->nn_in, s));
        nn_unpack_kernel<<<nblk(n), 256, 0, s>>>(g, nn_out16(w->net), v, out); xc_count_launch();
      } else {
        // V-cycle; r = v - A z its residual (nn_r[0..n)); the network's
        // direction for r, nz; A nz (nn_r[n..2n)); z += alpha nz with the
        // least-squares alpha = (r . A nz) / (A nz . A nz)
        float* r = w->nn_r;
        float* anz = w->nn_r + n;
        XC_TRY(precond<T>(w, H, k, cfg, v, out, s));
        XC_TRY(apply_scaled<T>(w, H, k, out, v, r, s));
        XC_TRY(dot_self<T>(w, H, r, n, 5, s));
        nn_pack_kernel<float><<<nblk(npx), 256, 0, s>>>(g, r, w->nn_logeta, w->hdev + 6, unit, w->nn_in, 4);
        xc_count_launch();
        XC_TRY(nn_forward_async(w->net, w->nn_in, s));
        nn_unpack_kernel<<<nblk(n), 256, 0, s>>>(g, nn_out16(w->net), nullptr, w->nn_z); xc_count_launch();
        XC_TRY(apply_scaled<T>(w, H, k, w->nn_z, nullptr, anz, s));
        double* dots = w->hdev + 8;   // free until this step's Gram-Schmidt
        const int nb = launch_multidot<float>(n, 2, r, n, anz, w->part, s);
        pdl(PDL_ON, multidot_final_kernel, 2, KB, s, 2, nb, w->part, dots);
        nn_axpy_kernel<<<nblk(n), 256, 0, s>>>(n, dots, w->hdev + 5, w->nn_z, out); xc_count_launch();
      }
      XC_LAUNCH_CHECK();
      return XC_OK;
    }
  }
  return precond<T>(w, H, k, cfg, v, out, s, phys_out);
}

// The launches of one Arnoldi step k: z_k = M v_k; w = A z_k; two classical
// Gram-Schmidt passes against v_0..v_k (coefficients to hdev[8..]); ||w||^2 to
// hdev[2]; v_{k+1} = w / ||w||; the H column to the pinned host mirror.
template <typename T>
int arnoldi_launches(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, int kk, cudaStream_t s,
                     bool with_precond = true, bool host_copy = true) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  T* vk = H.V + (size_t)kk * n;
  T* zk = H.Z + (size_t)kk * n;
  T* wv = H.V + (size_t)(kk + 1) * n;
  if (kk + 1 > 32) { xc_set_error("fgmres: restart above 32 basis vectors"); return XC_BAD_ARG; }
  // with the multigrid preconditioner z_k stays in physical variables
  // (Z[k] = S z_k): the operator takes it as it is, and the combine of the
  // cycle's update applies S^-1 once, instead of an S^-1 pass after every
  // preconditioner and an S pass before every operator
  const bool zphys = with_precond && cfg.learned == 0;
  if (with_precond) XC_TRY(apply_precond<T>(w, H, k, cfg, vk, zk, s, zphys));
  if (zphys) {
    pdl(PDL_ON, stokes_apply_kernel<T>, grid2(g), blk2(), s, g, k, vop(H, 0), (const T*)H.cp, (const T*)H.scl,
        (const T*)zk, (const T*)nullptr, wv);
  } else {
    XC_TRY(apply_scaled<T>(w, H, k, zk, nullptr, wv, s));
  }
  double* hd = w->hdev + 8;
  for (int pass = 0; pass < cfg.gs_passes; ++pass) {
    const int nb = launch_multidot<T>(n, kk + 1, H.V, n, wv, w->part, s);
    pdl(PDL_ON, multidot_final_kernel, kk + 1, KB, s, kk + 1, nb, w->part, hd + pass * kMaxRestart);
    if (pass + 1 < cfg.gs_passes) {
      pdl(PDL_ON, multiaxpy_kernel<T>, nblk(n), 256, s, n, kk + 1, H.V, n, hd + pass * kMaxRestart, wv);
    } else {
      // the last pass also forms ||w||^2 (-> hdev[2], 1/||w|| -> hdev[6])
      const int nbn = (int)std::min<long long>(nblk(n), (long long)KGMAX);
      pdl(PDL_ON, multiaxpy_norm_kernel<T>, nbn, KB, s, n, kk + 1, (const T*)H.V, n,
          (const double*)(hd + pass * kMaxRestart), wv, w->part);
      pdl(PDL_ON, norm_final_kernel, 1, KB, s, nbn, (const double*)w->part, w->hdev + 2, w->hdev + 6);
    }
  }
  pdl(PDL_ON, normalize_kernel<T>, nblk(n), 256, s, n, w->hdev + 6, wv);
  if (host_copy)
    XC_CUDA_TRY(cudaMemcpyAsync(w->hhost, w->hdev, sizeof(double) * (8 + 2 * kMaxRestart), cudaMemcpyDeviceToHost, s));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// ---- the FGMRES least-squares problem on the device --------------------------
// A restart cycle starts from g = (beta, 0, ...); its counters carry the
// iterations of earlier cycles of the same solve.
__global__ void krylov_start_kernel(KrylovDev* kd, double beta, double bnorm, double stop, int maxit, int its) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i <= kMaxRestart; ++i) kd->gv[i] = 0.0;
  kd->gv[0] = beta;
  kd->bnorm = bnorm;
  kd->stop = stop;
  kd->relres = beta / bnorm;
  kd->maxit = maxit;
  kd->its = its;
  kd->kk = 0;
  kd->done = 0;
  kd->bad = 0;
}

// the IF condition of an Arnoldi step's graph: run the step only while the
// cycle has not met its target, broken down or used up its iterations
__global__ void krylov_gate_kernel(const KrylovDev* kd, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  cudaGraphSetConditional(h, (kd->done == 0 && kd->its < kd->maxit) ? 1u : 0u);
}

// column kk of the Hessenberg matrix from the Gram-Schmidt coefficients (one
// or two passes, summed; hd[8..], hd[8 + kMaxRestart..]) and ||w||^2 (hd[2]);
// the earlier rotations applied to it, a new rotation zeroing its subdiagonal
// entry, the residual estimate |g_{kk+1}| / ||rhs||.  The same operations as
// the host's least-squares update.
__global__ void krylov_givens_kernel(KrylovDev* kd, const double* __restrict__ hd, int two_pass, int kk,
                                     KrylovStatus* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double* col = kd->Hm + (size_t)kk * (kMaxRestart + 1);
  const double* h1 = hd + 8;
  const double* h2 = hd + 8 + kMaxRestart;
  for (int i = 0; i <= kk; ++i) col[i] = h1[i] + (two_pass ? h2[i] : 0.0);
  const double hn = sqrt(hd[2]);
  col[kk + 1] = hn;
  for (int i = 0; i < kk; ++i) {
    const double a = col[i], b = col[i + 1];
    col[i] = kd->cs[i] * a + kd->sn[i] * b;
    col[i + 1] = -kd->sn[i] * a + kd->cs[i] * b;
  }
  const double a = col[kk], b = col[kk + 1];
  const double r = hypot(a, b);
  kd->cs[kk] = r > 0 ? a / r : 1.0;
  kd->sn[kk] = r > 0 ? b / r : 0.0;
  col[kk] = r;
  col[kk + 1] = 0.0;
  kd->gv[kk + 1] = -kd->sn[kk] * kd->gv[kk];
  kd->gv[kk] = kd->cs[kk] * kd->gv[kk];
  const double relres = fabs(kd->gv[kk + 1]) / kd->bnorm;
  const int bad = !isfinite(relres);
  kd->its += 1;
  kd->kk = kk + 1;
  kd->relres = relres;
  if (bad || relres <= kd->stop || hn == 0.0) kd->done = 1;
  kd->bad |= bad;
  status->relres = relres;
  status->its = kd->its;
  status->kk = kd->kk;
  status->done = kd->done;
  status->bad = kd->bad;
  __threadfence_system();
}

// back substitution for the coefficients of the cycle's kk basis vectors
// (to coef[0..kk)), and a final status for the host
__global__ void krylov_solve_kernel(KrylovDev* kd, double* coef, KrylovStatus* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int kk = kd->kk;
  for (int i = kk - 1; i >= 0; --i) {
    double sacc = kd->gv[i];
    for (int j = i + 1; j < kk; ++j) sacc -= kd->Hm[(size_t)j * (kMaxRestart + 1) + i] * kd->yv[j];
    kd->yv[i] = sacc / kd->Hm[(size_t)i * (kMaxRestart + 1) + i];
    coef[i] = kd->yv[i];
  }
  status->relres = kd->relres;
  status->its = kd->its;
  status->kk = kk;
  status->done = kd->done;
  status->bad = kd->bad;
  __threadfence_system();
}

// x += Z coef over the kk basis vectors the cycle used (kk read on the device)
template <typename T>
__global__ void combine_dev_kernel(long long n, const KrylovDev* __restrict__ kd, const T* __restrict__ Z,
                                   long long ldz, const double* __restrict__ coef, T* x,
                                   const T* __restrict__ dscl) {
  __shared__ T ys[kMaxRestart];
  const int m = kd->kk;
  if (threadIdx.x < m) ys[threadIdx.x] = (T)coef[threadIdx.x];
  __syncthreads();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const T* zk = Z + t;
  if (dscl) {
    x[t] += combine_sum<T>(ys, m, zk, ldz) / dscl[t];
    return;
  }
  T s = x[t];
  for (int k = 0; k < m; ++k, zk += ldz) s += ys[k] * *zk;
  x[t] = s;
}

unsigned long long graph_key(const OpConst& k, const SolveCfg& cfg) {
  unsigned long long h = 1469598103934665603ULL;
  auto mix = [&](double v) {
    unsigned long long b;
    std::memcpy(&b, &v, sizeof(b));
    h = (h ^ b) * 1099511628211ULL;
  };
  mix(cfg.omega_v); mix(cfg.omega_p); mix(cfg.nu); mix(cfg.nu_post); mix(cfg.coarse_sweeps); mix(cfg.coarse_cells); mix(cfg.small_cells); mix(cfg.nu_p); mix(cfg.gs_passes); mix(cfg.pdl ? 1.0 : 0.0); mix(cfg.tiled ? 1.0 : 0.0); mix(cfg.cmass); mix(cfg.kplane); mix((double)cfg.pfuse_cells); mix(cfg.stage_small ? 1.0 : 0.0); mix(cfg.direct_coarse ? 1.0 : 0.0); mix((double)cfg.learned); mix(cfg.row_block ? 1.0 : 0.0); mix((double)cfg.cluster_cells);
  mix(k.mms); mix(k.pin_u); mix(k.pin_p); mix(k.open_cnv); mix(k.sds); mix(k.top_cnv); mix(k.bot_cnv);
  return h | 1ULL;
}

template <typename T>
void drop_graphs(Hier<T>& H, int e) {
  for (int q = 0; q < kMaxRestart; ++q) {
    if (H.gexec[e][q]) { cudaGraphExecDestroy(H.gexec[e][q]); H.gexec[e][q] = nullptr; }
    if (H.cexec[e][q]) { cudaGraphExecDestroy(H.cexec[e][q]); H.cexec[e][q] = nullptr; }
  }
  H.gkey[e] = 0;
}

// Arnoldi step kk as a CUDA graph captured on first use (the buffers are fixed
// per context, so a graph stays valid across solves while the key holds)
template <typename T>
int arnoldi_step(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, int kk, cudaStream_t s) {
  const unsigned long long key = graph_key(k, cfg);
  int e = H.gkey[0] == key ? 0 : (H.gkey[1] == key ? 1 : -1);
  if (e < 0) {
    e = 1 - H.glast;   // replace the set used less recently
    drop_graphs(H, e);
    H.gkey[e] = key;
  }
  H.glast = e;
  cudaGraphExec_t* gexec = H.gexec[e];
  long long* gnodes = H.gnodes[e];
  if (!gexec[kk]) {
    cudaGraph_t graph = nullptr;
    XC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    // launches recorded into the graph run only when it is launched: count
    // them from this thread's counter and take them out of the totals
    const long long before = g_xc_thread_launches;
    int st = arnoldi_launches<T>(w, H, k, cfg, kk, s);
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (st != XC_OK) { if (graph) cudaGraphDestroy(graph); return st; }
    if (ce != cudaSuccess) { xc_set_error("graph capture failed: %s", cudaGetErrorString(ce)); return XC_CUDA; }
    gnodes[kk] = g_xc_thread_launches - before;
    g_xc_thread_launches = before;
    g_xc_launches.fetch_sub(gnodes[kk]);
    ce = cudaGraphInstantiate(&gexec[kk], graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) { gexec[kk] = nullptr; xc_set_error("graph instantiate: %s", cudaGetErrorString(ce)); return XC_CUDA; }
  }
  XC_CUDA_TRY(cudaGraphLaunch(gexec[kk], s));
  g_xc_launches.fetch_add(gnodes[kk]);
  return XC_OK;
}

// Arnoldi step kk as a conditional graph: a gate kernel sets the IF condition
// from the device least-squares state, and the body -- the step's launches
// without the host copy, then the Givens update -- runs only while the cycle
// goes on.  Returns XC_CUDA (with the reason) when the graph cannot be built.
template <typename T>
int build_cond_step(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, int kk, cudaStream_t s,
                    cudaGraphExec_t* exec, long long nodes[2]) {
  cudaGraph_t graph = nullptr;
  XC_CUDA_TRY(cudaGraphCreate(&graph, 0));
  auto fail = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    xc_set_error("conditional Arnoldi graph: %s: %s", what, cudaGetErrorString(e));
    return XC_CUDA;
  };
  cudaGraphConditionalHandle handle;
  cudaError_t e = cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return fail(e, "handle");
  KrylovDev* kd = H.kd;
  void* gate_args[2] = {&kd, &handle};
  cudaKernelNodeParams kp = {};
  kp.func = (void*)krylov_gate_kernel;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(32);
  kp.kernelParams = gate_args;
  cudaGraphNode_t gate;
  e = cudaGraphAddKernelNode(&gate, graph, nullptr, 0, &kp);
  if (e != cudaSuccess) return fail(e, "gate node");
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  e = cudaGraphAddNode(&cnode, graph, &gate, nullptr, 1, &cp);
  if (e != cudaSuccess) return fail(e, "conditional node");
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "capture");
  const long long before = g_xc_thread_launches;
  int st = arnoldi_launches<T>(w, H, k, cfg, kk, s, true, false);
  if (st == XC_OK) {
    krylov_givens_kernel<<<1, 32, 0, s>>>(H.kd, w->hdev, cfg.gs_passes > 1 ? 1 : 0, kk, H.ks_dev);
    xc_count_launch();
  }
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(s, &captured);
  nodes[0] = 1;
  nodes[1] = g_xc_thread_launches - before;
  g_xc_thread_launches = before;
  g_xc_launches.fetch_sub(nodes[1]);
  if (st != XC_OK) { cudaGraphDestroy(graph); return st; }
  if (e != cudaSuccess) return fail(e, "end capture");
  e = cudaGraphInstantiate(exec, graph, 0);
  if (e != cudaSuccess) { *exec = nullptr; return fail(e, "instantiate"); }
  cudaGraphDestroy(graph);
  return XC_OK;
}

// the conditional graph of step kk for this configuration, built on first use
template <typename T>
int cond_step(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, int kk, cudaStream_t s) {
  const unsigned long long key = graph_key(k, cfg);
  int e = H.gkey[0] == key ? 0 : (H.gkey[1] == key ? 1 : -1);
  if (e < 0) {
    e = 1 - H.glast;
    drop_graphs(H, e);
    H.gkey[e] = key;
  }
  H.glast = e;
  if (!H.cexec[e][kk]) XC_TRY(build_cond_step<T>(w, H, k, cfg, kk, s, &H.cexec[e][kk], H.cnodes[e][kk]));
  XC_CUDA_TRY(cudaGraphLaunch(H.cexec[e][kk], s));
  g_xc_launches.fetch_add(H.cnodes[e][kk][0]);
  return XC_OK;
}

// Hessenberg least-squares problem of (F)GMRES, on the host: one Givens
// rotation per new column, the residual estimate |g_{k+1}|, back substitution.
struct HessLS {
  int m;
  std::vector<double> Hm, cs, sn, gv, yv;
  explicit HessLS(int m_) : m(m_), Hm((size_t)(m_ + 1) * m_), cs(m_), sn(m_), gv(m_ + 1), yv(m_) {}
  void start(double beta) {
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
  }
  // column kk from the Gram-Schmidt coefficients (one or two passes, summed)
  // and ||w||; returns the new residual estimate |g_{kk+1}|
  double add(int kk, const double* h1, const double* h2, double hn) {
    double* col = &Hm[(size_t)kk * (m + 1)];
    for (int i = 0; i <= kk; ++i) col[i] = h1[i] + (h2 ? h2[i] : 0.0);
    col[kk + 1] = hn;
    for (int i = 0; i < kk; ++i) {
      double a = col[i], b = col[i + 1];
      col[i] = cs[i] * a + sn[i] * b;
      col[i + 1] = -sn[i] * a + cs[i] * b;
    }
    double a = col[kk], b = col[kk + 1];
    double r = std::hypot(a, b);
    cs[kk] = r > 0 ? a / r : 1.0;
    sn[kk] = r > 0 ? b / r : 0.0;
    col[kk] = r;
    col[kk + 1] = 0.0;
    gv[kk + 1] = -sn[kk] * gv[kk];
    gv[kk] = cs[kk] * gv[kk];
    return std::fabs(gv[kk + 1]);
  }
  // coefficients of the first kk basis vectors -> yv
  void solve(int kk) {
    for (int i = kk - 1; i >= 0; --i) {
      double sacc = gv[i];
      for (int j = i + 1; j < kk; ++j) sacc -= Hm[(size_t)j * (m + 1) + i] * yv[j];
      yv[i] = sacc / Hm[(size_t)i * (m + 1) + i];
    }
  }
};

// fgmres flags.  FG_ZERO_GUESS: start from y = 0 (set here), so the first
// residual is rhs itself and no operator application is needed.  FG_TRUST_EST:
// stop on the Givens estimate without recomputing the true residual (an inner
// solve whose caller forms the exact FP64 residual anyway).
constexpr int FG_ZERO_GUESS = 1;
constexpr int FG_TRUST_EST = 2;

// Right-preconditioned FGMRES(m) on the scaled system S LL S y = rhs, from the
// initial guess in H.y (updated in place).  *its_out = iterations used,
// *relres_out = ||rhs - A y|| / ||rhs|| of the true residual at the last restart
// (the estimate under FG_TRUST_EST).
// rhs_norm2 >= 0 (with FG_ZERO_GUESS): ||rhs||^2 is known on the host and its
// reciprocal root already sits in hdev[6] (the FP64 norm of the residual the
// FP32 rhs was rounded from), so no reduction or synchronisation is needed
template <typename T>
int fgmres(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, const T* rhs, double rtol,
           int maxit, int* its_out, double* relres_out, cudaStream_t s, int flags = 0, double rhs_norm2 = -1.0) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  const int m = H.m;
  double* hh = w->hhost;
  const bool zero = (flags & FG_ZERO_GUESS) != 0;
  const bool known = zero && rhs_norm2 >= 0.0;
  if (!known) XC_TRY(dot_self<T>(w, H, rhs, n, 0, s));
  if (zero) {
    XC_CUDA_TRY(cudaMemsetAsync(H.y, 0, sizeof(T) * n, s));
    // V[0] = rhs / ||rhs|| with the reciprocal left on the device
    scale_kernel<T><<<nblk(n), 256, 0, s>>>(n, w->hdev + 6, rhs, H.V); xc_count_launch();
  }
  double rhs2 = rhs_norm2;
  if (!known) {
    XC_CUDA_TRY(cudaMemcpyAsync(hh, w->hdev, sizeof(double), cudaMemcpyDeviceToHost, s));
    XC_CUDA_TRY(cudaStreamSynchronize(s));
    rhs2 = hh[0];
  }
  const double bnorm = std::sqrt(rhs2) > 0 ? std::sqrt(rhs2) : 1.0;
  int its = 0;
  double relres = 1.0;
  HessLS ls(m);
  for (int cycle = 0;; ++cycle) {
    double beta;
    if (zero && cycle == 0) {
      beta = std::sqrt(rhs2);
      relres = beta > 0 ? 1.0 : 0.0;
      if (!(relres > rtol) || its >= maxit) break;
    } else {
      // r = rhs - A y  -> V[0]
      XC_TRY(apply_scaled<T>(w, H, k, H.y, rhs, H.V, s));
      XC_TRY(dot_self<T>(w, H, H.V, n, 0, s));
      XC_CUDA_TRY(cudaMemcpyAsync(hh, w->hdev, sizeof(double), cudaMemcpyDeviceToHost, s));
      XC_CUDA_TRY(cudaStreamSynchronize(s));
      beta = std::sqrt(hh[0]);
      relres = beta / bnorm;
      if (!(relres > rtol) || its >= maxit) break;
      if (!std::isfinite(beta)) { *its_out = its; *relres_out = relres; xc_set_error("fgmres: non-finite residual"); return XC_NAN; }
      scale_kernel<T><<<nblk(n), 256, 0, s>>>(n, w->hdev + 6, H.V, H.V); xc_count_launch();
    }
    if (cfg.device_givens && !H.cond_broken) {
      // the cycle with the least-squares problem on the device: the host
      // queues step kk + 1 before it looks at step kk's outcome, so the GPU
      // never waits for it; a step queued after the cycle stopped is skipped
      // by its gate
      krylov_start_kernel<<<1, 32, 0, s>>>(H.kd, beta, bnorm, rtol * 0.5, maxit, its);
      xc_count_launch();
      const int its0 = its;
      int launched = 0, st = XC_OK;
      for (int kk = 0; kk < m; ++kk) {
        st = cond_step<T>(w, H, k, cfg, kk, s);
        if (st != XC_OK) break;
        XC_CUDA_TRY(cudaEventRecord(H.kev[kk & 1], s));
        ++launched;
        if (kk >= 1) {
          XC_CUDA_TRY(cudaEventSynchronize(H.kev[(kk - 1) & 1]));
          const volatile KrylovStatus* ks = H.ks_host;
          if (ks->done || ks->its >= maxit) break;
        }
      }
      if (st != XC_OK && launched == 0 && its == its0) {
        // no conditional graph could be built (nothing ran): host Givens
        // for this hierarchy from now on
        H.cond_broken = true;
      } else {
        if (st != XC_OK) return st;
        krylov_solve_kernel<<<1, 32, 0, s>>>(H.kd, w->hdev + 8, H.ks_dev);
        xc_count_launch();
        combine_dev_kernel<T><<<nblk(n), 256, 0, s>>>(n, H.kd, H.Z, n, w->hdev + 8, H.y,
                                                      cfg.learned == 0 ? (const T*)H.scl : nullptr);
        xc_count_launch();
        XC_LAUNCH_CHECK();
        XC_CUDA_TRY(cudaStreamSynchronize(s));
        const volatile KrylovStatus* ks = H.ks_host;
        const int ran = ks->its - its0;
        const int e = H.glast;
        for (int q = 0; q < ran && q < m; ++q) g_xc_launches.fetch_add(H.cnodes[e][q][1]);
        w->dev_steps += ran;
        its = ks->its;
        relres = ks->relres;
        if (ks->bad) { xc_set_error("fgmres: breakdown"); *its_out = its; *relres_out = relres; return XC_NAN; }
        if ((flags & FG_TRUST_EST) && (relres <= rtol || its >= maxit)) break;
        continue;
      }
    }
    ls.start(beta);
    int kk = 0;
    for (; kk < m && its < maxit; ++kk) {
      // z_k = M v_k, v_{k+1} = A z_k orthogonalised and normalised, H column
      // copied to pinned host memory -- one CUDA graph launch per iteration
      XC_TRY(arnoldi_step<T>(w, H, k, cfg, kk, s));
      XC_CUDA_TRY(cudaStreamSynchronize(s));
      XC_LAUNCH_CHECK();
      const double hn = std::sqrt(hh[2]);
      ++its;
      relres = ls.add(kk, hh + 8, cfg.gs_passes > 1 ? hh + 8 + kMaxRestart : nullptr, hn) / bnorm;
      if (!std::isfinite(relres)) { xc_set_error("fgmres: breakdown"); return XC_NAN; }
      if (relres <= rtol * 0.5 || hn == 0.0) { ++kk; break; }
    }
    // back substitution and update y += Z yv
    ls.solve(kk);
    XC_CUDA_TRY(cudaMemcpyAsync(w->hdev + 8, ls.yv.data(), sizeof(double) * kk, cudaMemcpyHostToDevice, s));
    combine_kernel<T><<<nblk(n), 256, 0, s>>>(n, kk, H.Z, n, w->hdev + 8, H.y,
                                              cfg.learned == 0 ? (const T*)H.scl : nullptr);
    xc_count_launch();
    XC_LAUNCH_CHECK();
    if ((flags & FG_TRUST_EST) && (relres <= rtol || its >= maxit)) break;
  }
  *its_out = its;
  *relres_out = relres;
  return XC_OK;
}

// The mixed solver's outer loop as FGMRES(m) in FP64 on S LL S y = rhs (from
// the initial guess in d.y), preconditioned by the whole FP32 inner solve:
// z_k = inner FGMRES on v_k to a reduction of inner_rtol, then w = A z_k
// orthogonalised in FP64.  Unlike plain refinement (y += inner(r) per pass)
// it keeps every correction and combines them by the FP64 least-squares
// problem.  *its_out counts FP32 inner iterations, *outer_out inner solves.
int fgmres_outer(StokesWork* w, const OpConst& k, const SolveCfg& cfg, const SolveCfg& icfg, const double* rhs,
                 double rtol, int maxit, double inner_rtol, int inner_maxit, int* its_out, int* outer_out,
                 double* relres_out, cudaStream_t s) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  Hier<double>& H = w->d;
  const int m = H.m;
  double* hh = w->hhost;
  XC_TRY(dot_self<double>(w, H, rhs, n, 0, s));
  XC_CUDA_TRY(cudaMemcpyAsync(hh, w->hdev, sizeof(double), cudaMemcpyDeviceToHost, s));
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  const double bnorm = std::sqrt(hh[0]) > 0 ? std::sqrt(hh[0]) : 1.0;
  int its = 0, outer = 0;
  double relres = 1.0;
  HessLS ls(m);
  int status = XC_OK;
  while (status == XC_OK) {
    XC_TRY(apply_scaled<double>(w, H, k, H.y, rhs, H.V, s));
    XC_TRY(dot_self<double>(w, H, H.V, n, 0, s));
    XC_CUDA_TRY(cudaMemcpyAsync(hh, w->hdev, sizeof(double), cudaMemcpyDeviceToHost, s));
    XC_CUDA_TRY(cudaStreamSynchronize(s));
    const double beta = std::sqrt(hh[0]);
    relres = beta / bnorm;
    if (!std::isfinite(relres)) { xc_set_error("mixed solver: non-finite residual"); status = XC_NAN; break; }
    if (relres <= rtol || its >= maxit || outer >= 50) break;
    scale_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->hdev + 6, H.V, H.V); xc_count_launch();
    ls.start(beta);
    int kk = 0;
    for (; kk < m && its < maxit && outer < 50; ++kk) {
      double* vk = H.V + (size_t)kk * n;
      double* zk = H.Z + (size_t)kk * n;
      convert_kernel<double, float><<<nblk(n), 256, 0, s>>>(n, vk, w->f.w); xc_count_launch();
      int iits = 0;
      double irr = 1.0;
      XC_TRY(fgmres<float>(w, w->f, k, icfg, w->f.w, inner_rtol, inner_maxit, &iits, &irr, s,
                           FG_ZERO_GUESS | FG_TRUST_EST));
      its += iits;
      ++outer;
      convert_kernel<float, double><<<nblk(n), 256, 0, s>>>(n, w->f.y, zk); xc_count_launch();
      XC_TRY(arnoldi_launches<double>(w, H, k, cfg, kk, s, false));
      XC_CUDA_TRY(cudaStreamSynchronize(s));
      XC_LAUNCH_CHECK();
      const double hn = std::sqrt(hh[2]);
      relres = ls.add(kk, hh + 8, cfg.gs_passes > 1 ? hh + 8 + kMaxRestart : nullptr, hn) / bnorm;
      if (!std::isfinite(relres)) { xc_set_error("mixed solver: breakdown"); status = XC_NAN; ++kk; break; }
      // the FP64 Arnoldi relation makes the estimate accurate far below rtol;
      // the true residual above confirms it
      if (relres <= rtol * 0.9 || hn == 0.0) { ++kk; break; }
    }
    if (status != XC_OK) break;
    ls.solve(kk);
    XC_CUDA_TRY(cudaMemcpyAsync(w->hdev + 8, ls.yv.data(), sizeof(double) * kk, cudaMemcpyHostToDevice, s));
    combine_kernel<double><<<nblk(n), 256, 0, s>>>(n, kk, H.Z, n, w->hdev + 8, H.y, (const double*)nullptr);
    xc_count_launch();
    XC_LAUNCH_CHECK();
  }
  *its_out = its;
  *outer_out = outer;
  *relres_out = relres;
  return status;
}

// build the operator coefficients and both multigrid hierarchies for one solve
// (mg = false: the fine-level operator only -- the FP64 hierarchy of a mixed
// solve, whose multigrid is not used)
template <typename T>
int setup_hier(StokesWork* w, Hier<T>& H, const OpConst& k, const SolveCfg& cfg, xc_ctx* c, cudaStream_t s,
               bool mg = true) {
  for (int l = 0; l < (mg ? H.nv : 1); ++l) {
    const Geo& lg = H.vg[l];
    const double* eta = l ? w->eta[l] : (const double*)c->field[FLD_eta];
    const double* etaco = l ? w->etaco[l] : (const double*)c->field[FLD_etaco];
    const double* rho = l ? w->rho[l] : (const double*)c->field[FLD_rho];
    const double* rhow = l ? w->rhow[l] : (const double*)c->field[FLD_rhow];
    const double* rhou = l ? w->rhou[l] : (const double*)c->field[FLD_rhou];
    OpConst kl = k;
    if (l) kl.mms = 0;
    if (kFly<T>) {
      const long long nt = std::max((long long)lg.NW + lg.NU, (long long)(lg.Nz + 1) * (lg.Nx + 1));
      fly_coef_kernel<T><<<nblk(nt), 256, 0, s>>>(lg, kl, eta, etaco, rho, rhow, rhou, H.feta[l], H.fetaco[l],
                                                  H.fdw[l], H.fdu[l], H.fdbot[l]); xc_count_launch();
    } else {
      vel_coef_kernel<T><<<nblk((long long)lg.NW + lg.NU), 256, 0, s>>>(lg, kl, eta, etaco, rho, rhow, rhou,
                                                                        H.cw[l], H.cu[l]); xc_count_launch();
    }
    XC_LAUNCH_CHECK();
  }
  // DM planes, scaling, eta/rho (double), converted for FP32
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  double* cpd = w->d.cp;
  if ((void*)&H == (void*)&w->d) {
    // the FP64 hierarchy is always set up first; the FP32 one converts its planes
    p_coef_kernel<<<nblk(g.NP), 256, 0, s>>>(g, (const double*)c->field[FLD_rhow],
                                             (const double*)c->field[FLD_rhou], cpd); xc_count_launch();
    XC_LAUNCH_CHECK();
  } else {
    convert_kernel<double, T><<<nblk(4LL * g.NP), 256, 0, s>>>(4LL * g.NP, cpd, H.cp); xc_count_launch();
    convert_kernel<double, T><<<nblk(n), 256, 0, s>>>(n, w->d.scl, H.scl); xc_count_launch();
    convert_kernel<double, T><<<nblk((long long)g.Nz * g.Nx), 256, 0, s>>>((long long)g.Nz * g.Nx, w->d.etarho,
                                                                          H.etarho); xc_count_launch();
  }
  if (!mg) return XC_OK;
  // pressure hierarchy
  p_kcoef_kernel<T><<<nblk((long long)(g.Nz + 1) * g.Nx), 256, 0, s>>>(
      g, (const double*)c->field[FLD_rhow], (const double*)c->field[FLD_rhou], w->d.cw[0], w->d.cu[0], cfg.kplane,
      H.kx[0], H.kz[0], H.kr); xc_count_launch();
  XC_LAUNCH_CHECK();
  H.pdpin[0] = (T)1.0;
  for (int l = 1; l < H.np_lv; ++l) {
    dim3 blk(32, 8);
    p_coarsen_kernel<T><<<grid2d(H.pNz[l] + 1, H.pNx[l], blk), blk, 0, s>>>(H.pNz[l], H.pNx[l], H.kx[l - 1],
                                                                            H.kz[l - 1], H.kx[l], H.kz[l]); xc_count_launch();
    H.pdpin[l] = H.pdpin[l - 1] / (T)4;
    XC_LAUNCH_CHECK();
  }
  // inverses of small coarsest levels
  int lv = 0, lp = 0;
  while (!vel_coarsest(H, cfg, lv)) ++lv;
  while (!p_coarsest(H, cfg, lp)) ++lp;
  H.vdirect = cfg.direct_coarse && (long long)H.vg[lv].NW + H.vg[lv].NU <= kDenseMax;
  H.pdirect = cfg.direct_coarse && (long long)H.pNz[lp] * H.pNx[lp] <= kDenseMax;
  if (H.vdirect) {
    vel_dense_inv_kernel<T><<<1, 256, 0, s>>>(H.vg[lv], level_const(k, lv), vop(H, lv), H.vinv, H.dok);
    xc_count_launch();
  }
  if (H.pdirect) {
    p_dense_inv_kernel<T><<<1, 256, 0, s>>>(H.pNz[lp], H.pNx[lp], H.kx[lp], H.kz[lp], H.ppin[lp], H.pdpin[lp],
                                             H.pinv, H.dok + 1);
    xc_count_launch();
  }
  XC_LAUNCH_CHECK();
  return XC_OK;
}

}  // namespace

int stokes_create(xc_ctx* c) {
  c->stokes = nullptr;
  if (c->Nz < 4 || c->Nx < 4) return XC_OK;   // no solver for tiny grids
  // the kernels index a level's unknowns with 32-bit integers
  if (3LL * (c->Nz + 2) * (c->Nx + 2) >= (1LL << 31)) {
    xc_set_error("stokes: grid %dx%d has too many unknowns for 32-bit indexing", c->Nz, c->Nx);
    return XC_BAD_ARG;
  }
  std::call_once(g_md_once, md_grid_init);
  // the one-CTA V-cycles stage their levels in up to kStageMaxBytes of shared memory
  cudaFuncSetAttribute(vel_vcycle_small_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageMaxBytes);
  cudaFuncSetAttribute(vel_vcycle_small_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageMaxBytes);
  cudaFuncSetAttribute(p_vcycle_small_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageMaxBytes);
  cudaFuncSetAttribute(p_vcycle_small_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageMaxBytes);
  XC_CUDA_TRY(cudaGetLastError());
  StokesWork* w = new StokesWork();
  std::memset((void*)w, 0, sizeof(StokesWork));
  c->stokes = w;
  w->g = make_geo(c->Nz, c->Nx, c->p.h);
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  XC_TRY(alloc_hier<double>(w, w->d, 30));
  for (int l = 1; l < w->d.nv; ++l) {
    const Geo& lg = w->d.vg[l];
    XC_CUDA_TRY(cudaMalloc(&w->eta[l], sizeof(double) * lg.Nz * lg.Nx));
    XC_CUDA_TRY(cudaMalloc(&w->etaco[l], sizeof(double) * (lg.Nz + 1) * (lg.Nx + 1)));
    XC_CUDA_TRY(cudaMalloc(&w->rho[l], sizeof(double) * lg.Nz * lg.Nx));
    XC_CUDA_TRY(cudaMalloc(&w->rhow[l], sizeof(double) * (lg.Nz + 1) * lg.Nx));
    XC_CUDA_TRY(cudaMalloc(&w->rhou[l], sizeof(double) * lg.Nz * (lg.Nx + 1)));
  }
  XC_CUDA_TRY(cudaMalloc(&w->RR, sizeof(double) * n));
  XC_CUDA_TRY(cudaMalloc(&w->x, sizeof(double) * n));
  XC_CUDA_TRY(cudaMalloc(&w->r, sizeof(double) * n));
  XC_CUDA_TRY(cudaMalloc(&w->part, sizeof(double) * KGMAX * (kMaxRestart + 1)));
  XC_CUDA_TRY(cudaMalloc(&w->hdev, sizeof(double) * (8 + 2 * kMaxRestart)));
  XC_CUDA_TRY(cudaMallocHost(&w->hhost, sizeof(double) * (8 + 2 * kMaxRestart + kMaxRestart)));
  const int Nz = g.Nz, Nx = g.Nx;
  XC_CUDA_TRY(cudaMalloc(&w->fz, sizeof(double) * (Nz - 1) * Nx));
  XC_CUDA_TRY(cudaMalloc(&w->uz, sizeof(double) * (Nz - 1) * (Nx + 1)));
  XC_CUDA_TRY(cudaMalloc(&w->wz, sizeof(double) * Nz * Nx));
  XC_CUDA_TRY(cudaMalloc(&w->fx, sizeof(double) * Nz * (Nx + 1)));
  XC_CUDA_TRY(cudaMalloc(&w->ux, sizeof(double) * Nz * (Nx + 2)));
  XC_CUDA_TRY(cudaMalloc(&w->wx, sizeof(double) * (Nz + 1) * (Nx + 1)));
  XC_CUDA_TRY(cudaMalloc(&w->advz, sizeof(double) * (Nz - 1) * Nx));
  XC_CUDA_TRY(cudaMalloc(&w->advx, sizeof(double) * Nz * (Nx + 1)));
  XC_CUDA_TRY(cudaEventCreate(&w->ev0));
  XC_CUDA_TRY(cudaEventCreate(&w->ev1));
  w->ok = true;
  return XC_OK;
}

void stokes_destroy(xc_ctx* c) {
  StokesWork* w = c->stokes;
  if (!w) return;
  free_hier<double>(w->d);
  if (w->f_alloc) free_hier<float>(w->f);
  for (int l = 1; l < kMaxLevels; ++l) {
    cudaFree(w->eta[l]); cudaFree(w->etaco[l]); cudaFree(w->rho[l]); cudaFree(w->rhow[l]); cudaFree(w->rhou[l]);
  }
  cudaFree(w->RR); cudaFree(w->x); cudaFree(w->r); cudaFree(w->part); cudaFree(w->hdev);
  cudaFreeHost(w->hhost);
  cudaFree(w->fz); cudaFree(w->uz); cudaFree(w->wz); cudaFree(w->fx); cudaFree(w->ux); cudaFree(w->wx);
  cudaFree(w->advz); cudaFree(w->advx); cudaFree(w->srcw); cudaFree(w->srcu); cudaFree(w->srcp);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  if (w->net) xc_nn_destroy(w->net);
  cudaFree(w->nn_in); cudaFree(w->nn_logeta); cudaFree(w->nn_r); cudaFree(w->nn_z); cudaFree(w->nn_xprev);
  cudaFree(w->nn_dv);
  delete w;
  c->stokes = nullptr;
}

// ---------------------------------------------------------------------------
// C ABI of the learned preconditioner
// ---------------------------------------------------------------------------
static int nn_buffers(StokesWork* w) {
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  if (!w->nn_in) XC_CUDA_TRY(cudaMalloc(&w->nn_in, sizeof(float) * (size_t)g.Nz * g.Nx * 4));
  if (!w->nn_logeta) XC_CUDA_TRY(cudaMalloc(&w->nn_logeta, sizeof(float) * (size_t)g.Nz * g.Nx));
  if (!w->nn_r) XC_CUDA_TRY(cudaMalloc(&w->nn_r, sizeof(float) * 2 * n));
  if (!w->nn_z) XC_CUDA_TRY(cudaMalloc(&w->nn_z, sizeof(float) * n));
  if (!w->nn_xprev) XC_CUDA_TRY(cudaMalloc(&w->nn_xprev, sizeof(double) * n));
  if (!w->nn_dv) XC_CUDA_TRY(cudaMalloc(&w->nn_dv, sizeof(double) * 2 * n));
  return XC_OK;
}

extern "C" int xc_set_learned_preconditioner(xc_ctx* c, const float* params, long long nparams) {
  if (!c || !c->stokes) { xc_set_error("xc_set_learned_preconditioner: no Stokes solver in this context"); return XC_BAD_ARG; }
  StokesWork* w = c->stokes;
  if (!params) {
    if (w->net) xc_nn_destroy(w->net);
    w->net = nullptr;
    return XC_OK;
  }
  if (!w->net) XC_TRY(xc_nn_create(c->Nz, c->Nx, 1, 4, 3, 0, &w->net));
  if (nparams != xc_nn_param_count(w->net)) {
    xc_set_error("xc_set_learned_preconditioner: %lld parameters given, the network has %lld", nparams,
                 xc_nn_param_count(w->net));
    return XC_BAD_ARG;
  }
  XC_TRY(xc_nn_set_params(w->net, params));
  XC_TRY(nn_buffers(w));
  // the FP32 inner graphs of the next solve are captured with the network
  return XC_OK;
}

extern "C" int xc_learned_sample(xc_ctx* c, const float* v, int after_vcycle, float* in, float* target,
                                 double rtol, int maxit, int* iterations) {
  if (!c || !c->stokes || !v || !in || !target) { xc_set_error("xc_learned_sample: null argument"); return XC_BAD_ARG; }
  StokesWork* w = c->stokes;
  if (!w->have_k || !w->last_fp64_mg) {
    xc_set_error("xc_learned_sample: needs a previous FP64 fluidmech solve on this context (its operator and multigrid)");
    return XC_BAD_ARG;
  }
  XC_TRY(nn_buffers(w));
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  const long long npx = (long long)g.Nz * g.Nx;
  cudaStream_t s = c->stream;
  nn_logeta_kernel<<<nblk(npx), 256, 0, s>>>(g.Nz, g.Nx, (const double*)c->field[FLD_eta], c->p.etam0,
                                             w->nn_logeta);
  xc_count_launch();
  convert_kernel<float, double><<<nblk(n), 256, 0, s>>>(n, v, w->d.w); xc_count_launch();
  XC_LAUNCH_CHECK();
  // the system solved: S LL S z = v, or for the V-cycle's residual
  // r = v - S LL S M(v) (M one FP64 V-cycle of the multigrid preconditioner)
  double* rhs = w->d.w;
  if (after_vcycle) {
    double* zmg = w->nn_dv;
    double* r = w->nn_dv + n;
    XC_TRY(precond<double>(w, w->d, w->last_k, w->last_cfg, w->d.w, zmg, s));
    XC_TRY(apply_scaled<double>(w, w->d, w->last_k, zmg, w->d.w, r, s));
    rhs = r;
  }
  int its = 0;
  double rr = 1.0;
  XC_TRY(fgmres<double>(w, w->d, w->last_k, w->last_cfg, rhs, rtol, maxit, &its, &rr, s, FG_ZERO_GUESS));
  // the input at unit norm, as every Krylov vector and every normalised
  // V-cycle residual enters the network
  XC_TRY(dot_self<double>(w, w->d, rhs, n, 5, s));
  nn_pack_kernel<double><<<nblk(npx), 256, 0, s>>>(g, rhs, w->nn_logeta, w->hdev + 6, sqrtf((float)npx), in, 4);
  xc_count_launch();
  XC_CUDA_TRY(cudaMemsetAsync(target, 0, sizeof(float) * npx * 3, s));
  nn_target_kernel<<<nblk(n), 256, 0, s>>>(g, w->d.y, target); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  if (iterations) *iterations = its;
  if (!(rr <= rtol)) {
    xc_set_error("xc_learned_sample: the FP64 solve stopped at %.3e after %d iterations", rr, its);
    return XC_NOT_CONVERGED;
  }
  return XC_OK;
}

extern "C" int xc_stokes_apply_scaled(xc_ctx* c, const float* v, float* y) {
  if (!c || !c->stokes || !v || !y) { xc_set_error("xc_stokes_apply_scaled: null argument"); return XC_BAD_ARG; }
  StokesWork* w = c->stokes;
  if (!w->have_k) { xc_set_error("xc_stokes_apply_scaled: needs a previous fluidmech solve"); return XC_BAD_ARG; }
  const Geo& g = w->g;
  const long long n = (long long)g.NW + g.NU + g.NP;
  cudaStream_t s = c->stream;
  convert_kernel<float, double><<<nblk(n), 256, 0, s>>>(n, v, w->d.w); xc_count_launch();
  XC_TRY(apply_scaled<double>(w, w->d, w->last_k, w->d.w, nullptr, w->d.V, s));
  convert_kernel<double, float><<<nblk(n), 256, 0, s>>>(n, w->d.V, y); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  return XC_OK;
}

int fluidmech_impl(xc_ctx* c, const double coefs[6], double dt, const xc_solver_opts* opts,
                   xc_solver_stats* stats, const MmsData* mms, const std::function<int()>* before_solve) {
  StokesWork* w = c->stokes;
  if (!w || !w->ok) { xc_set_error("fluidmech: grid too small for the Stokes solver (need Nz, Nx >= 4)"); return XC_BAD_ARG; }
  xc_solver_opts o;
  if (opts) o = *opts;
  else {
    std::memset(&o, 0, sizeof(o));
    o.kind = XC_SOLVER_FGMRES_FP64; o.rtol = 1e-10; o.maxit = 500; o.restart = 30; o.inner_rtol = 1e-4; o.inner_maxit = 60;
  }
  if (o.restart < 2) o.restart = 30;
  if (o.restart > 30) o.restart = 30;
  const Geo& g = w->g;
  const int Nz = g.Nz, Nx = g.Nx;
  const long long n = (long long)g.NW + g.NU + g.NP;
  cudaStream_t s = c->stream;
  const xc_params& p = c->p;
  w->dev_steps = 0;
  XC_CUDA_TRY(cudaEventRecord(w->ev0, s));
  dim3 blk(32, 8);
  // MFS update + mean (fluidmech.jl:115-127)
  if (!mms) {
    mfs_kernel<<<grid2d(Nz, Nx, blk), blk, 0, s>>>(Nz, Nx, coefs[0], coefs[1], coefs[2], coefs[3], coefs[4], coefs[5],
                                                   dt, p.alpha, CF(c, FLD_rho), CF(c, FLD_rhoo), CF(c, FLD_rhooo),
                                                   CF(c, FLD_advn_rho), F(c, FLD_drhodt), CF(c, FLD_drhodto),
                                                   CF(c, FLD_drhodtoo), F(c, FLD_MFS)); xc_count_launch();
    XC_LAUNCH_CHECK();
  }
  XC_TRY(reduce_to(c, RED_SUM, CF(c, FLD_MFS), CView{nullptr, 0}, nullptr, Nz, Nx, c->dscal + SC_MFS_MEAN, s,
                   (double)Nz * (double)Nx));
  // momentum advection of the current W, U (fluidmech.jl:236-240, 310-318)
  mom_prep_kernel<<<grid2d(Nz + 1, Nx + 2, blk), blk, 0, s>>>(Nz, Nx, CF(c, FLD_W), CF(c, FLD_U), CF(c, FLD_rhow),
                                                              CF(c, FLD_rhou), w->fz, w->uz, w->wz, w->fx, w->ux,
                                                              w->wx); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_TRY(stencil_advect_flux(w->fz, Nz - 1, false, Nz - 1, Nx, advect_scheme(p.ADVN, p), p.xBC, p.zBC, CView{w->uz, Nz - 1},
                             CView{w->wz, Nz}, p.h, DView{w->advz, Nz - 1}, DView{nullptr, 0}, DView{nullptr, 0}, s));
  XC_TRY(stencil_advect_flux(w->fx, Nz, false, Nz, Nx + 1, advect_scheme(p.ADVN, p), p.xBC, p.zBC, CView{w->ux, Nz},
                             CView{w->wx, Nz + 1}, p.h, DView{w->advx, Nz}, DView{nullptr, 0}, DView{nullptr, 0}, s));
  // operator constants
  OpConst k;
  k.a1 = coefs[0]; k.gamma = p.gamma; k.dt = dt; k.g0 = p.g0; k.idt = 1.0 / dt;
  k.sds = p.sds; k.top_cnv = p.top_cnv; k.bot_cnv = p.bot_cnv;
  k.sailor = mms ? 0 : 1;
  k.mms = mms ? 1 : 0;
  k.open_cnv = c->p.open_cnv ? 1 : 0;
  if (mms && k.open_cnv) {
    xc_set_error("fluidmech: the MMS branch with open_cnv = true is not supported");
    return XC_BAD_ARG;
  }
  int pin_z, pin_x;
  double pin_p_val = 0, pin_u_val = 0;
  k.pin_u = -1;
  if (mms) {
    pin_z = (int)std::nearbyint((Nz + 2) * 3.0 / 8.0) - 1;
    pin_x = (int)std::nearbyint((Nx + 2) / 2.0) - 1;
    int uz_ = (int)std::nearbyint((Nz + 2) / 2.0) - 1, ux_ = (int)std::nearbyint((Nx + 2) / 2.0) - 1;
    k.pin_u = ux_ * (Nz + 2) + uz_;
    pin_p_val = mms->P_exact[(size_t)pin_x * (Nz + 2) + pin_z];
    pin_u_val = mms->U_exact[(size_t)ux_ * (Nz + 2) + uz_];
  } else {
    pin_z = (int)std::nearbyint(Nz / 2.0) - 1;
    pin_x = (int)std::nearbyint(Nx / 2.0) - 1;
  }
  // the pressure pin: one interior cell, or (open bottom) the whole last
  // interior row of P, which p_row and scl_kernel handle (fluidmech.jl:426-429,
  // 478-487)
  k.pin_p = k.open_cnv ? -1 : pin_x * (Nz + 2) + pin_z;
  // RHS
  if (mms) {
    if (!w->srcw) {
      XC_CUDA_TRY(cudaMalloc(&w->srcw, sizeof(double) * g.NW));
      XC_CUDA_TRY(cudaMalloc(&w->srcu, sizeof(double) * g.NU));
      XC_CUDA_TRY(cudaMalloc(&w->srcp, sizeof(double) * g.NP));
    }
    XC_CUDA_TRY(cudaMemcpyAsync(w->srcw, mms->src_W, sizeof(double) * g.NW, cudaMemcpyHostToDevice, s));
    XC_CUDA_TRY(cudaMemcpyAsync(w->srcu, mms->src_U, sizeof(double) * g.NU, cudaMemcpyHostToDevice, s));
    XC_CUDA_TRY(cudaMemcpyAsync(w->srcp, mms->src_P, sizeof(double) * g.NP, cudaMemcpyHostToDevice, s));
  }
  RhsArgs ra{coefs[0], coefs[1], coefs[2], dt, p.g0, p.D, p.h, k.open_cnv ? 1.0 : 0.0, 1.0 / dt, mms ? 1 : 0, k.pin_p,
             k.pin_u};
  rhs_kernel<<<nblk(n), 256, 0, s>>>(g, ra, CF(c, FLD_Drho), CF(c, FLD_rhoWo), CF(c, FLD_rhoWoo), CF(c, FLD_rhoUo),
                                     CF(c, FLD_rhoUoo), CF(c, FLD_MFS), w->advz, w->advx, c->dscal + SC_MFS_MEAN,
                                     w->srcw, w->srcu, w->srcp, pin_p_val, pin_u_val, w->RR); xc_count_launch();
  XC_LAUNCH_CHECK();
  // coarse coefficient fields
  for (int l = 1; l < w->d.nv; ++l) {
    const Geo& lg = w->d.vg[l];
    const double* eta = l > 1 ? w->eta[l - 1] : (const double*)c->field[FLD_eta];
    const double* etaco = l > 1 ? w->etaco[l - 1] : (const double*)c->field[FLD_etaco];
    const double* rho = l > 1 ? w->rho[l - 1] : (const double*)c->field[FLD_rho];
    const double* rhow = l > 1 ? w->rhow[l - 1] : (const double*)c->field[FLD_rhow];
    const double* rhou = l > 1 ? w->rhou[l - 1] : (const double*)c->field[FLD_rhou];
    coarsen_fields_kernel<<<grid2d(lg.Nz + 1, lg.Nx + 1, blk), blk, 0, s>>>(
        lg.Nz, lg.Nx, eta, etaco, rho, rhow, rhou, w->eta[l], w->etaco[l], w->rho[l], w->rhow[l], w->rhou[l],
        o.coarse_viscosity_mean); xc_count_launch();
    XC_LAUNCH_CHECK();
  }
  SolveCfg cfg;
  // The manufactured-solution system is the inertia-free limit, where damped
  // Jacobi smooths the grad-div coupled viscous rows poorly: four sweeps per
  // level and long Jacobi runs on a 16x16 coarsest level converge in about a
  // third of the iterations of the defaults there.
  if (mms) { cfg.nu = 4; cfg.nu_post = 4; cfg.coarse_cells = 256; cfg.coarse_sweeps = 200; }
  if (o.smooth_sweeps > 0) cfg.nu = cfg.nu_post = o.smooth_sweeps;
  if (o.post_sweeps > 0) cfg.nu_post = o.post_sweeps;
  if (o.omega_velocity > 0) cfg.omega_v = o.omega_velocity;
  if (o.schur_full_diagonal) { cfg.kplane = 0; cfg.cmass = 0.0; }
  if (o.schur_mass > 0) cfg.cmass = o.schur_mass;
  if (o.coarse_cells > 0) cfg.coarse_cells = o.coarse_cells;
  if (o.coarse_sweeps > 0) cfg.coarse_sweeps = o.coarse_sweeps;
  if (o.small_cells != 0) cfg.small_cells = o.small_cells;
  if (o.pressure_sweeps > 0) cfg.nu_p = o.pressure_sweeps;
  cfg.pdl = !o.serial_launch;
  cfg.tiled = o.tiled_sweep != 0;
  cfg.row_block = o.row_block_sweep != 0;
  cfg.device_givens = o.device_givens != 0;
  cfg.cluster_cells = o.cluster_cells < 0 ? 0 : (o.cluster_cells > 0 ? o.cluster_cells : 0);
  cfg.stage_small = o.stage_small_levels != 0;
  cfg.direct_coarse = !o.jacobi_coarse;
  if (o.fused_pressure_cells != 0) cfg.pfuse_cells = o.fused_pressure_cells < 0 ? 0 : o.fused_pressure_cells;
  g_xc_pdl = cfg.pdl;
  // the FP32 inner solve only has to reduce its residual by inner_rtol (1e-2
  // to 3e-2 with at most ~30 basis vectors), so one Gram-Schmidt pass does;
  // the FP64 solve keeps two
  SolveCfg icfg = cfg;
  icfg.gs_passes = o.inner_gs_passes >= 2 ? 2 : 1;
  // learned preconditioner of the FP32 inner solves (plain refinement only)
  SolveCfg icfg_nn = icfg;
  if (o.learned != 0) {
    if (o.learned != 1 && o.learned != 2) { xc_set_error("fluidmech: learned must be 0, 1 or 2"); return XC_BAD_ARG; }
    if (o.kind != XC_SOLVER_MIXED || o.outer_solver == 1 || mms) {
      xc_set_error("fluidmech: the learned preconditioner serves the mixed solver's plain refinement only");
      return XC_BAD_ARG;
    }
    if (!w->net) {
      xc_set_error("fluidmech: no learned preconditioner set (xc_set_learned_preconditioner)");
      return XC_BAD_ARG;
    }
    icfg_nn.learned = o.learned;
  }
  w->last_k = k;
  w->have_k = true;
  w->last_cfg = cfg;
  w->last_fp64_mg = o.kind != XC_SOLVER_MIXED;
  XC_TRY(setup_hier<double>(w, w->d, k, cfg, c, s, o.kind != XC_SOLVER_MIXED));
  if (o.learned != 0) {
    nn_logeta_kernel<<<nblk((long long)Nz * Nx), 256, 0, s>>>(Nz, Nx, (const double*)c->field[FLD_eta], p.etam0,
                                                             w->nn_logeta);
    xc_count_launch();
    XC_LAUNCH_CHECK();
  }
  int fallbacks = 0;
  scl_kernel<<<nblk(n), 256, 0, s>>>(g, k, w->d.cw[0], w->d.cu[0], CF(c, FLD_rho), CF(c, FLD_eta), w->d.scl,
                                     w->d.etarho); xc_count_launch();
  XC_LAUNCH_CHECK();
  // initial guess: the current W, U, P
  pack_kernel<<<nblk(n), 256, 0, s>>>(g, CF(c, FLD_W), CF(c, FLD_U), CF(c, FLD_P), w->x); xc_count_launch();
  XC_LAUNCH_CHECK();
  int its = 0, refinements = 0;
  double relres = 1.0;
  int status = XC_OK;
  // scaled rhs S RR -> r (double)
  mul_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->RR, w->d.scl, w->r); xc_count_launch();
  if (o.kind == XC_SOLVER_MIXED) {
    if (!w->f_alloc) { XC_TRY(alloc_hier<float>(w, w->f, 30)); w->f_alloc = true; }
    XC_TRY(setup_hier<float>(w, w->f, k, cfg, c, s));
    if (before_solve) XC_TRY((*before_solve)());
    if (o.outer_solver == 1) {
      div_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->x, w->d.scl, w->d.y); xc_count_launch();
      status = fgmres_outer(w, k, cfg, icfg, w->r, o.rtol, o.maxit, o.inner_rtol, o.inner_maxit, &its,
                            &refinements, &relres, s);
      mul_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->d.y, w->d.scl, w->x); xc_count_launch();
      XC_LAUNCH_CHECK();
    } else {
    // plain refinement: FP64 norm of the scaled rhs
    XC_TRY(dot_self<double>(w, w->d, w->r, n, 3, s));
    XC_CUDA_TRY(cudaMemcpyAsync(w->hhost, w->hdev, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
    XC_CUDA_TRY(cudaStreamSynchronize(s));
    const double bn = std::sqrt(w->hhost[3]) > 0 ? std::sqrt(w->hhost[3]) : 1.0;
    // the FP64 operator reuses d.V[0] as residual storage
    double* res = w->d.V;
    // the learned preconditioner serves a pass only while its passes at
    // least halve the FP64 residual; the multigrid takes the rest of the solve
    bool learned_on = o.learned != 0, judge = false;
    double relres_before = 0.0;
    for (int outer = 0; outer < 50; ++outer) {
      // res = S RR - S LL x (FP64), the operator applied to the physical x
      pdl(PDL_ON, stokes_apply_kernel<double>, grid2(g), blk2(), s, g, k, vop(w->d, 0), w->d.cp, w->d.scl, w->x,
          (const double*)w->r, res);
      XC_LAUNCH_CHECK();
      XC_TRY(dot_self<double>(w, w->d, res, n, 3, s));
      XC_CUDA_TRY(cudaMemcpyAsync(w->hhost, w->hdev, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
      XC_CUDA_TRY(cudaStreamSynchronize(s));
      relres = std::sqrt(w->hhost[3]) / bn;
      if (judge) {
        judge = false;
        if (!(relres <= 0.5 * relres_before)) {
          // restore the iterate of before the pass and go on without the network
          XC_CUDA_TRY(cudaMemcpyAsync(w->x, w->nn_xprev, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
          learned_on = false;
          ++fallbacks;
          continue;
        }
      }
      if (!std::isfinite(relres)) { xc_set_error("mixed solver: non-finite residual"); status = XC_NAN; break; }
      if (relres <= o.rtol || its >= o.maxit) break;
      ++refinements;
      // inner FP32 solve of S LL S dy = res from dy = 0.  Its right-hand side
      // lives in f.w, which the FP32 Krylov and multigrid code never writes
      // (f.t is the operator's scratch, f.V / f.Z the basis).
      convert_kernel<double, float><<<nblk(n), 256, 0, s>>>(n, res, w->f.w); xc_count_launch();
      const float* frhs = w->f.w;
      int iits = 0;
      double irr = 1.0;
      const double rn2 = w->hhost[3];
      if (learned_on) {
        XC_CUDA_TRY(cudaMemcpyAsync(w->nn_xprev, w->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        relres_before = relres;
        judge = true;
      }
      XC_TRY(fgmres<float>(w, w->f, k, learned_on ? icfg_nn : icfg, frhs, o.inner_rtol, o.inner_maxit, &iits,
                           &irr, s, FG_ZERO_GUESS | FG_TRUST_EST, rn2));
      its += iits;
      if (learned_on && !(irr <= o.inner_rtol)) {
        // the learned inner solve missed its reduction: the multigrid
        // preconditioner redoes this pass from zero and takes the rest of
        // the solve.  (Its right-hand side's norm is recomputed: the device
        // reciprocal the first attempt started from has been overwritten.)
        ++fallbacks;
        judge = false;
        learned_on = false;
        XC_TRY(fgmres<float>(w, w->f, k, icfg, frhs, o.inner_rtol, o.inner_maxit, &iits, &irr, s,
                             FG_ZERO_GUESS | FG_TRUST_EST, -1.0));
        its += iits;
      }
      refine_update_kernel<float><<<nblk(n), 256, 0, s>>>(n, w->f.y, w->d.scl, w->x); xc_count_launch();
      XC_LAUNCH_CHECK();
    }
    }
  } else {
    if (before_solve) XC_TRY((*before_solve)());
    div_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->x, w->d.scl, w->d.y); xc_count_launch();
    status = fgmres<double>(w, w->d, k, cfg, w->r, o.rtol, o.maxit, &its, &relres, s);
    mul_kernel<double><<<nblk(n), 256, 0, s>>>(n, w->d.y, w->d.scl, w->x); xc_count_launch();
    // true FP64 residual of the final iterate
    if (status == XC_OK) {
      XC_TRY(apply_scaled<double>(w, w->d, k, w->d.y, w->r, w->d.V, s));
      XC_TRY(dot_self<double>(w, w->d, w->d.V, n, 3, s));
      XC_TRY(dot_self<double>(w, w->d, w->r, n, 4, s));
      XC_CUDA_TRY(cudaMemcpyAsync(w->hhost, w->hdev, sizeof(double) * 5, cudaMemcpyDeviceToHost, s));
      XC_CUDA_TRY(cudaStreamSynchronize(s));
      relres = std::sqrt(w->hhost[3]) / (std::sqrt(w->hhost[4]) > 0 ? std::sqrt(w->hhost[4]) : 1.0);
    }
  }
  unpack_kernel<<<nblk(n), 256, 0, s>>>(g, w->x, F(c, FLD_W), F(c, FLD_U), F(c, FLD_P)); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_CUDA_TRY(cudaEventRecord(w->ev1, s));
  XC_CUDA_TRY(cudaEventSynchronize(w->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, w->ev0, w->ev1);
  if (stats) {
    stats->iterations = its;
    stats->refinements = refinements;
    stats->rel_residual = relres;
    stats->converged = relres <= o.rtol;
    stats->seconds = ms * 1e-3;
    stats->learned_fallbacks = fallbacks;
    stats->device_givens_steps = (int)w->dev_steps;
  }
  if (o.learned != 0) XC_TRY(nn_check(w->net, s));
  if (status != XC_OK) return status;
  if (!(relres <= o.rtol)) {
    xc_set_error("fluidmech: not converged, relative residual %.3e after %d iterations", relres, its);
    return XC_NOT_CONVERGED;
  }
  return XC_OK;
}

// CUDA-event timing of one solver kernel on the last solve's operator
// Timing of the fine-level Jacobi sweep on copies of its operands (viscosity
// fields or coefficient planes, unknowns, right-hand side, result) that
// together exceed twice the L2: launches cycle through the copies back to back,
// so each reads operands the others have evicted and no launch gap is timed.
template <typename T>
int sweep_bench(cudaStream_t s, const Geo& g, const OpConst& k, const Hier<T>& H, int iters, float* ms_out,
                bool row_block = false) {
  const size_t nvv = (size_t)g.NW + g.NU;
  std::vector<std::pair<const void*, size_t>> src;   // operand, bytes
  if (kFly<T>) {
    src = {{H.feta[0], sizeof(T) * g.Nz * g.Nx}, {H.fetaco[0], sizeof(T) * (g.Nz + 1) * (g.Nx + 1)},
           {H.fdw[0], sizeof(T) * g.NW}, {H.fdu[0], sizeof(T) * g.NU}};
  } else {
    src = {{H.cw[0], sizeof(T) * 10 * g.NW}, {H.cu[0], sizeof(T) * 10 * g.NU}};
  }
  src.push_back({H.vx[0], sizeof(T) * nvv});
  src.push_back({H.vb[0], sizeof(T) * nvv});
  src.push_back({H.vx2[0], sizeof(T) * nvv});
  size_t per_copy = 0;
  for (auto& a : src) per_copy += a.second;
  const size_t l2x2 = (size_t)2 * 132 * 1000 * 1000;
  const int nc = (int)std::max<size_t>(2, (l2x2 + per_copy - 1) / per_copy + 1);
  std::vector<std::vector<void*>> cp(nc, std::vector<void*>(src.size(), nullptr));
  int st = XC_OK;
  for (int q = 0; q < nc && st == XC_OK; ++q)
    for (size_t a = 0; a < src.size(); ++a) {
      if (cudaMalloc(&cp[q][a], src[a].second) != cudaSuccess ||
          cudaMemcpyAsync(cp[q][a], src[a].first, src[a].second, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        xc_set_error("xc_bench_kernel: operand copies: %s", cudaGetErrorString(cudaGetLastError()));
        st = XC_CUDA;
        break;
      }
    }
  auto op_of = [&](int q) {
    VOp<T> o{};
    const auto& v = cp[q];
    if (kFly<T>) {
      o.eta = (const T*)v[0]; o.etaco = (const T*)v[1]; o.dw = (const T*)v[2]; o.du = (const T*)v[3];
      o.dbot = H.fdbot[0];
    } else {
      o.cw = (const T*)v[0]; o.cu = (const T*)v[1];
    }
    return o;
  };
  const size_t xo = src.size() - 3;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (st == XC_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) st = XC_CUDA;
  if (st == XC_OK) {
    for (int it = -nc; it < iters; ++it) {   // one untimed pass over all copies first
      if (it == 0) cudaEventRecord(e0, s);
      const int q = ((it % nc) + nc) % nc;
      if constexpr (kFly<T>) {
        if (row_block) {
          vel_sweep_rb_kernel<1><<<grid_rb(g), blk2(), 0, s>>>(g, k, op_of(q), (const T*)cp[q][xo],
                                                               (const T*)cp[q][xo + 1], (T*)cp[q][xo + 2], (T)0.7,
                                                               (const T*)nullptr);
          xc_count_launch();
          continue;
        }
      }
      vel_sweep2d_kernel<T, 1><<<grid2(g), blk2(), 0, s>>>(g, k, op_of(q), (const T*)cp[q][xo],
                                                           (const T*)cp[q][xo + 1], (T*)cp[q][xo + 2], (T)0.7,
                                                           (const T*)nullptr);
      xc_count_launch();
    }
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      xc_set_error("xc_bench_kernel: %s", cudaGetErrorString(e));
      st = XC_CUDA;
    } else {
      cudaEventElapsedTime(ms_out, e0, e1);
      *ms_out /= (float)iters;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  for (auto& v : cp)
    for (void* p : v) cudaFree(p);
  return st;
}

int stokes_bench(xc_ctx* c, int which, int iters, double out[4]) {
  StokesWork* w = c->stokes;
  if (!w || !w->have_k || ((which == 2 || which == 5) && !w->f_alloc)) {
    xc_set_error("xc_bench_kernel: run xc_fluidmech (mixed for kernel 2) first");
    return XC_BAD_ARG;
  }
  const Geo& g = w->g;
  const OpConst& k = w->last_k;
  cudaStream_t s = c->stream;
  const double cells = (double)g.Nz * g.Nx;
  // algorithmic bytes: read the unknowns (W, U; and P for the apply) or the
  // unknowns and the right-hand side (W, U, bW, bU for a sweep) and the
  // operator's material fields (eta, etaco, rho, rhow, rhou), write the
  // result: 11 arrays, FP64 88 B/cell, FP32 44 B/cell
  out[1] = (which == 2 || which == 5 ? 44.0 : 88.0) * cells;
  out[2] = 52.0 * cells;            // 2 flops per stencil entry, ~26 entries per cell
  out[3] = cells;
  if (which == 2 || which == 3 || which == 5) {
    float ms = 0;
    XC_TRY(which == 3 ? sweep_bench<double>(s, g, k, w->d, iters, &ms)
                      : sweep_bench<float>(s, g, k, w->f, iters, &ms, which == 5));
    out[0] = ms;
    return XC_OK;
  }
  // the apply: every launch is timed alone after a write of 256 MiB (twice the
  // L2), so the time is that of a launch whose operands come from HBM
  const size_t flush_bytes = 256u << 20;
  void* flush = nullptr;
  XC_CUDA_TRY(cudaMalloc(&flush, flush_bytes));
  cudaEvent_t e0, e1;
  XC_CUDA_TRY(cudaEventCreate(&e0));
  XC_CUDA_TRY(cudaEventCreate(&e1));
  double total_ms = 0;
  for (int it = -1; it < iters; ++it) {
    cudaMemsetAsync(flush, it & 0xff, flush_bytes, s);
    cudaEventRecord(e0, s);
    stokes_apply_kernel<double><<<grid2(g), blk2(), 0, s>>>(g, k, vop(w->d, 0), w->d.cp, w->d.scl, w->d.t,
                                                            nullptr, w->d.w); xc_count_launch();
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaFree(flush);
      xc_set_error("xc_bench_kernel: %s", cudaGetErrorString(e));
      return XC_CUDA;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (it >= 0) total_ms += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(flush);
  XC_LAUNCH_CHECK();
  out[0] = total_ms / iters;
  return XC_OK;
}
