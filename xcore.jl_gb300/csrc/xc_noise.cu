// noise! on the GPU: Ornstein-Uhlenbeck update, FFT Gaussian filter,
// re-standardisation, staggered differences, tapers and speed magnitudes.
//
// Reference: src/noise.jl:138-270 (and the NoiseState precompute 61-107).
//
// The filter.  compute_fft_filter (noise.jl:244-270) zero-pads psi by `pad`
// rows, applies exp(-s^2 (kz^2 + kx^2)) in 2-D Fourier space and unpads.  That
// spectrum is a product exp(-s^2 kz^2) * exp(-s^2 kx^2), so the operator is a
// z-direction circular convolution (period Nz+pad) followed by an x-direction
// circular convolution (period Nx), each with a real, even kernel c[d].  Only
// the Nz unpadded rows are kept and the input is zero outside them, so the
// z-pass is a linear convolution of the Nz-long column with c over lags
// |d| < Nz; it is evaluated exactly with a power-of-two FFT of length
// M >= 2 Nz - 1 (no wrap-around can reach the kept rows).  The x-pass uses a
// length-Nx FFT directly when Nx is a power of two (then the multiplier IS the
// reference's exp(-s^2 kx^2)), otherwise the same linear-convolution form.
// Two real lines are packed into one complex FFT (real kernel => the real and
// imaginary parts stay separate).  Mathematically this is the reference
// operator; the FFTs are hand-written radix-2 shared-memory transforms.
#include <cmath>
#include <complex>
#include <mutex>
#include <vector>

#include "xc_internal.cuh"

namespace {

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int next_pow2(int n) { int m = 1; while (m < n) m <<= 1; return m; }

// host radix-2 FFT (precompute only)
void host_fft(std::vector<std::complex<double>>& a) {
  const int n = (int)a.size();
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    for (int k = 0; k < len / 2; ++k) {
      double ang = -2.0 * M_PI * (double)k / (double)len;
      std::complex<double> w(std::cos(ang), std::sin(ang));
      for (int i = 0; i < n; i += len) {
        std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
    }
  }
}

// wavenumbers 2*pi*fftfreq(n, 1/h) (noise.jl:100-101, AbstractFFTs arithmetic)
std::vector<double> wavenumbers(int n, double h) {
  std::vector<double> k(n);
  int nn = (n + 1) >> 1;
  double mult = 2.0 * M_PI * ((1.0 / h) / (double)n);
  for (int i = 0; i < n; ++i) k[i] = (double)(i < nn ? i : i - n) * mult;
  return k;
}

}  // namespace

struct LineFilter {      // one 1-D convolution pass
  int L;                 // line length (input and output)
  int M;                 // FFT length
  int logM;
  double* khat;          // device, M real multipliers (already divided by M)
  double2* tw;           // device, M/2 twiddles exp(-2 pi i k / M)
};

struct NoisePlan {
  int padL0, padl0;
  double fL, fl;
  LineFilter ze, xe, zs, xs;   // e: sigma = L0h, pad = padL0; s: sigma = l0h, pad = padl0
};

namespace {

int build_line_filter(LineFilter& lf, int L, int period, double h, double sigma, bool direct_ok) {
  std::vector<double> kk = wavenumbers(period, h);
  std::vector<double> G(period);
  for (int k = 0; k < period; ++k) G[k] = std::exp(-(sigma * sigma) * (kk[k] * kk[k]));
  std::vector<double> khat;
  if (direct_ok && period == L && is_pow2(L)) {
    lf.M = L;
    khat = G;
  } else {
    lf.M = next_pow2(2 * L - 1);
    // circular kernel c[d] = (1/n) sum_k G(k) cos(2 pi k d / n), real and even
    std::vector<double> cd(L);
    for (int d = 0; d < L; ++d) {
      long double acc = 0.0L;
      for (int k = 0; k < period; ++k) {
        long long kd = ((long long)k * d) % period;
        acc += (long double)G[k] * std::cos(2.0L * (long double)M_PI * (long double)kd / (long double)period);
      }
      cd[d] = (double)(acc / (long double)period);
    }
    std::vector<std::complex<double>> kb(lf.M, 0.0);
    for (int d = 0; d < L; ++d) kb[d] = cd[d % period];
    for (int d = 1; d < L; ++d) kb[lf.M - d] = cd[d % period];
    host_fft(kb);
    khat.resize(lf.M);
    for (int k = 0; k < lf.M; ++k) khat[k] = kb[k].real();
  }
  lf.L = L;
  lf.logM = 0;
  while ((1 << lf.logM) < lf.M) ++lf.logM;
  for (auto& v : khat) v /= (double)lf.M;       // fold the inverse transform's 1/M
  std::vector<double2> tw(lf.M / 2 > 0 ? lf.M / 2 : 1);
  for (int k = 0; k < lf.M / 2; ++k) {
    long double ang = -2.0L * (long double)M_PI * (long double)k / (long double)lf.M;
    tw[k] = make_double2((double)std::cos(ang), (double)std::sin(ang));
  }
  XC_CUDA_TRY(cudaMalloc(&lf.khat, sizeof(double) * lf.M));
  XC_CUDA_TRY(cudaMalloc(&lf.tw, sizeof(double2) * tw.size()));
  XC_CUDA_TRY(cudaMemcpy(lf.khat, khat.data(), sizeof(double) * lf.M, cudaMemcpyHostToDevice));
  XC_CUDA_TRY(cudaMemcpy(lf.tw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice));
  return XC_OK;
}

void free_line_filter(LineFilter& lf) {
  if (lf.khat) cudaFree(lf.khat);
  if (lf.tw) cudaFree(lf.tw);
  lf.khat = nullptr;
  lf.tw = nullptr;
}

// complex product with two of its four products fused into FMAs (four FP64
// instructions instead of six; this file is otherwise compiled without FMA
// contraction, and the FFT's results are a different rounding of the
// reference's FFTW transform in any case)
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, -(a.y * b.y)), __fma_rn(a.x, b.y, a.y * b.x));
}

// in-place radix-2 DIT FFT of P transforms of length M stored back to back in
// shared memory (input in bit-reversed order); inverse = conjugated twiddles
__device__ void smem_fft(double2* buf, int P, int M, int logM, const double2* __restrict__ tw,
                         bool inverse) {
  const int nb = P * (M >> 1);
  for (int s = 1; s <= logM; ++s) {
    const int half = 1 << (s - 1);
    const int stride = M >> s;       // twiddle index step
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      int t = b / (M >> 1), r = b % (M >> 1);
      int grp = r / half, k = r % half;
      int i0 = t * M + grp * 2 * half + k;
      double2 w = tw[k * stride];
      if (inverse) w.y = -w.y;
      double2 u = buf[i0], v = cmul(buf[i0 + half], w);
      buf[i0] = make_double2(u.x + v.x, u.y + v.y);
      buf[i0 + half] = make_double2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

__device__ __forceinline__ int bitrev(int i, int logM) { return __brev(i) >> (32 - logM); }

// Filter lines of a column-major (rows x cols) array along `axis` (0: lines
// are columns of length rows; 1: lines are rows of length cols).  Each CTA
// takes P line pairs.  in and out may not alias.
__global__ void line_filter_kernel(CView in, DView out, int rows, int cols, int axis, int M,
                                   int logM, const double* __restrict__ khat,
                                   const double2* __restrict__ tw, int P) {
  XC_PDL_WAIT();
  extern __shared__ double2 buf[];
  const int L = axis == 0 ? rows : cols;
  const int nlines = axis == 0 ? cols : rows;
  const int pair0 = blockIdx.x * P;
  // load: line pair (2q, 2q+1) -> complex, bit-reversed positions
  for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
    int t = e / M, k = e % M;
    int la = 2 * (pair0 + t), lb = la + 1;
    double re = 0.0, im = 0.0;
    if (k < L) {
      if (axis == 0) {
        if (la < nlines) re = AT(in, k, la);
        if (lb < nlines) im = AT(in, k, lb);
      } else {
        if (la < nlines) re = AT(in, la, k);
        if (lb < nlines) im = AT(in, lb, k);
      }
    }
    buf[t * M + bitrev(k, logM)] = make_double2(re, im);
  }
  __syncthreads();
  smem_fft(buf, P, M, logM, tw, false);
  // multiply by the real spectrum, then bit-reverse in place for the inverse
  for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
    int k = e % M;
    double g = khat[k];
    buf[e].x *= g;
    buf[e].y *= g;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < P * M; e += blockDim.x) {
    int t = e / M, k = e % M, r = bitrev(k, logM);
    if (k < r) {
      double2 a = buf[t * M + k];
      buf[t * M + k] = buf[t * M + r];
      buf[t * M + r] = a;
    }
  }
  __syncthreads();
  smem_fft(buf, P, M, logM, tw, true);
  for (int e = threadIdx.x; e < P * L; e += blockDim.x) {
    int t = e / L, k = e % L;
    int la = 2 * (pair0 + t), lb = la + 1;
    double2 v = buf[t * M + k];
    if (axis == 0) {
      if (la < nlines) AT(out, k, la) = v.x;
      if (lb < nlines) AT(out, k, lb) = v.y;
    } else {
      if (la < nlines) AT(out, la, k) = v.x;
      if (lb < nlines) AT(out, lb, k) = v.y;
    }
  }
}

int run_line_filter(const LineFilter& lf, CView in, DView out, int rows, int cols, int axis,
                    cudaStream_t s) {
  const int nlines = axis == 0 ? cols : rows;
  const int npairs = (nlines + 1) / 2;
  int P = 1;
  while (P * 2 * lf.M * (int)sizeof(double2) <= 64 * 1024 && P * 2 <= 8) P *= 2;
  size_t smem = (size_t)P * lf.M * sizeof(double2);
  if (smem > 48 * 1024) {
    // set to the largest need seen so far, never lowered: a graph may hold
    // launches of several filter lengths, captured in any order
    static std::mutex mu;
    static size_t limit = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (smem > limit) limit = smem;
    XC_CUDA_TRY(cudaFuncSetAttribute(line_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  }
  int threads = lf.M * P >= 1024 ? 512 : 256;
  xc_launch(line_filter_kernel, (npairs + P - 1) / P, threads, smem, s, in, out, rows, cols, axis, lf.M,
                                                                 lf.logM, lf.khat, lf.tw, P);
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// OU update (noise.jl:160-183), one thread per cell
__global__ void ou_kernel(int Nz, int Nx, double Xi, double L0h, double i2L0h, double i2l0h, double txi0,
                          double dt, double cdt, double fL, double fl, CView V, CView vx, CView fReL, CView ke, CView chi,
                          CView ks, CView psieo, CView psixo, CView psiso, CView re, CView rs,
                          DView psie, DView psix, DView psis) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    // The reference's twelve divisions (noise.jl:160-176) folded to five with
    // the same values up to rounding (these fields carry the 1e-12 tolerance):
    // 1/tau_e = 2 (V + eps) / L0h and 1/tau_s = 2 (vx + eps) / l0h as
    // products, and tau' = 1 / (1/tau + c) + dt with c = 1 / (100 dt) entering
    // only as -dt / tau' = -dt u / (1 + dt u), u = 1/tau + c.  An FP64 division
    // costs about ten FP64 instructions on this GPU's narrow FP64 pipe.
    const double ve = AT(V, j, i) + XC_EPS, vs = AT(vx, j, i) + XC_EPS;
    const double taue = L0h / (2.0 * ve);
    const double itaue = ve * i2L0h, itaus = vs * i2l0h;   // i2L0h = 2 / L0h, i2l0h = 2 / l0h
    double St = txi0 / (taue + XC_EPS);
    double fr = AT(fReL, j, i), k = AT(ke, j, i), ch = AT(chi, j, i);
    double sge = Xi * sqrt(jmax(0.0, (fr * k) * itaue));
    double sgx = Xi * sqrt(jmax(0.0, ((((ch * fr) * k) * itaue) * St) / (1.0 + St * St)));
    double sgs = Xi * sqrt(jmax(0.0, (ch * AT(ks, j, i)) * itaus));
    const double ue = itaue + cdt, us = itaus + cdt;   // cdt = 1 / (100 dt)
    double Fte = exp(((-dt) * ue) / (1.0 + dt * ue)), Fts = exp(((-dt) * us) / (1.0 + dt * us));
    double ae = sqrt(jmax(0.0, 1.0 - Fte * Fte)), as = sqrt(jmax(0.0, 1.0 - Fts * Fts));
    double r1 = AT(re, j, i), r2 = AT(rs, j, i);
    AT(psie, j, i) = Fte * AT(psieo, j, i) + ((ae * sge) * fL) * r1;
    AT(psix, j, i) = Fte * AT(psixo, j, i) + ((ae * sgx) * fL) * r1;
    AT(psis, j, i) = Fts * AT(psiso, j, i) + ((as * sgs) * fl) * r2;
  });
}

// re-standardise to the raw mean/std (noise.jl:261-267); st = {raw mean,
// raw sum sq dev, flt mean, flt sum sq dev} per field
// (the two standard deviations, the same for every cell, are formed once per
// block by the same operations)
// (the ratio raw std / filtered std, the same for every cell, is formed once
// per block: the per-cell FP64 division of (v - mean) raw / flt becomes a
// product, within the 1e-12 tolerance of these fields)
__global__ void rescale_kernel(int Nz, int Nx, DView f0, DView f1, DView f2, const double* st) {
  XC_PDL_WAIT();
  __shared__ double ratio[3];
  __shared__ int use[3];
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const double nm1 = (double)Nz * (double)Nx - 1.0;
    for (int q = 0; q < 3; ++q) {
      const double raw_std = sqrt(st[4 * q + 1] / nm1), flt_std = sqrt(st[4 * q + 3] / nm1);
      use[q] = flt_std > XC_EPS;
      ratio[q] = raw_std / flt_std;
    }
  }
  __syncthreads();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (j >= Nz || i >= Nx) return;
  DView fs[3] = {f0, f1, f2};
  for (int q = 0; q < 3; ++q) {
    const double* s = st + 4 * q;
    if (use[q]) {
      double v = AT(fs[q], j, i);
      AT(fs[q], j, i) = ((v - s[2]) * ratio[q]) + s[0];
    }
  }
}

__device__ __forceinline__ int icz_c(int j, int Nz) { return j == 0 ? 0 : (j == Nz + 1 ? Nz - 1 : j - 1); }
__device__ __forceinline__ int icx_p(int i, int Nx) { return i == 0 ? Nx - 1 : (i == Nx + 1 ? 0 : i - 1); }

// grid.icz / grid.icx extension (closed z, periodic x: noise.jl:143-144)
__device__ __forceinline__ double ext(CView f, int a, int b, int Nz, int Nx) {
  return AT(f, icz_c(a, Nz), icx_p(b, Nx));
}
__device__ __forceinline__ double corner_avg(CView pe, int j, int i, int Nz, int Nx) {
  return (((ext(pe, j, i, Nz, Nx) + ext(pe, j, i + 1, Nz, Nx)) + ext(pe, j + 1, i, Nz, Nx)) +
          ext(pe, j + 1, i + 1, Nz, Nx)) / 4.0;
}

// staggered noise fluxes (noise.jl:195-220), one thread per (j, i) of (Nz+2, Nx+2)
// exp(y) where only 1 - exp(y) is used: below y = -38, exp(y) < 3.2e-17 is
// under half an ulp of 1 (2^-54), so 1 - exp(y) rounds to exactly 1.0 and
// the exponential -- some twenty FP64 instructions -- is skipped without
// changing a bit (the crystal-fraction taper, a / 1e-4 with a >= 0.004)
__device__ __forceinline__ double exp_tail(double y) { return y < -38.0 ? 0.0 : exp(y); }

__global__ void stagger_kernel(int Nz, int Nx, CView pe, CView px, CView ps, CView chiw,
                               CView muw, CView chiu, CView muu, DView xieu, DView xiew,
                               DView xixu, DView xixw, DView xisu, DView xisw) {
  XC_PDL_WAIT();
  for_tiles(Nz + 2, Nx + 2, [&](int j, int i) {
    if (j > Nz + 1 || i > Nx + 1) return;
    if (i <= Nx) {   // (Nz+2, Nx+1): xieu = xieu_int[icz, :], xixu, xisu
      int jj = icz_c(j, Nz);
      AT(xieu, j, i) = corner_avg(pe, jj + 1, i, Nz, Nx) - corner_avg(pe, jj, i, Nz, Nx);
      double a = AT(chiu, j, i), b = AT(muu, j, i);
      double tap = (1.0 - exp_tail((-a) / 1e-4)) * (1.0 - exp_tail((-jmax(0.0, b - 0.4)) / 0.05));
      AT(xixu, j, i) = (-(ext(px, j, i + 1, Nz, Nx) - ext(px, j, i, Nz, Nx))) * tap;
      AT(xisu, j, i) = (-(ext(ps, j, i + 1, Nz, Nx) - ext(ps, j, i, Nz, Nx))) * tap;
    }
    if (j <= Nz) {   // (Nz+1, Nx+2): xiew = xiew_int[:, icx], xixw, xisw
      int ii = icx_p(i, Nx);
      AT(xiew, j, i) = -(corner_avg(pe, j, ii + 1, Nz, Nx) - corner_avg(pe, j, ii, Nz, Nx));
      double a = AT(chiw, j, i), b = AT(muw, j, i);
      double tap = (1.0 - exp_tail((-a) / 1e-4)) * (1.0 - exp_tail((-jmax(0.0, b - 0.4)) / 0.05));
      AT(xixw, j, i) = (-(ext(px, j + 1, i, Nz, Nx) - ext(px, j, i, Nz, Nx))) * tap;
      AT(xisw, j, i) = (-(ext(ps, j + 1, i, Nz, Nx) - ext(ps, j, i, Nz, Nx))) * tap;
    }
  });
}

// speed magnitudes (noise.jl:223-236)
__global__ void speeds_kernel(int Nz, int Nx, CView xisw, CView xisu, CView xixw, CView xixu,
                              CView xiew, CView xieu, DView xis, DView xix, DView xie) {
  XC_PDL_WAIT();
  for_tiles(Nz, Nx, [&](int j, int i) {
    if (j >= Nz || i >= Nx) return;
    double wz = (AT(xisw, j, i + 1) + AT(xisw, j + 1, i + 1)) / 2.0;
    double wx = (AT(xisu, j + 1, i) + AT(xisu, j + 1, i + 1)) / 2.0;
    AT(xis, j, i) = sqrt(wz * wz + wx * wx);
    wz = (AT(xixw, j, i + 1) + AT(xixw, j + 1, i + 1)) / 2.0;
    wx = (AT(xixu, j + 1, i) + AT(xixu, j + 1, i + 1)) / 2.0;
    AT(xix, j, i) = sqrt(wz * wz + wx * wx);
    wz = (AT(xiew, j, i + 1) + AT(xiew, j + 1, i + 1)) / 2.0;
    wx = (AT(xieu, j + 1, i) + AT(xieu, j + 1, i + 1)) / 2.0;
    AT(xie, j, i) = sqrt(wz * wz + wx * wx);
  });
}

}  // namespace

int noise_plan_create(xc_ctx* c) {
  NoisePlan* np = new NoisePlan();
  c->noise = np;
  const double h = c->p.h, L0h = c->p.L0h, l0h = c->p.l0h;
  np->padL0 = 4 * (int)std::ceil(L0h / h);
  np->padl0 = 4 * (int)std::ceil(l0h / h);
  np->fL = 2.0 / std::sqrt(1.0 - std::exp(-(h * h) / (2.0 * (L0h * L0h))));
  np->fl = 2.0 / std::sqrt(1.0 - std::exp(-(h * h) / (2.0 * (l0h * l0h))));
  const int Nz = c->Nz, Nx = c->Nx;
  XC_TRY(build_line_filter(np->ze, Nz, Nz + np->padL0, h, L0h, false));
  XC_TRY(build_line_filter(np->xe, Nx, Nx, h, L0h, true));
  XC_TRY(build_line_filter(np->zs, Nz, Nz + np->padl0, h, l0h, false));
  XC_TRY(build_line_filter(np->xs, Nx, Nx, h, l0h, true));
  return XC_OK;
}

void noise_plan_destroy(xc_ctx* c) {
  if (!c->noise) return;
  free_line_filter(c->noise->ze);
  free_line_filter(c->noise->xe);
  free_line_filter(c->noise->zs);
  free_line_filter(c->noise->xs);
  delete c->noise;
  c->noise = nullptr;
}

int noise_impl(xc_ctx* c, double dt, int first_iter, const double* re, const double* rs, cudaStream_t s_in,
               double* partials) {
  const int Nz = c->Nz, Nx = c->Nx;
  const xc_params& p = c->p;
  cudaStream_t s = s_in ? s_in : c->stream;
  NoisePlan* np = c->noise;
  const size_t nb = sizeof(double) * (size_t)Nz * Nx;
  if (first_iter) {
    if (re) XC_CUDA_TRY(cudaMemcpyAsync(c->field[FLD_re], re, nb, cudaMemcpyHostToDevice, s));
    if (rs) XC_CUDA_TRY(cudaMemcpyAsync(c->field[FLD_rs], rs, nb, cudaMemcpyHostToDevice, s));
  }
  dim3 blk(32, 8);
  xc_launch(ou_kernel, dim3(persistent_grid((const void*)ou_kernel, Nz, Nx)), blk, 0, s, Nz, Nx, p.Xi, p.L0h,
      2.0 / p.L0h, 2.0 / p.l0h, p.txi0, dt,
      1.0 / (1e2 * dt), np->fL, np->fl, CF(c, FLD_V),
      CF(c, FLD_vx),
      CF(c, FLD_fReL), CF(c, FLD_ke), CF(c, FLD_chi), CF(c, FLD_ks), CF(c, FLD_psieo),
      CF(c, FLD_psixo), CF(c, FLD_psiso), CF(c, FLD_re), CF(c, FLD_rs), F(c, FLD_psie),
      F(c, FLD_psix), F(c, FLD_psis));
  XC_LAUNCH_CHECK();
  // filtered fields in tmp[2..4], z-pass intermediate in tmp[5]
  DView flt[3] = {DView{c->tmp[2], Nz}, DView{c->tmp[3], Nz}, DView{c->tmp[4], Nz}};
  DView mid{c->tmp[5], Nz};
  const int src[3] = {FLD_psie, FLD_psix, FLD_psis};
  const LineFilter* zf[3] = {&np->ze, &np->ze, &np->zs};
  const LineFilter* xf[3] = {&np->xe, &np->xe, &np->xs};
  double* st = c->dscal + SC_NOISE_STATS;
  const double n = (double)Nz * (double)Nx;
  for (int q = 0; q < 3; ++q) {
    XC_TRY(run_line_filter(*zf[q], CF(c, src[q]), mid, Nz, Nx, 0, s));
    XC_TRY(run_line_filter(*xf[q], CView{mid.p, Nz}, flt[q], Nz, Nx, 1, s));
  }
  // the six means in one launch, then the six centred sums of squares
  // (mean and corrected std of noise.jl:261-264)
  RedJob means[6], devs[6];
  for (int q = 0; q < 3; ++q) {
    CView raw = CF(c, src[q]), fv{flt[q].p, Nz};
    means[2 * q] = red_job(RED_SUM, raw, CView{nullptr, 0}, nullptr, Nz, Nx, st + 4 * q + 0, n);
    means[2 * q + 1] = red_job(RED_SUM, fv, CView{nullptr, 0}, nullptr, Nz, Nx, st + 4 * q + 2, n);
    devs[2 * q] = red_job(RED_SUM, raw, CView{nullptr, 0}, st + 4 * q + 0, Nz, Nx, st + 4 * q + 1);
    devs[2 * q + 1] = red_job(RED_SUM, fv, CView{nullptr, 0}, st + 4 * q + 2, Nz, Nx, st + 4 * q + 3);
  }
  XC_TRY(reduce_batch(c, means, 6, s, partials));
  XC_TRY(reduce_batch(c, devs, 6, s, partials));
  xc_launch(rescale_kernel, grid2d(Nz, Nx, blk), blk, 0, s, Nz, Nx, flt[0], flt[1], flt[2], st);
  XC_LAUNCH_CHECK();
  xc_launch(stagger_kernel, dim3(persistent_grid((const void*)stagger_kernel, Nz + 2, Nx + 2)), blk, 0, s, Nz, Nx,
      CView{flt[0].p, Nz},
      CView{flt[1].p, Nz}, CView{flt[2].p, Nz}, CF(c, FLD_chiw),
      CF(c, FLD_muw), CF(c, FLD_chiu), CF(c, FLD_muu), F(c, FLD_xieu), F(c, FLD_xiew),
      F(c, FLD_xixu), F(c, FLD_xixw), F(c, FLD_xisu), F(c, FLD_xisw));
  XC_LAUNCH_CHECK();
  xc_launch(speeds_kernel, dim3(persistent_grid((const void*)speeds_kernel, Nz, Nx)), blk, 0, s, Nz, Nx,
      CF(c, FLD_xisw), CF(c, FLD_xisu),
      CF(c, FLD_xixw), CF(c, FLD_xixu), CF(c, FLD_xiew),
      CF(c, FLD_xieu), F(c, FLD_xis), F(c, FLD_xix), F(c, FLD_xie));
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// time the FFT line filter (z pass of psie) with CUDA events on the context stream
int noise_bench_zpass(xc_ctx* c, int iters, double out[4]) {
  const int Nz = c->Nz, Nx = c->Nx;
  NoisePlan* np = c->noise;
  cudaEvent_t e0, e1;
  XC_CUDA_TRY(cudaEventCreate(&e0));
  XC_CUDA_TRY(cudaEventCreate(&e1));
  int st = XC_OK;
  for (int it = -1; it < iters && st == XC_OK; ++it) {
    if (it == 0) cudaEventRecord(e0, c->stream);
    st = run_line_filter(np->ze, CF(c, FLD_psie), DView{c->tmp[5], Nz}, Nz, Nx, 0, c->stream);
  }
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != XC_OK) return st;
  const double M = np->ze.M, logM = np->ze.logM;
  out[0] = ms / iters;
  out[1] = 16.0 * Nz * (double)Nx;                   // read psi, write the filtered field
  out[2] = (double)((Nx + 1) / 2) * 2.0 * 5.0 * M * logM;   // forward + inverse complex FFT per line pair
  out[3] = (double)Nz * Nx;
  return XC_OK;
}
