// Internal declarations shared by the translation units of libxcore_gb300.
#pragma once

#include <cmath>
#include <functional>
#include <utility>

#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <cstddef>
#include <cstdio>
#include <string>

#include "xcore_gb300.h"

// ---------------------------------------------------------------------------
// field registry: name, shape code, element size.  Shape codes follow the
// reference sizes (src/state.jl:57-69, 143-163; src/noise.jl:25-35).
// ---------------------------------------------------------------------------
enum ShapeCode : int {
  SH_C = 0,   // (Nz,   Nx)
  SH_ZF,      // (Nz+1, Nx)     z-faces, x-interior
  SH_XF,      // (Nz,   Nx+1)   x-faces, z-interior
  SH_W,       // (Nz+1, Nx+2)   W-shaped (z-faces with x ghost columns), also qz
  SH_U,       // (Nz+2, Nx+1)   U-shaped (x-faces with z ghost rows), also qx
  SH_CO,      // (Nz+1, Nx+1)   corners
  SH_P        // (Nz+2, Nx+2)   pressure with ghost ring
};

// X-macro: (identifier, shape, element bytes)
#define XC_FIELDS(F)                                                                   \
  F(W, SH_W, 8) F(U, SH_U, 8) F(P, SH_P, 8) F(eta, SH_C, 8) F(etaco, SH_CO, 8)         \
  F(rho, SH_C, 8) F(rhow, SH_ZF, 8) F(rhou, SH_XF, 8) F(Drho, SH_ZF, 8)                \
  F(rhoo, SH_C, 8) F(rhooo, SH_C, 8) F(drhodt, SH_C, 8) F(drhodto, SH_C, 8)            \
  F(drhodtoo, SH_C, 8) F(MFS, SH_C, 8) F(rhoWo, SH_ZF, 8) F(rhoWoo, SH_ZF, 8)          \
  F(rhoUo, SH_XF, 8) F(rhoUoo, SH_XF, 8)                                               \
  F(x, SH_C, 8) F(m, SH_C, 8) F(X, SH_C, 8) F(M, SH_C, 8) F(Xo, SH_C, 8)               \
  F(Xoo, SH_C, 8) F(Mo, SH_C, 8) F(Moo, SH_C, 8) F(chi, SH_C, 8) F(mu, SH_C, 8)        \
  F(hasx, SH_C, 1) F(hasm, SH_C, 1)                                                    \
  F(chiw, SH_W, 8) F(muw, SH_W, 8) F(chiu, SH_U, 8) F(muu, SH_U, 8)                    \
  F(x_w, SH_ZF, 8) F(m_w, SH_ZF, 8) F(x_u, SH_XF, 8) F(m_u, SH_XF, 8)                  \
  F(Drhom, SH_ZF, 8) F(Drhox, SH_ZF, 8) F(Pl, SH_C, 8) F(Pt, SH_C, 8)                  \
  F(etamix, SH_C, 8) F(etae, SH_C, 8) F(ke, SH_C, 8) F(kx, SH_C, 8)                    \
  F(etat, SH_C, 8) F(etas, SH_C, 8) F(etasw, SH_ZF, 8) F(ks, SH_C, 8)                  \
  F(V, SH_C, 8) F(Div_V, SH_C, 8) F(exx, SH_C, 8) F(ezz, SH_C, 8) F(exz, SH_CO, 8)     \
  F(eII, SH_C, 8) F(vx, SH_C, 8) F(vm, SH_C, 8) F(txx, SH_C, 8) F(tzz, SH_C, 8)        \
  F(txz, SH_CO, 8) F(tII, SH_C, 8) F(fReL, SH_C, 8) F(ReL, SH_C, 8) F(ReD, SH_C, 8)    \
  F(Ra, SH_C, 8) F(fRel, SH_C, 8) F(Rel, SH_C, 8) F(Red, SH_C, 8) F(Rc, SH_C, 8)       \
  F(Wx, SH_W, 8) F(Wm, SH_W, 8) F(Ux, SH_U, 8) F(Um, SH_U, 8) F(wx, SH_W, 8)           \
  F(wm, SH_W, 8) F(bndtaperw, SH_W, 8) F(bndshape, SH_C, 8)                            \
  F(advn_X, SH_C, 8) F(advn_M, SH_C, 8) F(advn_rho, SH_C, 8)                           \
  F(qx_advn_X, SH_U, 8) F(qz_advn_X, SH_W, 8) F(qx_advn_M, SH_U, 8)                    \
  F(qz_advn_M, SH_W, 8) F(qx_dffn_X, SH_U, 8) F(qz_dffn_X, SH_W, 8)                    \
  F(qx_dffn_M, SH_U, 8) F(qz_dffn_M, SH_W, 8) F(dffn_X, SH_C, 8) F(Gx, SH_C, 8)        \
  F(dXdt, SH_C, 8) F(dXdto, SH_C, 8) F(dXdtoo, SH_C, 8)                                \
  F(psie, SH_C, 8) F(psix, SH_C, 8) F(psis, SH_C, 8) F(psieo, SH_C, 8)                 \
  F(psixo, SH_C, 8) F(psiso, SH_C, 8) F(re, SH_C, 8) F(rs, SH_C, 8)                    \
  F(xiew, SH_W, 8) F(xieu, SH_U, 8) F(xixw, SH_W, 8) F(xixu, SH_U, 8)                  \
  F(xisw, SH_W, 8) F(xisu, SH_U, 8) F(xie, SH_C, 8) F(xix, SH_C, 8) F(xis, SH_C, 8)    \
  F(res_Wo, SH_W, 8) F(res_Uo, SH_U, 8) F(res_Po, SH_P, 8) F(res_Xo, SH_C, 8)          \
  F(res_MFSo, SH_C, 8)

enum FieldId : int {
#define XC_ENUM(name, sh, eb) FLD_##name,
  XC_FIELDS(XC_ENUM)
#undef XC_ENUM
  FLD_COUNT
};

struct Shape { int rows, cols; };

inline Shape shape_of(int code, int Nz, int Nx) {
  switch (code) {
    case SH_C: return {Nz, Nx};
    case SH_ZF: return {Nz + 1, Nx};
    case SH_XF: return {Nz, Nx + 1};
    case SH_W: return {Nz + 1, Nx + 2};
    case SH_U: return {Nz + 2, Nx + 1};
    case SH_CO: return {Nz + 1, Nx + 1};
    default: return {Nz + 2, Nx + 2};
  }
}

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------
void xc_set_error(const char* fmt, ...);

#define XC_CUDA_TRY(call)                                                               \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      xc_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));  \
      return XC_CUDA;                                                                   \
    }                                                                                   \
  } while (0)

#define XC_LAUNCH_CHECK() XC_CUDA_TRY(cudaGetLastError())

// number of kernels this library has launched (host side): process-wide, and
// per host thread for the bookkeeping of stream capture (contexts may be
// driven from several threads at once)
extern std::atomic<long long> g_xc_launches;
extern thread_local long long g_xc_thread_launches;
inline void xc_count_launch() {
  ++g_xc_thread_launches;
  g_xc_launches.fetch_add(1, std::memory_order_relaxed);
}

// Programmatic dependent launch: a kernel that begins with XC_PDL_WAIT()
// waits there for the grid before it on the stream to finish and flush its
// memory (a no-op when launched without the attribute), so it may be launched
// with programmatic stream serialization -- scheduled while the previous
// kernel drains instead of after it, hiding the launch gap.
#define XC_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")

// launch with programmatic stream serialization (the kernel must begin with
// XC_PDL_WAIT()), counted like a plain launch
template <typename... KArgs, typename... Args>
inline void xc_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
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
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
  xc_count_launch();
}

#define XC_TRY(expr)               \
  do {                             \
    int s_ = (expr);               \
    if (s_ != XC_OK) return s_;    \
  } while (0)

// ---------------------------------------------------------------------------
// device views
// ---------------------------------------------------------------------------
struct DView {        // column-major view of a field (or a sub-block of one)
  double* p;
  int ld;             // leading dimension (rows of the parent array)
};

struct CView {
  const double* p;
  int ld;
};

__host__ __device__ inline DView dview(double* p, int ld) { return DView{p, ld}; }
__host__ __device__ inline CView cview(const double* p, int ld) { return CView{p, ld}; }

#define AT(v, j, i) ((v).p[(size_t)(i) * (size_t)(v).ld + (size_t)(j)])

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct NoisePlan;     // xc_noise.cu
struct StokesWork;    // xc_stokes.cu

struct xc_ctx {
  xc_params p;
  int Nz, Nx;
  int device;
  cudaStream_t stream;
  // noise! of a Picard sweep runs on `side` while phsevo! and fluidmech! run
  // on `stream` (it reads only fields of the previous update!); ev_fork /
  // ev_join order it, red_partials_side is its reduction scratch
  cudaStream_t side;
  cudaEvent_t ev_fork, ev_join;
  double* red_partials_side;
  char* arena;
  size_t arena_bytes;
  void* field[FLD_COUNT];
  void* own[FLD_COUNT];      // the context's own storage of each field (field[] may be bound elsewhere)
  Shape shape[FLD_COUNT];
  int elem[FLD_COUNT];
  // scratch
  double* red_partials;      // block partials of reductions
  int red_partials_len;
  double* dscal;             // device scalars (64 slots)
  double* hscal;             // pinned host mirror of dscal
  double* tmp[8];            // full-size (Nz+2)x(Nx+2) FP64 temporaries
  NoisePlan* noise;
  StokesWork* stokes;
};

// device scalar slots
enum ScalarSlot : int {
  SC_EMAX_ETA = 0,
  SC_EMAX_ETAS = 1,
  SC_MFS_MEAN = 2,
  SC_NOISE_STATS = 8,       // 3 fields x 4 values (raw mean, raw std, flt mean, flt std)
  SC_RESNORM = 24,          // 8 sums of squares
  SC_DT = 40,               // 5 maxima
  SC_SUMS = 48,             // 12 conservation sums
};

inline DView F(xc_ctx* c, int id) { return DView{(double*)c->field[id], c->shape[id].rows}; }
inline CView CF(xc_ctx* c, int id) { return CView{(const double*)c->field[id], c->shape[id].rows}; }

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
constexpr int kNumSMs = 152;

inline dim3 grid2d(int rows, int cols, dim3 blk) {
  return dim3((unsigned)((rows + blk.x - 1) / blk.x), (unsigned)((cols + blk.y - 1) / blk.y));
}

// Persistent 2-D launches of 32 x 8 threads: a grid of one wave -- as many
// CTAs as the SMs hold at the kernel's occupancy -- strides over the 32 x 8
// tiles of a rows x cols domain, so no last wave runs partly empty (the
// FP64 kernels of the path run 3-4 waves of their data-sized grids).  f(j, i)
// is the body of one cell; a `return` in it ends that cell.
template <typename F>
__device__ __forceinline__ void for_tiles(int rows, int cols, F&& f) {
  const int nbx = (rows + 31) / 32, nt = nbx * ((cols + 7) / 8);
  for (int t = blockIdx.x; t < nt; t += gridDim.x)
    f((t % nbx) * 32 + (int)threadIdx.x, (t / nbx) * 8 + (int)threadIdx.y);
}
// CTAs of such a launch of `kernel` over rows x cols
unsigned persistent_grid(const void* kernel, int rows, int cols);

// Julia's max / min of two Float64 (Base.max / Base.min on IEEE floats): a
// NaN argument gives NaN -- CUDA's fmax / fmin return the other argument
// instead -- and zeros are ordered -0.0 < +0.0, so max(0.0, -0.0) is +0.0 and
// min(0.0, -0.0) is -0.0 whatever the argument order (a plain a > b ? a : b
// returns the second argument for two zeros).  Either result is independent
// of the order in which a reduction combines its values.
__host__ __device__ __forceinline__ bool jsignbit(double a) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(a) < 0;
#else
  return std::signbit(a);
#endif
}
__host__ __device__ __forceinline__ double jmax(double a, double b) {
  if (a > b) return a;
  if (b > a) return b;
  return (a != a || b != b) ? a + b : (jsignbit(a) ? b : a);
}
__host__ __device__ __forceinline__ double jmin(double a, double b) {
  if (a < b) return a;
  if (b < a) return b;
  return (a != a || b != b) ? a + b : (jsignbit(a) ? a : b);
}

// deterministic reductions (xc_reduce.cu): CTA partials, combined in a fixed
// order by the last CTA to finish; up to kMaxRedJobs reductions per launch
enum RedOp : int { RED_SUM = 0, RED_MAX = 1, RED_MIN = 2, RED_SUMSQ = 3, RED_MAXABS = 4,
                   RED_SUMSQDIFF = 5, RED_SUMLOG = 6 /* sum of log(max(a, floor)) */ };
constexpr int kMaxRedJobs = 32;
struct RedJob {
  const double* a;
  const double* b;           // second operand of RED_SUMSQDIFF
  const double* center;      // device scalar: sum of (a - *center)^2 instead of op
  double* out;               // device result: reduction / divisor
  double divisor;
  double floor;              // RED_SUMLOG floor (eps by default)
  int lda, ldb, rows, cols;
  int op;
  int nblk;                  // set by reduce_batch
};
RedJob red_job(int op, CView a, CView b, const double* center, int rows, int cols, double* out,
               double divisor = 1.0);
// njobs independent reductions, kMaxRedJobs per launch, on stream s with
// scratch `partials` (c->red_partials when null)
int reduce_batch(xc_ctx* c, const RedJob* jobs, int njobs, cudaStream_t s, double* partials = nullptr);
// reduce a column-major view of rows x cols into dscal[slot] (device); b may be
// null unless op == RED_SUMSQDIFF (sum of (a-b)^2)
int reduce_view(xc_ctx* c, int op, CView a, CView b, int rows, int cols, int slot);
// general form: optional center (sum of (a - *center)^2), result / divisor into *out
int reduce_to(xc_ctx* c, int op, CView a, CView b, const double* center, int rows, int cols,
              double* out, cudaStream_t s, double divisor = 1.0, double* partials = nullptr);
int reduce_partials_len();
// copy device scalars [first, first+n) to the pinned host mirror and wait
int fetch_scalars(xc_ctx* c, int first, int n);

// ---------------------------------------------------------------------------
// entry points implemented per translation unit (status-returning, on c->stream)
// ---------------------------------------------------------------------------
// scheme code of WENO5 with its weights over a common denominator (one
// division per reconstruction), selected by xc_params.weno_weights = 1
constexpr int kWeno5OneDiv = 105;
inline int advect_scheme(int scheme, const xc_params& p) {
  return scheme == XC_WENO5 && p.weno_weights == 1 ? kWeno5OneDiv : scheme;
}
int stencil_advect_flux(const double* f, int ldf, bool halod, int Nz, int Nx, int scheme,
                        int xBC, int zBC, CView u, CView w, double h,
                        DView adv, DView qx_int, DView qz_int, cudaStream_t s);
int stencil_diffus_flux(const double* f, const double* k, int ld, bool halod, int Nz, int Nx,
                        int xBC, int zBC, double h, DView dff, DView qx_int, DView qz_int,
                        cudaStream_t s);
int pad_face_fluxes(DView qx, DView qz, int Nz, int Nx, int xBC, int zBC, cudaStream_t s);
int scheme_halo(int scheme);

int phsevo_impl(xc_ctx* c, int scheme, const double coefs[6], double dt, double alpha);
int update_impl(xc_ctx* c);
int phase_velocities_impl(xc_ctx* c);
int store_previous_impl(xc_ctx* c);
int store_noise_impl(xc_ctx* c);
int snapshot_impl(xc_ctx* c);
int update_dt_impl(xc_ctx* c, double dt_prev, double* dt_out);
int resnorm_impl(xc_ctx* c, double dt, double out[3]);
// the two above as their device reductions (into c->dscal, on s or c->stream;
// nothing synchronises, so a graph can hold them) and the host arithmetic on
// the fetched sums (c->hscal)
int update_dt_reduce(xc_ctx* c, cudaStream_t s = nullptr);
void update_dt_finish(const xc_ctx* c, double dt_prev, double* dt_out);
int resnorm_reduce(xc_ctx* c, cudaStream_t s = nullptr);
void resnorm_finish(const xc_ctx* c, double dt, double out[3]);
int sums_impl(xc_ctx* c, double out[12]);
int history_impl(xc_ctx* c, double out[58]);
int print_stats_impl(xc_ctx* c, double out[24]);

int noise_plan_create(xc_ctx* c);
void noise_plan_destroy(xc_ctx* c);
// on stream s (c->stream when null) with reduction scratch partials (c->red_partials when null)
int noise_impl(xc_ctx* c, double dt, int first_iter, const double* re, const double* rs,
               cudaStream_t s = nullptr, double* partials = nullptr);

int stokes_create(xc_ctx* c);
void stokes_destroy(xc_ctx* c);
struct MmsData { const double *src_W, *src_U, *src_P, *W_exact, *U_exact, *P_exact; };
int stokes_bench(xc_ctx* c, int which, int iters, double out[4]);
// before_solve (may be null) is called once on the host after the solve's
// right-hand side and setup have been enqueued and before its iterations:
// the step forks noise! there, so that it runs beside the latency-bound
// iterations rather than beside the FP64 assembly kernels
int fluidmech_impl(xc_ctx* c, const double coefs[6], double dt, const xc_solver_opts* opts,
                   xc_solver_stats* stats, const MmsData* mms, const std::function<int()>* before_solve = nullptr);

// machine epsilon of Float64 and its square root (eps(T), sqrt(eps(T)))
#define XC_EPS 2.220446049250313080847e-16
#define XC_SQRT_EPS 1.4901161193847656e-08
