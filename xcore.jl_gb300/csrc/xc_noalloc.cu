// xc_update_dt_noalloc: the CFL time-step reduction of xc_update_dt for callers
// that cannot let a library allocate device memory.
//
// Who needs it: a caller whose process already owns the device memory through
// its own pool (a Julia session with CUDA.jl, a framework with a caching
// allocator) cannot have a library call cudaMalloc behind its back -- the pool
// may hold all free memory, and cudaMalloc / cudaFree also synchronise the
// whole device, which a time-step loop that queues work on its own streams
// must avoid.  This entry point therefore takes every input and the output as
// the caller's device pointers, keeps its block partials in a fixed static
// device array, and calls no allocating routine.
//
// The scratch: g_dt_scratch below, 5 x XC_NOALLOC_MAX_BLOCKS doubles (80 KiB)
// in every device that loads the library, for the life of the process.  Each
// call writes every slot it later reads, so nothing has to start at zero and
// no value carries over from the previous call.  All calls share the array:
// calls that overlap on the GPU (for example issued on two streams without
// ordering between them) race on it and must not be made.
#include <mutex>

#include "xc_internal.cuh"

namespace {

constexpr int XC_NOALLOC_MAX_BLOCKS = 2048;   // partials per reduced array
constexpr int XC_NOALLOC_CHUNK = 4096;        // elements reduced by one CTA
constexpr int XC_NOALLOC_THREADS = 256;
constexpr int XC_NOALLOC_MAX_DEVICES = 64;

// block partials of the five maxima: max(kx), max|Wx|, max|Wm|, max|Ux|, max|Um|
static __device__ __align__(256) double g_dt_scratch[5 * XC_NOALLOC_MAX_BLOCKS];

std::mutex g_setup_mutex;
double* g_scratch_addr[XC_NOALLOC_MAX_DEVICES] = {nullptr};

// device address of g_dt_scratch for the current device (looked up once per
// device; in host code the symbol itself is only a host-side stand-in).  The
// address lives as long as the device's primary context: a cudaDeviceReset,
// or a release and re-creation of the primary context, unloads the module
// and makes the kept address stale, so this entry point must not be called
// after such a reset in the same process.
int scratch_for_current_device(double** out) {
  int dev = 0;
  XC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= XC_NOALLOC_MAX_DEVICES) {
    xc_set_error("xc_update_dt_noalloc: device index %d out of range", dev);
    return XC_BAD_ARG;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dt_scratch);
    if (e != cudaSuccess || !p) {
      xc_set_error("xc_update_dt_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                   cudaGetErrorString(e));
      return XC_CUDA;
    }
    g_scratch_addr[dev] = (double*)p;
  }
  *out = g_scratch_addr[dev];
  return XC_OK;
}

struct DtInputs {
  const double* a[5];
  long long n[5];
};

// warp shuffles, then the eight warp maxima in order (Julia's max: NaN wins)
__device__ __forceinline__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = jmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = sh[0];
  for (int k = 1; k < XC_NOALLOC_THREADS / 32; ++k) r = jmax(r, sh[k]);
  return r;
}

// CTA (x, y) reduces elements [x*CHUNK, (x+1)*CHUNK) of array y into scratch
__global__ void __launch_bounds__(XC_NOALLOC_THREADS) dt_partial_kernel(DtInputs in, double* scratch) {
  __shared__ double sh[XC_NOALLOC_THREADS / 32];
  const int y = blockIdx.y;
  const long long n = in.n[y];
  const long long base = (long long)blockIdx.x * XC_NOALLOC_CHUNK;
  double m = -INFINITY;
  for (long long t = base + threadIdx.x; t < n && t < base + XC_NOALLOC_CHUNK; t += XC_NOALLOC_THREADS) {
    double v = in.a[y][t];
    m = jmax(m, y == 0 ? v : fabs(v));
  }
  const double r = block_max(m, sh);
  if (threadIdx.x == 0) scratch[(size_t)y * XC_NOALLOC_MAX_BLOCKS + blockIdx.x] = r;
}

// combine the partials and evaluate update_dt (src/update.jl:494-502) with
// Julia's min / max, as xc_update_dt does
__global__ void __launch_bounds__(XC_NOALLOC_THREADS) dt_final_kernel(const double* scratch, DtInputs in,
                                                                      double h, double CFL, double dtmax,
                                                                      double dt_prev, double* dt_out) {
  __shared__ double sh[XC_NOALLOC_THREADS / 32];
  __shared__ double mx[5];
  for (int y = 0; y < 5; ++y) {
    const int nb = (int)((in.n[y] + XC_NOALLOC_CHUNK - 1) / XC_NOALLOC_CHUNK);
    double m = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += XC_NOALLOC_THREADS)
      m = jmax(m, scratch[(size_t)y * XC_NOALLOC_MAX_BLOCKS + b]);
    const double r = block_max(m, sh);
    if (threadIdx.x == 0) mx[y] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double dtk = (h / 2.0) * (h / 2.0) / mx[0];
    double vmax = jmax(jmax(jmax(mx[1], mx[2]), mx[3]), mx[4]) + XC_EPS;
    double dta = (h / 2.0) / vmax;
    *dt_out = jmin(jmin(1.5 * dt_prev, jmin(dtk, CFL * dta)), dtmax);
  }
}

}  // namespace

extern "C" int xc_update_dt_noalloc(const double* kx, const double* Wx, const double* Wm, const double* Ux,
                                    const double* Um, int Nz, int Nx, double h, double CFL, double dtmax,
                                    double dt_prev, double* dt_out, void* stream) {
  if (!kx || !Wx || !Wm || !Ux || !Um || !dt_out || Nz < 1 || Nx < 1 || !(h > 0)) {
    xc_set_error("xc_update_dt_noalloc: null pointer or bad size");
    return XC_BAD_ARG;
  }
  DtInputs in;
  in.a[0] = kx; in.n[0] = (long long)Nz * Nx;
  in.a[1] = Wx; in.n[1] = (long long)(Nz + 1) * (Nx + 2);
  in.a[2] = Wm; in.n[2] = in.n[1];
  in.a[3] = Ux; in.n[3] = (long long)(Nz + 2) * (Nx + 1);
  in.a[4] = Um; in.n[4] = in.n[3];
  const long long limit = (long long)XC_NOALLOC_MAX_BLOCKS * XC_NOALLOC_CHUNK;
  long long nmax = 0;
  for (int y = 0; y < 5; ++y) nmax = in.n[y] > nmax ? in.n[y] : nmax;
  if (nmax > limit) {
    xc_set_error("xc_update_dt_noalloc: grid %dx%d needs %lld elements per array; the static scratch holds "
                 "%lld (%d blocks of %d) -- use xc_update_dt for larger grids",
                 Nz, Nx, nmax, limit, XC_NOALLOC_MAX_BLOCKS, XC_NOALLOC_CHUNK);
    return XC_BAD_ARG;
  }
  double* scratch = nullptr;
  XC_TRY(scratch_for_current_device(&scratch));
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid((unsigned)((nmax + XC_NOALLOC_CHUNK - 1) / XC_NOALLOC_CHUNK), 5);
  dt_partial_kernel<<<grid, XC_NOALLOC_THREADS, 0, s>>>(in, scratch); xc_count_launch();
  XC_LAUNCH_CHECK();
  dt_final_kernel<<<1, XC_NOALLOC_THREADS, 0, s>>>(scratch, in, h, CFL, dtmax, dt_prev, dt_out); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}
