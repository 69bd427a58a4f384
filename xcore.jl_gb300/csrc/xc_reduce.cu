// Deterministic FP64 reductions: a fixed grid of CTAs each reduces a fixed
// strided subset in a fixed order, then one CTA combines the partials.  The
// same inputs always give the same bits (no floating-point atomics).
//
// Used for the global reductions on the path: minimum(eta) / minimum(etas)
// (src/update.jl:331,396), maximum(kx) and maximum(abs, W*/U*) (update.jl:497-499),
// mean(MFS) (src/fluidmech.jl:127), mean/std in the FFT filter
// (src/noise.jl:261-264), the L2 norms of compute_resnorm (src/diagnose.jl:60-65)
// and the FP64 conservation sums (src/history.jl:122-145).
#include "xc_internal.cuh"

namespace {

constexpr int RB = 256;        // threads per reduction CTA
constexpr int RG = 2 * kNumSMs;  // CTAs in the partial pass

__device__ __forceinline__ double red_identity(int op) {
  switch (op) {
    case RED_MAX: case RED_MAXABS: return -INFINITY;
    case RED_MIN: return INFINITY;
    default: return 0.0;
  }
}

__device__ __forceinline__ double red_combine(int op, double a, double b) {
  switch (op) {
    case RED_MAX: case RED_MAXABS: return fmax(a, b);
    case RED_MIN: return fmin(a, b);
    default: return a + b;
  }
}

__device__ __forceinline__ double block_reduce(int op, double v, double* sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = RB / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] = red_combine(op, sh[tid], sh[tid + s]);
    __syncthreads();
  }
  return sh[0];
}

__global__ void __launch_bounds__(RB) partial_kernel(int op, CView a, CView b, const double* center,
                                                     int rows, int cols, double* partials) {
  __shared__ double sh[RB];
  const long long n = (long long)rows * cols;
  double acc = red_identity(op);
  const double ctr = center ? *center : 0.0;
  for (long long t = blockIdx.x * (long long)RB + threadIdx.x; t < n; t += (long long)RG * RB) {
    int j = (int)(t % rows), i = (int)(t / rows);
    double v = AT(a, j, i);
    switch (op) {
      case RED_SUMSQ: v = v * v; break;
      case RED_MAXABS: v = fabs(v); break;
      case RED_SUMSQDIFF: { double d = v - AT(b, j, i); v = d * d; } break;
      case RED_SUMLOG: v = log(fmax(v, XC_EPS)); break;
      default: break;
    }
    if (center) { double d = AT(a, j, i) - ctr; v = d * d; }
    acc = red_combine(op, acc, v);
  }
  double r = block_reduce(op, acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

__global__ void __launch_bounds__(RB) final_kernel(int op, const double* partials, int n,
                                                   double* out, double divisor) {
  __shared__ double sh[RB];
  double acc = red_identity(op);
  for (int t = threadIdx.x; t < n; t += RB) acc = red_combine(op, acc, partials[t]);
  double r = block_reduce(op, acc, sh);
  if (threadIdx.x == 0) *out = divisor == 1.0 ? r : r / divisor;
}

}  // namespace

int reduce_to(xc_ctx* c, int op, CView a, CView b, const double* center, int rows, int cols,
              double* out, cudaStream_t s, double divisor, double* partials) {
  double* part = partials ? partials : c->red_partials;
  int combine_op = (op == RED_SUMSQ || op == RED_SUMSQDIFF || op == RED_SUMLOG) ? RED_SUM : op;
  if (center) combine_op = RED_SUM;
  partial_kernel<<<RG, RB, 0, s>>>(op, a, b, center, rows, cols, part); xc_count_launch();
  XC_LAUNCH_CHECK();
  final_kernel<<<1, RB, 0, s>>>(combine_op, part, RG, out, divisor); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int reduce_view(xc_ctx* c, int op, CView a, CView b, int rows, int cols, int slot) {
  return reduce_to(c, op, a, b, nullptr, rows, cols, c->dscal + slot, c->stream);
}

int fetch_scalars(xc_ctx* c, int first, int n) {
  XC_CUDA_TRY(cudaMemcpyAsync(c->hscal + first, c->dscal + first, sizeof(double) * n,
                              cudaMemcpyDeviceToHost, c->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return XC_OK;
}

int reduce_partials_len() { return RG; }
