// Deterministic FP64 reductions: a fixed grid of CTAs each reduces a fixed
// strided subset in a fixed order, and the last CTA of a reduction to finish
// combines the CTA partials in a fixed order.  The same inputs always give the
// same bits (no floating-point atomics; the one atomic is an integer arrival
// counter that only decides WHICH CTA does the combine, not its order).
//
// Several independent reductions run as one launch (one row of CTAs per
// reduction, blockIdx.y), so update_dt's five maxima, compute_resnorm's nine
// sums of squares or record_history!'s statistics cost one launch each.
//
// min / max follow Julia's minimum / maximum: a NaN anywhere gives NaN (CUDA's
// fmin / fmax would drop it).
//
// Used for the global reductions on the path: minimum(eta) / minimum(etas)
// (src/update.jl:331,396), maximum(kx) and maximum(abs, W*/U*) (update.jl:497-499),
// mean(MFS) (src/fluidmech.jl:127), mean/std in the FFT filter
// (src/noise.jl:261-264), the L2 norms of compute_resnorm (src/diagnose.jl:60-65),
// the FP64 conservation sums (src/history.jl:122-145) and the field statistics
// of record_history! / print_step! (history.jl:183-222, diagnose.jl:92-182).
#include "xc_internal.cuh"

namespace {

constexpr int RB = 256;          // threads per reduction CTA
constexpr int RG = 2 * kNumSMs;  // most CTAs one reduction uses

__device__ __forceinline__ double red_identity(int op) {
  switch (op) {
    case RED_MAX: case RED_MAXABS: return -INFINITY;
    case RED_MIN: return INFINITY;
    default: return 0.0;
  }
}

__device__ __forceinline__ double red_combine(int op, double a, double b) {
  switch (op) {
    case RED_MAX: case RED_MAXABS: return jmax(a, b);
    case RED_MIN: return jmin(a, b);
    default: return a + b;
  }
}

// warp shuffles (fixed butterfly) then the 8 warp results in order: the same
// bits for the same per-thread values
__device__ __forceinline__ double block_reduce(int op, double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = red_combine(op, v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = sh[0];
  for (int k = 1; k < RB / 32; ++k) r = red_combine(op, r, sh[k]);
  return r;
}

struct RedBatch {
  RedJob job[kMaxRedJobs];
};

// One thread's share of a reduction: the element transform and the combine
// fixed at compile time.  (With the operation switched per element, the
// compiler predicates every case, and on GB300's narrow FP64 pipe the
// predicated-off FP64 instructions cost as much issue time as the live ones.)
// The linear index t over rows x cols (column-major) advances by a fixed
// stride without a per-element division.
template <int OP, bool CENTER>
__device__ __forceinline__ double red_thread(const RedJob& J, double ctr) {
  constexpr int COMB = (OP == RED_SUMSQ || OP == RED_SUMSQDIFF || OP == RED_SUMLOG || CENTER) ? RED_SUM : OP;
  double acc = red_identity(COMB);
  const long long n = (long long)J.rows * J.cols;
  const long long stride = (long long)J.nblk * RB;
  const int sq = (int)(stride / J.rows), sr = (int)(stride % J.rows);
  long long t = (long long)blockIdx.x * RB + threadIdx.x;
  int i = (int)(t / J.rows), j = (int)(t % J.rows);
  for (; t < n; t += stride) {
    const double a = J.a[(size_t)i * J.lda + j];
    double v;
    if (CENTER) {
      const double d = a - ctr;
      v = d * d;
    } else if (OP == RED_SUMSQ) {
      v = a * a;
    } else if (OP == RED_MAXABS) {
      v = fabs(a);
    } else if (OP == RED_SUMSQDIFF) {
      const double d = a - J.b[(size_t)i * J.ldb + j];
      v = d * d;
    } else if (OP == RED_SUMLOG) {
      v = log(jmax(a, J.floor));
    } else {
      v = a;
    }
    acc = red_combine(COMB, acc, v);
    j += sr;
    i += sq;
    if (j >= J.rows) { j -= J.rows; ++i; }
  }
  return acc;
}

__global__ void __launch_bounds__(RB) batch_reduce_kernel(RedBatch B, double* partials, unsigned* counters) {
  XC_PDL_WAIT();
  __shared__ double sh[RB / 32];
  __shared__ int last;
  const RedJob& J = B.job[blockIdx.y];
  if ((int)blockIdx.x >= J.nblk) return;
  const int op = J.op;
  const int comb = (op == RED_SUMSQ || op == RED_SUMSQDIFF || op == RED_SUMLOG || J.center) ? RED_SUM : op;
  double acc;
  if (J.center) {
    acc = red_thread<RED_SUM, true>(J, *J.center);
  } else {
    switch (op) {   // uniform per CTA: a branch, not per-element predication
      case RED_MAX: acc = red_thread<RED_MAX, false>(J, 0.0); break;
      case RED_MIN: acc = red_thread<RED_MIN, false>(J, 0.0); break;
      case RED_SUMSQ: acc = red_thread<RED_SUMSQ, false>(J, 0.0); break;
      case RED_MAXABS: acc = red_thread<RED_MAXABS, false>(J, 0.0); break;
      case RED_SUMSQDIFF: acc = red_thread<RED_SUMSQDIFF, false>(J, 0.0); break;
      case RED_SUMLOG: acc = red_thread<RED_SUMLOG, false>(J, 0.0); break;
      default: acc = red_thread<RED_SUM, false>(J, 0.0); break;
    }
  }
  double r = block_reduce(comb, acc, sh);
  double* part = partials + (size_t)blockIdx.y * RG;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = r;
    __threadfence();
    const unsigned prev = atomicAdd(counters + blockIdx.y, 1u);
    last = (prev == (unsigned)J.nblk - 1u);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = red_identity(comb);
  for (int k = threadIdx.x; k < J.nblk; k += RB) v = red_combine(comb, v, __ldcg(part + k));
  r = block_reduce(comb, v, sh);
  if (threadIdx.x == 0) {
    *J.out = J.divisor == 1.0 ? r : r / J.divisor;
    counters[blockIdx.y] = 0u;   // ready for the next launch on this scratch
  }
}

int blocks_for(long long n) {
  long long b = (n + (long long)RB * 8 - 1) / ((long long)RB * 8);
  if (b < 1) b = 1;
  if (b > RG) b = RG;
  return (int)b;
}

}  // namespace

RedJob red_job(int op, CView a, CView b, const double* center, int rows, int cols, double* out, double divisor) {
  RedJob J;
  J.a = a.p; J.b = b.p; J.center = center; J.out = out; J.divisor = divisor; J.floor = XC_EPS;
  J.lda = a.ld; J.ldb = b.ld; J.rows = rows; J.cols = cols; J.op = op; J.nblk = 0;
  return J;
}

int reduce_batch(xc_ctx* c, const RedJob* jobs, int njobs, cudaStream_t s, double* partials) {
  double* part = partials ? partials : c->red_partials;
  unsigned* counters = (unsigned*)(part + (size_t)kMaxRedJobs * RG);
  for (int k0 = 0; k0 < njobs; k0 += kMaxRedJobs) {
    const int nj = njobs - k0 < kMaxRedJobs ? njobs - k0 : kMaxRedJobs;
    RedBatch B;
    int gx = 1;
    for (int k = 0; k < nj; ++k) {
      B.job[k] = jobs[k0 + k];
      if (B.job[k].rows < 1 || B.job[k].cols < 1) {
        xc_set_error("reduction over an empty array (%d x %d)", B.job[k].rows, B.job[k].cols);
        return XC_BAD_ARG;
      }
      B.job[k].nblk = blocks_for((long long)B.job[k].rows * B.job[k].cols);
      gx = B.job[k].nblk > gx ? B.job[k].nblk : gx;
    }
    xc_launch(batch_reduce_kernel, dim3((unsigned)gx, (unsigned)nj), RB, 0, s, B, part, counters);
    XC_LAUNCH_CHECK();
  }
  return XC_OK;
}

int reduce_to(xc_ctx* c, int op, CView a, CView b, const double* center, int rows, int cols,
              double* out, cudaStream_t s, double divisor, double* partials) {
  RedJob J = red_job(op, a, b, center, rows, cols, out, divisor);
  return reduce_batch(c, &J, 1, s, partials);
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

// doubles of one reduction scratch: the CTA partials of kMaxRedJobs
// reductions, then kMaxRedJobs arrival counters (zeroed at creation)
int reduce_partials_len() { return kMaxRedJobs * RG + kMaxRedJobs; }
