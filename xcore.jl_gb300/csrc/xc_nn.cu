// The learned preconditioner's network: a 4-level U-Net (16, 32, 64, 128
// channels, 3x3 convolutions, ReLU, 2x2 average pooling, nearest upsampling
// with additive skips), BF16 weights and activations, FP32 accumulation,
// trained on the GPU by its own forward and backward kernels and Adam.
//
// Forward, at level l (H >> l, W >> l, 16 << l channels):
//   a0 = relu(c0a(in))      x0 = relu(c0b(a0))
//   a1 = relu(c1a(pool x0)) x1 = relu(c1b(a1))
//   a2 = relu(c2a(pool x1)) x2 = relu(c2b(a2))
//   a3 = relu(c3a(pool x2)) x3 = relu(c3b(a3))
//   u2 = up(c3u(x3)) + x2   y2 = relu(c2d(u2))
//   u1 = up(c2u(y2)) + x1   y1 = relu(c1d(u1))
//   u0 = up(c1u(y1)) + x0   y0 = relu(c0d(u0))
//   out = cout(y0)          (FP32, first kOutCh channels used)
// The input has kInCh used channels of 16 (zero padded).  Every convolution
// runs on the tcgen05 kernel of xc_nn_conv.cu; the data gradient of a
// convolution is the forward convolution of dY with the flipped, transposed
// weights, its weight gradient the tcgen05 wgrad GEMM.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "xc_internal.cuh"
#include "xc_nn.cuh"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kLayers = 15;
enum { C0A, C0B, C1A, C1B, C2A, C2B, C3A, C3B, C3U, C2D, C2U, C1D, C1U, C0D, COUT };
// (input channels, output channels, level, relu)
const int kSpec[kLayers][4] = {
    {16, 16, 0, 1},  {16, 16, 0, 1},  {16, 32, 1, 1},  {32, 32, 1, 1},  {32, 64, 2, 1},
    {64, 64, 2, 1},  {64, 128, 3, 1}, {128, 128, 3, 1}, {128, 64, 3, 0}, {64, 64, 2, 1},
    {64, 32, 2, 0},  {32, 32, 1, 1},  {32, 16, 1, 0},  {16, 16, 0, 1},  {16, 16, 0, 0}};

int nblk(long long n, int t = 256) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// NHWC elementwise kernels (8 BF16 per 16-byte vector)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void unpack8(const uint4& q, float (&f)[8]) {
  const bf16* e = reinterpret_cast<const bf16*>(&q);
#pragma unroll
  for (int j = 0; j < 8; ++j) f[j] = __bfloat162float(e[j]);
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  uint4 q;
  bf16* e = reinterpret_cast<bf16*>(&q);
#pragma unroll
  for (int j = 0; j < 8; ++j) e[j] = __float2bfloat16_rn(f[j]);
  return q;
}

// y[b][h][w][:] = mean of x over the 2x2 block (x is 2h x 2w)
__global__ void pool2_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, int B, int h, int w, int C) {
  const long long nv = (long long)B * h * w * (C / 8);
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const int cv = (int)(t % (C / 8));
  const long long p = t / (C / 8);
  const int xx = (int)(p % w), yy = (int)((p / w) % h), b = (int)(p / ((long long)w * h));
  const int W2 = 2 * w;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const size_t src = (((size_t)b * 2 * h + 2 * yy + (q >> 1)) * W2 + 2 * xx + (q & 1)) * C / 8 + cv;
    float f[8];
    unpack8(reinterpret_cast<const uint4*>(x)[src], f);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] += f[j];
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] *= 0.25f;
  reinterpret_cast<uint4*>(y)[t] = pack8(acc);
}

// u[b][Y][X] = t[b][Y/2][X/2] + skip[b][Y][X]  (u is H x W, t is H/2 x W/2)
__global__ void up_add_kernel(const bf16* __restrict__ t, const bf16* __restrict__ skip, bf16* __restrict__ u,
                              int B, int H, int W, int C) {
  const long long nv = (long long)B * H * W * (C / 8);
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int cv = (int)(i % (C / 8));
  const long long p = i / (C / 8);
  const int X = (int)(p % W), Y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
  const size_t src = (((size_t)b * (H / 2) + Y / 2) * (W / 2) + X / 2) * (C / 8) + cv;
  float a[8], s[8];
  unpack8(reinterpret_cast<const uint4*>(t)[src], a);
  unpack8(reinterpret_cast<const uint4*>(skip)[i], s);
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] += s[j];
  reinterpret_cast<uint4*>(u)[i] = pack8(a);
}

// d = y > 0 ? d : 0 (ReLU backward from the stored post-activation y)
__global__ void relu_mask_kernel(bf16* __restrict__ d, const bf16* __restrict__ y, long long nv) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nv) return;
  float a[8], b[8];
  unpack8(reinterpret_cast<const uint4*>(d)[i], a);
  unpack8(reinterpret_cast<const uint4*>(y)[i], b);
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = b[j] > 0.0f ? a[j] : 0.0f;
  reinterpret_cast<uint4*>(d)[i] = pack8(a);
}

// dt[b][y][x] = sum of du over the 2x2 block (upsampling backward)
__global__ void up_back_kernel(const bf16* __restrict__ du, bf16* __restrict__ dt, int B, int h, int w, int C) {
  const long long nv = (long long)B * h * w * (C / 8);
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const int cv = (int)(t % (C / 8));
  const long long p = t / (C / 8);
  const int xx = (int)(p % w), yy = (int)((p / w) % h), b = (int)(p / ((long long)w * h));
  const int W2 = 2 * w;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const size_t src = (((size_t)b * 2 * h + 2 * yy + (q >> 1)) * W2 + 2 * xx + (q & 1)) * C / 8 + cv;
    float f[8];
    unpack8(reinterpret_cast<const uint4*>(du)[src], f);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] += f[j];
  }
  reinterpret_cast<uint4*>(dt)[t] = pack8(acc);
}

// dx[b][Y][X] = dskip[b][Y][X] + dp[b][Y/2][X/2] / 4  (pooling backward + skip)
__global__ void pool_back_add_kernel(const bf16* __restrict__ dskip, const bf16* __restrict__ dp,
                                     bf16* __restrict__ dx, int B, int H, int W, int C) {
  const long long nv = (long long)B * H * W * (C / 8);
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int cv = (int)(i % (C / 8));
  const long long p = i / (C / 8);
  const int X = (int)(p % W), Y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
  const size_t src = (((size_t)b * (H / 2) + Y / 2) * (W / 2) + X / 2) * (C / 8) + cv;
  float a[8], s[8];
  unpack8(reinterpret_cast<const uint4*>(dp)[src], a);
  unpack8(reinterpret_cast<const uint4*>(dskip)[i], s);
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = s[j] + 0.25f * a[j];
  reinterpret_cast<uint4*>(dx)[i] = pack8(a);
}

// per-channel partial sums of d over pixel stripes (bias gradient, pass 1)
constexpr int kBiasBlocks = 256;
__global__ void bias_partial_kernel(const bf16* __restrict__ d, long long npix, int C, float* __restrict__ part) {
  // thread c of the block sums channel c over pixels blockIdx.x, + gridDim.x, ...
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    float s = 0.0f;
    for (long long p = blockIdx.x; p < npix; p += gridDim.x) s += __bfloat162float(d[p * C + c]);
    part[(size_t)blockIdx.x * C + c] = s;
  }
}
__global__ void bias_final_kernel(const float* __restrict__ part, int nb, int C, float* db, int accumulate) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.0f;
  for (int k = 0; k < nb; ++k) s += part[(size_t)k * C + c];
  db[c] = accumulate ? db[c] + s : s;
}

// BF16 copies of the FP32 master weights: w16 [Cout][9][Cin] and the flipped,
// transposed wf16 [Cin][9][Cout] with wf[ci][t][co] = w[co][8 - t][ci]
__global__ void weights_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ w16, bf16* __restrict__ wf16,
                                    int Cin, int Cout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 9 * Cin * Cout) return;
  const int ci = i % Cin, t = (i / Cin) % 9, co = i / (9 * Cin);
  const bf16 v = __float2bfloat16_rn(w[i]);
  w16[i] = v;
  wf16[((size_t)ci * 9 + (8 - t)) * Cout + co] = v;
}

// Adam (bias-corrected), FP32 master parameters
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float c1, float c2,
                            float eps) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// input pack: FP32 [npix][kInCh] -> BF16 [npix][16] (zero padded)
__global__ void pack_input_kernel(const float* __restrict__ in, bf16* __restrict__ x, long long npix, int cin) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= npix) return;
  float f[8];
  for (int h = 0; h < 2; ++h) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = 8 * h + j;
      f[j] = c < cin ? in[p * cin + c] : 0.0f;
    }
    reinterpret_cast<uint4*>(x)[p * 2 + h] = pack8(f);
  }
}

// loss: mean over used pixels of sum_c (out[c] - target[c])^2 for the first
// cout channels; per-block partial loss, and dout = 2 (out - target) / n in
// BF16 (channels >= cout get zero gradient)
__global__ void mse_kernel(const float* __restrict__ out, const float* __restrict__ target, int cout,
                           long long npix, float inv_n, bf16* __restrict__ dout, float* __restrict__ part) {
  __shared__ float sh[256];
  float acc = 0.0f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
       p += (long long)gridDim.x * blockDim.x) {
    float f[8];
    for (int h = 0; h < 2; ++h) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = 8 * h + j;
        float d = 0.0f;
        if (c < cout) {
          d = out[p * 16 + c] - target[p * cout + c];
          acc += d * d;
        }
        f[j] = 2.0f * d * inv_n;
      }
      reinterpret_cast<uint4*>(dout)[p * 2 + h] = pack8(f);
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void sum_final_kernel(const float* __restrict__ part, int n, float scale, float* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float s = 0.0f;
    for (int k = 0; k < n; ++k) s += part[k];
    *out = s * scale;
  }
}

// output unpack: FP32 [npix][16] -> [npix][cout]
__global__ void unpack_output_kernel(const float* __restrict__ o16, float* __restrict__ out, long long npix,
                                     int cout) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= npix * cout) return;
  const long long p = i / cout;
  const int c = (int)(i % cout);
  out[i] = o16[p * 16 + c];
}

}  // namespace

// ---------------------------------------------------------------------------
// the network object
// ---------------------------------------------------------------------------
struct xc_nn {
  int H, W, B;
  int in_ch, out_ch;
  // parameters: one FP32 block [w_0 b_0 w_1 b_1 ...], gradients and Adam
  // moments alike; BF16 copies of the weights (plain and flipped)
  float* params;
  float* grads;
  float* m1;
  float* m2;
  long long nparams;
  long long woff[kLayers], boff[kLayers];
  bf16* w16[kLayers];
  bf16* wf16[kLayers];
  int adam_t;
  // activations (BF16 NHWC) of one batch, and their gradients
  bf16 *in0, *a0, *x0, *p1, *a1, *x1, *p2, *a2, *x2, *p3, *a3, *x3, *t3, *u2, *y2, *t2, *u1, *y1, *t1, *u0, *y0;
  float* out16;       // FP32 [npix0][16]
  bf16* gl[4][3];     // three gradient buffers per level, sized for the level's widest tensor
  float* partial;     // wgrad scratch
  int partial_blocks;
  float* bias_part;
  float* loss_part;
  float* loss;
  int* err;
  std::vector<void*> allocs;
  cudaStream_t stream;
};

namespace {

template <typename T>
int nn_alloc(xc_nn* n, T** p, size_t count) {
  void* q = nullptr;
  XC_CUDA_TRY(cudaMalloc(&q, sizeof(T) * count));
  n->allocs.push_back(q);
  *p = (T*)q;
  return XC_OK;
}

long long npix(const xc_nn* n, int level) { return (long long)n->B * (n->H >> level) * (n->W >> level); }

int conv(xc_nn* n, int L, const bf16* x, bf16* y, float* y32, cudaStream_t s) {
  const int lev = kSpec[L][2];
  return nn_conv3x3_fwd(x, n->w16[L], n->params + n->boff[L], y, y32, n->B, n->H >> lev, n->W >> lev, kSpec[L][0],
                        kSpec[L][1], kSpec[L][3], n->err, s);
}

// data gradient of layer L: dx = conv(dy, flipped weights), no bias
int conv_dgrad(xc_nn* n, int L, const bf16* dy, bf16* dx, cudaStream_t s) {
  const int lev = kSpec[L][2];
  return nn_conv3x3_fwd(dy, n->wf16[L], nullptr, dx, nullptr, n->B, n->H >> lev, n->W >> lev, kSpec[L][1],
                        kSpec[L][0], 0, n->err, s);
}

int conv_wgrad(xc_nn* n, int L, const bf16* x, const bf16* dy, cudaStream_t s) {
  const int lev = kSpec[L][2];
  const int H = n->H >> lev, W = n->W >> lev;
  XC_TRY(nn_conv3x3_wgrad(x, dy, n->grads + n->woff[L], n->partial, n->partial_blocks, n->B, H, W, kSpec[L][0],
                          kSpec[L][1], 1.0f, 0, n->err, s));
  const int C = kSpec[L][1];
  bias_partial_kernel<<<kBiasBlocks, 128, 0, s>>>(dy, npix(n, lev), C, n->bias_part); xc_count_launch();
  bias_final_kernel<<<1, 128, 0, s>>>(n->bias_part, kBiasBlocks, C, n->grads + n->boff[L], 0); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int pool(xc_nn* n, int lev_out, const bf16* x, bf16* y, int C, cudaStream_t s) {
  const long long nv = npix(n, lev_out) * (C / 8);
  pool2_kernel<<<nblk(nv), 256, 0, s>>>(x, y, n->B, n->H >> lev_out, n->W >> lev_out, C); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int up_add(xc_nn* n, int lev_out, const bf16* t, const bf16* skip, bf16* u, int C, cudaStream_t s) {
  const long long nv = npix(n, lev_out) * (C / 8);
  up_add_kernel<<<nblk(nv), 256, 0, s>>>(t, skip, u, n->B, n->H >> lev_out, n->W >> lev_out, C); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int relu_mask(xc_nn* n, int lev, bf16* d, const bf16* y, int C, cudaStream_t s) {
  const long long nv = npix(n, lev) * (C / 8);
  relu_mask_kernel<<<nblk(nv), 256, 0, s>>>(d, y, nv); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int up_back(xc_nn* n, int lev_out, const bf16* du, bf16* dt, int C, cudaStream_t s) {
  const long long nv = npix(n, lev_out) * (C / 8);
  up_back_kernel<<<nblk(nv), 256, 0, s>>>(du, dt, n->B, n->H >> lev_out, n->W >> lev_out, C); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int pool_back_add(xc_nn* n, int lev_out, const bf16* dskip, const bf16* dp, bf16* dx, int C, cudaStream_t s) {
  const long long nv = npix(n, lev_out) * (C / 8);
  pool_back_add_kernel<<<nblk(nv), 256, 0, s>>>(dskip, dp, dx, n->B, n->H >> lev_out, n->W >> lev_out, C);
  xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int refresh_bf16(xc_nn* n, cudaStream_t s) {
  for (int L = 0; L < kLayers; ++L) {
    const int ne = 9 * kSpec[L][0] * kSpec[L][1];
    weights_bf16_kernel<<<nblk(ne), 256, 0, s>>>(n->params + n->woff[L], n->w16[L], n->wf16[L], kSpec[L][0],
                                                  kSpec[L][1]);
    xc_count_launch();
  }
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int forward(xc_nn* n, const float* in, cudaStream_t s) {
  const long long p0 = npix(n, 0);
  pack_input_kernel<<<nblk(p0), 256, 0, s>>>(in, n->in0, p0, n->in_ch); xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_TRY(conv(n, C0A, n->in0, n->a0, nullptr, s));
  XC_TRY(conv(n, C0B, n->a0, n->x0, nullptr, s));
  XC_TRY(pool(n, 1, n->x0, n->p1, 16, s));
  XC_TRY(conv(n, C1A, n->p1, n->a1, nullptr, s));
  XC_TRY(conv(n, C1B, n->a1, n->x1, nullptr, s));
  XC_TRY(pool(n, 2, n->x1, n->p2, 32, s));
  XC_TRY(conv(n, C2A, n->p2, n->a2, nullptr, s));
  XC_TRY(conv(n, C2B, n->a2, n->x2, nullptr, s));
  XC_TRY(pool(n, 3, n->x2, n->p3, 64, s));
  XC_TRY(conv(n, C3A, n->p3, n->a3, nullptr, s));
  XC_TRY(conv(n, C3B, n->a3, n->x3, nullptr, s));
  XC_TRY(conv(n, C3U, n->x3, n->t3, nullptr, s));
  XC_TRY(up_add(n, 2, n->t3, n->x2, n->u2, 64, s));
  XC_TRY(conv(n, C2D, n->u2, n->y2, nullptr, s));
  XC_TRY(conv(n, C2U, n->y2, n->t2, nullptr, s));
  XC_TRY(up_add(n, 1, n->t2, n->x1, n->u1, 32, s));
  XC_TRY(conv(n, C1D, n->u1, n->y1, nullptr, s));
  XC_TRY(conv(n, C1U, n->y1, n->t1, nullptr, s));
  XC_TRY(up_add(n, 0, n->t1, n->x0, n->u0, 16, s));
  XC_TRY(conv(n, C0D, n->u0, n->y0, nullptr, s));
  XC_TRY(conv(n, COUT, n->y0, nullptr, n->out16, s));
  return XC_OK;
}

// backward from dout (BF16 [npix0][16], in gl[0][0]); fills n->grads
int backward(xc_nn* n, cudaStream_t s) {
  bf16** G0 = n->gl[0];
  bf16** G1 = n->gl[1];
  bf16** G2 = n->gl[2];
  bf16** G3 = n->gl[3];
  // level 0 output
  XC_TRY(conv_wgrad(n, COUT, n->y0, G0[0], s));
  XC_TRY(conv_dgrad(n, COUT, G0[0], G0[1], s));          // d y0
  XC_TRY(relu_mask(n, 0, G0[1], n->y0, 16, s));
  XC_TRY(conv_wgrad(n, C0D, n->u0, G0[1], s));
  XC_TRY(conv_dgrad(n, C0D, G0[1], G0[2], s));          // d u0 = d x0 (skip part)
  XC_TRY(up_back(n, 1, G0[2], G1[0], 16, s));           // d t1
  XC_TRY(conv_wgrad(n, C1U, n->y1, G1[0], s));
  XC_TRY(conv_dgrad(n, C1U, G1[0], G1[1], s));          // d y1 (32 ch)
  XC_TRY(relu_mask(n, 1, G1[1], n->y1, 32, s));
  XC_TRY(conv_wgrad(n, C1D, n->u1, G1[1], s));
  XC_TRY(conv_dgrad(n, C1D, G1[1], G1[2], s));          // d u1 = d x1 (skip part)
  XC_TRY(up_back(n, 2, G1[2], G2[0], 32, s));           // d t2
  XC_TRY(conv_wgrad(n, C2U, n->y2, G2[0], s));
  XC_TRY(conv_dgrad(n, C2U, G2[0], G2[1], s));          // d y2 (64)
  XC_TRY(relu_mask(n, 2, G2[1], n->y2, 64, s));
  XC_TRY(conv_wgrad(n, C2D, n->u2, G2[1], s));
  XC_TRY(conv_dgrad(n, C2D, G2[1], G2[2], s));          // d u2 = d x2 (skip part)
  XC_TRY(up_back(n, 3, G2[2], G3[0], 64, s));           // d t3
  XC_TRY(conv_wgrad(n, C3U, n->x3, G3[0], s));
  XC_TRY(conv_dgrad(n, C3U, G3[0], G3[1], s));          // d x3 (128)
  XC_TRY(relu_mask(n, 3, G3[1], n->x3, 128, s));
  XC_TRY(conv_wgrad(n, C3B, n->a3, G3[1], s));
  XC_TRY(conv_dgrad(n, C3B, G3[1], G3[2], s));          // d a3
  XC_TRY(relu_mask(n, 3, G3[2], n->a3, 128, s));
  XC_TRY(conv_wgrad(n, C3A, n->p3, G3[2], s));
  XC_TRY(conv_dgrad(n, C3A, G3[2], G3[0], s));          // d p3 (64)
  XC_TRY(pool_back_add(n, 2, G2[2], G3[0], G2[0], 64, s));   // d x2
  XC_TRY(relu_mask(n, 2, G2[0], n->x2, 64, s));
  XC_TRY(conv_wgrad(n, C2B, n->a2, G2[0], s));
  XC_TRY(conv_dgrad(n, C2B, G2[0], G2[1], s));          // d a2
  XC_TRY(relu_mask(n, 2, G2[1], n->a2, 64, s));
  XC_TRY(conv_wgrad(n, C2A, n->p2, G2[1], s));
  XC_TRY(conv_dgrad(n, C2A, G2[1], G2[2], s));          // d p2 (32)
  XC_TRY(pool_back_add(n, 1, G1[2], G2[2], G1[0], 32, s));   // d x1
  XC_TRY(relu_mask(n, 1, G1[0], n->x1, 32, s));
  XC_TRY(conv_wgrad(n, C1B, n->a1, G1[0], s));
  XC_TRY(conv_dgrad(n, C1B, G1[0], G1[1], s));          // d a1
  XC_TRY(relu_mask(n, 1, G1[1], n->a1, 32, s));
  XC_TRY(conv_wgrad(n, C1A, n->p1, G1[1], s));
  XC_TRY(conv_dgrad(n, C1A, G1[1], G1[2], s));          // d p1 (16)
  XC_TRY(pool_back_add(n, 0, G0[2], G1[2], G0[0], 16, s));   // d x0
  XC_TRY(relu_mask(n, 0, G0[0], n->x0, 16, s));
  XC_TRY(conv_wgrad(n, C0B, n->a0, G0[0], s));
  XC_TRY(conv_dgrad(n, C0B, G0[0], G0[1], s));          // d a0
  XC_TRY(relu_mask(n, 0, G0[1], n->a0, 16, s));
  XC_TRY(conv_wgrad(n, C0A, n->in0, G0[1], s));
  return XC_OK;
}

int loss_and_dout(xc_nn* n, const float* target, cudaStream_t s) {
  const long long p0 = npix(n, 0);
  const float inv_n = 1.0f / (float)p0;
  mse_kernel<<<256, 256, 0, s>>>(n->out16, target, n->out_ch, p0, inv_n, n->gl[0][0], n->loss_part); xc_count_launch();
  sum_final_kernel<<<1, 32, 0, s>>>(n->loss_part, 256, inv_n, n->loss); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

int check_err(xc_nn* n, cudaStream_t s, const char* what) {
  int h = 0;
  XC_CUDA_TRY(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  XC_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) {
    xc_set_error("%s: a bounded wait inside a convolution kernel ran out (code %d)", what, h);
    return XC_TIMEOUT;
  }
  return XC_OK;
}

// He-normal initial weights from a host generator (splitmix64 + Box-Muller),
// zero biases; the output layer starts small
void init_params(xc_nn* n, unsigned long long seed, std::vector<float>& h) {
  h.assign((size_t)n->nparams, 0.0f);
  unsigned long long st = seed * 0x9E3779B97F4A7C15ULL + 1;
  auto next = [&]() {
    unsigned long long z = (st += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int L = 0; L < kLayers; ++L) {
    const int fan_in = 9 * (L == C0A ? n->in_ch : kSpec[L][0]);
    const double sd = std::sqrt(2.0 / fan_in) * (L == COUT ? 0.1 : 1.0);
    const long long ne = 9LL * kSpec[L][0] * kSpec[L][1];
    for (long long i = 0; i < ne; ++i) {
      const double u1 = next() + 1e-300, u2 = next();
      h[(size_t)(n->woff[L] + i)] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// internal entry points (the Stokes solver's learned preconditioner)
// ---------------------------------------------------------------------------
int nn_forward_async(xc_nn* n, const float* in, cudaStream_t s) { return forward(n, in, s); }
const float* nn_out16(const xc_nn* n) { return n->out16; }
int nn_check(xc_nn* n, cudaStream_t s) { return check_err(n, s, "learned preconditioner"); }

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int xc_nn_create(int H, int W, int batch, int in_ch, int out_ch, unsigned long long seed, xc_nn** out) {
  if (!out) { xc_set_error("xc_nn_create: null output"); return XC_BAD_ARG; }
  *out = nullptr;
  if (H < 8 || W < 8 || H % 8 || W % 8 || batch < 1 || in_ch < 1 || in_ch > 16 || out_ch < 1 || out_ch > 16) {
    xc_set_error("xc_nn_create: need H, W multiples of 8, batch >= 1, 1 <= in_ch, out_ch <= 16");
    return XC_BAD_ARG;
  }
  // every level must tile into 128-pixel tiles (checked again per launch)
  for (int l = 0; l < 4; ++l) {
    const int w = W >> l, h = H >> l;
    const int bw = w >= 128 ? 128 : w;
    if (128 % bw || w % bw || h % (128 / bw)) {
      xc_set_error("xc_nn_create: level %d (%d x %d) does not tile into 128-pixel tiles", l, h, w);
      return XC_BAD_ARG;
    }
  }
  xc_nn* n = new xc_nn();
  n->H = H; n->W = W; n->B = batch; n->in_ch = in_ch; n->out_ch = out_ch;
  auto fail = [&](int st) { xc_nn_destroy(n); return st; };
  if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) {
    xc_set_error("xc_nn_create: stream creation failed");
    return fail(XC_CUDA);
  }
  long long off = 0;
  for (int L = 0; L < kLayers; ++L) {
    n->woff[L] = off;
    off += 9LL * kSpec[L][0] * kSpec[L][1];
    n->boff[L] = off;
    off += kSpec[L][1];
    off = (off + 3) & ~3LL;   // 16-byte aligned blocks
  }
  n->nparams = off;
  int st = XC_OK;
#define NN_ALLOC(p, cnt) if ((st = nn_alloc(n, &(p), (size_t)(cnt))) != XC_OK) return fail(st)
  NN_ALLOC(n->params, off);
  NN_ALLOC(n->grads, off);
  NN_ALLOC(n->m1, off);
  NN_ALLOC(n->m2, off);
  for (int L = 0; L < kLayers; ++L) {
    NN_ALLOC(n->w16[L], 9 * kSpec[L][0] * kSpec[L][1]);
    NN_ALLOC(n->wf16[L], 9 * kSpec[L][0] * kSpec[L][1]);
  }
  const long long p[4] = {npix(n, 0), npix(n, 1), npix(n, 2), npix(n, 3)};
  NN_ALLOC(n->in0, p[0] * 16); NN_ALLOC(n->a0, p[0] * 16); NN_ALLOC(n->x0, p[0] * 16);
  NN_ALLOC(n->u0, p[0] * 16); NN_ALLOC(n->y0, p[0] * 16);
  NN_ALLOC(n->p1, p[1] * 16); NN_ALLOC(n->t1, p[1] * 16);
  NN_ALLOC(n->a1, p[1] * 32); NN_ALLOC(n->x1, p[1] * 32); NN_ALLOC(n->u1, p[1] * 32); NN_ALLOC(n->y1, p[1] * 32);
  NN_ALLOC(n->p2, p[2] * 32); NN_ALLOC(n->t2, p[2] * 32);
  NN_ALLOC(n->a2, p[2] * 64); NN_ALLOC(n->x2, p[2] * 64); NN_ALLOC(n->u2, p[2] * 64); NN_ALLOC(n->y2, p[2] * 64);
  NN_ALLOC(n->p3, p[3] * 64); NN_ALLOC(n->t3, p[3] * 64);
  NN_ALLOC(n->a3, p[3] * 128); NN_ALLOC(n->x3, p[3] * 128);
  NN_ALLOC(n->out16, p[0] * 16);
  const int widest[4] = {16, 32, 64, 128};
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k < 3; ++k) NN_ALLOC(n->gl[l][k], p[l] * widest[l]);
  n->partial_blocks = 2 * kNumSMs / 9 + 1;
  NN_ALLOC(n->partial, (size_t)n->partial_blocks * 9 * 128 * 128);
  NN_ALLOC(n->bias_part, (size_t)kBiasBlocks * 128);
  NN_ALLOC(n->loss_part, 256);
  NN_ALLOC(n->loss, 1);
  NN_ALLOC(n->err, 1);
#undef NN_ALLOC
  cudaStream_t s = n->stream;
  std::vector<float> h;
  init_params(n, seed, h);
  if (cudaMemcpyAsync(n->params, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(n->m1, 0, sizeof(float) * off, s) != cudaSuccess ||
      cudaMemsetAsync(n->m2, 0, sizeof(float) * off, s) != cudaSuccess ||
      cudaMemsetAsync(n->grads, 0, sizeof(float) * off, s) != cudaSuccess ||
      cudaMemsetAsync(n->err, 0, sizeof(int), s) != cudaSuccess) {
    xc_set_error("xc_nn_create: initialisation copy failed");
    return fail(XC_CUDA);
  }
  if ((st = refresh_bf16(n, s)) != XC_OK) return fail(st);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    xc_set_error("xc_nn_create: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(XC_CUDA);
  }
  *out = n;
  return XC_OK;
}

extern "C" int xc_nn_destroy(xc_nn* n) {
  if (!n) return XC_OK;
  if (n->stream) cudaStreamSynchronize(n->stream);
  for (void* p : n->allocs) cudaFree(p);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
  return XC_OK;
}

extern "C" long long xc_nn_param_count(const xc_nn* n) { return n ? n->nparams : 0; }

extern "C" int xc_nn_layout(const xc_nn* n, long long* woff, long long* boff, int* spec) {
  if (!n || !woff || !boff || !spec) { xc_set_error("xc_nn_layout: null argument"); return XC_BAD_ARG; }
  for (int L = 0; L < kLayers; ++L) {
    woff[L] = n->woff[L];
    boff[L] = n->boff[L];
    for (int k = 0; k < 4; ++k) spec[4 * L + k] = kSpec[L][k];
  }
  return XC_OK;
}

extern "C" int xc_nn_get_params(xc_nn* n, float* host) {
  if (!n || !host) { xc_set_error("xc_nn_get_params: null argument"); return XC_BAD_ARG; }
  XC_CUDA_TRY(cudaMemcpyAsync(host, n->params, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost, n->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(n->stream));
  return XC_OK;
}

extern "C" int xc_nn_set_params(xc_nn* n, const float* host) {
  if (!n || !host) { xc_set_error("xc_nn_set_params: null argument"); return XC_BAD_ARG; }
  XC_CUDA_TRY(cudaMemcpyAsync(n->params, host, sizeof(float) * n->nparams, cudaMemcpyHostToDevice, n->stream));
  XC_TRY(refresh_bf16(n, n->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(n->stream));
  return XC_OK;
}

extern "C" int xc_nn_get_grads(xc_nn* n, float* host) {
  if (!n || !host) { xc_set_error("xc_nn_get_grads: null argument"); return XC_BAD_ARG; }
  XC_CUDA_TRY(cudaMemcpyAsync(host, n->grads, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost, n->stream));
  XC_CUDA_TRY(cudaStreamSynchronize(n->stream));
  return XC_OK;
}

extern "C" int xc_nn_forward(xc_nn* n, const float* in, float* out, void* stream) {
  if (!n || !in || !out) { xc_set_error("xc_nn_forward: null argument"); return XC_BAD_ARG; }
  cudaStream_t s = stream ? (cudaStream_t)stream : n->stream;
  XC_TRY(forward(n, in, s));
  const long long p0 = npix(n, 0);
  unpack_output_kernel<<<nblk(p0 * n->out_ch), 256, 0, s>>>(n->out16, out, p0, n->out_ch); xc_count_launch();
  XC_LAUNCH_CHECK();
  return check_err(n, s, "xc_nn_forward");
}

extern "C" int xc_nn_loss_grad(xc_nn* n, const float* in, const float* target, float* loss, void* stream) {
  if (!n || !in || !target) { xc_set_error("xc_nn_loss_grad: null argument"); return XC_BAD_ARG; }
  cudaStream_t s = stream ? (cudaStream_t)stream : n->stream;
  XC_TRY(forward(n, in, s));
  XC_TRY(loss_and_dout(n, target, s));
  XC_TRY(backward(n, s));
  if (loss) XC_CUDA_TRY(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  return check_err(n, s, "xc_nn_loss_grad");
}

extern "C" int xc_nn_train_step(xc_nn* n, const float* in, const float* target, float lr, float* loss,
                                void* stream) {
  if (!n || !in || !target) { xc_set_error("xc_nn_train_step: null argument"); return XC_BAD_ARG; }
  cudaStream_t s = stream ? (cudaStream_t)stream : n->stream;
  XC_TRY(forward(n, in, s));
  XC_TRY(loss_and_dout(n, target, s));
  XC_TRY(backward(n, s));
  ++n->adam_t;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, (float)n->adam_t), c2 = 1.0f - std::pow(b2, (float)n->adam_t);
  adam_kernel<<<nblk(n->nparams), 256, 0, s>>>(n->params, n->grads, n->m1, n->m2, n->nparams, lr, b1, b2, c1, c2,
                                               1e-8f);
  xc_count_launch();
  XC_LAUNCH_CHECK();
  XC_TRY(refresh_bf16(n, s));
  if (loss) XC_CUDA_TRY(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  return check_err(n, s, "xc_nn_train_step");
}
