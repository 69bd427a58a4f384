// 3x3 convolutions of the learned preconditioner's U-Net on the 5th-generation
// tensor cores (tcgen05), BF16 operands with FP32 accumulation in TMEM.
//
// Activations are NHWC BF16 (channels contiguous), weights [Cout][9][Cin]
// BF16 (tap t = 3 * (dy + 1) + (dx + 1)).  Zero padding at the image edge.
//
// Forward (and the data gradient, which is the forward convolution of dY with
// the flipped, transposed weights): an implicit GEMM with M = 128 pixels of
// one tile, N = Cout, K = 9 taps x Cin.  For every (tap, channel chunk) a TMA
// load brings the tile's 128 pixels shifted by the tap -- out-of-image pixels
// arrive as zeros, which is the padding -- and the Cout x chunk weight block,
// both in the K-major swizzled layout the tensor core reads; a 4-stage
// mbarrier ring overlaps the loads with the MMAs; one thread issues the MMAs;
// the accumulator (128 lanes x Cout FP32 columns of TMEM) is read back by all
// four warps for the epilogue (bias, ReLU, BF16 and/or FP32 store).
//
// Weight gradient: dW[co][t][ci] = sum_p dY[p][co] X[p + off(t)][ci], a GEMM
// with M = Cout (zero-padded to 128), N = Cin, K = pixels.  Both operands are
// channel-contiguous in memory, i.e. MN-major; the CTA's threads transpose
// each 128-pixel tile into the K-major swizzled layout in shared memory
// (double buffered), one thread issues the MMAs, and the per-CTA FP32 partial
// sums are reduced over CTAs in a fixed order (deterministic).
#include <cstring>
#include <mutex>

#include <cuda_bf16.h>

#include "xc_internal.cuh"
#include "xc_nn.cuh"
#include "xc_nn_tc.cuh"

using namespace xcnn;

namespace {

// ---------------------------------------------------------------------------
// tensor maps (driver entry point looked up through the runtime)
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

CUtensorMapSwizzle swizzle_for(int row_bytes) {
  return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                          : (row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

// NHWC BF16 activations as (C, W, H, B), box (kc, bw, bh, 1)
int make_act_map(CUtensorMap* tm, const void* p, int B, int H, int W, int C, int kc, int bw, int bh) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) { xc_set_error("cuTensorMapEncodeTiled is not available from the driver"); return XC_CUDA; }
  if (((uintptr_t)p & 15u) != 0) { xc_set_error("conv3x3: activation pointer not 16-byte aligned"); return XC_BAD_ARG; }
  cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
  cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  cuuint32_t box[4] = {(cuuint32_t)kc, (cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(p), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { xc_set_error("cuTensorMapEncodeTiled (activations) failed: %d", (int)r); return XC_CUDA; }
  return XC_OK;
}

// weights [Cout][9][Cin] BF16 as (Cin, 9, Cout), box (kc, 1, Cout)
int make_weight_map(CUtensorMap* tm, const void* p, int Cin, int Cout, int kc) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) { xc_set_error("cuTensorMapEncodeTiled is not available from the driver"); return XC_CUDA; }
  if (((uintptr_t)p & 15u) != 0) { xc_set_error("conv3x3: weight pointer not 16-byte aligned"); return XC_BAD_ARG; }
  cuuint64_t dims[3] = {(cuuint64_t)Cin, 9, (cuuint64_t)Cout};
  cuuint64_t strides[2] = {(cuuint64_t)Cin * 2, (cuuint64_t)9 * Cin * 2};
  cuuint32_t box[3] = {(cuuint32_t)kc, 1, (cuuint32_t)Cout};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(p), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { xc_set_error("cuTensorMapEncodeTiled (weights) failed: %d", (int)r); return XC_CUDA; }
  return XC_OK;
}

struct ConvArgs {
  int B, H, W, Cin, nkc, bw, bh;
  const float* bias;        // [Cout] or null
  int relu;                 // 1: max(v, 0) after the bias
  __nv_bfloat16* out;       // NHWC [.., Cout] or null
  float* out_f32;           // NHWC [.., Cout] or null
  int* err;                 // set to a nonzero code when a bounded wait ran out
};

constexpr int kStages = 4;

template <int KC, int NOUT>
struct FwdCfg {
  static constexpr uint32_t kRowBytes = KC * 2;
  static constexpr uint32_t kABytes = 128u * KC * 2;
  static constexpr uint32_t kBBytes = NOUT * KC * 2;
  static constexpr uint32_t kAStride = (kABytes + 1023u) & ~1023u;
  static constexpr uint32_t kBStride = (kBBytes + 1023u) & ~1023u;
  static constexpr uint32_t kStage = kAStride + kBStride;
  static constexpr uint32_t kSmem = kStages * kStage + 1024u;
  static constexpr uint32_t kTmemCols = tmem_cols_for(NOUT);
};

__device__ __forceinline__ void flag_error(int* err, int code) {
  if (err) atomicExch(err, code);
}

template <int KC, int NOUT>
__global__ void __launch_bounds__(128, 1) conv3x3_fwd_kernel(const __grid_constant__ CUtensorMap tmA,
                                                             const __grid_constant__ CUtensorMap tmB,
                                                             ConvArgs a) {
  using Cfg = FwdCfg<KC, NOUT>;
  constexpr uint32_t SBO = 8u * Cfg::kRowBytes;
  constexpr uint32_t LAYOUT = layout_for_row_bytes(Cfg::kRowBytes);
  constexpr uint32_t IDESC = idesc_bf16(128, NOUT);
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar_full[kStages];
  __shared__ __align__(8) uint64_t bar_empty[kStages];
  __shared__ __align__(8) uint64_t bar_done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_done;
  const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_x = a.W / a.bw, tiles_y = a.H / a.bh;
  const int b = blockIdx.x / (tiles_x * tiles_y);
  const int rem = blockIdx.x - b * tiles_x * tiles_y;
  const int y0 = (rem / tiles_x) * a.bh, x0 = (rem % tiles_x) * a.bw;
  const int nk = 9 * a.nkc;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    mbar_init(smem_u32(&bar_done), 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_slot), Cfg::kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  int issued = 0;   // loads issued by the producer thread
  if (warp == 0 && lane == 0) {
    // TMA producer: slot s is refilled once the MMAs that read it completed
    for (int kk = 0; kk < nk; ++kk) {
      const int s = kk % kStages;
      if (kk >= kStages && !mbar_wait(smem_u32(&bar_empty[s]), ((kk / kStages) - 1) & 1)) {
        flag_error(a.err, 1);
        break;
      }
      const int tap = kk / a.nkc, kc = kk - tap * a.nkc;
      const int dy = tap / 3 - 1, dx = tap % 3 - 1;
      const uint32_t full = smem_u32(&bar_full[s]);
      const uint32_t sa = base + s * Cfg::kStage;
      mbar_expect_tx(full, Cfg::kABytes + Cfg::kBBytes);
      tma_load_4d(sa, &tmA, kc * KC, x0 + dx, y0 + dy, b, full);
      tma_load_3d(sa + Cfg::kAStride, &tmB, kc * KC, tap, 0, full);
      issued = kk + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kk = 0; kk < nk; ++kk) {
      const int s = kk % kStages;
      if (!mbar_wait(smem_u32(&bar_full[s]), (kk / kStages) & 1)) {
        flag_error(a.err, 2);
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t sa = base + s * Cfg::kStage, sb = sa + Cfg::kAStride;
#pragma unroll
      for (int k = 0; k < KC / 16; ++k)
        umma_bf16(tmem, smem_desc(sa + k * 32, SBO, LAYOUT), smem_desc(sb + k * 32, SBO, LAYOUT), IDESC,
                  (kk | k) != 0 ? 1u : 0u);
      umma_commit(smem_u32(&bar_empty[s]));
    }
    if (ok) umma_commit(smem_u32(&bar_done));
  }
  __syncwarp();

  // epilogue: warp w owns TMEM lanes (tile rows) 32w..32w+31; one thread
  // waits for the last MMA and tells the others (uniform control flow)
  if (threadIdx.x == 0) {
    s_done = mbar_wait(smem_u32(&bar_done), 0) ? 1 : 0;
    if (!s_done) flag_error(a.err, 3);
  }
  __syncthreads();
  tc_fence_after();
  if (s_done) {
    const int m = warp * 32 + lane;
    const int py = y0 + m / a.bw, px = x0 + m % a.bw;
    const size_t pix = ((size_t)b * a.H + py) * a.W + px;
#pragma unroll
    for (int c0 = 0; c0 < NOUT; c0 += 16) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float t = __uint_as_float(r[j]) + (a.bias ? a.bias[c0 + j] : 0.0f);
        v[j] = a.relu ? fmaxf(t, 0.0f) : t;
      }
      if (a.out_f32) {
        float4* o = reinterpret_cast<float4*>(a.out_f32 + pix * NOUT + c0);
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      }
      if (a.out) {
        uint32_t pk[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
          pk[j] = *reinterpret_cast<uint32_t*>(&h);
        }
        uint4* o = reinterpret_cast<uint4*>(a.out + pix * NOUT + c0);
        o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      }
    }
  }
  // after a wait ran out, the producer waits (bounded) for its loads still in
  // flight before the CTA's shared memory is released
  if (!s_done && warp == 0 && lane == 0) {
    for (int kk = issued - kStages > 0 ? issued - kStages : 0; kk < issued; ++kk)
      mbar_wait(smem_u32(&bar_full[kk % kStages]), (kk / kStages) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, Cfg::kTmemCols);
  }
}

template <int KC, int NOUT>
int launch_fwd(const CUtensorMap& ta, const CUtensorMap& tb, const ConvArgs& a, int tiles, cudaStream_t s) {
  using Cfg = FwdCfg<KC, NOUT>;
  static bool attr = false;
  if (!attr) {
    XC_CUDA_TRY(cudaFuncSetAttribute(conv3x3_fwd_kernel<KC, NOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)Cfg::kSmem));
    attr = true;
  }
  conv3x3_fwd_kernel<KC, NOUT><<<tiles, 128, Cfg::kSmem, s>>>(ta, tb, a); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

template <int KC>
int launch_fwd_n(int Cout, const CUtensorMap& ta, const CUtensorMap& tb, const ConvArgs& a, int tiles,
                 cudaStream_t s) {
  switch (Cout) {
    case 16: return launch_fwd<KC, 16>(ta, tb, a, tiles, s);
    case 32: return launch_fwd<KC, 32>(ta, tb, a, tiles, s);
    case 64: return launch_fwd<KC, 64>(ta, tb, a, tiles, s);
    case 128: return launch_fwd<KC, 128>(ta, tb, a, tiles, s);
    default: xc_set_error("conv3x3: Cout must be 16, 32, 64 or 128 (got %d)", Cout); return XC_BAD_ARG;
  }
}

bool tile_shape(int H, int W, int* bw, int* bh) {
  if (W <= 0 || H <= 0) return false;
  *bw = W >= 128 ? 128 : W;
  if (128 % *bw != 0 || W % *bw != 0) return false;
  *bh = 128 / *bw;
  return H % *bh == 0;
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
struct WgradArgs {
  const __nv_bfloat16* x;    // NHWC [B][H][W][Cin]
  const __nv_bfloat16* dy;   // NHWC [B][H][W][Cout]
  float* partial;            // [gridDim.x][Cout][9][Cin]
  int B, H, W, Cin, Cout, bw, bh, tiles;
  int* err;
};

template <int CIN>
struct WgCfg {
  // per stage: A = 128 rows (Cout, zero padded) x 128 pixels, B = CIN rows x
  // 128 pixels, each as two K chunks of 64 pixels (128-byte swizzled rows)
  static constexpr uint32_t kAChunk = 128u * 128u;           // bytes of one 64-pixel chunk of A
  static constexpr uint32_t kBChunk = CIN * 128u;
  static constexpr uint32_t kStage = 2 * kAChunk + 2 * kBChunk;
  static constexpr uint32_t kSmem = 2 * kStage + 1024u;
  static constexpr uint32_t kTmemCols = tmem_cols_for(CIN);
};

template <int CIN>
__global__ void __launch_bounds__(128, 1) conv3x3_wgrad_kernel(WgradArgs a) {
  using Cfg = WgCfg<CIN>;
  constexpr uint32_t IDESC = idesc_bf16(128, CIN);
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar_mma[2];
  __shared__ __align__(8) uint64_t bar_done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_ok;
  const uint32_t base = (smem_u32(dsm) + 1023u) & ~1023u;
  uint8_t* gbase = dsm + (base - smem_u32(dsm));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tap = blockIdx.y;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int tiles_x = a.W / a.bw, tiles_y = a.H / a.bh;

  // zero both stages once: the A rows at and above Cout stay zero
  for (uint32_t o = threadIdx.x * 16u; o < 2 * Cfg::kStage; o += 128u * 16u)
    *reinterpret_cast<uint4*>(gbase + o) = make_uint4(0, 0, 0, 0);
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar_mma[0]), 1);
    mbar_init(smem_u32(&bar_mma[1]), 1);
    mbar_init(smem_u32(&bar_done), 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_slot), Cfg::kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  bool ok = true;
  int it = 0;
  for (int t = blockIdx.x; t < a.tiles; t += gridDim.x, ++it) {
    const int s = it & 1;
    // the MMAs issued two tiles ago read this stage: one thread waits, all
    // follow its verdict (uniform control flow)
    if (it >= 2) {
      if (threadIdx.x == 0) s_ok = mbar_wait(smem_u32(&bar_mma[s]), ((it >> 1) - 1) & 1) ? 1 : 0;
      __syncthreads();
      if (!s_ok) {
        ok = false;
        break;
      }
    }
    uint8_t* stA = gbase + s * Cfg::kStage;
    uint8_t* stB = stA + 2 * Cfg::kAChunk;
    const int b = t / (tiles_x * tiles_y);
    const int rem = t - b * tiles_x * tiles_y;
    const int y0 = (rem / tiles_x) * a.bh, x0 = (rem % tiles_x) * a.bw;
    // thread m stages pixel m of the tile: dY[p][:] into A column m, and
    // X[p + off(tap)][:] (zero outside the image) into B column m
    const int m = threadIdx.x;
    const int py = y0 + m / a.bw, px = x0 + m % a.bw;
    const size_t pix = ((size_t)b * a.H + py) * a.W + px;
    uint8_t* ach = stA + (m >> 6) * Cfg::kAChunk;
    uint8_t* bch = stB + (m >> 6) * Cfg::kBChunk;
    const uint32_t kin = (uint32_t)(m & 63);
    const uint4* gdy = reinterpret_cast<const uint4*>(a.dy + pix * a.Cout);
    for (int v = 0; v < a.Cout / 8; ++v) {
      uint4 q = gdy[v];
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        *reinterpret_cast<__nv_bfloat16*>(ach + swz_offset((uint32_t)(v * 8 + j), kin, 128)) = e[j];
    }
    const int sy = py + dy, sx = px + dx;
    const bool in = sy >= 0 && sy < a.H && sx >= 0 && sx < a.W;
    const uint4* gx = reinterpret_cast<const uint4*>(a.x + (((size_t)b * a.H + (in ? sy : 0)) * a.W + (in ? sx : 0)) * CIN);
    for (int v = 0; v < CIN / 8; ++v) {
      uint4 q = in ? gx[v] : make_uint4(0, 0, 0, 0);
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        *reinterpret_cast<__nv_bfloat16*>(bch + swz_offset((uint32_t)(v * 8 + j), kin, 128)) = e[j];
    }
    fence_async_shared();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t sa = base + s * Cfg::kStage, sb = sa + 2 * Cfg::kAChunk;
#pragma unroll
      for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int k = 0; k < 4; ++k)
          umma_bf16(tmem, smem_desc(sa + c * Cfg::kAChunk + k * 32, 1024, kLayoutSW128),
                    smem_desc(sb + c * Cfg::kBChunk + k * 32, 1024, kLayoutSW128), IDESC,
                    (it | c | k) != 0 ? 1u : 0u);
      umma_commit(smem_u32(&bar_mma[s]));
    }
  }
  if (threadIdx.x == 0) {
    umma_commit(smem_u32(&bar_done));
    s_ok = (ok && mbar_wait(smem_u32(&bar_done), 0)) ? 1 : 0;
    if (!s_ok) flag_error(a.err, 4);
  }
  __syncthreads();
  tc_fence_after();
  if (s_ok) {
    // TMEM lane = output channel co, column = input channel ci
    const int co = warp * 32 + lane;
    float* dst = a.partial + (((size_t)blockIdx.x * a.Cout + co) * 9 + tap) * CIN;
#pragma unroll
    for (int c0 = 0; c0 < CIN; c0 += 16) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      tmem_ld_wait();
      if (co < a.Cout) {
        float4* o = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
        for (int j = 0; j < 4; ++j)
          o[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]), __uint_as_float(r[4 * j + 2]),
                             __uint_as_float(r[4 * j + 3]));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, Cfg::kTmemCols);
  }
}

// dW = sum over CTAs of the partials, in CTA order; scale, optional accumulate
__global__ void wgrad_reduce_kernel(const float* partial, int nblk, int n, float* dw, float scale, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int k = 0; k < nblk; ++k) s += partial[(size_t)k * n + i];
  dw[i] = accumulate ? dw[i] + scale * s : scale * s;
}

template <int CIN>
int launch_wgrad(const WgradArgs& a, int nblk, cudaStream_t s) {
  using Cfg = WgCfg<CIN>;
  static bool attr = false;
  if (!attr) {
    XC_CUDA_TRY(cudaFuncSetAttribute(conv3x3_wgrad_kernel<CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)Cfg::kSmem));
    attr = true;
  }
  conv3x3_wgrad_kernel<CIN><<<dim3(nblk, 9), 128, Cfg::kSmem, s>>>(a); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// internal entry points (xc_nn.cuh)
// ---------------------------------------------------------------------------
int nn_conv3x3_fwd(const void* x, const void* w, const float* bias, void* y, float* y_f32, int B, int H, int W,
                   int Cin, int Cout, int relu, int* err, cudaStream_t s) {
  int bw = 0, bh = 0;
  if (!tile_shape(H, W, &bw, &bh) || B < 1) {
    xc_set_error("conv3x3: image %dx%d does not tile into 128-pixel tiles (W a multiple of 128, or a power of two "
                 "below it dividing H's tiling)", H, W);
    return XC_BAD_ARG;
  }
  if (Cin != 16 && Cin != 32 && Cin != 64 && Cin != 128) {
    xc_set_error("conv3x3: Cin must be 16, 32, 64 or 128 (got %d)", Cin);
    return XC_BAD_ARG;
  }
  if (!y && !y_f32) { xc_set_error("conv3x3: no output"); return XC_BAD_ARG; }
  const int kc = Cin >= 64 ? 64 : Cin;
  CUtensorMap ta, tb;
  XC_TRY(make_act_map(&ta, x, B, H, W, Cin, kc, bw, bh));
  XC_TRY(make_weight_map(&tb, w, Cin, Cout, kc));
  ConvArgs a{B, H, W, Cin, Cin / kc, bw, bh, bias, relu, (__nv_bfloat16*)y, y_f32, err};
  const int tiles = B * (H / bh) * (W / bw);
  switch (kc) {
    case 16: return launch_fwd_n<16>(Cout, ta, tb, a, tiles, s);
    case 32: return launch_fwd_n<32>(Cout, ta, tb, a, tiles, s);
    default: return launch_fwd_n<64>(Cout, ta, tb, a, tiles, s);
  }
}

int nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, float* partial, int partial_blocks, int B, int H,
                     int W, int Cin, int Cout, float scale, int accumulate, int* err, cudaStream_t s) {
  int bw = 0, bh = 0;
  if (!tile_shape(H, W, &bw, &bh) || B < 1) {
    xc_set_error("conv3x3 wgrad: image %dx%d does not tile into 128-pixel tiles", H, W);
    return XC_BAD_ARG;
  }
  if ((Cout != 16 && Cout != 32 && Cout != 64 && Cout != 128) ||
      (Cin != 16 && Cin != 32 && Cin != 64 && Cin != 128)) {
    xc_set_error("conv3x3 wgrad: channels must be 16, 32, 64 or 128 (Cin %d, Cout %d)", Cin, Cout);
    return XC_BAD_ARG;
  }
  const int tiles = B * (H / bh) * (W / bw);
  const int nblk = tiles < partial_blocks ? tiles : partial_blocks;
  WgradArgs a{(const __nv_bfloat16*)x, (const __nv_bfloat16*)dy, partial, B, H, W, Cin, Cout, bw, bh, tiles, err};
  switch (Cin) {
    case 16: XC_TRY(launch_wgrad<16>(a, nblk, s)); break;
    case 32: XC_TRY(launch_wgrad<32>(a, nblk, s)); break;
    case 64: XC_TRY(launch_wgrad<64>(a, nblk, s)); break;
    default: XC_TRY(launch_wgrad<128>(a, nblk, s)); break;
  }
  const int n = 9 * Cout * Cin;
  wgrad_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(partial, nblk, n, dw, scale, accumulate); xc_count_launch();
  XC_LAUNCH_CHECK();
  return XC_OK;
}

// ---------------------------------------------------------------------------
// C ABI: one convolution / weight gradient on caller device pointers
// ---------------------------------------------------------------------------
namespace {

// a device int for the kernels' bounded-wait error flag, on the stream
struct ErrFlag {
  int* d = nullptr;
  int init(cudaStream_t s) {
    XC_CUDA_TRY(cudaMallocAsync((void**)&d, sizeof(int), s));
    XC_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(int), s));
    return XC_OK;
  }
  // wait for the stream and turn a raised flag into XC_TIMEOUT
  int check(cudaStream_t s, const char* what) {
    int h = 0;
    XC_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    XC_CUDA_TRY(cudaStreamSynchronize(s));
    if (h != 0) {
      xc_set_error("%s: a bounded wait inside the kernel ran out (code %d)", what, h);
      return XC_TIMEOUT;
    }
    return XC_OK;
  }
  ~ErrFlag() {
    if (d) cudaFree(d);
  }
};

}  // namespace

extern "C" int xc_nn_conv3x3(const void* x, const void* w, const float* bias, void* y, float* y_f32, int B, int H,
                             int W, int Cin, int Cout, int relu, void* stream) {
  if (!x || !w) { xc_set_error("xc_nn_conv3x3: null pointer"); return XC_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  ErrFlag e;
  XC_TRY(e.init(s));
  XC_TRY(nn_conv3x3_fwd(x, w, bias, y, y_f32, B, H, W, Cin, Cout, relu, e.d, s));
  return e.check(s, "xc_nn_conv3x3");
}

extern "C" int xc_nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, int B, int H, int W, int Cin,
                                   int Cout, void* stream) {
  if (!x || !dy || !dw) { xc_set_error("xc_nn_conv3x3_wgrad: null pointer"); return XC_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  ErrFlag e;
  XC_TRY(e.init(s));
  const int blocks = 2 * kNumSMs / 9 + 1;
  float* partial = nullptr;
  XC_CUDA_TRY(cudaMallocAsync((void**)&partial, sizeof(float) * (size_t)blocks * 9 * Cin * Cout, s));
  int st = nn_conv3x3_wgrad(x, dy, dw, partial, blocks, B, H, W, Cin, Cout, 1.0f, 0, e.d, s);
  cudaFreeAsync(partial, s);
  if (st != XC_OK) return st;
  return e.check(s, "xc_nn_conv3x3_wgrad");
}
