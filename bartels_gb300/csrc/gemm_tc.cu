// BF16 x BF16 -> FP32 GEMM on the 5th-generation tensor cores (tcgen05), for
// the per-vertex linear layers of the learned preconditioner:
//
//   Y[M x N] = act(X[M x K] W^T + bias) (+ R),   W stored N x K (K contiguous)
//
// One CTA (4 warps) per 128-row tile. Thread 0 loads the X tile and all of W
// with TMA into 128-byte-swizzled shared memory, waits on an mbarrier, issues
// K/16 tcgen05.mma (M=128, N, K=16) into a TMEM accumulator of N columns and
// commits to a second mbarrier. Each warp then reads its 32 TMEM lanes (= 32
// rows) with tcgen05.ld and applies the epilogue: bias, ReLU, residual, FP32
// and / or BF16 stores. Every wait is bounded: on time-out the kernel records
// an error code, still waits (bounded) for its own copies and MMAs, frees its
// TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "internal.cuh"
#include "lpcg_internal.cuh"
#include "tcgen05.cuh"

namespace bartels {

constexpr int kGemmThreads = 128;
constexpr int kWaitLimit = 1 << 22;

template <int N, int K>
struct GemmSmem {
  static constexpr int kAtoms = K / 64;                 // 64-element (128-byte) K slices
  static constexpr int kABytes = 128 * 128;             // one 128-row x 128-byte slice
  static constexpr int kBBytes = N * 128;               // one N-row x 128-byte slice
  static constexpr int kBytes = kAtoms * (kABytes + kBBytes);
  static constexpr int kDyn = kBytes + 1024 + 64;       // alignment slack + barriers
};

template <int N, int K>
__global__ void __launch_bounds__(kGemmThreads)
k_gemm_tc(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w, int M,
          const float *__restrict__ bias, const float *resid, int ldr, int relu, float *__restrict__ ypre, int ldp,
          float *y, int ldy, __nv_bfloat16 *__restrict__ y2, int ldy2, int *__restrict__ err, int probe_polls) {
  using S = GemmSmem<N, K>;
  static_assert(N == 64 || N == 128, "N must be 64 or 128");
  static_assert(K % 64 == 0 && K <= 256, "K must be a multiple of 64");
  extern __shared__ unsigned char dyn[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(dyn) + 1023) & ~uintptr_t(1023));
  unsigned char *sa = base;                                  // kAtoms x kABytes
  unsigned char *sb = base + S::kAtoms * S::kABytes;         // kAtoms x kBBytes
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + S::kBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
  __shared__ int s_fail;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * 128;

  if (threadIdx.x == 0) {
    s_fail = 0;
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::fence_barrier_init();
    tc::prefetch_tmap(&tmap_x);
    tc::prefetch_tmap(&tmap_w);
  }
  if (warp == 0) tc::tmem_alloc(tslot, N);
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  if (threadIdx.x == 0 && probe_polls > 0) {
    // failure-path probe: no copy and no MMA is issued, so nothing is in
    // flight; the bounded wait on a barrier nothing arrives on runs out and
    // the CTA takes the error path below (flag, no epilogue, TMEM freed)
    tc::mbar_wait(&bars[0], 0, probe_polls);
    s_fail = 1;
  } else if (threadIdx.x == 0) {
    tc::mbar_expect_tx(&bars[0], S::kAtoms * (S::kABytes + S::kBBytes));
#pragma unroll
    for (int a = 0; a < S::kAtoms; ++a) {
      tc::tma_load_2d(sa + a * S::kABytes, &tmap_x, 64 * a, row0, &bars[0]);
      tc::tma_load_2d(sb + a * S::kBBytes, &tmap_w, 64 * a, 0, &bars[0]);
    }
    bool ok = tc::mbar_wait(&bars[0], 0, kWaitLimit);
    if (!ok) {
      s_fail = 1;
      tc::mbar_wait(&bars[0], 0, kWaitLimit);  // let the copies land before the CTA's memory is reused
    } else {
      tc::fence_after_sync();
      constexpr uint32_t idesc = tc::idesc_bf16_f32(128, N);
#pragma unroll
      for (int k = 0; k < K / 16; ++k) {
        const int a = k / 4, kk = k % 4;  // 4 x 16 BF16 = 128 bytes per slice
        const uint64_t ad = tc::desc_k_sw128(tc::smem_u32(sa + a * S::kABytes) + 32 * kk);
        const uint64_t bd = tc::desc_k_sw128(tc::smem_u32(sb + a * S::kBBytes) + 32 * kk);
        tc::mma_bf16(tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
      }
      tc::mma_commit(&bars[1]);
    }
  }
  __syncthreads();
  const bool loaded = s_fail == 0;
  bool done = loaded && tc::mbar_wait(&bars[1], 0, kWaitLimit);
  if (loaded && !done) {
    if (lane == 0) atomicExch(&s_fail, 2);
    tc::mbar_wait(&bars[1], 0, kWaitLimit);
  }
  tc::fence_after_sync();
  __syncthreads();
  if (s_fail == 0) {
    const int row = row0 + 32 * warp + lane;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(taddr + c, v);
      if (row < M) {
        float rv[16];
        if (resid) {  // 16-byte loads of the residual row segment
          const float4 *r4 = reinterpret_cast<const float4 *>(resid + (int64_t)row * ldr + c);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float4 q = r4[i];
            rv[4 * i] = q.x;
            rv[4 * i + 1] = q.y;
            rv[4 * i + 2] = q.z;
            rv[4 * i + 3] = q.w;
          }
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float t = v[i] + (bias ? bias[c + i] : 0.f);
          if (ypre) ypre[(int64_t)row * ldp + c + i] = t;
          if (relu) t = fmaxf(t, 0.f);
          if (resid) t += rv[i];
          v[i] = t;
        }
        if (y) {
          float4 *o = reinterpret_cast<float4 *>(y + (int64_t)row * ldy + c);
#pragma unroll
          for (int i = 0; i < 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
        if (y2) {
          __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(y2 + (int64_t)row * ldy2 + c);
#pragma unroll
          for (int i = 0; i < 8; ++i) o[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicMax(err, s_fail);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, N);
}

// ------------------------------------------------------------------ host ---
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_mutex;

static int tensor_map_encoder() {
  std::lock_guard<std::mutex> lk(g_encode_mutex);
  if (g_encode) return BARTELS_OK;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
    return fail(BARTELS_E_DEVICE, "cuTensorMapEncodeTiled is not available from the driver");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return BARTELS_OK;
}

// BF16 row-major matrix [rows x cols] with row stride ld (elements), read in
// boxes of 64 columns x box_rows rows, 128-byte swizzle, zero fill past the end.
static int make_map(CUtensorMap *m, const __nv_bfloat16 *p, int rows, int cols, int ld, int box_rows) {
  if (reinterpret_cast<uintptr_t>(p) % 16 != 0 || (ld * 2) % 16 != 0)
    return fail(BARTELS_E_INVALID_ARG, "GEMM operand must be 16-byte aligned with a 16-byte multiple row stride");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(p), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(BARTELS_E_DEVICE, "cuTensorMapEncodeTiled failed");
  return BARTELS_OK;
}

template <int N, int K>
static int launch_gemm_t(bartels_ctx ctx, const GemmArgs &g) {
  using S = GemmSmem<N, K>;
  static bool attr = false;
  if (!attr) {
    BT_CUDA(cudaFuncSetAttribute(k_gemm_tc<N, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kDyn));
    attr = true;
  }
  CUtensorMap mx, mw;
  BT_CHECK(make_map(&mx, g.x, g.M, K, g.ldx, 128));
  BT_CHECK(make_map(&mw, g.w, N, K, K, N));
  const int grid = (g.M + 127) / 128;
  BT_LAUNCH(ctx, (k_gemm_tc<N, K>), grid, kGemmThreads, S::kDyn, mx, mw, g.M, g.bias, g.resid, g.ldr, g.relu, g.ypre,
            g.ldp, g.y, g.ldy, g.y2, g.ldy2, g.err, g.probe_polls);
  return BARTELS_OK;
}

int gemm_bf16(bartels_ctx ctx, const GemmArgs &g) {
  if (g.M <= 0) return BARTELS_OK;
  BT_CHECK(tensor_map_encoder());
  if ((g.y && (g.ldy % 4 != 0 || reinterpret_cast<uintptr_t>(g.y) % 16 != 0)) ||
      (g.y2 && (g.ldy2 % 2 != 0 || reinterpret_cast<uintptr_t>(g.y2) % 4 != 0)) ||
      (g.resid && (g.ldr % 4 != 0 || reinterpret_cast<uintptr_t>(g.resid) % 16 != 0)))
    return fail(BARTELS_E_INVALID_ARG, "GEMM output / residual must be 16-byte aligned with a multiple-of-4 row stride");
  if (g.N == 128 && g.K == 64) return launch_gemm_t<128, 64>(ctx, g);
  if (g.N == 64 && g.K == 128) return launch_gemm_t<64, 128>(ctx, g);
  if (g.N == 64 && g.K == 64) return launch_gemm_t<64, 64>(ctx, g);
  if (g.N == 128 && g.K == 128) return launch_gemm_t<128, 128>(ctx, g);
  return fail(BARTELS_E_UNSUPPORTED, "GEMM shape: N and K must be 64 or 128");
}

}  // namespace bartels
