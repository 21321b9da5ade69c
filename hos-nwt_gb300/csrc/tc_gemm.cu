// Tensor-core GEMM for the surrogate's dense contractions (sm_103a).
//
//   D[m, n] = act( sum_k A[m, k] B[n, k] + bias[n] )      (FP32 accumulate)
//
// A (M x K) and B (N x K) are BF16, row-major with K contiguous ("K-major"
// for both operands); D is FP32 or BF16, row-major with leading dimension
// ldd.  One CTA computes one 128 x BN tile:
//   - warp 0, one thread: TMA loads of 128 x 64 A and BN x 64 B tiles
//     (128-byte swizzle) into a kStages-deep shared-memory ring, each stage
//     signalled on an mbarrier with its byte count;
//   - warp 1, one thread: tcgen05.mma (kind::f16, BF16 inputs, FP32
//     accumulator in tensor memory), four K=16 steps per stage; a
//     tcgen05.commit per stage frees the stage for the next TMA load, and a
//     last commit signals the epilogue;
//   - all four warps: tcgen05.ld of their 32 accumulator lanes, bias and
//     activation, stores.
// Every wait on an mbarrier is bounded: on timeout the CTA records an error
// code in a device flag, skips its remaining work, frees its tensor memory
// and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hosnwt_internal.h"

namespace hos {
namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;         // one 128-byte swizzle atom of BF16
constexpr int kStages = 4;
constexpr int kThreads = 128;
constexpr unsigned kSpinLimit = 1u << 22;  // try_wait polls (each may suspend briefly): seconds at most

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Wait for the phase of the given parity to complete; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
// rows of 128 bytes, 8-row groups 1024 bytes apart (SBO), descriptor
// version 1, layout type 2 (128-byte swizzle).  The tile starts on a
// 1024-byte boundary; the K=16 slices inside the atom are addressed by
// advancing the start address by 32 bytes.
__device__ __forceinline__ uint64_t sw128_desc(unsigned saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                  // leading byte offset (unused with swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                  // descriptor version
  d |= (uint64_t)2 << 61;                  // 128-byte swizzle
  return d;
}

// Instruction descriptor: FP32 accumulator, BF16 A and B, both K-major,
// N = bn, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int bn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float x) {
  // tanh form of the Gaussian error linear unit
  const float c = 0.7978845608028654f;  // sqrt(2 / pi)
  return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}

struct GemmArgs {
  int M, N, K;
  void* D;
  long long ldd;
  int d_bf16;          // 1: D is BF16, else FP32
  const float* bias;   // N entries or null
  int act;             // 0 none, 1 GELU
  const float* Dadd;   // optional FP32 M x N (ldd) added before the activation
  unsigned* err;       // error flag (1: a wait timed out; 2: the wait for the
                       // MMAs to finish timed out too, so the CTA exited
                       // without freeing its tensor memory: treat the
                       // context as unusable)
};

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage ring: kStages x (A 128x64, B BNx64) BF16
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2;
  unsigned char* sA = base;
  unsigned char* sB = base + kStages * kABytes;
  __shared__ uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ int keep_tmem;  // 1: MMAs may still write the accumulator
  __shared__ int n_issued, n_consumed;  // stages loaded by TMA / read by the MMAs
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int nk = (g.K + kBK - 1) / kBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    keep_tmem = 0;
    n_issued = n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    // BN fp32 columns of tensor memory (a power of two, at least 32)
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(BN < 32 ? 32 : BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    // producer
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages, r = kb / kStages;
      if (kb >= kStages && !mbar_wait(&empty_bar[s], (unsigned)((r - 1) & 1))) {
        abort_flag = 1;
        break;
      }
      mbar_expect_tx(&full_bar[s], kABytes + kBBytes);
      tma_load_2d(sA + s * kABytes, &mapA, kb * kBK, m0, &full_bar[s]);
      tma_load_2d(sB + s * kBBytes, &mapB, kb * kBK, n0, &full_bar[s]);
      n_issued = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_bf16(BN);
    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages, r = kb / kStages;
      if (!mbar_wait(&full_bar[s], (unsigned)(r & 1))) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t da = sw128_desc(smem_u32(sA + s * kABytes));
      const uint64_t db = sw128_desc(smem_u32(sB + s * kBBytes));
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk)
        mma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (kb > 0 || kk > 0) ? 1 : 0);
      mma_commit(&empty_bar[s]);
      n_consumed = kb + 1;
    }
    if (!ok) abort_flag = 1;
    mma_commit(&done_bar);  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  // epilogue: every warp waits for the accumulator
  bool ready = mbar_wait(&done_bar, 0u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  ready = __syncthreads_and(ready) != 0;
  if (!ready || abort_flag) {
    if (threadIdx.x == 0) {
      atomicExch(g.err, 1u);
      // let the TMA loads still in flight land before the CTA exits, and
      // the MMAs finish before their tensor memory is freed
      for (int kb = n_consumed; kb < n_issued; ++kb)
        (void)mbar_wait(&full_bar[kb % kStages], (unsigned)((kb / kStages) & 1));
      if (!ready && !mbar_wait(&done_bar, 0u)) {
        // the MMAs did not report completion: freeing their tensor memory
        // now could let another CTA's accumulator be overwritten
        keep_tmem = 1;
        atomicExch(g.err, 2u);
      }
    }
  } else {
    // Every MMA has completed, so the stage ring is free: each warp passes
    // its 32 accumulator rows through a 32 x 16 shared-memory tile (rows
    // padded to 17 words: conflict-free both ways) so that a half-warp then
    // reads, combines and stores 16 consecutive columns of one row.
    float* tile = reinterpret_cast<float*>(base) + warp * (32 * 17);
    const int half = lane >> 4, cl = lane & 15;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) tile[lane * 17 + i] = v[i];
      __syncwarp();
      const int col = n0 + c0 + cl;
      const float bcol = (g.bias && col < g.N) ? g.bias[col] : 0.0f;
#pragma unroll 4
      for (int r = half; r < 32; r += 2) {
        const int row = m0 + warp * 32 + r;
        if (row < g.M && col < g.N) {
          float x = tile[r * 17 + cl] + bcol;
          if (g.Dadd) x += g.Dadd[(long long)row * g.ldd + col];
          if (g.act == 1) x = gelu(x);
          if (g.d_bf16)
            ((__nv_bfloat16*)g.D)[(long long)row * g.ldd + col] = __float2bfloat16(x);
          else
            ((float*)g.D)[(long long)row * g.ldd + col] = x;
        }
      }
      __syncwarp();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0 && !keep_tmem)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN < 32 ? 32 : BN)
                 : "memory");
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)p;
  }
  return fn;
}

// rows x cols BF16 matrix, row stride ld elements, box box_rows x 64
bool make_map(CUtensorMap* m, const void* ptr, int rows, int cols, long long ld, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, const GemmArgs& g, cudaStream_t st) {
  const size_t smem = 1024 + (size_t)kStages * (kBM + BN) * kBK * 2;
  static PerDeviceOnce attr;
  attr.run([&] { cudaFuncSetAttribute(k_tc_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
  const dim3 grid((g.M + kBM - 1) / kBM, (g.N + BN - 1) / BN);
  k_tc_gemm<BN><<<grid, kThreads, smem, st>>>(ma, mb, g);
  return cudaGetLastError();
}

}  // namespace

// D = act(A B^T + bias [+ Dadd]); see the file comment.  A: M x K (lda),
// B: N x K (ldb), both BF16; K, lda, ldb multiples of 8 and both base
// addresses 16-byte aligned (the TMA rules).  Returns a cudaError_t value
// (cudaErrorInvalidValue for shapes the kernel does not take).
int tc_gemm_bf16(const void* A, long long lda, const void* B, long long ldb, void* D, long long ldd, int d_bf16,
                 int M, int N, int K, const float* bias, int act, const float* Dadd, unsigned* err,
                 cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0 || (K % 8) || (lda % 8) || (ldb % 8) || ((uintptr_t)A & 15) ||
      ((uintptr_t)B & 15) || !err)
    return (int)cudaErrorInvalidValue;
  const int bn = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
  CUtensorMap ma, mb;
  if (!make_map(&ma, A, M, K, lda, kBM) || !make_map(&mb, B, N, K, ldb, bn)) return (int)cudaErrorInvalidValue;
  GemmArgs g{M, N, K, D, ldd, d_bf16, bias, act, Dadd, err};
  cudaError_t e;
  if (bn == 32) e = launch_gemm<32>(ma, mb, g, st);
  else if (bn == 64) e = launch_gemm<64>(ma, mb, g, st);
  else e = launch_gemm<128>(ma, mb, g, st);
  return (int)e;
}

}  // namespace hos

extern "C" int hosnwt_tc_gemm_bf16(const void* A, long long lda, const void* B, long long ldb, void* D,
                                   long long ldd, int d_bf16, int M, int N, int K, const float* bias, int act,
                                   const float* Dadd, unsigned* err, void* stream) {
  const int e = hos::tc_gemm_bf16(A, lda, B, ldb, D, ldd, d_bf16, M, N, K, bias, act, Dadd, err,
                                  (cudaStream_t)stream);
  return e == 0 ? HOSNWT_OK : (e == (int)cudaErrorInvalidValue ? HOSNWT_ERR_ARG : HOSNWT_ERR_CUDA);
}
