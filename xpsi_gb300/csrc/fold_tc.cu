// fold_tc.cu -- K5 (mixed form): the instrument-response fold
//   out[b][K][N] = M[K][q] @ in[b][q][N]
// on the 5th-generation tensor cores (tcgen05), replacing the numpy dot of
// xpsi/Instrument.py:192-197 for the mixed-precision batched path.
//
// All signals of a batch share M, so the fold is one GEMM
//   C[m][n] = sum_k A[m][k] B[n][k],  A = M (m: channel), B[n][k] = in[b][k][p]
// with n = b N + p.  Precision: 3xTF32 split products -- every FP64 operand
// x is held as hi + lo with hi = x rounded to TF32 and lo = the remainder
// rounded to TF32, and C = A_hi B_hi + A_hi B_lo + A_lo B_hi is accumulated
// in FP32 in tensor memory (relative error ~1e-7, FP32 class; the dropped
// A_lo B_lo term is ~2^-22 relative).
//
// Kernel: one CTA (4 warps) per 128 x 128 tile of C.  Per 32-wide K block the
// elected thread issues four TMA tile loads (A_hi, A_lo, B_hi, B_lo; 128 rows
// x 128 bytes each, 128-byte swizzle) completing on an mbarrier, then the
// three tcgen05.mma per 8-wide K step (M = N = 128, K = 8) into an FP32
// accumulator of 128 TMEM columns, committed to a second mbarrier; each
// warp reads its 32 TMEM lanes (rows) with tcgen05.ld after every step and
// sums the steps in registers, then stores FP64.  Every mbarrier wait is
// bounded; on a timeout the tile is written as NaN, the status word gets 1
// (2 if the second, bounded wait for the copies and MMAs in flight runs out
// as well) and the kernel frees its TMEM.
#include <cuda.h>

#include "common.cuh"
#include "kernels.h"

namespace xg {
namespace {

constexpr int kTM = 128, kTN = 128, kTK = 32;  // tile rows, tile columns, K block
constexpr int kFoldThreads = 128;
constexpr uint32_t kPartBytes = kTM * kTK * 4;  // one operand part: 128 rows x 128 B
constexpr uint32_t kStageBytes = 4 * kPartBytes;
constexpr long kSpinLimit = 1L << 22;
constexpr long kSelfTestSpinLimit = 1L << 10;
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase with the given parity; false on timeout
__device__ bool mbar_wait(uint64_t *bar, uint32_t parity, long limit = kSpinLimit) {
  for (long i = 0; i < limit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, kind::tf32
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on `bar` when every tcgen05.mma issued so far by this thread is done
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// float rounded to TF32 (10 explicit mantissa bits), kept in an FP32 word
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  return __uint_as_float(u);
}

// hi/lo split of an FP64 operand matrix into part 0 (hi) and part 1 (lo)
// rows of a [2][rows_pad][k_pad] FP32 array, zero-padded
__global__ void split_a_kernel(const double *M, int ldM, int K, int q, int rows_pad, int k_pad,
                               float *out) {
  const long n = (long)rows_pad * k_pad;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const int m = (int)(t / k_pad), k = (int)(t - (long)m * k_pad);
    const double v = (m < K && k < q) ? M[(size_t)m * ldM + k] : 0.0;
    const float hi = tf32_round((float)v);
    out[t] = hi;
    out[n + t] = tf32_round((float)(v - (double)hi));
  }
}
// B[n][k] = in[b][k][p], n = b N + p
__global__ void split_b_kernel(const double *in, int batch, int q, int N, int rows_pad,
                               int k_pad, float *out) {
  const long n_all = (long)rows_pad * k_pad;
  const long cols = (long)batch * N;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n_all;
       t += (long)gridDim.x * blockDim.x) {
    const long n = t / k_pad;
    const int k = (int)(t - n * k_pad);
    double v = 0.0;
    if (n < cols && k < q) {
      const long b = n / N, p = n - b * N;
      v = in[((size_t)b * q + k) * N + p];
    }
    const float hi = tf32_round((float)v);
    out[t] = hi;
    out[n_all + t] = tf32_round((float)(v - (double)hi));
  }
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows
// of 128 bytes, 8-row groups 1024 bytes apart (stride byte offset); the
// leading byte offset is unused for this layout
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3fff);  // start address
  d |= (uint64_t)1 << 16;                  // leading byte offset (16 B; unused)
  d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
  d |= (uint64_t)1 << 46;                  // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                  // layout: 128-byte swizzle
  return d;
}
// instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N = 128
constexpr uint32_t kIdescTf32 =
    (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);

// selftest: the producer issues no copies and its waits give up after a
// short limit (the timeout path, with nothing in flight)
__global__ void __launch_bounds__(kFoldThreads) fold_tc_kernel(
    const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
    int K, int q_pad, int rows_a, int rows_b, int N, long cols, double *out, int32_t *status,
    int selftest) {
  extern __shared__ __align__(1024) unsigned char fsm[];
  __shared__ __align__(8) uint64_t bar_full, bar_mma;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(fsm) + 1023) & ~uintptr_t(1023));
  unsigned char *sA_hi = base, *sA_lo = base + kPartBytes;
  unsigned char *sB_hi = base + 2 * kPartBytes, *sB_lo = base + 3 * kPartBytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kTM;
  const long n0 = (long)blockIdx.x * kTN;
  if (threadIdx.x == 0) {
    mbar_init(&bar_full, 1);
    mbar_init(&bar_mma, 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  // Per K step (8 along K) the elected thread issues the three split
  // products into the TMEM accumulator (fresh each step) and waits for them;
  // every warp then reads its lanes' partial and adds it to FP32 registers
  // (round to nearest).  The tensor core's accumulation then spans only 3
  // products per step instead of all 3 x q / 8, which keeps its rounding
  // bias at the FP32 level of one step's partial.
  const int m = m0 + warp * 32 + lane;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  float acc[kTN];
#pragma unroll
  for (int c = 0; c < kTN; c++) acc[c] = 0.0f;
  const int nkb = q_pad / kTK;
  int step = 0;
  // s_fail is written by thread 0 only and read by every thread only after
  // the barrier that follows the write, so all threads leave together
  for (int kb = 0; kb < nkb; kb++) {
    if (threadIdx.x == 0) {
      const long limit = selftest ? kSelfTestSpinLimit : kSpinLimit;
      if (!selftest) {
        mbar_expect_tx(&bar_full, kStageBytes);
        const int x = kb * kTK;
        tma_load_2d(sA_hi, &mapA, x, m0, &bar_full);
        tma_load_2d(sA_lo, &mapA, x, rows_a + m0, &bar_full);
        tma_load_2d(sB_hi, &mapB, x, (int)n0, &bar_full);
        tma_load_2d(sB_lo, &mapB, x, rows_b + (int)n0, &bar_full);
      }
      if (!mbar_wait(&bar_full, (uint32_t)(kb & 1), limit)) {
        s_fail = 1;
        // let the copy land (bounded); if it does not, say so
        if (!mbar_wait(&bar_full, (uint32_t)(kb & 1), limit)) s_fail = 2;
      }
    }
    __syncthreads();
    if (s_fail) break;
    for (int ks = 0; ks < kTK / 8; ks++, step++) {
      if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t off = (uint32_t)ks * 32;  // 8 TF32 = 32 bytes along K
        const uint64_t ah = smem_desc_sw128(smem_u32(sA_hi) + off);
        const uint64_t al = smem_desc_sw128(smem_u32(sA_lo) + off);
        const uint64_t bh = smem_desc_sw128(smem_u32(sB_hi) + off);
        const uint64_t bl = smem_desc_sw128(smem_u32(sB_lo) + off);
        mma_tf32(tmem, ah, bh, kIdescTf32, 0u);
        mma_tf32(tmem, ah, bl, kIdescTf32, 1u);
        mma_tf32(tmem, al, bh, kIdescTf32, 1u);
        mma_commit(&bar_mma);
        if (!mbar_wait(&bar_mma, (uint32_t)(step & 1))) {
          s_fail = 1;
          // let the MMAs finish (bounded); if they do not, say so
          if (!mbar_wait(&bar_mma, (uint32_t)(step & 1))) s_fail = 2;
        }
      }
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (s_fail) break;
#pragma unroll
      for (int c = 0; c < kTN / 32; c++) {
        uint32_t r[32];
        tmem_ld32(lane_base + (uint32_t)(c * 32), r);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 32; j++) acc[c * 32 + j] += __uint_as_float(r[j]);
      }
      // the next step's MMA overwrites the accumulator: every read first
      tc_fence_before();
      __syncthreads();
    }
  }
  tc_fence_after();
  const bool fail = s_fail != 0;
  if (fail && threadIdx.x == 0 && status != nullptr) atomicMax(status, s_fail);
  if (m < K) {
#pragma unroll
    for (int c = 0; c < kTN; c++) {
      const long n = n0 + c;
      if (n < cols) {
        const long b = n / N, p = n - b * N;
        out[((size_t)b * K + m) * N + p] = fail ? nan("") : (double)acc[c];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

// [2 * rows][k_pad] FP32 array, boxes of 32 x 128 elements, 128-byte swizzle
int make_map(CUtensorMap *map, float *base, int rows2, int k_pad) {
  EncodeTiled enc = encode_fn();
  if (!enc) return -1;
  cuuint64_t dims[2] = {(cuuint64_t)k_pad, (cuuint64_t)rows2};
  cuuint64_t strides[1] = {(cuuint64_t)k_pad * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)kTK, (cuuint32_t)kTM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

}  // namespace

size_t fold_tc_scratch_bytes(const FoldArgs &a) {
  const size_t rows_a = (size_t)((a.K + kTM - 1) / kTM) * kTM;
  const size_t cols = (size_t)a.batch * a.N;
  const size_t rows_b = (cols + kTN - 1) / kTN * kTN;
  const size_t k_pad = (size_t)((a.q + kTK - 1) / kTK) * kTK;
  return 2 * (rows_a + rows_b) * k_pad * sizeof(float);
}

int launch_fold_tc(const FoldArgs &a, void *scratch, cudaStream_t st) {
  if (a.batch <= 0 || a.K <= 0 || a.N <= 0) return 0;
  const int rows_a = (a.K + kTM - 1) / kTM * kTM;
  const long cols = (long)a.batch * a.N;
  const long rows_b = (cols + kTN - 1) / kTN * kTN;
  const int k_pad = (a.q + kTK - 1) / kTK * kTK;
  if (rows_b > (1L << 30)) return -3;
  float *A2 = static_cast<float *>(scratch);
  float *B2 = A2 + (size_t)2 * rows_a * k_pad;
  split_a_kernel<<<(unsigned)((2L * rows_a * k_pad / 2 + 255) / 256), 256, 0, st>>>(
      a.M, a.ldM, a.K, a.q, rows_a, k_pad, A2);
  const long nb = rows_b * k_pad;
  const unsigned gb = (unsigned)std::min<long>((nb + 255) / 256, 152L * 64);
  split_b_kernel<<<gb, 256, 0, st>>>(a.in, a.batch, a.q, a.N, (int)rows_b, k_pad, B2);
  CUtensorMap mapA, mapB;
  if (make_map(&mapA, A2, 2 * rows_a, k_pad) || make_map(&mapB, B2, (int)(2 * rows_b), k_pad))
    return -4;
  const size_t smem = kStageBytes + 1024;
  // the attribute is per device: set it on every launch (cheap)
  if (cudaFuncSetAttribute(fold_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -5;
  dim3 grid((unsigned)(rows_b / kTN), (unsigned)(rows_a / kTM));
  fold_tc_kernel<<<grid, kFoldThreads, smem, st>>>(mapA, mapB, a.K, k_pad, rows_a,
                                                   (int)rows_b, a.N, cols, a.out, a.status, 0);
  return 0;
}

int launch_fold_tc_timeout_selftest(const FoldArgs &a, void *scratch, cudaStream_t st) {
  if (a.batch <= 0 || a.K <= 0 || a.N <= 0 || a.status == nullptr) return -3;
  const int rows_a = (a.K + kTM - 1) / kTM * kTM;
  const long cols = (long)a.batch * a.N;
  const long rows_b = (cols + kTN - 1) / kTN * kTN;
  const int k_pad = (a.q + kTK - 1) / kTK * kTK;
  float *A2 = static_cast<float *>(scratch);
  float *B2 = A2 + (size_t)2 * rows_a * k_pad;
  CUtensorMap mapA, mapB;
  if (make_map(&mapA, A2, 2 * rows_a, k_pad) || make_map(&mapB, B2, (int)(2 * rows_b), k_pad))
    return -4;
  const size_t smem = kStageBytes + 1024;
  if (cudaFuncSetAttribute(fold_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -5;
  // one tile: its waits run out, the kernel reports and returns
  fold_tc_kernel<<<dim3(1, 1), kFoldThreads, smem, st>>>(mapA, mapB, a.K, k_pad, rows_a,
                                                         (int)rows_b, a.N, cols, a.out, a.status,
                                                         1);
  return 0;
}

}  // namespace xg
