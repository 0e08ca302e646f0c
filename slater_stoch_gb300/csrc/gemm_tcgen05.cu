// gemm_tcgen05.cu -- split-BF16 "TN" GEMM on Blackwell 5th-generation tensor cores (sm_103a).
//
//   C_partial[ks] = sum over the ks-th K slice of  Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T
//
// A*, B*: [P][K] bf16, K contiguous (both operands K-major), C fp32 [P][P].
// One CTA computes a 128x128 tile of one K slice:
//   warp 0 lane 0  : TMA producer (cp.async.bulk.tensor, 128B swizzle) into a STAGES-deep ring;
//   warp 1 lane 0  : MMA issuer (tcgen05.mma.cta_group::1.kind::f16, M=N=128, K=16 per instr,
//                    3 products per K step into one FP32 TMEM accumulator);
//   warps 0..3     : epilogue, tcgen05.ld of the 128x128 accumulator (one TMEM lane per row).
// Every mbarrier wait is bounded; on timeout the CTA records an error code, stops issuing
// work, drains, frees its TMEM and returns.  The hi/lo split keeps ~16 significant bits of
// each operand; the omitted lo*lo term is 2^-16 relative.  FP32 accumulation runs over at
// most 2^17 K steps per launch before the caller sums slices in FP64.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "shared.cuh"
#include "ss_common.cuh"

namespace ss {

namespace {

constexpr int BM = 128, BN = 128, BK = 64;     // BK bf16 = 128 bytes (one swizzle row)
constexpr int STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 2;        // 16 KiB
constexpr int STAGE_BYTES = 4 * TILE_BYTES;    // Ahi, Alo, Bhi, Blo
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr uint32_t TMEM_COLS = 128;
constexpr uint32_t SPIN_LIMIT = 1u << 26;      // bounded waits (~seconds)

enum : int { ERR_FULL_WAIT = 1, ERR_EMPTY_WAIT = 2, ERR_ACC_WAIT = 3 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// bounded parity wait; returns false if the limit was reached
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < SPIN_LIMIT; it++) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, void* dst, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// tcgen05 shared-memory descriptor, K-major operand, 128B swizzle:
// start>>4 [0,14), LBO>>4 [16,30), SBO>>4 [32,46), 0b001 [46,49), swizzle mode 2 (128B) [61,64)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;    // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;  // SBO: 8 rows x 128 B
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// instruction descriptor, kind::f16: D=F32 [4,6), A=BF16 [7,10), B=BF16 [10,13), K-major A/B,
// N>>3 [17,23), M>>4 [24,29)
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__global__ void __launch_bounds__(128, 1)
    split_bf16_gemm_kernel(const __grid_constant__ CUtensorMap tAhi, const __grid_constant__ CUtensorMap tAlo,
                           const __grid_constant__ CUtensorMap tBhi, const __grid_constant__ CUtensorMap tBlo,
                           int P, int ktiles, int tiles_per_split, float* __restrict__ Cp, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full_bar = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty_bar = full_bar + STAGES;
  uint64_t* acc_bar = empty_bar + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(acc_bar + 1);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = blockIdx.x, tn = blockIdx.y, ks = blockIdx.z;
  const int kt0 = ks * tiles_per_split;
  const int nkt = max(0, min(ktiles, kt0 + tiles_per_split) - kt0);

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(acc_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  int issued = 0;  // stages the producer filled (read by the producer lane only)
  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int t = 0; t < nkt; t++) {
      const int s = t % STAGES;
      const uint32_t ph = (uint32_t)((t / STAGES) & 1);
      if (!mbar_wait(&empty_bar[s], ph ^ 1u)) {
        atomicExch(err, ERR_EMPTY_WAIT);
        s_abort = 1;
        break;
      }
      if (*(volatile int*)&s_abort) break;
      uint8_t* st = smem + s * STAGE_BYTES;
      mbar_expect_tx(&full_bar[s], STAGE_BYTES);
      const int x = (kt0 + t) * BK;
      tma_load_2d(&tAhi, st, &full_bar[s], x, tm * BM);
      tma_load_2d(&tAlo, st + TILE_BYTES, &full_bar[s], x, tm * BM);
      tma_load_2d(&tBhi, st + 2 * TILE_BYTES, &full_bar[s], x, tn * BN);
      tma_load_2d(&tBlo, st + 3 * TILE_BYTES, &full_bar[s], x, tn * BN);
      issued = t + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    for (int t = 0; t < nkt; t++) {
      const int s = t % STAGES;
      const uint32_t ph = (uint32_t)((t / STAGES) & 1);
      if (!mbar_wait(&full_bar[s], ph)) {
        atomicExch(err, ERR_FULL_WAIT);
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++) {
        const uint32_t koff = kk * 32;  // 16 bf16 = 32 bytes inside the 128-byte swizzle row
        const uint64_t ahi = smem_desc_sw128(base + koff);
        const uint64_t alo = smem_desc_sw128(base + TILE_BYTES + koff);
        const uint64_t bhi = smem_desc_sw128(base + 2 * TILE_BYTES + koff);
        const uint64_t blo = smem_desc_sw128(base + 3 * TILE_BYTES + koff);
        mma_bf16(tmem, ahi, bhi, (t > 0 || kk > 0) ? 1u : 0u);
        mma_bf16(tmem, ahi, blo, 1u);
        mma_bf16(tmem, alo, bhi, 1u);
      }
      mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
    }
    mma_commit(acc_bar);  // arrives once every issued MMA has completed
  }
  __syncwarp();

  // epilogue: each warp owns TMEM lanes [32w, 32w+32) = output rows
  const bool have_acc = nkt > 0;
  bool ok = true;
  if (have_acc) ok = mbar_wait(acc_bar, 0);
  if (!ok && lane == 0) atomicExch(err, ERR_ACC_WAIT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = tm * BM + warp * 32 + lane;
  float* crow = Cp + (size_t)ks * P * P + (size_t)row * P;
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 32) {
    uint32_t v[32];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (row < P) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int col = tn * BN + c0 + j;
        if (col < P) crow[col] = (have_acc && ok) ? __uint_as_float(v[j]) : 0.f;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // After an abort, TMA loads the MMA warp never consumed may still be writing into shared
  // memory: the producer waits (bounded) for the last load of every stage before the CTA exits.
  // Stage s last received load t = issued-1-((issued-1-s) mod STAGES); its phase parity is
  // (t / STAGES) & 1 and no later load was issued into it, so the parity wait is unambiguous.
  if (warp == 0 && lane == 0 && *(volatile int*)&s_abort) {
    for (int s = 0; s < STAGES && s < issued; s++) {
      const int t = issued - 1 - ((issued - 1 - s) % STAGES);
      if (!mbar_wait(&full_bar[s], (uint32_t)((t / STAGES) & 1))) atomicExch(err, ERR_FULL_WAIT);
    }
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int make_map(CUtensorMap* m, const void* base, int rows, int64_t K) {
  std::call_once(g_encode_once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  if (!g_encode) {
    ss_set_error_msg("cuTensorMapEncodeTiled is not available from the driver");
    return SS_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {BK, BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    ss_set_error_msg("cuTensorMapEncodeTiled failed (%d) rows=%d K=%lld", (int)r, rows, (long long)K);
    return SS_ERR_CUDA;
  }
  return SS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Allocation-free variant of the contraction.
//
// Callers that cannot allocate device memory (an application that hands all of its device
// memory to its own pool, or code running where cudaMalloc is not allowed) still need the
// FP32 partial products of the K slices somewhere.  They live in this fixed file-scope device
// array, which every GPU that loads the library holds until the process exits.  Host code
// must not pass the symbol itself to a kernel (on the host it is only a stand-in); its device
// address is looked up once per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------------------
constexpr size_t NOALLOC_FLAG_BYTES = 256;                 // bounded-wait error flag
constexpr size_t NOALLOC_PARTIAL_BYTES = (size_t)16 << 20;  // 16 MiB of FP32 K-slice partials
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_FLAG_BYTES + NOALLOC_PARTIAL_BYTES];

__global__ void noalloc_sum_slices(int64_t PP, int ksplit, const float* __restrict__ Cp, float* __restrict__ C) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= PP) return;
  double v = 0.0;
  for (int t = 0; t < ksplit; t++) v += (double)Cp[t * PP + e];
  C[e] = (float)v;
}

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};
}  // namespace

int launch_split_bf16_gemm(cudaStream_t st, const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo,
                           int P, int64_t K, int ksplit, float* c_partial, int* err_flag);

}  // namespace ss

extern "C" int ss_split_bf16_gemm_noalloc(void* stream, int P, int64_t K, const uint16_t* a_hi, const uint16_t* a_lo,
                                          const uint16_t* b_hi, const uint16_t* b_lo, int ksplit, float* c) {
  using namespace ss;
  if (P <= 0 || K <= 0 || K % 64 != 0 || !a_hi || !a_lo || !b_hi || !b_lo || !c || ksplit < 0) {
    ss_set_error_msg("ss_split_bf16_gemm_noalloc: need P > 0, K a positive multiple of 64, device buffers");
    return SS_ERR_ARG;
  }
  const size_t cap = NOALLOC_PARTIAL_BYTES / sizeof(float);  // floats of partial products
  const size_t PP = (size_t)P * P;
  if (PP > cap) {
    ss_set_error_msg("ss_split_bf16_gemm_noalloc: P=%d needs %zu bytes of partials, more than the fixed "
                     "%zu-byte scratch (P <= 2048)", P, PP * sizeof(float), NOALLOC_PARTIAL_BYTES);
    return SS_ERR_ARG;
  }
  const int T = (P + 127) / 128;
  int dev = 0;
  SS_CUDA_TRY(cudaGetDevice(&dev));
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (ksplit == 0) ksplit = (int)std::max<int64_t>(1, std::min<int64_t>(K / 64, (2 * sms) / (T * T)));
  ksplit = (int)std::min<size_t>((size_t)ksplit, cap / PP);
  if (dev < 0 || dev >= 64) {
    ss_set_error_msg("ss_split_bf16_gemm_noalloc: device %d out of range", dev);
    return SS_ERR_ARG;
  }
  void* base;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {  // first call on this device: look up the array's device address
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        ss_set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        return SS_ERR_CUDA;
      }
      g_noalloc_ptr[dev] = p;
    }
    base = g_noalloc_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  int* err = (int*)base;
  float* partial = (float*)((unsigned char*)base + NOALLOC_FLAG_BYTES);
  SS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));  // the flag must start at zero
  int rc = launch_split_bf16_gemm(st, a_hi, a_lo, b_hi, b_lo, P, K, ksplit, partial, err);
  if (rc) return rc;
  noalloc_sum_slices<<<(unsigned)((PP + 255) / 256), 256, 0, st>>>((int64_t)PP, ksplit, partial, c);
  SS_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  SS_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SS_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    ss_set_error_msg("tcgen05 GEMM: a bounded wait gave up (code %d)", herr);
    return SS_ERR_TIMEOUT;
  }
  return SS_OK;
}

namespace ss {

int launch_split_bf16_gemm(cudaStream_t st, const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo,
                           int P, int64_t K, int ksplit, float* c_partial, int* err_flag) {
  if (P <= 0 || K <= 0 || K % BK != 0 || ksplit <= 0) {
    ss_set_error_msg("split_bf16_gemm: bad shape P=%d K=%lld ksplit=%d", P, (long long)K, ksplit);
    return SS_ERR_ARG;
  }
  if (((uintptr_t)a_hi | (uintptr_t)a_lo | (uintptr_t)b_hi | (uintptr_t)b_lo) & 15u) {
    ss_set_error_msg("split_bf16_gemm: operands must be 16-byte aligned");
    return SS_ERR_ARG;
  }
  CUtensorMap mAhi, mAlo, mBhi, mBlo;
  int rc = make_map(&mAhi, a_hi, P, K);
  if (!rc) rc = make_map(&mAlo, a_lo, P, K);
  if (!rc) rc = make_map(&mBhi, b_hi, P, K);
  if (!rc) rc = make_map(&mBlo, b_lo, P, K);
  if (rc) return rc;
  const int ktiles = (int)(K / BK);
  const int per = (ktiles + ksplit - 1) / ksplit;
  const int T = (P + BM - 1) / BM;
  // the dynamic shared-memory opt-in is held per device: set it before every launch (cheap), so
  // any device and any thread launching here has it, with no process-wide flag to race on
  SS_CUDA_TRY(cudaFuncSetAttribute(split_bf16_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
  dim3 grid((unsigned)T, (unsigned)T, (unsigned)ksplit);
  split_bf16_gemm_kernel<<<grid, 128, SMEM_BYTES, st>>>(mAhi, mAlo, mBhi, mBlo, P, ktiles, per, c_partial, err_flag);
  SS_CUDA_TRY(cudaGetLastError());
  return SS_OK;
}

}  // namespace ss
