// Chemistry surrogate: a small MLP (BF16 weights, FP32 accumulation) that
// maps a cell's (T, log p, Box-Cox Y, log dt) to its chemistry increment,
// with the kernels that train it and the per-cell gate that decides whether
// a cell keeps the surrogate's answer or goes to the implicit integrator.
//
// The dense layers run on the fifth-generation tensor cores: one CTA of eight
// warps owns a 128-row tile of the output, stages A (activations) and B
// (weights) tiles of 64 k-columns in shared memory in the no-swizzle
// core-matrix layout, and one thread issues tcgen05.mma (M = 128, N = BN,
// K = 16 per instruction) into a TMEM accumulator of BN FP32 columns. The
// operand tiles are double-buffered: the next tile is written while the
// tensor core reads the previous one, and a tcgen05.commit per tile arrives
// on that buffer's mbarrier. The epilogue reads the accumulator with
// tcgen05.ld (warps w and w + 4 share TMEM lanes 32w..32w+31, i.e. those
// rows of the tile, and split the columns) and fuses bias, GELU and the
// GELU derivative of the backward pass. Every wait is bounded (a wall-clock limit read from %globaltimer);
// a wait that runs out sets the module's error word, the kernel frees its
// TMEM and returns, and the host reads the word after the call.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/edyn_surrogate.h"

namespace edyn {
namespace mlp {

constexpr int BM = 128;  // tile rows (TMEM lanes)
constexpr int BK = 64;   // k-columns per staged tile
constexpr int GEMM_THREADS = 256;  // eight warps: two per TMEM lane quarter in the epilogue
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s

__device__ unsigned g_err;
// Limit of the waits that gate the next step of a GEMM (operand copies
// landed, a buffer free again). A wait that runs out stops the GEMM; the
// drain waits afterwards (copies and products already issued) always keep
// the full WAIT_NS. 0 makes every gating wait give up at once, which is how
// a test reaches the failure path without a stuck barrier.
__device__ unsigned long long g_wait_ns = WAIT_NS;

enum Epi : int { EPI_F32 = 0, EPI_GELU = 1, EPI_DGELU = 2 };

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int lda, ldb, M, N, K;
  int epi;
  const float* bias;  // [N] or null
  float* C32;         // fp32 output (EPI_F32: the result; EPI_GELU: the pre-activation), or null
  int ldc;
  __nv_bfloat16* C16; // bf16 output (EPI_GELU: gelu(z); EPI_DGELU: acc * gelu'(z)), or null
                      // (EPI_DGELU writes the same values to C32 in FP32 when C32 is given)
  int ldc16;
  const float* Z;     // EPI_DGELU: the forward pre-activation
  int ldz;
  int c16_tiled;      // EPI_GELU: C16 written in the tiled layout (128-row blocks, K = N) instead of row-major
};

// Tiled layout of a row-major [R][K] matrix for the bulk-copy GEMM: blocks
// of BR rows x 64 k-columns, block (r / BR, k / 64) at element
// ((r / BR) * (K / 64) + k / 64) * BR * 64, each block in the core-matrix
// layout of the shared-memory tiles (element (r, k) of the block at
// ((r / 8) * 8 + k / 8) * 64 + (r % 8) * 8 + k % 8). A block is one
// contiguous bulk copy.
__host__ __device__ __forceinline__ size_t tiled_off(int r, int k, int BR, int K) {
  const int rl = r % BR, kl = k % 64;
  return ((size_t)(r / BR) * (K / 64) + k / 64) * (size_t)BR * 64 + ((rl >> 3) * 8 + (kl >> 3)) * 64 + (rl & 7) * 8 +
         (kl & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

// Bounded wait for the phase of the given parity to complete. false: the
// limit ran out (limit 0: at once, without polling).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, unsigned long long limit = WAIT_NS) {
  if (limit == 0) return false;
  const uint32_t a = smem_u32(b);
  const unsigned long long t0 = gtime();
  for (int it = 0; it < (1 << 26); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 255) == 255 && gtime() - t0 > limit) break;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of
// 8 rows x 16 bytes (128 contiguous bytes); lbo = byte step between core
// matrices along K, sbo = byte step between 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;  // descriptor version of the fifth-generation tensor core
  return d;          // base offset 0, absolute lbo mode, swizzle none
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive FP32 columns of this thread's TMEM lane, one wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float dgelu(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Copies rows [r0, r0 + R) x k-columns [k0, k0 + 64) of a row-major bf16
// matrix into the core-matrix layout: element (r, k) at byte
// ((r / 8) * 8 + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2, so lbo = 128
// and sbo = 1024. Rows at or past nrows are written as zeros. Each thread
// moves 16 bytes per piece; eight consecutive threads fill one 128-byte core
// matrix.
template <int R>
__device__ __forceinline__ void stage_tile(char* dst, const __nv_bfloat16* src, int ld, int r0, int nrows, int k0) {
  constexpr int PIECES = R * BK / 8;
#pragma unroll 4
  for (int q = threadIdx.x; q < PIECES; q += blockDim.x) {
    const int rl = q & 7, kc = (q >> 3) & 7, g = q >> 6;
    const int r = g * 8 + rl;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r0 + r < nrows) v = *reinterpret_cast<const uint4*>(src + (size_t)(r0 + r) * ld + k0 + kc * 8);
    *reinterpret_cast<uint4*>(dst + (g * 8 + kc) * 128 + rl * 16) = v;
  }
}

// Reads the 128 x BN FP32 accumulator from TMEM and applies the fused
// epilogue of a. A warp may read only its quarter of the TMEM lanes
// (warp w: lanes 32 (w % 4) .. + 31, i.e. those rows of the tile), so the
// eight warps of a CTA pair up on each quarter and split its columns.
template <int BN>
__device__ __forceinline__ void epilogue(const GemmArgs& a, uint32_t tmem, int m0, int n0) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = warp & 3, half_cols = warp >> 2;
  const int row = m0 + quarter * 32 + lane;
  const bool live = row < a.M;
  for (int c32 = half_cols * (BN / 2); c32 < (half_cols + 1) * (BN / 2); c32 += 32) {
    float w32[32];
    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c32, w32);
    if (!live) continue;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const float* v = w32 + 16 * half;
      const int col = n0 + c32 + 16 * half;
      if (a.epi == EPI_F32) {
        float* o = a.C32 + (size_t)row * a.ldc + col;
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          float4 q;
          q.x = v[i] + (a.bias ? a.bias[col + i] : 0.f);
          q.y = v[i + 1] + (a.bias ? a.bias[col + i + 1] : 0.f);
          q.z = v[i + 2] + (a.bias ? a.bias[col + i + 2] : 0.f);
          q.w = v[i + 3] + (a.bias ? a.bias[col + i + 3] : 0.f);
          *reinterpret_cast<float4*>(o + i) = q;
        }
      } else if (a.epi == EPI_GELU) {
        __align__(16) __nv_bfloat16 h[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float z = v[i] + (a.bias ? a.bias[col + i] : 0.f);
          if (a.C32) a.C32[(size_t)row * a.ldc + col + i] = z;
          h[i] = __float2bfloat16_rn(gelu(z));
        }
        if (a.c16_tiled) {
          *reinterpret_cast<uint4*>(a.C16 + tiled_off(row, col, BM, a.N)) = reinterpret_cast<const uint4*>(h)[0];
          *reinterpret_cast<uint4*>(a.C16 + tiled_off(row, col + 8, BM, a.N)) = reinterpret_cast<const uint4*>(h)[1];
        } else {
          uint4* o = reinterpret_cast<uint4*>(a.C16 + (size_t)row * a.ldc16 + col);
          o[0] = reinterpret_cast<const uint4*>(h)[0];
          o[1] = reinterpret_cast<const uint4*>(h)[1];
        }
      } else {
        __align__(16) __nv_bfloat16 h[16];
        const float* z = a.Z + (size_t)row * a.ldz + col;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float g = v[i] * dgelu(z[i]);
          if (a.C32) a.C32[(size_t)row * a.ldc + col + i] = g;
          h[i] = __float2bfloat16_rn(g);
        }
        uint4* o = reinterpret_cast<uint4*>(a.C16 + (size_t)row * a.ldc16 + col);
        o[0] = reinterpret_cast<const uint4*>(h)[0];
        o[1] = reinterpret_cast<const uint4*>(h)[1];
      }
    }
  }
}

template <int BN>
__global__ void __launch_bounds__(GEMM_THREADS, 1) k_gemm(GemmArgs a) {
  constexpr int A_BYTES = BM * BK * 2;
  constexpr int B_BYTES = BN * BK * 2;
  constexpr int STAGE = A_BYTES + B_BYTES;
  extern __shared__ __align__(1024) char smem[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  char* base = smem + ((1024 - (smem_u32(smem) & 1023)) & 1023);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t IDESC = idesc_bf16(BM, BN);

  const int nk = a.K / BK;
  const unsigned long long wait_ns = g_wait_ns;
  bool ok = true;
  int last = -1;  // last tile whose products were issued
  for (int kt = 0; kt < nk && ok; ++kt) {
    const int buf = kt & 1;
    char* sa = base + buf * STAGE;
    char* sb = sa + A_BYTES;
    if (kt >= 2) ok = mbar_wait(&bar[buf], ((kt - 2) >> 1) & 1, wait_ns);  // the tensor core is done with this buffer
    ok = __syncthreads_and(ok);
    if (!ok) break;
    stage_tile<BM>(sa, a.A, a.lda, m0, a.M, kt * BK);
    stage_tile<BN>(sb, a.B, a.ldb, n0, a.N, kt * BK);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor-core reads
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (int s = 0; s < BK / 16; ++s)
        mma_bf16(tmem, sdesc(a0 + s * 256, 128, 1024), sdesc(b0 + s * 256, 128, 1024), IDESC,
                 (kt > 0 || s > 0) ? 1u : 0u);
      mma_commit(&bar[buf]);
    }
    last = kt;
  }
  // the commit of the last issued tile arrives once every product before it
  // is done; wait for it even after a failed wait, so no product is in
  // flight when the accumulator is freed
  if (last >= 0 && !mbar_wait(&bar[last & 1], (last >> 1) & 1)) ok = false;
  ok = __syncthreads_and(ok) && last == nk - 1;
  tc_fence_after();

  if (ok) epilogue<BN>(a, tmem, m0, n0);
  if (!ok && threadIdx.x == 0) atomicOr(&g_err, 1u);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
  }
}

template <int BN>
constexpr int gemm_smem() {
  return 2 * (BM * BK * 2 + BN * BK * 2) + 1024;
}

template <int BN>
cudaError_t launch_gemm(const GemmArgs& a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, gemm_smem<BN>());
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((a.M + BM - 1) / BM, a.N / BN);
  k_gemm<BN><<<grid, GEMM_THREADS, gemm_smem<BN>(), s>>>(a);
  return cudaGetLastError();
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

// One contiguous global -> shared copy by the bulk-copy (TMA) engine; its
// bytes complete the transaction count of the mbarrier.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

// C = A B^T with both operands pre-tiled (tiled_off: A in 128-row blocks,
// B in BN-row blocks): every stage of the ST-deep ring is two bulk copies,
// 16 KB of A and BN x 128 bytes of B. Thread 0 issues the products of tile
// kt as soon as its copies land, commits them to the stage's "empty"
// barrier, and only then refills the stage of tile kt - 1 with tile
// kt + ST - 1, so the tensor core always has the next products queued.
// Every BN keeps at least two CTAs per SM (shared memory and TMEM), so one
// CTA's epilogue runs under another's copies and products.
template <int BN, int ST>
__global__ void __launch_bounds__(GEMM_THREADS, 1) k_gemm_tiled(GemmArgs a) {
  constexpr int A_BYTES = BM * BK * 2;
  constexpr int B_BYTES = BN * BK * 2;
  constexpr int STAGE = A_BYTES + B_BYTES;
  extern __shared__ __align__(1024) char smem[];
  __shared__ uint64_t full[ST], empty[ST];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_last;
  const int warp = threadIdx.x >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  char* base = smem + ((1024 - (smem_u32(smem) & 1023)) & 1023);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < ST; ++q) {
      mbar_init(&full[q], 1);
      mbar_init(&empty[q], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t IDESC = idesc_bf16(BM, BN);
  const int nk = a.K / BK;
  const char* gA = reinterpret_cast<const char*>(a.A) + (size_t)blockIdx.x * nk * A_BYTES;
  const char* gB = reinterpret_cast<const char*>(a.B) + (size_t)blockIdx.y * nk * B_BYTES;
  const unsigned long long wait_ns = g_wait_ns;
  bool ok = true;
  int last = -1, produced = 0;
  if (threadIdx.x == 0) {
    auto produce = [&](int kt) -> bool {
      const int q = kt % ST;
      if (kt >= ST && !mbar_wait(&empty[q], ((kt / ST) - 1) & 1, wait_ns)) return false;
      char* sa = base + q * STAGE;
      mbar_expect_tx(&full[q], STAGE);
      bulk_g2s(sa, gA + (size_t)kt * A_BYTES, A_BYTES, &full[q]);
      bulk_g2s(sa + A_BYTES, gB + (size_t)kt * B_BYTES, B_BYTES, &full[q]);
      produced = kt + 1;
      return true;
    };
    for (int kt = 0; kt < ST - 1 && kt < nk && ok; ++kt) ok = produce(kt);
    for (int kt = 0; kt < nk && ok; ++kt) {
      const int q = kt % ST;
      if (!mbar_wait(&full[q], (kt / ST) & 1, wait_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(base + q * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
      for (int k = 0; k < BK / 16; ++k)
        mma_bf16(tmem, sdesc(a0 + k * 256, 128, 1024), sdesc(b0 + k * 256, 128, 1024), IDESC,
                 (kt > 0 || k > 0) ? 1u : 0u);
      mma_commit(&empty[q]);
      last = kt;
      if (kt + ST - 1 < nk) ok = produce(kt + ST - 1);
    }
    // nothing may be in flight when the CTA leaves: the copies issued but
    // not consumed, and the products of the last issued tile
    for (int kt = last + 1; kt < produced; ++kt) mbar_wait(&full[kt % ST], (kt / ST) & 1);
    if (last >= 0 && !mbar_wait(&empty[last % ST], (last / ST) & 1)) ok = false;
  }
  if (threadIdx.x == 0) s_last = last;
  ok = __syncthreads_and(ok);
  ok = ok && s_last == nk - 1;
  tc_fence_after();
  if (ok) epilogue<BN>(a, tmem, m0, n0);
  if (!ok && threadIdx.x == 0) atomicOr(&g_err, 1u);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
  }
}

constexpr int TILED_STAGES = 2;  // 97 KB at BN = 256: two CTAs per SM, one's epilogue under the other's products

template <int BN>
constexpr int gemm_tiled_smem() {
  return TILED_STAGES * (BM * BK * 2 + BN * BK * 2) + 1024;
}

template <int BN>
cudaError_t launch_gemm_tiled(const GemmArgs& a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tiled<BN, TILED_STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         gemm_tiled_smem<BN>());
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid(a.M / BM, a.N / BN);
  k_gemm_tiled<BN, TILED_STAGES><<<grid, GEMM_THREADS, gemm_tiled_smem<BN>(), s>>>(a);
  return cudaGetLastError();
}

// Row-major [R][K] bf16 -> tiled layout with BR-row blocks; rows R..Rp-1 of
// the last block (Rp = R rounded up to BR) are zero. One thread per 8
// consecutive k-columns.
__global__ void k_tile(const __nv_bfloat16* in, int R, int K, int BR, __nv_bfloat16* out) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int Rp = (R + BR - 1) / BR * BR;
  if (q >= (long)Rp * (K / 8)) return;
  const int r = (int)(q / (K / 8)), k = (int)(q % (K / 8)) * 8;
  uint4 v = make_uint4(0, 0, 0, 0);
  if (r < R) v = *reinterpret_cast<const uint4*>(in + (size_t)r * K + k);
  *reinterpret_cast<uint4*>(out + tiled_off(r, k, BR, K)) = v;
}

// out[c][r] = in[r][c] for a rows x cols bf16 matrix (32 x 32 tiles).
__global__ void k_transpose(const __nv_bfloat16* in, int rows, int cols, __nv_bfloat16* out) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = blockIdx.y * 32 + j;
    if (r < rows && c < cols) t[j][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  const int r = blockIdx.y * 32 + threadIdx.x;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int cc = blockIdx.x * 32 + j;
    if (r < rows && cc < cols) out[(size_t)cc * rows + r] = t[threadIdx.x][j];
  }
}

// out[c] = sum over rows of X[r][c] (one thread per column, rows in chunks
// reduced in FP64 then added atomically).
__global__ void k_colsum(const float* X, int rows, int cols, int rows_per_block, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int r0 = blockIdx.y * rows_per_block, r1 = min(rows, r0 + rows_per_block);
  double s = 0;
  for (int r = r0; r < r1; ++r) s += X[(size_t)r * cols + c];
  atomicAdd(out + c, (float)s);
}

// Mean-square-error gradient over the first cols_real columns:
// dY = 2 (Y - T) / (rows * cols_real); padded columns get 0. loss += sum of
// squares / (rows * cols_real).
__global__ void k_mse(const float* Y, const float* T, int rows, int cols, int cols_real, float* dY32,
                      __nv_bfloat16* dY16, double* loss) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)rows * cols;
  const double inv = 1.0 / ((double)rows * cols_real);
  double sq = 0;
  if (i < n) {
    const int c = (int)(i % cols);
    float g = 0.f;
    if (c < cols_real) {
      const float d = Y[i] - T[i];
      sq = (double)d * d * inv;
      g = (float)(2.0 * d * inv);
    }
    dY32[i] = g;
    dY16[i] = __float2bfloat16_rn(g);
  }
  for (int o = 16; o; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  if ((threadIdx.x & 31) == 0 && sq != 0) atomicAdd(loss, sq);
}

// Adam on FP32 master weights, then their BF16 copy.
__global__ void k_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16* w16) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (w16) w16[i] = __float2bfloat16_rn(wi);
}

// Network inputs of one cell (yiT = Y_1..Y_ns, T): T, log p, Box-Cox(Y_k)
// with lambda 0.1, log dt, standardised as (x - mu) * isig and zero-padded
// to ldx columns. p = rho R T sum Y_k / W_k (SI: rho kg/m^3, W kg/mol).
__global__ void k_features(int n, int ns, const double* rho, const double* dt, const double* yiT, const double* wmol,
                           const float* mu, const float* isig, __nv_bfloat16* X, int ldx) {
  const int cell = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (cell >= n) return;
  const double* y = yiT + (size_t)cell * (ns + 1);
  const double T = y[ns];
  double s = 0;
  for (int k = lane; k < ns; k += 32) s += y[k] / wmol[k];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const double p = rho[cell] * 8.31446261815324 * T * s;
  __nv_bfloat16* xr = X + (size_t)cell * ldx;
  for (int j = lane; j < ldx; j += 32) {
    float raw = 0.f;
    if (j == 0) raw = (float)T;
    else if (j == 1) raw = (float)log(p);
    else if (j < ns + 2) raw = (float)((pow(fmax(y[j - 2], 1e-30), 0.1) - 1.0) * 10.0);
    else if (j == ns + 2) raw = (float)log(dt[cell]);
    xr[j] = __float2bfloat16_rn((raw - mu[j]) * isig[j]);
  }
}

// Candidate state of one cell from the network output. The network
// predicts the correction of the explicit increment dt f0 in units of its
// own size: component k (0..ns-1 the Y_k, ns the T) takes
//   y1 = y0 + dt f0 + (out_j osig_j + omu_j) (|dt f0| + floor_k),
// output column j = 0 for T and k + 1 for Y_k; floor_k = yfloor for the
// species, tfloor for T; Y_k clipped at 0.
__global__ void k_decode(int n, int ns, const float* out, int ldo, const float* omu, const float* osig,
                         const double* yiT0, const double* f0, const double* dt, double yfloor, double tfloor,
                         double* yiT1) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)n * (ns + 1)) return;
  const long cell = i / (ns + 1);
  const int k = (int)(i % (ns + 1));
  const int j = k == ns ? 0 : k + 1;
  const double e = dt[cell] * f0[i];
  const double c = (double)out[cell * ldo + j] * osig[j] + omu[j];
  const double v = yiT0[i] + e + c * (fabs(e) + (k == ns ? tfloor : yfloor));
  yiT1[i] = k == ns ? v : fmax(v, 0.0);
}

// Per-cell acceptance of a candidate y1 over dt from y0, given the FP64
// right-hand sides f0 = f(y0) and f1 = f(y1):
//  * trapezoidal residual r = y1 - y0 - dt (f0 + f1) / 2 within
//    atol + rtol max(|y0|, |y1|) in every component (no atol on T);
//  * every element's moles sum_k a_ek Y_k / W_k kept within etol of its
//    value at y0 (relative).
// A second candidate (ya, fa), if given, is tried where the first fails and
// copied into y1 when it passes. accept[cell] = 1 (first candidate), 2
// (second) or 0; count[0], count[1] += the cells accepted by each.
__device__ __forceinline__ bool gate_one(int ns, int ne, const double* y0, const double* y1, const double* f0,
                                         const double* f1, double h, const double* wmol, const double* elem,
                                         double rtol, double atol, double etol, int lane) {
  bool good = true;
  for (int k = lane; k <= ns; k += 32) {
    const double a = y0[k], b = y1[k];
    const double r = b - a - 0.5 * h * (f0[k] + f1[k]);
    const double sc = (k == ns ? 0.0 : atol) + rtol * fmax(fabs(a), fabs(b));
    good = good && isfinite(b) && fabs(r) <= sc;
  }
  for (int e = 0; e < ne; ++e) {
    double s0 = 0, s1 = 0;
    for (int k = lane; k < ns; k += 32) {
      const double c = elem[e * ns + k] / wmol[k];
      s0 += c * y0[k];
      s1 += c * y1[k];
    }
    for (int q = 16; q; q >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, q);
      s1 += __shfl_xor_sync(0xffffffffu, s1, q);
    }
    if (s0 > 0) good = good && fabs(s1 - s0) <= etol * s0;
  }
  return __all_sync(0xffffffffu, good);
}

__global__ void k_gate(int n, int ns, int ne, const double* yiT0, double* yiT1, const double* f0, const double* f1,
                       const double* ya, const double* fa, const double* dt, const double* wmol, const double* elem,
                       double rtol, double atol, double etol, int* accept, unsigned* count) {
  const int cell = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (cell >= n) return;
  const size_t o = (size_t)cell * (ns + 1);
  const double h = dt[cell];
  int a = gate_one(ns, ne, yiT0 + o, yiT1 + o, f0 + o, f1 + o, h, wmol, elem, rtol, atol, etol, lane) ? 1 : 0;
  if (!a && ya && gate_one(ns, ne, yiT0 + o, ya + o, f0 + o, fa + o, h, wmol, elem, rtol, atol, etol, lane)) {
    for (int k = lane; k <= ns; k += 32) yiT1[o + k] = ya[o + k];
    a = 2;
  }
  if (lane == 0) {
    accept[cell] = a;
    if (a) atomicAdd(count + (a - 1), 1u);
  }
}

// Indices of the rejected cells (accept == 0), in cell order, and their
// number. One CTA of 1024 threads; each thread takes four consecutive flags
// per round (4096 cells a round), a warp-shuffle scan and a scan of the 32
// warp totals give every rejected cell its place.
__global__ void __launch_bounds__(1024) k_compact_scan(int n, const int* accept, int* idx, int* nrej) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c0 = 0; c0 < n; c0 += 4 * 1024) {
    const int base = c0 + 4 * threadIdx.x;
    int f[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) f[j] = (base + j < n && !accept[base + j]) ? 1 : 0;
    const int mine = f[0] + f[1] + f[2] + f[3];
    int incl = mine;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    int off = carry;
    for (int w = 0; w < warp; ++w) off += warp_tot[w];
    off += incl - mine;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (f[j]) idx[off++] = base + j;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < 32; ++w) t += warp_tot[w];
      carry += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *nrej = carry;
}

// The compacted rows' inputs, gathered grid-wide: rho_p, dt_p and the
// (ns + 1)-value rows yiT_p of the *nrej cells listed in idx.
__global__ void k_compact_gather(int ns, const int* idx, const int* nrej, const double* rho, const double* dt,
                                 const double* yiT, double* rho_p, double* dt_p, double* yiT_p) {
  const long total = *nrej;
  const long row = ns + 1;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total * row; q += (long)gridDim.x * blockDim.x) {
    const long j = q / row, k = q - j * row;
    const int c = idx[j];
    yiT_p[q] = yiT[(size_t)c * row + k];
    if (k == 0) {
      rho_p[j] = rho[c];
      dt_p[j] = dt[c];
    }
  }
}

// yiT1[idx[j]] = yiT_p[j] for the packed rows the integrator advanced.
__global__ void k_scatter(int m, int ns, const int* idx, const double* yiT_p, double* yiT1) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long)m * (ns + 1)) return;
  const long j = q / (ns + 1);
  yiT1[(size_t)idx[j] * (ns + 1) + q % (ns + 1)] = yiT_p[q];
}

inline cudaStream_t S(void* s) { return (cudaStream_t)s; }
inline int rc(cudaError_t e) { return e == cudaSuccess ? EDYN_OK : EDYN_E_CUDA; }

}  // namespace mlp
}  // namespace edyn

using namespace edyn::mlp;

extern "C" {

int edyn_mlp_gemm(const void* A, int lda, const void* B, int ldb, int M, int N, int K, int epi, const float* bias,
                  float* C32, int ldc, void* C16, int ldc16, const float* Z, int ldz, void* stream) {
  if (!A || !B || M <= 0 || N <= 0 || K <= 0 || N % 64 || K % BK || lda % 8 || ldb % 8 || lda < K || ldb < K)
    return EDYN_E_ARG;
  if ((((uintptr_t)A) | ((uintptr_t)B)) & 15) return EDYN_E_ARG;
  if (epi == EPI_F32 && (!C32 || ldc % 4 || ldc < N || (((uintptr_t)C32) & 15))) return EDYN_E_ARG;
  if (epi != EPI_F32 && (!C16 || ldc16 % 8 || ldc16 < N || (((uintptr_t)C16) & 15))) return EDYN_E_ARG;
  if (epi != EPI_F32 && C32 && ldc < N) return EDYN_E_ARG;
  if (epi == EPI_DGELU && (!Z || ldz < N)) return EDYN_E_ARG;
  if (epi < EPI_F32 || epi > EPI_DGELU) return EDYN_E_ARG;
  GemmArgs a{(const __nv_bfloat16*)A, (const __nv_bfloat16*)B, lda, ldb, M, N, K, epi, bias, C32, ldc,
             (__nv_bfloat16*)C16, ldc16, Z, ldz, 0};
  cudaError_t e;
  if (N % 256 == 0) e = launch_gemm<256>(a, S(stream));
  else if (N % 128 == 0) e = launch_gemm<128>(a, S(stream));
  else e = launch_gemm<64>(a, S(stream));
  return rc(e);
}

int edyn_mlp_tile_rows(int N) { return N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : 64; }

int edyn_mlp_tile(const void* in, int R, int K, int BR, void* out, void* stream) {
  if (!in || !out || R <= 0 || K <= 0 || K % 64 || (BR != 64 && BR != 128 && BR != 256)) return EDYN_E_ARG;
  if ((((uintptr_t)in) | ((uintptr_t)out)) & 15) return EDYN_E_ARG;
  const long tot = (long)((R + BR - 1) / BR * BR) * (K / 8);
  k_tile<<<(unsigned)((tot + 255) / 256), 256, 0, S(stream)>>>((const __nv_bfloat16*)in, R, K, BR,
                                                              (__nv_bfloat16*)out);
  return rc(cudaGetLastError());
}

int edyn_mlp_gemm_tiled(const void* At, const void* Bt, int M, int N, int K, int epi, const float* bias, float* C32,
                        int ldc, void* C16, int ldc16, int c16_tiled, void* stream) {
  if (!At || !Bt || M <= 0 || M % BM || N <= 0 || N % 64 || K <= 0 || K % BK) return EDYN_E_ARG;
  if ((((uintptr_t)At) | ((uintptr_t)Bt)) & 15) return EDYN_E_ARG;
  if (epi == EPI_F32 && (!C32 || ldc % 4 || ldc < N || (((uintptr_t)C32) & 15))) return EDYN_E_ARG;
  if (epi == EPI_GELU && (!C16 || (((uintptr_t)C16) & 15) || (!c16_tiled && (ldc16 % 8 || ldc16 < N))))
    return EDYN_E_ARG;
  if (epi == EPI_GELU && C32 && ldc < N) return EDYN_E_ARG;
  if (epi != EPI_F32 && epi != EPI_GELU) return EDYN_E_ARG;
  GemmArgs a{(const __nv_bfloat16*)At, (const __nv_bfloat16*)Bt, 0, 0, M, N, K, epi, bias, C32, ldc,
             (__nv_bfloat16*)C16, ldc16, nullptr, 0, epi == EPI_GELU ? c16_tiled : 0};
  cudaError_t e;
  switch (edyn_mlp_tile_rows(N)) {
    case 256: e = launch_gemm_tiled<256>(a, S(stream)); break;
    case 128: e = launch_gemm_tiled<128>(a, S(stream)); break;
    default: e = launch_gemm_tiled<64>(a, S(stream)); break;
  }
  return rc(e);
}

int edyn_mlp_set_wait_limit(unsigned long long ns) {
  return cudaMemcpyToSymbol(g_wait_ns, &ns, sizeof(ns)) == cudaSuccess ? EDYN_OK : EDYN_E_CUDA;
}

int edyn_mlp_status(void* stream) {
  unsigned h = 0;
  if (cudaMemcpyFromSymbolAsync(&h, g_err, sizeof(h), 0, cudaMemcpyDeviceToHost, S(stream)) != cudaSuccess)
    return EDYN_E_CUDA;
  if (cudaStreamSynchronize(S(stream)) != cudaSuccess) return EDYN_E_CUDA;
  if (h) {
    const unsigned z = 0;
    cudaMemcpyToSymbolAsync(g_err, &z, sizeof(z), 0, cudaMemcpyHostToDevice, S(stream));
    cudaStreamSynchronize(S(stream));
    return EDYN_E_SURR;
  }
  return EDYN_OK;
}

int edyn_mlp_transpose(const void* in, int rows, int cols, void* out, void* stream) {
  if (!in || !out || rows <= 0 || cols <= 0) return EDYN_E_ARG;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), blk(32, 8);
  k_transpose<<<grid, blk, 0, S(stream)>>>((const __nv_bfloat16*)in, rows, cols, (__nv_bfloat16*)out);
  return rc(cudaGetLastError());
}

int edyn_mlp_colsum(const float* X, int rows, int cols, float* out, void* stream) {
  if (!X || !out || rows <= 0 || cols <= 0) return EDYN_E_ARG;
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * cols, S(stream));
  if (e != cudaSuccess) return EDYN_E_CUDA;
  const int rpb = 256;
  dim3 grid((cols + 127) / 128, (rows + rpb - 1) / rpb);
  k_colsum<<<grid, 128, 0, S(stream)>>>(X, rows, cols, rpb, out);
  return rc(cudaGetLastError());
}

int edyn_mlp_mse(const float* Y, const float* T, int rows, int cols, int cols_real, float* dY32, void* dY16,
                 double* loss, void* stream) {
  if (!Y || !T || !dY32 || !dY16 || !loss || rows <= 0 || cols <= 0 || cols_real <= 0 || cols_real > cols)
    return EDYN_E_ARG;
  const long n = (long)rows * cols;
  k_mse<<<(unsigned)((n + 255) / 256), 256, 0, S(stream)>>>(Y, T, rows, cols, cols_real, dY32,
                                                           (__nv_bfloat16*)dY16, loss);
  return rc(cudaGetLastError());
}

int edyn_mlp_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                  int step, void* w16, void* stream) {
  if (!w || !g || !m || !v || n <= 0 || step < 1) return EDYN_E_ARG;
  const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, S(stream)>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2,
                                                            (__nv_bfloat16*)w16);
  return rc(cudaGetLastError());
}

int edyn_mlp_features(int n, int ns, const double* rho, const double* dt, const double* yiT, const double* wmol,
                      const float* mu, const float* isig, void* X, int ldx, void* stream) {
  if (n <= 0 || ns <= 0 || ldx < ns + 3 || ldx % 8 || !rho || !dt || !yiT || !wmol || !mu || !isig || !X)
    return EDYN_E_ARG;
  k_features<<<(n + 7) / 8, 256, 0, S(stream)>>>(n, ns, rho, dt, yiT, wmol, mu, isig, (__nv_bfloat16*)X, ldx);
  return rc(cudaGetLastError());
}

int edyn_mlp_decode(int n, int ns, const float* out, int ldo, const float* omu, const float* osig, const double* yiT0,
                    const double* f0, const double* dt, double yfloor, double tfloor, double* yiT1, void* stream) {
  if (n <= 0 || ns <= 0 || ldo < ns + 1 || !out || !omu || !osig || !yiT0 || !f0 || !dt || !yiT1) return EDYN_E_ARG;
  const long tot = (long)n * (ns + 1);
  k_decode<<<(unsigned)((tot + 255) / 256), 256, 0, S(stream)>>>(n, ns, out, ldo, omu, osig, yiT0, f0, dt, yfloor,
                                                                 tfloor, yiT1);
  return rc(cudaGetLastError());
}

int edyn_mlp_gate(int n, int ns, int ne, const double* yiT0, double* yiT1, const double* f0, const double* f1,
                  const double* ya, const double* fa, const double* dt, const double* wmol, const double* elem,
                  double rtol, double atol, double etol, int* accept, unsigned* count, void* stream) {
  if (n <= 0 || ns <= 0 || ne < 0 || !yiT0 || !yiT1 || !f0 || !f1 || !dt || !wmol || (ne && !elem) || !accept ||
      !count || (!ya != !fa))
    return EDYN_E_ARG;
  k_gate<<<(n + 7) / 8, 256, 0, S(stream)>>>(n, ns, ne, yiT0, yiT1, f0, f1, ya, fa, dt, wmol, elem, rtol, atol, etol,
                                             accept, count);
  return rc(cudaGetLastError());
}

int edyn_mlp_compact(int n, int ns, const int* accept, const double* rho, const double* dt, const double* yiT,
                     int* idx, double* rho_p, double* dt_p, double* yiT_p, int* nrej, void* stream) {
  if (n <= 0 || ns <= 0 || !accept || !rho || !dt || !yiT || !idx || !rho_p || !dt_p || !yiT_p || !nrej)
    return EDYN_E_ARG;
  k_compact_scan<<<1, 1024, 0, S(stream)>>>(n, accept, idx, nrej);
  const long rows = (long)n * (ns + 1);
  const unsigned grid = (unsigned)std::min<long>((rows + 255) / 256, 152L * 16);
  k_compact_gather<<<grid, 256, 0, S(stream)>>>(ns, idx, nrej, rho, dt, yiT, rho_p, dt_p, yiT_p);
  return rc(cudaGetLastError());
}

int edyn_mlp_scatter(int m, int ns, const int* idx, const double* yiT_p, double* yiT1, void* stream) {
  if (m < 0 || ns <= 0) return EDYN_E_ARG;
  if (m == 0) return EDYN_OK;
  if (!idx || !yiT_p || !yiT1) return EDYN_E_ARG;
  const long tot = (long)m * (ns + 1);
  k_scatter<<<(unsigned)((tot + 255) / 256), 256, 0, S(stream)>>>(m, ns, idx, yiT_p, yiT1);
  return rc(cudaGetLastError());
}

}  // extern "C"
