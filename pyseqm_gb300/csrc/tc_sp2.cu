// SP2 purification with the squarings on the 5th-generation tensor cores (tcgen05).
//
// Split-precision product: the FP32 iterate X (symmetric, eigenvalues in [0, 1], so
// |X_ij| <= 1) is split per element into FP16 hi + lo parts, X = Xh + Xl + O(2^-22 |X|)
// (FP16 keeps 11 significant bits and X needs no range beyond it; below 6e-5 the parts
// are subnormal, an absolute error under 6e-8), and
//     X^2 ~= Xh Xh + Xh Xl + Xl Xh          (Xl Xl ~ 2^-22 |X|^2 dropped)
// is accumulated in FP32 in tensor memory (TMEM) by three chains of
// tcgen05.mma.kind::f16 (F16 x F16 -> FP32), M = N = 128, K = 16 per instruction.
// Only tiles with tile_m <= tile_n are computed; off-diagonal tiles are written
// with their mirror.  The diagonal tiles add their diagonal to the molecule's
// trace (FP64).  One CTA (128 threads) per 128x128 output tile; operands are
// converted FP32 -> FP16 hi/lo while staged into shared memory in the canonical
// K-major no-swizzle layout (8x8 core matrices, 16-byte rows).
//
// The SP2 driver (SP2.py:9-85 semantics, per molecule) then keeps X^2 or 2X - X^2
// by the trace test; at convergence the FP64 density is refined by McWeeny steps
// X <- 3 X^2 - 2 X^3 in FP64, restoring idempotency to FP64 level.
//
// Every wait on an mbarrier is bounded: on time-out the kernel raises an error
// flag, still releases its TMEM and returns, so the host gets an error status.
#include <cuda_fp16.h>
#include <math.h>

#include "common.cuh"
#include "sp2_common.cuh"

namespace seqm {

constexpr int TC_M = 128, TC_N = 128, TC_K = 64;  // output tile and K slice (16-bit elements)
constexpr int TC_THREADS = 128;
constexpr int TILE_BYTES = TC_M * TC_K * 2;  // one 16-bit operand tile: 16 KB
constexpr uint32_t TC_FMT = 0;                // kind::f16 operand format: 0 = F16 (1 would be BF16)
constexpr uint32_t WAIT_LIMIT = 1u << 26;     // mbarrier polls before giving up

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D = F32, A = B = F16, both K-major, N = 128, M = 128
__host__ __device__ constexpr uint32_t make_idesc() {
  return (1u << 4) | (TC_FMT << 7) | (TC_FMT << 10) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// returns false when the phase did not complete within WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row, k) of a 128 x 64 16-bit tile in the canonical K-major
// no-swizzle layout: 8x8 core matrices of 128 contiguous bytes, K-neighbours 128 B
// apart (LBO), M-neighbours 8 * 128 = 1024 B apart (SBO)
__device__ __forceinline__ uint32_t tile_off(int row, int k) {
  return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// stage rows [r0, r0+128) x cols [k0, k0+64) of X (FP32, n x n, row-major) as FP16 hi and lo
__device__ __forceinline__ void stage_split(const float *__restrict__ X, int n, int r0, int k0, uint8_t *hi,
                                            uint8_t *lo) {
  for (int v = threadIdx.x; v < TC_M * (TC_K / 8); v += TC_THREADS) {
    const int row = v >> 3, kc = (v & 7) * 8;
    const int gr = r0 + row;
    __align__(16) __half h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int gk = k0 + kc + e;
      const float x = (gr < n && gk < n) ? X[(size_t)gr * n + gk] : 0.0f;
      const __half xh = __float2half_rn(x);
      h[e] = xh;
      l[e] = __float2half_rn(x - __half2float(xh));
    }
    const uint32_t off = tile_off(row, kc);
    *reinterpret_cast<uint4 *>(hi + off) = *reinterpret_cast<const uint4 *>(h);
    *reinterpret_cast<uint4 *>(lo + off) = *reinterpret_cast<const uint4 *>(l);
  }
}

// X2 = X X (split FP16, FP32 accumulate) for the molecules with run[m] != 0
__global__ void __launch_bounds__(TC_THREADS) k_tc_square(seqm_batch b, const float *__restrict__ X,
                                                          float *__restrict__ X2, const int64_t *__restrict__ off,
                                                          const double *__restrict__ st, double *__restrict__ trace,
                                                          int *__restrict__ err) {
  const int m = blockIdx.z;
  if (st[SP2_NS * m + S_RUN] == 0.0) return;
  const int n = b.mol_norb[m];
  const int tm = blockIdx.y, tn = blockIdx.x;
  if (tm > tn || tm * TC_M >= n || tn * TC_N >= n) return;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *Ah = smem, *Al = smem + TILE_BYTES, *Bh = smem + 2 * TILE_BYTES, *Bl = smem + 3 * TILE_BYTES;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const float *Xm = X + off[m];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) tmem_alloc(&tmem_base, TC_N);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_d = tmem_base;
  const uint32_t idesc = make_idesc();
  uint32_t phase = 0;
  const int nk = (n + TC_K - 1) / TC_K;
  for (int kt = 0; kt < nk; ++kt) {
    stage_split(Xm, n, tm * TC_M, kt * TC_K, Ah, Al);
    stage_split(Xm, n, tn * TC_N, kt * TC_K, Bh, Bl);
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t ah = smem_u32(Ah), al = smem_u32(Al), bh = smem_u32(Bh), bl = smem_u32(Bl);
#pragma unroll
      for (int kk = 0; kk < TC_K / 16; ++kk) {  // K = 16 per MMA: two core matrices (256 B) along K
        const uint32_t ko = kk * 256;
        umma_bf16(tmem_d, make_desc(ah + ko, 128, 1024), make_desc(bh + ko, 128, 1024), idesc, (kt | kk) != 0);
        umma_bf16(tmem_d, make_desc(ah + ko, 128, 1024), make_desc(bl + ko, 128, 1024), idesc, 1);
        umma_bf16(tmem_d, make_desc(al + ko, 128, 1024), make_desc(bh + ko, 128, 1024), idesc, 1);
      }
      umma_commit(&bar);
    }
    // the staging buffers are rewritten next iteration: wait for this slice's MMAs
    if (!mbar_wait(&bar, phase)) atomicExch(&failed, 1);
    phase ^= 1;
    __syncthreads();
    if (failed) break;
  }
  tc_fence_after();
  if (!failed) {
    // epilogue: warp w owns accumulator rows 32w..32w+31 (TMEM lanes)
    const int row = tm * TC_M + warp * 32 + lane;
    double tr = 0.0;
    float *Y = X2 + off[m];
#pragma unroll 1
    for (int c0 = 0; c0 < TC_N; c0 += 32) {
      float v[32];
      tmem_ld32(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row < n) {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int col = tn * TC_N + c0 + i;
          if (col < n) {
            Y[(size_t)row * n + col] = v[i];
            if (tm != tn) Y[(size_t)col * n + row] = v[i];
            else if (col == row) tr += (double)v[i];
          }
        }
      }
    }
    if (tm == tn && trace) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
      if (lane == 0) atomicAdd(&trace[m], tr);
    }
  } else if (threadIdx.x == 0) {
    atomicExch(err, SEQM_E_CUDA);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem_d, TC_N);
}


}  // namespace seqm

using namespace seqm;

extern "C" int seqm_density_sp2_tc(const seqm_batch *bp, const double *F, double *P, void *work, double eps,
                                   const uint8_t *active, int32_t *status, int max_iter, int mcweeny_steps,
                                   void *stream) {
  if (!bp || !work || !F || !P) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  eps = eps > 1.0e-3 ? 1.0e-3 : (eps < 1.0e-7 ? 1.0e-7 : eps);
  int64_t total = 0;
  if (cudaMemcpyAsync(&total, b.mol_mat_off + b.nmol, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return SEQM_E_CUDA;
  // work: X f32 [T] | X2 f32 [T] | (pad) | Y f64 [T] | Z f64 [T] | state [SP2_NS nmol] |
  //       row bounds 2 [nmol max_norb] | counters i32 [2]   (FP32 blocks share the FP64 offsets)
  float *X = static_cast<float *>(work);
  float *X2 = X + total;
  double *Y = reinterpret_cast<double *>(X2 + total + (total & 1));
  double *Z = Y + total;
  double *st = Z + total;
  double *rowlo = st + (size_t)SP2_NS * b.nmol;
  double *rowhi = rowlo + (size_t)b.nmol * b.max_norb;
  int *cnt = reinterpret_cast<int *>(rowhi + (size_t)b.nmol * b.max_norb);
  if (cudaMemsetAsync(cnt, 0, 2 * sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
  k_sp2_rows<<<rows_grid(b), 256, 0, s>>>(b, F, rowlo, rowhi, active);
  k_sp2_bounds<<<b.nmol, 256, 0, s>>>(b, rowlo, rowhi, st, active);
  k_sp2_scale<float><<<ew_grid(b), EW_THREADS, 0, s>>>(b, F, X, st);
  k_sp2_start<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st);
  const int tiles = (b.max_norb + TC_M - 1) / TC_M;
  const size_t smem = 4 * TILE_BYTES + 1024;
  if (cudaFuncSetAttribute(k_tc_square, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SEQM_E_CUDA;
  const dim3 grid(tiles, tiles, b.nmol);
  int rc = SEQM_OK;
  for (int it = 0; it < max_iter; ++it) {
    if (cudaMemsetAsync(cnt, 0, sizeof(int), s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    k_tc_square<<<grid, TC_THREADS, smem, s>>>(b, X, X2, b.mol_mat_off, st, nullptr, cnt + 1);
    k_sp2_step<float><<<ew_grid(b), EW_THREADS, 0, s>>>(b, X, X2, st);
    k_sp2_check<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st, eps, 1, cnt);
    if ((it + 1) % SP2_SYNC_EVERY != 0 && it + 1 < max_iter) continue;  // finished molecules skip the extra steps
    int h[2] = {0, 0};
    if (cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    if (h[1] != 0) { rc = h[1]; break; }
    if (h[0] == 0) break;
  }
  if (rc != SEQM_OK) return rc;
  if (status) k_sp2_status<<<(b.nmol + 127) / 128, 128, 0, s>>>(b.nmol, st, active, status);
  // one FP32 McWeeny step X <- 3X^2 - 2X^3 takes the eigenvalues from the tensor-core level
  // (~1e-4 off 0/1 at the relaxed stop) to the FP32 accumulation level (~1e-6), so one
  // FP64-accurate step (mcweeny) then reaches ~1e-11
  float *X3 = reinterpret_cast<float *>(Y);
  k_sym_gemm<float><<<gemm64_grid(b), MW_THREADS, 0, s>>>(b, X, X, X2, active, nullptr);
  k_sym_gemm<float><<<gemm64_grid(b), MW_THREADS, 0, s>>>(b, X2, X, X3, active, nullptr);
  k_mw32<<<ew_grid(b), EW_THREADS, 0, s>>>(b, X2, X3, X, active);
  k_ew_sym<float><<<ew_grid(b), EW_THREADS, 0, s>>>(b, X, 1.0, 1.0, P, active);  // P = X + X^T
  mcweeny(b, P, Y, Z, X, X2, active, mcweeny_steps, s);  // X, X2 are free after P = X + X^T
  return launch_check();
}
