// SP2 purification with the squarings on the 5th-generation tensor cores (tcgen05).
//
// Split-precision product: the FP32 iterate X (symmetric, eigenvalues in [0, 1], so
// |X_ij| <= 1) is kept alongside a copy split per element into FP16 hi + lo parts,
// X = Xh + Xl + O(2^-22 |X|) (FP16 keeps 11 significant bits and X needs no range
// beyond it; below 6e-5 the parts are subnormal, an absolute error under 6e-8), and
//     X^2 ~= Xh Xh + Xh Xl + Xl Xh          (Xl Xl ~ 2^-22 |X|^2 dropped)
// is accumulated in FP32 in tensor memory (TMEM) by three chains of
// tcgen05.mma.kind::f16 (F16 x F16 -> FP32), M = N = 128, K = 16 per instruction.
//
// The split copy is stored as 128-row x 32-k tiles (8 KB per part), already in the
// canonical K-major no-swizzle operand layout (8x8 core matrices of 16-byte rows, K
// neighbours 128 B apart, 8-row groups 512 B apart), so one bulk asynchronous copy
// (cp.async.bulk, completing on an mbarrier) moves an operand tile into shared memory
// with no conversion.  One CTA per upper 128x128 output tile of a molecule: thread 0
// issues the copies of a 3-stage ring (A hi/lo, B hi/lo per stage), thread 32 issues
// the MMAs and frees each stage with tcgen05.commit, and after the last K slice all
// four warps run the epilogue.  X is symmetric, so the B operand (columns of X) is
// the same kind of row tile as A.
//
// The epilogue finishes the SP2 step in the same kernel: it forms
// X' = X^2 or 2X - X^2 (the branch chosen per molecule from tr X and ||X||_F^2 of the
// previous step, SP2.py:58-64), writes X' in FP32 in place (tile and mirror tile,
// through a shared-memory transpose), writes the split tiles of X' into the other
// buffer of a ping-pong pair, and adds tr X' and ||X'||_F^2 (FP64) to the molecule's
// state.  The driver (SP2.py:9-85 semantics, per molecule) then tests convergence;
// at convergence the density is refined by one FP32 McWeeny step and FP64-accurate
// McWeeny steps, restoring idempotency to ~1e-11 or better.
//
// Every wait on an mbarrier is bounded: on time-out the kernel raises an error flag,
// waits (bounded) for its copies in flight, releases its TMEM and returns, so the host
// gets an error status.
#include <cuda_fp16.h>
#include <math.h>

#include "common.cuh"
#include "sp2_common.cuh"

namespace seqm {

constexpr int TC_M = 128, TC_N = 128;               // output tile
constexpr int TC_KT = 32;                           // k width of a stored split tile and of a pipeline stage
constexpr int TC_STAGES = 3;
constexpr int TC_THREADS = 128;
constexpr int SPLIT_TILE_BYTES = TC_M * TC_KT * 2;  // 8 KB: 128 rows x 32 k, FP16
constexpr int STAGE_BYTES = 4 * SPLIT_TILE_BYTES;   // A hi, A lo, B hi, B lo
constexpr int EPI_LD = TC_N + 1;                    // FP32 staging row stride: rows and columns conflict-free
constexpr size_t TC_SMEM = (size_t)TC_STAGES * STAGE_BYTES + 1024;  // + alignment slack
static_assert(TC_M * EPI_LD * 4 <= TC_STAGES * STAGE_BYTES, "epilogue staging reuses the pipeline buffers");
constexpr uint32_t TC_FMT = 0;                      // kind::f16 operand format: 0 = F16 (1 would be BF16)
constexpr uint32_t WAIT_LIMIT = 1u << 26;           // mbarrier polls before giving up

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

// instruction descriptor: D = F32, A = B = F16 (same type for both, as kind::f16 requires),
// both K-major, N = 128, M = 128
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

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bulk asynchronous copy global -> this CTA's shared memory, completing `bytes` on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  uint64_t g;
  asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(g), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// byte offset of element (row, k) of a 128 x 32 FP16 tile in the canonical K-major
// no-swizzle layout: 8x8 core matrices of 128 contiguous bytes, K neighbours 128 B
// apart (LBO), 8-row groups 4 * 128 = 512 B apart (SBO)
__host__ __device__ __forceinline__ uint32_t tile_off(int row, int k) {
  return (uint32_t)((row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
constexpr uint32_t TC_LBO = 128, TC_SBO = 512;

__host__ __device__ __forceinline__ int64_t split_tiles(int n) {
  return (int64_t)((n + TC_M - 1) / TC_M) * ((n + TC_KT - 1) / TC_KT);
}

// 8 FP32 values -> FP16 hi and lo parts, stored as 16 bytes each
__device__ __forceinline__ void split8(const float *v, uint8_t *hi, uint8_t *lo) {
  __align__(16) __half h[8], l[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const __half xh = __float2half_rn(v[e]);
    h[e] = xh;
    l[e] = __float2half_rn(v[e] - __half2float(xh));
  }
  *reinterpret_cast<uint4 *>(hi) = *reinterpret_cast<const uint4 *>(h);
  *reinterpret_cast<uint4 *>(lo) = *reinterpret_cast<const uint4 *>(l);
}

// exclusive prefix sum of each molecule's split-tile count (one CTA of 1024 threads);
// xs_off[nmol] = total
__global__ void __launch_bounds__(1024) k_tc_tile_offsets(seqm_batch b, int64_t *__restrict__ xs_off) {
  __shared__ int64_t part[1024];
  const int per = (b.nmol + 1023) / 1024;
  const int m0 = threadIdx.x * per, m1 = min(b.nmol, m0 + per);
  int64_t s = 0;
  for (int m = m0; m < m1; ++m) s += split_tiles(b.mol_norb[m]);
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t base = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int m = m0; m < m1; ++m) {
    xs_off[m] = base;
    base += split_tiles(b.mol_norb[m]);
  }
  if (threadIdx.x == 1023) xs_off[b.nmol] = part[1023];
}

// Power-of-two exponent e of a molecule's operand scale: with dmax[m] = max |A| (float bits),
// A 2^-e has its largest element in [0.5, 1), so a matrix of small elements (the McWeeny
// correction D, ~1e-6) keeps FP16's 11 significant bits instead of falling into its subnormal
// range.  No dmax or an all-zero matrix: e = 0.
__device__ __forceinline__ int split_exp(const uint32_t *dmax, int m, int fixed = 0) {
  if (!dmax) return fixed;
  const float mx = __uint_as_float(dmax[m]);
  if (!(mx > 0.0f) || !(mx < INFINITY)) return 0;
  int e = 0;
  frexpf(mx, &e);
  return e;
}

// split tiles of the FP32 X of running molecules (scaled by 2^-e of split_exp, or by 2^-fixed_exp
// without dmax): CTA (kb, rb, m) writes tile (rb, kb)
__global__ void __launch_bounds__(128) k_tc_split(seqm_batch b, const float *__restrict__ X, uint8_t *__restrict__ Xh,
                                                  uint8_t *__restrict__ Xl, const int64_t *__restrict__ xs_off,
                                                  const double *__restrict__ st, const uint8_t *__restrict__ active,
                                                  const uint32_t *__restrict__ dmax = nullptr, int fixed_exp = 0) {
  const int m = blockIdx.z;
  if (st ? st[SP2_NS * m + S_RUN] == 0.0 : (active && !active[m])) return;  // running molecules, or active ones
  const int n = b.mol_norb[m];
  const int nb = (n + TC_M - 1) / TC_M, nk = (n + TC_KT - 1) / TC_KT;
  const int rb = blockIdx.y, kb = blockIdx.x;
  if (rb >= nb || kb >= nk) return;
  const float scale = ldexpf(1.0f, -split_exp(dmax, m, fixed_exp));
  const float *Xm = X + b.mol_mat_off[m];
  const size_t tile = (size_t)(xs_off[m] + (int64_t)rb * nk + kb) * SPLIT_TILE_BYTES;
  for (int g = threadIdx.x; g < TC_M * TC_KT / 8; g += 128) {
    const int row = g >> 2, kc = (g & 3) * 8;
    const int gr = rb * TC_M + row, gk = kb * TC_KT + kc;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = (gr < n && gk + e < n) ? scale * Xm[(size_t)gr * n + gk + e] : 0.0f;
    split8(v, Xh + tile + tile_off(row, kc), Xl + tile + tile_off(row, kc));
  }
}

// Upper tile (tm <= tn) of linear index t in a grouped order: the tile columns are cut into bands
// of TC_BAND columns and each band is walked row by row, so the CTAs resident at one time (two
// per SM) read about TC_BAND + 300 / TC_BAND row blocks of split tiles, which stay in L2, where
// a plain column-by-column walk cycles through every row block of a large molecule.
// Returns false for t beyond the nb (nb + 1) / 2 tiles.
constexpr int TC_BAND = 16;
__device__ __forceinline__ bool upper_tile(int t, int nb, int &tm, int &tn) {
  int base = 0;
  for (int lo = 0; lo < nb; lo += TC_BAND) {
    const int w = min(nb, lo + TC_BAND) - lo;
    const int cnt = lo * w + w * (w + 1) / 2;  // rows above the band's diagonal block, then the block
    if (t < base + cnt) {
      int r = t - base;
      if (r < lo * w) {
        tm = r / w;
        tn = lo + r % w;
        return true;
      }
      r -= lo * w;
      int row = lo, len = w;
      while (r >= len) {
        r -= len;
        ++row;
        --len;
      }
      tm = row;
      tn = row + r;
      return true;
    }
    base += cnt;
  }
  return false;
}

// One SP2 step of every running molecule: X' = X^2 or 2X - X^2 (see the file comment).
// Grid: (upper tiles of the largest molecule, molecules); block: 128 threads.
// Operands and epilogue of a plain split product (PROD launches of k_tc_step): C = cY Y + cAB A B,
// B's split tiles in Bh / Bl (A's are the kernel's Xh / Xl), Y an FP32 matrix (NULL: C = cAB A B);
// A and B must commute (functions of one symmetric matrix), so that A B is symmetric and its upper
// tiles with their mirrors are the whole product.  A split with the scale of dmax (k_tc_split)
// has cAB multiplied back by 2^e per molecule (exact).  full: every tile of a general product of
// two symmetric matrices (grid of nb^2 tiles per molecule, no mirrors).
struct TcProduct {
  const uint8_t *Bh, *Bl;
  const float *Y;
  float cY, cAB;
  const uint8_t *active;
  const uint32_t *dmax;
  int full;
};

template <bool PROD>
__global__ void __launch_bounds__(TC_THREADS) k_tc_step(seqm_batch b, float *__restrict__ X,
                                                        const uint8_t *__restrict__ Xh,
                                                        const uint8_t *__restrict__ Xl, uint8_t *__restrict__ Yh,
                                                        uint8_t *__restrict__ Yl,
                                                        const int64_t *__restrict__ xs_off,
                                                        double *__restrict__ st, int *__restrict__ err, TcProduct pp) {
  const int m = blockIdx.y;
  double *s = st + SP2_NS * m;
  if (PROD ? (pp.active && !pp.active[m]) : s[S_RUN] == 0.0) return;
  const int n = b.mol_norb[m];
  const int nb = (n + TC_M - 1) / TC_M, nk = (n + TC_KT - 1) / TC_KT;
  int tm, tn;
  const bool all_tiles = PROD && pp.full;
  if (all_tiles) {
    if ((int)blockIdx.x >= nb * nb) return;
    tm = (int)blockIdx.x / nb;
    tn = (int)blockIdx.x % nb;
  } else if (!upper_tile(blockIdx.x, nb, tm, tn)) {
    return;
  }
  const bool mirror = !all_tiles && tm != tn;

  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed, sh_issued, sh_consumed;
  __shared__ double red[2][TC_THREADS / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) tmem_alloc(&tmem_base, TC_N);
  if (threadIdx.x == 0) {
    for (int i = 0; i < TC_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&done, 1);
    failed = 0;
    sh_issued = 0;
    sh_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_d = tmem_base;
  const uint8_t *tiles_h = Xh + (size_t)xs_off[m] * SPLIT_TILE_BYTES;
  const uint8_t *tiles_l = Xl + (size_t)xs_off[m] * SPLIT_TILE_BYTES;
  const uint8_t *btiles_h = PROD ? pp.Bh + (size_t)xs_off[m] * SPLIT_TILE_BYTES : tiles_h;
  const uint8_t *btiles_l = PROD ? pp.Bl + (size_t)xs_off[m] * SPLIT_TILE_BYTES : tiles_l;
  const size_t rowA = (size_t)tm * nk * SPLIT_TILE_BYTES, rowB = (size_t)tn * nk * SPLIT_TILE_BYTES;

  if (threadIdx.x == 0) {
    // producer: the four operand tiles of K slice kb into stage kb % TC_STAGES
    for (int kb = 0; kb < nk; ++kb) {
      const int si = kb % TC_STAGES;
      if (kb >= TC_STAGES && !mbar_wait(&empty[si], ((kb / TC_STAGES) - 1) & 1)) {
        atomicExch(&failed, 1);
        break;
      }
      uint8_t *dst = smem + si * STAGE_BYTES;
      const size_t ko = (size_t)kb * SPLIT_TILE_BYTES;
      mbar_expect_tx(&full[si], STAGE_BYTES);
      bulk_g2s(dst, tiles_h + rowA + ko, SPLIT_TILE_BYTES, &full[si]);
      bulk_g2s(dst + SPLIT_TILE_BYTES, tiles_l + rowA + ko, SPLIT_TILE_BYTES, &full[si]);
      bulk_g2s(dst + 2 * SPLIT_TILE_BYTES, btiles_h + rowB + ko, SPLIT_TILE_BYTES, &full[si]);
      bulk_g2s(dst + 3 * SPLIT_TILE_BYTES, btiles_l + rowB + ko, SPLIT_TILE_BYTES, &full[si]);
      sh_issued = kb + 1;
    }
  } else if (threadIdx.x == 32) {
    // MMA issuer: 3 products x 2 instructions (K = 16 each) per stage, then free the stage
    const uint32_t idesc = make_idesc();
    for (int kb = 0; kb < nk; ++kb) {
      const int si = kb % TC_STAGES;
      if (!mbar_wait(&full[si], (kb / TC_STAGES) & 1)) {
        atomicExch(&failed, 1);
        break;
      }
      tc_fence_after();
      const uint32_t ah = smem_u32(smem + si * STAGE_BYTES), al = ah + SPLIT_TILE_BYTES;
      const uint32_t bh = ah + 2 * SPLIT_TILE_BYTES, bl = ah + 3 * SPLIT_TILE_BYTES;
#pragma unroll
      for (int kk = 0; kk < TC_KT / 16; ++kk) {
        const uint32_t ko = kk * 256;  // two core matrices along K
        umma_f16(tmem_d, make_desc(ah + ko, TC_LBO, TC_SBO), make_desc(bh + ko, TC_LBO, TC_SBO), idesc,
                 (kb | kk) != 0);
        umma_f16(tmem_d, make_desc(ah + ko, TC_LBO, TC_SBO), make_desc(bl + ko, TC_LBO, TC_SBO), idesc, 1);
        umma_f16(tmem_d, make_desc(al + ko, TC_LBO, TC_SBO), make_desc(bh + ko, TC_LBO, TC_SBO), idesc, 1);
      }
      umma_commit(&empty[si]);
      sh_consumed = kb + 1;
    }
    umma_commit(&done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  if (!mbar_wait(&done, 0)) atomicExch(&failed, 1);
  __syncthreads();
  if (failed) {
    // let the copies still in flight land before the shared memory is released
    if (threadIdx.x == 0)
      for (int kb = sh_consumed; kb < sh_issued; ++kb) mbar_wait(&full[kb % TC_STAGES], (kb / TC_STAGES) & 1);
    if (threadIdx.x == 0) atomicExch(err, SEQM_E_CUDA);
  } else {
    tc_fence_after();
    float *stg = reinterpret_cast<float *>(smem);  // 128 x EPI_LD staging; the stages are idle now
    const size_t mo = b.mol_mat_off[m];
    float *Xm = X + mo;
    // old X tile (a product: the Y tile) into staging (coalesced rows)
    const float *Sm = PROD ? (pp.Y ? pp.Y + mo : nullptr) : Xm;
    for (int r = warp; r < TC_M; r += TC_THREADS / 32) {
      const int gr = tm * TC_M + r;
#pragma unroll
      for (int c = lane; c < TC_N; c += 32) {
        const int gc = tn * TC_N + c;
        stg[r * EPI_LD + c] = (Sm && gr < n && gc < n) ? Sm[(size_t)gr * n + gc] : 0.0f;
      }
    }
    __syncthreads();
    // X' row by row: thread i owns accumulator row i (TMEM lane i)
    const double nocc = (double)b.mol_nocc[m], t1 = PROD ? 0.0 : s[S_T1], t2 = PROD ? 0.0 : s[S_T2];
    const float cab = PROD ? ldexpf(pp.cAB, split_exp(pp.dmax, m)) : 0.0f;
    const bool sq = fabs(t2 - nocc) < fabs(2.0 * t1 - t2 - nocc);
    const int i = threadIdx.x, gi = tm * TC_M + i;
    // ||X'||_F^2 in FP32 per 32 columns, then FP64 (the sums of squares carry the tensor-core
    // noise of X' anyway; the trace, which decides convergence, is summed in FP64)
    double tr = 0.0, f2 = 0.0;
#pragma unroll 1
    for (int c0 = 0; c0 < TC_N; c0 += 32) {
      float v[32];
      tmem_ld32(tmem_d + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      float q2 = 0.0f;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int c = c0 + j;
        const float x = stg[i * EPI_LD + c];
        float y = PROD ? fmaf(cab, v[j], pp.cY * x) : (sq ? v[j] : 2.0f * x - v[j]);
        if (gi >= n || tn * TC_N + c >= n) y = 0.0f;  // keep the padding of the split tiles zero
        stg[i * EPI_LD + c] = y;
        q2 = fmaf(y, y, q2);
        if (tm == tn && c == i) tr += (double)y;
      }
      f2 += (double)q2;
    }
    if (tm != tn) f2 *= 2.0;  // the mirror tile
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      tr += __shfl_xor_sync(0xffffffffu, tr, o);
      f2 += __shfl_xor_sync(0xffffffffu, f2, o);
    }
    if (lane == 0) {
      red[0][warp] = tr;
      red[1][warp] = f2;
    }
    __syncthreads();
    if (!PROD && threadIdx.x == 0) {  // (the barrier above also orders the staging rows)
      double a = 0.0, c = 0.0;
      for (int w = 0; w < TC_THREADS / 32; ++w) {
        a += red[0][w];
        c += red[1][w];
      }
      if (a != 0.0) atomicAdd(&s[S_ACC_T], a);
      if (c != 0.0) atomicAdd(&s[S_ACC_F], c);
    }
    // X' in FP32: the tile and its mirror, coalesced rows
    for (int r = warp; r < TC_M; r += TC_THREADS / 32) {
      const int gr = tm * TC_M + r, gr2 = tn * TC_M + r;
#pragma unroll
      for (int c = lane; c < TC_N; c += 32) {
        const int gc = tn * TC_N + c, gc2 = tm * TC_N + c;
        if (gr < n && gc < n) Xm[(size_t)gr * n + gc] = stg[r * EPI_LD + c];
        if (mirror && gr2 < n && gc2 < n) Xm[(size_t)gr2 * n + gc2] = stg[c * EPI_LD + r];
      }
    }
    // split tiles of X': tile (tm, 4 tn + q) and mirror tile (tn, 4 tm + q), 8 k per store
    uint8_t *oh = Yh ? Yh + (size_t)xs_off[m] * SPLIT_TILE_BYTES : nullptr;
    uint8_t *ol = Yl ? Yl + (size_t)xs_off[m] * SPLIT_TILE_BYTES : nullptr;
    for (int g = threadIdx.x; oh && g < TC_M * (TC_N / 8); g += TC_THREADS) {
      const int r = g >> 4, cg = (g & 15) * 8, q = cg / TC_KT, kc = cg % TC_KT;
      float v[8];
      const int kb1 = (tn * TC_N) / TC_KT + q;
      if (kb1 < nk) {
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = stg[r * EPI_LD + cg + e];
        const size_t tile = ((size_t)tm * nk + kb1) * SPLIT_TILE_BYTES + tile_off(r, kc);
        split8(v, oh + tile, ol + tile);
      }
      const int kb2 = (tm * TC_N) / TC_KT + q;
      if (tm != tn && kb2 < nk) {
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = stg[(cg + e) * EPI_LD + r];
        const size_t tile = ((size_t)tn * nk + kb2) * SPLIT_TILE_BYTES + tile_off(r, kc);
        split8(v, oh + tile, ol + tile);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem_d, TC_N);
}

// ----------------------------------------------------------------- work layout
struct TcWork {
  size_t x, x2, y, z, st, rowlo, rowhi, cnt, xs_off, rmask, dmax, xs[4], total;
};

inline TcWork tc_work_layout(int64_t T, int nmol, int maxn) {
  TcWork w{};
  size_t o = 0;
  auto take = [&](size_t bytes, size_t align) {
    o = (o + align - 1) / align * align;
    const size_t r = o;
    o += bytes;
    return r;
  };
  const size_t t = (size_t)(T > 0 ? T : 0), nm = (size_t)(nmol > 0 ? nmol : 0), mx = (size_t)(maxn > 0 ? maxn : 0);
  w.x = take(4 * t, 256);
  w.x2 = take(4 * t, 256);
  w.y = take(8 * t, 256);
  w.z = take(8 * t, 256);
  w.st = take(8 * SP2_NS * nm, 256);
  w.rowlo = take(8 * nm * mx, 256);
  w.rowhi = take(8 * nm * mx, 256);
  w.cnt = take(16, 256);
  w.xs_off = take(8 * (nm + 1), 256);
  w.rmask = take(nm, 256);
  w.dmax = take(4 * nm, 256);
  // sum over molecules of ceil(n/128) ceil(n/32) <= (T + nmol (159 maxn + 3937)) / 4096
  const size_t tiles = (t + nm * (159 * mx + 3937) + 4095) / 4096;
  for (int q = 0; q < 4; ++q) w.xs[q] = take(tiles * SPLIT_TILE_BYTES, 1024);
  w.total = o;
  return w;
}

// molecules whose density takes the FP64-accurate McWeeny step: active with value 1 (2 marks an
// SCF iteration allowed to keep the FP32-level density; see the convergence test)
__global__ void k_refine_mask(int nmol, const uint8_t *__restrict__ active, uint8_t *__restrict__ rmask) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < nmol) rmask[m] = active ? (active[m] == 1) : 1;
}

// FP64-accurate McWeeny step X <- X + D (I - 2X), D = X^2 - X (X = P/2), of the tensor-core form:
// X^2 from FP32 pairs (k_sym_gemm_pair, its cross term Xh Xl a split product on the tensor cores),
// the correction product as a split product on the tensor cores with D scaled to FP16's range per
// molecule.  Buffers: Y, Z FP64 and Df, Bf FP32 of the batch's matrix size (Y doubles as the FP32
// correction, Bf as the cross term once split), xs[0..3] split tiles.
inline void mcweeny_tc(const seqm_batch &b, double *P, double *Y, double *Z, float *Df, float *Bf, uint8_t *const *xs,
                       const int64_t *xs_off, double *st, int *err, uint32_t *dmax, const uint8_t *rmask, int steps,
                       cudaStream_t s) {
  float *Cf = reinterpret_cast<float *>(Y);
  const int nb = (b.max_norb + TC_M - 1) / TC_M, nk = (b.max_norb + TC_KT - 1) / TC_KT;
  const dim3 grid((unsigned)(nb * (nb + 1) / 2), (unsigned)b.nmol), split((unsigned)nk, (unsigned)nb, (unsigned)b.nmol);
  const dim3 grid_full((unsigned)(nb * nb), (unsigned)b.nmol);
  for (int k = 0; k < steps; ++k) {
    k_ew_axpby<<<ew_grid(b), EW_THREADS, 0, s>>>(b, 0.5, P, 0.0, nullptr, Z, rmask);  // Z = X
    k_split_pair<<<ew_grid(b), EW_THREADS, 0, s>>>(b, Z, Df, Bf, rmask);             // Xh, Xl
    k_tc_split<<<split, 128, 0, s>>>(b, Df, xs[0], xs[1], xs_off, nullptr, rmask);
    k_tc_split<<<split, 128, 0, s>>>(b, Bf, xs[2], xs[3], xs_off, nullptr, rmask, nullptr, -24);  // 2^24 Xl
    k_tc_step<true><<<grid_full, TC_THREADS, TC_SMEM, s>>>(b, Bf, xs[0], xs[1], nullptr, nullptr, xs_off, st, err,
                                                          TcProduct{xs[2], xs[3], nullptr, 0.0f, 0x1p-24f, rmask,
                                                                    nullptr, 1});  // Bf = M = Xh Xl
    k_sym_gemm_pair<<<pair_gemm_grid(b), DF_THREADS, 0, s>>>(b, Df, Bf, Y, rmask);   // Y = X^2
    cudaMemsetAsync(dmax, 0, sizeof(uint32_t) * b.nmol, s);
    k_mw_split<<<ew_grid(b), EW_THREADS, 0, s>>>(b, Y, Z, Df, Bf, rmask, dmax);      // D, I - 2X, max |D|
    k_tc_split<<<split, 128, 0, s>>>(b, Df, xs[0], xs[1], xs_off, nullptr, rmask, dmax);
    k_tc_split<<<split, 128, 0, s>>>(b, Bf, xs[2], xs[3], xs_off, nullptr, rmask);
    k_tc_step<true><<<grid, TC_THREADS, TC_SMEM, s>>>(b, Cf, xs[0], xs[1], nullptr, nullptr, xs_off, st, err,
                                                     TcProduct{xs[2], xs[3], nullptr, 0.0f, 1.0f, rmask, dmax});
    k_mw_update<<<ew_grid(b), EW_THREADS, 0, s>>>(b, Z, Cf, P, rmask);              // P = 2 (X + D (I - 2X))
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" size_t seqm_sp2_tc_work_bytes(int64_t total_matrix_elements, int nmol, int max_norb) {
  return tc_work_layout(total_matrix_elements, nmol, max_norb).total;
}

extern "C" int seqm_density_sp2_tc(const seqm_batch *bp, const double *F, double *P, void *work, double eps,
                                   const uint8_t *active, int32_t *status, int max_iter, int mcweeny_steps,
                                   void *stream) {
  if (!bp || !work || !F || !P) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  if (b.nmol > 65535) return SEQM_E_TOO_LARGE;  // molecules are the grid's y dimension
  if ((reinterpret_cast<uintptr_t>(work) & 255) != 0) return SEQM_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  eps = eps > 1.0e-3 ? 1.0e-3 : (eps < 1.0e-7 ? 1.0e-7 : eps);
  int64_t total = 0;
  if (batch_total(b, s, &total) != SEQM_OK) return SEQM_E_CUDA;
  const TcWork w = tc_work_layout(total, b.nmol, b.max_norb);
  uint8_t *base = static_cast<uint8_t *>(work);
  float *X = reinterpret_cast<float *>(base + w.x);
  float *X2 = reinterpret_cast<float *>(base + w.x2);
  double *Y = reinterpret_cast<double *>(base + w.y);
  double *Z = reinterpret_cast<double *>(base + w.z);
  double *st = reinterpret_cast<double *>(base + w.st);
  double *rowlo = reinterpret_cast<double *>(base + w.rowlo);
  double *rowhi = reinterpret_cast<double *>(base + w.rowhi);
  int *cnt = reinterpret_cast<int *>(base + w.cnt);
  int64_t *xs_off = reinterpret_cast<int64_t *>(base + w.xs_off);
  uint8_t *xs[4] = {base + w.xs[0], base + w.xs[1], base + w.xs[2], base + w.xs[3]};  // hi, lo of two buffers
  if (cudaMemsetAsync(cnt, 0, LC_WORDS * sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
  k_sp2_rows<<<rows_grid(b), 256, 0, s>>>(b, F, rowlo, rowhi, active);
  k_sp2_bounds<<<b.nmol, 256, 0, s>>>(b, rowlo, rowhi, st, active);
  k_sp2_scale<float><<<ew_grid(b), EW_THREADS, 0, s>>>(b, F, X, st);
  k_sp2_start<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st);
  k_tc_tile_offsets<<<1, 1024, 0, s>>>(b, xs_off);
  const int nb = (b.max_norb + TC_M - 1) / TC_M, nk = (b.max_norb + TC_KT - 1) / TC_KT;
  k_tc_split<<<dim3(nk, nb, b.nmol), 128, 0, s>>>(b, X, xs[0], xs[1], xs_off, st, nullptr);
  {
    static SmemLimit limit;
    int rc0 = limit.ensure(k_tc_step<false>, TC_SMEM);
    static SmemLimit limit_prod;
    if (rc0 == SEQM_OK) rc0 = limit_prod.ensure(k_tc_step<true>, TC_SMEM);
    if (rc0 != SEQM_OK) return rc0;
  }
  const dim3 grid((unsigned)(nb * (nb + 1) / 2), (unsigned)b.nmol);
  int rc = SEQM_OK, cur = 0;
  if (stream_capturing(s)) {
    // inside a CUDA graph capture: the step loop becomes a WHILE node ended on the device; one
    // trip takes two steps so that the split-tile buffers ping-pong back to where they started
    // (a molecule that stops after the first step of a trip is skipped by the second)
    const cudaError_t e = capture_while_loop(s, [&](cudaGraph_t body, cudaGraphConditionalHandle h) {
      cudaGraphNode_t n[5];
      cudaError_t r = cudaSuccess;
      for (int half = 0; half < 2 && r == cudaSuccess; ++half) {
        const int c = half;
        r = add_kernel_node(body, &n[2 * half], half ? &n[1] : nullptr, half ? 1 : 0, k_tc_step<false>, grid,
                            dim3(TC_THREADS), TC_SMEM, b, X, (const uint8_t *)xs[2 * c], (const uint8_t *)xs[2 * c + 1],
                            xs[2 - 2 * c], xs[3 - 2 * c], (const int64_t *)xs_off, st, cnt + LC_ERR, TcProduct{});
        if (r == cudaSuccess)
          r = add_kernel_node(body, &n[2 * half + 1], &n[2 * half], 1, k_sp2_check, dim3((b.nmol + 127) / 128),
                              dim3(128), 0, b, st, eps, 1, cnt + LC_RUN);
      }
      if (r == cudaSuccess)
        r = add_kernel_node(body, &n[4], &n[3], 1, k_sp2_loop_tail, dim3(1), dim3(1), 0, cnt, h, (max_iter + 1) / 2);
      return r;
    });
    if (e != cudaSuccess) return SEQM_E_CUDA;
  } else
  for (int it = 0; it < max_iter; ++it) {
    if (cudaMemsetAsync(cnt, 0, sizeof(int), s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    k_tc_step<false><<<grid, TC_THREADS, TC_SMEM, s>>>(b, X, xs[2 * cur], xs[2 * cur + 1], xs[2 - 2 * cur],
                                                    xs[3 - 2 * cur], xs_off, st, cnt + 1, TcProduct{});
    k_sp2_check<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st, eps, 1, cnt);
    cur ^= 1;
    if ((it + 1) % SP2_SYNC_EVERY != 0 && it + 1 < max_iter) continue;  // finished molecules skip the extra steps
    int h[2] = {0, 0};
    if (cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    if (h[1] != 0) { rc = h[1]; break; }
    if (h[0] == 0) break;
  }
  if (rc != SEQM_OK) return rc;
  // one FP32 McWeeny step X <- 3X^2 - 2X^3 takes the eigenvalues from the tensor-core level
  // (~1e-4 off 0/1 at the relaxed stop) to the FP32 accumulation level (~1e-6), so one
  // FP64-accurate step (mcweeny) then reaches ~1e-11.  Its two products run as split products
  // on the tensor cores (FP32-level accuracy, like an FP32 CUDA-core product): X2 = X X with its
  // split tiles, then X <- 3 X2 - 2 X2 X
  k_tc_split<<<dim3(nk, nb, b.nmol), 128, 0, s>>>(b, X, xs[0], xs[1], xs_off, nullptr, active);
  k_tc_step<true><<<grid, TC_THREADS, TC_SMEM, s>>>(b, X2, xs[0], xs[1], xs[2], xs[3], xs_off, st, cnt + LC_ERR,
                                                   TcProduct{xs[0], xs[1], nullptr, 0.0f, 1.0f, active});
  k_tc_step<true><<<grid, TC_THREADS, TC_SMEM, s>>>(b, X, xs[2], xs[3], nullptr, nullptr, xs_off, st, cnt + LC_ERR,
                                                   TcProduct{xs[0], xs[1], X2, 3.0f, -2.0f, active});
  k_ew_sym<float><<<ew_grid(b), EW_THREADS, 0, s>>>(b, X, 1.0, 1.0, P, active);  // P = X + X^T
  // FP64-accurate steps for the molecules that want them (X, X2 and the split tiles are free now)
  uint8_t *rmask = base + w.rmask;
  k_refine_mask<<<(b.nmol + 255) / 256, 256, 0, s>>>(b.nmol, active, rmask);
  mcweeny_tc(b, P, Y, Z, X, X2, xs, xs_off, st, cnt + LC_ERR, reinterpret_cast<uint32_t *>(base + w.dmax), rmask,
             mcweeny_steps, s);
  // after the products, so that a product kernel that gave up waiting shows in status too
  if (status) k_sp2_status<<<(b.nmol + 127) / 128, 128, 0, s>>>(b.nmol, st, active, status, cnt + LC_ERR);
  return launch_check();
}
