// Shared SP2 machinery (plain FP64 and tensor-core forms): multi-CTA elementwise passes
// over (chunk, molecule) grids with per-molecule FP64 accumulators, so a large
// molecule's n^2 elements are spread over the whole GPU, and the FP64 symmetric
// tile product used for FP64 squarings and McWeeny refinement.
//
// Per-molecule state (doubles, SP2_NS per molecule):
//   err0, err1 (trace errors of the last two steps), err2, running flag, steps,
//   t1 = tr X, t2 = ||X||_F^2 = tr X^2 (X symmetric), accumulators for the new X,
//   Gershgorin bounds h1, hN.
#pragma once

#include <math.h>

#include <tuple>

#include "common.cuh"

namespace seqm {
namespace {  // internal linkage: this header is compiled into more than one translation unit

enum { S_ERR0 = 0, S_ERR1, S_ERR2, S_RUN, S_STEPS, S_T1, S_T2, S_ACC_T, S_ACC_F, S_H1, S_HN, SP2_NS };
constexpr int EW_THREADS = 256;
// the SP2 drivers read the running count back every SP2_SYNC_EVERY steps; a molecule that
// stopped earlier is skipped by every kernel of the steps in between
constexpr int SP2_SYNC_EVERY = 4;
constexpr int EW_CHUNK = EW_THREADS * 8;  // elements per CTA of an elementwise pass


__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// add per-CTA partial sums of (a, b) into acc[0], acc[1]
__device__ __forceinline__ void cta_accumulate2(double a, double b, double *acc) {
  __shared__ double ra[EW_THREADS / 32], rb[EW_THREADS / 32];
  a = warp_sum(a);
  b = warp_sum(b);
  if ((threadIdx.x & 31) == 0) { ra[threadIdx.x >> 5] = a; rb[threadIdx.x >> 5] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int w = 0; w < EW_THREADS / 32; ++w) { sa += ra[w]; sb += rb[w]; }
    if (sa != 0.0) atomicAdd(acc, sa);
    if (sb != 0.0) atomicAdd(acc + 1, sb);
  }
}

// Gershgorin row bounds of F, one warp per row: lo[i] = a_ii - r_i, hi[i] = a_ii + r_i
__global__ void k_sp2_rows(seqm_batch b, const double *__restrict__ F, double *__restrict__ rowlo,
                           double *__restrict__ rowhi, const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= n) return;
  const double *Fr = F + b.mol_mat_off[m] + (size_t)row * n;
  double s = 0.0;
  for (int j = lane; j < n; j += 32) s += fabs(Fr[j]);
  s = warp_sum(s);
  if (lane == 0) {
    const double aii = Fr[row], ri = s - fabs(aii);
    rowlo[(size_t)m * b.max_norb + row] = aii - ri;
    rowhi[(size_t)m * b.max_norb + row] = aii + ri;
  }
}

// per molecule: h1 = min lo, hN = max hi; clear the accumulators
__global__ void k_sp2_bounds(seqm_batch b, const double *__restrict__ rowlo, const double *__restrict__ rowhi,
                             double *__restrict__ st, const uint8_t *__restrict__ active) {
  const int m = blockIdx.x;
  double *s = st + SP2_NS * m;
  if (active && !active[m]) {
    if (threadIdx.x == 0) s[S_RUN] = 0.0;
    return;
  }
  const int n = b.mol_norb[m];
  double lo = INFINITY, hi = -INFINITY;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    lo = fmin(lo, rowlo[(size_t)m * b.max_norb + i]);
    hi = fmax(hi, rowhi[(size_t)m * b.max_norb + i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ double rl[32], rh[32];
  if ((threadIdx.x & 31) == 0) { rl[threadIdx.x >> 5] = lo; rh[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x / 32); ++w) { lo = fmin(lo, rl[w]); hi = fmax(hi, rh[w]); }
    lo = fmin(lo, rl[0]);
    hi = fmax(hi, rh[0]);
    s[S_H1] = lo; s[S_HN] = hi; s[S_ACC_T] = 0.0; s[S_ACC_F] = 0.0; s[S_RUN] = 1.0; s[S_STEPS] = 0.0;
  }
}

// X0 = (hN I - F)/(hN - h1) (SP2.py:36-43), accumulating tr X0 and ||X0||^2
template <class T>
__global__ void __launch_bounds__(EW_THREADS) k_sp2_scale(seqm_batch b, const double *__restrict__ F,
                                                          T *__restrict__ X, double *__restrict__ st) {
  const int m = blockIdx.y;
  double *s = st + SP2_NS * m;
  if (s[S_RUN] == 0.0) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const double h1 = s[S_H1], hN = s[S_HN], inv = 1.0 / (hN - h1);
  const size_t mo = b.mol_mat_off[m];
  const DiagTest diagonal(n);  // n^2 < 2^32 for every molecule a batch holds
  double tr = 0.0, f2 = 0.0;
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const bool d = diagonal((uint32_t)idx);
    // the FP64 form divides as SP2.py:36-43 does; the FP32 iterate takes the reciprocal
    const double a = (d ? hN : 0.0) - F[mo + idx];
    const T v = (T)(sizeof(T) == 8 ? a / (hN - h1) : a * inv);
    X[mo + idx] = v;
    if (d) tr += (double)v;
    f2 += (double)v * (double)v;
  }
  cta_accumulate2(tr, f2, s + S_ACC_T);
}

// after the X0 pass: t1, t2 and the initial trace error
__global__ void k_sp2_start(seqm_batch b, double *__restrict__ st) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.nmol) return;
  double *s = st + SP2_NS * m;
  if (s[S_RUN] == 0.0) return;
  s[S_T1] = s[S_ACC_T];
  s[S_T2] = s[S_ACC_F];
  const double e = fabs(s[S_T1] - (double)b.mol_nocc[m]);
  s[S_ERR0] = e; s[S_ERR1] = e; s[S_ERR2] = e;
  s[S_ACC_T] = 0.0; s[S_ACC_F] = 0.0;
}

// keep X^2 or 2X - X^2 by the trace test (SP2.py:58-64), with tr X^2 = ||X||_F^2
template <class T>
__global__ void __launch_bounds__(EW_THREADS) k_sp2_step(seqm_batch b, T *__restrict__ X, const T *__restrict__ X2,
                                                         double *__restrict__ st) {
  const int m = blockIdx.y;
  double *s = st + SP2_NS * m;
  if (s[S_RUN] == 0.0) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const double nocc = (double)b.mol_nocc[m], t1 = s[S_T1], t2 = s[S_T2];
  const bool sq = fabs(t2 - nocc) < fabs(2.0 * t1 - t2 - nocc);
  const size_t mo = b.mol_mat_off[m];
  const DiagTest diagonal(n);
  double tr = 0.0, f2 = 0.0;
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const T x = X[mo + idx], y = X2[mo + idx];
    const T v = sq ? y : (T)2 * x - y;
    X[mo + idx] = v;
    if (diagonal((uint32_t)idx)) tr += (double)v;
    f2 += (double)v * (double)v;
  }
  cta_accumulate2(tr, f2, s + S_ACC_T);
}

// per molecule after a step: errors, convergence, next t1/t2; counts still-running molecules.
// relaxed: also stop when the error is below 1e-2 and no longer improving (SP2.py:76-80,
// the reference's rule for reduced precision)
__global__ void k_sp2_check(seqm_batch b, double *__restrict__ st, double eps, int relaxed, int *__restrict__ nrun) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= b.nmol) return;
  double *s = st + SP2_NS * m;
  if (s[S_RUN] == 0.0) return;
  const double e0 = fabs(s[S_ACC_T] - (double)b.mol_nocc[m]);
  const double e1 = s[S_ERR0], e2 = s[S_ERR1];
  s[S_ERR2] = e2; s[S_ERR1] = e1; s[S_ERR0] = e0;
  s[S_STEPS] += 1.0;
  s[S_T1] = s[S_ACC_T];
  s[S_T2] = s[S_ACC_F];
  s[S_ACC_T] = 0.0;
  s[S_ACC_F] = 0.0;
  const bool done = (e0 < eps && e1 < eps) || (relaxed && e0 < 1.0e-2 && e0 >= e2);
  if (done) s[S_RUN] = 0.0;
  else atomicAdd(nrun, 1);
}

// status[m] = steps, or -1 if still running at the cap, or SEQM_E_CUDA if the step kernel
// raised its error word (err, NULL: none)
__global__ void k_sp2_status(int nmol, const double *__restrict__ st, const uint8_t *__restrict__ active,
                             int32_t *__restrict__ status, const int *__restrict__ err) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmol || (active && !active[m])) return;
  const double *s = st + SP2_NS * m;
  status[m] = (err && *err) ? SEQM_E_CUDA : s[S_RUN] != 0.0 ? -1 : (int)s[S_STEPS];
}

// elementwise P = c1 * A + c2 * A^T (FP64 out) for active molecules (A in T precision)
template <class T>
__global__ void __launch_bounds__(EW_THREADS) k_ew_sym(seqm_batch b, const T *__restrict__ A, double c1, double c2,
                                                       double *__restrict__ P, const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const size_t mo = b.mol_mat_off[m];
  const FastDivU32 row((uint32_t)n);
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const size_t i = row.div((uint32_t)idx), j = idx - i * n;
    P[mo + idx] = c1 * (double)A[mo + idx] + c2 * (double)A[mo + j * n + i];
  }
}

// elementwise D = a * A + c * C (FP64) for active molecules
__global__ void __launch_bounds__(EW_THREADS) k_ew_axpby(seqm_batch b, double a, const double *__restrict__ A, double c,
                                                         const double *__restrict__ C, double *__restrict__ D,
                                                         const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const size_t mo = b.mol_mat_off[m];
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS)
    D[mo + idx] = a * A[mo + idx] + (C ? c * C[mo + idx] : 0.0);
}

// C = A B (T = double or float) with A symmetric.  When B and the product are symmetric too
// (X X, functions of one X; FULL = false) only the upper
// MW_T x MW_T output tiles are computed and each is written with its mirror (FULL: every tile,
// no mirror, for a general B).  With A
// symmetric, the A slab A[i0.., k0..] is read as rows of A[k0.., i0..], so both slabs
// load along rows (coalesced) and are stored K-major without a transpose.  Small tiles
// keep the FP64 pipes of all SMs busy on one molecule (a 1296-AO matrix gives 861
// upper tiles); the next K slab is prefetched into registers during the FMAs.
constexpr int MW_T = 32, MW_K = 32, MW_THREADS = 256;
template <class T>
struct vec2;
template <>
struct vec2<double> {
  using type = double2;
};
template <>
struct vec2<float> {
  using type = float2;
};
template <class T, bool FULL = false>
__global__ void __launch_bounds__(MW_THREADS) k_sym_gemm(seqm_batch b, const T *__restrict__ Am,
                                                         const T *__restrict__ Bm, T *__restrict__ Cm,
                                                         const uint8_t *__restrict__ active,
                                                         const double *__restrict__ st) {
  const int m = blockIdx.z;
  if (active && !active[m]) return;
  if (st && st[SP2_NS * m + S_RUN] == 0.0) return;
  const int n = b.mol_norb[m];
  const int i0 = blockIdx.y * MW_T, j0 = blockIdx.x * MW_T;
  if (i0 >= n || j0 >= n || (!FULL && blockIdx.y > blockIdx.x)) return;
  const size_t mo = b.mol_mat_off[m];
  const T *A = Am + mo, *B = Bm + mo;
  __shared__ __align__(16) T As[2][MW_K][MW_T], Bs[2][MW_K][MW_T];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  // slab loader: element e = threadIdx.x + 256 q (q = 0..3) of the 32 x 32 slab, row kk = e / 32, col c = e % 32
  T ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = threadIdx.x + MW_THREADS * q, kk = e >> 5, c = e & 31;
      const bool kin = k0 + kk < n;
      ra[q] = (kin && i0 + c < n) ? A[(size_t)(k0 + kk) * n + i0 + c] : (T)0;
      rb[q] = (kin && j0 + c < n) ? B[(size_t)(k0 + kk) * n + j0 + c] : (T)0;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = threadIdx.x + MW_THREADS * q, kk = e >> 5, c = e & 31;
      As[buf][kk][c] = ra[q];
      Bs[buf][kk][c] = rb[q];
    }
  };
  T acc[2][2] = {};
  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < n; k0 += MW_K) {
    const bool more = k0 + MW_K < n;
    if (more) load(k0 + MW_K);
#pragma unroll
    for (int kk = 0; kk < MW_K; ++kk) {
      using V = typename vec2<T>::type;
      const V a = *reinterpret_cast<const V *>(&As[buf][kk][2 * ty]);
      const V c = *reinterpret_cast<const V *>(&Bs[buf][kk][2 * tx]);
      acc[0][0] += a.x * c.x;
      acc[0][1] += a.x * c.y;
      acc[1][0] += a.y * c.x;
      acc[1][1] += a.y * c.y;
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  T *C = Cm + mo;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int row = i0 + 2 * ty + r, col = j0 + 2 * tx + q;
      if (row < n && col < n) {
        C[(size_t)row * n + col] = acc[r][q];
        if (!FULL) C[(size_t)col * n + row] = acc[r][q];
      }
    }
}

// ------------------------------------------------------------------ device-driven step loop
// Loop counters of an SP2 call (int words of the driver's scratch): [0] molecules still running
// after the last check (summed by k_sp2_check), [1] error word, [2] loop trips taken.
enum { LC_RUN = 0, LC_ERR, LC_TRIPS, LC_WORDS };

// End of one trip of the device-driven loop: the trip counts, the running count is consumed, and
// the loop's condition (a CUDA graph WHILE node) stays set while molecules run, no error was
// raised and fewer than max_trips trips were taken.
__global__ void k_sp2_loop_tail(int *__restrict__ lc, cudaGraphConditionalHandle handle, int max_trips) {
  const int run = lc[LC_RUN];
  lc[LC_RUN] = 0;
  const int trips = ++lc[LC_TRIPS];
  cudaGraphSetConditional(handle, (run > 0 && lc[LC_ERR] == 0 && trips < max_trips) ? 1u : 0u);
}

// kernel node of `g` after `ndep` nodes: func<<<grid, block, smem>>>(args...), the arguments
// converted to the kernel's parameter types and copied into the node
template <typename... Params, typename... Args>
cudaError_t add_kernel_node(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *dep, size_t ndep,
                            void (*func)(Params...), dim3 grid, dim3 block, size_t smem, Args... args) {
  static_assert(sizeof...(Params) == sizeof...(Args), "argument count");
  struct Pack {
    std::tuple<Params...> v;
  } pack{std::tuple<Params...>(args...)};
  void *ptrs[sizeof...(Params) > 0 ? sizeof...(Params) : 1];
  std::apply([&](auto &...e) {
    int i = 0;
    ((ptrs[i++] = (void *)&e), ...);
  }, pack.v);
  cudaKernelNodeParams p = {};
  p.func = reinterpret_cast<void *>(func);
  p.gridDim = grid;
  p.blockDim = block;
  p.sharedMemBytes = (unsigned)smem;
  p.kernelParams = ptrs;
  p.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, dep, ndep, &p);
}

// While `s` is being captured into a CUDA graph, append a WHILE node whose body is built by
// body(graph, first_dependency_out...) and make the stream's next captured work depend on it.
// The body must end with k_sp2_loop_tail(handle); the node runs the body at least once per graph
// launch and again while the tail keeps the condition set, with no host involvement.
// Returns cudaSuccess or the first failing call's error.
template <typename BuildBody>
cudaError_t capture_while_loop(cudaStream_t s, BuildBody build_body) {
  cudaStreamCaptureStatus cs;
  unsigned long long id = 0;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t ndeps = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, &id, &g, &deps, &edges, &ndeps);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusActive || g == nullptr) return cudaErrorStreamCaptureInvalidated;
  cudaGraphConditionalHandle handle;
  if ((e = cudaGraphConditionalHandleCreate(&handle, g, 1u, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = handle;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t loop;
  if ((e = cudaGraphAddNode(&loop, g, deps, edges, ndeps, &np)) != cudaSuccess) return e;
  if ((e = build_body(np.conditional.phGraph_out[0], handle)) != cudaSuccess) return e;
  return cudaStreamUpdateCaptureDependencies(s, &loop, nullptr, 1, cudaStreamSetCaptureDependencies);
}

inline bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
}

// grid helpers
inline dim3 ew_grid(const seqm_batch &b) {
  const size_t nn = (size_t)b.max_norb * b.max_norb;
  return dim3((unsigned)((nn + EW_CHUNK - 1) / EW_CHUNK), (unsigned)b.nmol);
}
inline dim3 rows_grid(const seqm_batch &b) { return dim3((unsigned)((b.max_norb + 7) / 8), (unsigned)b.nmol); }
inline dim3 gemm64_grid(const seqm_batch &b) {
  const unsigned t = (unsigned)((b.max_norb + MW_T - 1) / MW_T);
  return dim3(t, t, (unsigned)b.nmol);
}

// ------------------------------------------------------------- FP64-accurate X^2 in FP32 pairs
// GB300 issues FP32 at 64x its FP64 rate, so the one FP64-accurate product of a McWeeny step
// is formed from FP32 pairs (double-float arithmetic; Dekker 1971, Knuth's TwoSum): X = Xh + Xl
// with Xh = fl32(X), Xl = fl32(X - Xh) (|Xl| <= 2^-24 |X|), and
//   X^2 = Xh Xh + (M + M^T) + Xl Xl,   M = Xh Xl  (X symmetric, so Xl Xh = M^T),
// where per term Xh_ik Xh_kj = p + e exactly (p = fl32(product), e = fma(Xh_ik, Xh_kj, -p)) and
// the p's are summed exactly into (s, c) by TwoSum, e and the TwoSum errors summed in FP32 into c
// (10 FP32 instructions per term).  M, a product of relative size 2^-24, is formed on the tensor
// cores as a split product of Xh and 2^24 Xl (error 2^-22 of a 2^-24 term) and added at the end;
// Xl Xl (2^-48) is dropped.  For |X| <= 1 with X^2 ~ X (a density) the result's error is ~K 2^-48
// at most (about 1e-11 for K = 6000, ~1e-13 typically), FP64 level for the McWeeny correction
// D = X^2 - X.
__global__ void __launch_bounds__(EW_THREADS) k_split_pair(seqm_batch b, const double *__restrict__ X,
                                                           float *__restrict__ Xh, float *__restrict__ Xl,
                                                           const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const size_t mo = b.mol_mat_off[m];
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const double x = X[mo + idx];
    const float h = (float)x;
    Xh[mo + idx] = h;
    Xl[mo + idx] = (float)(x - (double)h);
  }
}

// C = Xh Xh (double-float) + M + M^T (symmetric Xh, M in FP32, C in FP64): upper 64 x 64 output
// tiles with their mirror, 256 threads of 4 x 4 outputs, 16-deep K slabs double-buffered in shared
// memory and read along rows of Xh (symmetric), so every global load is coalesced.
constexpr int DF_T = 64, DF_K = 16, DF_THREADS = 256;
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float p) {
  const float t = s + p;
  const float z = t - s;
  c += (s - (t - z)) + (p - z);
  s = t;
}
__global__ void __launch_bounds__(DF_THREADS) k_sym_gemm_pair(seqm_batch b, const float *__restrict__ Xh,
                                                              const float *__restrict__ M, double *__restrict__ Cm,
                                                              const uint8_t *__restrict__ active) {
  const int m = blockIdx.z;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const int i0 = blockIdx.y * DF_T, j0 = blockIdx.x * DF_T;
  if (i0 >= n || j0 >= n || blockIdx.y > blockIdx.x) return;
  const size_t mo = b.mol_mat_off[m];
  const float *H = Xh + mo;
  __shared__ __align__(16) float Ah[2][DF_K][DF_T], Bh[2][DF_K][DF_T];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  // slab loader: element e = threadIdx.x + 256 q (q = 0..3) of the 16 x 64 slab, row e / 64, col e % 64
  float rah[4], rbh[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = threadIdx.x + DF_THREADS * q, kk = e >> 6, c = e & 63;
      const bool kin = k0 + kk < n;
      const size_t ra = (size_t)(k0 + kk) * n + i0 + c, rb = (size_t)(k0 + kk) * n + j0 + c;
      rah[q] = (kin && i0 + c < n) ? H[ra] : 0.0f;
      rbh[q] = (kin && j0 + c < n) ? H[rb] : 0.0f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = threadIdx.x + DF_THREADS * q, kk = e >> 6, c = e & 63;
      Ah[buf][kk][c] = rah[q];
      Bh[buf][kk][c] = rbh[q];
    }
  };
  float s[4][4] = {}, c[4][4] = {};
  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < n; k0 += DF_K) {
    const bool more = k0 + DF_K < n;
    if (more) load(k0 + DF_K);
#pragma unroll 4
    for (int kk = 0; kk < DF_K; ++kk) {
      const float4 ah = *reinterpret_cast<const float4 *>(&Ah[buf][kk][4 * ty]);
      const float4 bh = *reinterpret_cast<const float4 *>(&Bh[buf][kk][4 * tx]);
      const float av[4] = {ah.x, ah.y, ah.z, ah.w}, bv[4] = {bh.x, bh.y, bh.z, bh.w};
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float p = av[r] * bv[q];
          const float e = fmaf(av[r], bv[q], -p);
          two_sum_acc(s[r][q], c[r][q], p);
          c[r][q] += e;
        }
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  double *C = Cm + mo;
  const float *Mm = M + mo;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int row = i0 + 4 * ty + r, col = j0 + 4 * tx + q;
      if (row < n && col < n) {
        const double cross = (double)Mm[(size_t)row * n + col] + (double)Mm[(size_t)col * n + row];
        const double v = (double)s[r][q] + ((double)c[r][q] + cross);
        C[(size_t)row * n + col] = v;
        C[(size_t)col * n + row] = v;
      }
    }
}

inline dim3 pair_gemm_grid(const seqm_batch &b) {
  const unsigned t = (unsigned)((b.max_norb + DF_T - 1) / DF_T);
  return dim3(t, t, (unsigned)b.nmol);
}

// McWeeny step X <- 3 X^2 - 2 X^3 written as X + D (I - 2X) with D = X^2 - X: X^2 FP64-accurate
// gives D exactly, and the correction D (I - 2X), a product of a matrix of the size
// of the idempotency error, is formed at FP32 level (relative error ~1e-7 of a term <= |D|),
// so every step is FP64-accurate at one FP64-accurate product instead of two.
// Df = float(Y - Z), Bf = float(I - 2 Z); with dmax, also max |Df| of each molecule (as the bits
// of a non-negative float, which order like the unsigned integers)
__global__ void __launch_bounds__(EW_THREADS) k_mw_split(seqm_batch b, const double *__restrict__ Y,
                                                         const double *__restrict__ Z, float *__restrict__ Df,
                                                         float *__restrict__ Bf, const uint8_t *__restrict__ active,
                                                         uint32_t *__restrict__ dmax = nullptr) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const size_t mo = b.mol_mat_off[m];
  const DiagTest diagonal(n);
  float mx = 0.0f;
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const double z = Z[mo + idx];
    const float d = (float)(Y[mo + idx] - z);
    Df[mo + idx] = d;
    Bf[mo + idx] = (float)((diagonal((uint32_t)idx) ? 1.0 : 0.0) - 2.0 * z);
    mx = fmaxf(mx, fabsf(d));
  }
  if (!dmax) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(dmax + m, __float_as_uint(mx));
}

// P = 2 (Z + C)
__global__ void __launch_bounds__(EW_THREADS) k_mw_update(seqm_batch b, const double *__restrict__ Z,
                                                          const float *__restrict__ C, double *__restrict__ P,
                                                          const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const size_t mo = b.mol_mat_off[m];
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS)
    P[mo + idx] = 2.0 * (Z[mo + idx] + (double)C[mo + idx]);
}

}  // namespace
}  // namespace seqm
