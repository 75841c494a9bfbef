// SP2 density purification, plain FP64 (SP2.py:9-85 restated per molecule).
//
// X0 = (hN I - F)/(hN - h1) with Gershgorin bounds h1, hN; each step forms X^2
// (batched tiled FP64 GEMM, one grid slice per molecule) and keeps X^2 or
// 2X - X^2, whichever brings the trace closer to nocc; a molecule stops when
// the trace error of the last two steps is below eps.  Each molecule runs at its
// own size (the reference zero-pads the batch to its largest basis).
#include <math.h>

#include "common.cuh"

namespace seqm {

constexpr int NT_S = 256;

template <int NT>
__device__ double sp2_block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < NT / 32; ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  double s = red[0];
  __syncthreads();
  return s;
}

// state per molecule: [0] err0 (this step), [1] err1 (previous), [2] running flag, [3] steps
__global__ void __launch_bounds__(NT_S) k_sp2_init(seqm_batch b, const double *__restrict__ F, double *__restrict__ X,
                                                   double *__restrict__ st, const uint8_t *__restrict__ active) {
  __shared__ double red[NT_S / 32];
  const int m = blockIdx.x;
  double *s = st + 4 * m;
  if (active && !active[m]) {
    if (threadIdx.x == 0) s[2] = 0.0;
    return;
  }
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m];
  const double *Fm = F + mo;
  double *Xm = X + mo;
  double lo = INFINITY, hi = -INFINITY;
  for (int i = threadIdx.x; i < n; i += NT_S) {
    double rsum = 0.0;
    for (int j = 0; j < n; ++j) rsum += fabs(Fm[(size_t)i * n + j]);
    double aii = Fm[(size_t)i * n + i];
    double ri = rsum - fabs(aii);
    lo = fmin(lo, aii - ri);
    hi = fmax(hi, aii + ri);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ double rlo[NT_S / 32], rhi[NT_S / 32];
  if ((threadIdx.x & 31) == 0) { rlo[threadIdx.x >> 5] = lo; rhi[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < NT_S / 32; ++w) { rlo[0] = fmin(rlo[0], rlo[w]); rhi[0] = fmax(rhi[0], rhi[w]); }
  }
  __syncthreads();
  const double h1 = rlo[0], hN = rhi[0];
  double tr = 0.0;
  for (size_t idx = threadIdx.x; idx < (size_t)n * n; idx += NT_S) {
    size_t i = idx / n, j = idx - i * n;
    double v = ((i == j ? hN : 0.0) - Fm[idx]) / (hN - h1);
    Xm[idx] = v;
    if (i == j) tr += v;
  }
  tr = sp2_block_sum<NT_S>(tr, red);
  if (threadIdx.x == 0) {
    double e = fabs(tr - (double)b.mol_nocc[m]);
    s[0] = e;
    s[1] = e;
    s[2] = 1.0;
    s[3] = 0.0;
  }
}

// C = X X for running molecules; 64x64 tiles, 16-deep k slices, 4x4 per thread
constexpr int GT = 64, GK = 16;
__global__ void __launch_bounds__(256) k_sp2_gemm(seqm_batch b, const double *__restrict__ X, double *__restrict__ C,
                                                  const double *__restrict__ st) {
  const int m = blockIdx.z;
  if (st[4 * m + 2] == 0.0) return;
  const int n = b.mol_norb[m];
  const int i0 = blockIdx.y * GT, j0 = blockIdx.x * GT;
  if (i0 >= n || j0 >= n) return;
  const size_t mo = b.mol_mat_off[m];
  const double *Xm = X + mo;
  __shared__ double As[GK][GT + 1], Bs[GK][GT + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < n; k0 += GK) {
    for (int e = threadIdx.x; e < GK * GT; e += 256) {
      int kk = e / GT, ii = e - kk * GT;
      int row = i0 + ii, col = k0 + kk;
      As[kk][ii] = (row < n && col < n) ? Xm[(size_t)row * n + col] : 0.0;
      int krow = k0 + kk, jcol = j0 + ii;
      Bs[kk][ii] = (krow < n && jcol < n) ? Xm[(size_t)krow * n + jcol] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      double a[4], bb[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) bb[c] = Bs[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * bb[c];
    }
    __syncthreads();
  }
  double *Cm = C + mo;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int row = i0 + ty * 4 + r, col = j0 + tx * 4 + c;
      if (row < n && col < n) Cm[(size_t)row * n + col] = acc[r][c];
    }
}

// choose X^2 or 2X - X^2 by the trace test, update the errors and the running flag
__global__ void __launch_bounds__(NT_S) k_sp2_update(seqm_batch b, double *__restrict__ X, const double *__restrict__ X2,
                                                     double *__restrict__ st, double eps, int *__restrict__ running) {
  __shared__ double red[NT_S / 32];
  const int m = blockIdx.x;
  double *s = st + 4 * m;
  if (s[2] == 0.0) return;
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m];
  double *Xm = X + mo;
  const double *X2m = X2 + mo;
  const double nocc = (double)b.mol_nocc[m];
  double t1 = 0.0, t2 = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_S) {
    t1 += Xm[(size_t)i * n + i];
    t2 += X2m[(size_t)i * n + i];
  }
  t1 = sp2_block_sum<NT_S>(t1, red);
  t2 = sp2_block_sum<NT_S>(t2, red);
  const bool sq = fabs(t2 - nocc) < fabs(2.0 * t1 - t2 - nocc);
  double tr = 0.0;
  for (size_t idx = threadIdx.x; idx < (size_t)n * n; idx += NT_S) {
    double v = sq ? X2m[idx] : 2.0 * Xm[idx] - X2m[idx];
    Xm[idx] = v;
    size_t i = idx / n;
    if (idx == i * n + i) tr += v;
  }
  tr = sp2_block_sum<NT_S>(tr, red);
  if (threadIdx.x == 0) {
    double e1 = s[0], e0 = fabs(tr - nocc);
    s[1] = e1;
    s[0] = e0;
    s[3] += 1.0;
    if (e0 < eps && e1 < eps) s[2] = 0.0;
    else atomicAdd(running, 1);
  }
}

__global__ void k_sp2_finish(seqm_batch b, const double *__restrict__ X, double *__restrict__ P,
                             const double *__restrict__ st, const uint8_t *__restrict__ active, int32_t *status) {
  const int m = blockIdx.x;
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m];
  for (size_t idx = threadIdx.x; idx < (size_t)n * n; idx += blockDim.x) P[mo + idx] = 2.0 * X[mo + idx];
  if (threadIdx.x == 0 && status) status[m] = st[4 * m + 2] != 0.0 ? -1 : (int)st[4 * m + 3];
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_density_sp2(const seqm_batch *bp, const double *F, double *P, double *work, double eps,
                                const uint8_t *active, int32_t *status, int max_iter, void *stream) {
  if (!bp || !work) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  eps = eps > 1.0e-3 ? 1.0e-3 : (eps < 1.0e-7 ? 1.0e-7 : eps);  // SP2.py:27-30 (float64)
  int64_t total = 0;
  if (cudaMemcpyAsync(&total, b.mol_mat_off + b.nmol, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return SEQM_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SEQM_E_CUDA;
  double *X = work, *X2 = work + total, *st = work + 2 * total;
  int *running = nullptr;
  if (cudaMallocAsync((void **)&running, sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
  k_sp2_init<<<b.nmol, NT_S, 0, s>>>(b, F, X, st, active);
  dim3 grid((b.max_norb + GT - 1) / GT, (b.max_norb + GT - 1) / GT, b.nmol);
  int rc = SEQM_OK;
  for (int it = 0; it < max_iter; ++it) {
    if (cudaMemsetAsync(running, 0, sizeof(int), s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    k_sp2_gemm<<<grid, 256, 0, s>>>(b, X, X2, st);
    k_sp2_update<<<b.nmol, NT_S, 0, s>>>(b, X, X2, st, eps, running);
    int h = 0;
    if (cudaMemcpyAsync(&h, running, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    if (h == 0) break;
  }
  if (rc == SEQM_OK) {
    k_sp2_finish<<<b.nmol, 256, 0, s>>>(b, X, P, st, active, status);
    rc = launch_check();
  }
  cudaFreeAsync(running, s);
  return rc;
}
