// Pulay DIIS converger, per molecule (scf_forward2, seqm/seqm_functions/scf_loop.py:639-1132,
// with its default schedule: no direct or adaptive steps before the Pulay steps).
//
// Per iteration of a still-active molecule, before its density step:
//   ring slot c = (c + 1) mod 10, stored count = min(count + 1, 10)
//   FOCK[c] = F,  R[c] = F P - P F  (the commutator; its largest element is the DIIS error)
//   EMAT row c, columns j < count: <R[c], R[j]> over the upper triangle
//   with >= 2 stored: EVEC = EMAT[:count+1, :count+1] read through its lower triangle (as the
//   reference's eigh does, so entries written before the ring wrapped stay in use), the
//   count x count block divided by EVEC[c][c]; eigen-decomposition; pseudo-inverse over
//   |lambda| > 1e-13; coefficients x_k = -(EVEC^+)[k][count]; F <- sum_k x_k FOCK[k];
//   condition number max|lambda| / min|lambda| > 1e7 resets the history after the iteration.
// After the density step: P <- P/2 + Pnew/2 while fewer than 2 are stored, else P <- Pnew.
// The convergence test adds max |F P - P F| <= 50 eps (scf_loop.py:130-132).
//
// The reference keeps one ring counter for the whole batch and resets every molecule when any
// one is ill-conditioned; here each molecule has its own counter and reset, so a molecule's
// SCF does not depend on its batch mates (its trajectory is the reference's for the molecule
// run alone).
#include <math.h>

#include "common.cuh"
#include "sp2_common.cuh"

namespace seqm {
namespace {

constexpr int DN = 10;                 // history depth (nFock)
constexpr int DM = DN + 1;             // EMAT order
constexpr int ST_COUNTER = 0, ST_COUNT = 1, ST_RESET = 2, ST_EMAT = 3;
constexpr int DIIS_NS = ST_EMAT + DM * DM;
static_assert(DIIS_NS == SEQM_DIIS_STATE, "header and library disagree on the DIIS state size");
constexpr int NT_D = 512;

__device__ __forceinline__ bool live(const uint8_t *active, int m) { return active == nullptr || active[m]; }

// EMAT after a (re)start: the lower triangle of (I - 1)
__device__ __forceinline__ void emat_fresh(double *E) {
  for (int i = 0; i < DM; ++i)
    for (int j = 0; j < DM; ++j) E[i * DM + j] = i > j ? -1.0 : 0.0;
}

__global__ void k_diis_init(int nmol, double *__restrict__ st, double *__restrict__ derr) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmol) return;
  double *s = st + (size_t)DIIS_NS * m;
  s[ST_COUNTER] = -1.0;
  s[ST_COUNT] = 0.0;
  s[ST_RESET] = 0.0;
  emat_fresh(s + ST_EMAT);
  derr[m] = 1.0e308;
}

// apply a pending reset, advance the ring, count the iteration
__global__ void k_diis_advance(int nmol, double *__restrict__ st, const uint8_t *__restrict__ active,
                               int32_t *__restrict__ iters) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmol || !live(active, m)) return;
  double *s = st + (size_t)DIIS_NS * m;
  if (s[ST_RESET] != 0.0) {
    s[ST_COUNTER] = -1.0;
    s[ST_COUNT] = 0.0;
    s[ST_RESET] = 0.0;
    emat_fresh(s + ST_EMAT);
  }
  s[ST_COUNTER] = (double)(((int)s[ST_COUNTER] + 1) % DN);
  s[ST_COUNT] = fmin(s[ST_COUNT] + 1.0, (double)DN);
  if (iters) iters[m] += 1;
}

template <int NV>
__device__ void block_reduce_vec(double *v, double *red /* [NT_D/32][NV] */, bool is_max_first) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, x, o);
      x = (is_max_first && q == 0) ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[warp * NV + q] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    const int q = threadIdx.x;
    double x = red[q];
    for (int w = 1; w < NT_D / 32; ++w) x = (is_max_first && q == 0) ? fmax(x, red[w * NV + q]) : x + red[w * NV + q];
    red[q] = x;  // warp 0's slots hold the results (read after the next barrier)
  }
  __syncthreads();
}

// store FOCK[c] = F and R[c] = G - G^T (G = F P), the DIIS error and the EMAT row c; one CTA
// per molecule, reductions in a fixed order
__global__ void __launch_bounds__(NT_D) k_diis_store(seqm_batch b, const double *__restrict__ F,
                                                     const double *__restrict__ G, double *__restrict__ hist,
                                                     int64_t T, double *__restrict__ st, double *__restrict__ derr,
                                                     const uint8_t *__restrict__ active) {
  __shared__ double red[(NT_D / 32) * (DN + 1)];
  const int m = blockIdx.x;
  if (!live(active, m)) return;
  double *s = st + (size_t)DIIS_NS * m;
  const int c = (int)s[ST_COUNTER], cnt = (int)s[ST_COUNT];
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m], nn = (size_t)n * n;
  double *Fh = hist, *Rh = hist + (size_t)DN * T;
  double acc[DN + 1];  // [0] max |R|, [1 + j] <R_c, R_j> over the full matrix
#pragma unroll
  for (int q = 0; q <= DN; ++q) acc[q] = 0.0;
  for (size_t idx = threadIdx.x; idx < nn; idx += NT_D) {
    const size_t i = idx / n, j = idx - i * n;
    const double r = G[mo + idx] - G[mo + j * n + i];
    Fh[(size_t)c * T + mo + idx] = F[mo + idx];
    Rh[(size_t)c * T + mo + idx] = r;
    acc[0] = fmax(acc[0], fabs(r));
#pragma unroll
    for (int q = 0; q < DN; ++q)
      if (q < cnt) acc[1 + q] += r * (q == c ? r : Rh[(size_t)q * T + mo + idx]);
  }
  block_reduce_vec<DN + 1>(acc, red, true);
  if (threadIdx.x == 0) {
    derr[m] = red[0];
    // the reference's dot runs over the upper triangle; R is antisymmetric with a zero diagonal
    for (int q = 0; q < cnt; ++q) s[ST_EMAT + c * DM + q] = 0.5 * red[1 + q];
  }
}

// cyclic Jacobi eigen-decomposition of a small symmetric matrix (row-major, order k <= DM)
__device__ void small_eig(double *A, double *Q, int k) {
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) Q[i * DM + j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) {
        const double a = A[i * DM + j] * A[i * DM + j];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1.0e-32 * tot) break;
    for (int p = 0; p < k - 1; ++p)
      for (int q = p + 1; q < k; ++q) {
        const double apq = A[p * DM + q];
        if (apq == 0.0) continue;
        const double theta = (A[q * DM + q] - A[p * DM + p]) / (2.0 * apq);
        double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
        if (theta < 0.0) t = -t;
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < k; ++r) {  // A <- A J
          const double x = A[r * DM + p], y = A[r * DM + q];
          A[r * DM + p] = cs * x - sn * y;
          A[r * DM + q] = sn * x + cs * y;
        }
        for (int r = 0; r < k; ++r) {  // A <- J^T A
          const double x = A[p * DM + r], y = A[q * DM + r];
          A[p * DM + r] = cs * x - sn * y;
          A[q * DM + r] = sn * x + cs * y;
        }
        for (int r = 0; r < k; ++r) {  // Q <- Q J (columns are eigenvectors)
          const double x = Q[r * DM + p], y = Q[r * DM + q];
          Q[r * DM + p] = cs * x - sn * y;
          Q[r * DM + q] = sn * x + cs * y;
        }
      }
  }
}

// F <- sum_k x_k FOCK[k] with the DIIS coefficients (molecules with >= 2 stored)
__global__ void __launch_bounds__(NT_D) k_diis_extrapolate(seqm_batch b, double *__restrict__ F,
                                                           const double *__restrict__ hist, int64_t T,
                                                           double *__restrict__ st,
                                                           const uint8_t *__restrict__ active) {
  __shared__ double A[DM * DM], Q[DM * DM], x[DN];
  const int m = blockIdx.x;
  if (!live(active, m)) return;
  double *s = st + (size_t)DIIS_NS * m;
  const int c = (int)s[ST_COUNTER], cnt = (int)s[ST_COUNT];
  if (cnt < 2) return;
  if (threadIdx.x == 0) {
    const int k = cnt + 1;
    const double *E = s + ST_EMAT;
    const double denom = fmax(E[c * DM + c], 1.0e-15);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j <= i; ++j) {
        double v = E[i * DM + j];
        if (i < cnt && j < cnt) v /= denom;
        A[i * DM + j] = v;
        A[j * DM + i] = v;
      }
    small_eig(A, Q, k);
    double amax = 0.0, amin = INFINITY;
    for (int i = 0; i < k; ++i) {
      amax = fmax(amax, fabs(A[i * DM + i]));
      amin = fmin(amin, fabs(A[i * DM + i]));
    }
    if (!(amin > 0.0) || amax / amin > 1.0e7) s[ST_RESET] = 1.0;
    for (int r = 0; r < cnt; ++r) {
      double v = 0.0;
      for (int i = 0; i < k; ++i) {
        const double l = A[i * DM + i];
        if (fabs(l) > 1.0e-13) v += Q[r * DM + i] * Q[(k - 1) * DM + i] / l;
      }
      x[r] = -v;
    }
  }
  __syncthreads();
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m], nn = (size_t)n * n;
  for (size_t idx = threadIdx.x; idx < nn; idx += NT_D) {
    double v = 0.0;
    for (int r = 0; r < cnt; ++r) v += x[r] * hist[(size_t)r * T + mo + idx];
    F[mo + idx] = v;
  }
}

// P <- P/2 + Pnew/2 (fewer than 2 stored) or Pnew; Pold <- P
__global__ void __launch_bounds__(EW_THREADS) k_diis_mix(seqm_batch b, double *__restrict__ P,
                                                         const double *__restrict__ Pnew, double *__restrict__ Pold,
                                                         const double *__restrict__ st,
                                                         const uint8_t *__restrict__ active) {
  const int m = blockIdx.y;
  if (!live(active, m)) return;
  const int n = b.mol_norb[m];
  const size_t nn = (size_t)n * n, base = (size_t)blockIdx.x * EW_CHUNK;
  if (base >= nn) return;
  const bool lin = st[(size_t)DIIS_NS * m + ST_COUNT] < 2.0;
  const size_t mo = b.mol_mat_off[m];
  for (size_t idx = base + threadIdx.x; idx < nn && idx < base + EW_CHUNK; idx += EW_THREADS) {
    const double p = P[mo + idx];
    Pold[mo + idx] = p;
    P[mo + idx] = lin ? 0.5 * p + 0.5 * Pnew[mo + idx] : Pnew[mo + idx];
  }
}

int64_t matrix_total(const seqm_batch &b, cudaStream_t s, int *rc) {
  int64_t total = 0;
  if (batch_total(b, s, &total) != SEQM_OK) *rc = SEQM_E_CUDA;
  return total;
}

}  // namespace
}  // namespace seqm

using namespace seqm;

extern "C" int seqm_diis_init(const seqm_batch *bp, double *state, double *diis_err, void *stream) {
  if (!bp || !state || !diis_err) return SEQM_E_ARG;
  const seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  k_diis_init<<<(b.nmol + 127) / 128, 128, 0, (cudaStream_t)stream>>>(b.nmol, state, diis_err);
  return launch_check();
}

extern "C" int seqm_diis_extrapolate(const seqm_batch *bp, double *F, const double *P, double *hist, double *state,
                                     double *diis_err, const uint8_t *active, int32_t *iters, void *stream) {
  if (!bp || !F || !P || !hist || !state || !diis_err) return SEQM_E_ARG;
  const seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  if (b.nmol > 65535) return SEQM_E_TOO_LARGE;  // molecules are a grid dimension of the product
  cudaStream_t s = (cudaStream_t)stream;
  int rc = SEQM_OK;
  const int64_t T = matrix_total(b, s, &rc);
  if (rc != SEQM_OK) return rc;
  double *G = hist + (size_t)2 * DN * T;  // F P
  k_diis_advance<<<(b.nmol + 127) / 128, 128, 0, s>>>(b.nmol, state, active, iters);
  k_sym_gemm<double, true><<<gemm64_grid(b), MW_THREADS, 0, s>>>(b, F, P, G, active, nullptr);
  k_diis_store<<<b.nmol, NT_D, 0, s>>>(b, F, G, hist, T, state, diis_err, active);
  k_diis_extrapolate<<<b.nmol, NT_D, 0, s>>>(b, F, hist, T, state, active);
  return launch_check();
}

extern "C" int seqm_diis_mix(const seqm_batch *bp, double *P, const double *Pnew, double *Pold, const double *state,
                             const uint8_t *active, void *stream) {
  if (!bp || !P || !Pnew || !Pold || !state) return SEQM_E_ARG;
  const seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  k_diis_mix<<<ew_grid(b), EW_THREADS, 0, (cudaStream_t)stream>>>(b, P, Pnew, Pold, state, active);
  return launch_check();
}
