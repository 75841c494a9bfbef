// Batched symmetric eigensolver + closed-shell density (FP64), one CTA per molecule.
//
// Replaces sym_eig_trunc (seqm/seqm_functions/diag.py:110-241), which packs F,
// pads every molecule to the batch's largest basis with shifted diagonal
// entries, calls torch.linalg.eigh and forms P = 2 C_occ C_occ^T per molecule.
// Here each molecule is solved at its own size, so there is no padding.
//
// Algorithm: parallel cyclic Jacobi with the round-robin ("circle") ordering:
// each step rotates n/2 disjoint (p,q) pairs at once.  The matrix A lives in
// shared memory (row stride odd to spread banks); a thread owns a 2x2 block
// (pair i rows) x (pair j cols), applies both one-sided rotations and writes the
// block and its mirror, so every element is touched once per step.  The
// eigenvectors are kept as ROWS of a per-molecule scratch block in global
// memory (L2-resident); warp w rotates rows p,q of pair w with coalesced
// accesses.  Rotations with |a_pq| <= 1e-13 ||A||_F are skipped; the solve stops
// after a sweep without rotations.  Eigenvalues are ranked, and P is formed from
// whichever of the occupied / virtual sets is smaller (P = 2 (I - C_v C_v^T)).
#include <math.h>

#include "common.cuh"

namespace seqm {

constexpr int NT_J = 256;
constexpr int JMAX_N = 160;
constexpr int JMAX_P = JMAX_N / 2;

__global__ void __launch_bounds__(NT_J) k_jacobi(seqm_batch b, const double *__restrict__ F, double *__restrict__ P,
                                                 double *__restrict__ evals, double *__restrict__ evecs,
                                                 double *__restrict__ work, const int64_t *__restrict__ row_off,
                                                 const uint8_t *__restrict__ active, int32_t *__restrict__ status,
                                                 int max_sweeps, const uint8_t *__restrict__ warm) {
  extern __shared__ double A[];
  __shared__ double rc[JMAX_P], rs[JMAX_P], rt[JMAX_P];
  __shared__ int rp[JMAX_P], rq[JMAX_P], rflag[JMAX_P];
  __shared__ double dg[JMAX_N];
  __shared__ int rank[JMAX_N];
  __shared__ double red[NT_J / 32];
  __shared__ int any_rot;

  const int m = b.mol_order[blockIdx.x];
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  if (n <= 0) return;
  const int lda = n | 1;
  const size_t mo = b.mol_mat_off[m];
  const double *Fm = F + mo;
  double *V = work + mo;  // row k = eigenvector k (column k of C)
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  // warm start: V already holds orthonormal rows (the previous SCF step's eigenvectors)
  const bool is_warm = warm != nullptr && warm[m] != 0 && P != nullptr;
  double f2 = 0.0;
  for (int idx = tid; idx < n * n; idx += NT_J) {
    int i = idx / n, j = idx - i * n;
    double v = Fm[idx];
    A[i * lda + j] = v;
    if (!is_warm) V[idx] = i == j ? 1.0 : 0.0;
    f2 += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) f2 += __shfl_xor_sync(0xffffffffu, f2, o);
  if (lane == 0) red[wid] = f2;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < NT_J / 32; ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  const double tol = 1.0e-13 * sqrt(red[0]);

  if (is_warm) {
    // A <- V F V^T in two FP64 products, 4x4 register tiles per thread:
    //   G = V F   (F in shared memory, V rows from L2) -> the P block as temporary
    //   A = G V^T (upper-triangle tiles, mirrored)      -> shared memory
    double *G = P + mo;
    const int nt = (n + 3) >> 2;
    for (int t = tid; t < nt * nt; t += NT_J) {
      const int k0 = (t / nt) * 4, j0 = (t % nt) * 4;
      double acc[4][4] = {};
      for (int i = 0; i < n; ++i) {
        double v[4], f[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = (k0 + r < n) ? V[(size_t)(k0 + r) * n + i] : 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) f[c] = (j0 + c < n) ? A[i * lda + j0 + c] : 0.0;
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] += v[r] * f[c];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (k0 + r < n && j0 + c < n) G[(size_t)(k0 + r) * n + j0 + c] = acc[r][c];
    }
    __syncthreads();
    for (int t = tid; t < nt * nt; t += NT_J) {
      const int kb = t / nt, lb = t % nt;
      if (kb > lb) continue;
      const int k0 = kb * 4, l0 = lb * 4;
      double acc[4][4] = {};
      for (int j = 0; j < n; ++j) {
        double g[4], v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) g[r] = (k0 + r < n) ? G[(size_t)(k0 + r) * n + j] : 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] = (l0 + c < n) ? V[(size_t)(l0 + c) * n + j] : 0.0;
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] += g[r] * v[c];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int k = k0 + r, l = l0 + c;
          if (k < n && l < n && k <= l) {
            A[k * lda + l] = acc[r][c];
            A[l * lda + k] = acc[r][c];
          }
        }
    }
    __syncthreads();
  }

  const int npad = n + (n & 1), np = npad / 2, nsteps = npad - 1;
  int sweeps = -1;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    if (tid == 0) any_rot = 0;
    __syncthreads();
    for (int step = 0; step < nsteps; ++step) {
      // ---- rotations of this step's disjoint pairs
      if (tid < np) {
        int a, c;
        if (tid == 0) { a = npad - 1; c = step; }
        else { a = (step + tid) % (npad - 1); c = (step - tid + npad - 1) % (npad - 1); }
        int p = min(a, c), q = max(a, c);
        rp[tid] = p;
        rq[tid] = q;
        int fl = 0;
        double cc = 1.0, ss = 0.0, tt = 0.0;
        if (q < n) {
          double apq = A[p * lda + q];
          if (fabs(apq) > tol) {
            double app = A[p * lda + p], aqq = A[q * lda + q];
            double theta = (aqq - app) / (2.0 * apq);
            double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
            if (theta < 0.0) t = -t;
            cc = 1.0 / sqrt(t * t + 1.0);
            ss = t * cc;
            tt = t;
            fl = 1;
            any_rot = 1;
          }
        }
        rc[tid] = cc;
        rs[tid] = ss;
        rt[tid] = tt;
        rflag[tid] = fl;
      }
      __syncthreads();
      // ---- A <- J^T A J on 2x2 blocks (i <= j), block and mirror written by one thread
      for (int it = tid; it < np * np; it += NT_J) {
        const int i = it / np, j = it - i * np;
        if (j < i) continue;
        const int fi = rflag[i], fj = rflag[j];
        if (!(fi | fj)) continue;
        const int p = rp[i], q = rq[i];
        if (i == j) {
          const double t = rt[i], apq = A[p * lda + q];
          A[p * lda + p] -= t * apq;
          A[q * lda + q] += t * apq;
          A[p * lda + q] = 0.0;
          A[q * lda + p] = 0.0;
          continue;
        }
        const int r = rp[j], s = rq[j];
        const bool qv = q < n, sv = s < n;
        double x00 = A[p * lda + r];
        double x01 = sv ? A[p * lda + s] : 0.0;
        double x10 = qv ? A[q * lda + r] : 0.0;
        double x11 = (qv && sv) ? A[q * lda + s] : 0.0;
        if (fi) {
          const double c = rc[i], sn = rs[i];
          double y00 = c * x00 - sn * x10, y10 = sn * x00 + c * x10;
          double y01 = c * x01 - sn * x11, y11 = sn * x01 + c * x11;
          x00 = y00; x10 = y10; x01 = y01; x11 = y11;
        }
        if (fj) {
          const double c = rc[j], sn = rs[j];
          double z00 = c * x00 - sn * x01, z01 = sn * x00 + c * x01;
          double z10 = c * x10 - sn * x11, z11 = sn * x10 + c * x11;
          x00 = z00; x01 = z01; x10 = z10; x11 = z11;
        }
        A[p * lda + r] = x00;
        A[r * lda + p] = x00;
        if (sv) { A[p * lda + s] = x01; A[s * lda + p] = x01; }
        if (qv) { A[q * lda + r] = x10; A[r * lda + q] = x10; }
        if (qv && sv) { A[q * lda + s] = x11; A[s * lda + q] = x11; }
      }
      // ---- eigenvector rows p,q: warp per pair, lanes along the row (coalesced)
      for (int i = wid; i < np; i += NT_J / 32) {
        if (!rflag[i]) continue;
        const double c = rc[i], sn = rs[i];
        double *vp = V + (size_t)rp[i] * n, *vq = V + (size_t)rq[i] * n;
        for (int k = lane; k < n; k += 32) {
          double a = vp[k], bq = vq[k];
          vp[k] = c * a - sn * bq;
          vq[k] = sn * a + c * bq;
        }
      }
      __syncthreads();
    }
    if (!any_rot) { sweeps = sweep + 1; break; }
    __syncthreads();
  }
  if (tid == 0 && status) status[m] = sweeps;

  // ---- eigenvalues, ranks (ascending; ties by index)
  for (int k = tid; k < n; k += NT_J) dg[k] = A[k * lda + k];
  __syncthreads();
  for (int k = tid; k < n; k += NT_J) {
    const double d = dg[k];
    int r = 0;
    for (int j = 0; j < n; ++j) r += (dg[j] < d) || (dg[j] == d && j < k);
    rank[k] = r;
  }
  __syncthreads();
  if (evals) {
    double *e = evals + row_off[m];
    for (int k = tid; k < n; k += NT_J) e[rank[k]] = dg[k];
  }
  if (evecs) {
    double *E = evecs + mo;
    for (int idx = tid; idx < n * n; idx += NT_J) {
      int k = idx / n, i = idx - k * n;
      E[(size_t)rank[k] * n + i] = V[idx];
    }
  }
  if (!P) return;
  // ---- density from the smaller of the occupied / virtual sets, staged in shared memory
  const int nocc = b.mol_nocc[m];
  const bool use_occ = nocc <= n - nocc;
  const int nsel = use_occ ? nocc : n - nocc;
  double *U = A;  // nsel rows of length n (A is no longer needed)
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += NT_J) {
    int k = idx / n, i = idx - k * n;
    int r = rank[k];
    int slot = use_occ ? r : r - nocc;
    if (slot >= 0 && slot < nsel) U[slot * n + i] = V[idx];
  }
  __syncthreads();
  double *Pm = P + mo;
  for (int it = tid; it < n * n; it += NT_J) {
    const int a = it / n, c = it - a * n;
    if (c < a) continue;
    double s = 0.0;
    for (int k = 0; k < nsel; ++k) s += U[k * n + a] * U[k * n + c];
    double v = use_occ ? 2.0 * s : (a == c ? 2.0 : 0.0) - 2.0 * s;
    Pm[(size_t)a * n + c] = v;
    Pm[(size_t)c * n + a] = v;
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_density_jacobi(const seqm_batch *bp, const double *F, double *P, double *evals, double *evecs,
                                   double *work, const int64_t *mol_row_off, const uint8_t *active, int32_t *status,
                                   int max_sweeps, const uint8_t *warm, void *stream) {
  if (!bp || !work) return SEQM_E_ARG;
  if (warm && !P) return SEQM_E_ARG;  // a warm start uses P's block as temporary storage
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  if (b.max_norb > JMAX_N) return SEQM_E_TOO_LARGE;
  int lda = b.max_norb | 1;
  size_t smem = (size_t)b.max_norb * lda * sizeof(double);
  if (smem < 8) smem = 8;
  if (cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SEQM_E_CUDA;
  k_jacobi<<<b.nmol, NT_J, smem, (cudaStream_t)stream>>>(b, F, P, evals, evecs, work, mol_row_off, active, status,
                                                         max_sweeps, warm);
  return launch_check();
}

// ---------------------------------------------------------------------------
// Allocation-free variant of seqm_density_jacobi.
//
// Some callers cannot call cudaMalloc: a host program that carves the GPU's memory
// into a fixed pool up front (an MD engine or a long-running serving process that
// owns every byte it hands out), or one that must not stall the device in the middle
// of its pipeline (cudaMalloc/cudaFree synchronise).  For them the eigenvector
// scratch of the Jacobi kernel lives in the fixed device array below instead of a
// caller-provided `work` buffer.  The array is part of this library's image: every
// GPU that loads the library holds these 16 MiB until the process exits.
//
// Limit: the batch's dense matrices must fit, i.e. sum over molecules of norb^2
// <= SEQM_NOALLOC_JACOBI_DOUBLES (2^21 doubles = 16 MiB); larger batches get
// SEQM_E_TOO_LARGE and nothing is launched.
//
// The array is shared by every call and keeps the previous call's contents.  The
// kernel writes every scratch entry it later reads (each molecule's block starts
// from the identity), so no clearing is needed; but two calls that overlap on the
// GPU (different streams, or different host threads) use the same memory and race.
constexpr size_t NOALLOC_DOUBLES = size_t(1) << 21;
static_assert(NOALLOC_DOUBLES == SEQM_NOALLOC_JACOBI_DOUBLES, "header and library disagree on the scratch size");
static __device__ __align__(256) double g_jacobi_scratch[NOALLOC_DOUBLES];

#include <mutex>

namespace {
std::mutex g_scratch_mu;
double *g_scratch_addr[256] = {};  // device address of g_jacobi_scratch, per device ordinal

// Host code may not use g_jacobi_scratch's name as an address: it is a host-side
// stand-in.  Resolve the real device address once per device, with that device
// current, and cache it.
int jacobi_scratch_address(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SEQM_E_CUDA;
  if (dev < 0 || dev >= 256) return SEQM_E_ARG;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_jacobi_scratch) != cudaSuccess || p == nullptr) return SEQM_E_CUDA;
    g_scratch_addr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[dev];
  return SEQM_OK;
}
}  // namespace

extern "C" int seqm_density_jacobi_noalloc(const seqm_batch *bp, const double *F, double *P, double *evals,
                                           double *evecs, const int64_t *mol_row_off, const uint8_t *active,
                                           int32_t *status, int max_sweeps, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  if (b.max_norb > JMAX_N) return SEQM_E_TOO_LARGE;
  cudaStream_t s = (cudaStream_t)stream;
  // total dense-matrix size = mat_off[nmol] (device); one small read, then the size check
  int64_t total = 0;
  if (cudaMemcpyAsync(&total, b.mol_mat_off + b.nmol, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return SEQM_E_CUDA;
  if (total < 0 || (size_t)total > NOALLOC_DOUBLES) return SEQM_E_TOO_LARGE;
  double *work = nullptr;
  int rc = jacobi_scratch_address(&work);
  if (rc != SEQM_OK) return rc;
  int lda = b.max_norb | 1;
  size_t smem = (size_t)b.max_norb * lda * sizeof(double);
  if (smem < 8) smem = 8;
  if (cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SEQM_E_CUDA;
  k_jacobi<<<b.nmol, NT_J, smem, s>>>(b, F, P, evals, evecs, work, mol_row_off, active, status, max_sweeps,
                                      nullptr);
  return launch_check();
}
