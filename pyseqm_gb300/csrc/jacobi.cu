// Batched symmetric eigensolver + closed-shell density, one CTA per molecule.
//
// Replaces sym_eig_trunc (seqm/seqm_functions/diag.py:110-241), which packs F,
// pads every molecule to the batch's largest basis with shifted diagonal
// entries, calls torch.linalg.eigh and forms P = 2 C_occ C_occ^T per molecule.
// Here each molecule is solved at its own size, so there is no padding.
//
// Algorithm: parallel cyclic Jacobi with the round-robin ("circle") ordering:
// each step rotates n/2 disjoint (p,q) pairs at once.  A lives in shared memory
// (odd row stride); a thread owns a 2x2 block (pair i rows) x (pair j cols),
// applies both one-sided rotations and writes the block and its mirror, so every
// element is touched once per step.  Eigenvector ROWS are rotated by one warp per
// pair with coalesced accesses.  A sweep starts only if max |a_pq| > tol, and
// rotations with |a_pq| <= tol are skipped.
//
// GB300's FP64 rate is ~1/64 of FP32, so the sweeps that only need to bring the
// off-diagonal down to ~1e-6 run in FP32 when that pays:
//   warm start (previous SCF step's eigenvector rows V in `work`): A = V F V^T;
//   cold start: A = F, V = I.
//   If cold, or the previous call needed >= mixed_threshold sweeps:
//     FP32 Jacobi on (float)A accumulating W (both in shared memory),
//     V <- W V in FP64, one Newton-Schulz step V <- 1.5 V - 0.5 (V V^T) V
//     (restores orthonormality from ~1e-6 to ~1e-12), A = V F V^T again;
//   FP64 polish sweeps to max |a_pq| <= 1e-13 ||F||_F.
// Eigenvalues are ranked, and P is formed from whichever of the occupied /
// virtual sets is smaller (P = 2 (I - C_v C_v^T)).
#include <math.h>

#include <atomic>

#include <type_traits>

#include "common.cuh"

namespace seqm {

constexpr int NT_J = 512;  // threads of the largest CTAs; smaller molecules run in smaller CTAs
#define NTB ((int)blockDim.x)
#define NTB_W ((int)(blockDim.x >> 5))
constexpr int JMAX_N = 160;
constexpr int JMAX_P = JMAX_N / 2;

struct JShared {
  double rc[JMAX_P], rs[JMAX_P], rt[JMAX_P], rdp[JMAX_P], rdq[JMAX_P];
  int rp[JMAX_P], rq[JMAX_P], rflag[JMAX_P];
  double red[NT_J / 32];
};

__device__ double jblock_reduce(double v, double *red, bool is_max) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : v + u;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = red[0];
  for (int w = 1; w < NTB_W; ++w) s = is_max ? fmax(s, red[w]) : s + red[w];
  __syncthreads();
  return s;
}

// 4x4-register-tile product out(k, j) <- sum_l L(k, l) R(l, j), k, j < n (upper tiles only if
// asked), accumulated in T
template <class T, class LF, class RF, class OF>
__device__ void tile_product_t(int n, bool upper_only, LF L, RF R, OF out) {
  const int nt = (n + 3) >> 2;
  for (int t = threadIdx.x; t < nt * nt; t += NTB) {
    const int kb = t / nt, jb = t % nt;
    if (upper_only && kb > jb) continue;
    const int k0 = kb * 4, j0 = jb * 4;
    T acc[4][4] = {};
#pragma unroll 2
    for (int l = 0; l < n; ++l) {
      T a[4], c[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = (k0 + r < n) ? L(k0 + r, l) : T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) c[q] = (j0 + q < n) ? R(l, j0 + q) : T(0);
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] += a[r] * c[q];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (k0 + r < n && j0 + q < n) out(k0 + r, j0 + q, acc[r][q]);
  }
}

template <class LF, class RF, class OF>
__device__ void tile_product(int n, bool upper_only, LF L, RF R, OF out) {
  tile_product_t<double>(n, upper_only, L, R, out);
}

// 4x4-register-tile product out(k, j) <- sum_l L(k, l) R(l, j) for k < M, j < N, l < K,
// accumulated in T; with upper_only (M == N) only the tiles on or above the diagonal
template <class T, class LF, class RF, class OF>
__device__ void tile_product_mnk_t(int M, int N, int K, bool upper_only, LF L, RF R, OF out) {
  const int mt = (M + 3) >> 2, nt = (N + 3) >> 2;
  for (int t = threadIdx.x; t < mt * nt; t += NTB) {
    const int kb = t / nt, jb = t % nt;
    if (upper_only && kb > jb) continue;
    const int k0 = kb * 4, j0 = jb * 4;
    T acc[4][4] = {};
#pragma unroll 2
    for (int l = 0; l < K; ++l) {
      T a[4], c[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = (k0 + r < M) ? L(k0 + r, l) : T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) c[q] = (j0 + q < N) ? R(l, j0 + q) : T(0);
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] += a[r] * c[q];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (k0 + r < M && j0 + q < N) out(k0 + r, j0 + q, acc[r][q]);
  }
}

template <class LF, class RF, class OF>
__device__ void tile_product_mnk(int M, int N, int K, LF L, RF R, OF out) {
  tile_product_mnk_t<double>(M, N, K, false, L, R, out);
}

// ------------------------------------------------- FP64-accurate products on the FP32 pipe
// GB300 retires FP32 at ~64x its FP64 rate (and converts between them on the FP64 pipe), so
// the density step's FP64-accurate products run as double-float arithmetic (Dekker 1971;
// Knuth's TwoSum): each FP64 operand is split into FP32 hi + lo with integer instructions only,
// each term a*b = p + e exactly (p = fl32(ah bh), e = fma(ah, bh, -p)) plus the FP32 cross terms
// ah bl + al bh, the p's summed exactly into (s, c) by TwoSum and the rest into c.  Error
// ~K 2^-48 relative at most (K the summation length), FP64 level for these products, at about
// 13 FP32 and ~12 integer instructions per term instead of one FP64 FMA.

// x = hi + lo, hi = x's sign, exponent and top 23 mantissa bits (truncated), lo = the remaining
// 29 bits rounded to FP32 (together ~48 bits); integer instructions and one int-to-float
// conversion, no FP64 pipe.  |x| below 2^-126 gives 0 (far below every term that matters here).
__device__ __forceinline__ void split_f64(double x, float &hi, float &lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned int top = (unsigned int)(u >> 32), sign = top & 0x80000000u;
  const int E = (int)((top >> 20) & 0x7FFu) - 1023 + 127;  // FP32 exponent field of x
  if (E <= 0) { hi = 0.0f; lo = 0.0f; return; }
  if (E >= 255) { hi = __double2float_rn(x); lo = 0.0f; return; }  // beyond FP32 range (not expected)
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  hi = __uint_as_float(sign | ((unsigned int)E << 23) | (unsigned int)(m >> 29));
  const unsigned int r = (unsigned int)(m & 0x1FFFFFFFull);  // x - hi = r 2^(e - 1075)
  const float scale = E > 52 ? __uint_as_float((unsigned int)(E - 52) << 23) : 0.0f;
  const float l = __uint2float_rn(r) * scale;
  lo = sign ? -l : l;
}

__device__ __forceinline__ void split_val(double x, float &hi, float &lo) { split_f64(x, hi, lo); }
// an operand already split into FP32 hi + lo (split once where it is produced)
struct DFPair {
  float h, l;
};
__device__ __forceinline__ void split_val(DFPair x, float &hi, float &lo) {
  hi = x.h;
  lo = x.l;
}
__device__ __forceinline__ void split_val(float x, float &hi, float &lo) {
  hi = x;
  lo = 0.0f;
}

__device__ __forceinline__ void two_sum_acc(float &s, float &c, float p) {
  const float t = s + p;
  const float z = t - s;
  c += (s - (t - z)) + (p - z);
  s = t;
}

// out(k, j) <- sum_l L(k, l) R(l, j) for k < M, j < N, l < K, 4x4 register tiles, FP64-accurate
// from double-float arithmetic (above); L and R return doubles (split on load) or floats (exact
// FP32 values, lo = 0: the terms are then exact before the summation); out receives a double.
template <class LF, class RF, class OF>
__device__ void tile_product_df(int M, int N, int K, bool upper_only, LF L, RF R, OF out) {
  const int mt = (M + 3) >> 2, nt = (N + 3) >> 2;
  for (int t = threadIdx.x; t < mt * nt; t += NTB) {
    const int kb = t / nt, jb = t % nt;
    if (upper_only && kb > jb) continue;
    const int k0 = kb * 4, j0 = jb * 4;
    float s[4][4] = {}, c[4][4] = {};
#pragma unroll 2
    for (int l = 0; l < K; ++l) {
      float ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        if (k0 + r < M) split_val(L(k0 + r, l), ah[r], al[r]);
        else ah[r] = al[r] = 0.0f;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (j0 + q < N) split_val(R(l, j0 + q), bh[q], bl[q]);
        else bh[q] = bl[q] = 0.0f;
      }
      // exact FP32 operands (both lo parts zero) need no cross terms
      constexpr bool exact = std::is_same<decltype(L(0, 0)), float>::value &&
                             std::is_same<decltype(R(0, 0)), float>::value;
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float p = ah[r] * bh[q];
          const float e = fmaf(ah[r], bh[q], -p);
          two_sum_acc(s[r][q], c[r][q], p);
          if (exact) {
            c[r][q] += e;
          } else {
            const float x = fmaf(ah[r], bl[q], al[r] * bh[q]);
            c[r][q] += e + x;
          }
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (k0 + r < M && j0 + q < N) out(k0 + r, j0 + q, (double)s[r][q] + (double)c[r][q]);
  }
}

// A (shared, holding F on entry) <- V F V^T; G (global n x n) is scratch
// (pair: FP64-accurate double-float products on the FP32 pipe, else FP64 products)
__device__ void form_vfvt(double *A, int lda, const double *V, double *G, int n, bool pair) {
  auto L1 = [&](int k, int l) { return V[(size_t)k * n + l]; };
  auto R1 = [&](int l, int j) { return A[l * lda + j]; };
  auto O1 = [&](int k, int j, double v) { G[(size_t)k * n + j] = v; };
  if (pair) tile_product_df(n, n, n, false, L1, R1, O1);
  else tile_product(n, false, L1, R1, O1);
  __syncthreads();
  auto L2 = [&](int k, int j) { return G[(size_t)k * n + j]; };
  auto R2 = [&](int j, int l) { return V[(size_t)l * n + j]; };
  auto O2 = [&](int k, int l, double v) {
    if (k <= l) { A[k * lda + l] = v; A[l * lda + k] = v; }
  };
  if (pair) tile_product_df(n, n, n, true, L2, R2, O2);
  else tile_product(n, true, L2, R2, O2);
  __syncthreads();
}

// A32 (float, shared, overlaying A) <- V F V^T in FP32 from V and F (global, FP64).  Both
// operands of the first product are converted once into A's shared space (F32 in the half A32
// takes, V^T in the other) so that the products read FP32 operands from shared memory
// (conversions to and from FP64 issue on the FP64 pipe); V F goes to G (global scratch, floats),
// and V F V^T overwrites F32, which is dead by then.  A's FP64 contents are not used.  Input to
// FP32 sweeps, which need no more precision.
__device__ void form_vfvt32(double *A, int lda, const double *V, const double *Fm, double *G, int n) {
  float *A32 = reinterpret_cast<float *>(A), *F32 = A32, *V32T = A32 + (size_t)n * lda;
  float *T32 = reinterpret_cast<float *>(G);
  for (int idx = threadIdx.x; idx < n * n; idx += NTB) {
    const int i = idx / n, j = idx - i * n;
    V32T[j * n + i] = (float)V[idx];
    F32[idx] = (float)Fm[idx];
  }
  __syncthreads();
  tile_product_t<float>(
      n, false, [&](int k, int l) { return V32T[l * n + k]; }, [&](int l, int j) { return F32[l * n + j]; },
      [&](int k, int j, float v) { T32[k * n + j] = v; });
  __syncthreads();
  tile_product_t<float>(
      n, true, [&](int k, int j) { return T32[k * n + j]; }, [&](int j, int l) { return V32T[j * n + l]; },
      [&](int k, int l, float v) {
        if (k <= l) { A32[k * lda + l] = v; A32[l * lda + k] = v; }
      });
  __syncthreads();
}

template <class T>
__device__ double offdiag_max(const T *A, int lda, int n, double *red) {
  T mx = T(0);
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x >> 5; i < n; i += NTB_W)
    for (int j = lane; j < n; j += 32)
      if (i != j) mx = fmax(mx, fabs(A[i * lda + j]));
  return jblock_reduce((double)mx, red, true);
}

// Jacobi sweeps on A (shared memory, stride lda) accumulating the rotations into the
// rows of V (stride n, shared or global).  Returns the sweeps performed, or -1 if
// max |a_pq| > tol after max_sweeps.  With ratio > 0 only the pairs whose coupling exceeds
// ratio times their diagonal splitting rotate (a selective sweep).
template <class T>
__device__ int jacobi_solve(T *A, int lda, T *V, int n, double tol, int max_sweeps, JShared &sh,
                            double ratio = 0.0) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int npad = n + (n & 1), np = npad / 2, nsteps = npad - 1;
  const T ttol = (T)tol, tratio = (T)ratio;
  // rotation parameters kept in the arithmetic type (a conversion from or to FP64 issues on
  // the FP64 pipe), in the shared arrays' storage
  T *rc = reinterpret_cast<T *>(sh.rc), *rs = reinterpret_cast<T *>(sh.rs), *rt = reinterpret_cast<T *>(sh.rt);
  T *rdp = reinterpret_cast<T *>(sh.rdp), *rdq = reinterpret_cast<T *>(sh.rdq);  // rotated diagonal
  // FP32 path: this warp's rotations of a step, slots wid, wid + warps, ... (<= 32 for every
  // launch class: np <= 16 at 2 warps, <= 32 at 4, <= 80 at 8 or more)
  const int nrot = np > wid ? (np - wid + NTB_W - 1) / NTB_W : 0;
  for (int sweep = 0; sweep <= max_sweeps; ++sweep) {
    if (offdiag_max(A, lda, n, sh.red) <= tol) return sweep;
    if (sweep == max_sweeps) break;
    for (int step = 0; step < nsteps; ++step) {
      if constexpr (sizeof(T) == 8) {
      if (tid < np) {
        // round-robin partners of slot tid at this step (no integer division)
        int a = npad - 1, c = step;
        if (tid != 0) {
          a = step + tid;
          if (a >= npad - 1) a -= npad - 1;
          c = step - tid;
          if (c < 0) c += npad - 1;
        }
        const int p = min(a, c), q = max(a, c);
        sh.rp[tid] = p;
        sh.rq[tid] = q;
        int fl = 0;
        T cc = 1, ss = 0, tt = 0;
        if (q < n) {
          const T apq = A[p * lda + q], app = A[p * lda + p], aqq = A[q * lda + q];
          if (fabs(apq) > ttol && (tratio == T(0) || fabs(apq) > tratio * fabs(aqq - app))) {
            const T theta = (aqq - app) / (T(2) * apq);
            T t = T(1) / (fabs(theta) + sqrt(theta * theta + T(1)));
            if (theta < T(0)) t = -t;
            cc = T(1) / sqrt(t * t + T(1));
            ss = t * cc;
            tt = t;
            fl = 1;
          }
        }
        rc[tid] = cc;
        rs[tid] = ss;
        rt[tid] = tt;
        if (fl) {
          rdp[tid] = A[p * lda + p] - tt * A[p * lda + q];
          rdq[tid] = A[q * lda + q] + tt * A[p * lda + q];
        }
        sh.rflag[tid] = fl;
      }
      __syncthreads();
      }
      if constexpr (sizeof(T) == 4) {
        // FP32: A <- J^T A J as a row pass (rows p, q of A and of V, lanes along the rows) and a
        // column pass (columns p, q of A, lanes down the columns; the odd stride keeps them
        // conflict-free); the pass writes the rotated 2x2 block exactly (a_pq = 0).  Every warp
        // computes the parameters of its own rotations (slots wid, wid + warps, ...; lane k the
        // k-th) and hands them to its lanes by shuffles, so a step takes two barriers and no
        // shared-memory round trip for them (a rotation's pivots lie in its own two rows, which no
        // other warp touches before the row pass).  Above 96 basis functions each lane loads all
        // of its (at most JMAX_N / 32) elements of the two rows or columns before it stores any
        // (the rows are disjoint, but only this order lets the loads overlap; measured 11-28 %
        // faster there); smaller molecules, whose lanes hold at most three elements, keep the
        // plain loop (the unrolled form was slower for them)
        constexpr int KL = (JMAX_N + 31) / 32;
        constexpr unsigned FULL = 0xffffffffu;
        const bool wide = n > 96;
        int mp = 0, mq = 0, mfl = 0;
        T mc = 1, ms = 0, mdp = 0, mdq = 0;
        if (lane < nrot) {
          const int slot = wid + NTB_W * lane;
          int a = npad - 1, c = step;
          if (slot != 0) {
            a = step + slot;
            if (a >= npad - 1) a -= npad - 1;
            c = step - slot;
            if (c < 0) c += npad - 1;
          }
          mp = min(a, c);
          mq = max(a, c);
          if (mq < n) {
            const T apq = A[mp * lda + mq], app = A[mp * lda + mp], aqq = A[mq * lda + mq];
            if (fabs(apq) > ttol && (tratio == T(0) || fabs(apq) > tratio * fabs(aqq - app))) {
              const T theta = (aqq - app) / (T(2) * apq);
              T t = T(1) / (fabs(theta) + sqrt(theta * theta + T(1)));
              if (theta < T(0)) t = -t;
              mc = T(1) / sqrt(t * t + T(1));
              ms = t * mc;
              mdp = app - t * apq;
              mdq = aqq + t * apq;
              mfl = 1;
            }
          }
        }
        for (int k = 0; k < nrot; ++k) {
          if (!__shfl_sync(FULL, mfl, k)) continue;  // uniform over the warp
          const int p = __shfl_sync(FULL, mp, k), q = __shfl_sync(FULL, mq, k);
          const T c = __shfl_sync(FULL, mc, k), sn = __shfl_sync(FULL, ms, k);
          T *ap = A + p * lda, *aq = A + q * lda;
          T *vp = V + (size_t)p * n, *vq = V + (size_t)q * n;
          if (wide) {
            T a[KL], b[KL], e[KL], f[KL];
#pragma unroll
            for (int u = 0; u < KL; ++u) {
              const int kk = lane + 32 * u;
              if (kk < n) {
                a[u] = ap[kk];
                b[u] = aq[kk];
                e[u] = vp[kk];
                f[u] = vq[kk];
              }
            }
#pragma unroll
            for (int u = 0; u < KL; ++u) {
              const int kk = lane + 32 * u;
              if (kk < n) {
                ap[kk] = c * a[u] - sn * b[u];
                aq[kk] = sn * a[u] + c * b[u];
                vp[kk] = c * e[u] - sn * f[u];
                vq[kk] = sn * e[u] + c * f[u];
              }
            }
          } else {
            for (int kk = lane; kk < n; kk += 32) {
              const T a = ap[kk], b = aq[kk], e = vp[kk], f = vq[kk];
              ap[kk] = c * a - sn * b;
              aq[kk] = sn * a + c * b;
              vp[kk] = c * e - sn * f;
              vq[kk] = sn * e + c * f;
            }
          }
        }
        __syncthreads();
        for (int k = 0; k < nrot; ++k) {
          if (!__shfl_sync(FULL, mfl, k)) continue;
          const int p = __shfl_sync(FULL, mp, k), q = __shfl_sync(FULL, mq, k);
          const T c = __shfl_sync(FULL, mc, k), sn = __shfl_sync(FULL, ms, k);
          const T dp = __shfl_sync(FULL, mdp, k), dq = __shfl_sync(FULL, mdq, k);
          if (wide) {
            T a[KL], b[KL];
#pragma unroll
            for (int u = 0; u < KL; ++u) {
              const int kk = lane + 32 * u;
              if (kk < n) {
                a[u] = A[kk * lda + p];
                b[u] = A[kk * lda + q];
              }
            }
#pragma unroll
            for (int u = 0; u < KL; ++u) {
              const int kk = lane + 32 * u;
              if (kk < n) {
                T xp = c * a[u] - sn * b[u], xq = sn * a[u] + c * b[u];
                if (kk == p) { xp = dp; xq = T(0); }
                if (kk == q) { xp = T(0); xq = dq; }
                A[kk * lda + p] = xp;
                A[kk * lda + q] = xq;
              }
            }
          } else {
            for (int kk = lane; kk < n; kk += 32) {
              const T a = A[kk * lda + p], b = A[kk * lda + q];
              T xp = c * a - sn * b, xq = sn * a + c * b;
              if (kk == p) { xp = dp; xq = T(0); }
              if (kk == q) { xp = T(0); xq = dq; }
              A[kk * lda + p] = xp;
              A[kk * lda + q] = xq;
            }
          }
        }
        __syncthreads();
        continue;
      }
      if constexpr (sizeof(T) == 8) {
        // A <- J^T A J on 2x2 blocks (pair i rows, pair j cols, i <= j): block row i per warp,
        // lanes along j; each block and its mirror written by one thread
        for (int i = wid; i < np; i += NTB_W) {
          const int fi = sh.rflag[i];
          const int p = sh.rp[i], q = sh.rq[i];
          const bool qv = q < n;
          const T ci = rc[i], si = rs[i];
          for (int j = i + lane; j < np; j += 32) {
            const int fj = sh.rflag[j];
            if (!(fi | fj)) continue;
            if (j == i) {
              const T t = rt[i], apq = A[p * lda + q];
              A[p * lda + p] -= t * apq;
              A[q * lda + q] += t * apq;
              A[p * lda + q] = T(0);
              A[q * lda + p] = T(0);
              continue;
            }
            const int r = sh.rp[j], s = sh.rq[j];
            const bool sv = s < n;
            T x00 = A[p * lda + r];
            T x01 = sv ? A[p * lda + s] : T(0);
            T x10 = qv ? A[q * lda + r] : T(0);
            T x11 = (qv && sv) ? A[q * lda + s] : T(0);
            if (fi) {
              T y00 = ci * x00 - si * x10, y10 = si * x00 + ci * x10;
              T y01 = ci * x01 - si * x11, y11 = si * x01 + ci * x11;
              x00 = y00; x10 = y10; x01 = y01; x11 = y11;
            }
            if (fj) {
              const T c = rc[j], sn = rs[j];
              T z00 = c * x00 - sn * x01, z01 = sn * x00 + c * x01;
              T z10 = c * x10 - sn * x11, z11 = sn * x10 + c * x11;
              x00 = z00; x01 = z01; x10 = z10; x11 = z11;
            }
            A[p * lda + r] = x00;
            A[r * lda + p] = x00;
            if (sv) { A[p * lda + s] = x01; A[s * lda + p] = x01; }
            if (qv) { A[q * lda + r] = x10; A[r * lda + q] = x10; }
            if (qv && sv) { A[q * lda + s] = x11; A[s * lda + q] = x11; }
          }
        }
        // eigenvector rows p,q: warp per pair, lanes along the row (coalesced / conflict-free)
        for (int i = wid; i < np; i += NTB_W) {
          if (!sh.rflag[i]) continue;
          const T c = rc[i], sn = rs[i];
          T *vp = V + (size_t)sh.rp[i] * n, *vq = V + (size_t)sh.rq[i] * n;
          for (int k = lane; k < n; k += 32) {
            const T a = vp[k], bq = vq[k];
            vp[k] = c * a - sn * bq;
            vq[k] = sn * a + c * bq;
          }
        }
        __syncthreads();
      }
    }
  }
  return -1;
}

// diagonal of A as eigenvalue estimates, their ascending ranks (ties by index) and the
// index of each rank (order[r])
// ascending ranks of dg (ties by index) and the index of each rank
__device__ void rank_values(const double *dg, int n, int *rank, int *order) {
  for (int k = threadIdx.x; k < n; k += NTB) {
    const double d = dg[k];
    int r = 0;
    for (int j = 0; j < n; ++j) r += (dg[j] < d) || (dg[j] == d && j < k);
    rank[k] = r;
    order[r] = k;
  }
  __syncthreads();
}

template <class T>
__device__ void rank_diag(const T *A, int lda, int n, double *dg, int *rank, int *order) {
  for (int k = threadIdx.x; k < n; k += NTB) dg[k] = (double)A[k * lda + k];
  __syncthreads();
  rank_values(dg, n, rank, order);
}

// largest coupling over diagonal splitting, max_{i<j} |a_ij| / |a_ii - a_jj|
__device__ double coupling_ratio(const double *A, int lda, int n, double *red) {
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < n * n; idx += NTB) {
    const int i = idx / n, j = idx - i * n;
    if (j <= i) continue;
    const double a = fabs(A[i * lda + j]), d = fabs(A[i * lda + i] - A[j * lda + j]);
    mx = fmax(mx, a > 0.0 ? (d > 0.0 ? a / d : INFINITY) : 0.0);
  }
  return jblock_reduce(mx, red, true);
}

// largest first-order occupied-virtual rotation |a_uo| / (HOMO-LUMO gap of the diagonal);
// +inf when the gap is not positive
template <class T>
__device__ double ov_theta(const T *A, int lda, int n, int nocc, const double *dg, const int *order, double *red) {
  const double gap = dg[order[nocc]] - dg[order[nocc - 1]];
  const int nv = n - nocc;
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < nocc * nv; idx += NTB) {
    const int o = order[idx / nv], u = order[nocc + idx % nv];
    mx = fmax(mx, fabs((double)A[u * lda + o]));
  }
  mx = jblock_reduce(mx, red, true);
  return gap > 0.0 ? mx / gap : INFINITY;
}

// FP32 sweeps on (float)A to max |a_pq| <= tol32 with the rotations W in shared memory,
// V <- W V (or W) in FP64, one Newton-Schulz step (FP64 where it matters), A = V F V^T
// again.  Returns the FP32 sweeps taken.
__device__ int fp32_stage(double *A, int lda, double *V, double *G, const double *Fm, int n, double tol32,
                          bool is_warm, bool a32_ready, JShared &sh) {
  const int tid = threadIdx.x;
  float *A32 = reinterpret_cast<float *>(A), *W32 = A32 + (size_t)n * lda;
  if (!a32_ready) {  // A (FP64) -> A32 in place, through G
    for (int idx = tid; idx < n * n; idx += NTB) {
      int i = idx / n, j = idx - i * n;
      G[idx] = A[i * lda + j];
    }
    __syncthreads();
    for (int idx = tid; idx < n * n; idx += NTB) {
      int i = idx / n, j = idx - i * n;
      A32[i * lda + j] = (float)G[idx];
    }
  }
  for (int idx = tid; idx < n * n; idx += NTB) {
    int i = idx / n, j = idx - i * n;
    W32[idx] = i == j ? 1.0f : 0.0f;  // rows of stride n, as jacobi_solve expects
  }
  __syncthreads();
  int s32 = jacobi_solve<float>(A32, lda, W32, n, tol32, 20, sh);
  if (s32 < 0) s32 = 20;
  __syncthreads();
  // V <- W V (warm) or W (cold), in FP64
  if (is_warm) {
    tile_product_df(
        n, n, n, false, [&](int k, int l) { return W32[k * n + l]; }, [&](int l, int j) { return V[(size_t)l * n + j]; },
        [&](int k, int j, double v) { G[(size_t)k * n + j] = v; });
  } else {
    for (int idx = tid; idx < n * n; idx += NTB) G[idx] = (double)W32[idx];
  }
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += NTB) V[idx] = G[idx];
  __syncthreads();
  // one Newton-Schulz step V <- V - (S - I) V / 2 with S = V V^T = W W^T (V was orthonormal):
  // D = W W^T - I in FP64 from the FP32 W (exact products), stored as FP32 over the idle A32
  // (|D| ~ 1e-6, so FP32 keeps it to ~1e-13), and the small correction D V in FP32
  float *D32 = A32;
  tile_product_df(
      n, n, n, true, [&](int k, int l) { return W32[k * n + l]; }, [&](int l, int j) { return W32[j * n + l]; },
      [&](int k, int j, double v) {
        if (k <= j) {
          const float d = (float)(v - (k == j ? 1.0 : 0.0));
          D32[k * lda + j] = d;
          D32[j * lda + k] = d;
        }
      });
  __syncthreads();
  tile_product_t<float>(
      n, false, [&](int k, int l) { return D32[k * lda + l]; }, [&](int l, int j) { return (float)V[(size_t)l * n + j]; },
      [&](int k, int j, float v) { G[(size_t)k * n + j] = V[(size_t)k * n + j] - 0.5 * (double)v; });
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += NTB) {
    int i = idx / n, j = idx - i * n;
    V[idx] = G[idx];
    A[i * lda + j] = Fm[idx];
  }
  __syncthreads();
  form_vfvt(A, lda, V, G, n, true);
  return s32;
}

// Density from a nearly diagonal A = V F V^T without further sweeps: the smaller of the
// occupied / virtual sets S is rotated to first order towards its complement T,
//   c_s' = v_s + sum_t theta_ts v_t,  theta_ts = a_ts / (a_ss - a_tt),
// re-orthonormalised (Loewdin, C'' = (I - E/2) C' with E = C' C'^T - I, exact to O(theta^4)),
// and P = 2 C''^T C'' (occupied) or 2 (I - C''^T C'') (virtual).  The remaining error is
// second order in the off-diagonal of A over the gap.  G: global scratch (P's block).
__device__ void newton_density(double *A, int lda, const double *V, double *G, double *Pm, int n, int nocc,
                               const double *dg, const int *order) {
  const bool use_occ = nocc <= n - nocc;
  const int nsel = use_occ ? nocc : n - nocc, ncomp = n - nsel;
  const int s0 = use_occ ? 0 : nocc, t0 = use_occ ? nocc : 0;
  double *Th = G, *C1 = G + (size_t)nsel * ncomp;
  for (int idx = threadIdx.x; idx < nsel * ncomp; idx += NTB) {
    const int i = idx / ncomp, t = idx - i * ncomp;
    const int s = order[s0 + i], u = order[t0 + t];
    Th[idx] = A[u * lda + s] / (dg[s] - dg[u]);
  }
  __syncthreads();
  tile_product_mnk(
      nsel, n, ncomp, [&](int i, int t) { return Th[(size_t)i * ncomp + t]; },
      [&](int t, int k) { return V[(size_t)order[t0 + t] * n + k]; },
      [&](int i, int k, double v) { C1[(size_t)i * n + k] = V[(size_t)order[s0 + i] * n + k] + v; });
  __syncthreads();
  double *E = A, *U = A + (size_t)nsel * nsel;  // A is no longer needed
  tile_product_mnk(
      nsel, nsel, n, [&](int i, int k) { return C1[(size_t)i * n + k]; },
      [&](int k, int j) { return C1[(size_t)j * n + k]; },
      [&](int i, int j, double v) { E[i * nsel + j] = v - (i == j ? 1.0 : 0.0); });
  __syncthreads();
  tile_product_mnk(
      nsel, n, nsel, [&](int i, int l) { return E[i * nsel + l]; }, [&](int l, int k) { return C1[(size_t)l * n + k]; },
      [&](int i, int k, double v) { U[i * n + k] = C1[(size_t)i * n + k] - 0.5 * v; });
  __syncthreads();
  for (int it = threadIdx.x; it < n * n; it += NTB) {
    const int a = it / n, c = it - a * n;
    if (c < a) continue;
    double s = 0.0;
    for (int k = 0; k < nsel; ++k) s += U[k * n + a] * U[k * n + c];
    const double v = use_occ ? 2.0 * s : (a == c ? 2.0 : 0.0) - 2.0 * s;
    Pm[(size_t)a * n + c] = v;
    Pm[(size_t)c * n + a] = v;
  }
}

constexpr double NEWTON_THETA = 1.0e-5;  // largest occupied-virtual rotation the first-order density takes
constexpr double EIG_PT_RATIO = 3.0e-3;  // largest coupling / splitting for second-order eigenvalues
// a warm start whose largest occupied-virtual ratio |a_st| / gap is at most ROT_THETA takes one
// rotation (rotate_orth) instead of FP32 sweeps, when its ||Theta||_F stays within ROT_NORM
// (W = I + K + K^2 / 2 orthogonal to ||K||^4 / 4 <= 2.5e-9, which the lift's Newton-Schulz step removes)
constexpr double ROT_THETA = 1.0e-3;
constexpr double ROT_NORM = 1.0e-2;
constexpr int ROT_ITERS = 3;  // fixed-point passes of the rotation's Sylvester equation

// The lift of FP32 rotations W (float, rows of stride n behind A32 in shared memory, orthogonal
// to FP32 accuracy) to FP64-orthonormal eigenvector rows, without FP64 rotation work:
// X = W V (warm) or W (cold) is formed in FP32 and stored in V, so X holds FP32 values whose
// products are exact; D = X X^T - I is summed to FP64 accuracy (double-float) from X^T staged in
// shared memory (conflict-free rows) and kept as FP32 (|D| ~ 1e-6); one Newton-Schulz step
// V <- X - D X / 2 (the small product D X in FP32) leaves the rows of V orthonormal to ~1e-13.
// A32 is dead on entry.  G (floats): X32; shared: V (warm) over A32 for X = W V, then X^T, and
// W32, then D.
__device__ void lift_rotations(double *A, int lda, double *V, double *G, int n, bool is_warm) {
  const int tid = threadIdx.x;
  float *A32 = reinterpret_cast<float *>(A), *W32 = A32 + (size_t)n * lda;
  float *X32 = reinterpret_cast<float *>(G);
  if (is_warm) {
    // V in FP32 over the swept A32 (dead now), so that both operands of X = W V are in shared memory
    float *V32 = A32;
    for (int idx = tid; idx < n * n; idx += NTB) V32[idx] = (float)V[idx];
    __syncthreads();
    tile_product_t<float>(
        n, false, [&](int k, int l) { return W32[k * n + l]; }, [&](int l, int j) { return V32[l * n + j]; },
        [&](int k, int j, float v) {
          X32[k * n + j] = v;
          V[(size_t)k * n + j] = (double)v;
        });
  } else {
    for (int idx = tid; idx < n * n; idx += NTB) {
      X32[idx] = W32[idx];
      V[idx] = (double)W32[idx];
    }
  }
  __syncthreads();
  float *XT = A32;  // X^T as FP32, stride lda (A32 and W32 are no longer needed)
  for (int idx = tid; idx < n * n; idx += NTB) {
    int i = idx / n, j = idx - i * n;
    XT[j * lda + i] = X32[idx];
  }
  __syncthreads();
  // exact FP32 products summed to FP64 accuracy on the FP32 pipe; D over the dead W32, so that
  // the correction D X reads both operands from shared memory (X as X^T's columns)
  float *D32s = W32;
  tile_product_df(
      n, n, n, true, [&](int k, int l) { return XT[l * lda + k]; }, [&](int l, int j) { return XT[l * lda + j]; },
      [&](int k, int j, double v) {
        if (k <= j) {
          const float d = (float)(v - (k == j ? 1.0 : 0.0));
          D32s[k * n + j] = d;
          D32s[j * n + k] = d;
        }
      });
  __syncthreads();
  tile_product_t<float>(
      n, false, [&](int k, int l) { return D32s[k * n + l]; }, [&](int l, int j) { return XT[j * lda + l]; },
      [&](int k, int j, float v) { V[(size_t)k * n + j] -= 0.5 * (double)v; });
  __syncthreads();
}

// FP32 sweeps for the density-only step: A32 (float, overlaying A) is swept to
// max |a_pq| <= tol32 with the rotations W (float, behind A32); dg / rank / order take the swept
// diagonal; then the lift above.  Returns the FP32 sweeps taken.
__device__ int fp32_sweeps_orth(double *A, int lda, double *V, double *G, int n, double tol32, bool is_warm,
                                double *dg, int *rank, int *order, JShared &sh) {
  float *A32 = reinterpret_cast<float *>(A), *W32 = A32 + (size_t)n * lda;
  for (int idx = threadIdx.x; idx < n * n; idx += NTB) {
    int i = idx / n, j = idx - i * n;
    W32[idx] = i == j ? 1.0f : 0.0f;
  }
  __syncthreads();
  int s32 = jacobi_solve<float>(A32, lda, W32, n, tol32, 20, sh);
  if (s32 < 0) s32 = 20;
  __syncthreads();
  rank_diag(A32, lda, n, dg, rank, order);
  lift_rotations(A, lda, V, G, n, is_warm);
  return s32;
}

// A warm start whose occupied-virtual block is small, brought to block-diagonal form by one
// rotation instead of FP32 sweeps.  With S the smaller of the occupied / virtual sets (ranks from
// dg, the diagonal of A32 = V F V^T) and T its complement, the rotation W = exp(K), K_st =
// Theta_st = -K_ts, zeroes the S-T block of W A W^T to first order in Theta when
//   Theta_st (d_s - d_t) = a_st + (Theta A'_TT)_st - (A'_SS Theta)_st   (A' without its diagonal d),
// which ROT_ITERS fixed-point passes solve from Theta = 0 (the first gives the first-order
// theta_st = a_st / (d_s - d_t); the others take in the couplings within the two blocks that
// earlier rotations leave in a warm start); the S-T block left is of third order in Theta, next to
// A32's FP32 rounding.  W = I + K + K^2 / 2 (K^2 = -Theta Theta^T on S x S, -Theta^T Theta on
// T x T; W W^T - I = K^4 / 4) in FP32 in the sweeps' rotation buffer, then lift_rotations.  The
// blocks within S and T stay as they are: the density needs the S subspace only.  Shared: A'_TT
// and A'_SS (permuted to rank order) where W is formed afterwards; G (floats): Theta^T, Theta
// Theta^T and Theta^T Theta in [0, n^2 - st), a_ST and two Theta buffers in [n^2, n^2 + 3 st)
// (st = |S| |T| <= n^2 / 4).  Returns false, with A32 and V untouched, when ||Theta||_F exceeds
// ROT_NORM (or is not finite) before or after the passes.
__device__ bool rotate_orth(double *A, int lda, double *V, double *G, int n, int nocc, const double *dg,
                            const int *rank, const int *order, double *red) {
  const int tid = threadIdx.x;
  const bool use_occ = nocc <= n - nocc;
  const int nsel = use_occ ? nocc : n - nocc, ncomp = n - nsel;
  const int s0 = use_occ ? 0 : nocc, t0 = use_occ ? nocc : 0;
  const int st = nsel * ncomp;
  const float *A32 = reinterpret_cast<const float *>(A);
  float *W32 = reinterpret_cast<float *>(A) + (size_t)n * lda;
  float *Att = W32, *Ass = W32 + ncomp * ncomp;  // ncomp^2 + nsel^2 <= n^2
  float *Gf = reinterpret_cast<float *>(G);
  float *ThT = Gf, *Qt = Gf + st, *Qs = Qt + ncomp * ncomp;  // st + ncomp^2 + nsel^2 = n^2 - st
  float *Ast = Gf + (size_t)n * n, *cur = Ast + st, *nxt = cur + st;
  const float rot_norm2 = (float)(ROT_NORM * ROT_NORM);
  for (int idx = tid; idx < ncomp * ncomp; idx += NTB) {
    const int u = idx / ncomp, t = idx - u * ncomp;
    Att[idx] = u == t ? 0.0f : A32[order[t0 + u] * lda + order[t0 + t]];
  }
  for (int idx = tid; idx < nsel * nsel; idx += NTB) {
    const int i = idx / nsel, j = idx - i * nsel;
    Ass[idx] = i == j ? 0.0f : A32[order[s0 + i] * lda + order[s0 + j]];
  }
  double nrm = 0.0;
  for (int idx = tid; idx < st; idx += NTB) {
    const int i = idx / ncomp, t = idx - i * ncomp;
    const int rs = order[s0 + i], rt = order[t0 + t];
    const float a = A32[rs * lda + rt], th = a / (float)(dg[rs] - dg[rt]);
    Ast[idx] = a;
    cur[idx] = th;
    nrm += (double)th * th;
  }
  nrm = jblock_reduce(nrm, red, false);  // synchronises: the gathered blocks and Theta complete
  if (!(nrm <= rot_norm2)) return false;
  for (int it = 1; it < ROT_ITERS; ++it) {
    tile_product_mnk_t<float>(
        nsel, ncomp, ncomp, false, [&](int i, int u) { return cur[i * ncomp + u]; },
        [&](int u, int t) { return Att[u * ncomp + t]; },
        [&](int i, int t, float v) { nxt[i * ncomp + t] = Ast[i * ncomp + t] + v; });
    __syncthreads();
    tile_product_mnk_t<float>(
        nsel, ncomp, nsel, false, [&](int i, int j) { return Ass[i * nsel + j]; },
        [&](int j, int t) { return cur[j * ncomp + t]; },
        [&](int i, int t, float v) {
          nxt[i * ncomp + t] = (nxt[i * ncomp + t] - v) / (float)(dg[order[s0 + i]] - dg[order[t0 + t]]);
        });
    __syncthreads();
    float *sw = cur;
    cur = nxt;
    nxt = sw;
  }
  nrm = 0.0;
  for (int idx = tid; idx < st; idx += NTB) {
    const float th = cur[idx];
    nrm += (double)th * th;
    const int i = idx / ncomp, t = idx - i * ncomp;
    ThT[t * nsel + i] = th;
  }
  nrm = jblock_reduce(nrm, red, false);  // synchronises: Theta^T complete
  if (!(nrm <= rot_norm2)) return false;
  tile_product_mnk_t<float>(
      nsel, nsel, ncomp, false, [&](int i, int u) { return ThT[u * nsel + i]; },
      [&](int u, int j) { return ThT[u * nsel + j]; }, [&](int i, int j, float v) { Qs[i * nsel + j] = v; });
  tile_product_mnk_t<float>(
      ncomp, ncomp, nsel, false, [&](int t, int i) { return cur[i * ncomp + t]; },
      [&](int i, int u) { return cur[i * ncomp + u]; }, [&](int t, int u, float v) { Qt[t * ncomp + u] = v; });
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += NTB) {  // A'_TT, A'_SS dead: W over them
    const int r = idx / n, c = idx - r * n;
    const int kr = rank[r], kc = rank[c];
    const bool sr = (unsigned)(kr - s0) < (unsigned)nsel, sc = (unsigned)(kc - s0) < (unsigned)nsel;
    const float dl = r == c ? 1.0f : 0.0f;
    float w;
    if (sr && !sc) w = cur[(kr - s0) * ncomp + (kc - t0)];
    else if (!sr && sc) w = -cur[(kc - s0) * ncomp + (kr - t0)];
    else if (sr) w = dl - 0.5f * Qs[(kr - s0) * nsel + (kc - s0)];
    else w = dl - 0.5f * Qt[(kr - t0) * ncomp + (kc - t0)];
    W32[idx] = w;
  }
  __syncthreads();
  lift_rotations(A, lda, V, G, n, true);
  return true;
}

// First-order density from orthonormal eigenvector rows V that nearly diagonalise F, with
// only the coupling block in FP64: for the smaller of the occupied / virtual sets S (ranks
// from dg) and its complement T,
//   a_st = ((V_S F) V_T^T)_st,  theta_st = a_st / (dg_s - dg_t),
// and, if max |theta| <= NEWTON_THETA, C' = V_S + Theta V_T, Loewdin E = C' C'^T - I =
// Theta Theta^T (V orthonormal), U = C' - E C' / 2, P = 2 U^T U (S occupied) or 2 (I - U^T U).
// The products of small quantities (Theta V_T, Theta Theta^T, E C') run in FP32 on FP32
// copies (rounding ~1e-7 of terms <= 1e-5); V_S F, the coupling block and U^T U in FP64.  The
// diagonal dg only enters the denominators, where FP32 accuracy is enough.
// Every operand of the double-float products is split into FP32 hi + lo once, where it is
// produced (F and V on entry, V_S F and U by their products), instead of on each of the ~n/4
// loads by the register tiles.  Scratch, in doubles (sn = nsel n, tn = ncomp n, st = nsel ncomp;
// S shared, >= n^2; G global, P's block, n^2):
//   S: F split [0, n^2)                  -> V_T split [0, tn) | Theta [tn, tn + st), later C'32 |
//                                           E32 [tn + st, tn + st + nsel^2 / 2); U split over V_T
//   G: V_S split [0, sn), later Theta32 | V_S F split [sn, 2 sn), later C' (FP64); then P
// (tn + st = n^2 - nsel^2, 2 sn <= n^2 as nsel <= n / 2).  Returns false, with P untouched, when
// the rotation is too large (or the gap not positive).
__device__ bool newton_density_ov(double *S, const double *V, const double *Fm, double *G, double *Pm, int n,
                                  int nocc, const double *dg, const int *order, double *red) {
  const bool use_occ = nocc <= n - nocc;
  const int nsel = use_occ ? nocc : n - nocc, ncomp = n - nsel;
  const int s0 = use_occ ? 0 : nocc, t0 = use_occ ? nocc : 0;
  const size_t nn = (size_t)n * n, sn = (size_t)nsel * n, tn = (size_t)ncomp * n, st = (size_t)nsel * ncomp;
  float *Fh = reinterpret_cast<float *>(S), *Fl = Fh + nn;
  float *Vsh = reinterpret_cast<float *>(G), *Vsl = Vsh + sn;          // V_S rows, split
  float *Gsh = reinterpret_cast<float *>(G + sn), *Gsl = Gsh + sn;    // (V_S F)^T: n rows of nsel, split
  for (int idx = threadIdx.x; idx < n * n; idx += NTB) split_f64(Fm[idx], Fh[idx], Fl[idx]);
  for (int idx = threadIdx.x; idx < (int)sn; idx += NTB) {
    const int i = idx / n, l = idx - i * n;
    split_f64(V[(size_t)order[s0 + i] * n + l], Vsh[idx], Vsl[idx]);
  }
  __syncthreads();
  tile_product_df(
      nsel, n, n, false, [&](int i, int l) { return DFPair{Vsh[(size_t)i * n + l], Vsl[(size_t)i * n + l]}; },
      [&](int l, int j) { return DFPair{Fh[(size_t)l * n + j], Fl[(size_t)l * n + j]}; },
      [&](int i, int j, double v) { split_f64(v, Gsh[(size_t)j * nsel + i], Gsl[(size_t)j * nsel + i]); });
  __syncthreads();
  // F is dead: the V_T rows, split, over it
  float *Vth = reinterpret_cast<float *>(S), *Vtl = Vth + tn;
  double *Th = S + tn;
  for (int idx = threadIdx.x; idx < (int)tn; idx += NTB) {
    const int t = idx / n, l = idx - t * n;
    split_f64(V[(size_t)order[t0 + t] * n + l], Vth[idx], Vtl[idx]);
  }
  __syncthreads();
  // a_st for t (rows of V_T) x s (columns of (V_S F)^T, contiguous)
  tile_product_df(
      ncomp, nsel, n, false, [&](int t, int l) { return DFPair{Vth[(size_t)t * n + l], Vtl[(size_t)t * n + l]}; },
      [&](int l, int i) { return DFPair{Gsh[(size_t)l * nsel + i], Gsl[(size_t)l * nsel + i]}; },
      [&](int t, int i, double v) {
        const double d = dg[order[s0 + i]] - dg[order[t0 + t]];
        Th[(size_t)i * ncomp + t] = d != 0.0 ? v / d : INFINITY;
      });
  __syncthreads();
  float *Th32 = reinterpret_cast<float *>(G);  // over the V_S split, dead now
  float *E32 = reinterpret_cast<float *>(S + tn + st);
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < (int)st; idx += NTB) {
    const double th = Th[idx], a = fabs(th);
    mx = fmax(mx, isnan(a) ? INFINITY : a);
    Th32[idx] = (float)th;
  }
  mx = jblock_reduce(mx, red, true);  // synchronises: Th32 complete, Th no longer read
  if (!(mx <= NEWTON_THETA)) return false;
  // products of small quantities in FP32 (V's hi part: V to 2^-23, on terms ~1e-5)
  float *C1_32 = reinterpret_cast<float *>(Th);  // Theta is dead
  double *C1 = G + sn;                            // over the V_S F split, dead
  tile_product_mnk_t<float>(
      nsel, n, ncomp, false, [&](int i, int t) { return Th32[i * ncomp + t]; },
      [&](int t, int k) { return Vth[(size_t)t * n + k]; },
      [&](int i, int k, float v) {
        const double c = V[(size_t)order[s0 + i] * n + k] + (double)v;
        C1_32[i * n + k] = (float)c;
        C1[(size_t)i * n + k] = c;
      });
  tile_product_mnk_t<float>(
      nsel, nsel, ncomp, false, [&](int i, int t) { return Th32[i * ncomp + t]; },
      [&](int t, int j) { return Th32[j * ncomp + t]; }, [&](int i, int j, float v) { E32[i * nsel + j] = v; });
  __syncthreads();
  float *Uh = reinterpret_cast<float *>(S), *Ul = Uh + sn;  // over the V_T split, dead (sn <= tn)
  tile_product_mnk_t<float>(
      nsel, n, nsel, false, [&](int i, int l) { return E32[i * nsel + l]; },
      [&](int l, int k) { return C1_32[l * n + k]; },
      [&](int i, int k, float v) {
        split_f64(C1[(size_t)i * n + k] - 0.5 * (double)v, Uh[(size_t)i * n + k], Ul[(size_t)i * n + k]);
      });
  __syncthreads();
  tile_product_df(
      n, n, nsel, true, [&](int a, int k) { return DFPair{Uh[(size_t)k * n + a], Ul[(size_t)k * n + a]}; },
      [&](int k, int c) { return DFPair{Uh[(size_t)k * n + c], Ul[(size_t)k * n + c]}; },
      [&](int a, int c, double s) {
        if (c < a) return;
        const double v = use_occ ? 2.0 * s : (a == c ? 2.0 : 0.0) - 2.0 * s;
        Pm[(size_t)a * n + c] = v;
        Pm[(size_t)c * n + a] = v;
      });
  return true;
}

__global__ void __launch_bounds__(NT_J) k_jacobi(seqm_batch b, const double *__restrict__ F, double *__restrict__ P,
                                                 double *__restrict__ evals, double *__restrict__ evecs,
                                                 double *__restrict__ work, const int64_t *__restrict__ row_off,
                                                 const uint8_t *__restrict__ active, int32_t *__restrict__ status,
                                                 int max_sweeps, uint8_t *__restrict__ warm,
                                                 int mixed_threshold, int density_only, int order_base, int cap) {
  extern __shared__ double A[];
  __shared__ JShared sh;
  __shared__ double dg[JMAX_N];
  __shared__ int rank[JMAX_N], order[JMAX_N];
  __shared__ double e2[JMAX_N];

  const int m = b.mol_order[order_base + blockIdx.x];
  if (active && !active[m]) return;
  const int n = b.mol_norb[m];
  if (n <= 0) return;
  if (n > JMAX_N) {  // larger bases go to the SP2 density step
    if (threadIdx.x == 0 && status) status[m] = -2;
    return;
  }
  if (n > cap) {  // size class of the launch does not hold this molecule (inconsistent classes)
    if (threadIdx.x == 0 && status) status[m] = -3;
    return;
  }
  const int lda = n | 1;
  const size_t mo = b.mol_mat_off[m];
  const double *Fm = F + mo;
  double *V = work + mo;  // row k = eigenvector k (column k of C)
  double *G = P ? P + mo : nullptr;  // P's block doubles as product scratch until P is written
  const int tid = threadIdx.x;
  const int nocc = b.mol_nocc[m];
  const bool is_warm = warm != nullptr && warm[m] != 0 && P != nullptr;
  const int hint = status ? status[m] : 0;
  const bool mixed = mixed_threshold > 0 && P != nullptr && (!is_warm || hint < 0 || hint >= mixed_threshold);
  // an SCF iteration needs P only: the FP64 polish may give way to the first-order density
  const bool want_newton = density_only && P != nullptr && evecs == nullptr && nocc > 0 && nocc < n;

  double f2 = 0.0;
  for (int idx = tid; idx < n * n; idx += NTB) {
    int i = idx / n, j = idx - i * n;
    double v = Fm[idx];
    A[i * lda + j] = v;
    if (!is_warm) V[idx] = i == j ? 1.0 : 0.0;
    f2 += v * v;
  }
  const double fro = sqrt(jblock_reduce(f2, sh.red, false));  // every thread has read warm[m] here
  if (warm != nullptr && tid == 0) warm[m] = 1;  // this call leaves valid eigenvector rows in work
  const double tol = 1.0e-13 * fro;
  const bool fp32_ok = mixed || (want_newton && mixed_threshold > 0);
  bool newton = false, a32_ready = false, a64_ready = false;
  int s32 = 0;
  if (density_only == 1 && want_newton && fp32_ok) {
    // SCF density step: F rotated by the previous eigenvectors in FP32 (warm) or F itself
    // (cold); FP32 sweeps unless the occupied-virtual block is already small; then the
    // first-order density from the FP64 coupling block alone
    float *A32 = reinterpret_cast<float *>(A);
    if (is_warm) {
      form_vfvt32(A, lda, V, Fm, G, n);
    } else {  // A (FP64) -> A32 in place, through G
      for (int idx = tid; idx < n * n; idx += NTB) {
        int i = idx / n, j = idx - i * n;
        G[idx] = A[i * lda + j];
      }
      __syncthreads();
      for (int idx = tid; idx < n * n; idx += NTB) {
        int i = idx / n, j = idx - i * n;
        A32[i * lda + j] = (float)G[idx];
      }
      __syncthreads();
    }
    rank_diag(A32, lda, n, dg, rank, order);
    const double th32 = is_warm ? ov_theta(A32, lda, n, nocc, dg, order, sh.red) : INFINITY;
    bool rotated = false;
    if (th32 > 0.5 * NEWTON_THETA) {
      // a small rotation in one step (reported as one FP32 sweep: its lift is the sweeps'),
      // otherwise sweeps
      rotated = th32 <= ROT_THETA && rotate_orth(A, lda, V, G, n, nocc, dg, rank, order, sh.red);
      s32 = rotated ? 1 : fp32_sweeps_orth(A, lda, V, G, n, 2.0e-7 * fro, is_warm, dg, rank, order, sh);
    }
    bool done = newton_density_ov(A, V, Fm, G, P + mo, n, nocc, dg, order, sh.red);
    if (!done && rotated) {  // the rotation left too large a coupling: sweeps from the rotated rows
      __syncthreads();
      form_vfvt32(A, lda, V, Fm, G, n);
      rank_diag(A32, lda, n, dg, rank, order);
      s32 = 1 + fp32_sweeps_orth(A, lda, V, G, n, 2.0e-7 * fro, true, dg, rank, order, sh);
      done = newton_density_ov(A, V, Fm, G, P + mo, n, nocc, dg, order, sh.red);
    }
    if (done) {
      if (tid == 0 && status) status[m] = s32;
      if (evals) {  // diagonal estimates (FP32 accuracy); the final step computes the eigenvalues
        double *e = evals + row_off[m];
        for (int k = tid; k < n; k += NTB) e[rank[k]] = dg[k];
      }
      return;
    }
    __syncthreads();
    // the rotation is too large for the first-order density: FP64 A = V F V^T (V orthonormal
    // here) and FP64 sweeps below
    for (int idx = tid; idx < n * n; idx += NTB) {
      int i = idx / n, j = idx - i * n;
      A[i * lda + j] = Fm[idx];
    }
    __syncthreads();
    form_vfvt(A, lda, V, G, n, true);
    a64_ready = true;
  } else if (density_only == 2 && evecs == nullptr && P != nullptr && fp32_ok) {
    // eigenvalues only: FP32 sweeps of the rotated F (warm) or F (cold), FP32 lift and
    // re-orthonormalisation, then A = V F V^T in FP64 for the second-order eigenvalues below
    float *A32 = reinterpret_cast<float *>(A);
    if (is_warm) {
      form_vfvt32(A, lda, V, Fm, G, n);
    } else {
      for (int idx = tid; idx < n * n; idx += NTB) {
        int i = idx / n, j = idx - i * n;
        G[idx] = A[i * lda + j];
      }
      __syncthreads();
      for (int idx = tid; idx < n * n; idx += NTB) {
        int i = idx / n, j = idx - i * n;
        A32[i * lda + j] = (float)G[idx];
      }
      __syncthreads();
    }
    s32 = fp32_sweeps_orth(A, lda, V, G, n, 2.0e-7 * fro, is_warm, dg, rank, order, sh);
    for (int idx = tid; idx < n * n; idx += NTB) {
      int i = idx / n, j = idx - i * n;
      A[i * lda + j] = Fm[idx];
    }
    __syncthreads();
    form_vfvt(A, lda, V, G, n, true);
    a64_ready = true;
    newton = true;  // nearly diagonal: try the second-order eigenvalues first
  } else if (is_warm && want_newton && fp32_ok) {
    // rotate in FP32 first: if the occupied-virtual block is already small, the FP64
    // rotation and the first-order density follow; otherwise the FP32 sweeps start from it
    // and the FP64 rotation is skipped
    form_vfvt32(A, lda, V, Fm, G, n);
    rank_diag(reinterpret_cast<const float *>(A), lda, n, dg, rank, order);
    if (ov_theta(reinterpret_cast<const float *>(A), lda, n, nocc, dg, order, sh.red) <= 0.5 * NEWTON_THETA) {
      for (int idx = tid; idx < n * n; idx += NTB) {
        int i = idx / n, j = idx - i * n;
        A[i * lda + j] = Fm[idx];
      }
      __syncthreads();
      form_vfvt(A, lda, V, G, n, true);
      rank_diag(A, lda, n, dg, rank, order);
      newton = ov_theta(A, lda, n, nocc, dg, order, sh.red) <= NEWTON_THETA;
      if (!newton) {  // rare: back to F in A for the FP32 stage below
        for (int idx = tid; idx < n * n; idx += NTB) {
          int i = idx / n, j = idx - i * n;
          A[i * lda + j] = Fm[idx];
        }
        __syncthreads();
        form_vfvt32(A, lda, V, Fm, G, n);
        a32_ready = true;
      }
    } else {
      a32_ready = true;
    }
  } else if (is_warm) {
    form_vfvt(A, lda, V, G, n, fp32_ok);  // FP64 products when the FP32 stages are off
    if (want_newton) {
      rank_diag(A, lda, n, dg, rank, order);
      newton = ov_theta(A, lda, n, nocc, dg, order, sh.red) <= NEWTON_THETA;
    }
  }
  if (!newton && fp32_ok && !a64_ready) {
    // before FP64 polish sweeps 3e-6 ||F|| is enough; the first-order density wants the
    // FP32 floor, so that the occupied-virtual rotation left over is ~1e-6
    s32 = fp32_stage(A, lda, V, G, Fm, n, (want_newton ? 2.0e-7 : 3.0e-6) * fro, is_warm, a32_ready, sh);
    if (want_newton) {
      rank_diag(A, lda, n, dg, rank, order);
      newton = ov_theta(A, lda, n, nocc, dg, order, sh.red) <= NEWTON_THETA;
    }
  }
  // eigenvalues without eigenvectors (density_only == 2): second order in the couplings of
  // the nearly diagonal A when each is small against its diagonal splitting (error of third
  // order, |a|^3 / delta^2); otherwise full sweeps
  bool eig_pt = false;
  int s64 = 0;
  if (density_only == 2 && newton) {
    eig_pt = coupling_ratio(A, lda, n, sh.red) <= EIG_PT_RATIO;
    if (!eig_pt) {
      // one selective FP64 sweep: rotate the pairs whose coupling is not small against their
      // splitting (near-degenerate levels), leave the rest to the second-order sum
      jacobi_solve<double>(A, lda, V, n, tol, 1, sh, 0.25 * EIG_PT_RATIO);
      s64 = 1;
      __syncthreads();
      eig_pt = coupling_ratio(A, lda, n, sh.red) <= EIG_PT_RATIO;
    }
    newton = eig_pt;
  }
  if (!newton) {
    const int sw = jacobi_solve<double>(A, lda, V, n, tol, max_sweeps, sh);
    s64 = sw < 0 ? -1 : s64 + sw;
  }
  __syncthreads();
  if (tid == 0 && status) status[m] = s64 < 0 ? -1 : s64 + s32;

  // ---- eigenvalues (ascending; ties by index)
  rank_diag(A, lda, n, dg, rank, order);
  if (eig_pt) {
    for (int k = tid; k < n; k += NTB) {
      const double akk = A[k * lda + k];
      double c = 0.0;
      for (int j = 0; j < n; ++j) {
        const double a = A[k * lda + j];
        // a zero coupling adds nothing, also between exactly degenerate diagonals (the
        // ratio test has excluded a nonzero coupling over a zero splitting)
        if (j != k && a != 0.0) c += a * a / (akk - A[j * lda + j]);
      }
      e2[k] = akk + c;
    }
    __syncthreads();
  }
  if (evals && !eig_pt) {
    double *e = evals + row_off[m];
    for (int k = tid; k < n; k += NTB) e[rank[k]] = dg[k];
  }
  if (evecs) {
    double *E = evecs + mo;
    for (int idx = tid; idx < n * n; idx += NTB) {
      int k = idx / n, i = idx - k * n;
      E[(size_t)rank[k] * n + i] = V[idx];
    }
  }
  if (!P) return;
  if (newton) {
    if (density_only != 2) newton_density(A, lda, V, G, P + mo, n, nocc, dg, order);
    if (eig_pt && evals) {
      __syncthreads();
      rank_values(e2, n, rank, order);
      double *e = evals + row_off[m];
      for (int k = tid; k < n; k += NTB) e[rank[k]] = e2[k];
    }
    return;
  }
  if (density_only == 2) return;  // eigenvalues only
  // ---- density from the smaller of the occupied / virtual sets, staged in shared memory
  const bool use_occ = nocc <= n - nocc;
  const int nsel = use_occ ? nocc : n - nocc;
  double *U = A;  // nsel rows of length n (A is no longer needed)
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += NTB) {
    int k = idx / n, i = idx - k * n;
    int r = rank[k];
    int slot = use_occ ? r : r - nocc;
    if (slot >= 0 && slot < nsel) U[slot * n + i] = V[idx];
  }
  __syncthreads();
  double *Pm = P + mo;
  for (int it = tid; it < n * n; it += NTB) {
    const int a = it / n, c = it - a * n;
    if (c < a) continue;
    double s = 0.0;
    for (int k = 0; k < nsel; ++k) s += U[k * n + a] * U[k * n + c];
    double v = use_occ ? 2.0 * s : (a == c ? 2.0 : 0.0) - 2.0 * s;
    Pm[(size_t)a * n + c] = v;
    Pm[(size_t)c * n + a] = v;
  }
}

// dynamic shared memory of a CTA for molecules of up to cap basis functions (A, stride cap | 1)
size_t jacobi_smem(int cap) {
  const size_t bytes = (size_t)cap * (cap | 1) * sizeof(double);
  return bytes < 8 ? 8 : bytes;
}

// k_jacobi's shared-memory limit: set once per device to the largest class (JMAX_N)
SmemLimit g_jacobi_smem;

// Side streams and events of the per-class launches, one set per host thread and device (a
// caller's threads each keep their own, so concurrent calls never share an event).  Created on a
// thread's first call with classes on a device; that call must not be under stream capture.
struct ClassStreams {
  cudaStream_t aux[SEQM_MAX_CLASSES - 1];
  cudaEvent_t fork, join[SEQM_MAX_CLASSES - 1];
};

ClassStreams *class_streams() {
  constexpr int MAX_DEV = 64;
  thread_local ClassStreams sets[MAX_DEV];
  thread_local bool made[MAX_DEV] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return nullptr;
  ClassStreams &cs = sets[dev];
  if (!made[dev]) {
    bool ok = cudaEventCreateWithFlags(&cs.fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; ok && i < SEQM_MAX_CLASSES - 1; ++i)
      ok = cudaStreamCreateWithFlags(&cs.aux[i], cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&cs.join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) return nullptr;  // fall back to one stream (a partial set is left unused)
    made[dev] = true;
  }
  return &cs;
}

// threads of a CTA for count molecules of up to cap basis functions: at least one per rotation
// pair (cap / 2 + 1) and enough warps for the products; small CTAs let several molecules share
// an SM, which pays when the class fills the GPU; a class of fewer molecules than SMs keeps the
// largest CTAs (latency of each solve)
int jacobi_threads(int cap, int count) {
  static std::atomic<int> sms[256];  // SM count per device ordinal, 0 = not yet queried
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 256) {
    int n = sms[dev].load(std::memory_order_relaxed);
    if (n == 0 && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      sms[dev].store(n, std::memory_order_relaxed);
    if (count < n) return NT_J;
  }
  return cap > 114 ? 512 : cap > 64 ? 256 : cap > 32 ? 128 : 64;
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_density_jacobi(const seqm_batch *bp, const double *F, double *P, double *evals, double *evecs,
                                   double *work, const int64_t *mol_row_off, const uint8_t *active, int32_t *status,
                                   int max_sweeps, uint8_t *warm, int mixed_threshold, int density_only,
                                   void *stream) {
  if (!bp || !work) return SEQM_E_ARG;
  if ((warm || mixed_threshold > 0) && !P) return SEQM_E_ARG;  // P's block is used as product scratch
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  const int cap = b.max_norb > JMAX_N ? JMAX_N : b.max_norb;  // larger molecules are skipped (status -2)
  const int rc0 = g_jacobi_smem.ensure(k_jacobi, jacobi_smem(JMAX_N));
  if (rc0 != SEQM_OK) return rc0;
  if (b.nclass <= 0) {
    k_jacobi<<<b.nmol, NT_J, jacobi_smem(cap), (cudaStream_t)stream>>>(
        b, F, P, evals, evecs, work, mol_row_off, active, status, max_sweeps, warm, mixed_threshold, density_only, 0,
        cap);
    return launch_check();
  }
  if (b.nclass > SEQM_MAX_CLASSES) return SEQM_E_ARG;
  int start = 0;
  for (int c = 0; c < b.nclass; ++c) {
    if (b.class_end[c] < start || b.class_end[c] > b.nmol) return SEQM_E_ARG;
    start = b.class_end[c];
  }
  if (start != b.nmol) return SEQM_E_ARG;
  // one launch per size class (mol_order is by descending norb): CTA threads and shared memory
  // sized for the class, so that several small molecules share an SM.  The classes solve
  // disjoint molecules, so classes after the first run on side streams forked from and joined
  // back to `stream`: their CTAs fill the SMs the largest class leaves idle in its last wave.
  cudaStream_t s = (cudaStream_t)stream;
  ClassStreams *side = b.nclass > 1 ? class_streams() : nullptr;
  if (side && cudaEventRecord(side->fork, s) != cudaSuccess) side = nullptr;
  start = 0;
  int rc = SEQM_OK;
  for (int c = 0; c < b.nclass; ++c) {
    const int end = b.class_end[c];
    const int ccap = b.class_norb[c] > cap ? cap : b.class_norb[c];
    cudaStream_t cs = s;
    if (side && c > 0) {
      cs = side->aux[c - 1];
      if (cudaStreamWaitEvent(cs, side->fork, 0) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    }
    if (end > start && ccap > 0) {
      k_jacobi<<<end - start, jacobi_threads(ccap, end - start), jacobi_smem(ccap), cs>>>(
          b, F, P, evals, evecs, work, mol_row_off, active, status, max_sweeps, warm, mixed_threshold, density_only,
          start, ccap);
      rc = launch_check();
      if (rc != SEQM_OK) break;
    }
    start = end;
  }
  if (side)  // join every side stream that was forked, also after an error
    for (int c = 1; c < b.nclass; ++c)
      if (cudaEventRecord(side->join[c - 1], side->aux[c - 1]) != cudaSuccess ||
          cudaStreamWaitEvent(s, side->join[c - 1], 0) != cudaSuccess)
        rc = SEQM_E_CUDA;
  return rc;
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
  // total dense-matrix size: b.mat_total, or mat_off[nmol] read back (one small read), then the size check
  int64_t total = 0;
  if (batch_total(b, s, &total) != SEQM_OK) return SEQM_E_CUDA;
  if (total < 0 || (size_t)total > NOALLOC_DOUBLES) return SEQM_E_TOO_LARGE;
  double *work = nullptr;
  int rc = jacobi_scratch_address(&work);
  if (rc != SEQM_OK) return rc;
  const size_t smem = jacobi_smem(b.max_norb);
  rc = g_jacobi_smem.ensure(k_jacobi, jacobi_smem(JMAX_N));
  if (rc != SEQM_OK) return rc;
  k_jacobi<<<b.nmol, NT_J, smem, s>>>(b, F, P, evals, evecs, work, mol_row_off, active, status, max_sweeps,
                                      nullptr, 0, 0, 0, b.max_norb);
  return launch_check();
}
