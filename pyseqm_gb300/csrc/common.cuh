// Shared definitions of the pyseqm_gb300 CUDA kernels (sm_103a, FP64).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/pyseqm_gb300.h"

namespace seqm {

// seqm/seqm_functions/constants.py:4,9 — MOPAC's eV per hartree and bohr radius
constexpr double EV = 27.21;
constexpr double A0 = 0.529167;
constexpr double OVERLAP_CUTOFF = 40.0;  // bohr, constants.py:23

// packed index (0..9) of the upper-triangle product (row, col) of one atom's s,px,py,pz
// (fock.py:7-18 order: ss, s-px, px-px, s-py, px-py, py-py, s-pz, px-pz, py-pz, pz-pz)
__host__ __device__ constexpr int k10_row(int k) {
  return k == 0 ? 0 : k == 1 ? 0 : k == 2 ? 1 : k == 3 ? 0 : k == 4 ? 1 : k == 5 ? 2 : k == 6 ? 0 : k == 7 ? 1 : k == 8 ? 2 : 3;
}
__host__ __device__ constexpr int k10_col(int k) { return k == 0 ? 0 : k <= 2 ? 1 : k <= 5 ? 2 : 3; }
// kind(mu, nu) -> packed index (fock.py:74-79)
__host__ __device__ constexpr int kind(int mu, int nu) {
  return mu >= nu ? (mu * (mu + 1)) / 2 + nu : (nu * (nu + 1)) / 2 + mu;
}

// divisor of ||dP||_F in the SCF convergence test: 4 per atom plus 9 per atom with 13 <= Z <= 17
// (9 nSuperHeavy + 4 nHeavy + 4 nHydro, scf_loop.py:245)
__device__ __forceinline__ double dm_norm(const seqm_batch &b, int m) {
  const int nat = b.mol_atom_off[m + 1] - b.mol_atom_off[m];
  return 4.0 * nat + (b.mol_nsuper ? 9.0 * b.mol_nsuper[m] : 0.0);
}

__device__ __forceinline__ double par(const seqm_batch &b, int slot, int atom) {
  return b.atom_par[(size_t)slot * b.natoms + atom];
}

// row-major index of pair (i<j) among n items (0-based i, j)
__host__ __device__ __forceinline__ int tri_index(int i, int j, int n) { return i * n - (i * (i + 1)) / 2 + (j - i - 1); }

// first atom of the molecule owning global pair index p of a class segment: binary search on offsets
__device__ __forceinline__ int find_mol(const int32_t *off, int nmol, int p) {
  int lo = 0, hi = nmol;  // off[lo] <= p < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (off[mid] <= p) lo = mid; else hi = mid;
  }
  return lo;
}

// AO index of local atom la inside its molecule's packed basis (heavy: 4 per atom, H: 1)
__device__ __forceinline__ int atom_ao(int la, int nheavy) { return la < nheavy ? 4 * la : 3 * nheavy + la; }

// Exact j / d for 32-bit j without a division instruction (the 32-bit integer division goes through
// conversions on a slow pipe): j / d = umulhi64(j, M) with M = ceil(2^64 / d), d >= 2 (the excess
// j (M - 2^64/d) / 2^64 < 2^-32 never carries a fraction <= 1 - 1/d over an integer).
struct FastDivU32 {
  unsigned long long M;
  uint32_t d;
  __device__ explicit FastDivU32(uint32_t dv) : M(~0ULL / (unsigned long long)dv + 1), d(dv) {}
  __device__ __forceinline__ uint32_t div(uint32_t j) const { return (uint32_t)__umul64hi((unsigned long long)j, M); }
};
// flat index j of an n x n matrix (n >= 1) lies on the diagonal: j is a multiple of n + 1
struct DiagTest {
  FastDivU32 q;
  __device__ explicit DiagTest(int n) : q((uint32_t)(n + 1)) {}
  __device__ __forceinline__ bool operator()(uint32_t j) const { return j == q.div(j) * q.d; }
};

inline int launch_check() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SEQM_OK : SEQM_E_CUDA;
}

// mol_mat_off[nmol] (dense matrix elements of the batch): the host copy in the struct when the
// caller filled it in, else read back from the device, which waits for the stream
inline int batch_total(const seqm_batch &b, cudaStream_t s, int64_t *total) {
  if (b.mat_total > 0) {
    *total = b.mat_total;
    return SEQM_OK;
  }
  *total = 0;
  if (cudaMemcpyAsync(total, b.mol_mat_off + b.nmol, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return SEQM_E_CUDA;
  return SEQM_OK;
}

// Dynamic shared-memory limit of one kernel, raised once per device to the largest size any
// launch of that kernel asks for and never lowered.  The attribute belongs to the device and
// the function, not to a stream or a thread: a caller that set it to its own size on every call
// could have another host thread lower it between that set and its launch.
struct SmemLimit {
  std::atomic<bool> done[256] = {};
  std::mutex mu;
  template <typename Kern>
  int ensure(Kern kern, size_t bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SEQM_E_CUDA;
    if (dev < 0 || dev >= 256) return SEQM_E_ARG;
    if (done[dev].load(std::memory_order_acquire)) return SEQM_OK;
    std::lock_guard<std::mutex> lock(mu);
    if (!done[dev].load(std::memory_order_relaxed)) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
        return SEQM_E_CUDA;
      done[dev].store(true, std::memory_order_release);
    }
    return SEQM_OK;
  }
};

}  // namespace seqm
