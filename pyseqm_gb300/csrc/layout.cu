// Device-side pair list of the ragged batch (the parser's pair enumeration, basics.py:219-403).
//
// Pairs come in three class segments (heavy-heavy, heavy-H, H-H), each enumerated row-major
// (i < j) inside its molecule; the per-molecule segment offsets are already in the batch, so
// every pair's two atoms follow from its index alone: one thread per pair finds its molecule by
// binary search on the segment offsets and inverts the row-major triangular index.  Building the
// list here saves the host from generating it and the upload of two int32 per pair.
#include <math.h>

#include "common.cuh"

namespace seqm {

// (i, j), i < j < n, of row-major index q among the pairs of n items
__device__ __forceinline__ void tri_pair(long long q, long long n, int &i, int &j) {
  auto start = [n](long long r) { return r * n - r * (r + 1) / 2; };  // first index of row r
  const double d = (double)(2 * n - 1);
  long long r = (long long)floor(0.5 * (d - sqrt(fmax(d * d - 8.0 * (double)q, 0.0))));
  if (r < 0) r = 0;
  while (r > 0 && start(r) > q) --r;
  while (r + 1 < n && start(r + 1) <= q) ++r;
  i = (int)r;
  j = (int)(q - start(r) + r + 1);
}

__global__ void k_build_pairs(seqm_batch b, int32_t *__restrict__ pi, int32_t *__restrict__ pj) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (long long)b.nxx + b.nxh + b.nhh) return;
  int seg, q;
  const int32_t *off;
  if (p < b.nxx) {
    seg = 0, q = (int)p, off = b.mol_xx_off;
  } else if (p < (long long)b.nxx + b.nxh) {
    seg = 1, q = (int)(p - b.nxx), off = b.mol_xh_off;
  } else {
    seg = 2, q = (int)(p - b.nxx - b.nxh), off = b.mol_hh_off;
  }
  const int m = find_mol(off, b.nmol, q);
  const int r = q - off[m];
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], ny = b.mol_atom_off[m + 1] - a0 - nh;
  int i, j;
  if (seg == 0) {
    tri_pair(r, nh, i, j);
    pi[p] = a0 + i;
    pj[p] = a0 + j;
  } else if (seg == 1) {
    pi[p] = a0 + r / ny;
    pj[p] = a0 + nh + r % ny;
  } else {
    tri_pair(r, ny, i, j);
    pi[p] = a0 + nh + i;
    pj[p] = a0 + nh + j;
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_build_pairs(const seqm_batch *bp, int32_t *pair_i, int32_t *pair_j, void *stream) {
  if (!bp || !pair_i || !pair_j) return SEQM_E_ARG;
  const seqm_batch &b = *bp;
  const long long np = (long long)b.nxx + b.nxh + b.nhh;
  if (np == 0) return SEQM_OK;
  if (b.nmol <= 0 || np > 0x7fffffffLL) return SEQM_E_ARG;
  k_build_pairs<<<(unsigned)((np + 255) / 256), 256, 0, (cudaStream_t)stream>>>(b, pair_i, pair_j);
  return launch_check();
}
