// Two-electron contraction G(P) for batches of general (not symmetric) AO densities: the
// matrix-vector product of the CIS / RPA excited-state solvers.
//
// Replaces makeA_pi_batched + makeA_pi_symm_batch (seqm/seqm_functions/rcis_batch.py:296-507),
// which split each transition density into its symmetric part (Coulomb, exchange and
// one-centre terms of a Fock build) and its antisymmetric part (exchange and the one-centre
// (s,p), (p,p') terms only).  Written for a general density P the two parts combine into:
//   diagonal block of atom A:   one-centre(P_AA^sym) + one-centre-anti(P_AA^anti)
//                               + sum_B J_B(P_BB^sym)                    (Coulomb from partners)
//   block (A, B), A != B:       G_AB = -1/2 sum P_AB (mu lam | nu sig)   (each block from its own
//                               block of P, so G_BA uses P_BA)
// With P symmetric this is the Fock build's two-electron part.  Layout: nvec density sets,
// each a full ragged batch (per-molecule norb x norb blocks at mol_mat_off), set v at
// P + v * stride.  One warp per atom (diagonal block), one thread per pair (off-diagonal
// blocks), blockIdx.y = set; every element is written once, no atomics.
#include <math.h>

#include "common.cuh"

namespace seqm {

namespace {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// packed symmetric density of one heavy atom's diagonal block: PX[k] = P_rc + P_cr (r < c), P_rr
__device__ __forceinline__ void packed_sym(const double *Pm, int n, int o, double *PX) {
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    const int r = k10_row(k), c = k10_col(k);
    PX[k] = r == c ? Pm[(size_t)(o + r) * n + o + c] : Pm[(size_t)(o + r) * n + o + c] + Pm[(size_t)(o + c) * n + o + r];
  }
}

__device__ void gen_diag(const seqm_batch &b, int a, int lane, const double *__restrict__ P,
                         const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                         const double *__restrict__ w_hh, double *__restrict__ G) {
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
  const int n = b.mol_norb[m], la = a - a0;
  const int xx0 = b.mol_xx_off[m], xh0 = b.mol_xh_off[m], hh0 = b.mol_hh_off[m];
  const size_t mo = b.mol_mat_off[m];
  const double *Pm = P + mo;
  double *Gm = G + mo;
  const double gss = par(b, SEQM_P_GSS, a);
  if (la < nh) {
    const int o = 4 * la;
    double f[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) f[k] = 0.0;
    for (int q = lane; q < nat - 1; q += 32) {
      if (q < nh - 1) {
        const int j = q < la ? q : q + 1;
        double PB[10];
        packed_sym(Pm, n, 4 * j, PB);
        if (j > la) {
          const double *w = w_xx + (size_t)100 * (xx0 + tri_index(la, j, nh));
#pragma unroll
          for (int k = 0; k < 10; ++k) {
            double s = 0.0;
#pragma unroll
            for (int l = 0; l < 10; ++l) s += PB[l] * w[k * 10 + l];
            f[k] += s;
          }
        } else {
          const double *w = w_xx + (size_t)100 * (xx0 + tri_index(j, la, nh));
#pragma unroll
          for (int l = 0; l < 10; ++l) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < 10; ++k) s += PB[k] * w[k * 10 + l];
            f[l] += s;
          }
        }
      } else {
        const int h = q - (nh - 1), oh = 4 * nh + h;
        const double *w = w_xh + (size_t)10 * (xh0 + la * ny + h);
        const double ph = Pm[(size_t)oh * n + oh];
#pragma unroll
        for (int k = 0; k < 10; ++k) f[k] += ph * w[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) f[k] = wsum(f[k]);
    // one-centre terms: symmetric part as the Fock build (fock.py:187-231), antisymmetric part
    // (rcis_batch.py:354-368) with opposite signs above and below the diagonal
    const double gsp = par(b, SEQM_P_GSP, a), gpp = par(b, SEQM_P_GPP, a);
    const double gp2 = par(b, SEQM_P_GP2, a), hsp = par(b, SEQM_P_HSP, a);
    double Ps[4][4], Pa[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double x = Pm[(size_t)(o + r) * n + o + c], y = Pm[(size_t)(o + c) * n + o + r];
        Ps[r][c] = 0.5 * (x + y);
        Pa[r][c] = 0.5 * (x - y);
      }
    const double f1 = gsp - 0.5 * hsp, f2 = 1.5 * hsp - 0.5 * gsp, f3 = 1.25 * gp2 - 0.25 * gpp,
                 f4 = 0.75 * gpp - 1.25 * gp2, a2 = 0.5 * hsp - 0.5 * gsp, a4 = 0.25 * gpp - 0.75 * gp2;
    const double Pss = Ps[0][0], Ppt = Ps[1][1] + Ps[2][2] + Ps[3][3];
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      const int r = k10_row(k), c = k10_col(k);
      double oc, an = 0.0;
      if (r == 0 && c == 0) oc = 0.5 * Pss * gss + Ppt * f1;
      else if (r == c) oc = Pss * f1 + 0.5 * Ps[r][r] * gpp + (Ppt - Ps[r][r]) * f3;
      else if (r == 0) { oc = Ps[0][c] * f2; an = Pa[0][c] * a2; }
      else { oc = Ps[r][c] * f4; an = Pa[r][c] * a4; }
      if (lane == k) {
        const double v = oc + f[k];
        Gm[(size_t)(o + r) * n + o + c] = v + an;
        if (r != c) Gm[(size_t)(o + c) * n + o + r] = v - an;
      }
    }
  } else {
    const int h = la - nh, o = 3 * nh + la;
    double f = 0.0;
    for (int q = lane; q < nat - 1; q += 32) {
      if (q < nh) {
        const double *w = w_xh + (size_t)10 * (xh0 + q * ny + h);
        double PB[10];
        packed_sym(Pm, n, 4 * q, PB);
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 10; ++k) s += PB[k] * w[k];
        f += s;
      } else {
        const int g0 = q - nh, g = g0 < h ? g0 : g0 + 1, og = 4 * nh + g;
        const double w = w_hh[hh0 + (g < h ? tri_index(g, h, ny) : tri_index(h, g, ny))];
        f += w * Pm[(size_t)og * n + og];
      }
    }
    f = wsum(f);
    if (lane == 0) Gm[(size_t)o * n + o] = 0.5 * Pm[(size_t)o * n + o] * gss + f;
  }
}

__global__ void __launch_bounds__(128) k_fock_general(seqm_batch b, const double *__restrict__ P0,
                                                      const double *__restrict__ w_xx,
                                                      const double *__restrict__ w_xh,
                                                      const double *__restrict__ w_hh, double *__restrict__ G0,
                                                      long long stride, const uint8_t *__restrict__ active) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ndiag = 32LL * b.natoms;
  const int npairs = b.nxx + b.nxh + b.nhh;
  const double *P = P0 + (size_t)blockIdx.y * stride;
  double *G = G0 + (size_t)blockIdx.y * stride;
  if (t < ndiag) {
    const int a = (int)(t >> 5);
    if (active && !active[b.atom_mol[a]]) return;
    gen_diag(b, a, (int)(t & 31), P, w_xx, w_xh, w_hh, G);
    return;
  }
  if (t - ndiag >= npairs) return;
  const int p = (int)(t - ndiag);
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  if (active && !active[m]) return;
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], n = b.mol_norb[m];
  const int oi = atom_ao(ia - a0, nh), oj = atom_ao(ja - a0, nh);
  const size_t mo = b.mol_mat_off[m];
  const double *Pm = P + mo;
  double *Gm = G + mo;
  if (p < b.nxx) {
    const double *w = w_xx + (size_t)100 * p;
    double Pu[4][4], Pl[4][4];  // P_AB and P_BA^T
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        Pu[l][s] = -0.5 * Pm[(size_t)(oi + l) * n + oj + s];
        Pl[l][s] = -0.5 * Pm[(size_t)(oj + s) * n + oi + l];
      }
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int nu = 0; nu < 4; ++nu) {
        double ku = 0.0, kl = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l)
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            const double x = w[kind(mu, l) * 10 + kind(nu, s)];
            ku += x * Pu[l][s];
            kl += x * Pl[l][s];
          }
        Gm[(size_t)(oi + mu) * n + oj + nu] = ku;
        Gm[(size_t)(oj + nu) * n + oi + mu] = kl;
      }
  } else if (p < b.nxx + b.nxh) {
    const double *w = w_xh + (size_t)10 * (p - b.nxx);
    double Pu[4], Pl[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      Pu[l] = -0.5 * Pm[(size_t)(oi + l) * n + oj];
      Pl[l] = -0.5 * Pm[(size_t)oj * n + oi + l];
    }
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
      double ku = 0.0, kl = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        ku += w[kind(mu, l)] * Pu[l];
        kl += w[kind(mu, l)] * Pl[l];
      }
      Gm[(size_t)(oi + mu) * n + oj] = ku;
      Gm[(size_t)oj * n + oi + mu] = kl;
    }
  } else {
    const double w = w_hh[p - b.nxx - b.nxh];
    Gm[(size_t)oi * n + oj] = -0.5 * w * Pm[(size_t)oi * n + oj];
    Gm[(size_t)oj * n + oi] = -0.5 * w * Pm[(size_t)oj * n + oi];
  }
}

}  // namespace

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_fock_general(const seqm_batch *bp, int nvec, const double *P, const double *w_xx,
                                 const double *w_xh, const double *w_hh, double *G, int64_t stride,
                                 const uint8_t *active, void *stream) {
  if (!bp || nvec < 0 || nvec > 65535 || stride < 0) return SEQM_E_ARG;
  seqm_batch b = *bp;
  const long long nt = 32LL * b.natoms + b.nxx + b.nxh + b.nhh;
  if (nt == 0 || nvec == 0) return SEQM_OK;
  dim3 grid((unsigned)((nt + 127) / 128), (unsigned)nvec);
  k_fock_general<<<grid, 128, 0, (cudaStream_t)stream>>>(b, P, w_xx, w_xh, w_hh, G, (long long)stride, active);
  return launch_check();
}
