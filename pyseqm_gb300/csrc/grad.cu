// Gradients of the SCF energy at a fixed (converged) density (FP64).
//
// The reference obtains forces by autograd with the SCF treated as a constant
// (SCF0, seqm/seqm_functions/scf_loop.py:1996-2031; Force.forward, basics.py:1315-1336):
// dE/dR flows only through the integrals, the overlaps and the core-core terms.
// Per atom pair (A, B) that part of the energy is
//
//   E_AB = sum_ab D_ab w_ab(R)                                 (two-electron + e1b/e2a)
//        + sum_{mu in A, nu in B} P_mu,nu (beta_mu + beta_nu) S_mu,nu(R)   (resonance)
//        + Enuc_AB(R)                                           (core-core)
//
// with D_ab = P_A[a] P_B[b] - 1/2 sum P_AB P_AB (exchange) - Z_B P_A[a] d_b0 - Z_A P_B[b] d_a0
// (unrestricted: P the total density and the exchange term sum_s P_s,AB P_s,AB).
// Each pair thread evaluates E_AB with dual numbers carrying d/d(Rj - Ri) (the same
// templated integral code as the forward kernel, recomputed rather than stored), so
// one pass gives the 3-vector gradient; a per-atom gather (no atomics) then forms
// dE/dR and the U_ss, U_pp, beta_s, beta_p parameter gradients.
#include <math.h>

#include "common.cuh"
#include "pair_math.cuh"

namespace seqm {

// weighted packed density of one atom's diagonal block (off-diagonal products count twice)
__device__ __forceinline__ void grad_packed(const double *Pm, int norb, int o, bool heavy, double *PX) {
#pragma unroll
  for (int k = 0; k < 10; ++k) PX[k] = 0.0;
  if (heavy) {
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      int r = k10_row(k), c = k10_col(k);
      PX[k] = Pm[(size_t)(o + r) * norb + o + c] * (r == c ? 1.0 : 2.0);
    }
  } else {
    PX[0] = Pm[(size_t)o * norb + o];
  }
}

// sum over the ordered orbital pairs (mu,lam) with kind = a and (nu,sig) with kind = c of
// Pab[mu][nu] Pab[lam][sig]  (the exchange contraction of fock.py:297-345, differentiated)
__device__ __forceinline__ double exch(const double Pab[4][4], int a, int c) {
  const int ra = k10_row(a), ca = k10_col(a), rc = k10_row(c), cc = k10_col(c);
  double s = Pab[ra][rc] * Pab[ca][cc];
  if (rc != cc) s += Pab[ra][cc] * Pab[ca][rc];
  if (ra != ca) {
    s += Pab[ca][rc] * Pab[ra][cc];
    if (rc != cc) s += Pab[ca][cc] * Pab[ra][rc];
  }
  return s;
}

// weighted packed symmetric part Rs = (R + R^T)/2 of one atom's diagonal block of a general
// matrix: Rs_rr, and 2 Rs_rc = R_rc + R_cr off the diagonal
__device__ __forceinline__ void grad_packed_sym(const double *Rm, int norb, int o, bool heavy, double *PX) {
#pragma unroll
  for (int k = 0; k < 10; ++k) PX[k] = 0.0;
  if (heavy) {
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      int r = k10_row(k), c = k10_col(k);
      PX[k] = r == c ? Rm[(size_t)(o + r) * norb + o + c]
                     : Rm[(size_t)(o + r) * norb + o + c] + Rm[(size_t)(o + c) * norb + o + r];
    }
  } else {
    PX[0] = Rm[(size_t)o * norb + o];
  }
}

// the same ordered contraction for two different blocks: sum X[mu][nu] Y[lam][sig]
__device__ __forceinline__ double exch2(const double X[4][4], const double Y[4][4], int a, int c) {
  const int ra = k10_row(a), ca = k10_col(a), rc = k10_row(c), cc = k10_col(c);
  double s = X[ra][rc] * Y[ca][cc];
  if (rc != cc) s += X[ra][cc] * Y[ca][rc];
  if (ra != ca) {
    s += X[ca][rc] * Y[ra][cc];
    if (rc != cc) s += X[ca][cc] * Y[ra][rc];
  }
  return s;
}

constexpr int GRAD_STRIDE = 7;  // per pair: dE/d(Rj-Ri) x3, d beta_s(i), d beta_p(i), d beta_s(j), d beta_p(j)

// EXC: gradient of a CIS / RPA excited state (rcis_grad_batch, rcis_grad_batch.py:10-259,
// include_ground_state): on top of the ground-state terms of P, the relaxed difference density
// D (Dd, symmetric) enters the Coulomb, core-attraction, exchange and resonance terms linearly
// (D_A P_B + P_A D_B, -Z D, -exch(D, P), D (beta + beta) S), and the transition density R (Rt)
// quadratically: 4 Rs_A Rs_B - 2 exch(Rs) - 2 exch(Ra) with Rs, Ra its symmetric and
// antisymmetric parts.  Restricted densities only.
template <bool EXC>
__global__ void __launch_bounds__(128) k_pair_grad(seqm_batch b, const double *__restrict__ P,
                                                   const double *__restrict__ Pbeta, const double *__restrict__ gE,
                                                   const double *__restrict__ gN, double *__restrict__ work,
                                                   const double *__restrict__ Dd, const double *__restrict__ Rt) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (p >= npairs) return;
  double *out = work + (size_t)GRAD_STRIDE * p;
  if (b.pair_skip && b.pair_skip[p]) {  // beyond pair_outer_cutoff: no term of this pair
    for (int k = 0; k < GRAD_STRIDE; ++k) out[k] = 0.0;
    return;
  }
  const int cls = p < b.nxx ? 2 : (p < b.nxx + b.nxh ? 1 : 0);
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  const double ge = gE[m], gn = gN[m];
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m];
  const int li = ia - a0, lj = ja - a0;
  const int oi = atom_ao(li, nh), oj = atom_ao(lj, nh);
  const bool hi = li < nh, hj = lj < nh;
  const int ni_ = hi ? 4 : 1, nj_ = hj ? 4 : 1;
  const double *Pm = P + b.mol_mat_off[m];
  // unrestricted (Pbeta != NULL): P is the alpha density; Coulomb, core and resonance terms
  // take the total density and the exchange term both spin densities
  const double *Qm = Pbeta ? Pbeta + b.mol_mat_off[m] : nullptr;
  double PA[10], PB[10], Pab[4][4], Pa_ab[4][4], Pb_ab[4][4];
  grad_packed(Pm, norb, oi, hi, PA);
  grad_packed(Pm, norb, oj, hj, PB);
  if (Qm) {
    double QA[10], QB[10];
    grad_packed(Qm, norb, oi, hi, QA);
    grad_packed(Qm, norb, oj, hj, QB);
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      PA[k] += QA[k];
      PB[k] += QB[k];
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const bool in = u < ni_ && v < nj_;
      const size_t ix = (size_t)(oi + u) * norb + oj + v;
      Pa_ab[u][v] = in ? Pm[ix] : 0.0;
      Pb_ab[u][v] = (in && Qm) ? Qm[ix] : 0.0;
      Pab[u][v] = Pa_ab[u][v] + Pb_ab[u][v];
    }
  double DA[10], DB[10], SA[10], SB[10], Dab[4][4], Sab[4][4], Tab[4][4];
  if (EXC) {
    const double *Dm = Dd + b.mol_mat_off[m], *Rm = Rt + b.mol_mat_off[m];
    grad_packed(Dm, norb, oi, hi, DA);
    grad_packed(Dm, norb, oj, hj, DB);
    grad_packed_sym(Rm, norb, oi, hi, SA);
    grad_packed_sym(Rm, norb, oj, hj, SB);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const bool in = u < ni_ && v < nj_;
        const double x = in ? Rm[(size_t)(oi + u) * norb + oj + v] : 0.0;
        const double y = in ? Rm[(size_t)(oj + v) * norb + oi + u] : 0.0;
        Dab[u][v] = in ? Dm[(size_t)(oi + u) * norb + oj + v] : 0.0;
        Sab[u][v] = 0.5 * (x + y);
        Tab[u][v] = 0.5 * (x - y);
      }
  }
  // Coulomb factor of D_ab (P_A[a] P_B[b], plus the excited-state terms)
  auto coul = [&](int a, int c) {
    double s = PA[a] * PB[c];
    if (EXC) s += DA[a] * PB[c] + PA[a] * DB[c] + 4.0 * SA[a] * SB[c];
    return s;
  };
  // exchange part of D: 1/2 exch(P) restricted, exch(Pa) + exch(Pb) unrestricted
  auto xch = [&](int a, int c) {
    double s = Qm ? exch(Pa_ab, a, c) + exch(Pb_ab, a, c) : 0.5 * exch(Pab, a, c);
    if (EXC) s += exch2(Dab, Pab, a, c) + 2.0 * (exch(Sab, a, c) + exch(Tab, a, c));
    return s;
  };
  // densities of the core-attraction terms: P, plus D for an excited state
  auto cA = [&](int a) { return EXC ? PA[a] + DA[a] : PA[a]; };
  auto cB = [&](int c) { return EXC ? PB[c] + DB[c] : PB[c]; };
  const double ZA = par(b, SEQM_P_TORE, ia), ZB = par(b, SEQM_P_TORE, ja);

  // geometry as dual numbers: seeds on the three components of Rj - Ri (Angstrom)
  const double dxv = b.atom_xyz[3 * ja] - b.atom_xyz[3 * ia];
  const double dyv = b.atom_xyz[3 * ja + 1] - b.atom_xyz[3 * ia + 1];
  const double dzv = b.atom_xyz[3 * ja + 2] - b.atom_xyz[3 * ia + 2];
  const Dual3 dx(dxv, 1.0, 0.0, 0.0), dy(dyv, 0.0, 1.0, 0.0), dz(dzv, 0.0, 0.0, 1.0);
  const Dual3 dist = sqrt(dx * dx + dy * dy + dz * dz);
  const Dual3 r = dist * (1.0 / A0);
  const Dual3 xv = dx / dist, yv = dy / dist, zv = dz / dist;
  const double r0a = par(b, SEQM_P_RHO0, ia), r0b = par(b, SEQM_P_RHO0, ja);
  Dual3 E(0.0), gam;
  if (ge != 0.0 || gn != 0.0) {
    Dual3 R[3][3];
    quat_rot<Dual3>(-xv, -yv, -zv, R);
    if (cls == 2) {
      Dual3 ri[22];
      local_xx<Dual3>(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_DD, ja), par(b, SEQM_P_QQ, ia), par(b, SEQM_P_QQ, ja),
                      r0a, r0b, par(b, SEQM_P_RHO1, ia), par(b, SEQM_P_RHO1, ja), par(b, SEQM_P_RHO2, ia),
                      par(b, SEQM_P_RHO2, ja), ri);
      rotate_xx<Dual3>(ri, R, [&](int a, int c, Dual3 w) {
        double D = coul(a, c) - xch(a, c);
        if (c == 0) D -= ZB * cA(a);
        if (a == 0) D -= ZA * cB(c);
        E += (ge * D) * w;
      });
      gam = ri[0];
    } else if (cls == 1) {
      Dual3 ri[4];
      local_xh<Dual3>(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_QQ, ia), r0a, r0b, par(b, SEQM_P_RHO1, ia),
                      par(b, SEQM_P_RHO2, ia), ri);
      rotate_xh<Dual3>(ri, R, [&](int a, Dual3 w) {
        double D = coul(a, 0) - xch(a, 0) - ZB * cA(a);
        if (a == 0) D -= ZA * cB(0);
        E += (ge * D) * w;
      });
      gam = ri[0];
    } else {
      gam = EV / sqrt(r * r + (r0a + r0b) * (r0a + r0b));
      double D = coul(0, 0) - xch(0, 0) - ZB * cA(0) - ZA * cB(0);
      E += (ge * D) * gam;
    }
    if (gn != 0.0) E += gn * core_core<Dual3>(b, ia, ja, r, gam);
  }
  // resonance term 2 sum P_AB H_AB with H_AB = S (beta_i + beta_j)/2
  Dual3 di[4][4];
  overlap_block<Dual3>((int)par(b, SEQM_P_QN, ia), (int)par(b, SEQM_P_QN, ja), r, xv, yv, zv, par(b, SEQM_P_ZS, ia),
                       par(b, SEQM_P_ZP, ia), par(b, SEQM_P_ZS, ja), par(b, SEQM_P_ZP, ja), di);
  const double bi[4] = {par(b, SEQM_P_BS, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia)};
  const double bj[4] = {par(b, SEQM_P_BS, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja)};
  double dbs_i = 0.0, dbp_i = 0.0, dbs_j = 0.0, dbp_j = 0.0;
  for (int u = 0; u < ni_; ++u)
    for (int v = 0; v < nj_; ++v) {
      const double pv = ge * (EXC ? Pab[u][v] + Dab[u][v] : Pab[u][v]);
      E += (pv * (bi[u] + bj[v])) * di[u][v];
      const double ps = pv * di[u][v].v;
      if (u == 0) dbs_i += ps; else dbp_i += ps;
      if (v == 0) dbs_j += ps; else dbp_j += ps;
    }
  out[0] = E.d0;
  out[1] = E.d1;
  out[2] = E.d2;
  out[3] = dbs_i;
  out[4] = dbp_i;
  out[5] = dbs_j;
  out[6] = dbp_j;
}

// per atom: dE/dR = sum over pairs where the atom is second (+g) and first (-g);
// parameter gradients: beta from the pair terms, U from the diagonal density
__global__ void k_atom_grad(seqm_batch b, const double *__restrict__ P, const double *__restrict__ Pbeta,
                            const double *__restrict__ gE, const double *__restrict__ work, double *__restrict__ dR,
                            double *__restrict__ dpar) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natoms) return;
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
  const int norb = b.mol_norb[m], la = a - a0;
  const int xx0 = b.mol_xx_off[m], xh0 = b.nxx + b.mol_xh_off[m], hh0 = b.nxx + b.nxh + b.mol_hh_off[m];
  double g0 = 0.0, g1 = 0.0, g2 = 0.0, dbs = 0.0, dbp = 0.0;
  auto first = [&](int p) {  // atom is pair_i: dE/dRi = -g
    const double *w = work + (size_t)GRAD_STRIDE * p;
    g0 -= w[0]; g1 -= w[1]; g2 -= w[2]; dbs += w[3]; dbp += w[4];
  };
  auto second = [&](int p) {  // atom is pair_j: dE/dRj = +g
    const double *w = work + (size_t)GRAD_STRIDE * p;
    g0 += w[0]; g1 += w[1]; g2 += w[2]; dbs += w[5]; dbp += w[6];
  };
  const double *Pm = P + b.mol_mat_off[m], *Qm = Pbeta ? Pbeta + b.mol_mat_off[m] : nullptr;
  auto ptot = [&](int o) { return Pm[(size_t)o * norb + o] + (Qm ? Qm[(size_t)o * norb + o] : 0.0); };
  double duss, dupp = 0.0;
  if (la < nh) {
    for (int j = la + 1; j < nh; ++j) first(xx0 + tri_index(la, j, nh));
    for (int h = 0; h < ny; ++h) first(xh0 + la * ny + h);
    for (int i = 0; i < la; ++i) second(xx0 + tri_index(i, la, nh));
    const int o = 4 * la;
    duss = ptot(o);
    for (int k = 1; k < 4; ++k) dupp += ptot(o + k);
  } else {
    const int h = la - nh, o = 3 * nh + la;
    for (int i = 0; i < nh; ++i) second(xh0 + i * ny + h);
    for (int g = h + 1; g < ny; ++g) first(hh0 + tri_index(h, g, ny));
    for (int g = 0; g < h; ++g) second(hh0 + tri_index(g, h, ny));
    duss = ptot(o);
  }
  dR[3 * a] = g0;
  dR[3 * a + 1] = g1;
  dR[3 * a + 2] = g2;
  if (dpar) {
    const size_t n = b.natoms;
    dpar[a] = gE[m] * duss;
    dpar[n + a] = gE[m] * dupp;
    dpar[2 * n + a] = dbs;
    dpar[3 * n + a] = dbp;
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_energy_grad(const seqm_batch *bp, const double *P, const double *Pbeta, const double *gE,
                                const double *gN, double *dR, double *dpar, double *work, void *stream) {
  if (!bp || !P || !gE || !gN || !dR || !work) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.natoms == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (npairs > 0) k_pair_grad<false><<<(npairs + 127) / 128, 128, 0, s>>>(b, P, Pbeta, gE, gN, work, nullptr, nullptr);
  k_atom_grad<<<(b.natoms + 127) / 128, 128, 0, s>>>(b, P, Pbeta, gE, work, dR, dpar);
  return launch_check();
}

extern "C" int seqm_energy_grad_excited(const seqm_batch *bp, const double *P, const double *D, const double *R,
                                        const double *gE, const double *gN, double *dR, double *work,
                                        void *stream) {
  if (!bp || !P || !D || !R || !gE || !gN || !dR || !work) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.natoms == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (npairs > 0) k_pair_grad<true><<<(npairs + 127) / 128, 128, 0, s>>>(b, P, nullptr, gE, gN, work, D, R);
  k_atom_grad<<<(b.natoms + 127) / 128, 128, 0, s>>>(b, P, nullptr, gE, work, dR, nullptr);
  return launch_check();
}
