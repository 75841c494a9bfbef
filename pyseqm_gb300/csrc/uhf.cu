// Unrestricted Hartree-Fock (UHF) Fock build and energy / convergence test (FP64).
//
// fock_u_batch (seqm/seqm_functions/fock_u_batch.py:18-100): for spin s (alpha, beta)
//   F_s = H + J(Pa + Pb) - K(P_s) + one-centre terms of (P_tot, P_s, P_other)
// with the Coulomb part J of the total density exactly as in the restricted build, the
// exchange part K of the spin density (instead of half the total), and the spin-resolved
// one-centre terms of _one_center_u (:103-146).  Same thread layout as the restricted
// k_fock: one warp per atom for the diagonal blocks (Coulomb gathered over the partners),
// one thread per pair for the off-diagonal blocks; both spins are written by the same
// thread, every element once.
//
// Energy (energy.py:44-45): 1/2 sum [(Pa + Pb) H + Pa Fa + Pb Fb]; the convergence test of
// get_error (scf_loop.py:106-147) on the spin-summed density change.
#include <math.h>

#include "common.cuh"

namespace seqm {
namespace {

__device__ __forceinline__ bool live(const uint8_t *active, int m) { return active == nullptr || active[m]; }

__device__ __forceinline__ double allsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// packed weighted total density of a heavy atom's diagonal block
__device__ __forceinline__ void packed_total(const double *Pa, const double *Pb, int norb, int o, double *PX) {
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    const int r = k10_row(k), c = k10_col(k);
    const size_t i = (size_t)(o + r) * norb + o + c;
    PX[k] = (Pa[i] + Pb[i]) * (r == c ? 1.0 : 2.0);
  }
}

__device__ void fock_u_diag(const seqm_batch &b, int a, int lane, const double *__restrict__ Pa,
                            const double *__restrict__ Pb, const double *__restrict__ H,
                            const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                            const double *__restrict__ w_hh, double *__restrict__ Fa, double *__restrict__ Fb) {
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
  const int norb = b.mol_norb[m], la = a - a0;
  const int xx0 = b.mol_xx_off[m], xh0 = b.mol_xh_off[m], hh0 = b.mol_hh_off[m];
  const size_t mo = b.mol_mat_off[m];
  const double *A = Pa + mo, *B = Pb + mo, *Hm = H + mo;
  double *FA = Fa + mo, *FB = Fb + mo;
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
        packed_total(A, B, norb, 4 * j, PB);
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
        const size_t i = (size_t)oh * norb + oh;
        const double ph = A[i] + B[i];
#pragma unroll
        for (int k = 0; k < 10; ++k) f[k] += ph * w[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) f[k] = allsum(f[k]);
    const double gsp = par(b, SEQM_P_GSP, a), gpp = par(b, SEQM_P_GPP, a);
    const double gp2 = par(b, SEQM_P_GP2, a), hsp = par(b, SEQM_P_HSP, a);
    double T[4][4], S[2][4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const size_t i = (size_t)(o + r) * norb + o + c;
        S[0][r][c] = A[i];
        S[1][r][c] = B[i];
        T[r][c] = A[i] + B[i];
      }
    const double Tpt = T[1][1] + T[2][2] + T[3][3];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const double(&Ps)[4][4] = S[s];
      const double(&Po)[4][4] = S[1 - s];
      const double Spt = Ps[1][1] + Ps[2][2] + Ps[3][3];
      double *Fm = s == 0 ? FA : FB;
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        const int r = k10_row(k), c = k10_col(k);
        double oc;
        if (r == 0 && c == 0) oc = Po[0][0] * gss + Tpt * gsp - Spt * hsp;
        else if (r == c)
          oc = T[0][0] * gsp - Ps[0][0] * hsp + Po[r][r] * gpp + (Tpt - T[r][r]) * gp2 -
               0.5 * (Spt - Ps[r][r]) * (gpp - gp2);
        else if (r == 0) oc = 2.0 * T[0][c] * hsp - Ps[0][c] * (hsp + gsp);
        else oc = T[r][c] * (gpp - gp2) - 0.5 * Ps[r][c] * (gpp + gp2);
        if (lane == k) {
          const double v = Hm[(size_t)(o + r) * norb + o + c] + oc + f[k];
          Fm[(size_t)(o + r) * norb + o + c] = v;
          Fm[(size_t)(o + c) * norb + o + r] = v;
        }
      }
    }
  } else {
    const int h = la - nh, o = 3 * nh + la;
    double f = 0.0;
    for (int q = lane; q < nat - 1; q += 32) {
      if (q < nh) {
        const double *w = w_xh + (size_t)10 * (xh0 + q * ny + h);
        double PB[10];
        packed_total(A, B, norb, 4 * q, PB);
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 10; ++k) s += PB[k] * w[k];
        f += s;
      } else {
        const int g0 = q - nh, g = g0 < h ? g0 : g0 + 1, og = 4 * nh + g;
        const double w = w_hh[hh0 + (g < h ? tri_index(g, h, ny) : tri_index(h, g, ny))];
        const size_t i = (size_t)og * norb + og;
        f += w * (A[i] + B[i]);
      }
    }
    f = allsum(f);
    if (lane == 0) {
      const size_t i = (size_t)o * norb + o;
      FA[i] = Hm[i] + B[i] * gss + f;  // the opposite spin's s population (_one_center_u, :118)
      FB[i] = Hm[i] + A[i] * gss + f;
    }
  }
}

__global__ void __launch_bounds__(128) k_fock_u(seqm_batch b, const double *__restrict__ Pa,
                                                const double *__restrict__ Pb, const double *__restrict__ H,
                                                const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                                                const double *__restrict__ w_hh, double *__restrict__ Fa,
                                                double *__restrict__ Fb, const uint8_t *__restrict__ active) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ndiag = 32LL * b.natoms;
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (t < ndiag) {
    const int a = (int)(t >> 5);
    if (!live(active, b.atom_mol[a])) return;
    fock_u_diag(b, a, (int)(t & 31), Pa, Pb, H, w_xx, w_xh, w_hh, Fa, Fb);
    return;
  }
  if (t - ndiag >= npairs) return;
  // off-diagonal block of pair p: F_s,AB = H_AB - sum P_s,AB (mu lam | nu sig)
  const int p = (int)(t - ndiag);
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  if (!live(active, m)) return;
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m];
  const int oi = atom_ao(ia - a0, nh), oj = atom_ao(ja - a0, nh);
  const size_t mo = b.mol_mat_off[m];
  const double *Hm = H + mo;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const double *Pm = (s == 0 ? Pa : Pb) + mo;
    double *Fm = (s == 0 ? Fa : Fb) + mo;
    if (p < b.nxx) {
      const double *w = w_xx + (size_t)100 * p;
      double Pp[4][4];
#pragma unroll
      for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int q = 0; q < 4; ++q) Pp[l][q] = -Pm[(size_t)(oi + l) * norb + oj + q];
#pragma unroll
      for (int mu = 0; mu < 4; ++mu)
#pragma unroll
        for (int nu = 0; nu < 4; ++nu) {
          double k = 0.0;
#pragma unroll
          for (int l = 0; l < 4; ++l)
#pragma unroll
            for (int q = 0; q < 4; ++q) k += w[kind(mu, l) * 10 + kind(nu, q)] * Pp[l][q];
          const double v = Hm[(size_t)(oi + mu) * norb + oj + nu] + k;
          Fm[(size_t)(oi + mu) * norb + oj + nu] = v;
          Fm[(size_t)(oj + nu) * norb + oi + mu] = v;
        }
    } else if (p < b.nxx + b.nxh) {
      const double *w = w_xh + (size_t)10 * (p - b.nxx);
      double Pp[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) Pp[l] = -Pm[(size_t)(oi + l) * norb + oj];
#pragma unroll
      for (int mu = 0; mu < 4; ++mu) {
        double k = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l) k += w[kind(mu, l)] * Pp[l];
        const double v = Hm[(size_t)(oi + mu) * norb + oj] + k;
        Fm[(size_t)(oi + mu) * norb + oj] = v;
        Fm[(size_t)oj * norb + oi + mu] = v;
      }
    } else {
      const double v = Hm[(size_t)oi * norb + oj] - w_hh[p - b.nxx - b.nxh] * Pm[(size_t)oi * norb + oj];
      Fm[(size_t)oi * norb + oj] = v;
      Fm[(size_t)oj * norb + oi] = v;
    }
  }
}

constexpr int NT_U = 256;

template <bool MAX>
__device__ double ureduce(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = MAX ? fmax(v, u) : v + u;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = red[0];
  for (int w = 1; w < NT_U / 32; ++w) s = MAX ? fmax(s, red[w]) : s + red[w];
  __syncthreads();
  return s;
}

// energy of both spins and (when Pao != NULL) the convergence test; one CTA per molecule
__global__ void __launch_bounds__(NT_U) k_energy_error_u(seqm_batch b, const double *__restrict__ Pa,
                                                         const double *__restrict__ Pb,
                                                         const double *__restrict__ Pao,
                                                         const double *__restrict__ Pbo, const double *__restrict__ H,
                                                         const double *__restrict__ Fa, const double *__restrict__ Fb,
                                                         double *Eelec, double *Eout, double *err, double *dm_err,
                                                         double *dm_el, uint8_t *active, double eps) {
  __shared__ double red[NT_U / 32];
  const int m = blockIdx.x;
  if (!live(active, m)) return;
  const int n = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m], nn = (size_t)n * n;
  double e = 0.0, fro = 0.0, mx = 0.0;
  for (size_t i = threadIdx.x; i < nn; i += NT_U) {
    const double a = Pa[mo + i], c = Pb[mo + i];
    e += (a + c) * H[mo + i] + a * Fa[mo + i] + c * Fb[mo + i];
    if (Pao) {
      const double d = (a - Pao[mo + i]) + (c - Pbo[mo + i]);
      fro += d * d;
      mx = fmax(mx, fabs(d));
    }
  }
  e = 0.5 * ureduce<false>(e, red);
  if (!Pao) {
    if (threadIdx.x == 0) Eout[m] = e;
    return;
  }
  fro = ureduce<false>(fro, red);
  mx = ureduce<true>(mx, red);
  if (threadIdx.x == 0) {
    Eout[m] = e;
    const double de = e - Eelec[m];
    err[m] = de;
    const bool bad = fabs(de) > eps;
    if (!bad) {
      dm_err[m] = sqrt(fro) / dm_norm(b, m);
      dm_el[m] = mx;
    }
    const bool nc = bad || dm_err[m] > eps * 2.0 || dm_el[m] > eps * 15.0;
    if (nc) Eelec[m] = e;
    if (active) active[m] = nc ? 1 : 0;
  }
}

}  // namespace
}  // namespace seqm

using namespace seqm;

extern "C" int seqm_fock_u(const seqm_batch *bp, const double *Pa, const double *Pb, const double *H,
                           const double *w_xx, const double *w_xh, const double *w_hh, double *Fa, double *Fb,
                           const uint8_t *active, void *stream) {
  if (!bp || !Pa || !Pb || !H || !Fa || !Fb) return SEQM_E_ARG;
  const seqm_batch b = *bp;
  const long long nt = 32LL * b.natoms + b.nxx + b.nxh + b.nhh;
  if (nt == 0) return SEQM_OK;
  k_fock_u<<<(unsigned)((nt + 127) / 128), 128, 0, (cudaStream_t)stream>>>(b, Pa, Pb, H, w_xx, w_xh, w_hh, Fa, Fb,
                                                                           active);
  return launch_check();
}

extern "C" int seqm_energy_error_u(const seqm_batch *bp, const double *Pa, const double *Pb, const double *Pa_old,
                                   const double *Pb_old, const double *H, const double *Fa, const double *Fb,
                                   double *Eelec, double *Eout, double *err, double *dm_err, double *dm_el,
                                   uint8_t *active, double eps, void *stream) {
  if (!bp || !Pa || !Pb || !H || !Fa || !Fb || !Eout) return SEQM_E_ARG;
  if ((Pa_old == nullptr) != (Pb_old == nullptr)) return SEQM_E_ARG;
  const seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  k_energy_error_u<<<b.nmol, NT_U, 0, (cudaStream_t)stream>>>(b, Pa, Pb, Pa_old, Pb_old, H, Fa, Fb, Eelec, Eout, err,
                                                              dm_err, dm_el, active, eps);
  return launch_check();
}
