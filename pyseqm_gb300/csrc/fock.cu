// Fock build, electronic energy + SCF convergence test, density mixing (FP64).
//
// Fock (fock.py:132-181): one thread per atom builds the atom's diagonal block
// (Hcore + one-centre two-electron terms + Coulomb J gathered from all of the
// atom's pairs), one thread per pair builds the off-diagonal block (Hcore +
// exchange K) and its transpose.  Every element of F is written exactly once,
// there are no atomics, and the result is bitwise symmetric.
#include <math.h>

#include "common.cuh"

namespace seqm {

__device__ __forceinline__ bool is_active(const uint8_t *active, int m) { return active == nullptr || active[m]; }

// packed (weighted) density of one atom's diagonal block: PX[k] = w_k P[r_k][c_k]
__device__ __forceinline__ void packed_atom_density(const double *Pm, int norb, int o, bool heavy, double *PX) {
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

__global__ void __launch_bounds__(128) k_fock(seqm_batch b, const double *__restrict__ P, const double *__restrict__ H,
                                              const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                                              const double *__restrict__ w_hh, double *__restrict__ F,
                                              const uint8_t *__restrict__ active) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (t >= b.natoms + npairs) return;
  if (t < b.natoms) {
    // ---------------- diagonal block of atom a
    const int a = t, m = b.atom_mol[a];
    if (!is_active(active, m)) return;
    const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
    const int norb = b.mol_norb[m], la = a - a0;
    const int xx0 = b.mol_xx_off[m], xh0 = b.mol_xh_off[m], hh0 = b.mol_hh_off[m];
    const size_t mo = b.mol_mat_off[m];
    const double *Pm = P + mo, *Hm = H + mo;
    double *Fm = F + mo;
    const double gss = par(b, SEQM_P_GSS, a), gsp = par(b, SEQM_P_GSP, a), gpp = par(b, SEQM_P_GPP, a);
    const double gp2 = par(b, SEQM_P_GP2, a), hsp = par(b, SEQM_P_HSP, a);
    if (la < nh) {
      const int o = 4 * la;
      double f[10], Pd[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) Pd[r][c] = Pm[(size_t)(o + r) * norb + o + c];
      // one-centre terms (fock.py:187-231)
      const double f1 = gsp - 0.5 * hsp, f2 = 1.5 * hsp - 0.5 * gsp, f3 = 1.25 * gp2 - 0.25 * gpp,
                   f4 = 0.75 * gpp - 1.25 * gp2;
      const double Pss = Pd[0][0], Ppt = Pd[1][1] + Pd[2][2] + Pd[3][3];
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        int r = k10_row(k), c = k10_col(k);
        double oc;
        if (r == 0 && c == 0) oc = 0.5 * Pss * gss + Ppt * f1;
        else if (r == c) oc = Pss * f1 + 0.5 * Pd[r][r] * gpp + (Ppt - Pd[r][r]) * f3;
        else if (r == 0) oc = Pd[0][c] * f2;
        else oc = Pd[r][c] * f4;
        f[k] = Hm[(size_t)(o + r) * norb + o + c] + oc;
      }
      // Coulomb from partners B: first-atom pairs (J_B = w . P_B), then second-atom pairs (P_B . w)
      for (int j = la + 1; j < nh; ++j) {
        const double *w = w_xx + (size_t)100 * (xx0 + tri_index(la, j, nh));
        double PB[10];
        packed_atom_density(Pm, norb, 4 * j, true, PB);
#pragma unroll
        for (int k = 0; k < 10; ++k) {
          double s = 0.0;
#pragma unroll
          for (int l = 0; l < 10; ++l) s += PB[l] * w[k * 10 + l];
          f[k] += s;
        }
      }
      for (int h = 0; h < ny; ++h) {
        const double *w = w_xh + (size_t)10 * (xh0 + la * ny + h);
        double ph = Pm[(size_t)(3 * nh + nh + h) * norb + 3 * nh + nh + h];
#pragma unroll
        for (int k = 0; k < 10; ++k) f[k] += ph * w[k];
      }
      for (int i = 0; i < la; ++i) {
        const double *w = w_xx + (size_t)100 * (xx0 + tri_index(i, la, nh));
        double PB[10];
        packed_atom_density(Pm, norb, 4 * i, true, PB);
#pragma unroll
        for (int l = 0; l < 10; ++l) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < 10; ++k) s += PB[k] * w[k * 10 + l];
          f[l] += s;
        }
      }
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        int r = k10_row(k), c = k10_col(k);
        Fm[(size_t)(o + r) * norb + o + c] = f[k];
        Fm[(size_t)(o + c) * norb + o + r] = f[k];
      }
    } else {
      const int h = la - nh, o = 3 * nh + la;
      const double Pss = Pm[(size_t)o * norb + o];
      double f = Hm[(size_t)o * norb + o] + (0.5 * Pss * gss + 0.0 * (gsp - 0.5 * hsp));
      for (int g = h + 1; g < ny; ++g) {
        int og = 3 * nh + nh + g;
        f += w_hh[hh0 + tri_index(h, g, ny)] * Pm[(size_t)og * norb + og];
      }
      for (int i = 0; i < nh; ++i) {
        const double *w = w_xh + (size_t)10 * (xh0 + i * ny + h);
        double PB[10];
        packed_atom_density(Pm, norb, 4 * i, true, PB);
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 10; ++k) s += PB[k] * w[k];
        f += s;
      }
      for (int g = 0; g < h; ++g) {
        int og = 3 * nh + nh + g;
        f += w_hh[hh0 + tri_index(g, h, ny)] * Pm[(size_t)og * norb + og];
      }
      Fm[(size_t)o * norb + o] = f;
    }
    return;
  }
  // ---------------- off-diagonal block of pair p: F_AB = H_AB - 1/2 sum P_AB (mu lam | nu sig)
  const int p = t - b.natoms;
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  if (!is_active(active, m)) return;
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m];
  const int oi = atom_ao(ia - a0, nh), oj = atom_ao(ja - a0, nh);
  const size_t mo = b.mol_mat_off[m];
  const double *Pm = P + mo, *Hm = H + mo;
  double *Fm = F + mo;
  if (p < b.nxx) {
    const double *w = w_xx + (size_t)100 * p;
    double Pp[4][4];
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int s = 0; s < 4; ++s) Pp[l][s] = -0.5 * Pm[(size_t)(oi + l) * norb + oj + s];
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int nu = 0; nu < 4; ++nu) {
        double k = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l)
#pragma unroll
          for (int s = 0; s < 4; ++s) k += w[kind(mu, l) * 10 + kind(nu, s)] * Pp[l][s];
        double v = Hm[(size_t)(oi + mu) * norb + oj + nu] + k;
        Fm[(size_t)(oi + mu) * norb + oj + nu] = v;
        Fm[(size_t)(oj + nu) * norb + oi + mu] = v;
      }
  } else if (p < b.nxx + b.nxh) {
    const double *w = w_xh + (size_t)10 * (p - b.nxx);
    double Pp[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) Pp[l] = -0.5 * Pm[(size_t)(oi + l) * norb + oj];
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
      double k = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) k += w[kind(mu, l)] * Pp[l];
      double v = Hm[(size_t)(oi + mu) * norb + oj] + k;
      Fm[(size_t)(oi + mu) * norb + oj] = v;
      Fm[(size_t)oj * norb + oi + mu] = v;
    }
  } else {
    double v = Hm[(size_t)oi * norb + oj] + w_hh[p - b.nxx - b.nxh] * (-0.5 * Pm[(size_t)oi * norb + oj]);
    Fm[(size_t)oi * norb + oj] = v;
    Fm[(size_t)oj * norb + oi] = v;
  }
}

// ---------------------------------------------------------------- block reductions
template <int NT>
__device__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < NT / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

template <int NT>
__device__ double block_max(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < NT / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    if (threadIdx.x == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

// ------------------------------------------------------ energy + convergence test
// Eelec = 1/2 sum P (H + F) (energy.py:26-49); get_error (scf_loop.py:106-147):
// not converged <=> |dE| > eps or ||dP||_F/(4 natoms) > 2 eps or max|dP| > 15 eps,
// the density terms refreshed only when the energy test passes.
constexpr int NT_RED = 256;
__global__ void __launch_bounds__(NT_RED) k_energy_error(seqm_batch b, const double *__restrict__ P,
                                                         const double *__restrict__ Pold, const double *__restrict__ H,
                                                         const double *__restrict__ F, double *Eelec, double *Eout,
                                                         double *err, double *dm_err, double *dm_el, uint8_t *active,
                                                         double eps) {
  __shared__ double red[NT_RED / 32];
  const int m = blockIdx.x;
  if (!is_active(active, m)) return;
  const int norb = b.mol_norb[m];
  const size_t mo = b.mol_mat_off[m], nn = (size_t)norb * norb;
  double e = 0.0, fro = 0.0, mx = 0.0;
  for (size_t i = threadIdx.x; i < nn; i += NT_RED) {
    double pv = P[mo + i];
    e += pv * (H[mo + i] + F[mo + i]);
    if (Pold) {
      double d = pv - Pold[mo + i];
      fro += d * d;
      mx = fmax(mx, fabs(d));
    }
  }
  e = 0.5 * block_sum<NT_RED>(e, red);
  if (!Pold) {
    if (threadIdx.x == 0) Eout[m] = e;
    return;
  }
  fro = block_sum<NT_RED>(fro, red);
  mx = block_max<NT_RED>(mx, red);
  if (threadIdx.x == 0) {
    Eout[m] = e;
    double de = e - Eelec[m];
    err[m] = de;
    bool bad = fabs(de) > eps;
    if (!bad) {
      int nat = b.mol_atom_off[m + 1] - b.mol_atom_off[m];
      dm_err[m] = sqrt(fro) / (4.0 * nat);
      dm_el[m] = mx;
    }
    bool nc = bad || dm_err[m] > eps * 2.0 || dm_el[m] > eps * 15.0;
    if (nc) Eelec[m] = e;
    if (active) active[m] = nc ? 1 : 0;
  }
}

// ------------------------------------------------------------------ mixing
// linear: P <- alpha P + (1 - alpha) Pnew (scf_loop.py:258-267);
// adaptive (scf_loop.py:360-420): every third iteration extrapolate
// P <- (1+FAC) Pnew - FAC P with FAC from the diagonal history; the diagonal is
// damped (|step| <= 0.05 after iteration 4), clamped to [0, 2] and renormalised
// to the new trace in at most 20 passes.  Each molecule stops its own
// renormalisation (the reference stops when the whole padded batch is done).
constexpr int NT_MIX = 256;
__global__ void __launch_bounds__(NT_MIX) k_mix(seqm_batch b, double *__restrict__ P, const double *__restrict__ Pnew,
                                                double *__restrict__ Pold, double *__restrict__ old2,
                                                const int64_t *__restrict__ row_off, int32_t *__restrict__ kit,
                                                int linear, double alpha, const uint8_t *__restrict__ active) {
  extern __shared__ double sm[];
  __shared__ double red[NT_MIX / 32];
  __shared__ int k_sh;
  const int m = blockIdx.x;
  if (!is_active(active, m)) return;
  const int n = b.mol_norb[m];
  if (threadIdx.x == 0) {
    k_sh = kit[m] + 1;  // 1-based iteration number of this molecule
    kit[m] = k_sh;
  }
  __syncthreads();
  const size_t mo = b.mol_mat_off[m];
  double *Pm = P + mo, *Po = Pold + mo;
  const double *Pn = Pnew + mo;
  if (linear) {
    const double oma = 1.0 - alpha;
    for (size_t i = threadIdx.x; i < (size_t)n * n; i += NT_MIX) {
      double pv = Pm[i];
      Po[i] = pv;
      Pm[i] = alpha * pv + oma * Pn[i];
    }
    return;
  }
  const int k = k_sh;
  double *dprev = sm, *di = sm + n;
  double *o2 = old2 + row_off[m];
  double num = 0.0, den = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_MIX) {
    double dp = Pm[(size_t)i * n + i], dc = Pn[(size_t)i * n + i];
    dprev[i] = dp;
    double d1 = dc - dp, d2 = dc - 2.0 * dp + o2[i];
    num += d1 * d1;
    den += d2 * d2;
  }
  const bool third = (k % 3) == 0;
  double fac = 0.0;
  if (third) {
    num = block_sum<NT_MIX>(num, red);
    den = block_sum<NT_MIX>(den, red);
    fac = (den > 0.0 && num < 100.0 * den) ? sqrt(num / den) : 0.0;
  } else {
    __syncthreads();
  }
  // off-diagonal (and provisional diagonal) update
  for (size_t idx = threadIdx.x; idx < (size_t)n * n; idx += NT_MIX) {
    double pv = Pm[idx];
    Po[idx] = pv;
    Pm[idx] = third ? (1.0 + fac) * Pn[idx] - fac * pv : Pn[idx];
  }
  // diagonal: damp, clamp, renormalise
  const double damp = k > 4 ? 0.05 : 1.0e10;
  double s0 = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_MIX) {
    double dc = Pn[(size_t)i * n + i], dp = dprev[i];
    double delta = dc - dp;
    double v = fabs(delta) > damp ? dp + (delta > 0.0 ? 1.0 : (delta < 0.0 ? -1.0 : 0.0)) * damp : dc + fac * delta;
    di[i] = fmin(fmax(v, 0.0), 2.0);
    s0 += dc;
  }
  double sum0 = block_sum<NT_MIX>(s0, red);
  for (int pass = 0; pass < 20; ++pass) {
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MIX) s2 += di[i];
    double sum2 = block_sum<NT_MIX>(s2, red);
    double sum3 = sum2 > 1.0e-3 ? sum0 / sum2 : 0.0;
    if (!(sum2 > 1.0e-3) || fabs(sum3 - 1.0) <= 1.0e-5) break;
    double nfull = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MIX) {
      double sc = fmax(di[i] * sum3, 0.0);
      bool full = sc > 2.0;
      di[i] = full ? 2.0 : sc;
      nfull += full ? 1.0 : 0.0;
    }
    nfull = block_sum<NT_MIX>(nfull, red);
    sum0 = sum0 - nfull * 2.0;
  }
  for (int i = threadIdx.x; i < n; i += NT_MIX) {
    Pm[(size_t)i * n + i] = di[i];
    o2[i] = dprev[i];
  }
}

// ----------------------------------------------------------- initial density
__global__ void k_initial_density(seqm_batch b, double *__restrict__ P) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natoms) return;
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m], la = a - a0;
  double *Pm = P + b.mol_mat_off[m];
  if (la < nh) {
    double v = par(b, SEQM_P_TORE, a) / 4.0;
    for (int k = 0; k < 4; ++k) Pm[(size_t)(4 * la + k) * norb + 4 * la + k] = v;
  } else {
    int o = 3 * nh + la;
    Pm[(size_t)o * norb + o] = 1.0;
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_fock(const seqm_batch *bp, const double *P, const double *H, const double *w_xx,
                         const double *w_xh, const double *w_hh, double *F, const uint8_t *active, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  long long nt = (long long)b.natoms + b.nxx + b.nxh + b.nhh;
  if (nt == 0) return SEQM_OK;
  k_fock<<<(unsigned)((nt + 127) / 128), 128, 0, (cudaStream_t)stream>>>(b, P, H, w_xx, w_xh, w_hh, F, active);
  return launch_check();
}

extern "C" int seqm_energy_error(const seqm_batch *bp, const double *P, const double *Pold, const double *H,
                                 const double *F, double *Eelec, double *Eout, double *err, double *dm_err,
                                 double *dm_el, uint8_t *active, double eps, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  k_energy_error<<<b.nmol, NT_RED, 0, (cudaStream_t)stream>>>(b, P, Pold, H, F, Eelec, Eout, err, dm_err, dm_el,
                                                             active, eps);
  return launch_check();
}

extern "C" int seqm_mix(const seqm_batch *bp, double *P, const double *Pnew, double *Pold, double *old2,
                        const int64_t *mol_row_off, int32_t *k, int linear, double alpha, const uint8_t *active,
                        void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  size_t smem = linear ? 0 : (size_t)2 * b.max_norb * sizeof(double);
  if (smem > 200 * 1024) return SEQM_E_TOO_LARGE;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(k_mix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SEQM_E_CUDA;
  k_mix<<<b.nmol, NT_MIX, smem, (cudaStream_t)stream>>>(b, P, Pnew, Pold, old2, mol_row_off, k, linear, alpha, active);
  return launch_check();
}

extern "C" int seqm_initial_density(const seqm_batch *bp, double *P, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.natoms == 0) return SEQM_OK;
  k_initial_density<<<(b.natoms + 127) / 128, 128, 0, (cudaStream_t)stream>>>(b, P);
  return launch_check();
}
