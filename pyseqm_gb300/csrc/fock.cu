// Fock build, electronic energy + SCF convergence test, density mixing (FP64).
//
// Fock (fock.py:132-181): one warp per atom builds the atom's diagonal block
// (Hcore + one-centre two-electron terms + Coulomb J gathered from all of the
// atom's pairs; see fock_diag), one thread per pair builds the off-diagonal block
// (Hcore + exchange K) and its transpose.  Every element of F is written exactly
// once, there are no atomics, and the result is bitwise symmetric.  The build is
// bound by the FP64 pipe (about 2 (456 XX + 36 XH + 3 HH) flops per pair against
// 8 (100 XX + 10 XH + 1 HH) integral bytes): the mapping keeps every FP64
// instruction's lanes busy and issues nothing in FP64 but the contractions.
//
// The energy / convergence test and the mixing run as thread-block clusters of
// up to 16 CTAs per molecule (more CTAs for larger molecules); the energy sums are
// combined through distributed shared memory in a fixed order.
#include <cooperative_groups.h>
#include <math.h>

#include "common.cuh"

namespace seqm {

namespace cg = cooperative_groups;

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

// butterfly sum: every lane ends with the same value, summed in the same order
__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// diagonal block of atom a (fock.py:187-231 one-centre terms, :277-294 Coulomb), one warp.
//
// A heavy atom's warp is three groups of ten lanes: lane k of group g accumulates output k of
// the packed block (k10_row/k10_col order) over the partners q = g, g + 3, g + 6, ..., one
// fused multiply-add per integral, and the three group sums are combined by two shuffles.
// Every FP64 instruction of the warp thus carries 30 useful lanes: the Coulomb term is the
// kernel's largest FP64 cost after the exchange blocks, and GB300's FP64 pipe, not memory,
// bounds the Fock build.  A hydrogen's warp splits its partners over the lanes and sums with a
// butterfly (one output).  The sums run in a fixed order, so the result is deterministic.
__device__ __forceinline__ void fock_diag(const seqm_batch &b, int a, int lane, const double *__restrict__ P,
                                          const double *__restrict__ H, const double *__restrict__ w_xx,
                                          const double *__restrict__ w_xh, const double *__restrict__ w_hh,
                                          double *__restrict__ F) {
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
  const int norb = b.mol_norb[m], la = a - a0;
  const int xx0 = b.mol_xx_off[m], xh0 = b.mol_xh_off[m], hh0 = b.mol_hh_off[m];
  const size_t mo = b.mol_mat_off[m];
  const double *Pm = P + mo, *Hm = H + mo;
  double *Fm = F + mo;
  const double gss = par(b, SEQM_P_GSS, a);
  if (la < nh) {
    const int o = 4 * la;
    const int g = lane / 10, k = lane - 10 * g;  // lanes 30, 31: g = 3, no partners
    double f = 0.0;
    for (int q = g; g < 3 && q < nat - 1; q += 3) {
      if (q < nh - 1) {
        const int j = q < la ? q : q + 1;
        double PB[10];
        packed_atom_density(Pm, norb, 4 * j, true, PB);
        if (j > la) {  // pair (A, B): row k of w, contiguous
          const double2 *w2 = reinterpret_cast<const double2 *>(w_xx + (size_t)100 * (xx0 + tri_index(la, j, nh)) +
                                                                10 * k);
#pragma unroll
          for (int l = 0; l < 5; ++l) {
            const double2 v = __ldg(w2 + l);
            f = fma(v.x, PB[2 * l], f);
            f = fma(v.y, PB[2 * l + 1], f);
          }
        } else {  // pair (B, A): column k of w
          const double *w = w_xx + (size_t)100 * (xx0 + tri_index(j, la, nh)) + k;
#pragma unroll
          for (int l = 0; l < 10; ++l) f = fma(PB[l], __ldg(w + 10 * l), f);
        }
      } else {
        const int h = q - (nh - 1), oh = 4 * nh + h;
        f = fma(Pm[(size_t)oh * norb + oh], __ldg(w_xh + (size_t)10 * (xh0 + la * ny + h) + k), f);
      }
    }
    const double f1 = __shfl_sync(0xffffffffu, f, (lane + 10) & 31);
    const double f2 = __shfl_sync(0xffffffffu, f, (lane + 20) & 31);
    if (lane < 10) {
      const double J = (f + f1) + f2;
      // one-centre terms (fock.py:187-231)
      const int r = k10_row(k), c = k10_col(k);
      const double gsp = par(b, SEQM_P_GSP, a), gpp = par(b, SEQM_P_GPP, a);
      const double gp2 = par(b, SEQM_P_GP2, a), hsp = par(b, SEQM_P_HSP, a);
      const double c1 = gsp - 0.5 * hsp, c2 = 1.5 * hsp - 0.5 * gsp, c3 = 1.25 * gp2 - 0.25 * gpp,
                   c4 = 0.75 * gpp - 1.25 * gp2;
      const double Pss = Pm[(size_t)o * norb + o];
      const double Ppt = Pm[(size_t)(o + 1) * norb + o + 1] + Pm[(size_t)(o + 2) * norb + o + 2] +
                         Pm[(size_t)(o + 3) * norb + o + 3];
      const double Prc = Pm[(size_t)(o + r) * norb + o + c];
      double oc;
      if (r == 0 && c == 0) oc = 0.5 * Pss * gss + Ppt * c1;
      else if (r == c) oc = Pss * c1 + 0.5 * Prc * gpp + (Ppt - Prc) * c3;
      else if (r == 0) oc = Prc * c2;
      else oc = Prc * c4;
      const double v = Hm[(size_t)(o + r) * norb + o + c] + oc + J;
      Fm[(size_t)(o + r) * norb + o + c] = v;
      Fm[(size_t)(o + c) * norb + o + r] = v;
    }
  } else {
    const int h = la - nh, o = 3 * nh + la;
    double f = 0.0;
    for (int q = lane; q < nat - 1; q += 32) {
      if (q < nh) {
        const double2 *w2 = reinterpret_cast<const double2 *>(w_xh + (size_t)10 * (xh0 + q * ny + h));
        double PB[10];
        packed_atom_density(Pm, norb, 4 * q, true, PB);
#pragma unroll
        for (int l = 0; l < 5; ++l) {
          const double2 v = __ldg(w2 + l);
          f = fma(v.x, PB[2 * l], f);
          f = fma(v.y, PB[2 * l + 1], f);
        }
      } else {
        const int g0 = q - nh, g = g0 < h ? g0 : g0 + 1, og = 4 * nh + g;
        const double w = w_hh[hh0 + (g < h ? tri_index(g, h, ny) : tri_index(h, g, ny))];
        f = fma(w, Pm[(size_t)og * norb + og], f);
      }
    }
    f = warp_allsum(f);
    if (lane == 0) {
      const double Pss = Pm[(size_t)o * norb + o];
      Fm[(size_t)o * norb + o] = Hm[(size_t)o * norb + o] + 0.5 * Pss * gss + f;
    }
  }
}

__global__ void __launch_bounds__(128) k_fock(seqm_batch b, const double *__restrict__ P, const double *__restrict__ H,
                                              const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                                              const double *__restrict__ w_hh, double *__restrict__ F,
                                              const uint8_t *__restrict__ active) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ndiag = 32LL * b.natoms;  // one warp per atom; warps never straddle the two roles
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (t < ndiag) {
    const int a = (int)(t >> 5);
    if (!is_active(active, b.atom_mol[a])) return;
    fock_diag(b, a, (int)(t & 31), P, H, w_xx, w_xh, w_hh, F);
    return;
  }
  if (t - ndiag >= npairs) return;
  // ---------------- off-diagonal block of pair p: F_AB = H_AB - 1/2 sum P_AB (mu lam | nu sig)
  const int p = (int)(t - ndiag);
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  if (!is_active(active, m)) return;
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m];
  const int oi = atom_ao(ia - a0, nh), oj = atom_ao(ja - a0, nh);
  const size_t mo = b.mol_mat_off[m];
  const double *Pm = P + mo, *Hm = H + mo;
  double *Fm = F + mo;
  if (p < b.nxx) {
    // K(mu, nu) = sum_{l,s} (mu l | nu s) P_AB(l, s), F_AB = H_AB - K / 2 (the halving is exact)
    const double2 *w2 = reinterpret_cast<const double2 *>(w_xx + (size_t)100 * p);
    double w[100];
#pragma unroll
    for (int i = 0; i < 50; ++i) {
      const double2 v = __ldg(w2 + i);
      w[2 * i] = v.x;
      w[2 * i + 1] = v.y;
    }
    double Pp[4][4];
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int s = 0; s < 4; ++s) Pp[l][s] = Pm[(size_t)(oi + l) * norb + oj + s];
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int nu = 0; nu < 4; ++nu) {
        double k = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l)
#pragma unroll
          for (int s = 0; s < 4; ++s) k = fma(w[kind(mu, l) * 10 + kind(nu, s)], Pp[l][s], k);
        const double v = fma(-0.5, k, Hm[(size_t)(oi + mu) * norb + oj + nu]);
        Fm[(size_t)(oi + mu) * norb + oj + nu] = v;
        Fm[(size_t)(oj + nu) * norb + oi + mu] = v;
      }
  } else if (p < b.nxx + b.nxh) {
    const double *w = w_xh + (size_t)10 * (p - b.nxx);
    double Pp[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) Pp[l] = Pm[(size_t)(oi + l) * norb + oj];
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
      double k = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) k = fma(__ldg(w + kind(mu, l)), Pp[l], k);
      const double v = fma(-0.5, k, Hm[(size_t)(oi + mu) * norb + oj]);
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
// not converged <=> |dE| > eps or ||dP||_F/(4 natoms + 9 nsuper) > 2 eps or max|dP| > 15 eps,
// the density terms refreshed only when the energy test passes.
//
// active[m] == 2 marks a molecule whose density of this iteration came from the tensor-core SP2
// without its FP64-accurate McWeeny step (that step costs about three times the rest of the
// iteration at thousands of basis functions, and the SCF tolerates the FP32-level density while
// the energy still moves by more than REFINE_DE).  Such a molecule is never retired on that
// density; it turns to 1 (refined densities from the next iteration on) once |dE| < REFINE_DE or
// after REFINE_ITERS iterations, and stays there.  The FP32-level density moves the energy by
// ~1e-3 eV between iterations at 6000 basis functions, far below REFINE_DE.
//
// One cluster of cs CTAs per molecule.  The molecule's elements are cut into ns
// interleaved slices (slice s: elements s*NT + t + k*ns*NT; ns grows with the
// molecule's size up to EE_SLICES); CTA rank r sums the slices s with s % cs == r,
// and rank 0 adds the slice sums in slice order through distributed shared memory,
// so the result does not depend on cs.
constexpr double REFINE_DE = 1.0;  // eV
constexpr int REFINE_ITERS = 8;
__device__ __forceinline__ void finish_error(const seqm_batch &b, int m, double e, double fro, double mx, double *Eelec,
                                        double *err, double *dm_err, double *dm_el, uint8_t *active, double eps,
                                        const double *diis_err, int *nactive, const int32_t *kit) {
  double de = e - Eelec[m];
  err[m] = de;
  // with DIIS, also max |F P - P F| > 50 eps (scf_loop.py:130-132)
  bool bad = fabs(de) > eps || (diis_err != nullptr && diis_err[m] > 50.0 * eps);
  if (!bad) {
    dm_err[m] = sqrt(fro) / dm_norm(b, m);
    dm_el[m] = mx;
  }
  const uint8_t a = active ? active[m] : 1;
  bool nc = bad || dm_err[m] > eps * 2.0 || dm_el[m] > eps * 15.0 || a == 2;
  if (nc) Eelec[m] = e;
  if (active) {
    const bool keep_unrefined = a == 2 && !(fabs(de) < REFINE_DE) && !(kit && kit[m] >= REFINE_ITERS);
    active[m] = !nc ? 0 : (keep_unrefined ? 2 : 1);
  }
  if (nc && nactive) atomicAdd(nactive, 1);
}

constexpr int NT_RED = 512, EE_SLICES = 16, EE_UNROLL = 4;
constexpr int EE_WARP_MAX = 160;  // larger molecules take the cluster kernel
__global__ void __launch_bounds__(NT_RED) k_energy_error(seqm_batch b, const double *__restrict__ P,
                                                         const double *__restrict__ Pold, const double *__restrict__ H,
                                                         const double *__restrict__ F, double *Eelec, double *Eout,
                                                         double *err, double *dm_err, double *dm_el, uint8_t *active,
                                                         double eps, const double *__restrict__ diis_err,
                                                         int *__restrict__ nactive,
                                                         const int32_t *__restrict__ kit, int cs) {
  __shared__ double wred[NT_RED / 32][3 * EE_SLICES];
  __shared__ double part[3 * EE_SLICES];
  cg::cluster_group cl = cg::this_cluster();
  const int m = blockIdx.x / cs, r = (int)cl.block_rank();
  if (!is_active(active, m)) return;  // uniform over the cluster
  const int norb = b.mol_norb[m];
  if (norb <= EE_WARP_MAX) return;  // k_energy_error_warp's molecule
  const size_t mo = b.mol_mat_off[m], nn = (size_t)norb * norb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // slices of this molecule: one per 8192 elements, at most EE_SLICES (a function of its size only)
  const int ns = (int)min((size_t)EE_SLICES, (nn + 8191) / 8192);
  const size_t stride = (size_t)ns * NT_RED;
  for (int s = r; s < ns; s += cs) {  // the slices of this CTA
    double e = 0.0, fro = 0.0, mx = 0.0;
    for (size_t i = (size_t)s * NT_RED + threadIdx.x; i < nn; i += EE_UNROLL * stride) {
      double pv[EE_UNROLL], hf[EE_UNROLL], po[EE_UNROLL];
#pragma unroll
      for (int u = 0; u < EE_UNROLL; ++u) {  // independent loads in flight
        const size_t j = i + u * stride;
        const bool in = j < nn;
        pv[u] = in ? P[mo + j] : 0.0;
        hf[u] = in ? H[mo + j] + F[mo + j] : 0.0;
        po[u] = (in && Pold) ? Pold[mo + j] : pv[u];
      }
#pragma unroll
      for (int u = 0; u < EE_UNROLL; ++u) {
        e += pv[u] * hf[u];
        const double d = pv[u] - po[u];
        fro += d * d;
        mx = fmax(mx, fabs(d));
      }
    }
    double v3[3] = {e, fro, mx};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double v = v3[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = q == 2 ? fmax(v, u) : v + u;
      }
      if (lane == 0) wred[warp][3 * s + q] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < 3 * ns && (threadIdx.x / 3) % cs == r) {
    const int j = threadIdx.x;
    double v = wred[0][j];
    for (int w = 1; w < NT_RED / 32; ++w) v = (j % 3 == 2) ? fmax(v, wred[w][j]) : v + wred[w][j];
    part[j] = v;
  }
  cl.sync();
  if (r == 0 && threadIdx.x == 0) {
    double e = 0.0, fro = 0.0, mx = 0.0;
    for (int s = 0; s < ns; ++s) {
      const double *q = cl.map_shared_rank(part, s % cs);
      e += q[3 * s];
      fro += q[3 * s + 1];
      mx = fmax(mx, q[3 * s + 2]);
    }
    e *= 0.5;
    Eout[m] = e;
    if (Pold) finish_error(b, m, e, fro, mx, Eelec, err, dm_err, dm_el, active, eps, diis_err, nactive, kit);
  }
  cl.sync();  // the other CTAs' shared memory stays alive until rank 0 has read it
}

// Molecules of up to EE_WARP_MAX basis functions: one warp per molecule streams its n^2
// elements (four independent loads per element, 32 B, coalesced across the lanes) and sums with
// a butterfly; eight molecules per CTA.  A molecule's sums depend only on its own size, as in
// the cluster kernel, which takes the larger molecules of the same batch.
constexpr int EE_WARPS = 8, EE_WUNROLL = 8;
// molecule of warp w: the scheduling order (descending size) when the batch has one, so the
// longest streams start first and the small molecules fill in behind them
__device__ __forceinline__ int warp_molecule(const seqm_batch &b, int w) {
  return b.nclass > 0 ? b.mol_order[w] : w;
}
__global__ void __launch_bounds__(32 * EE_WARPS) k_energy_error_warp(
    seqm_batch b, const double *__restrict__ P, const double *__restrict__ Pold, const double *__restrict__ H,
    const double *__restrict__ F, double *Eelec, double *Eout, double *err, double *dm_err, double *dm_el,
    uint8_t *active, double eps, const double *__restrict__ diis_err, int *__restrict__ nactive,
    const int32_t *__restrict__ kit) {
  const int w = blockIdx.x * EE_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= b.nmol) return;
  const int m = warp_molecule(b, w);
  if (!is_active(active, m)) return;  // uniform over the warp
  const int n = b.mol_norb[m];
  if (n > EE_WARP_MAX) return;
  const size_t mo = b.mol_mat_off[m];
  const int nn = n * n;
  const double *Pm = P + mo, *Hm = H + mo, *Fm = F + mo, *Om = Pold ? Pold + mo : nullptr;
  double e = 0.0, fro = 0.0, mx = 0.0;
  for (int i = lane; i < nn; i += 32 * EE_WUNROLL) {
    double pv[EE_WUNROLL], hf[EE_WUNROLL], po[EE_WUNROLL];
#pragma unroll
    for (int u = 0; u < EE_WUNROLL; ++u) {
      const int j = i + 32 * u;
      const bool in = j < nn;
      pv[u] = in ? Pm[j] : 0.0;
      hf[u] = in ? Hm[j] + Fm[j] : 0.0;
      po[u] = (in && Om) ? Om[j] : pv[u];
    }
#pragma unroll
    for (int u = 0; u < EE_WUNROLL; ++u) {
      e = fma(pv[u], hf[u], e);
      const double d = pv[u] - po[u];
      fro = fma(d, d, fro);
      mx = fmax(mx, fabs(d));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    fro += __shfl_xor_sync(0xffffffffu, fro, o);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) {
    e *= 0.5;
    Eout[m] = e;
    if (Pold) finish_error(b, m, e, fro, mx, Eelec, err, dm_err, dm_el, active, eps, diis_err, nactive, kit);
  }
}

// ------------------------------------------------------------------ mixing
// linear: P <- alpha P + (1 - alpha) Pnew (scf_loop.py:258-267);
// adaptive (scf_loop.py:360-420): every third iteration extrapolate
// P <- (1+FAC) Pnew - FAC P with FAC from the diagonal history; the diagonal is
// damped (|step| <= 0.05 after iteration 4), clamped to [0, occupation] and renormalised
// to the new trace in at most 20 passes.  Each molecule stops its own
// renormalisation (the reference stops when the whole padded batch is done).
//
// One cluster of cs CTAs per molecule: every CTA reads the diagonal history and
// forms FAC (identical arithmetic in each), the CTAs split the elementwise update,
// and rank 0 alone damps, clamps and renormalises the diagonal and writes it after
// a cluster barrier, over the provisional values of the elementwise pass.
constexpr int NT_MIX = 512, MIX_UNROLL = 4;
constexpr int MIX_WARP_MAX = 160;  // molecules up to this size are mixed by k_mix_warp
constexpr size_t MIX_SMEM_MAX = 200 * 1024;  // diagonal history of molecules up to 12800 AOs
__global__ void __launch_bounds__(NT_MIX) k_mix(seqm_batch b, double *__restrict__ P, const double *__restrict__ Pnew,
                                                double *__restrict__ Pold, double *__restrict__ old2,
                                                const int64_t *__restrict__ row_off, int32_t *__restrict__ kit,
                                                int linear, double alpha, double occ,
                                                const uint8_t *__restrict__ active, int cs) {
  extern __shared__ double sm[];
  __shared__ double red[NT_MIX / 32];
  cg::cluster_group cl = cg::this_cluster();
  const int m = blockIdx.x / cs, r = (int)cl.block_rank();
  if (!is_active(active, m)) return;  // uniform over the cluster
  const int n = b.mol_norb[m];
  if (n <= MIX_WARP_MAX) return;  // k_mix_warp's molecule
  const int k = kit[m] + 1;  // 1-based iteration number of this molecule
  const size_t mo = b.mol_mat_off[m], nn = (size_t)n * n;
  const size_t i0 = (size_t)r * NT_MIX + threadIdx.x, step = (size_t)cs * NT_MIX;
  double *Pm = P + mo, *Po = Pold + mo;
  const double *Pn = Pnew + mo;
  if (linear) {
    cl.sync();  // every CTA has read kit[m]
    if (r == 0 && threadIdx.x == 0) kit[m] = k;
    const double oma = 1.0 - alpha;
    for (size_t i = i0; i < nn; i += MIX_UNROLL * step) {
      double pv[MIX_UNROLL], pn[MIX_UNROLL];
#pragma unroll
      for (int u = 0; u < MIX_UNROLL; ++u) {
        const size_t j = i + u * step;
        pv[u] = j < nn ? Pm[j] : 0.0;
        pn[u] = j < nn ? Pn[j] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < MIX_UNROLL; ++u) {
        const size_t j = i + u * step;
        if (j < nn) {
          Po[j] = pv[u];
          Pm[j] = alpha * pv[u] + oma * pn[u];
        }
      }
    }
    return;
  }
  double *dprev = sm, *di = sm + n;
  double *o2 = old2 + row_off[m];
  double num = 0.0, den = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_MIX) {
    const double dp = Pm[(size_t)i * n + i], dc = Pn[(size_t)i * n + i];
    dprev[i] = dp;
    const double d1 = dc - dp, d2 = dc - 2.0 * dp + o2[i];
    num += d1 * d1;
    den += d2 * d2;
  }
  const bool third = (k % 3) == 0;
  double fac = 0.0;
  if (third) {
    num = block_sum<NT_MIX>(num, red);
    den = block_sum<NT_MIX>(den, red);
    fac = (den > 0.0 && num < 100.0 * den) ? sqrt(num / den) : 0.0;
  }
  cl.sync();  // every CTA has read kit[m], the diagonal of P and old2
  if (r == 0 && threadIdx.x == 0) kit[m] = k;
  // off-diagonal (and provisional diagonal) update
  for (size_t i = i0; i < nn; i += MIX_UNROLL * step) {
    double pv[MIX_UNROLL], pn[MIX_UNROLL];
#pragma unroll
    for (int u = 0; u < MIX_UNROLL; ++u) {
      const size_t j = i + u * step;
      pv[u] = j < nn ? Pm[j] : 0.0;
      pn[u] = j < nn ? Pn[j] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < MIX_UNROLL; ++u) {
      const size_t j = i + u * step;
      if (j < nn) {
        Po[j] = pv[u];
        Pm[j] = third ? (1.0 + fac) * pn[u] - fac * pv[u] : pn[u];
      }
    }
  }
  if (r == 0) {
    // diagonal: damp, clamp, renormalise
    const double damp = k > 4 ? 0.05 : 1.0e10;
    double s0 = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MIX) {
      const double dc = Pn[(size_t)i * n + i], dp = dprev[i];
      const double delta = dc - dp;
      const double v =
          fabs(delta) > damp ? dp + (delta > 0.0 ? 1.0 : (delta < 0.0 ? -1.0 : 0.0)) * damp : dc + fac * delta;
      di[i] = fmin(fmax(v, 0.0), occ);
      s0 += dc;
    }
    double sum0 = block_sum<NT_MIX>(s0, red);
    for (int pass = 0; pass < 20; ++pass) {
      double s2 = 0.0;
      for (int i = threadIdx.x; i < n; i += NT_MIX) s2 += di[i];
      const double sum2 = block_sum<NT_MIX>(s2, red);
      const double sum3 = sum2 > 1.0e-3 ? sum0 / sum2 : 0.0;
      if (!(sum2 > 1.0e-3) || fabs(sum3 - 1.0) <= 1.0e-5) break;
      double nfull = 0.0;
      for (int i = threadIdx.x; i < n; i += NT_MIX) {
        const double sc = fmax(di[i] * sum3, 0.0);
        const bool full = sc > occ;
        di[i] = full ? occ : sc;
        nfull += full ? 1.0 : 0.0;
      }
      nfull = block_sum<NT_MIX>(nfull, red);
      sum0 = sum0 - nfull * occ;
    }
  }
  cl.sync();  // every CTA's provisional diagonal is written
  if (r == 0) {
    for (int i = threadIdx.x; i < n; i += NT_MIX) {
      Pm[(size_t)i * n + i] = di[i];
      o2[i] = dprev[i];
    }
  }
}

// The same mixing for molecules of up to MIX_WARP_MAX basis functions, one warp per molecule
// (eight per CTA): the lanes hold the diagonal (at most five elements each) in registers, every
// sum of the adaptive step is a butterfly, and the elementwise update streams the molecule's
// matrices with coalesced loads.  A molecule's arithmetic depends only on its own size.
constexpr int MIX_WARPS = 8, MIX_DIAG = (MIX_WARP_MAX + 31) / 32, MIX_WUNROLL = 8;
__global__ void __launch_bounds__(32 * MIX_WARPS) k_mix_warp(seqm_batch b, double *__restrict__ P,
                                                             const double *__restrict__ Pnew, double *__restrict__ Pold,
                                                             double *__restrict__ old2,
                                                             const int64_t *__restrict__ row_off,
                                                             int32_t *__restrict__ kit, int linear, double alpha,
                                                             double occ, const uint8_t *__restrict__ active) {
  const int w = blockIdx.x * MIX_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= b.nmol) return;
  const int m = warp_molecule(b, w);
  if (!is_active(active, m)) return;  // uniform over the warp
  const int n = b.mol_norb[m];
  if (n > MIX_WARP_MAX) return;
  const int k = kit[m] + 1;
  const size_t mo = b.mol_mat_off[m];
  const int nn = n * n;
  double *Pm = P + mo, *Po = Pold + mo;
  const double *Pn = Pnew + mo;
  double dp[MIX_DIAG], dc[MIX_DIAG];
  double fac = 0.0;
  const bool third = !linear && (k % 3) == 0;
  double *o2 = linear ? nullptr : old2 + row_off[m];
  if (!linear) {
    double num = 0.0, den = 0.0;
#pragma unroll
    for (int t = 0; t < MIX_DIAG; ++t) {
      const int i = lane + 32 * t;
      dp[t] = i < n ? Pm[(size_t)i * n + i] : 0.0;
      dc[t] = i < n ? Pn[(size_t)i * n + i] : 0.0;
      const double o2v = i < n ? o2[i] : 0.0;
      const double d1 = dc[t] - dp[t], d2 = dc[t] - 2.0 * dp[t] + o2v;
      num = fma(d1, d1, num);
      den = fma(d2, d2, den);
    }
    if (third) {
      num = warp_allsum(num);
      den = warp_allsum(den);
      fac = (den > 0.0 && num < 100.0 * den) ? sqrt(num / den) : 0.0;
    }
  }
  __syncwarp();  // every lane has read its diagonal elements before any is overwritten
  if (lane == 0) kit[m] = k;
  const double oma = 1.0 - alpha;
  for (int i = lane; i < nn; i += 32 * MIX_WUNROLL) {
    double pv[MIX_WUNROLL], pn[MIX_WUNROLL];
#pragma unroll
    for (int u = 0; u < MIX_WUNROLL; ++u) {
      const int j = i + 32 * u;
      pv[u] = j < nn ? Pm[j] : 0.0;
      pn[u] = j < nn ? Pn[j] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < MIX_WUNROLL; ++u) {
      const int j = i + 32 * u;
      if (j < nn) {
        Po[j] = pv[u];
        Pm[j] = linear ? alpha * pv[u] + oma * pn[u] : (third ? (1.0 + fac) * pn[u] - fac * pv[u] : pn[u]);
      }
    }
  }
  if (linear) return;
  __syncwarp();  // the provisional diagonal is written before the final one replaces it
  // diagonal: damp, clamp, renormalise (as k_mix)
  const double damp = k > 4 ? 0.05 : 1.0e10;
  double di[MIX_DIAG], s0 = 0.0;
#pragma unroll
  for (int t = 0; t < MIX_DIAG; ++t) {
    const int i = lane + 32 * t;
    const double delta = dc[t] - dp[t];
    const double v = fabs(delta) > damp ? dp[t] + (delta > 0.0 ? 1.0 : (delta < 0.0 ? -1.0 : 0.0)) * damp
                                        : dc[t] + fac * delta;
    di[t] = i < n ? fmin(fmax(v, 0.0), occ) : 0.0;
    s0 += i < n ? dc[t] : 0.0;
  }
  double sum0 = warp_allsum(s0);
  for (int pass = 0; pass < 20; ++pass) {
    double s2 = 0.0;
#pragma unroll
    for (int t = 0; t < MIX_DIAG; ++t) s2 += di[t];
    const double sum2 = warp_allsum(s2);
    const double sum3 = sum2 > 1.0e-3 ? sum0 / sum2 : 0.0;
    if (!(sum2 > 1.0e-3) || fabs(sum3 - 1.0) <= 1.0e-5) break;
    double nfull = 0.0;
#pragma unroll
    for (int t = 0; t < MIX_DIAG; ++t) {
      const int i = lane + 32 * t;
      const double sc = fmax(di[t] * sum3, 0.0);
      const bool full = sc > occ;
      di[t] = i < n ? (full ? occ : sc) : 0.0;
      nfull += (i < n && full) ? 1.0 : 0.0;
    }
    nfull = warp_allsum(nfull);
    sum0 = sum0 - nfull * occ;
  }
#pragma unroll
  for (int t = 0; t < MIX_DIAG; ++t) {
    const int i = lane + 32 * t;
    if (i < n) {
      Pm[(size_t)i * n + i] = di[t];
      o2[i] = dp[t];
    }
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

// CTAs per molecule of the cluster kernels: more for larger molecules; 16 (above the portable
// cluster size of 8) where the kernel accepts it
template <typename... Params>
static int mol_cluster(void (*kern)(Params...), int max_norb) {
  if (max_norb <= 160) return 1;
  if (max_norb <= 320) return 2;
  if (max_norb <= 640) return 4;
  if (max_norb <= 1024) return 8;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess ? 16 : 8;
}

// grid of nmol clusters of cs CTAs each (cluster c = molecule c)
template <typename... Params, typename... Args>
static int launch_clusters(void (*kern)(Params...), int cs, int nmol, int nt, size_t smem, void *stream,
                           Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cs * (unsigned)nmol);
  cfg.blockDim = dim3((unsigned)nt);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = (cudaStream_t)stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)cs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kern, args...) != cudaSuccess) return SEQM_E_CUDA;
  return launch_check();
}

// energy + test of every molecule: the warp kernel for molecules up to EE_WARP_MAX basis
// functions, the cluster kernel (launched only when the batch holds larger ones) for the rest
template <typename... Args>
int launch_energy_error(const seqm_batch &b, void *stream, int *nactive, const int32_t *kit, Args... args) {
  k_energy_error_warp<<<(b.nmol + EE_WARPS - 1) / EE_WARPS, 32 * EE_WARPS, 0, (cudaStream_t)stream>>>(b, args...,
                                                                                                        nactive, kit);
  int rc = launch_check();
  if (rc != SEQM_OK || b.max_norb <= EE_WARP_MAX) return rc;
  const int cs = mol_cluster(k_energy_error, b.max_norb);
  return launch_clusters(k_energy_error, cs, b.nmol, NT_RED, 0, stream, b, args..., nactive, kit, cs);
}

extern "C" int seqm_fock(const seqm_batch *bp, const double *P, const double *H, const double *w_xx,
                         const double *w_xh, const double *w_hh, double *F, const uint8_t *active, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  long long nt = 32LL * b.natoms + b.nxx + b.nxh + b.nhh;
  if (nt == 0) return SEQM_OK;
  k_fock<<<(unsigned)((nt + 127) / 128), 128, 0, (cudaStream_t)stream>>>(b, P, H, w_xx, w_xh, w_hh, F, active);
  return launch_check();
}

extern "C" int seqm_energy_error(const seqm_batch *bp, const double *P, const double *Pold, const double *H,
                                 const double *F, double *Eelec, double *Eout, double *err, double *dm_err,
                                 double *dm_el, uint8_t *active, double eps, const double *diis_err, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  return launch_energy_error(b, stream, (int *)nullptr, (const int32_t *)nullptr, P, Pold, H, F, Eelec, Eout, err,
                             dm_err, dm_el, active, eps, diis_err);
}

extern "C" int seqm_scf_step(const seqm_batch *bp, const seqm_scf_state *st, void *stream) {
  if (!bp || !st || !st->P || !st->Pnew || !st->Pold || !st->H || !st->F || !st->active) return SEQM_E_ARG;
  if (st->mixing < -1 || st->mixing > 1) return SEQM_E_ARG;
  const seqm_batch &b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = SEQM_OK;
  if (st->mixing >= 0) {
    rc = seqm_mix(bp, st->P, st->Pnew, st->Pold, st->old2, st->mol_row_off, st->iters, st->mixing == 0, st->alpha,
                  st->occupation, st->active, stream);
    if (rc != SEQM_OK) return rc;
  }
  rc = seqm_fock(bp, st->P, st->H, st->w_xx, st->w_xh, st->w_hh, st->F, st->active, stream);
  if (rc != SEQM_OK) return rc;
  if (st->nactive && cudaMemsetAsync(st->nactive, 0, sizeof(int32_t), s) != cudaSuccess) return SEQM_E_CUDA;
  return launch_energy_error(b, stream, (int *)st->nactive, (const int32_t *)st->iters, (const double *)st->P,
                             (const double *)st->Pold, st->H, (const double *)st->F, st->Eelec, st->Eout, st->err,
                             st->dm_err, st->dm_el, st->active, st->eps, st->diis_err);
}

extern "C" int seqm_mix(const seqm_batch *bp, double *P, const double *Pnew, double *Pold, double *old2,
                        const int64_t *mol_row_off, int32_t *k, int linear, double alpha, double occupation,
                        const uint8_t *active, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  size_t smem = linear ? 0 : (size_t)2 * b.max_norb * sizeof(double);
  if (smem > MIX_SMEM_MAX) return SEQM_E_TOO_LARGE;
  if (smem > 0) {  // raised whatever the size: the kernel's static shared memory counts against the default 48 KB
    static SmemLimit limit;
    const int rc = limit.ensure(k_mix, MIX_SMEM_MAX);
    if (rc != SEQM_OK) return rc;
  }
  k_mix_warp<<<(b.nmol + MIX_WARPS - 1) / MIX_WARPS, 32 * MIX_WARPS, 0, (cudaStream_t)stream>>>(
      b, P, Pnew, Pold, old2, mol_row_off, k, linear, alpha, occupation, active);
  const int rc = launch_check();
  if (rc != SEQM_OK || b.max_norb <= MIX_WARP_MAX) return rc;
  const int cs = mol_cluster(k_mix, b.max_norb);
  return launch_clusters(k_mix, cs, b.nmol, NT_MIX, smem, stream, b, P, Pnew, Pold, old2, mol_row_off, k, linear, alpha,
                         occupation, active, cs);
}

extern "C" int seqm_initial_density(const seqm_batch *bp, double *P, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.natoms == 0) return SEQM_OK;
  k_initial_density<<<(b.natoms + 127) / 128, 128, 0, (cudaStream_t)stream>>>(b, P);
  return launch_check();
}
