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
                                          double *__restrict__ F, double *__restrict__ epart) {
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
    double ep = 0.0;
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
      const double h = Hm[(size_t)(o + r) * norb + o + c], v = h + oc + J;
      Fm[(size_t)(o + r) * norb + o + c] = v;
      Fm[(size_t)(o + c) * norb + o + r] = v;
      ep = (r == c ? 1.0 : 2.0) * Prc * (h + v);  // both triangles of the block
    }
    if (epart) {  // sum P (H + F) over the block: lanes 0-9 hold the packed elements
#pragma unroll
      for (int o2 = 8; o2 > 0; o2 >>= 1) ep += __shfl_down_sync(0xffffffffu, ep, o2);
      if (lane == 0) epart[a] = ep;
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
      const double Pss = Pm[(size_t)o * norb + o], h = Hm[(size_t)o * norb + o];
      const double v = h + 0.5 * Pss * gss + f;
      Fm[(size_t)o * norb + o] = v;
      if (epart) epart[a] = Pss * (h + v);
    }
  }
}

__global__ void __launch_bounds__(128) k_fock(seqm_batch b, const double *__restrict__ P, const double *__restrict__ H,
                                              const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                                              const double *__restrict__ w_hh, double *__restrict__ F,
                                              const uint8_t *__restrict__ active, double *__restrict__ epart) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ndiag = 32LL * b.natoms;  // one warp per atom; warps never straddle the two roles
  const int npairs = b.nxx + b.nxh + b.nhh;
  if (t < ndiag) {
    const int a = (int)(t >> 5);
    if (!is_active(active, b.atom_mol[a])) return;
    fock_diag(b, a, (int)(t & 31), P, H, w_xx, w_xh, w_hh, F, epart);
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
  double ep = 0.0;  // P (H + F) over the block and its transpose
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
        const double h = Hm[(size_t)(oi + mu) * norb + oj + nu], v = fma(-0.5, k, h);
        Fm[(size_t)(oi + mu) * norb + oj + nu] = v;
        Fm[(size_t)(oj + nu) * norb + oi + mu] = v;
        ep = fma(Pp[mu][nu], h + v, ep);
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
      const double h = Hm[(size_t)(oi + mu) * norb + oj], v = fma(-0.5, k, h);
      Fm[(size_t)(oi + mu) * norb + oj] = v;
      Fm[(size_t)oj * norb + oi + mu] = v;
      ep = fma(Pp[mu], h + v, ep);
    }
  } else {
    const double h = Hm[(size_t)oi * norb + oj], pij = Pm[(size_t)oi * norb + oj];
    const double v = h + w_hh[p - b.nxx - b.nxh] * (-0.5 * pij);
    Fm[(size_t)oi * norb + oj] = v;
    Fm[(size_t)oj * norb + oi] = v;
    ep = pij * (h + v);
  }
  if (epart) epart[(size_t)b.natoms + p] = 2.0 * ep;
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

// ----------------------------------------------------------- fused mixing (seqm_scf_step)
// The mixing of seqm_scf_step takes the change of P itself instead of leaving Pold for a separate
// energy pass.  Every update is P + c (Pnew - P) (linear: c = 1 - alpha; the adaptive
// extrapolation: c = 1 + FAC; otherwise P = Pnew), so with d = Pnew - P formed once the new element
// costs at most one FMA, and sum d^2 (times c^2) and max |d| (times |c|) give the ||dP|| terms of
// the convergence test.  Adaptive mixing first runs k_mix_diag (warp per molecule up to
// MIX_WARP_MAX basis functions, a CTA above): FAC from the diagonal history, the damped, clamped
// and renormalised diagonal written to P with old2 and the iteration count, and the diagonal's
// change and c left in the molecule's mixer slots; the streams then touch only the off-diagonal
// elements and carry no serial tail.  Linear mixing streams every element.  Per molecule the
// arithmetic depends only on its size.
constexpr int MIX_SMALL = 64;
// per-molecule mixer slots of the scratch: [0] sum d^2, [1] max |d| (diagonal, then all), [2] c
constexpr int MIX_SLOTS = 4;
// FP64 -> FP32 by truncation with integer instructions only (GB300 converts on its FP64 pipe):
// sign, rebiased exponent, top 23 mantissa bits; |d| < 2^-126 gives 0.  For |d| <= 2 (density
// elements and their changes) the exponent never overflows.
__device__ __forceinline__ float f32_trunc(double d) {
  const int hi = __double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  const unsigned bits = ((unsigned)hi & 0x80000000u) | ((unsigned)e << 23) | (((unsigned)hi & 0xfffffu) << 3) | (lo >> 29);
  return e > 0 ? __uint_as_float(bits) : 0.0f;
}

// Diagonal step of adaptive mixing (scf_loop.py:360-420), one warp per molecule of up to
// MIX_WARP_MAX basis functions (eight per CTA; each lane holds at most five diagonal elements).
__global__ void __launch_bounds__(32 * MIX_WARPS) k_mix_diag_warp(seqm_batch b, double *__restrict__ P,
                                                                  const double *__restrict__ Pnew,
                                                                  double *__restrict__ old2,
                                                                  const int64_t *__restrict__ row_off,
                                                                  int32_t *__restrict__ kit, double occ,
                                                                  const uint8_t *__restrict__ active,
                                                                  double *__restrict__ ms) {
  const int w = blockIdx.x * MIX_WARPS + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= b.nmol) return;
  const int m = warp_molecule(b, w);
  if (!is_active(active, m)) return;  // uniform over the warp
  const int n = b.mol_norb[m];
  if (n > MIX_WARP_MAX) return;
  const int k = kit[m] + 1;
  double *Pm = P + b.mol_mat_off[m];
  const double *Pn = Pnew + b.mol_mat_off[m];
  double *o2 = old2 + row_off[m];
  // slots a lane holds: the loops stop at the molecule's own count (uniform over the warp), as
  // every FP64 instruction costs the FP64 pipe the same however few of its lanes work
  const int nt = (n + 31) >> 5;
  double dp[MIX_DIAG] = {}, dc[MIX_DIAG] = {}, num = 0.0, den = 0.0;
#pragma unroll
  for (int t = 0; t < MIX_DIAG; ++t) {
    if (t >= nt) break;
    const int i = lane + 32 * t;
    dp[t] = i < n ? Pm[(size_t)i * n + i] : 0.0;
    dc[t] = i < n ? Pn[(size_t)i * n + i] : 0.0;
    const double o2v = i < n ? o2[i] : 0.0;
    const double d1 = dc[t] - dp[t], d2 = dc[t] - 2.0 * dp[t] + o2v;
    num = fma(d1, d1, num);
    den = fma(d2, d2, den);
  }
  double fac = 0.0;
  if (k % 3 == 0) {
    num = warp_allsum(num);
    den = warp_allsum(den);
    fac = (den > 0.0 && num < 100.0 * den) ? sqrt(num / den) : 0.0;
  }
  const double damp = k > 4 ? 0.05 : 1.0e10;
  double di[MIX_DIAG] = {}, s0 = 0.0;
#pragma unroll
  for (int t = 0; t < MIX_DIAG; ++t) {
    if (t >= nt) break;
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
    for (int t = 0; t < MIX_DIAG; ++t) {
      if (t >= nt) break;
      s2 += di[t];
    }
    const double sum2 = warp_allsum(s2);
    const double sum3 = sum2 > 1.0e-3 ? sum0 / sum2 : 0.0;
    if (!(sum2 > 1.0e-3) || fabs(sum3 - 1.0) <= 1.0e-5) break;
    double nfull = 0.0;
#pragma unroll
    for (int t = 0; t < MIX_DIAG; ++t) {
      if (t >= nt) break;
      const int i = lane + 32 * t;
      const double sc = fmax(di[t] * sum3, 0.0);
      const bool full = sc > occ;
      di[t] = i < n ? (full ? occ : sc) : 0.0;
      nfull += (i < n && full) ? 1.0 : 0.0;
    }
    nfull = warp_allsum(nfull);
    sum0 = sum0 - nfull * occ;
  }
  double dfro = 0.0, dmx = 0.0;
#pragma unroll
  for (int t = 0; t < MIX_DIAG; ++t) {
    if (t >= nt) break;
    const int i = lane + 32 * t;
    if (i < n) {
      Pm[(size_t)i * n + i] = di[t];
      o2[i] = dp[t];
      const double d = di[t] - dp[t];
      dfro = fma(d, d, dfro);
      dmx = fmax(dmx, fabs(d));
    }
  }
  dfro = warp_allsum(dfro);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dmx = fmax(dmx, __shfl_xor_sync(0xffffffffu, dmx, o));
  if (lane == 0) {
    kit[m] = k;
    double *slot = ms + MIX_SLOTS * m;
    slot[0] = dfro;
    slot[1] = dmx;
    slot[2] = k % 3 == 0 ? 1.0 + fac : 1.0;
  }
}

// The same for molecules above MIX_WARP_MAX basis functions: one CTA per molecule, the new
// diagonal kept in the molecule's scratch (L2-resident) through the renormalisation passes.
constexpr int NT_MD = 512;
// slice partials and scratch of molecule m in the 4 sum(norb) region (4 n doubles per molecule):
// mixer slices (2 each) at [0, 2n), the new diagonal at [2n, 3n), energy slices at [3n, 4n)
__device__ __forceinline__ double *mol_scratch(double *q, const int64_t *row_off, int m) { return q + 4 * row_off[m]; }

__global__ void __launch_bounds__(NT_MD) k_mix_diag_cta(seqm_batch b, double *__restrict__ P,
                                                        const double *__restrict__ Pnew, double *__restrict__ old2,
                                                        const int64_t *__restrict__ row_off,
                                                        int32_t *__restrict__ kit, double occ,
                                                        const uint8_t *__restrict__ active, double *__restrict__ ms,
                                                        double *__restrict__ q) {
  __shared__ double red[NT_MD / 32];
  const int m = blockIdx.x;
  if (!is_active(active, m)) return;
  const int n = b.mol_norb[m];
  if (n <= MIX_WARP_MAX) return;
  const int k = kit[m] + 1;
  double *Pm = P + b.mol_mat_off[m];
  const double *Pn = Pnew + b.mol_mat_off[m];
  double *o2 = old2 + row_off[m];
  double *di = mol_scratch(q, row_off, m) + 2 * (int64_t)n;
  double fac = 0.0;
  if (k % 3 == 0) {
    double num = 0.0, den = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MD) {
      const double dp = Pm[(size_t)i * n + i], dc = Pn[(size_t)i * n + i];
      const double d1 = dc - dp, d2 = dc - 2.0 * dp + o2[i];
      num += d1 * d1;
      den += d2 * d2;
    }
    num = block_sum<NT_MD>(num, red);
    den = block_sum<NT_MD>(den, red);
    fac = (den > 0.0 && num < 100.0 * den) ? sqrt(num / den) : 0.0;
  }
  const double damp = k > 4 ? 0.05 : 1.0e10;
  double s0 = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_MD) {
    const double dcv = Pn[(size_t)i * n + i], dpv = Pm[(size_t)i * n + i];
    const double delta = dcv - dpv;
    const double v =
        fabs(delta) > damp ? dpv + (delta > 0.0 ? 1.0 : (delta < 0.0 ? -1.0 : 0.0)) * damp : dcv + fac * delta;
    di[i] = fmin(fmax(v, 0.0), occ);
    s0 += dcv;
  }
  double sum0 = block_sum<NT_MD>(s0, red);
  for (int pass = 0; pass < 20; ++pass) {
    double s2 = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MD) s2 += di[i];
    const double sum2 = block_sum<NT_MD>(s2, red);
    const double sum3 = sum2 > 1.0e-3 ? sum0 / sum2 : 0.0;
    if (!(sum2 > 1.0e-3) || fabs(sum3 - 1.0) <= 1.0e-5) break;
    double nfull = 0.0;
    for (int i = threadIdx.x; i < n; i += NT_MD) {
      const double sc = fmax(di[i] * sum3, 0.0);
      const bool full = sc > occ;
      di[i] = full ? occ : sc;
      nfull += full ? 1.0 : 0.0;
    }
    nfull = block_sum<NT_MD>(nfull, red);
    sum0 = sum0 - nfull * occ;
  }
  double dfro = 0.0, dmx = 0.0;
  for (int i = threadIdx.x; i < n; i += NT_MD) {
    const double dpv = Pm[(size_t)i * n + i], d = di[i] - dpv;
    Pm[(size_t)i * n + i] = di[i];
    o2[i] = dpv;
    dfro += d * d;
    dmx = fmax(dmx, fabs(d));
  }
  dfro = block_sum<NT_MD>(dfro, red);
  dmx = block_max<NT_MD>(dmx, red);
  if (threadIdx.x == 0) {
    kit[m] = k;
    double *slot = ms + MIX_SLOTS * m;
    slot[0] = dfro;
    slot[1] = dmx;
    slot[2] = k % 3 == 0 ? 1.0 + fac : 1.0;
  }
}

// One thread's part of the fused stream: elements i0, i0 + STRIDE, ... below `end` (U at a time,
// loads first) of an n x n matrix starting at element 0.  COPY: P = Pnew, else P + c d.  The
// statistics of d run on the FP32 pipe from the integer-truncated f = fl32(d) rounded toward zero:
// sum f^2 in FP32 (non-negative terms: relative error at most the thread's term count times 2^-24)
// and max |f| (at most 2^-23 below max |d|), so an element costs one FP64 operation (d) when
// copying and two otherwise.  Measured on GB300 over a 3 GB stream: 6.6 TB/s when copying and
// 5.8 TB/s otherwise, where FP64 statistics or a 64-bit integer max took it to 3.6 TB/s.
// SKIP_DIAG (adaptive mixing): the diagonal, written by k_mix_diag, is skipped; the thread's
// (row, column) advance by the stride with integer adds only.
template <bool COPY, bool SKIP_DIAG, int U, int STRIDE, typename Idx>
__device__ __forceinline__ void fused_stream(double *__restrict__ Pm, const double *__restrict__ Pn, Idx i0, Idx end,
                                             uint32_t n, double c, float &fro, float &mx) {
  uint32_t row = 0, col = 0;
  constexpr uint32_t S = (uint32_t)STRIDE;
  const uint32_t drow = S / n, dcol = S % n;
  if (SKIP_DIAG) {
    row = (uint32_t)(i0 / n);
    col = (uint32_t)(i0 % n);
  }
  for (Idx i = i0; i < end; i += (Idx)U * STRIDE) {
    double *p = Pm + i;
    const double *q = Pn + i;
    const Idx rem = end - i;
    double pv[U], pn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      pv[u] = (Idx)(u * STRIDE) < rem ? p[u * STRIDE] : 0.0;
      pn[u] = (Idx)(u * STRIDE) < rem ? q[u * STRIDE] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool diag = SKIP_DIAG && row == col;
      if (SKIP_DIAG) {
        col += dcol;
        row += drow;
        if (col >= n) {
          col -= n;
          ++row;
        }
      }
      if ((Idx)(u * STRIDE) < rem && !diag) {
        const double d = pn[u] - pv[u];
        p[u * STRIDE] = COPY ? pn[u] : fma(c, d, pv[u]);
        const float f = f32_trunc(d);
        fro = fmaf(f, f, fro);
        mx = fmaxf(mx, fabsf(f));
      }
    }
  }
}
// the four forms of fused_stream, chosen by uniform flags
template <int U, int STRIDE, typename Idx>
__device__ __forceinline__ void fused_stream_any(bool copy, bool skip_diag, double *__restrict__ Pm,
                                                 const double *__restrict__ Pn, Idx i0, Idx end, uint32_t n, double c,
                                                 float &fro, float &mx) {
  if (copy) {
    if (skip_diag) fused_stream<true, true, U, STRIDE>(Pm, Pn, i0, end, n, c, fro, mx);
    else fused_stream<true, false, U, STRIDE>(Pm, Pn, i0, end, n, c, fro, mx);
  } else {
    if (skip_diag) fused_stream<false, true, U, STRIDE>(Pm, Pn, i0, end, n, c, fro, mx);
    else fused_stream<false, false, U, STRIDE>(Pm, Pn, i0, end, n, c, fro, mx);
  }
}
// the mixer's ||dP|| terms of molecule m from the stream's sums and (adaptive) the diagonal's
__device__ __forceinline__ void mix_finish(double *__restrict__ ms, int m, int linear, double c, bool copy,
                                           double fro, double mx) {
  double *slot = ms + MIX_SLOTS * m;
  const double cc = copy ? 1.0 : c;
  const double dfro = linear ? 0.0 : slot[0], dmx = linear ? 0.0 : slot[1];
  slot[0] = fma(cc * cc, fro, dfro);
  slot[1] = fmax(fabs(cc) * mx, dmx);
}

// The stream for molecules of up to MIX_WARP_MAX basis functions: G warps per molecule (G = 1:
// eight molecules per CTA, n <= MIX_SMALL; G = 8: one molecule per CTA, larger n, so that its
// stream keeps eight warps of loads in flight).
template <int G>
__global__ void __launch_bounds__(32 * MIX_WARPS) k_mix_fused(seqm_batch b, double *__restrict__ P,
                                                              const double *__restrict__ Pnew,
                                                              int32_t *__restrict__ kit, int linear, double alpha,
                                                              const uint8_t *__restrict__ active,
                                                              double *__restrict__ ms) {
  static_assert(G == 1 || G == MIX_WARPS, "a molecule takes one warp or the whole CTA");
  __shared__ double sfro[MIX_WARPS], smx[MIX_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * (MIX_WARPS / G) + warp / G;  // the molecule's slot in the scheduling order
  if (w >= b.nmol) return;
  const int m = warp_molecule(b, w);
  if (!is_active(active, m)) return;  // uniform over the group
  const int n = b.mol_norb[m];
  if (G == 1 ? n > MIX_SMALL : (n <= MIX_SMALL || n > MIX_WARP_MAX)) return;
  const double c = linear ? 1.0 - alpha : ms[MIX_SLOTS * m + 2];
  const bool copy = !linear && c == 1.0;
  const size_t mo = b.mol_mat_off[m];
  float fro32 = 0.0f, mx32 = 0.0f;
  fused_stream_any<MIX_WUNROLL, 32 * G>(copy, !linear, P + mo, Pnew + mo, (warp % G) * 32 + lane, n * n,
                                        (uint32_t)n, c, fro32, mx32);
  double fro = warp_allsum((double)fro32), mx = (double)mx32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (G > 1) {
    if (lane == 0) {
      sfro[warp] = fro;
      smx[warp] = mx;
    }
    __syncthreads();  // every warp has read kit[m] and added its sums
    if (warp != 0) return;
    fro = 0.0;
    mx = 0.0;
    for (int g = 0; g < G; ++g) {
      fro += sfro[g];
      mx = fmax(mx, smx[g]);
    }
  }
  if (lane == 0) {
    mix_finish(ms, m, linear, c, copy, fro, mx);
    if (linear) kit[m] += 1;  // (adaptive: k_mix_diag counted the iteration)
  }
}

// The stream of a molecule above MIX_WARP_MAX basis functions over the whole GPU: CTA (m, s)
// streams slice s (MG_SLICE elements), the slice sums go to the molecule's scratch, and its last
// CTA to finish (a counter) adds them in slice order.
constexpr int NT_MG = 512, MG_UNROLL = 4;
constexpr size_t MG_SLICE = (size_t)1 << 17;
__global__ void __launch_bounds__(NT_MG) k_mix_grid(seqm_batch b, double *__restrict__ P,
                                                     const double *__restrict__ Pnew,
                                                     const int64_t *__restrict__ row_off, int32_t *__restrict__ kit,
                                                     int linear, double alpha, const uint8_t *__restrict__ active,
                                                     double *__restrict__ ms, double *__restrict__ q,
                                                     int *__restrict__ counter) {
  __shared__ double red[NT_MG / 32];
  __shared__ int last;
  const int m = blockIdx.x;
  if (!is_active(active, m)) return;
  const int n = b.mol_norb[m];
  if (n <= MIX_WARP_MAX) return;
  const size_t nn = (size_t)n * n;
  const int ns = (int)((nn + MG_SLICE - 1) / MG_SLICE), s = blockIdx.y;
  if (s >= ns) return;
  const double c = linear ? 1.0 - alpha : ms[MIX_SLOTS * m + 2];
  const bool copy = !linear && c == 1.0;
  const size_t mo = b.mol_mat_off[m];
  double *qm = mol_scratch(q, row_off, m);
  const size_t e0 = (size_t)s * MG_SLICE, e1 = e0 + MG_SLICE < nn ? e0 + MG_SLICE : nn;
  float fro32 = 0.0f, mx32 = 0.0f;
  fused_stream_any<MG_UNROLL, NT_MG>(copy, !linear, P + mo, Pnew + mo, e0 + threadIdx.x, e1, (uint32_t)n, c, fro32,
                                     mx32);
  const double fro = block_sum<NT_MG>((double)fro32, red);
  const double mx = block_max<NT_MG>((double)mx32, red);
  if (threadIdx.x == 0) {
    qm[2 * s] = fro;
    qm[2 * s + 1] = mx;
    __threadfence();
    last = atomicAdd(counter + m, 1) == ns - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  // the slices in order: lane l sums slices l, l + 32, ..., then a butterfly
  double f = 0.0, x = 0.0;
  for (int t = threadIdx.x; t < ns; t += 32) {
    f += __ldcg(qm + 2 * t);
    x = fmax(x, __ldcg(qm + 2 * t + 1));
  }
  f = warp_allsum(f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  if (threadIdx.x == 0) {
    mix_finish(ms, m, linear, c, copy, f, x);
    if (linear) kit[m] += 1;
  }
}

// Energy and convergence test of seqm_scf_step from the Fock build's partial sums of P (H + F)
// (one per atom's diagonal block, one per pair's block with its transpose) and the mixer's
// ||dP|| terms.  A molecule's partials are four contiguous runs (its atoms, XX, XH, HH pairs),
// cut into slices of EF_SLICE entries; CTA (m, s), one warp, sums slice s, and a molecule with more
// than one slice is finished by its last CTA (a counter), which adds the slice sums in slice order.
// One warp per slice: GB300 issues an FP64 warp instruction at the same cost however few of its
// lanes work, so a wide tree reduction per small molecule would cost more than the sums.
constexpr int EF_THREADS = 32, EF_SLICE = 8192;
__device__ __forceinline__ int64_t energy_partials(const seqm_batch &b, int m, int64_t base[4], int64_t len[4]) {
  const int a0 = b.mol_atom_off[m];
  base[0] = a0;
  len[0] = b.mol_atom_off[m + 1] - a0;
  base[1] = (int64_t)b.natoms + b.mol_xx_off[m];
  len[1] = b.mol_xx_off[m + 1] - b.mol_xx_off[m];
  base[2] = (int64_t)b.natoms + b.nxx + b.mol_xh_off[m];
  len[2] = b.mol_xh_off[m + 1] - b.mol_xh_off[m];
  base[3] = (int64_t)b.natoms + b.nxx + b.nxh + b.mol_hh_off[m];
  len[3] = b.mol_hh_off[m + 1] - b.mol_hh_off[m];
  return len[0] + len[1] + len[2] + len[3];
}

__global__ void __launch_bounds__(EF_THREADS) k_energy_finish(
    seqm_batch b, const double *__restrict__ epart, const double *__restrict__ ms, double *__restrict__ q,
    int *__restrict__ counter, const int64_t *__restrict__ row_off, double *Eelec, double *Eout, double *err,
    double *dm_err, double *dm_el, uint8_t *active, double eps, int *__restrict__ nactive,
    const int32_t *__restrict__ kit) {
  const int m = blockIdx.x, lane = threadIdx.x;
  if (!is_active(active, m)) return;
  int64_t base[4], len[4];
  const int64_t L = energy_partials(b, m, base, len);
  const int ns = (int)((L + EF_SLICE - 1) / EF_SLICE), s = blockIdx.y;
  if (s >= ns) return;
  const int64_t v0 = (int64_t)s * EF_SLICE, v1 = v0 + EF_SLICE < L ? v0 + EF_SLICE : L;
  double e = 0.0;
  int64_t off = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int64_t lo = v0 > off ? v0 : off, hi = v1 < off + len[r] ? v1 : off + len[r];
    for (int64_t v = lo + lane; v < hi; v += 32) e += epart[base[r] + (v - off)];
    off += len[r];
  }
  e = warp_allsum(e);
  if (ns > 1) {
    double *qe = mol_scratch(q, row_off, m) + 3 * (int64_t)b.mol_norb[m];
    int last = 0;
    if (lane == 0) {
      qe[s] = e;
      __threadfence();
      last = atomicAdd(counter + m, 1) == ns - 1;
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) return;
    __threadfence();
    e = 0.0;
    for (int t = lane; t < ns; t += 32) e += __ldcg(qe + t);
    e = warp_allsum(e);
  }
  if (lane == 0) {
    e *= 0.5;
    Eout[m] = e;
    finish_error(b, m, e, ms[MIX_SLOTS * m], ms[MIX_SLOTS * m + 1], Eelec, err, dm_err, dm_el, active, eps, nullptr,
                 nactive, kit);
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
  k_fock<<<(unsigned)((nt + 127) / 128), 128, 0, (cudaStream_t)stream>>>(b, P, H, w_xx, w_xh, w_hh, F, active,
                                                                          nullptr);
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

// seqm_scf_step with a scratch buffer and mixing >= 0: mixing with the ||dP|| terms (adaptive: the
// diagonal step first), Fock build with the energy partials, energy and test from those (no Pold,
// no separate energy pass).  Scratch (doubles): mixer slots [MIX_SLOTS nmol], counters [2 nmol
// int32], energy partials [natoms + npairs], per-molecule slices [4 sum(norb)].
static int scf_step_fused(const seqm_batch &b, const seqm_scf_state *st, cudaStream_t s) {
  if (!st->mol_row_off || !st->iters || (st->mixing == 1 && !st->old2)) return SEQM_E_ARG;
  if (b.max_norb > 12800) return SEQM_E_TOO_LARGE;  // slices of a molecule fit its 4 norb scratch
  const size_t nm = (size_t)b.nmol, npairs = (size_t)b.nxx + b.nxh + b.nhh;
  double *ms = st->scratch;
  int *counter = reinterpret_cast<int *>(ms + MIX_SLOTS * nm);  // mixer [nmol], energy [nmol]
  double *epart = ms + (MIX_SLOTS + 1) * nm;
  double *q = epart + (size_t)b.natoms + npairs;
  const int linear = st->mixing == 0;
  const bool large = b.max_norb > MIX_WARP_MAX;
  const unsigned wgrid = (unsigned)((b.nmol + MIX_WARPS - 1) / MIX_WARPS);
  if (cudaMemsetAsync(counter, 0, 2 * nm * sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
  if (!linear) {
    k_mix_diag_warp<<<wgrid, 32 * MIX_WARPS, 0, s>>>(b, st->P, st->Pnew, st->old2, st->mol_row_off, st->iters,
                                                     st->occupation, st->active, ms);
    if (large)
      k_mix_diag_cta<<<b.nmol, NT_MD, 0, s>>>(b, st->P, st->Pnew, st->old2, st->mol_row_off, st->iters,
                                              st->occupation, st->active, ms, q);
  }
  k_mix_fused<1><<<wgrid, 32 * MIX_WARPS, 0, s>>>(b, st->P, st->Pnew, st->iters, linear, st->alpha, st->active, ms);
  k_mix_fused<MIX_WARPS><<<b.nmol, 32 * MIX_WARPS, 0, s>>>(b, st->P, st->Pnew, st->iters, linear, st->alpha,
                                                           st->active, ms);
  if (large) {
    const size_t nn = (size_t)b.max_norb * b.max_norb;
    k_mix_grid<<<dim3((unsigned)b.nmol, (unsigned)((nn + MG_SLICE - 1) / MG_SLICE)), NT_MG, 0, s>>>(
        b, st->P, st->Pnew, st->mol_row_off, st->iters, linear, st->alpha, st->active, ms, q, counter);
  }
  const long long nt = 32LL * b.natoms + (long long)npairs;
  if (nt > 0)
    k_fock<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(b, st->P, st->H, st->w_xx, st->w_xh, st->w_hh, st->F,
                                                        st->active, epart);
  if (st->nactive && cudaMemsetAsync(st->nactive, 0, sizeof(int32_t), s) != cudaSuccess) return SEQM_E_CUDA;
  // slices of the largest molecule's partials: at most its atoms and their pairs, at most the batch's
  const long long mx = b.max_norb, lmax_mol = mx + mx * (mx - 1) / 2, lmax_all = (long long)b.natoms + (long long)npairs;
  const long long lmax = lmax_mol < lmax_all ? lmax_mol : lmax_all;
  k_energy_finish<<<dim3((unsigned)b.nmol, (unsigned)((lmax + EF_SLICE - 1) / EF_SLICE)), EF_THREADS, 0, s>>>(
      b, epart, ms, q, counter + nm, st->mol_row_off, st->Eelec, st->Eout, st->err, st->dm_err, st->dm_el,
      st->active, st->eps, st->nactive, st->iters);
  return launch_check();
}

extern "C" int seqm_scf_step(const seqm_batch *bp, const seqm_scf_state *st, void *stream) {
  if (!bp || !st || !st->P || !st->Pnew || !st->Pold || !st->H || !st->F || !st->active) return SEQM_E_ARG;
  if (st->mixing < -1 || st->mixing > 1) return SEQM_E_ARG;
  const seqm_batch &b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (st->mixing >= 0 && st->scratch) return scf_step_fused(b, st, s);
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
