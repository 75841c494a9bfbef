// Two-centre integrals, overlaps and the core Hamiltonian (FP64).
//
// One thread per atom pair.  Pairs come in three class segments (heavy-heavy,
// heavy-H, H-H) so a warp runs one code path.  Per pair:
//   multipole local-frame integrals (two_elec_two_center_int_local_frame.py:18-293)
//   -> quaternion rotation to the molecular frame (two_elec_two_center_int.py:1384-1631)
//   -> w (100/10/1 doubles) + core-core repulsion (energy.py:91-134)
//   -> STO overlap (diat_overlap_PM6_SP.py:6-444) * (beta_i+beta_j)/2 written as the
//      off-diagonal block of the dense per-molecule Hcore (hcore.py:151-173).
// The diagonal Hcore blocks (U + electron-core attraction, hcore.py:127-150) are a
// per-atom gather over the atom's pairs, so no atomics are used anywhere.
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "pair_math.cuh"

namespace seqm {

// ------------------------------------------------------------------ per atom
// dd, qq (cal_par.py:11-28), rho0 = ev/2/gss, rho1/rho2 by five secant steps
// (cal_par.py:122-172, 207-245); only atoms with Z > 2 carry dd/qq/rho1/rho2.
__global__ void k_atom_prep(seqm_batch b) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natoms) return;
  int Z = b.atom_Z[a];
  double gss = par(b, SEQM_P_GSS, a);
  double *P = b.atom_par;
  size_t n = b.natoms;
  P[SEQM_P_RHO0 * n + a] = 0.5 * EV / gss;
  double dd = 0.0, qq = 0.0, rho1 = 0.0, rho2 = 0.0;
  if (Z > 2) {
    double qn = par(b, SEQM_P_QN, a);
    double zs = par(b, SEQM_P_ZS, a), zp = par(b, SEQM_P_ZP, a);
    dd = (2.0 * qn + 1.0) * pow(4.0 * zs * zp, qn + 0.5) / pow(zs + zp, 2.0 * qn + 2.0) / sqrt(3.0);
    qq = sqrt((4.0 * qn * qn + 6.0 * qn + 2.0) / 20.0) / zp;
    // rho1: hsp(d) = d/2 - 1/(2 sqrt(4 D1^2 + 1/d^2)), atomic units
    double hsp = par(b, SEQM_P_HSP, a) / EV;
    double d1 = pow(fabs(hsp) / (dd * dd), 1.0 / 3.0);
    if (hsp < 0.0) d1 = -d1;
    double d2 = d1 + 0.04;
    for (int it = 0; it < 5; ++it) {
      double h1 = 0.5 * d1 - 0.5 / sqrt(4.0 * dd * dd + 1.0 / (d1 * d1));
      double h2 = 0.5 * d2 - 0.5 / sqrt(4.0 * dd * dd + 1.0 / (d2 * d2));
      double d3 = fabs(h2 - h1) > 1.0e-16 ? d1 + (d2 - d1) * (hsp - h1) / (h2 - h1) : d2;
      d1 = d2;
      d2 = d3;
    }
    rho1 = 0.5 / d2;
    // rho2: hpp(q) = q/4 - 1/(2 sqrt(4 D2^2 + 1/q^2)) + 1/(4 sqrt(8 D2^2 + 1/q^2)); hpp >= 0.1 eV
    double hpp_ev = fmax(0.5 * (par(b, SEQM_P_GPP, a) - par(b, SEQM_P_GP2, a)), 0.1);
    double hpp = hpp_ev / EV;
    double q1 = pow(fabs(hpp) / 3.0 / (qq * qq * qq * qq), 0.2);
    if (hpp < 0.0) q1 = -q1;
    double q2 = q1 + 0.04;
    for (int it = 0; it < 5; ++it) {
      double f1 = 0.25 * q1 - 0.5 / sqrt(4.0 * qq * qq + 1.0 / (q1 * q1)) + 0.25 / sqrt(8.0 * qq * qq + 1.0 / (q1 * q1));
      double f2 = 0.25 * q2 - 0.5 / sqrt(4.0 * qq * qq + 1.0 / (q2 * q2)) + 0.25 / sqrt(8.0 * qq * qq + 1.0 / (q2 * q2));
      double q3 = fabs(f2 - f1) > 1.0e-16 ? q1 + (q2 - q1) * (hpp - f1) / (f2 - f1) : q2;
      q1 = q2;
      q2 = q3;
    }
    rho2 = 0.5 / q2;
  }
  P[SEQM_P_DD * n + a] = dd;
  P[SEQM_P_QQ * n + a] = qq;
  P[SEQM_P_RHO1 * n + a] = rho1;
  P[SEQM_P_RHO2 * n + a] = rho2;
}

// ------------------------------------------------------------- pair kernel
__global__ void __launch_bounds__(128) k_pairs(seqm_batch b, double *__restrict__ w_xx, double *__restrict__ w_xh,
                                               double *__restrict__ w_hh, double *__restrict__ H,
                                               double *__restrict__ enuc, int *__restrict__ err) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  int npairs = b.nxx + b.nxh + b.nhh;
  if (p >= npairs) return;
  const int cls = p < b.nxx ? 2 : (p < b.nxx + b.nxh ? 1 : 0);
  const int ia = b.pair_i[p], ja = b.pair_j[p];
  const int m = b.atom_mol[ia];
  const int a0 = b.mol_atom_off[m], nh = b.mol_nheavy[m], norb = b.mol_norb[m];
  if (b.pair_skip && b.pair_skip[p]) {
    // beyond pair_outer_cutoff: no integrals, no Hcore block, no core-core term
    if (cls == 2) {
      for (int k = 0; k < 100; ++k) w_xx[(size_t)100 * p + k] = 0.0;
    } else if (cls == 1) {
      for (int k = 0; k < 10; ++k) w_xh[(size_t)10 * (p - b.nxx) + k] = 0.0;
    } else {
      w_hh[p - b.nxx - b.nxh] = 0.0;
    }
    enuc[p] = 0.0;
    const int oi = atom_ao(ia - a0, nh), oj = atom_ao(ja - a0, nh);
    const int ni = ia - a0 < nh ? 4 : 1, nj = ja - a0 < nh ? 4 : 1;
    double *Hm = H + b.mol_mat_off[m];
    for (int u = 0; u < ni; ++u)
      for (int v = 0; v < nj; ++v) {
        Hm[(size_t)(oi + u) * norb + oj + v] = 0.0;
        Hm[(size_t)(oj + v) * norb + oi + u] = 0.0;
      }
    return;
  }
  // geometry: x = (Rj - Ri)/|Rj - Ri|, r in bohr (basics.py:316-334)
  double dx = b.atom_xyz[3 * ja] - b.atom_xyz[3 * ia];
  double dy = b.atom_xyz[3 * ja + 1] - b.atom_xyz[3 * ia + 1];
  double dz = b.atom_xyz[3 * ja + 2] - b.atom_xyz[3 * ia + 2];
  double dist = sqrt(dx * dx + dy * dy + dz * dz);
  double r = dist * (1.0 / A0);
  double xv = dx / dist, yv = dy / dist, zv = dz / dist;
  const double r0a = par(b, SEQM_P_RHO0, ia), r0b = par(b, SEQM_P_RHO0, ja);
  double R[3][3];
  quat_rot<double>(-xv, -yv, -zv, R);
  double gam;
  if (cls == 2) {
    double ri[22];
    local_xx<double>(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_DD, ja), par(b, SEQM_P_QQ, ia), par(b, SEQM_P_QQ, ja),
                     r0a, r0b, par(b, SEQM_P_RHO1, ia), par(b, SEQM_P_RHO1, ja), par(b, SEQM_P_RHO2, ia),
                     par(b, SEQM_P_RHO2, ja), ri);
    double *w = w_xx + (size_t)100 * p;
    rotate_xx<double>(ri, R, [&](int a, int c, double v) { w[a * 10 + c] = v; });
    gam = ri[0];
  } else if (cls == 1) {
    double ri[4];
    local_xh<double>(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_QQ, ia), r0a, r0b, par(b, SEQM_P_RHO1, ia),
                     par(b, SEQM_P_RHO2, ia), ri);
    double *w = w_xh + (size_t)10 * (p - b.nxx);
    rotate_xh<double>(ri, R, [&](int a, double v) { w[a] = v; });
    gam = ri[0];
  } else {
    gam = EV / sqrt(r * r + (r0a + r0b) * (r0a + r0b));
    w_hh[p - b.nxx - b.nxh] = gam;
  }
  enuc[p] = core_core<double>(b, ia, ja, r, gam);

  // overlap * (beta_i + beta_j)/2 -> off-diagonal Hcore block, written with its transpose
  double di[4][4];
  if (!overlap_block<double>((int)par(b, SEQM_P_QN, ia), (int)par(b, SEQM_P_QN, ja), r, xv, yv, zv,
                             par(b, SEQM_P_ZS, ia), par(b, SEQM_P_ZP, ia), par(b, SEQM_P_ZS, ja),
                             par(b, SEQM_P_ZP, ja), di)) {
    atomicExch(err, SEQM_E_UNSUPPORTED);
    return;
  }
  const int li = ia - a0, lj = ja - a0;
  const int oi = atom_ao(li, nh), oj = atom_ao(lj, nh);
  const int ni_ = li < nh ? 4 : 1, nj_ = lj < nh ? 4 : 1;
  const double bi[4] = {par(b, SEQM_P_BS, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia)};
  const double bj[4] = {par(b, SEQM_P_BS, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja)};
  double *Hm = H + b.mol_mat_off[m];
  for (int mu = 0; mu < ni_; ++mu)
    for (int nu = 0; nu < nj_; ++nu) {
      double v = di[mu][nu] * ((bi[mu] + bj[nu]) * 0.5);
      Hm[(size_t)(oi + mu) * norb + (oj + nu)] = v;
      Hm[(size_t)(oj + nu) * norb + (oi + mu)] = v;
    }
}

// ------------------------------------------------- diagonal Hcore blocks
// per atom: U_ss/U_pp on the diagonal, then electron-core attractions
// e1b = -Z_B (mu nu | s_B s_B) from pairs where the atom comes first, and
// e2a = -Z_A (s_A s_A | mu nu) from pairs where it comes second (hcore.py:127-150,
// two_elec_two_center_int.py:1535-1572); added in the reference's order.
__global__ void k_hcore_diag(seqm_batch b, const double *__restrict__ w_xx, const double *__restrict__ w_xh,
                             const double *__restrict__ w_hh, double *__restrict__ H) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= b.natoms) return;
  const int m = b.atom_mol[a];
  const int a0 = b.mol_atom_off[m], nat = b.mol_atom_off[m + 1] - a0, nh = b.mol_nheavy[m], ny = nat - nh;
  const int norb = b.mol_norb[m], la = a - a0;
  const int xx0 = b.mol_xx_off[m], xh0 = b.nxx + b.mol_xh_off[m], hh0 = b.nxx + b.nxh + b.mol_hh_off[m];
  double acc[10];
  const double uss = par(b, SEQM_P_USS, a), upp = par(b, SEQM_P_UPP, a);
#pragma unroll
  for (int k = 0; k < 10; ++k) acc[k] = 0.0;
  acc[0] = uss;
  double *Hm = H + b.mol_mat_off[m];
  if (la < nh) {
    acc[2] = upp; acc[5] = upp; acc[9] = upp;
    // first atom of heavy-heavy pairs (la, j>la), then of heavy-H pairs: e1b
    for (int j = la + 1; j < nh; ++j) {
      const double *w = w_xx + (size_t)100 * (xx0 + tri_index(la, j, nh));
      double tb = par(b, SEQM_P_TORE, a0 + j);
#pragma unroll
      for (int k = 0; k < 10; ++k) acc[k] += -tb * w[k * 10];
    }
    for (int h = 0; h < ny; ++h) {
      const double *w = w_xh + (size_t)10 * (xh0 - b.nxx + la * ny + h);
      double tb = par(b, SEQM_P_TORE, a0 + nh + h);
#pragma unroll
      for (int k = 0; k < 10; ++k) acc[k] += -tb * w[k];
    }
    // second atom of heavy-heavy pairs (i<la, la): e2a = -Z_i w[0][k]
    for (int i = 0; i < la; ++i) {
      const double *w = w_xx + (size_t)100 * (xx0 + tri_index(i, la, nh));
      double ta = par(b, SEQM_P_TORE, a0 + i);
#pragma unroll
      for (int k = 0; k < 10; ++k) acc[k] += -ta * w[k];
    }
    const int o = 4 * la;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      int r = k10_row(k), c = k10_col(k);
      Hm[(size_t)(o + r) * norb + o + c] = acc[k];
      Hm[(size_t)(o + c) * norb + o + r] = acc[k];
    }
  } else {
    const int h = la - nh;
    // first atom of H-H pairs (h, g>h): e1b
    for (int g = h + 1; g < ny; ++g) acc[0] += -1.0 * w_hh[hh0 - b.nxx - b.nxh + tri_index(h, g, ny)];
    // second atom of heavy-H pairs (i, h) then of H-H pairs (g<h, h): e2a
    // (the reference adds e2a in pair order: heavy partners come before hydrogen partners)
    for (int i = 0; i < nh; ++i)
      acc[0] += -par(b, SEQM_P_TORE, a0 + i) * w_xh[(size_t)10 * (xh0 - b.nxx + i * ny + h)];
    for (int g = 0; g < h; ++g) acc[0] += -1.0 * w_hh[hh0 - b.nxx - b.nxh + tri_index(g, h, ny)];
    const int o = 3 * nh + la;
    Hm[(size_t)o * norb + o] = acc[0];
  }
}

// per-molecule sum of a per-pair quantity (core-core energies), one CTA per molecule: a molecule
// of thousands of atoms has millions of pairs, which one warp would stream at a small fraction of
// the bandwidth; each thread keeps PS_UNROLL independent sums, added in a fixed order
constexpr int PS_THREADS = 1024, PS_UNROLL = 4;
__global__ void __launch_bounds__(PS_THREADS) k_pair_sum(seqm_batch b, const double *__restrict__ v,
                                                         double *__restrict__ out) {
  __shared__ double red[PS_THREADS / 32];
  const int m = blockIdx.x;
  const int64_t base[3] = {b.mol_xx_off[m], (int64_t)b.nxx + b.mol_xh_off[m],
                           (int64_t)b.nxx + b.nxh + b.mol_hh_off[m]};
  const int64_t len[3] = {b.mol_xx_off[m + 1] - b.mol_xx_off[m], b.mol_xh_off[m + 1] - b.mol_xh_off[m],
                          b.mol_hh_off[m + 1] - b.mol_hh_off[m]};
  double s[PS_UNROLL] = {};
#pragma unroll
  for (int r = 0; r < 3; ++r)
    for (int64_t p = threadIdx.x; p < len[r]; p += PS_UNROLL * PS_THREADS) {
#pragma unroll
      for (int u = 0; u < PS_UNROLL; ++u) {
        const int64_t q = p + (int64_t)u * PS_THREADS;
        if (q < len[r]) s[u] += v[base[r] + q];
      }
    }
  double t = (s[0] + s[1]) + (s[2] + s[3]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < PS_THREADS / 32; ++w) a += red[w];
    out[m] = a;
  }
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_hcore(const seqm_batch *bp, double *w_xx, double *w_xh, double *w_hh, double *H,
                          double *enuc_pair, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.method < SEQM_MNDO || b.method > SEQM_PM6_SP) return SEQM_E_ARG;
  if (b.method == SEQM_PM6_SP && (!b.pair_par || b.pair_zmax < 0)) return SEQM_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int npairs = b.nxx + b.nxh + b.nhh;
  if (b.natoms <= 0) return SEQM_OK;
  k_atom_prep<<<(b.natoms + 127) / 128, 128, 0, s>>>(b);
  // per-device error word (one int, kept for the process); calls from several host threads
  // (one stream each) take turns on it from the reset to the read-back
  static int *d_err[64] = {};
  static std::mutex err_lock;
  std::lock_guard<std::mutex> guard(err_lock);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return SEQM_E_CUDA;
  if (!d_err[dev] && cudaMalloc(&d_err[dev], sizeof(int)) != cudaSuccess) return SEQM_E_CUDA;
  if (cudaMemsetAsync(d_err[dev], 0, sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
  if (npairs > 0) {
    k_pairs<<<(npairs + 127) / 128, 128, 0, s>>>(b, w_xx, w_xh, w_hh, H, enuc_pair, d_err[dev]);
  }
  k_hcore_diag<<<(b.natoms + 127) / 128, 128, 0, s>>>(b, w_xx, w_xh, w_hh, H);
  int rc = launch_check();
  if (rc) return rc;
  int herr = 0;
  if (cudaMemcpyAsync(&herr, d_err[dev], sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SEQM_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SEQM_E_CUDA;
  return herr;
}

extern "C" int seqm_pair_sum(const seqm_batch *bp, const double *pair_val, double *mol_sum, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol <= 0) return SEQM_OK;
  k_pair_sum<<<b.nmol, PS_THREADS, 0, (cudaStream_t)stream>>>(b, pair_val, mol_sum);
  return launch_check();
}
