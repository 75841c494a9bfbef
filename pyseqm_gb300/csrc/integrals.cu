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

#include "common.cuh"

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
    double d1 = cbrt(fabs(hsp) / (dd * dd));
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

// --------------------------------------------------------- local integrals
__device__ __forceinline__ double inv_sqrt_ev(double c, double x) { return c / sqrt(x); }

// heavy-heavy: 22 integrals in the local frame (repp, MOPAC numbering 1..22 -> ri[0..21])
__device__ void local_xx(double r, double da, double db, double qa0, double qb0, double r0a, double r0b, double r1a,
                         double r1b, double r2a, double r2b, double *ri) {
  const double ev1 = EV / 2.0, ev2 = EV / 4.0, ev3 = EV / 8.0, ev4 = EV / 16.0;
  const double qa = qa0 * 2.0, qb = qb0 * 2.0, qa1 = qa0, qb1 = qb0;
  const double aee = (r0a + r0b) * (r0a + r0b), ade = (r1a + r0b) * (r1a + r0b), aqe = (r2a + r0b) * (r2a + r0b);
  const double aed = (r0a + r1b) * (r0a + r1b), aeq = (r0a + r2b) * (r0a + r2b), axx = (r1a + r1b) * (r1a + r1b);
  const double adq = (r1a + r2b) * (r1a + r2b), aqd = (r2a + r1b) * (r2a + r1b), aqq = (r2a + r2b) * (r2a + r2b);
  const double r2 = r * r;
#define SQ(x) ((x) * (x))
  double ee = EV / sqrt(r2 + aee);
  double dze = -ev1 / sqrt(SQ(r + da) + ade) + ev1 / sqrt(SQ(r - da) + ade);
  double e6 = ev1 / sqrt(r2 + aqe);
  double qzze = ev2 / sqrt(SQ(r - qa) + aqe) + ev2 / sqrt(SQ(r + qa) + aqe) - e6;
  double qxxe = ev1 / sqrt(r2 + qa * qa + aqe) - e6;
  double edz = -ev1 / sqrt(SQ(r - db) + aed) + ev1 / sqrt(SQ(r + db) + aed);
  double e12 = ev1 / sqrt(r2 + aeq);
  double eqzz = ev2 / sqrt(SQ(r - qb) + aeq) + ev2 / sqrt(SQ(r + qb) + aeq) - e12;
  double eqxx = ev1 / sqrt(r2 + qb * qb + aeq) - e12;
  double e20 = ev2 / sqrt(SQ(r + da) + adq), e22 = ev2 / sqrt(SQ(r - da) + adq);
  double e24 = ev2 / sqrt(SQ(r - db) + aqd), e26 = ev2 / sqrt(SQ(r + db) + aqd);
  double e36 = ev2 / sqrt(r2 + aqq), e39 = ev2 / sqrt(r2 + qa * qa + aqq), e40 = ev2 / sqrt(r2 + qb * qb + aqq);
  double e42 = ev3 / sqrt(SQ(r - qb) + aqq), e44 = ev3 / sqrt(SQ(r + qb) + aqq);
  double e46 = ev3 / sqrt(SQ(r + qa) + aqq), e48 = ev3 / sqrt(SQ(r - qa) + aqq);
  ri[0] = ee;
  ri[1] = -dze;
  ri[2] = ee + qzze;
  ri[3] = ee + qxxe;
  ri[4] = -edz;
  ri[5] = ev2 / sqrt(SQ(r + da - db) + axx) + ev2 / sqrt(SQ(r - da + db) + axx) - ev2 / sqrt(SQ(r - da - db) + axx) -
          ev2 / sqrt(SQ(r + da + db) + axx);
  ri[6] = ev1 / sqrt(r2 + SQ(da - db) + axx) - ev1 / sqrt(r2 + SQ(da + db) + axx);
  ri[7] = -edz + ev3 / sqrt(SQ(r + qa - db) + aqd) - ev3 / sqrt(SQ(r + qa + db) + aqd) +
          ev3 / sqrt(SQ(r - qa - db) + aqd) - ev3 / sqrt(SQ(r - qa + db) + aqd) - e24 + e26;
  ri[8] = -edz - e24 + ev2 / sqrt(SQ(r - db) + qa * qa + aqd) + e26 - ev2 / sqrt(SQ(r + db) + qa * qa + aqd);
  ri[9] = ev2 / sqrt(SQ(qa1 - db) + SQ(r + qa1) + aqd) - ev2 / sqrt(SQ(qa1 - db) + SQ(r - qa1) + aqd) -
          ev2 / sqrt(SQ(qa1 + db) + SQ(r + qa1) + aqd) + ev2 / sqrt(SQ(qa1 + db) + SQ(r - qa1) + aqd);
  ri[10] = ee + eqzz;
  ri[11] = ee + eqxx;
  ri[12] = -dze + ev3 / sqrt(SQ(r + da - qb) + adq) - ev3 / sqrt(SQ(r - da - qb) + adq) +
           ev3 / sqrt(SQ(r + da + qb) + adq) - ev3 / sqrt(SQ(r - da + qb) + adq) + e22 - e20;
  ri[13] = -dze - e20 + ev2 / sqrt(SQ(r + da) + qb * qb + adq) + e22 - ev2 / sqrt(SQ(r - da) + qb * qb + adq);
  ri[14] = ev2 / sqrt(SQ(da - qb1) + SQ(r - qb1) + adq) - ev2 / sqrt(SQ(da - qb1) + SQ(r + qb1) + adq) -
           ev2 / sqrt(SQ(da + qb1) + SQ(r - qb1) + adq) + ev2 / sqrt(SQ(da + qb1) + SQ(r + qb1) + adq);
  ri[15] = ee + eqzz + qzze + ev4 / sqrt(SQ(r + qa - qb) + aqq) + ev4 / sqrt(SQ(r + qa + qb) + aqq) +
           ev4 / sqrt(SQ(r - qa - qb) + aqq) + ev4 / sqrt(SQ(r - qa + qb) + aqq) - e48 - e46 - e42 - e44 + e36;
  ri[16] = ee + eqzz + qxxe + ev3 / sqrt(SQ(r - qb) + qa * qa + aqq) + ev3 / sqrt(SQ(r + qb) + qa * qa + aqq) - e42 -
           e44 - e39 + e36;
  ri[17] = ee + eqxx + qzze + ev3 / sqrt(SQ(r + qa) + qb * qb + aqq) + ev3 / sqrt(SQ(r - qa) + qb * qb + aqq) - e46 -
           e48 - e40 + e36;
  double qxxqxx = ev3 / sqrt(r2 + SQ(qa - qb) + aqq) + ev3 / sqrt(r2 + SQ(qa + qb) + aqq) - e39 - e40 + e36;
  ri[18] = ee + eqxx + qxxe + qxxqxx;
  ri[19] = ev3 / sqrt(SQ(r + qa1 - qb1) + SQ(qa1 - qb1) + aqq) - ev3 / sqrt(SQ(r + qa1 + qb1) + SQ(qa1 - qb1) + aqq) -
           ev3 / sqrt(SQ(r - qa1 - qb1) + SQ(qa1 - qb1) + aqq) + ev3 / sqrt(SQ(r - qa1 + qb1) + SQ(qa1 - qb1) + aqq) -
           ev3 / sqrt(SQ(r + qa1 - qb1) + SQ(qa1 + qb1) + aqq) + ev3 / sqrt(SQ(r + qa1 + qb1) + SQ(qa1 + qb1) + aqq) +
           ev3 / sqrt(SQ(r - qa1 - qb1) + SQ(qa1 + qb1) + aqq) - ev3 / sqrt(SQ(r - qa1 + qb1) + SQ(qa1 + qb1) + aqq);
  double qxxqyy = ev2 / sqrt(r2 + qa * qa + qb * qb + aqq) - e39 - e40 + e36;
  ri[20] = ee + eqxx + qxxe + qxxqyy;
  ri[21] = 0.5 * (qxxqxx - qxxqyy);
}

// heavy-hydrogen: 4 integrals (sigma-type only)
__device__ void local_xh(double r, double da, double qa0, double r0a, double r0b, double r1a, double r2a, double *ri) {
  const double ev1 = EV / 2.0, ev2 = EV / 4.0;
  const double aee = (r0a + r0b) * (r0a + r0b), ade = (r1a + r0b) * (r1a + r0b), aqe = (r2a + r0b) * (r2a + r0b);
  const double qa = qa0 * 2.0;
  double e6 = ev1 / sqrt(r * r + aqe);
  double ee = EV / sqrt(r * r + aee);
  ri[0] = ee;
  ri[1] = ev1 / sqrt(SQ(r + da) + ade) - ev1 / sqrt(SQ(r - da) + ade);
  ri[2] = ee + ev2 / sqrt(SQ(r + qa) + aqe) + ev2 / sqrt(SQ(r - qa) + aqe) - e6;
  ri[3] = ee + ev1 / sqrt(r * r + qa * qa + aqe) - e6;
}

// ---------------------------------------------------------------- rotation
// rotation matrix taking unit vector v onto +x via the quaternion (0, v_z, -v_y, 1+v_x);
// |1+v_x| < 1e-7 uses a half turn about z (two_elec_two_center_int.py:1576-1631)
__device__ void quat_rot(double vx, double vy, double vz, double R[3][3]) {
  double qx = 0.0, qy = vz, qz = -vy, qw = 1.0 + vx;
  if (fabs(qw) < 1.0e-7) { qx = 0.0; qy = 0.0; qz = 1.0; qw = 0.0; }
  double nrm = sqrt(qx * qx + qy * qy + qz * qz + qw * qw);
  qy /= nrm; qz /= nrm; qw /= nrm;
  R[0][0] = 1 - 2 * (qy * qy + qz * qz);
  R[0][1] = -2 * (qz * qw);
  R[0][2] = 2 * (qy * qw);
  R[1][0] = 2 * (qz * qw);
  R[1][1] = 1 - 2 * (qz * qz);
  R[1][2] = 2 * (qy * qz);
  R[2][0] = -2 * (qy * qw);
  R[2][1] = 2 * (qy * qz);
  R[2][2] = 1 - 2 * (qy * qy);
}

// heavy-heavy rotated block, w[a*10+b]; a = (kk,ll) of atom i, b = (mm,nn) of atom j
__device__ void rotate_xx(const double *ri, const double R[3][3], double *__restrict__ w) {
  const double *r0 = R[0], *r1 = R[1], *r2 = R[2];
  int a = 0;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
    for (int ll = 0; ll <= kk; ++ll, ++a) {
      int b = 0;
#pragma unroll
      for (int mm = 0; mm < 4; ++mm) {
#pragma unroll
        for (int nn = 0; nn <= mm; ++nn, ++b) {
          const int k = kk - 1, l = ll - 1, m = mm - 1, n = nn - 1;
          double val;
          if (kk == 0) {
            if (mm == 0) val = ri[0];
            else if (nn == 0) val = ri[4] * r0[m];
            else val = ri[10] * (r0[m] * r0[n]) + ri[11] * (r1[m] * r1[n] + r2[m] * r2[n]);
          } else if (ll == 0) {
            if (mm == 0) val = ri[1] * r0[k];
            else if (nn == 0) val = ri[5] * (r0[k] * r0[m]) + ri[6] * (r1[k] * r1[m] + r2[k] * r2[m]);
            else {
              double t0 = r0[k] * r0[m] * r0[n];
              double t1 = (r1[m] * r1[n] + r2[m] * r2[n]) * r0[k];
              double mix = r1[k] * (r1[n] * r0[m] + r1[m] * r0[n]) + r2[k] * (r2[m] * r0[n] + r2[n] * r0[m]);
              val = ri[12] * t0 + ri[13] * t1 + ri[14] * mix;
            }
          } else {
            if (mm == 0) val = ri[2] * (r0[k] * r0[l]) + ri[3] * (r1[k] * r1[l] + r2[k] * r2[l]);
            else if (nn == 0) {
              double t0 = r0[k] * r0[l] * r0[m];
              double t1 = (r1[k] * r1[l] + r2[k] * r2[l]) * r0[m];
              double t2 = r1[l] * r1[m] + r2[l] * r2[m];
              val = ri[7] * t0 + ri[8] * t1 + ri[9] * (r0[k] * t2 + r0[l] * (r1[k] * r1[m] + r2[k] * r2[m]));
            } else {
              val = ri[15] * (r0[k] * r0[l] * r0[m] * r0[n]);
              val += ri[16] * ((r1[k] * r1[l] + r2[k] * r2[l]) * r0[m] * r0[n]);
              val += ri[17] * ((r1[m] * r1[n] + r2[m] * r2[n]) * (r0[k] * r0[l]));
              val += ri[18] * (r1[k] * r1[l] * r1[m] * r1[n] + r2[k] * r2[l] * r2[m] * r2[n]);
              double mix1 = r0[m] * (r1[l] * r1[n] + r2[l] * r2[n]);
              double mix2 = r0[n] * (r1[l] * r1[m] + r2[l] * r2[m]);
              double val5 = r0[k] * (mix1 + mix2) +
                            r0[l] * (r0[m] * (r1[k] * r1[n] + r2[k] * r2[n]) + r0[n] * (r1[k] * r1[m] + r2[k] * r2[m]));
              val += ri[19] * val5;
              val += ri[20] * (r1[k] * r1[l] * r2[m] * r2[n] + r2[k] * r2[l] * r1[m] * r1[n]);
              val += ri[21] * ((r1[k] * r2[l] + r2[k] * r1[l]) * (r1[m] * r2[n] + r2[m] * r1[n]));
            }
          }
          w[a * 10 + b] = val;
        }
      }
    }
  }
}

__device__ void rotate_xh(const double *ri, const double R[3][3], double *__restrict__ w) {
  int a = 0;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
    for (int ll = 0; ll <= kk; ++ll, ++a) {
      const int k = kk - 1, l = ll - 1;
      double val;
      if (kk == 0) val = ri[0];
      else if (ll == 0) val = ri[1] * R[0][k];
      else val = ri[2] * R[0][k] * R[0][l] + ri[3] * (R[1][k] * R[1][l] + R[2][k] * R[2][l]);
      w[a] = val;
    }
  }
}

// ----------------------------------------------------------------- overlap
// auxiliary integrals A_k(x), k = 0..6 (diat_overlap_PM6_SP.py:464-519)
__device__ void aint(double x, double *a) {
  double xs = x != 0.0 ? x : INFINITY;
  a[0] = exp(-xs) / xs;
  a[1] = a[0] + a[0] / xs;
#pragma unroll
  for (int k = 2; k < 7; ++k) a[k] = a[0] + k * a[k - 1] / xs;
}

// auxiliary integrals B_k(x), k = 0..6 (diat_overlap_PM6_SP.py:522-670)
__device__ void bint(double x, double *b) {
  double ax = fabs(x);
  if (ax > 0.5) {
    double tx = exp(x) / x, tmx = -exp(-x) / x;
    b[0] = tx + tmx;
#pragma unroll
    for (int k = 1; k < 7; ++k) b[k] = ((k & 1) ? -tx : tx) + tmx + k * b[k - 1] / x;
  } else if (ax > 1.0e-6) {
    double x2 = x * x, x3 = x2 * x, x4 = x2 * x2, x5 = x4 * x, x6 = x4 * x2;
    b[0] = 2.0 + x2 / 3.0 + x4 / 60.0 + x6 / 2520.0;
    b[2] = 2.0 / 3.0 + x2 / 5.0 + x4 / 84.0 + x6 / 3240.0;
    b[4] = 2.0 / 5.0 + x2 / 7.0 + x4 / 108.0 + x6 / 3960.0;
    b[6] = 2.0 / 7.0 + x2 / 9.0 + x4 / 132.0 + x6 / 4680.0;
    b[1] = -2.0 / 3.0 * x - x3 / 15.0 - x5 / 420.0;
    b[3] = -2.0 / 5.0 * x - x3 / 21.0 - x5 / 540.0;
    b[5] = -2.0 / 7.0 * x - x3 / 27.0 - x5 / 660.0;
  } else {
    b[0] = 2.0; b[1] = 0.0; b[2] = 2.0 / 3.0; b[3] = 0.0; b[4] = 2.0 / 5.0; b[5] = 0.0; b[6] = 2.0 / 7.0;
  }
}

struct Sloc { double s111, s211, s121, s221, s222; };

// local-frame overlaps for the principal-quantum-number classes (diat_overlap_PM6_SP.py:56-312);
// returns false for an unsupported class (the reference raises ValueError)
__device__ bool overlap_local(int qni, int qnj, double r, double zsa, double zpa, double zsb, double zpb, Sloc &S) {
  S.s111 = S.s211 = S.s121 = S.s221 = S.s222 = 0.0;
  double A[7], B[7];
  const double s3 = sqrt(3.0), s10 = sqrt(10.0), s30 = sqrt(30.0);
  auto set = [&](double za, double zb) { aint(0.5 * r * (za + zb), A); bint(0.5 * r * (za - zb), B); };
  if (qni == 1 && qnj == 1) {
    set(zsa, zsb);
    S.s111 = pow(zsa * zsb * r * r, 1.5) * (A[2] * B[0] - B[2] * A[0]) / 4.0;
  } else if (qni == 2 && qnj == 1) {
    double r4 = r * r * r * r;
    set(zsa, zsb);
    S.s111 = pow(zsb, 1.5) * pow(zsa, 2.5) * r4 * (A[3] * B[0] - B[3] * A[0] + A[2] * B[1] - B[2] * A[1]) / (s3 * 8.0);
    set(zpa, zsb);
    S.s211 = pow(zsb, 1.5) * pow(zpa, 2.5) * r4 * (A[2] * B[0] - B[2] * A[0] + A[3] * B[1] - B[3] * A[1]) / 8.0;
  } else if (qni == 2 && qnj == 2) {
    double r5 = r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = pow(zsb * zsa, 2.5) * r5 * (A[4] * B[0] + B[4] * A[0] - 2.0 * A[2] * B[2]) / 48.0;
    set(zpa, zsb);
    S.s211 = pow(zsb * zpa, 2.5) * r5 *
             (A[3] * (B[0] - B[2]) - A[1] * (B[2] - B[4]) + B[3] * (A[0] - A[2]) - B[1] * (A[2] - A[4])) / (16.0 * s3);
    set(zsa, zpb);
    S.s121 = pow(zpb * zsa, 2.5) * r5 *
             (A[3] * (B[0] - B[2]) - A[1] * (B[2] - B[4]) - B[3] * (A[0] - A[2]) + B[1] * (A[2] - A[4])) / (16.0 * s3);
    set(zpa, zpb);
    double w = pow(zpb * zpa, 2.5) * r5 / 16.0;
    S.s221 = -w * (B[2] * (A[4] + A[0]) - A[2] * (B[4] + B[0]));
    S.s222 = 0.5 * w * (A[4] * (B[0] - B[2]) - B[4] * (A[0] - A[2]) - A[2] * B[0] + B[2] * A[0]);
  } else if (qni == 3 && qnj == 1) {
    double r5 = r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = pow(zsb, 1.5) * pow(zsa, 3.5) * r5 * (A[4] * B[0] + 2 * B[1] * A[3] - 2.0 * A[1] * B[3] - B[4] * A[0]) /
             (s10 * 24.0);
    set(zpa, zsb);
    S.s211 = pow(zsb, 1.5) * pow(zpa, 3.5) * r5 *
             (A[3] * (B[0] + B[2]) - A[1] * (B[4] + B[2]) + B[1] * (A[2] + A[4]) - B[3] * (A[2] + A[0])) / (8.0 * s30);
  } else if (qni == 3 && qnj == 2) {
    double r6 = r * r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = pow(zsb, 2.5) * pow(zsa, 3.5) * r6 *
             (A[5] * B[0] + B[1] * A[4] - 2 * B[2] * A[3] - 2.0 * A[2] * B[3] + B[4] * A[1] + B[5] * A[0]) / (s30 * 48.0);
    set(zpa, zsb);
    S.s211 = pow(zsb, 2.5) * pow(zpa, 3.5) * r6 *
             (A[4] * B[0] + B[1] * A[5] - 2.0 * B[3] * A[3] - 2.0 * A[2] * B[2] + A[1] * B[5] + A[0] * B[4]) / (48.0 * s10);
    set(zsa, zpb);
    S.s121 = pow(zpb, 2.5) * pow(zsa, 3.5) * r6 *
             ((A[4] * B[0] - A[5] * B[1]) + 2.0 * (A[3] * B[1] - A[4] * B[2]) - 2.0 * (A[1] * B[3] - A[2] * B[4]) -
              (A[0] * B[4] - A[1] * B[5])) / (48.0 * s10);
    set(zpa, zpb);
    S.s221 = pow(zpb, 2.5) * pow(zpa, 3.5) * r6 *
             ((A[3] * B[0] - A[5] * B[2]) + (A[2] * B[1] - A[4] * B[3]) - (A[1] * B[2] - A[3] * B[4]) -
              (A[0] * B[3] - A[2] * B[5])) / (16.0 * s30);
    S.s222 = pow(zpb, 2.5) * pow(zpa, 3.5) * r6 *
             ((A[5] - A[3]) * (B[0] - B[2]) + (A[4] - A[2]) * (B[1] - B[3]) - (A[3] - A[1]) * (B[2] - B[4]) -
              (A[2] - A[0]) * (B[3] - B[5])) / (32.0 * s30);
  } else if (qni == 3 && qnj == 3) {
    double r7 = r * r * r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = pow(zsb * zsa, 3.5) * r7 * (A[6] * B[0] - 3.0 * B[2] * A[4] + 3.0 * A[2] * B[4] - A[0] * B[6]) / 1440.0;
    set(zpa, zsb);
    S.s211 = pow(zsb * zpa, 3.5) * r7 *
             ((A[5] * B[0] + A[6] * B[1]) + (-A[4] * B[1] - A[5] * B[2]) - 2.0 * (A[3] * B[2] + A[4] * B[3]) -
              2.0 * (-A[2] * B[3] - A[3] * B[4]) + (A[1] * B[4] + A[2] * B[5]) + (-A[0] * B[5] - A[1] * B[6])) /
             (480.0 * s3);
    set(zsa, zpb);
    S.s121 = pow(zpb * zsa, 3.5) * r7 *
             ((A[5] * B[0] - A[6] * B[1]) + (A[4] * B[1] - A[5] * B[2]) - 2.0 * (A[3] * B[2] - A[4] * B[3]) -
              2.0 * (A[2] * B[3] - A[3] * B[4]) + (A[1] * B[4] - A[2] * B[5]) + (A[0] * B[5] - A[1] * B[6])) /
             (480.0 * s3);
    set(zpa, zpb);
    S.s221 = pow(zpb, 3.5) * pow(zpa, 3.5) * r7 *
             ((A[4] * B[0] - A[6] * B[2]) - 2.0 * (A[2] * B[2] - A[4] * B[4]) + (A[0] * B[4] - A[2] * B[6])) / 480.0;
    S.s222 = pow(zpb, 3.5) * pow(zpa, 3.5) * r7 *
             ((A[6] - A[4]) * (B[0] - B[2]) - 2.0 * (A[4] - A[2]) * (B[2] - B[4]) + (A[2] - A[0]) * (B[4] - B[6])) /
             960.0;
  } else {
    return false;
  }
  return true;
}
#undef SQ

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
  // geometry: x = (Rj - Ri)/|Rj - Ri|, r in bohr (basics.py:316-334)
  double dx = b.atom_xyz[3 * ja] - b.atom_xyz[3 * ia];
  double dy = b.atom_xyz[3 * ja + 1] - b.atom_xyz[3 * ia + 1];
  double dz = b.atom_xyz[3 * ja + 2] - b.atom_xyz[3 * ia + 2];
  double dist = sqrt(dx * dx + dy * dy + dz * dz);
  double r = dist * (1.0 / A0);
  double xv = dx / dist, yv = dy / dist, zv = dz / dist;
  const double r0a = par(b, SEQM_P_RHO0, ia), r0b = par(b, SEQM_P_RHO0, ja);
  double R[3][3];
  quat_rot(-xv, -yv, -zv, R);
  double gam;
  if (cls == 2) {
    double ri[22];
    local_xx(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_DD, ja), par(b, SEQM_P_QQ, ia), par(b, SEQM_P_QQ, ja), r0a, r0b,
             par(b, SEQM_P_RHO1, ia), par(b, SEQM_P_RHO1, ja), par(b, SEQM_P_RHO2, ia), par(b, SEQM_P_RHO2, ja), ri);
    rotate_xx(ri, R, w_xx + (size_t)100 * p);
    gam = ri[0];
  } else if (cls == 1) {
    double ri[4];
    local_xh(r, par(b, SEQM_P_DD, ia), par(b, SEQM_P_QQ, ia), r0a, r0b, par(b, SEQM_P_RHO1, ia),
             par(b, SEQM_P_RHO2, ia), ri);
    rotate_xh(ri, R, w_xh + (size_t)10 * (p - b.nxx));
    gam = ri[0];
  } else {
    gam = EV / sqrt(r * r + (r0a + r0b) * (r0a + r0b));
    w_hh[p - b.nxx - b.nxh] = gam;
  }

  // core-core repulsion (energy.py:91-134)
  {
    const int Zi = b.atom_Z[ia], Zj = b.atom_Z[ja];
    double rija = r * A0;
    double ti = par(b, SEQM_P_TORE, ia), tj = par(b, SEQM_P_TORE, ja);
    double t1 = ti * tj * gam;
    double tmp = exp(-par(b, SEQM_P_ALPHA, ia) * rija);
    double t2 = ((Zi == 7 || Zi == 8) && Zj == 1) ? tmp * rija : tmp;
    double t3 = exp(-par(b, SEQM_P_ALPHA, ja) * rija);
    double e = t1 * (1.0 + t2 + t3);
    int ng = b.method == SEQM_AM1 ? 4 : (b.method == SEQM_PM3 ? 2 : 0);
    if (ng) {
      double t4 = ti * tj / rija, t5 = 0.0, t6 = 0.0;
      for (int g = 0; g < ng; ++g) {
        double Ki = par(b, SEQM_P_K1 + g, ia), Li = par(b, SEQM_P_L1 + g, ia), Mi = par(b, SEQM_P_M1 + g, ia);
        double Kj = par(b, SEQM_P_K1 + g, ja), Lj = par(b, SEQM_P_L1 + g, ja), Mj = par(b, SEQM_P_M1 + g, ja);
        t5 += Ki * exp(-Li * (rija - Mi) * (rija - Mi));
        t6 += Kj * exp(-Lj * (rija - Mj) * (rija - Mj));
      }
      e += t4 * (t5 + t6);
    }
    enuc[p] = e;
  }

  // overlap * (beta_i + beta_j)/2 -> off-diagonal Hcore block, written with its transpose
  {
    double di[4][4] = {};
    if (r <= OVERLAP_CUTOFF) {
      Sloc S;
      if (!overlap_local((int)par(b, SEQM_P_QN, ia), (int)par(b, SEQM_P_QN, ja), r, par(b, SEQM_P_ZS, ia),
                         par(b, SEQM_P_ZP, ia), par(b, SEQM_P_ZS, ja), par(b, SEQM_P_ZP, ja), S)) {
        atomicExch(err, SEQM_E_UNSUPPORTED);
        return;
      }
      double Q[3][3];
      quat_rot(xv, yv, zv, Q);
      di[0][0] = S.s111;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        di[1 + a][0] = S.s211 * Q[0][a];
        di[0][1 + a] = -S.s121 * Q[0][a];
      }
      const double Mv[3] = {-S.s221, S.s222, S.s222};
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          di[1 + a][1 + c] = Q[0][a] * Mv[0] * Q[0][c] + Q[1][a] * Mv[1] * Q[1][c] + Q[2][a] * Mv[2] * Q[2][c];
    }
    const int li = ia - a0, lj = ja - a0;
    const int oi = atom_ao(li, nh), oj = atom_ao(lj, nh);
    const int ni_ = li < nh ? 4 : 1, nj_ = lj < nh ? 4 : 1;
    double bi[4] = {par(b, SEQM_P_BS, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia), par(b, SEQM_P_BP, ia)};
    double bj[4] = {par(b, SEQM_P_BS, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja), par(b, SEQM_P_BP, ja)};
    double *Hm = H + b.mol_mat_off[m];
    for (int mu = 0; mu < ni_; ++mu)
      for (int nu = 0; nu < nj_; ++nu) {
        double v = di[mu][nu] * ((bi[mu] + bj[nu]) * 0.5);
        Hm[(size_t)(oi + mu) * norb + (oj + nu)] = v;
        Hm[(size_t)(oj + nu) * norb + (oi + mu)] = v;
      }
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

// per-molecule sum of a per-pair quantity (core-core energies), warp per molecule
__global__ void k_pair_sum(seqm_batch b, const double *__restrict__ v, double *__restrict__ out) {
  int m = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int lane = threadIdx.x & 31;
  if (m >= b.nmol) return;
  double s = 0.0;
  for (int p = b.mol_xx_off[m] + lane; p < b.mol_xx_off[m + 1]; p += 32) s += v[p];
  for (int p = b.mol_xh_off[m] + lane; p < b.mol_xh_off[m + 1]; p += 32) s += v[b.nxx + p];
  for (int p = b.mol_hh_off[m] + lane; p < b.mol_hh_off[m + 1]; p += 32) s += v[b.nxx + b.nxh + p];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[m] = s;
}

}  // namespace seqm

using namespace seqm;

extern "C" int seqm_hcore(const seqm_batch *bp, double *w_xx, double *w_xh, double *w_hh, double *H,
                          double *enuc_pair, void *stream) {
  if (!bp) return SEQM_E_ARG;
  seqm_batch b = *bp;
  cudaStream_t s = (cudaStream_t)stream;
  int npairs = b.nxx + b.nxh + b.nhh;
  if (b.natoms <= 0) return SEQM_OK;
  k_atom_prep<<<(b.natoms + 127) / 128, 128, 0, s>>>(b);
  static int *d_err[64] = {};  // per-device error word (one int, kept for the process)
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
  k_pair_sum<<<(b.nmol + 7) / 8, 256, 0, (cudaStream_t)stream>>>(b, pair_val, mol_sum);
  return launch_check();
}
