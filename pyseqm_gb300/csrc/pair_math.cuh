// Per-pair integral mathematics, templated on the scalar type.
//
// T = double: the forward integrals (integrals.cu).
// T = Dual3:  the same code carrying d/dx, d/dy, d/dz of the interatomic vector
//             (forward-mode derivatives), used by the gradient kernel (grad.cu)
//             to differentiate w, the overlap and the core-core energy of a pair
//             without storing any integral derivative.
#pragma once

#include <math.h>

#include "common.cuh"

namespace seqm {

// the double overloads stay visible next to the Dual3 ones declared below
using ::exp;
using ::pow;
using ::sqrt;

// ----------------------------------------------------------------- dual numbers
struct Dual3 {
  double v, d0, d1, d2;
  __device__ Dual3() : v(0), d0(0), d1(0), d2(0) {}
  __device__ Dual3(double x) : v(x), d0(0), d1(0), d2(0) {}
  __device__ Dual3(double x, double a, double b, double c) : v(x), d0(a), d1(b), d2(c) {}
};
__device__ __forceinline__ Dual3 operator+(Dual3 a, Dual3 b) { return Dual3(a.v + b.v, a.d0 + b.d0, a.d1 + b.d1, a.d2 + b.d2); }
__device__ __forceinline__ Dual3 operator-(Dual3 a, Dual3 b) { return Dual3(a.v - b.v, a.d0 - b.d0, a.d1 - b.d1, a.d2 - b.d2); }
__device__ __forceinline__ Dual3 operator-(Dual3 a) { return Dual3(-a.v, -a.d0, -a.d1, -a.d2); }
__device__ __forceinline__ Dual3 operator*(Dual3 a, Dual3 b) {
  return Dual3(a.v * b.v, a.d0 * b.v + a.v * b.d0, a.d1 * b.v + a.v * b.d1, a.d2 * b.v + a.v * b.d2);
}
__device__ __forceinline__ Dual3 operator/(Dual3 a, Dual3 b) {
  double q = a.v / b.v, ib = 1.0 / b.v;
  return Dual3(q, (a.d0 - q * b.d0) * ib, (a.d1 - q * b.d1) * ib, (a.d2 - q * b.d2) * ib);
}
__device__ __forceinline__ Dual3 operator+(Dual3 a, double b) { return Dual3(a.v + b, a.d0, a.d1, a.d2); }
__device__ __forceinline__ Dual3 operator+(double b, Dual3 a) { return Dual3(a.v + b, a.d0, a.d1, a.d2); }
__device__ __forceinline__ Dual3 operator-(Dual3 a, double b) { return Dual3(a.v - b, a.d0, a.d1, a.d2); }
__device__ __forceinline__ Dual3 operator-(double b, Dual3 a) { return Dual3(b - a.v, -a.d0, -a.d1, -a.d2); }
__device__ __forceinline__ Dual3 operator*(Dual3 a, double b) { return Dual3(a.v * b, a.d0 * b, a.d1 * b, a.d2 * b); }
__device__ __forceinline__ Dual3 operator*(double b, Dual3 a) { return Dual3(a.v * b, a.d0 * b, a.d1 * b, a.d2 * b); }
__device__ __forceinline__ Dual3 operator/(Dual3 a, double b) { return Dual3(a.v / b, a.d0 / b, a.d1 / b, a.d2 / b); }
__device__ __forceinline__ Dual3 operator/(double a, Dual3 b) {
  double q = a / b.v, s = -q / b.v;
  return Dual3(q, s * b.d0, s * b.d1, s * b.d2);
}
__device__ __forceinline__ Dual3 &operator+=(Dual3 &a, Dual3 b) { a = a + b; return a; }
__device__ __forceinline__ Dual3 sqrt(Dual3 a) {
  double r = ::sqrt(a.v), s = 0.5 / r;
  return Dual3(r, s * a.d0, s * a.d1, s * a.d2);
}
__device__ __forceinline__ Dual3 exp(Dual3 a) {
  double e = ::exp(a.v);
  return Dual3(e, e * a.d0, e * a.d1, e * a.d2);
}
__device__ __forceinline__ Dual3 pow(Dual3 a, double p) {
  double r = ::pow(a.v, p), s = p * ::pow(a.v, p - 1.0);
  return Dual3(r, s * a.d0, s * a.d1, s * a.d2);
}
__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const Dual3 &x) { return x.v; }

// ------------------------------------------------------------ local integrals
#define SQ(x) ((x) * (x))
// heavy-heavy: 22 integrals in the local frame (repp, MOPAC numbering 1..22 -> ri[0..21])
template <class T>
__device__ void local_xx(T r, double da, double db, double qa0, double qb0, double r0a, double r0b, double r1a,
                         double r1b, double r2a, double r2b, T *ri) {
  const double ev1 = EV / 2.0, ev2 = EV / 4.0, ev3 = EV / 8.0, ev4 = EV / 16.0;
  const double qa = qa0 * 2.0, qb = qb0 * 2.0, qa1 = qa0, qb1 = qb0;
  const double aee = (r0a + r0b) * (r0a + r0b), ade = (r1a + r0b) * (r1a + r0b), aqe = (r2a + r0b) * (r2a + r0b);
  const double aed = (r0a + r1b) * (r0a + r1b), aeq = (r0a + r2b) * (r0a + r2b), axx = (r1a + r1b) * (r1a + r1b);
  const double adq = (r1a + r2b) * (r1a + r2b), aqd = (r2a + r1b) * (r2a + r1b), aqq = (r2a + r2b) * (r2a + r2b);
  const T r2 = r * r;
  T ee = EV / sqrt(r2 + aee);
  T dze = -ev1 / sqrt(SQ(r + da) + ade) + ev1 / sqrt(SQ(r - da) + ade);
  T e6 = ev1 / sqrt(r2 + aqe);
  T qzze = ev2 / sqrt(SQ(r - qa) + aqe) + ev2 / sqrt(SQ(r + qa) + aqe) - e6;
  T qxxe = ev1 / sqrt(r2 + qa * qa + aqe) - e6;
  T edz = -ev1 / sqrt(SQ(r - db) + aed) + ev1 / sqrt(SQ(r + db) + aed);
  T e12 = ev1 / sqrt(r2 + aeq);
  T eqzz = ev2 / sqrt(SQ(r - qb) + aeq) + ev2 / sqrt(SQ(r + qb) + aeq) - e12;
  T eqxx = ev1 / sqrt(r2 + qb * qb + aeq) - e12;
  T e20 = ev2 / sqrt(SQ(r + da) + adq), e22 = ev2 / sqrt(SQ(r - da) + adq);
  T e24 = ev2 / sqrt(SQ(r - db) + aqd), e26 = ev2 / sqrt(SQ(r + db) + aqd);
  T e36 = ev2 / sqrt(r2 + aqq), e39 = ev2 / sqrt(r2 + qa * qa + aqq), e40 = ev2 / sqrt(r2 + qb * qb + aqq);
  T e42 = ev3 / sqrt(SQ(r - qb) + aqq), e44 = ev3 / sqrt(SQ(r + qb) + aqq);
  T e46 = ev3 / sqrt(SQ(r + qa) + aqq), e48 = ev3 / sqrt(SQ(r - qa) + aqq);
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
  T qxxqxx = ev3 / sqrt(r2 + SQ(qa - qb) + aqq) + ev3 / sqrt(r2 + SQ(qa + qb) + aqq) - e39 - e40 + e36;
  ri[18] = ee + eqxx + qxxe + qxxqxx;
  ri[19] = ev3 / sqrt(SQ(r + qa1 - qb1) + SQ(qa1 - qb1) + aqq) - ev3 / sqrt(SQ(r + qa1 + qb1) + SQ(qa1 - qb1) + aqq) -
           ev3 / sqrt(SQ(r - qa1 - qb1) + SQ(qa1 - qb1) + aqq) + ev3 / sqrt(SQ(r - qa1 + qb1) + SQ(qa1 - qb1) + aqq) -
           ev3 / sqrt(SQ(r + qa1 - qb1) + SQ(qa1 + qb1) + aqq) + ev3 / sqrt(SQ(r + qa1 + qb1) + SQ(qa1 + qb1) + aqq) +
           ev3 / sqrt(SQ(r - qa1 - qb1) + SQ(qa1 + qb1) + aqq) - ev3 / sqrt(SQ(r - qa1 + qb1) + SQ(qa1 + qb1) + aqq);
  T qxxqyy = ev2 / sqrt(r2 + qa * qa + qb * qb + aqq) - e39 - e40 + e36;
  ri[20] = ee + eqxx + qxxe + qxxqyy;
  ri[21] = 0.5 * (qxxqxx - qxxqyy);
}

// heavy-hydrogen: 4 integrals (sigma-type only)
template <class T>
__device__ void local_xh(T r, double da, double qa0, double r0a, double r0b, double r1a, double r2a, T *ri) {
  const double ev1 = EV / 2.0, ev2 = EV / 4.0;
  const double aee = (r0a + r0b) * (r0a + r0b), ade = (r1a + r0b) * (r1a + r0b), aqe = (r2a + r0b) * (r2a + r0b);
  const double qa = qa0 * 2.0;
  T e6 = ev1 / sqrt(r * r + aqe);
  T ee = EV / sqrt(r * r + aee);
  ri[0] = ee;
  ri[1] = ev1 / sqrt(SQ(r + da) + ade) - ev1 / sqrt(SQ(r - da) + ade);
  ri[2] = ee + ev2 / sqrt(SQ(r + qa) + aqe) + ev2 / sqrt(SQ(r - qa) + aqe) - e6;
  ri[3] = ee + ev1 / sqrt(r * r + qa * qa + aqe) - e6;
}

// ---------------------------------------------------------------- rotation
// rotation matrix taking unit vector v onto +x via the quaternion (0, v_z, -v_y, 1+v_x);
// |1+v_x| < 1e-7 uses a half turn about z (two_elec_two_center_int.py:1576-1631)
template <class T>
__device__ void quat_rot(T vx, T vy, T vz, T R[3][3]) {
  T qy = vz, qz = -vy, qw = 1.0 + vx;
  if (fabs(val(qw)) < 1.0e-7) { qy = T(0.0); qz = T(1.0); qw = T(0.0); }
  T nrm = sqrt(qy * qy + qz * qz + qw * qw);
  qy = qy / nrm; qz = qz / nrm; qw = qw / nrm;
  R[0][0] = 1.0 - 2.0 * (qy * qy + qz * qz);
  R[0][1] = -2.0 * (qz * qw);
  R[0][2] = 2.0 * (qy * qw);
  R[1][0] = 2.0 * (qz * qw);
  R[1][1] = 1.0 - 2.0 * (qz * qz);
  R[1][2] = 2.0 * (qy * qz);
  R[2][0] = -2.0 * (qy * qw);
  R[2][1] = 2.0 * (qy * qz);
  R[2][2] = 1.0 - 2.0 * (qy * qy);
}

// heavy-heavy rotated block: sink(a, b, value) for a = (kk,ll) of atom i, b = (mm,nn) of atom j
template <class T, class Sink>
__device__ void rotate_xx(const T *ri, const T R[3][3], Sink sink) {
  const T *r0 = R[0], *r1 = R[1], *r2 = R[2];
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
          T val;
          if (kk == 0) {
            if (mm == 0) val = ri[0];
            else if (nn == 0) val = ri[4] * r0[m];
            else val = ri[10] * (r0[m] * r0[n]) + ri[11] * (r1[m] * r1[n] + r2[m] * r2[n]);
          } else if (ll == 0) {
            if (mm == 0) val = ri[1] * r0[k];
            else if (nn == 0) val = ri[5] * (r0[k] * r0[m]) + ri[6] * (r1[k] * r1[m] + r2[k] * r2[m]);
            else {
              T t0 = r0[k] * r0[m] * r0[n];
              T t1 = (r1[m] * r1[n] + r2[m] * r2[n]) * r0[k];
              T mix = r1[k] * (r1[n] * r0[m] + r1[m] * r0[n]) + r2[k] * (r2[m] * r0[n] + r2[n] * r0[m]);
              val = ri[12] * t0 + ri[13] * t1 + ri[14] * mix;
            }
          } else {
            if (mm == 0) val = ri[2] * (r0[k] * r0[l]) + ri[3] * (r1[k] * r1[l] + r2[k] * r2[l]);
            else if (nn == 0) {
              T t0 = r0[k] * r0[l] * r0[m];
              T t1 = (r1[k] * r1[l] + r2[k] * r2[l]) * r0[m];
              T t2 = r1[l] * r1[m] + r2[l] * r2[m];
              val = ri[7] * t0 + ri[8] * t1 + ri[9] * (r0[k] * t2 + r0[l] * (r1[k] * r1[m] + r2[k] * r2[m]));
            } else {
              val = ri[15] * (r0[k] * r0[l] * r0[m] * r0[n]);
              val += ri[16] * ((r1[k] * r1[l] + r2[k] * r2[l]) * r0[m] * r0[n]);
              val += ri[17] * ((r1[m] * r1[n] + r2[m] * r2[n]) * (r0[k] * r0[l]));
              val += ri[18] * (r1[k] * r1[l] * r1[m] * r1[n] + r2[k] * r2[l] * r2[m] * r2[n]);
              T mix1 = r0[m] * (r1[l] * r1[n] + r2[l] * r2[n]);
              T mix2 = r0[n] * (r1[l] * r1[m] + r2[l] * r2[m]);
              T val5 = r0[k] * (mix1 + mix2) +
                       r0[l] * (r0[m] * (r1[k] * r1[n] + r2[k] * r2[n]) + r0[n] * (r1[k] * r1[m] + r2[k] * r2[m]));
              val += ri[19] * val5;
              val += ri[20] * (r1[k] * r1[l] * r2[m] * r2[n] + r2[k] * r2[l] * r1[m] * r1[n]);
              val += ri[21] * ((r1[k] * r2[l] + r2[k] * r1[l]) * (r1[m] * r2[n] + r2[m] * r1[n]));
            }
          }
          sink(a, b, val);
        }
      }
    }
  }
}

template <class T, class Sink>
__device__ void rotate_xh(const T *ri, const T R[3][3], Sink sink) {
  int a = 0;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
    for (int ll = 0; ll <= kk; ++ll, ++a) {
      const int k = kk - 1, l = ll - 1;
      T val;
      if (kk == 0) val = ri[0];
      else if (ll == 0) val = ri[1] * R[0][k];
      else val = ri[2] * R[0][k] * R[0][l] + ri[3] * (R[1][k] * R[1][l] + R[2][k] * R[2][l]);
      sink(a, val);
    }
  }
}

// ----------------------------------------------------------------- overlap
// auxiliary integrals A_k(x), k = 0..6 (diat_overlap_PM6_SP.py:464-519)
template <class T>
__device__ void aint(T x, T *a) {
  T xs = val(x) != 0.0 ? x : T(INFINITY);
  a[0] = exp(-xs) / xs;
  a[1] = a[0] + a[0] / xs;
#pragma unroll
  for (int k = 2; k < 7; ++k) a[k] = a[0] + (double)k * a[k - 1] / xs;
}

// auxiliary integrals B_k(x), k = 0..6 (diat_overlap_PM6_SP.py:522-670)
template <class T>
__device__ void bint(T x, T *b) {
  double ax = fabs(val(x));
  if (ax > 0.5) {
    T tx = exp(x) / x, tmx = -exp(-x) / x;
    b[0] = tx + tmx;
#pragma unroll
    for (int k = 1; k < 7; ++k) b[k] = ((k & 1) ? -tx : tx) + tmx + (double)k * b[k - 1] / x;
  } else if (ax > 1.0e-6) {
    T x2 = x * x, x3 = x2 * x, x4 = x2 * x2, x5 = x4 * x, x6 = x4 * x2;
    b[0] = 2.0 + x2 / 3.0 + x4 / 60.0 + x6 / 2520.0;
    b[2] = 2.0 / 3.0 + x2 / 5.0 + x4 / 84.0 + x6 / 3240.0;
    b[4] = 2.0 / 5.0 + x2 / 7.0 + x4 / 108.0 + x6 / 3960.0;
    b[6] = 2.0 / 7.0 + x2 / 9.0 + x4 / 132.0 + x6 / 4680.0;
    b[1] = -2.0 / 3.0 * x - x3 / 15.0 - x5 / 420.0;
    b[3] = -2.0 / 5.0 * x - x3 / 21.0 - x5 / 540.0;
    b[5] = -2.0 / 7.0 * x - x3 / 27.0 - x5 / 660.0;
  } else {
    b[0] = T(2.0); b[1] = T(0.0); b[2] = T(2.0 / 3.0); b[3] = T(0.0); b[4] = T(2.0 / 5.0); b[5] = T(0.0);
    b[6] = T(2.0 / 7.0);
  }
}

template <class T>
struct Sloc { T s111, s211, s121, s221, s222; };

// local-frame overlaps for the principal-quantum-number classes (diat_overlap_PM6_SP.py:56-312);
// returns false for an unsupported class (the reference raises ValueError)
template <class T>
__device__ bool overlap_local(int qni, int qnj, T r, double zsa, double zpa, double zsb, double zpb, Sloc<T> &S) {
  S.s111 = S.s211 = S.s121 = S.s221 = S.s222 = T(0.0);
  T A[7], B[7];
  const double s3 = ::sqrt(3.0), s10 = ::sqrt(10.0), s30 = ::sqrt(30.0);
  auto set = [&](double za, double zb) { aint(0.5 * r * (za + zb), A); bint(0.5 * r * (za - zb), B); };
  if (qni == 1 && qnj == 1) {
    set(zsa, zsb);
    S.s111 = pow(zsa * zsb * r * r, 1.5) * (A[2] * B[0] - B[2] * A[0]) / 4.0;
  } else if (qni == 2 && qnj == 1) {
    T r4 = r * r * r * r;
    set(zsa, zsb);
    S.s111 = ::pow(zsb, 1.5) * ::pow(zsa, 2.5) * r4 * (A[3] * B[0] - B[3] * A[0] + A[2] * B[1] - B[2] * A[1]) /
             (s3 * 8.0);
    set(zpa, zsb);
    S.s211 = ::pow(zsb, 1.5) * ::pow(zpa, 2.5) * r4 * (A[2] * B[0] - B[2] * A[0] + A[3] * B[1] - B[3] * A[1]) / 8.0;
  } else if (qni == 2 && qnj == 2) {
    T r5 = r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = ::pow(zsb * zsa, 2.5) * r5 * (A[4] * B[0] + B[4] * A[0] - 2.0 * A[2] * B[2]) / 48.0;
    set(zpa, zsb);
    S.s211 = ::pow(zsb * zpa, 2.5) * r5 *
             (A[3] * (B[0] - B[2]) - A[1] * (B[2] - B[4]) + B[3] * (A[0] - A[2]) - B[1] * (A[2] - A[4])) / (16.0 * s3);
    set(zsa, zpb);
    S.s121 = ::pow(zpb * zsa, 2.5) * r5 *
             (A[3] * (B[0] - B[2]) - A[1] * (B[2] - B[4]) - B[3] * (A[0] - A[2]) + B[1] * (A[2] - A[4])) / (16.0 * s3);
    set(zpa, zpb);
    T w = ::pow(zpb * zpa, 2.5) * r5 / 16.0;
    S.s221 = -w * (B[2] * (A[4] + A[0]) - A[2] * (B[4] + B[0]));
    S.s222 = 0.5 * w * (A[4] * (B[0] - B[2]) - B[4] * (A[0] - A[2]) - A[2] * B[0] + B[2] * A[0]);
  } else if (qni == 3 && qnj == 1) {
    T r5 = r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = ::pow(zsb, 1.5) * ::pow(zsa, 3.5) * r5 * (A[4] * B[0] + 2.0 * B[1] * A[3] - 2.0 * A[1] * B[3] - B[4] * A[0]) /
             (s10 * 24.0);
    set(zpa, zsb);
    S.s211 = ::pow(zsb, 1.5) * ::pow(zpa, 3.5) * r5 *
             (A[3] * (B[0] + B[2]) - A[1] * (B[4] + B[2]) + B[1] * (A[2] + A[4]) - B[3] * (A[2] + A[0])) / (8.0 * s30);
  } else if (qni == 3 && qnj == 2) {
    T r6 = r * r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = ::pow(zsb, 2.5) * ::pow(zsa, 3.5) * r6 *
             (A[5] * B[0] + B[1] * A[4] - 2.0 * B[2] * A[3] - 2.0 * A[2] * B[3] + B[4] * A[1] + B[5] * A[0]) /
             (s30 * 48.0);
    set(zpa, zsb);
    S.s211 = ::pow(zsb, 2.5) * ::pow(zpa, 3.5) * r6 *
             (A[4] * B[0] + B[1] * A[5] - 2.0 * B[3] * A[3] - 2.0 * A[2] * B[2] + A[1] * B[5] + A[0] * B[4]) /
             (48.0 * s10);
    set(zsa, zpb);
    S.s121 = ::pow(zpb, 2.5) * ::pow(zsa, 3.5) * r6 *
             ((A[4] * B[0] - A[5] * B[1]) + 2.0 * (A[3] * B[1] - A[4] * B[2]) - 2.0 * (A[1] * B[3] - A[2] * B[4]) -
              (A[0] * B[4] - A[1] * B[5])) / (48.0 * s10);
    set(zpa, zpb);
    S.s221 = ::pow(zpb, 2.5) * ::pow(zpa, 3.5) * r6 *
             ((A[3] * B[0] - A[5] * B[2]) + (A[2] * B[1] - A[4] * B[3]) - (A[1] * B[2] - A[3] * B[4]) -
              (A[0] * B[3] - A[2] * B[5])) / (16.0 * s30);
    S.s222 = ::pow(zpb, 2.5) * ::pow(zpa, 3.5) * r6 *
             ((A[5] - A[3]) * (B[0] - B[2]) + (A[4] - A[2]) * (B[1] - B[3]) - (A[3] - A[1]) * (B[2] - B[4]) -
              (A[2] - A[0]) * (B[3] - B[5])) / (32.0 * s30);
  } else if (qni == 3 && qnj == 3) {
    T r7 = r * r * r * r * r * r * r;
    set(zsa, zsb);
    S.s111 = ::pow(zsb * zsa, 3.5) * r7 * (A[6] * B[0] - 3.0 * B[2] * A[4] + 3.0 * A[2] * B[4] - A[0] * B[6]) / 1440.0;
    set(zpa, zsb);
    S.s211 = ::pow(zsb * zpa, 3.5) * r7 *
             ((A[5] * B[0] + A[6] * B[1]) + (-A[4] * B[1] - A[5] * B[2]) - 2.0 * (A[3] * B[2] + A[4] * B[3]) -
              2.0 * (-A[2] * B[3] - A[3] * B[4]) + (A[1] * B[4] + A[2] * B[5]) + (-A[0] * B[5] - A[1] * B[6])) /
             (480.0 * s3);
    set(zsa, zpb);
    S.s121 = ::pow(zpb * zsa, 3.5) * r7 *
             ((A[5] * B[0] - A[6] * B[1]) + (A[4] * B[1] - A[5] * B[2]) - 2.0 * (A[3] * B[2] - A[4] * B[3]) -
              2.0 * (A[2] * B[3] - A[3] * B[4]) + (A[1] * B[4] - A[2] * B[5]) + (A[0] * B[5] - A[1] * B[6])) /
             (480.0 * s3);
    set(zpa, zpb);
    S.s221 = ::pow(zpb, 3.5) * ::pow(zpa, 3.5) * r7 *
             ((A[4] * B[0] - A[6] * B[2]) - 2.0 * (A[2] * B[2] - A[4] * B[4]) + (A[0] * B[4] - A[2] * B[6])) / 480.0;
    S.s222 = ::pow(zpb, 3.5) * ::pow(zpa, 3.5) * r7 *
             ((A[6] - A[4]) * (B[0] - B[2]) - 2.0 * (A[4] - A[2]) * (B[2] - B[4]) + (A[2] - A[0]) * (B[4] - B[6])) /
             960.0;
  } else {
    return false;
  }
  return true;
}
#undef SQ

// 4x4 molecular-frame overlap of pair (i, j) with unit vector x = (Rj-Ri)/|Rj-Ri|
// (diat_overlap_PM6_SP.py:376-392); returns false for unsupported classes
template <class T>
__device__ bool overlap_block(int qni, int qnj, T r, T xv, T yv, T zv, double zsa, double zpa, double zsb, double zpb,
                              T di[4][4]) {
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) di[a][c] = T(0.0);
  if (val(r) > OVERLAP_CUTOFF) return true;
  Sloc<T> S;
  if (!overlap_local(qni, qnj, r, zsa, zpa, zsb, zpb, S)) return false;
  T Q[3][3];
  quat_rot(xv, yv, zv, Q);
  di[0][0] = S.s111;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    di[1 + a][0] = S.s211 * Q[0][a];
    di[0][1 + a] = -S.s121 * Q[0][a];
  }
  const T Mv[3] = {-S.s221, S.s222, S.s222};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      di[1 + a][1 + c] = Q[0][a] * Mv[0] * Q[0][c] + Q[1][a] * Mv[1] * Q[1][c] + Q[2][a] * Mv[2] * Q[2][c];
  return true;
}

// sum of the Gaussian core-core corrections of atoms i and j times Z_i Z_j / R (energy.py:128-131)
template <class T>
__device__ T core_gauss(const seqm_batch &b, int ia, int ja, T rija, int ng, double ti, double tj) {
  T t4 = ti * tj / rija, t5 = T(0.0), t6 = T(0.0);
  for (int g = 0; g < ng; ++g) {
    const double Ki = par(b, SEQM_P_K1 + g, ia), Li = par(b, SEQM_P_L1 + g, ia), Mi = par(b, SEQM_P_M1 + g, ia);
    const double Kj = par(b, SEQM_P_K1 + g, ja), Lj = par(b, SEQM_P_L1 + g, ja), Mj = par(b, SEQM_P_M1 + g, ja);
    t5 += Ki * exp(-Li * ((rija - Mi) * (rija - Mi)));
    t6 += Kj * exp(-Lj * ((rija - Mj) * (rija - Mj)));
  }
  return t4 * (t5 + t6);
}

// PM6 core-core repulsion of one pair (energy.py:135-171): the unpolarisable-core term
// 1e-8 ((Z_i^1/3 + Z_j^1/3) / R)^12, the diatomic factor 1 + 2 chi exp(-alp (R + 3e-4 R^6))
// (exp(-alp R^2) for C-H, N-H, O-H) on Z_i Z_j gamma_core, where gamma_core takes each atom's
// rho_core in place of rho0 when nonzero, the C-C and Si-O corrections and the Gaussians.
// R in Angstrom, r in bohr (the Si-O term takes r, as the reference does).
template <class T>
__device__ T core_core_pm6(const seqm_batch &b, int ia, int ja, T r) {
  const int Zi = b.atom_Z[ia], Zj = b.atom_Z[ja];
  const double ti = par(b, SEQM_P_TORE, ia), tj = par(b, SEQM_P_TORE, ja);
  double alp = 0.0, chi = 0.0, cz = 0.0;
  if (b.pair_par && Zi >= 0 && Zj >= 0 && Zi <= b.pair_zmax && Zj <= b.pair_zmax) {
    const double *q = b.pair_par + 3 * ((size_t)Zi * (b.pair_zmax + 1) + Zj);
    alp = q[0];
    chi = q[1];
    cz = q[2];
  }
  const double rci = par(b, SEQM_P_RHOCORE, ia), rcj = par(b, SEQM_P_RHOCORE, ja);
  const double r0 = (rci != 0.0 ? rci : par(b, SEQM_P_RHO0, ia)) + (rcj != 0.0 ? rcj : par(b, SEQM_P_RHO0, ja));
  T rija = r * A0;
  T u = cz / rija;
  T u3 = u * u * u;
  T unpol = 1.0e-8 * (u3 * u3) * (u3 * u3);
  T gcore = (ti * tj * EV) / sqrt(r * r + r0 * r0);
  const bool xh = (Zi == 6 || Zi == 7 || Zi == 8) && Zj == 1;
  T arg;
  if (xh) {
    arg = rija * rija;
  } else {
    T r2 = rija * rija;
    arg = rija + 0.0003 * (r2 * r2 * r2);
  }
  T e = unpol + gcore * (1.0 + (2.0 * chi) * exp(-alp * arg));
  if (Zi == 6 && Zj == 6) e = e + gcore * (9.28 * exp(-5.98 * rija));
  if (Zi == 14 && Zj == 8) e = e - gcore * (0.0007 * exp(-((r - 2.9) * (r - 2.9))));
  return e + core_gauss<T>(b, ia, ja, rija, 4, ti, tj);
}

// core-core repulsion of one pair (energy.py:91-171); gam = (s_A s_A | s_B s_B)
template <class T>
__device__ T core_core(const seqm_batch &b, int ia, int ja, T r, T gam) {
  if (b.method == SEQM_PM6_SP) return core_core_pm6<T>(b, ia, ja, r);
  const int Zi = b.atom_Z[ia], Zj = b.atom_Z[ja];
  T rija = r * A0;
  const double ti = par(b, SEQM_P_TORE, ia), tj = par(b, SEQM_P_TORE, ja);
  T t1 = ti * tj * gam;
  T tmp = exp(-par(b, SEQM_P_ALPHA, ia) * rija);
  T t2 = ((Zi == 7 || Zi == 8) && Zj == 1) ? tmp * rija : tmp;
  T t3 = exp(-par(b, SEQM_P_ALPHA, ja) * rija);
  T e = t1 * (1.0 + t2 + t3);
  const int ng = b.method == SEQM_AM1 ? 4 : (b.method == SEQM_PM3 ? 2 : 0);
  if (ng) e = e + core_gauss<T>(b, ia, ja, rija, ng, ti, tj);
  return e;
}

}  // namespace seqm
