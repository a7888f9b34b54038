// g3_fatbra.cuh -- the composite-bra / pair-ket form of the four-particle
// geminal Coulomb integrals G4_MD_xgVepg and G4_MD_xgVeeg (XC1_G4_MD.f:
// 796-1125, 1559-1978) used by the gam_3 builder (k_gam3.cu, whose header
// comment gives the derivation).  Every function is __host__ __device__ so
// the tests can compare it, compiled as plain C++, with the element-wise
// md_math.cuh integrals.  R = double (FP64 path) or float (mixed path); the
// Boys function, the seeds (-alpha)^m F_m(T) and their sum are FP64 in both.
#pragma once
#include <math.h>

#include "md_math.cuh"

#if defined(__CUDACC__)
#define G3_HD __host__ __device__ __forceinline__
#else
#define G3_HD inline
#endif

namespace neoxc {
namespace g3 {

// C(t,i) 2^(2i-t) in the precision of the contraction
template <class R>
G3_HD R hermc_r(int t, int i) {
  if constexpr (sizeof(R) == sizeof(float)) return hermc32(t, i);
  else return (R)hermc(t, i);
}

// ---- pair records (FP64, 32 doubles each) ----------------------------------
// [0] p  [1..3] P  [4] c_a c_b  [5..19] E[d][t] (t <= 4)  [20..22] t_max[d]
// [23] S  [24] Q (screening magnitudes, see k_gam3.cu)
enum { kRP = 0, kRX = 1, kRC = 4, kRE = 5, kRT = 20, kRS = 23, kRQ = 24, kRLen = 32 };

G3_HD int pair_index(int i, int j) {
  return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
}

// Record of one primitive pair (A, B) with contraction coefficients ca, cb.
G3_HD void fill_pair_record(const md::Prim& A, const md::Prim& B, double ca, double cb,
                            double* out) {
  md::Pair pr;
  md::gauss_pair(A, B, pr);
  out[kRP] = pr.p;
  for (int d = 0; d < 3; d++) out[kRX + d] = pr.P[d];
  out[kRC] = ca * cb;
  double ang = 1.0;
  const double sig = 1.0 / sqrt(pr.p);
  for (int d = 0; d < 3; d++) {
    double tmp[2 * md::TMX + 1];
    const int tl = A.l[d] + B.l[d];
    md::hermite_e(A.l[d], B.l[d], pr.K[d], A.a, B.a, pr.p, pr.q, pr.Q[d], tmp);
    for (int k = 0; k < 5; k++) out[kRE + 5 * d + k] = k <= tl ? tmp[k] : 0.0;
    out[kRT + d] = (double)tl;
    for (int k = 0; k < A.l[d]; k++) ang *= fabs(pr.P[d] - A.c[d]) + sig;
    for (int k = 0; k < B.l[d]; k++) ang *= fabs(pr.P[d] - B.c[d]) + sig;
  }
  const double cab = fabs(ca * cb);
  const double pi = 3.14159265358979323846;
  out[kRS] = cab * pow(pi / pr.p, 1.5) * pr.K[0] * pr.K[1] * pr.K[2] * ang;
  out[kRQ] = cab * sqrt(fabs(md::gfvee(A, A, B, B)));
  for (int k = 25; k < kRLen; k++) out[k] = 0.0;
}

// ---- composite bra -----------------------------------------------------------
template <class R, int NW>
struct Bra {
  R W[3][NW + 1];   // W'_d
  R Z;              // composite exponent (Tx4 for Vep, W1 for Vee)
  R C[3];           // composite centre
  R pref;           // C0 * CB0
  double wgt;       // sign x b_k b_l x contraction coefficients of the bra's pairs
  double est;       // screening estimate of the bra's factors
  int N[3];
};

// derivatives of prod_k exp(-xi_k (c_k . x)^2), x = (x0, x1, x2), at X;
// extents X0, X1, X2 (D[(n0*X1 + n1)*X2 + n2]); the recurrence of dgauss3.
template <class R, int X0, int X1, int X2>
G3_HD void dgauss3t(int nk, const R* xi, const R (*c)[3], const R* X,
                    const int* N, R* D) {
  R grad[3] = {0, 0, 0}, H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  R expo = R(0);
  for (int k = 0; k < nk; k++) {
    const R u = c[k][0] * X[0] + c[k][1] * X[1] + c[k][2] * X[2];
    expo -= xi[k] * u * u;
    for (int i = 0; i < 3; i++) {
      grad[i] += R(2) * xi[k] * u * c[k][i];
      for (int j = 0; j < 3; j++) H[i][j] += R(2) * xi[k] * c[k][i] * c[k][j];
    }
  }
  const R base = exp(expo);
#define DD(a, b, e) D[((a) * X1 + (b)) * X2 + (e)]
  for (int n0 = 0; n0 <= N[0]; n0++)
    for (int n1 = 0; n1 <= N[1]; n1++)
      for (int n2 = 0; n2 <= N[2]; n2++) {
        if (n0 + n1 + n2 == 0) { DD(0, 0, 0) = base; continue; }
        int m[3] = {n0, n1, n2};
        const int i = n0 > 0 ? 0 : (n1 > 0 ? 1 : 2);
        m[i] -= 1;
        R v = -grad[i] * DD(m[0], m[1], m[2]);
        for (int j = 0; j < 3; j++)
          if (m[j] > 0) {
            int r[3] = {m[0], m[1], m[2]};
            r[j] -= 1;
            v -= H[i][j] * (R)m[j] * DD(r[0], r[1], r[2]);
          }
        DD(n0, n1, n2) = v;
      }
#undef DD
}

G3_HD double binom_d(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; i++) r = r * (double)(n - k + i) / (double)i;
  return r;
}

// W'_d[x0+x1+x2] = sum E0[t0] E1[t1] E2[t2] sum_x C(t,x) cof^x D(t - x):
// slots 0, 1 electrons (extent 2LE+1), slot 2 the proton (2LN+1).
template <class R, int LE, int LN, int NW>
G3_HD void fold_bra(const double* r0, const double* r1, const double* r2, int nk,
                    const R* xi, const R (*c)[3], const R* cof, Bra<R, NW>& b) {
  constexpr int X0 = 2 * LE + 1, X2 = 2 * LN + 1;
  R D[X0 * X0 * X2];
  R pw[3][5];
  for (int i = 0; i < 3; i++) {
    pw[i][0] = R(1);
    for (int k = 1; k < 5; k++) pw[i][k] = pw[i][k - 1] * cof[i];
  }
  const double* rr[3] = {r0, r1, r2};
  for (int d = 0; d < 3; d++) {
    int tl[3];
    R X[3];
    for (int i = 0; i < 3; i++) {
      tl[i] = (int)rr[i][kRT + d];
      X[i] = (R)rr[i][kRX + d];
    }
    dgauss3t<R, X0, X0, X2>(nk, xi, c, X, tl, D);
    for (int n = 0; n <= NW; n++) b.W[d][n] = R(0);
    for (int t0 = 0; t0 <= tl[0]; t0++)
      for (int t1 = 0; t1 <= tl[1]; t1++)
        for (int t2 = 0; t2 <= tl[2]; t2++) {
          const R e = (R)r0[kRE + 5 * d + t0] * (R)r1[kRE + 5 * d + t1] *
                      (R)r2[kRE + 5 * d + t2];
          for (int x0 = 0; x0 <= t0; x0++)
            for (int x1 = 0; x1 <= t1; x1++)
              for (int x2 = 0; x2 <= t2; x2++) {
                const R cc = (R)(binom_d(t0, x0) * binom_d(t1, x1) * binom_d(t2, x2)) *
                             pw[0][x0] * pw[1][x1] * pw[2][x2] *
                             D[((t0 - x0) * X0 + (t1 - x1)) * X2 + (t2 - x2)];
                b.W[d][x0 + x1 + x2] += e * cc;
              }
        }
    b.N[d] = tl[0] + tl[1] + tl[2];
  }
}

// G4_MD_xgVepg's composite (XC1_G4_MD.f:1559-1978): e1 (r1), e2 (r2), proton
// (rp); geminals gam14 = gk (e1-p), gam24 = gl (e2-p); Coulomb partner e3.
template <class R, int LE, int LN, int NW>
G3_HD void build_bra_vep(const double* r1, const double* r2, const double* rp,
                         R gk, R gl, Bra<R, NW>& b) {
  const R kPiT = R(3.14159265358979e+00);
  const R P1 = (R)r1[kRP], P2 = (R)r2[kRP], P4 = (R)rp[kRP];
  const R C0 = (kPiT / (P1 + gk)) * sqrt(kPiT / (P1 + gk));
  const R C1 = (P1 * gk) / (P1 + gk);
  const R S4 = C1 + P4;
  const R CB0 = (kPiT / (P2 + gl)) * sqrt(kPiT / (P2 + gl));
  const R CB1 = (P2 * gl) / (P2 + gl);
  const R Tx4 = S4 + CB1;
  const R xcof = (S4 + CB1) * (C1 + P4);
  const R cof[3] = {S4 * C1 / xcof, CB1 / (S4 + CB1), S4 * P4 / xcof};
  for (int d = 0; d < 3; d++) {
    const R sm4 = (C1 * (R)r1[kRX + d] + P4 * (R)rp[kRX + d]) / (C1 + P4);
    b.C[d] = (S4 * sm4 + CB1 * (R)r2[kRX + d]) / (S4 + CB1);
  }
  const R xi[3] = {(P4 * C1) / (P4 + C1), (S4 * CB1) / (S4 + CB1), R(0)};
  const R c[3][3] = {{R(1), R(0), R(-1)},
                     {C1 / (C1 + P4), R(-1), P4 / (C1 + P4)},
                     {R(0), R(0), R(0)}};
  fold_bra<R, LE, LN, NW>(r1, r2, rp, 2, xi, c, cof, b);
  b.Z = Tx4;
  b.pref = C0 * CB0;
}

// G4_MD_xgVeeg's composite (XC1_G4_MD.f:796-1125): e1 (r1), e3 (r3), proton
// (rp); geminals gam14 = gk (e1-p), gam34 = gl (e3-p); Coulomb partner e2.
template <class R, int LE, int LN, int NW>
G3_HD void build_bra_vee(const double* r1, const double* r3, const double* rp,
                         R gk, R gl, Bra<R, NW>& b) {
  const R kPiT = R(3.14159265358979e+00);
  const R P1 = (R)r1[kRP], P3 = (R)r3[kRP], P4 = (R)rp[kRP];
  const R xsum = P4 + gk + gl;
  const R C0 = (kPiT / xsum) * sqrt(kPiT / xsum);
  const R C1 = (P4 * gk) / xsum, C3 = (P4 * gl) / xsum;
  const R C13 = (gk * gl) / xsum;
  const R S1 = P1 + C1, S3 = P3 + C3;
  const R CB0 = (kPiT / (S3 + C13)) * sqrt(kPiT / (S3 + C13));
  const R CB1 = (S3 * C13) / (S3 + C13);
  const R W1 = S1 + CB1;
  const R cof[3] = {P1 / (S1 + CB1), (CB1 / (S1 + CB1)) * (P3 / (P3 + C3)),
                    (C1 / (S1 + CB1)) + (CB1 / (S1 + CB1)) * (C3 / (P3 + C3))};
  for (int d = 0; d < 3; d++)
    b.C[d] = cof[0] * (R)r1[kRX + d] + cof[1] * (R)r3[kRX + d] + cof[2] * (R)rp[kRX + d];
  const R xi[3] = {P1 * C1 / (P1 + C1), P3 * C3 / (P3 + C3), S1 * CB1 / (S1 + CB1)};
  const R c[3][3] = {{R(1), R(0), R(-1)},
                     {R(0), R(1), R(-1)},
                     {P1 / (P1 + C1), -P3 / (P3 + C3), C1 / (P1 + C1) - C3 / (P3 + C3)}};
  fold_bra<R, LE, LN, NW>(r1, r3, rp, 3, xi, c, cof, b);
  b.Z = W1;
  b.pref = C0 * CB0;
}

// One (bra, ket) Coulomb integral, pref C4 sum_tuv W_x W_y W_z R_tuv, with
// W_d = W'_d (*) Ek_d (Ek: the ket's Hermite coefficients times (-1)^t) and
// the Hermite-Coulomb sum in factorised form:
//   sum_m (-alpha)^m F_m(T) sum_{i+j+k=m} A_x[i] A_y[j] A_z[k],
//   A_d[i] = sum_t W_d[t] C(t,i) 2^(2i-t) R_d^(2i-t).
template <class R, int NW, int NK>
G3_HD double fb_eval(const Bra<R, NW>& b, R pk, const R* Xk, const R (*Ek)[NK + 1],
                     const int* tk) {
  constexpr int NT = NW + NK;
  const R zk = b.Z + pk;
  const R alpha = (b.Z * pk) / zk;
  R Rv[3], R2 = R(0);
  for (int d = 0; d < 3; d++) {
    Rv[d] = b.C[d] - Xk[d];
    R2 += Rv[d] * Rv[d];
  }
  const R T = alpha * R2;
  const R kPiT = R(3.14159265358979e+00);
  const R C4 = (R(2) * kPiT * kPiT * sqrt(kPiT)) / (b.Z * pk * sqrt(zk));
  R A[3][NT + 1];
  int L = 0;
  for (int d = 0; d < 3; d++) {
    const int nb = b.N[d], nkd = tk[d], n = nb + nkd;
    R W[NT + 1];
    for (int m = 0; m <= n; m++) {
      R acc = R(0);
      const int lo = m - nb > 0 ? m - nb : 0, hi = m < nkd ? m : nkd;
      for (int t = lo; t <= hi; t++) acc += b.W[d][m - t] * Ek[d][t];
      W[m] = acc;
    }
    R xp[NT + 1];
    xp[0] = R(1);
    for (int k = 1; k <= n; k++) xp[k] = xp[k - 1] * Rv[d];
    for (int i = 0; i <= n; i++) A[d][i] = R(0);
    for (int t = 0; t <= n; t++)
      for (int i = (t + 1) / 2; i <= t; i++) A[d][i] += W[t] * hermc_r<R>(t, i) * xp[2 * i - t];
    L += n;
  }
  const int nx = b.N[0] + tk[0], ny = b.N[1] + tk[1], nz = b.N[2] + tk[2];
  R Bxy[2 * NT + 1];
  for (int m = 0; m <= nx + ny; m++) Bxy[m] = R(0);
  for (int i = 0; i <= nx; i++)
    for (int j = 0; j <= ny; j++) Bxy[i + j] += A[0][i] * A[1][j];
  // seeds (-alpha)^m F_m(T) and the final sum in FP64
  const double s = boys_sum(L, T, (double)alpha, [&](int m) {
    R bm = R(0);
    const int lo = m - nz > 0 ? m - nz : 0, hi = m < nx + ny ? m : nx + ny;
    for (int i = lo; i <= hi; i++) bm += Bxy[i] * A[2][m - i];
    return bm;
  });
  return (double)(b.pref * C4) * s;
}

}  // namespace g3
}  // namespace neoxc
