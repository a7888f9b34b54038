/*
 * prim.c -- ORACLE (test infrastructure only; never linked by the product).
 *
 * CPU restatement of the NEO-RXCHF L1/L2 arithmetic: Boys function,
 * underflow flush, Gaussian products, Hermite expansion coefficients,
 * Hermite Coulomb R_tuv, derivative-of-Gaussian products, and the
 * McMurchie-Davidson geminal primitive integrals.  Loop nests, summation
 * order and constants follow the cited reference routines; build with
 * -ffp-contract=off (the reference is built with -fp-model strict).
 * Loop-invariant sub-expressions the reference recomputes inside its
 * Hermite loops are evaluated once here: the same operations on the same
 * operands, so the values are unchanged.
 */
#include "neoxc_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* pi as truncated in the MD kernels: XC1_G3_MD.f:355 parameter(pi=...) */
#define PI_T 3.14159265358979e+00

/* Fortran x**n with an integer exponent (repeated product; n>=0). */
static double ipow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; i++) r = r * x;
  return r;
}

/* AC_Integrals/common.f:317-348 XGAMMAF */
void orc_xgammaf(double *F, double T, int M) {
  const double TMAX = 20.0, ACCY = 1.0e-12, SQRPI = 0.88622692545275801365;
  double PT5PM = 0.5 + M;
  if (T > TMAX) {
    F[0] = SQRPI / sqrt(T);
    for (int L = 1; L <= M; L++) F[L] = F[L - 1] * (1.0 * L - 0.5) / T;
  } else {
    double TI2 = T * 2.0, EXPTI = exp(-T);
    double TERM = 0.5 / PT5PM, SUMK = TERM;
    for (int K = 1; K <= 1000; K++) {
      TERM = TERM * T / (PT5PM + K);
      SUMK = SUMK + TERM;
      if (TERM < ACCY) break;
    }
    F[M] = EXPTI * SUMK;
    for (int L = M - 1; L >= 0; L--)
      F[L] = (F[L + 1] * TI2 + EXPTI) / (2.0 * L + 1.0);
  }
}

/* common.f:351-365 iboys2 (iboys short-circuits here, common.f:486-490) */
double orc_iboys2(int m, double x) {
  double F[64];
  orc_xgammaf(F, x, m);
  return F[m];
}

/* AC_Integrals/underflow.f:2-11 */
double orc_underflow(double x) { return fabs(x) < 1.0e-100 ? 0.0 : x; }

/* CS_Integrals/XC1_int_tools.f:341-464 RTUV */
double orc_rtuv(int tL, int uL, int vL, int nL, double expt, double alpha,
                double XPC, double YPC, double ZPC) {
  const int dt = tL + 2, du = uL + 2, dv = vL + 2, dn = nL + 2;
  double *R = (double *)calloc((size_t)dt * du * dv * dn, sizeof(double));
#define R_(t, u, v, n) R[(t) + dt * ((u) + du * ((v) + dv * (n)))]
  for (int n = 0; n <= nL; n++)
    R_(0, 0, 0, n) = pow(-2.0 * alpha, (double)n) * orc_iboys2(n, expt);
  for (int n = 0; n <= nL; n++) R_(1, 0, 0, n) = XPC * R_(0, 0, 0, n + 1);
  for (int t = 2; t <= tL; t++)
    for (int n = 0; n <= nL; n++)
      R_(t, 0, 0, n) =
          (double)(t - 1) * R_(t - 2, 0, 0, n + 1) + XPC * R_(t - 1, 0, 0, n + 1);
  for (int t = 0; t <= tL; t++)
    for (int n = 0; n <= nL; n++) R_(t, 1, 0, n) = YPC * R_(t, 0, 0, n + 1);
  for (int u = 2; u <= uL; u++)
    for (int t = 0; t <= tL; t++)
      for (int n = 0; n <= nL; n++)
        R_(t, u, 0, n) = (double)(u - 1) * R_(t, u - 2, 0, n + 1) +
                         YPC * R_(t, u - 1, 0, n + 1);
  for (int t = 0; t <= tL; t++)
    for (int u = 0; u <= uL; u++)
      for (int n = 0; n <= nL; n++) R_(t, u, 1, n) = ZPC * R_(t, u, 0, n + 1);
  for (int v = 2; v <= vL; v++)
    for (int t = 0; t <= tL; t++)
      for (int u = 0; u <= uL; u++)
        for (int n = 0; n <= nL; n++)
          R_(t, u, v, n) = (double)(v - 1) * R_(t, u, v - 2, n + 1) +
                           ZPC * R_(t, u, v - 1, n + 1);
  double out = R_(tL, uL, vL, 0);
#undef R_
  free(R);
  return out;
}

/* AC_Integrals/common.f:214-313 auxR2 */
double orc_auxR2(int NMAX, int LMAX, int MMAX, double alp, double a,
                 double b, double c) {
  const int JMAX = NMAX + MMAX + LMAX, JD = JMAX + 1;
  double T = alp * ((a * a) + (b * b) + (c * c));
  double *Rm = (double *)calloc((size_t)(MMAX + 1) * JD, sizeof(double));
  double *Rl = (double *)calloc((size_t)(LMAX + 1) * JD, sizeof(double));
  double *Rn = (double *)calloc((size_t)(NMAX + 1) * JD, sizeof(double));
  /* 1-based (im, j) -> [(im-1) + (MMAX+1)*(j-1)] */
#define RM(i, j) Rm[((i) - 1) + (MMAX + 1) * ((j) - 1)]
#define RL(i, j) Rl[((i) - 1) + (LMAX + 1) * ((j) - 1)]
#define RN(i, j) Rn[((i) - 1) + (NMAX + 1) * ((j) - 1)]
  for (int im = 1; im <= MMAX + 1; im++) {
    int m = im - 1;
    if (im >= 3) {
      for (int j = 1; j <= JMAX; j++)
        RM(im, j) = (c * RM(im - 1, j + 1)) + ((double)(m - 1) * RM(im - 2, j + 1));
    } else if (im == 2) {
      for (int j = 1; j <= JMAX; j++) RM(im, j) = c * RM(im - 1, j + 1);
    } else {
      for (int jp = 1; jp <= JMAX + 1; jp++) {
        int j = jp - 1;
        RM(im, jp) = ipow(-2.0 * alp, j) * orc_iboys2(j, T);
      }
    }
  }
  for (int il = 1; il <= LMAX + 1; il++) {
    int l = il - 1;
    if (il >= 3) {
      for (int j = 1; j <= JMAX; j++)
        RL(il, j) = (b * RL(il - 1, j + 1)) + ((double)(l - 1) * RL(il - 2, j + 1));
    } else if (il == 2) {
      for (int j = 1; j <= JMAX; j++) RL(il, j) = b * RL(il - 1, j + 1);
    } else {
      for (int jp = 1; jp <= JMAX + 1; jp++) RL(il, jp) = RM(MMAX + 1, jp);
    }
  }
  for (int in = 1; in <= NMAX + 1; in++) {
    int n = in - 1;
    if (in >= 3) {
      for (int j = 1; j <= JMAX; j++)
        RN(in, j) = (a * RN(in - 1, j + 1)) + ((double)(n - 1) * RN(in - 2, j + 1));
    } else if (in == 2) {
      for (int j = 1; j <= JMAX; j++) RN(in, j) = a * RN(in - 1, j + 1);
    } else {
      for (int jp = 1; jp <= JMAX + 1; jp++) RN(in, jp) = RL(LMAX + 1, jp);
    }
  }
  double out = RN(NMAX + 1, 1);
#undef RM
#undef RL
#undef RN
  free(Rm); free(Rl); free(Rn);
  return out;
}

/* XC1_int_tools.f:136-227 ghec (common.f:37-110 hecod computes the same
 * recursion with the identically-zero top terms omitted). */
void orc_ghec(int iLim, int jLim, double KAB, double a, double b, double p,
              double q, double Qx, double *EOUT) {
  const int di = iLim + 1, dj = jLim + 1, dt = iLim + jLim + 2;
  double E[8 * 8 * 18];
  double *Ep = E;
  double *heap = NULL;
  if (di * dj * dt > (int)(sizeof(E) / sizeof(E[0])))
    Ep = heap = (double *)malloc(sizeof(double) * di * dj * dt);
#define E_(i, j, t) Ep[(i) + di * ((j) + dj * (t))]
  for (int k = 0; k < di * dj * dt; k++) Ep[k] = 0.0;
  double x1 = 1.0 / (2.0 * p);
  double x2 = -q * Qx / a;
  E_(0, 0, 0) = KAB;
  for (int i = 1; i <= iLim; i++) {
    E_(i, 0, 0) = x2 * E_(i - 1, 0, 0) + E_(i - 1, 0, 1);
    for (int t = 1; t <= i; t++) {
      double x3 = (double)(t + 1);
      E_(i, 0, t) = x1 * E_(i - 1, 0, t - 1) + x2 * E_(i - 1, 0, t) +
                    x3 * E_(i - 1, 0, t + 1);
    }
  }
  x2 = q * Qx / b;
  for (int j = 1; j <= jLim; j++)
    for (int i = 0; i <= iLim; i++) {
      E_(i, j, 0) = x2 * E_(i, j - 1, 0) + E_(i, j - 1, 1);
      for (int t = 1; t <= i + j; t++) {
        double x3 = (double)(t + 1);
        E_(i, j, t) = x1 * E_(i, j - 1, t - 1) + x2 * E_(i, j - 1, t) +
                      x3 * E_(i, j - 1, t + 1);
      }
    }
  for (int t = 0; t <= iLim + jLim; t++) EOUT[t] = E_(iLim, jLim, t);
#undef E_
  free(heap);
}

/* XC1_int_tools.f:2-46 Gauss_prod and :49-88 Gauss_prod_1D (per dim) */
static void gauss_prod_1d(double A, double B, double Am, double Bm,
                          double *KAB, double *qAB, double *P, double *Pm,
                          double *Qm) {
  *qAB = A * B / (A + B);
  *Qm = Am - Bm;
  *KAB = exp(-*qAB * *Qm * *Qm);
  *P = A + B;
  *Pm = (A * Am + B * Bm) / (A + B);
}
static void gauss_prod(double A, double B, const double *Am, const double *Bm,
                       double *KAB, double *qAB, double *P, double *Pm,
                       double *Qm) {
  *qAB = A * B / (A + B);
  for (int d = 0; d < 3; d++) Qm[d] = Am[d] - Bm[d];
  for (int d = 0; d < 3; d++) KAB[d] = exp(-*qAB * Qm[d] * Qm[d]);
  *P = A + B;
  for (int d = 0; d < 3; d++) Pm[d] = (A * Am[d] + B * Bm[d]) / (A + B);
}

/* XC1_int_tools.f cbinom */
static double cbinom(int n, int k) {
  double nfac = 1.0, kfac = 1.0, nkfac = 1.0;
  if (!(n == 0 || n == 1))
    for (int i = n; i >= 1; i--) nfac = nfac * (double)i;
  if (!(k == 0 || k == 1))
    for (int i = k; i >= 1; i--) kfac = kfac * (double)i;
  int nk = n - k;
  if (!(nk == 0 || nk == 1))
    for (int i = nk; i >= 1; i--) nkfac = nkfac * (double)i;
  return nfac / (kfac * nkfac);
}

/* common.f:185-212 HermiteH */
static double hermiteH(int n, double x) {
  double A[64];
  A[1] = 2.0 * x;
  A[2] = (4.0 * x * x) - 2.0;
  for (int i = 2; i <= n; i++)
    A[i + 1] = (2.0 * x * A[i]) - (2.0 * (double)i * A[i - 1]);
  return n == 0 ? 1.0 : A[n];
}

/* common.f:116-150 gdel_Ax and :158-180 gdel_x */
double orc_gdel_x(int N, double x, double alp, double Ax) {
  double y = sqrt(alp) * (x - Ax);
  double dy = ipow(-1.0, N) * hermiteH(N, y) * exp(-y * y);
  double xj = ipow(-sqrt(alp), N);
  double gAx = xj * dy;
  return ipow(-1.0, N) * gAx;
}

/* XC1_G3_MD.f:2139-2179 DKGx */
static double dkgx(int n1, int n2, int n3, double xi, double f, double g,
                   double h, double x1, double x2, double x3) {
  int nt = n1 + n2 + n3;
  double u = f * x1 + g * x2 + h * x3;
  double c1 = (ipow(f, n1)) * (ipow(g, n2)) * (ipow(h, n3));
  return c1 * orc_gdel_x(nt, u, xi, 0.0);
}

/* XC1_G4_MD.f:1427-1470 DKGx_4 */
static double dkgx4(int n1, int n2, int n3, int n4, double xi, double e,
                    double f, double g, double h, double x1, double x2,
                    double x3, double x4) {
  int nt = n1 + n2 + n3 + n4;
  double u = e * x1 + f * x2 + g * x3 + h * x4;
  double c1 = (ipow(e, n1)) * (ipow(f, n2)) * (ipow(g, n3)) * (ipow(h, n4));
  return c1 * orc_gdel_x(nt, u, xi, 0.0);
}

/* Three derivative-Gaussian factors GK1..GK3 of the 3-particle kernels. */
typedef struct { double xi[3], f[3], g[3], h[3]; } gk3;

/* XC1_G3_MD.f:2049-2136 G3xggs_DGK123 */
static double dgk123(int xb1, int xb2, int xb3, const gk3 *k, double x1,
                     double x2, double x3) {
  double s = 0.0;
  for (int i1 = 0; i1 <= xb1; i1++) {
    double bi1 = cbinom(xb1, i1);
    for (int i2 = 0; i2 <= xb2; i2++) {
      double bi2 = cbinom(xb2, i2);
      for (int i3 = 0; i3 <= xb3; i3++) {
        double bi3 = cbinom(xb3, i3);
        double d1 = dkgx(xb1 - i1, xb2 - i2, xb3 - i3, k->xi[0], k->f[0],
                         k->g[0], k->h[0], x1, x2, x3);
        for (int j1 = 0; j1 <= i1; j1++) {
          double bj1 = cbinom(i1, j1);
          for (int j2 = 0; j2 <= i2; j2++) {
            double bj2 = cbinom(i2, j2);
            for (int j3 = 0; j3 <= i3; j3++) {
              double bj3 = cbinom(i3, j3);
              double d2 = dkgx(i1 - j1, i2 - j2, i3 - j3, k->xi[1], k->f[1],
                               k->g[1], k->h[1], x1, x2, x3);
              double d3 = dkgx(j1, j2, j3, k->xi[2], k->f[2], k->g[2],
                               k->h[2], x1, x2, x3);
              double ans = bi1 * bi2 * bi3 * bj1 * bj2 * bj3 * d1 * d2 * d3;
              s = s + ans;
            }
          }
        }
      }
    }
  }
  return s;
}

/* XC1_G3_MD.f:588-647 G3xggs_dfKKK_prep, :1091-1149 vec_dhermite_prep,
 * :1676-1735 vee_dhermite_prep (identical formulas) */
static void dfkkk_prep(double p1, double c1, double p2, double c2, double s1,
                       double s2, double gam12, gk3 *k) {
  k->xi[0] = (p1 * c1) / (p1 + c1);
  k->f[0] = 1.0; k->g[0] = 0.0; k->h[0] = -1.0;
  k->xi[1] = (p2 * c2) / (p2 + c2);
  k->f[1] = 0.0; k->g[1] = 1.0; k->h[1] = -1.0;
  k->xi[2] = (s1 * s2 * gam12) / (s1 * s2 + s1 * gam12 + s2 * gam12);
  k->f[2] = p1 / (p1 + c1);
  k->g[2] = -p2 / (p2 + c2);
  k->h[2] = (c1 / (p1 + c1)) - (c2 / (p2 + c2));
}

/* XC1_G3_MD.f:90-293 G3_MD_xggs1D */
static double g3_xggs1d(int I1, double A1, double Am1, int I2, double A2,
                        double Am2, int I3, double A3, double Am3, int L1,
                        double B1, double Bm1, int L2, double B2, double Bm2,
                        int L3, double B3, double Bm3, const double *gam) {
  double gam13 = gam[1] + gam[4];
  double gam23 = gam[2] + gam[5];
  double gam12 = gam[0] + gam[3];
  double KAB1, KAB2, KAB3, qAB1, qAB2, qAB3, P1, P2, P3, Pm1, Pm2, Pm3, Q1,
      Q2, Q3;
  gauss_prod_1d(A1, B1, Am1, Bm1, &KAB1, &qAB1, &P1, &Pm1, &Q1);
  gauss_prod_1d(A2, B2, Am2, Bm2, &KAB2, &qAB2, &P2, &Pm2, &Q2);
  gauss_prod_1d(A3, B3, Am3, Bm3, &KAB3, &qAB3, &P3, &Pm3, &Q3);
  double Et1[24], Et2[24], Et3[24];
  orc_ghec(I1, L1, KAB1, A1, B1, P1, qAB1, Q1, Et1);
  orc_ghec(I2, L2, KAB2, A2, B2, P2, qAB2, Q2, Et2);
  orc_ghec(I3, L3, KAB3, A3, B3, P3, qAB3, Q3, Et3);
  double xsum = P3 + gam13 + gam23;
  double C0 = sqrt(PI_T / xsum);
  double C1 = (P3 * gam13) / xsum;
  double C2 = (P3 * gam23) / xsum;
  double C12 = (gam13 * gam23) / xsum;
  gam12 = gam12 + C12;
  double K13, q13, S1, Sm1, SQ1, K23, q23, S2, Sm2, SQ2;
  gauss_prod_1d(P1, C1, Pm1, Pm3, &K13, &q13, &S1, &Sm1, &SQ1);
  gauss_prod_1d(P2, C2, Pm2, Pm3, &K23, &q23, &S2, &Sm2, &SQ2);
  double tv1 = (S1 * S2 + S1 * gam12 + S2 * gam12);
  double tv2 = PI_T * PI_T / tv1;
  double C3 = sqrt(tv2);
  gk3 k;
  k.xi[0] = P1 * C1 / (P1 + C1);
  k.f[0] = 1.0; k.g[0] = 0.0; k.h[0] = -1.0;
  k.xi[1] = P2 * C2 / (P2 + C2);
  k.f[1] = 0.0; k.g[1] = 1.0; k.h[1] = -1.0;
  k.xi[2] = S1 * S2 * gam12 / (S1 * S2 + S1 * gam12 + S2 * gam12);
  k.f[2] = P1 / (P1 + C1);
  k.g[2] = -P2 / (P2 + C2);
  k.h[2] = C1 / (P1 + C1) - C2 / (P2 + C2);
  double ans = 0.0;
  for (int t1 = 0; t1 <= I1 + L1; t1++)
    for (int t2 = 0; t2 <= I2 + L2; t2++)
      for (int t3 = 0; t3 <= I3 + L3; t3++) {
        double df = dgk123(t1, t2, t3, &k, Pm1, Pm2, Pm3);
        double xans = Et1[t1] * Et2[t2] * Et3[t3] * df;
        ans = ans + xans;
      }
  return ans * C0 * C3;
}

/* XC1_G3_MD.f:2-87 G3_MD_xggs */
double orc_g3_xggs(const orc_prim *A, const orc_prim *B, const double *gam) {
  double I[3];
  for (int d = 0; d < 3; d++)
    I[d] = g3_xggs1d(A[0].l[d], A[0].a, A[0].c[d], A[1].l[d], A[1].a,
                     A[1].c[d], A[2].l[d], A[2].a, A[2].c[d], B[0].l[d],
                     B[0].a, B[0].c[d], B[1].l[d], B[1].a, B[1].c[d],
                     B[2].l[d], B[2].a, B[2].c[d], gam);
  return I[0] * I[1] * I[2];
}

/* XC1_G3_MD.f:2680-2866 G3_MD_T1d */
static double g3_t1d(int I1, double a1, double Am1, int I2, double a2,
                     double Am2, int I3, double a3, double Am3, int L1,
                     double b1, double Bm1, int L2, double b2, double Bm2,
                     int L3, double b3, double Bm3, const double *gam) {
  double x[11];
  for (int i = 0; i < 11; i++) x[i] = 0.0;
  double gB13 = gam[4];
  double XB1B3 = Bm1 - Bm3;
#define XG(l1, l3) g3_xggs1d(I1, a1, Am1, I2, a2, Am2, I3, a3, Am3, l1, b1, \
                             Bm1, L2, b2, Bm2, l3, b3, Bm3, gam)
  if (L1 > 0) {
    if (L1 > 1) x[1] = XG(L1 - 2, L3);
    x[2] = XG(L1 - 1, L3);
    x[3] = XG(L1 - 1, L3 + 1);
  }
  x[4] = XG(L1, L3);
  x[5] = XG(L1, L3 + 1);
  x[6] = XG(L1, L3 + 2);
  x[7] = XG(L1 + 1, L3);
  x[8] = XG(L1 + 1, L3 + 1);
  x[9] = XG(L1 + 2, L3);
#undef XG
  const double two = 2.0, four = 4.0, eight = 8.0, one = 1.0;
  double dL1 = (double)L1;
  double ans = (double)(L1 * (L1 - 1)) * x[1]
             - four * gB13 * XB1B3 * dL1 * x[2]
             + four * gB13 * dL1 * x[3]
             - two * b1 * (two * dL1 + one) * x[4]
             - four * gB13 * dL1 * x[4]
             + four * gB13 * gB13 * XB1B3 * XB1B3 * x[4]
             - two * gB13 * x[4]
             - eight * gB13 * gB13 * XB1B3 * x[5]
             + four * gB13 * gB13 * x[6]
             + eight * b1 * gB13 * XB1B3 * x[7]
             + eight * gB13 * gB13 * XB1B3 * x[7]
             - eight * b1 * gB13 * x[8]
             - eight * gB13 * gB13 * x[8]
             + (four * b1 * b1 + eight * b1 * gB13 + four * gB13 * gB13) * x[9];
  return ans;
}

/* XC1_G3_MD.f:2546-2677 G3_MD_KE */
double orc_g3_ke(const orc_prim *A, const orc_prim *B, const double *gam,
                 double xmass) {
  double S[3], T[3];
  for (int d = 0; d < 3; d++) {
    S[d] = g3_xggs1d(A[0].l[d], A[0].a, A[0].c[d], A[1].l[d], A[1].a,
                     A[1].c[d], A[2].l[d], A[2].a, A[2].c[d], B[0].l[d],
                     B[0].a, B[0].c[d], B[1].l[d], B[1].a, B[1].c[d],
                     B[2].l[d], B[2].a, B[2].c[d], gam);
  }
  for (int d = 0; d < 3; d++) {
    T[d] = g3_t1d(A[0].l[d], A[0].a, A[0].c[d], A[1].l[d], A[1].a,
                  A[1].c[d], A[2].l[d], A[2].a, A[2].c[d], B[0].l[d],
                  B[0].a, B[0].c[d], B[1].l[d], B[1].a, B[1].c[d],
                  B[2].l[d], B[2].a, B[2].c[d], gam);
  }
  double x = (T[0] * S[1] * S[2] + S[0] * T[1] * S[2] + S[0] * S[1] * T[2]);
  return -0.5 * x / xmass;
}

/* Hermite E tables for three particles, x/y/z. */
typedef struct {
  double P[3], Pm[3][3];
  double E[3][3][24]; /* [particle][dim][t] */
} e3tab;

static void e3_build(const orc_prim *A, const orc_prim *B, int np, e3tab *e,
                     double Pm[][3], double *P) {
  for (int i = 0; i < np; i++) {
    double KAB[3], qAB, Q[3];
    gauss_prod(A[i].a, B[i].a, A[i].c, B[i].c, KAB, &qAB, &P[i], Pm[i], Q);
    for (int d = 0; d < 3; d++)
      orc_ghec(A[i].l[d], B[i].l[d], KAB[d], A[i].a, B[i].a, P[i], qAB, Q[d],
               e->E[i < 3 ? i : 0][d]);
  }
}

/* XC1_G3_MD.f:1300-1371 g3_VxC_RTUV and :1968-2046 g3_RTUV */
static double g3_rtuv_c(int xb1, int yb1, int zb1, int xb2, int yb2, int zb2,
                        int xb3, int yb3, int zb3, double expT, double alpha,
                        double f, double g, double h, double Pm[3][3],
                        const double *C) {
  double Rm[3];
  for (int d = 0; d < 3; d++) {
    Rm[d] = (f * Pm[0][d]) + (g * Pm[1][d]) + (h * Pm[2][d]);
    if (C) Rm[d] = Rm[d] - C[d];
  }
  int NRx = xb1 + yb1 + zb1, NRy = xb2 + yb2 + zb2, NRz = xb3 + yb3 + zb3;
  int N = xb1 + xb2 + xb3, L = yb1 + yb2 + yb3, M = zb1 + zb2 + zb3;
  double c1 = (ipow(f, NRx)) * (ipow(g, NRy)) * (ipow(h, NRz));
  return c1 * orc_rtuv(N, L, M, N + L + M, expT, alpha, Rm[0], Rm[1], Rm[2]);
}

/* XC1_G3_MD.f:1152-1295 g3_vec_dhermite / :1737-1873 g3_vee_dhermite */
static double g3_dhermite(const int *t, const int *u, const int *v,
                          const gk3 *k, double bf, double bg, double bh,
                          double expT, double alpha, double Pm[3][3],
                          const double *C) {
  double Dgf = 0.0;
  for (int xb1 = 0; xb1 <= t[0]; xb1++) {
    double btx1 = cbinom(t[0], xb1);
    for (int xb2 = 0; xb2 <= t[1]; xb2++) {
      double btx2 = cbinom(t[1], xb2);
      for (int xb3 = 0; xb3 <= t[2]; xb3++) {
        double btx3 = cbinom(t[2], xb3);
        double dfx = dgk123(t[0] - xb1, t[1] - xb2, t[2] - xb3, k, Pm[0][0],
                            Pm[1][0], Pm[2][0]);
        for (int yb1 = 0; yb1 <= u[0]; yb1++) {
          double buy1 = cbinom(u[0], yb1);
          for (int yb2 = 0; yb2 <= u[1]; yb2++) {
            double buy2 = cbinom(u[1], yb2);
            for (int yb3 = 0; yb3 <= u[2]; yb3++) {
              double buy3 = cbinom(u[2], yb3);
              double dfy = dgk123(u[0] - yb1, u[1] - yb2, u[2] - yb3, k,
                                  Pm[0][1], Pm[1][1], Pm[2][1]);
              for (int zb1 = 0; zb1 <= v[0]; zb1++) {
                double bvz1 = cbinom(v[0], zb1);
                for (int zb2 = 0; zb2 <= v[1]; zb2++) {
                  double bvz2 = cbinom(v[1], zb2);
                  for (int zb3 = 0; zb3 <= v[2]; zb3++) {
                    double bvz3 = cbinom(v[2], zb3);
                    double dfz = dgk123(v[0] - zb1, v[1] - zb2, v[2] - zb3,
                                        k, Pm[0][2], Pm[1][2], Pm[2][2]);
                    double dfB = g3_rtuv_c(xb1, yb1, zb1, xb2, yb2, zb2, xb3,
                                           yb3, zb3, expT, alpha, bf, bg, bh,
                                           Pm, C);
                    double ans = btx1 * btx2 * btx3 * buy1 * buy2 * buy3 *
                                 bvz1 * bvz2 * bvz3 * dfx * dfy * dfz * dfB;
                    Dgf = Dgf + ans;
                  }
                }
              }
            }
          }
        }
      }
    }
  }
  return Dgf;
}

/* XC1_G3_MD.f:711-1088 G3_MD_xgVxCg (C != NULL) and
 * XC1_G3_MD.f:1376-1675 G3_MD_xgVeeg (C == NULL).  Both evaluate the
 * Boys-lemma reduction of particle 3 and the Hermite loops identically;
 * they differ in the final Coulomb factor. */
static double g3_coulomb(const orc_prim *A, const orc_prim *B,
                         const double *gam, const double *C) {
  double gam13 = gam[1] + gam[4];
  double gam23 = gam[2] + gam[5];
  double gam12s = gam[0] + gam[3];
  double P[3], Pm[3][3];
  e3tab e;
  e3_build(A, B, 3, &e, Pm, P);
  /* loop invariants of the reference's 9-deep Hermite loop */
  double xsum = P[2] + gam13 + gam23;
  double C0 = pow(PI_T / xsum, 1.5);           /* SFBoys2, :230-270 */
  double C1 = (P[2] * gam13) / xsum;
  double C2 = (P[2] * gam23) / xsum;
  double C12 = (gam13 * gam23) / xsum;
  double gam12 = gam12s;
  gam12 = gam12 + C12;
  double K13[3], q13, S1, Sm1[3], SQ1[3], K23[3], q23, S2, Sm2[3], SQ2[3];
  gauss_prod(P[0], C1, Pm[0], Pm[2], K13, &q13, &S1, Sm1, SQ1);
  gauss_prod(P[1], C2, Pm[1], Pm[2], K23, &q23, &S2, Sm2, SQ2);
  double p1 = P[0], p2 = P[1], s1 = S1, s2 = S2, c1 = C1, c2 = C2;
  double C3, alpha, expT, bf, bg, bh;
  if (C) {
    double tv1 = (s2 + gam12);
    double tv2 = (S1 * S2 + S1 * gam12 + S2 * gam12);
    double tv3 = tv2 / tv1;
    C3 = sqrt(ipow(PI_T / tv1, 3)) * (2.0 * PI_T / tv3);
    double Sm[3];
    for (int d = 0; d < 3; d++)
      Sm[d] = ((s1 * s2 + s1 * gam12) / tv2) * Sm1[d] +
              ((s2 * gam12) / tv2) * Sm2[d];
    double R2 = (C[0] - Sm[0]) * (C[0] - Sm[0]) +
                (C[1] - Sm[1]) * (C[1] - Sm[1]) +
                (C[2] - Sm[2]) * (C[2] - Sm[2]);
    alpha = tv3;
    expT = alpha * R2;
    bf = (s1 * s2 + s1 * gam12) / (s1 * s2 + s1 * gam12 + s2 * gam12) *
         (p1 / (p1 + c1));
    bg = (s2 * gam12) / (s1 * s2 + s1 * gam12 + s2 * gam12) * (p2 / (p2 + c2));
    bh = (s1 * s2 + s1 * gam12) / (s1 * s2 + s1 * gam12 + s2 * gam12) *
             (c1 / (p1 + c1)) +
         (s2 * gam12) / (s1 * s2 + s1 * gam12 + s2 * gam12) * (c2 / (p2 + c2));
  } else {
    double tv1 = (S1 * S2 + S1 * gam12 + S2 * gam12) * sqrt(S1 + S2);
    double tv3 = (S1 * S2 + S1 * gam12 + S2 * gam12) * (S1 + S2);
    double R2 = (Sm1[0] - Sm2[0]) * (Sm1[0] - Sm2[0]) +
                (Sm1[1] - Sm2[1]) * (Sm1[1] - Sm2[1]) +
                (Sm1[2] - Sm2[2]) * (Sm1[2] - Sm2[2]);
    C3 = (2.0 * sqrt(ipow(PI_T, 5))) / tv1;
    alpha = (S1 * S1 * S2 * S2) / (tv3);
    expT = alpha * R2;
    bf = bg = bh = 0.0; /* set from the dfKKK prep below */
  }
  gk3 k;
  dfkkk_prep(p1, c1, p2, c2, s1, s2, gam12, &k);
  if (!C) { bf = k.f[2]; bg = k.g[2]; bh = k.h[2]; }
  double out = 0.0;
  int tl[3], ul[3], vl[3];
  for (int i = 0; i < 3; i++) {
    tl[i] = A[i].l[0] + B[i].l[0];
    ul[i] = A[i].l[1] + B[i].l[1];
    vl[i] = A[i].l[2] + B[i].l[2];
  }
  int t[3], u[3], v[3];
  for (t[0] = 0; t[0] <= tl[0]; t[0]++)
  for (u[0] = 0; u[0] <= ul[0]; u[0]++)
  for (v[0] = 0; v[0] <= vl[0]; v[0]++)
  for (t[1] = 0; t[1] <= tl[1]; t[1]++)
  for (u[1] = 0; u[1] <= ul[1]; u[1]++)
  for (v[1] = 0; v[1] <= vl[1]; v[1]++)
  for (t[2] = 0; t[2] <= tl[2]; t[2]++)
  for (u[2] = 0; u[2] <= ul[2]; u[2]++)
  for (v[2] = 0; v[2] <= vl[2]; v[2]++) {
    double Dgf = g3_dhermite(t, u, v, &k, bf, bg, bh, expT, alpha, Pm, C);
    double ans = C0 * C3 * e.E[0][0][t[0]] * e.E[1][0][t[1]] *
                 e.E[2][0][t[2]] * e.E[0][1][u[0]] * e.E[1][1][u[1]] *
                 e.E[2][1][u[2]] * e.E[0][2][v[0]] * e.E[1][2][v[1]] *
                 e.E[2][2][v[2]] * Dgf;
    out = out + ans;
  }
  return out;
}

double orc_g3_xgvxcg(const orc_prim *A, const orc_prim *B, const double *gam,
                     const double *C) {
  return g3_coulomb(A, B, gam, C);
}
double orc_g3_xgveeg(const orc_prim *A, const orc_prim *B, const double *gam) {
  return g3_coulomb(A, B, gam, NULL);
}

/* XC1_G2_MD.f:3-187 G2_MD_xggs; particles (A1,B1) and (A2,B2) */
double orc_g2_xggs(const orc_prim *A1, const orc_prim *A2,
                   const orc_prim *B1, const orc_prim *B2, double gamma1,
                   double gamma2) {
  double GAM = gamma1 + gamma2;
  double K1[3], q1, P1, Pm1[3], Q1[3], K2[3], q2, P2, Pm2[3], Q2[3];
  gauss_prod(A1->a, B1->a, A1->c, B1->c, K1, &q1, &P1, Pm1, Q1);
  gauss_prod(A2->a, B2->a, A2->c, B2->c, K2, &q2, &P2, Pm2, Q2);
  double E1[3][24], E2[3][24];
  for (int d = 0; d < 3; d++) {
    orc_ghec(A1->l[d], B1->l[d], K1[d], A1->a, B1->a, P1, q1, Q1[d], E1[d]);
    orc_ghec(A2->l[d], B2->l[d], K2[d], A2->a, B2->a, P2, q2, Q2[d], E2[d]);
  }
  double qP = (P1 * P2 * GAM) / (P1 * P2 + P1 * GAM + P2 * GAM);
  double c1 = pow(PI_T * PI_T / (P1 * P2 + P1 * GAM + P2 * GAM), 1.5);
  double s = 0.0;
  for (int t1 = 0; t1 <= A1->l[0] + B1->l[0]; t1++)
  for (int u1 = 0; u1 <= A1->l[1] + B1->l[1]; u1++)
  for (int v1 = 0; v1 <= A1->l[2] + B1->l[2]; v1++)
  for (int t2 = 0; t2 <= A2->l[0] + B2->l[0]; t2++)
  for (int u2 = 0; u2 <= A2->l[1] + B2->l[1]; u2++)
  for (int v2 = 0; v2 <= A2->l[2] + B2->l[2]; v2++) {
    double c2 = pow(-1.0, (double)(t2 + u2 + v2));
    double dgx = orc_gdel_x(t1 + t2, Pm1[0], qP, Pm2[0]);
    double dgy = orc_gdel_x(u1 + u2, Pm1[1], qP, Pm2[1]);
    double dgz = orc_gdel_x(v1 + v2, Pm1[2], qP, Pm2[2]);
    double ans = c1 * c2 * E1[0][t1] * E2[0][t2] * E1[1][u1] * E2[1][u2] *
                 E1[2][v1] * E2[2][v2] * dgx * dgy * dgz;
    s = s + ans;
  }
  return s;
}

/* Four-particle derivative-Gaussian set (XC1_G4_MD.f). */
typedef struct { int ngk; double xi[3], e[3], f[3], g[3], h[3]; } gk4;

/* XC1_G4_MD.f:1331-1424 G4xggs_DGK123 and :2151-2223 G4xggs_DGK12 */
static double dgk4(const int *xb, const gk4 *k, const double *x) {
  double s = 0.0;
  for (int i1 = 0; i1 <= xb[0]; i1++) {
    double bi1 = cbinom(xb[0], i1);
  for (int i2 = 0; i2 <= xb[1]; i2++) {
    double bi2 = cbinom(xb[1], i2);
  for (int i3 = 0; i3 <= xb[2]; i3++) {
    double bi3 = cbinom(xb[2], i3);
  for (int i4 = 0; i4 <= xb[3]; i4++) {
    double bi4 = cbinom(xb[3], i4);
    double d1 = dkgx4(xb[0] - i1, xb[1] - i2, xb[2] - i3, xb[3] - i4,
                      k->xi[0], k->e[0], k->f[0], k->g[0], k->h[0], x[0],
                      x[1], x[2], x[3]);
    if (k->ngk == 2) {
      double d2 = dkgx4(i1, i2, i3, i4, k->xi[1], k->e[1], k->f[1], k->g[1],
                        k->h[1], x[0], x[1], x[2], x[3]);
      double ans = bi1 * bi2 * bi3 * bi4 * d1 * d2;
      s = s + ans;
      continue;
    }
    for (int j1 = 0; j1 <= i1; j1++) {
      double bj1 = cbinom(i1, j1);
    for (int j2 = 0; j2 <= i2; j2++) {
      double bj2 = cbinom(i2, j2);
    for (int j3 = 0; j3 <= i3; j3++) {
      double bj3 = cbinom(i3, j3);
    for (int j4 = 0; j4 <= i4; j4++) {
      double bj4 = cbinom(i4, j4);
      double d2 = dkgx4(i1 - j1, i2 - j2, i3 - j3, i4 - j4, k->xi[1],
                        k->e[1], k->f[1], k->g[1], k->h[1], x[0], x[1],
                        x[2], x[3]);
      double d3 = dkgx4(j1, j2, j3, j4, k->xi[2], k->e[2], k->f[2], k->g[2],
                        k->h[2], x[0], x[1], x[2], x[3]);
      double ans = bi1 * bi2 * bi3 * bi4 * bj1 * bj2 * bj3 * bj4 * d1 * d2 *
                   d3;
      s = s + ans;
    }}}}
  }}}}
  return s;
}

/* XC1_G4_MD.f:1473-1556 G4_RTUV */
static double g4_rtuv(const int *xb, const int *yb, const int *zb,
                      double expT, double alpha, const double *cof,
                      double Pm[4][3]) {
  double W[3];
  for (int d = 0; d < 3; d++)
    W[d] = (cof[0] * Pm[0][d]) + (cof[1] * Pm[1][d]) + (cof[2] * Pm[2][d]) +
           (cof[3] * Pm[3][d]);
  int N = xb[0] + xb[1] + xb[2] + xb[3];
  int L = yb[0] + yb[1] + yb[2] + yb[3];
  int M = zb[0] + zb[1] + zb[2] + zb[3];
  double c1 = ipow(cof[0], xb[0] + yb[0] + zb[0]);
  double c2 = ipow(cof[1], xb[1] + yb[1] + zb[1]);
  double c3 = ipow(cof[2], xb[2] + yb[2] + zb[2]);
  double c4 = ipow(cof[3], xb[3] + yb[3] + zb[3]);
  return c1 * c2 * c3 * c4 *
         orc_rtuv(N, L, M, N + L + M, expT, alpha, W[0], W[1], W[2]);
}

/* XC1_G4_MD.f:1173-1328 G4_xgVee_dhermite / :1981-2148 G4_xgVep_dhermite */
static double g4_dhermite(const int *t, const int *u, const int *v,
                          const gk4 *k, const double *cof, double expT,
                          double alpha, double Pm[4][3]) {
  double Dgf = 0.0;
  int xb[4], yb[4], zb[4], a[4];
  double X[4], Y[4], Z[4];
  for (int i = 0; i < 4; i++) { X[i] = Pm[i][0]; Y[i] = Pm[i][1]; Z[i] = Pm[i][2]; }
  for (xb[0] = 0; xb[0] <= t[0]; xb[0]++) {
    double bt1 = cbinom(t[0], xb[0]);
  for (xb[1] = 0; xb[1] <= t[1]; xb[1]++) {
    double bt2 = cbinom(t[1], xb[1]);
  for (xb[2] = 0; xb[2] <= t[2]; xb[2]++) {
    double bt3 = cbinom(t[2], xb[2]);
  for (xb[3] = 0; xb[3] <= t[3]; xb[3]++) {
    double bt4 = cbinom(t[3], xb[3]);
    for (int i = 0; i < 4; i++) a[i] = t[i] - xb[i];
    double dfx = dgk4(a, k, X);
    for (yb[0] = 0; yb[0] <= u[0]; yb[0]++) {
      double bu1 = cbinom(u[0], yb[0]);
    for (yb[1] = 0; yb[1] <= u[1]; yb[1]++) {
      double bu2 = cbinom(u[1], yb[1]);
    for (yb[2] = 0; yb[2] <= u[2]; yb[2]++) {
      double bu3 = cbinom(u[2], yb[2]);
    for (yb[3] = 0; yb[3] <= u[3]; yb[3]++) {
      double bu4 = cbinom(u[3], yb[3]);
      for (int i = 0; i < 4; i++) a[i] = u[i] - yb[i];
      double dfy = dgk4(a, k, Y);
      for (zb[0] = 0; zb[0] <= v[0]; zb[0]++) {
        double bv1 = cbinom(v[0], zb[0]);
      for (zb[1] = 0; zb[1] <= v[1]; zb[1]++) {
        double bv2 = cbinom(v[1], zb[1]);
      for (zb[2] = 0; zb[2] <= v[2]; zb[2]++) {
        double bv3 = cbinom(v[2], zb[2]);
      for (zb[3] = 0; zb[3] <= v[3]; zb[3]++) {
        double bv4 = cbinom(v[3], zb[3]);
        for (int i = 0; i < 4; i++) a[i] = v[i] - zb[i];
        double dfz = dgk4(a, k, Z);
        double dfB = g4_rtuv(xb, yb, zb, expT, alpha, cof, Pm);
        double ans = bt1 * bt2 * bt3 * bt4 * bu1 * bu2 * bu3 * bu4 * bv1 *
                     bv2 * bv3 * bv4 * dfx * dfy * dfz * dfB;
        Dgf = Dgf + ans;
      }}}}
    }}}}
  }}}}
  return Dgf;
}

static void e4_build(const orc_prim *A, const orc_prim *B, double E[4][3][24],
                     double Pm[4][3], double *P) {
  for (int i = 0; i < 4; i++) {
    double KAB[3], qAB, Q[3];
    gauss_prod(A[i].a, B[i].a, A[i].c, B[i].c, KAB, &qAB, &P[i], Pm[i], Q);
    for (int d = 0; d < 3; d++)
      orc_ghec(A[i].l[d], B[i].l[d], KAB[d], A[i].a, B[i].a, P[i], qAB, Q[d],
               E[i][d]);
  }
}

static double g4_hermite_sum(const orc_prim *A, const orc_prim *B,
                             double E[4][3][24], double pref, const gk4 *k,
                             const double *cof, double expT, double alpha,
                             double Pm[4][3]) {
  int tl[4], ul[4], vl[4];
  for (int i = 0; i < 4; i++) {
    tl[i] = A[i].l[0] + B[i].l[0];
    ul[i] = A[i].l[1] + B[i].l[1];
    vl[i] = A[i].l[2] + B[i].l[2];
  }
  double out = 0.0;
  int t[4], u[4], v[4];
  for (t[0] = 0; t[0] <= tl[0]; t[0]++)
  for (u[0] = 0; u[0] <= ul[0]; u[0]++)
  for (v[0] = 0; v[0] <= vl[0]; v[0]++)
  for (t[1] = 0; t[1] <= tl[1]; t[1]++)
  for (u[1] = 0; u[1] <= ul[1]; u[1]++)
  for (v[1] = 0; v[1] <= vl[1]; v[1]++)
  for (t[2] = 0; t[2] <= tl[2]; t[2]++)
  for (u[2] = 0; u[2] <= ul[2]; u[2]++)
  for (v[2] = 0; v[2] <= vl[2]; v[2]++)
  for (t[3] = 0; t[3] <= tl[3]; t[3]++)
  for (u[3] = 0; u[3] <= ul[3]; u[3]++)
  for (v[3] = 0; v[3] <= vl[3]; v[3]++) {
    double Dgf = g4_dhermite(t, u, v, k, cof, expT, alpha, Pm);
    double ans = pref * E[0][0][t[0]] * E[1][0][t[1]] * E[2][0][t[2]] *
                 E[3][0][t[3]] * E[0][1][u[0]] * E[1][1][u[1]] *
                 E[2][1][u[2]] * E[3][1][u[3]] * E[0][2][v[0]] *
                 E[1][2][v[1]] * E[2][2][v[2]] * E[3][2][v[3]] * Dgf;
    out = out + ans;
  }
  return out;
}

/* XC1_G4_MD.f:796-1125 G4_MD_xgVeeg (+ :1126-1170 prep_fKKK) */
double orc_g4_xgveeg(const orc_prim *A, const orc_prim *B, double gam14,
                     double gam34) {
  double E[4][3][24], Pm[4][3], P[4];
  e4_build(A, B, E, Pm, P);
  const double PI = PI_T;
  double xsum = P[3] + gam14 + gam34;                 /* SFBoys2 */
  double C0 = pow(PI / xsum, 1.5);
  double C1 = (P[3] * gam14) / xsum;
  double C3 = (P[3] * gam34) / xsum;
  double C13 = (gam14 * gam34) / xsum;
  double K14[3], q14, S1, Sm1[3], SQ1[3], K34[3], q34, S3, Sm3[3], SQ3[3];
  gauss_prod(P[0], C1, Pm[0], Pm[3], K14, &q14, &S1, Sm1, SQ1);
  gauss_prod(P[2], C3, Pm[2], Pm[3], K34, &q34, &S3, Sm3, SQ3);
  double CB0 = (PI / (S3 + C13)) * sqrt(PI / (S3 + C13));
  double CB1 = (S3 * C13) / (S3 + C13);
  double KS[3], qS, W1, Wm[3], WQ[3];
  gauss_prod(S1, CB1, Sm1, Sm3, KS, &qS, &W1, Wm, WQ);
  double cof[4];
  cof[0] = P[0] / (S1 + CB1);
  cof[1] = -1.0;
  cof[2] = (CB1 / (S1 + CB1)) * (P[2] / (P[2] + C3));
  cof[3] = (C1 / (S1 + CB1)) + (CB1 / (S1 + CB1)) * (C3 / (P[2] + C3));
  double RWP[3];
  for (int d = 0; d < 3; d++)
    RWP[d] = cof[0] * Pm[0][d] + cof[1] * Pm[1][d] + cof[2] * Pm[2][d] +
             cof[3] * Pm[3][d];
  double R2 = RWP[0] * RWP[0] + RWP[1] * RWP[1] + RWP[2] * RWP[2];
  double C4 = (2.0 * PI * PI * sqrt(PI)) / (W1 * P[1] * sqrt(W1 + P[1]));
  double alpha = (W1 * P[1]) / (W1 + P[1]);
  double expT = alpha * R2;
  gk4 k;
  k.ngk = 3;
  k.xi[0] = P[0] * C1 / (P[0] + C1);
  k.xi[1] = P[2] * C3 / (P[2] + C3);
  k.xi[2] = S1 * CB1 / (S1 + CB1);
  k.e[0] = 1.0; k.f[0] = 0.0; k.g[0] = 0.0; k.h[0] = -1.0;
  k.e[1] = 0.0; k.f[1] = 0.0; k.g[1] = 1.0; k.h[1] = -1.0;
  k.e[2] = P[0] / (P[0] + C1);
  k.f[2] = 0.0;
  k.g[2] = -P[2] / (P[2] + C3);
  k.h[2] = C1 / (P[0] + C1) - C3 / (P[2] + C3);
  return g4_hermite_sum(A, B, E, C0 * CB0 * C4, &k, cof, expT, alpha, Pm);
}

/* XC1_G4_MD.f:1559-1978 G4_MD_xgVepg */
double orc_g4_xgvepg(const orc_prim *A, const orc_prim *B, double gam14,
                     double gam24) {
  double E[4][3][24], Pm[4][3], P[4];
  e4_build(A, B, E, Pm, P);
  const double PI = PI_T;
  double C0 = (PI / (P[0] + gam14)) * sqrt(PI / (P[0] + gam14));
  double C1 = (P[0] * gam14) / (P[0] + gam14);
  double K14[3], q14, S4, Sm4[3], SQ4[3];
  gauss_prod(C1, P[3], Pm[0], Pm[3], K14, &q14, &S4, Sm4, SQ4);
  double CB0 = (PI / (P[1] + gam24)) * sqrt(PI / (P[1] + gam24));
  double CB1 = (P[1] * gam24) / (P[1] + gam24);
  double KS[3], qS, Tx4, Tm4[3], TQ4[3];
  gauss_prod(S4, CB1, Sm4, Pm[1], KS, &qS, &Tx4, Tm4, TQ4);
  double xcof = (S4 + CB1) * (C1 + P[3]);
  double cof[4];
  cof[0] = S4 * C1 / xcof;
  cof[1] = CB1 / (S4 + CB1);
  cof[2] = -1.0;
  cof[3] = S4 * P[3] / xcof;
  double RTP[3];
  for (int d = 0; d < 3; d++) RTP[d] = Tm4[d] - Pm[2][d];
  double R2 = RTP[0] * RTP[0] + RTP[1] * RTP[1] + RTP[2] * RTP[2];
  double C4 = (2.0 * PI * PI * sqrt(PI)) / (P[2] * Tx4 * sqrt(P[2] + Tx4));
  double alpha = (P[2] * Tx4) / (P[2] + Tx4);
  double expT = alpha * R2;
  gk4 k;
  k.ngk = 2;
  k.xi[0] = (P[3] * C1) / (P[3] + C1);
  k.e[0] = 1.0; k.f[0] = 0.0; k.g[0] = 0.0; k.h[0] = -1.0;
  k.xi[1] = (S4 * CB1) / (S4 + CB1);
  k.e[1] = C1 / (C1 + P[3]); k.f[1] = -1.0; k.g[1] = 0.0;
  k.h[1] = P[3] / (C1 + P[3]);
  k.xi[2] = 0.0; k.e[2] = k.f[2] = k.g[2] = k.h[2] = 0.0;
  return g4_hermite_sum(A, B, E, C0 * CB0 * C4, &k, cof, expT, alpha, Pm);
}

/* ---- two-centre AC integrals (AC_Integrals: ovlap.f, ke.f, vec.f, vee.f) ----------------------- */

/* common.f:3-34 omega1D */
static void omega1d(int I, int J, double a, double b, double AX, double BX,
                    double *p, double *q, double *PX, double *QX, double *xK,
                    double *E) {
  *p = a + b;
  *PX = ((a * AX) + (b * BX)) / (a + b);
  *q = (a * b) / (a + b);
  *QX = AX - BX;
  *xK = exp(-*q * *QX * *QX);
  orc_ghec(I, J, *xK, a, b, *p, *q, *QX, E);
}

/* ovlap.f:25-70 gfovlap_1D */
static double gfovlap_1d(int I1, double a1, double A1, int L1, double b1,
                         double B1) {
  double PI = acos(-1.0);
  double p, q, PX, QX, xK, E[24];
  omega1d(I1, L1, a1, b1, A1, B1, &p, &q, &PX, &QX, &xK, E);
  return E[0] * sqrt(PI / p);
}

/* ovlap.f:2-22 gfovlap */
double orc_gfovlap(const orc_prim *A, const orc_prim *B) {
  double s[3];
  for (int d = 0; d < 3; d++)
    s[d] = gfovlap_1d(A->l[d], A->a, A->c[d], B->l[d], B->a, B->c[d]);
  return s[0] * s[1] * s[2];
}

/* ke.f:62-120 Lapx1 */
static double lapx1(int I1, double a1, double A1, int L1, double b1,
                    double B1) {
  double d1 = 0.0, p1 = 0.0;
  if (L1 - 1 >= 0) d1 = (double)(L1 * (L1 - 1));
  double d2 = -2.0 * b1 * (double)((2 * L1) + 1);
  double d3 = 4.0 * b1 * b1;
  if (L1 - 2 >= 0) p1 = gfovlap_1d(I1, a1, A1, L1 - 2, b1, B1);
  double p2 = gfovlap_1d(I1, a1, A1, L1, b1, B1);
  double p3 = gfovlap_1d(I1, a1, A1, L1 + 2, b1, B1);
  return (d1 * p1) + (d2 * p2) + (d3 * p3);
}

/* ke.f:2-59 gfke */
double orc_gfke(const orc_prim *A, const orc_prim *B, double xmass) {
  double S[3], T[3];
  for (int d = 0; d < 3; d++)
    S[d] = gfovlap_1d(A->l[d], A->a, A->c[d], B->l[d], B->a, B->c[d]);
  for (int d = 0; d < 3; d++) {
    double dd = lapx1(A->l[d], A->a, A->c[d], B->l[d], B->a, B->c[d]);
    T[d] = -dd * 0.50 / xmass;
  }
  return (T[0] * S[1] * S[2]) + (S[0] * T[1] * S[2]) + (S[0] * S[1] * T[2]);
}

/* vec.f:2-94 gfvec with vec.f:97-124 hint1 */
double orc_gfvec(const orc_prim *A, const orc_prim *B, const double *C) {
  double p, q, P[3], Q, xK, e[3][24];
  for (int d = 0; d < 3; d++)
    omega1d(A->l[d], B->l[d], A->a, B->a, A->c[d], B->c[d], &p, &q, &P[d],
            &Q, &xK, e[d]);
  double PI = acos(-1.0);
  double PC[3];
  for (int d = 0; d < 3; d++) PC[d] = P[d] - C[d];
  double xsum = 0.0;
  for (int it = 0; it <= A->l[0] + B->l[0]; it++)
  for (int iu = 0; iu <= A->l[1] + B->l[1]; iu++)
  for (int iv = 0; iv <= A->l[2] + B->l[2]; iv++) {
    double E1 = e[0][it] * e[1][iu] * e[2][iv];
    double R = orc_auxR2(it, iu, iv, p, PC[0], PC[1], PC[2]);
    double herm = 2.0 * PI * R / p;
    xsum = xsum + (E1 * herm);
  }
  return xsum;
}

/* vee.f:3-78 gfvee with hint2 (:80-150) and get_coefEE (:153-) */
double orc_gfvee(const orc_prim *A1, const orc_prim *A2, const orc_prim *B1,
                 const orc_prim *B2) {
  double p1, q1, P1[3], Q1, K1, e1[3][24];
  double p2, q2, P2[3], Q2, K2, e2[3][24];
  for (int d = 0; d < 3; d++) {
    omega1d(A1->l[d], B1->l[d], A1->a, B1->a, A1->c[d], B1->c[d], &p1, &q1,
            &P1[d], &Q1, &K1, e1[d]);
    omega1d(A2->l[d], B2->l[d], A2->a, B2->a, A2->c[d], B2->c[d], &p2, &q2,
            &P2[d], &Q2, &K2, e2[d]);
  }
  double PI = acos(-1.0);
  double gamma = 0.0;
  /* get_coefEE */
  double c1 = (2.0 * sqrt(ipow(PI, 5)));
  double c2 = ((p1 * p2) + (p1 * gamma) + (p2 * gamma)) * sqrt(p1 + p2);
  double coe2 = c1 / c2;
  double bc1 = (p1 * p2) * (p1 * p2);
  double bc2 = (p1 * p2) + (p1 * gamma) + (p2 * gamma);
  double bc3 = p1 + p2;
  double beta = bc1 / (bc2 * bc3);
  double vec[3];
  for (int d = 0; d < 3; d++) vec[d] = P1[d] - P2[d];
  double xsum = 0.0;
  for (int it1 = 0; it1 <= A1->l[0] + B1->l[0]; it1++)
  for (int iu1 = 0; iu1 <= A1->l[1] + B1->l[1]; iu1++)
  for (int iv1 = 0; iv1 <= A1->l[2] + B1->l[2]; iv1++)
  for (int it2 = 0; it2 <= A2->l[0] + B2->l[0]; it2++)
  for (int iu2 = 0; iu2 <= A2->l[1] + B2->l[1]; iu2++)
  for (int iv2 = 0; iv2 <= A2->l[2] + B2->l[2]; iv2++) {
    double coe1 = ipow(-1.0, it2 + iu2 + iv2);
    double R = orc_auxR2(it1 + it2, iu1 + iu2, iv1 + iv2, beta, vec[0],
                         vec[1], vec[2]);
    double herm = coe1 * coe2 * R;
    double E1 = e1[0][it1] * e1[1][iu1] * e1[2][iv1];
    double E2 = e2[0][it2] * e2[1][iu2] * e2[2][iv2];
    xsum = xsum + (E1 * E2 * herm);
  }
  return xsum;
}

/* ---- two-particle geminal kernels used by gam_1 (XC1_G2_MD.f, g2.f) ------- */

/* XC1_G2_MD.f:383-461 g2_vec_prefactors and :465-624 g2_dhermite_vec,
 * summed as G2_MD_xggvec (:190-378): Coulomb attraction of particle 1 to the
 * point C between geminal-correlated particles (A1,B1) and (A2,B2). */
double orc_g2_xggvec(const orc_prim *A1, const orc_prim *A2,
                     const orc_prim *B1, const orc_prim *B2, double gamma1,
                     double gamma2, const double *C) {
  double GAM = gamma1 + gamma2;
  double K1[3], q1, P1, Pm1[3], Q1[3], K2[3], q2, P2, Pm2[3], Q2[3];
  gauss_prod(A1->a, B1->a, A1->c, B1->c, K1, &q1, &P1, Pm1, Q1);
  gauss_prod(A2->a, B2->a, A2->c, B2->c, K2, &q2, &P2, Pm2, Q2);
  double E1[3][24], E2[3][24];
  for (int d = 0; d < 3; d++) {
    orc_ghec(A1->l[d], B1->l[d], K1[d], A1->a, B1->a, P1, q1, Q1[d], E1[d]);
    orc_ghec(A2->l[d], B2->l[d], K2[d], A2->a, B2->a, P2, q2, Q2[d], E2[d]);
  }
  /* g2_vec_prefactors */
  double s = (P1 * P2 + P1 * GAM + P2 * GAM) / (P2 + GAM);
  double alpha = s;
  double c1 = pow(PI_T / (P2 + GAM), 3.0 / 2.0) * 2.0 * PI_T / s;
  double xx = P1 * P2 + P1 * GAM + P2 * GAM;
  double Sm[3], RCS[3];
  for (int d = 0; d < 3; d++)
    Sm[d] = ((P1 * P2 + P1 * GAM) * Pm1[d] + P2 * GAM * Pm2[d]) / xx;
  for (int d = 0; d < 3; d++) RCS[d] = C[d] - Sm[d];
  double R2CS = RCS[0] * RCS[0] + RCS[1] * RCS[1] + RCS[2] * RCS[2];
  double expT = alpha * R2CS;
  double qP = (P1 * P2 * GAM) / xx;
  double DC1 = (P1 * P2 + P1 * GAM) / xx;
  double DC2 = (P2 * GAM) / xx;
  double out = 0.0;
  for (int t1 = 0; t1 <= A1->l[0] + B1->l[0]; t1++)
  for (int u1 = 0; u1 <= A1->l[1] + B1->l[1]; u1++)
  for (int v1 = 0; v1 <= A1->l[2] + B1->l[2]; v1++)
  for (int t2 = 0; t2 <= A2->l[0] + B2->l[0]; t2++)
  for (int u2 = 0; u2 <= A2->l[1] + B2->l[1]; u2++)
  for (int v2 = 0; v2 <= A2->l[2] + B2->l[2]; v2++) {
    /* g2_dhermite_vec */
    double Dgf = 0.0;
    for (int xb1 = 0; xb1 <= t1; xb1++) {
      int ax1 = t1 - xb1;
      double a1 = cbinom(t1, xb1);
      for (int yb1 = 0; yb1 <= u1; yb1++) {
        int ay1 = u1 - yb1;
        double a2 = cbinom(u1, yb1);
        for (int zb1 = 0; zb1 <= v1; zb1++) {
          int az1 = v1 - zb1;
          double a3 = cbinom(v1, zb1);
          for (int xb2 = 0; xb2 <= t2; xb2++) {
            int ax2 = t2 - xb2;
            double b1 = cbinom(t2, xb2);
            for (int yb2 = 0; yb2 <= u2; yb2++) {
              int ay2 = u2 - yb2;
              double b2 = cbinom(u2, yb2);
              for (int zb2 = 0; zb2 <= v2; zb2++) {
                int az2 = v2 - zb2;
                double b3 = cbinom(v2, zb2);
                double C1 = ipow(-1.0, ax2 + ay2 + az2);
                double C2 = ipow(-DC1, xb1 + yb1 + zb1);
                double C3 = ipow(-DC2, xb2 + yb2 + zb2);
                double dgx = orc_gdel_x(ax1 + ax2, Pm1[0], qP, Pm2[0]);
                double dgy = orc_gdel_x(ay1 + ay2, Pm1[1], qP, Pm2[1]);
                double dgz = orc_gdel_x(az1 + az2, Pm1[2], qP, Pm2[2]);
                double dgxyz = dgx * dgy * dgz;
                int nLim = xb1 + yb1 + zb1 + xb2 + yb2 + zb2;
                double dfxyz = orc_rtuv(xb1 + xb2, yb1 + yb2, zb1 + zb2, nLim,
                                        expT, alpha, RCS[0], RCS[1], RCS[2]);
                Dgf = Dgf + a1 * a2 * a3 * b1 * b2 * b3 * C1 * C2 * C3 *
                                dgxyz * dfxyz;
              }
            }
          }
        }
      }
    }
    double ans = c1 * E1[0][t1] * E2[0][t2] * E1[1][u1] * E2[1][u2] *
                 E1[2][v1] * E2[2][v2] * Dgf;
    out = out + ans;
  }
  return out;
}

/* XC1_G2_MD.f:801-859 g2_ee_prefactors and :863-960 g2_dhermite_vee,
 * summed as G2_MD_xggvee (:630-796): Coulomb repulsion between the two
 * geminal-correlated particles. */
double orc_g2_xggvee(const orc_prim *A1, const orc_prim *A2,
                     const orc_prim *B1, const orc_prim *B2, double gamma1,
                     double gamma2) {
  double GAM = gamma1 + gamma2;
  double K1[3], q1, P1, Pm1[3], Q1[3], K2[3], q2, P2, Pm2[3], Q2[3];
  gauss_prod(A1->a, B1->a, A1->c, B1->c, K1, &q1, &P1, Pm1, Q1);
  gauss_prod(A2->a, B2->a, A2->c, B2->c, K2, &q2, &P2, Pm2, Q2);
  double E1[3][24], E2[3][24];
  for (int d = 0; d < 3; d++) {
    orc_ghec(A1->l[d], B1->l[d], K1[d], A1->a, B1->a, P1, q1, Q1[d], E1[d]);
    orc_ghec(A2->l[d], B2->l[d], K2[d], A2->a, B2->a, P2, q2, Q2[d], E2[d]);
  }
  /* g2_ee_prefactors */
  double xx = P1 * P2 + P1 * GAM + P2 * GAM;
  double c0 = (2.0 * pow(PI_T, 5.0 / 2.0)) / (xx * sqrt(P1 + P2));
  double qP = (P1 * P2 * GAM) / (P1 * P2 + P1 * GAM + P2 * GAM);
  double alpha = (P1 * P1 * P2 * P2) / (xx * (P1 + P2));
  double X[3];
  for (int d = 0; d < 3; d++) X[d] = Pm1[d] - Pm2[d];
  double R2 = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
  double expT = alpha * R2;
  double out = 0.0;
  for (int t1 = 0; t1 <= A1->l[0] + B1->l[0]; t1++)
  for (int u1 = 0; u1 <= A1->l[1] + B1->l[1]; u1++)
  for (int v1 = 0; v1 <= A1->l[2] + B1->l[2]; v1++)
  for (int t2 = 0; t2 <= A2->l[0] + B2->l[0]; t2++)
  for (int u2 = 0; u2 <= A2->l[1] + B2->l[1]; u2++)
  for (int v2 = 0; v2 <= A2->l[2] + B2->l[2]; v2++) {
    double c2 = pow(-1.0, (double)(t2 + u2 + v2));
    int Nt = t1 + t2, Nu = u1 + u2, Nv = v1 + v2;
    /* g2_dhermite_vee */
    double Dgf = 0.0;
    for (int xb1 = 0; xb1 <= Nt; xb1++) {
      int argx = Nt - xb1;
      double bx = cbinom(Nt, xb1);
      for (int yb1 = 0; yb1 <= Nu; yb1++) {
        int argy = Nu - yb1;
        double by = cbinom(Nu, yb1);
        for (int zb1 = 0; zb1 <= Nv; zb1++) {
          int argz = Nv - zb1;
          double bz = cbinom(Nv, zb1);
          double dgx = orc_gdel_x(argx, Pm1[0], qP, Pm2[0]);
          double dgy = orc_gdel_x(argy, Pm1[1], qP, Pm2[1]);
          double dgz = orc_gdel_x(argz, Pm1[2], qP, Pm2[2]);
          double dgxyz = dgx * dgy * dgz;
          int nLim = xb1 + yb1 + zb1;
          double dfxyz =
              orc_rtuv(xb1, yb1, zb1, nLim, expT, alpha, X[0], X[1], X[2]);
          Dgf = Dgf + bx * by * bz * dgxyz * dfxyz;
        }
      }
    }
    double ans = c0 * c2 * E1[0][t1] * E2[0][t2] * E1[1][u1] * E2[1][u2] *
                 E1[2][v1] * E2[2][v2] * Dgf;
    out = out + ans;
  }
  return out;
}

/* g2.f:200-234 pgi_hint0_1D (pi truncated to 3.141592650 there) */
static double pgi_hint0_1d(int it1, int it2, double p1, double p2,
                           double gamma, double P1, double P2) {
  const double PI = 3.141592650;
  double coe1 = ipow(-1.0, it2);
  double s = (p1 * p2) + (p1 * gamma) + (p2 * gamma);
  double q = (p1 * p2 * gamma) / s;
  double gd0 = orc_gdel_x(it1 + it2, P1, q, P2);
  return coe1 * sqrt(PI * PI / s) * gd0;
}

/* g2.f:915-1009 pgiovlap_1D: 1-D overlap of two particles coupled by the
 * geminal exp(-(gamA+gamB) x12^2) */
static double pgiovlap_1d(int I1, double alp1, double A1, int I2, double alp2,
                          double A2, int L1, double beta1, double B1, int L2,
                          double beta2, double B2, double gamA, double gamB) {
  double gamma = gamA + gamB;
  double p1, q1, P1, Q1, K1, ex1[24];
  double p2, q2, P2, Q2, K2, ex2[24];
  omega1d(I1, L1, alp1, beta1, A1, B1, &p1, &q1, &P1, &Q1, &K1, ex1);
  omega1d(I2, L2, alp2, beta2, A2, B2, &p2, &q2, &P2, &Q2, &K2, ex2);
  double xsum = 0.0;
  for (int it1 = 0; it1 <= I1 + L1; it1++)
    for (int it2 = 0; it2 <= I2 + L2; it2++) {
      double herm = pgi_hint0_1d(it1, it2, p1, p2, gamma, P1, P2);
      xsum = xsum + (ex1[it1] * ex2[it2] * herm);
    }
  return xsum;
}

/* g2.f:768-825 pgi_calcS2 */
static double pgi_calcs2(int I1, double alp1, double A1, int I2, double alp2,
                         double A2, int L1, double beta1, double B1, int L2,
                         double beta2, double B2, double gA, double gB) {
  double p1 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 + 1, beta1, B1, L2, beta2, B2, gA, gB);
  double p2 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2 + 1, beta2, B2, gA, gB);
  double p3 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2, beta2, B2, gA, gB);
  return p1 - p2 + ((B1 - B2) * p3);
}

/* g2.f:829-911 pgi_calcS3 */
static double pgi_calcs3(int I1, double alp1, double A1, int I2, double alp2,
                         double A2, int L1, double beta1, double B1, int L2,
                         double beta2, double B2, double gA, double gB) {
  double X12 = B1 - B2;
  double p1 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 + 2, beta1, B1, L2, beta2, B2, gA, gB);
  double p2 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2 + 2, beta2, B2, gA, gB);
  double p3 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2, beta2, B2, gA, gB);
  double p4 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 + 1, beta1, B1, L2 + 1, beta2, B2, gA, gB);
  double p5 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2 + 1, beta2, B2, gA, gB);
  double p6 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 + 1, beta1, B1, L2, beta2, B2, gA, gB);
  return p1 + p2 + (X12 * X12 * p3) - (2.0 * p4) - (2.0 * X12 * p5) +
         (2.0 * X12 * p6);
}

/* g2.f:655-765 pgi_Lapx1: 1-D Laplacian of particle 1 with the geminal */
static double pgi_lapx1(int I1, double alp1, double A1, int I2, double alp2,
                        double A2, int L1, double beta1, double B1, int L2,
                        double beta2, double B2, double gA, double gB) {
  double d1 = 0.0, c1, c2, p1 = 0.0, p2, p3, q1 = 0.0, q2, t1, t2;
  if (L1 - 1 >= 0) d1 = (double)(L1 * (L1 - 1));
  double d2 = -2.0 * beta1 * (double)((2 * L1) + 1);
  double d3 = 4.0 * beta1 * beta1;
  c1 = (double)L1;
  c2 = -2.0 * beta1;
  if (L1 - 2 >= 0)
    p1 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 - 2, beta1, B1, L2, beta2, B2, gA, gB);
  p2 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2, beta2, B2, gA, gB);
  p3 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1 + 2, beta1, B1, L2, beta2, B2, gA, gB);
  double W1 = (d1 * p1) + (d2 * p2) + (d3 * p3);
  if (L1 - 1 >= 0)
    q1 = pgi_calcs2(I1, alp1, A1, I2, alp2, A2, L1 - 1, beta1, B1, L2, beta2, B2, gA, gB);
  q2 = pgi_calcs2(I1, alp1, A1, I2, alp2, A2, L1 + 1, beta1, B1, L2, beta2, B2, gA, gB);
  double W2 = -2.0 * gB * ((c1 * q1) + (c2 * q2));
  t1 = pgiovlap_1d(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2, beta2, B2, gA, gB);
  t2 = pgi_calcs3(I1, alp1, A1, I2, alp2, A2, L1, beta1, B1, L2, beta2, B2, gA, gB);
  double W3 = (-2.0 * gB * t1) + (4.0 * gB * gB * t2);
  return W1 + (2.0 * W2) + W3;
}

/* g2.f:545-651 pgike1: kinetic energy of particle 1 (mass xmass1) between
 * geminal-correlated pairs; also returns the overlap Sx Sy Sz in *sval. */
double orc_pgike1(const orc_prim *A1, const orc_prim *A2, const orc_prim *B1,
                  const orc_prim *B2, double gamA, double gamB, double xmass1,
                  double *sval) {
  double S[3], T[3];
  for (int d = 0; d < 3; d++)
    S[d] = pgiovlap_1d(A1->l[d], A1->a, A1->c[d], A2->l[d], A2->a, A2->c[d],
                       B1->l[d], B1->a, B1->c[d], B2->l[d], B2->a, B2->c[d],
                       gamA, gamB);
  for (int d = 0; d < 3; d++) {
    double dd = pgi_lapx1(A1->l[d], A1->a, A1->c[d], A2->l[d], A2->a, A2->c[d],
                          B1->l[d], B1->a, B1->c[d], B2->l[d], B2->a, B2->c[d],
                          gamA, gamB);
    T[d] = -dd * 0.50 / xmass1;
  }
  if (sval) *sval = S[0] * S[1] * S[2];
  return (T[0] * S[1] * S[2]) + (S[0] * T[1] * S[2]) + (S[0] * S[1] * T[2]);
}
