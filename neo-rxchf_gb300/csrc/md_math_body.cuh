// md_math_body.cuh -- McMurchie-Davidson geminal integrals, written for the
// GPU and usable as plain C++ (every function is __host__ __device__).
// Included by md_math.cuh (real = double, namespace md: the FP64 path that
// matches the reference) and md_math32.cuh (real = float, namespace md32:
// the mixed-precision path).  In both instances the Boys function, the
// seeds (-alpha)^m F_m(T) and the final Hermite-Coulomb sum are FP64; md32's
// Gaussian-product set-up, Hermite and derivative tables and the Hermite
// folds are FP32.  The mixed gam_2 build re-evaluates every md32 result
// whose contribution is large with md (dynamic precision, k_md.cu).
//
// The reference evaluates each primitive integral as a 9- or 12-deep loop
// over Hermite indices, and inside every iteration re-derives the Boys'
// lemma constants, a triple-nested Leibniz expansion of the derivative of
// a product of Gaussians (DKG123 / DGK123, XC1_G3_MD.f:1876-2136) and one
// R_tuv recursion per Hermite triple (RTUV, XC1_int_tools.f:341-464).
// Here the same integrals are evaluated in factorised MD form:
//   * loop invariants (Gaussian products, Boys' lemma) once per call;
//   * the derivatives of prod_k exp(-xi_k u_k^2) at the product centres as
//     a table per Cartesian direction, from the exact three-term recurrence
//       D(n+e_i) = -g_i D(n) - sum_j H_ij n_j D(n-e_j),
//     (g = grad Q, H = Hessian Q, Q = sum_k xi_k u_k^2);
//   * per direction a vector W_d[n] that folds the Hermite coefficients,
//     the binomial split between the Gaussian part and the Coulomb part,
//     and the chain-rule powers of the Coulomb-centre coefficients;
//   * I = C * sum_{n,l,m} Wx Wy Wz R_nlm evaluated in factorised form
//     (contract_wr: the derivatives of F_0(alpha |R|^2) split per
//     direction, so no R_tuv table is built).
// The Boys function keeps the branch structure of the reference's XGAMMAF
// (common.f:317-348): for T > 20 the asymptotic form without the exp(-T)
// term and upward recursion, exactly as there; for T <= 20 the reference
// sums the series to a 1e-12 cutoff, and here F_M(T) comes from a
// pretabulated seven-term Taylor expansion (the standard grid method, e.g.
// Helgaker, Jorgensen, Olsen, Molecular Electronic-Structure Theory, 9.8.5)
// followed by the same downward recursion; the two agree to ~2.4e-12
// relative (the series' truncation; the table itself is exact to ~1e-15).
// Constants: pi truncated to 3.14159265358979 in the MD kernels
// (XC1_G3_MD.f, XC1_G4_MD.f, XC1_G2_MD.f), acos(-1) in the two-centre
// integrals (AC_Integrals vee.f, vec.f, ovlap.f, ke.f).
#include <math.h>

// Small helpers are force-inlined; the large integral routines are kept as
// separate device functions (NX_BIG) so the builder kernels compile in
// seconds instead of unrolling every call site.
#ifndef NX_HD
#if defined(__CUDACC__)
#define NX_HD __host__ __device__ __forceinline__
#define NX_BIG static __host__ __device__ __noinline__
#else
#define NX_HD inline
#define NX_BIG static inline
#endif
#endif

#ifndef NX_BOYS_RINV_DEFINED
#define NX_BOYS_RINV_DEFINED
namespace neoxc {
// 1/(2j + 1) for j = 0..31, the divisors of the Boys downward recursion
// F_j = (2T F_(j+1) + exp(-T)) / (2j + 1) (orders up to 22 are used).
constexpr int kBoysRinv = 32;
#define NX_BOYS_RINV_VALUES \
    1.0, 0.3333333333333333, 0.2, 0.14285714285714285, \
    0.1111111111111111, 0.09090909090909091, 0.07692307692307693, 0.06666666666666667, \
    0.058823529411764705, 0.05263157894736842, 0.047619047619047616, 0.043478260869565216, \
    0.04, 0.037037037037037035, 0.034482758620689655, 0.03225806451612903, \
    0.030303030303030304, 0.02857142857142857, 0.02702702702702703, 0.02564102564102564, \
    0.024390243902439025, 0.023255813953488372, 0.022222222222222223, 0.02127659574468085, \
    0.02040816326530612, 0.0196078431372549, 0.018867924528301886, 0.01818181818181818, \
    0.017543859649122806, 0.01694915254237288, 0.01639344262295082, 0.015873015873015872
#if defined(__CUDACC__)
static __device__ const double kBoysRinvDev[kBoysRinv] = {NX_BOYS_RINV_VALUES};
#endif
static const double kBoysRinvHost[kBoysRinv] = {NX_BOYS_RINV_VALUES};
#undef NX_BOYS_RINV_VALUES
NX_HD double boys_rinv(int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&kBoysRinvDev[j]);
#else
  return kBoysRinvHost[j];
#endif
}

// C(t,i) 2^(2i-t) = t! 2^(2i-t) / ((2i-t)! (t-i)!) for t, i <= 16 (zero
// outside ceil(t/2) <= i <= t): d^t/dX^t f(a X^2) = sum_i C(t,i) (2aX)^(2i-t)
// a^(t-i) f^(i)(a X^2), the coefficients of the factorised Hermite-Coulomb
// sum (contract_wr).
#define NX_HERMC_VALUES \
    1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 2, 4, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 12, 8, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 12, 48, 16, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 120, 160, 32, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 120, 720, 480, 64, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 1680, 3360, 1344, 128, 0, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 1680, 13440, 13440, 3584, 256, 0, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 0, 30240, 80640, 48384, 9216, 512, 0, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 0, 30240, 302400, 403200, 161280, 23040, 1024, 0, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 0, 0, 665280, 2217600, 1774080, 506880, 56320, 2048, 0, 0, 0, 0, 0, \
    0, 0, 0, 0, 0, 0, 665280, 7983360, 13305600, 7096320, 1520640, 135168, 4096, 0, 0, 0, 0, \
    0, 0, 0, 0, 0, 0, 0, 17297280, 69189120, 69189120, 26357760, 4392960, 319488, 8192, 0, 0, 0, \
    0, 0, 0, 0, 0, 0, 0, 17297280, 242161920, 484323840, 322882560, 92252160, 12300288, 745472, 16384, 0, 0, \
    0, 0, 0, 0, 0, 0, 0, 0, 518918400, 2421619200, 2905943040, 1383782400, 307507200, 33546240, 1720320, 32768, 0, \
    0, 0, 0, 0, 0, 0, 0, 0, 518918400, 8302694400, 19372953600, 15498362880, 5535129600, 984023040, 89456640, 3932160, 65536
#if defined(__CUDACC__)
static __device__ const double kHermCDev[17 * 17] = {NX_HERMC_VALUES};
#endif
static const double kHermCHost[17 * 17] = {NX_HERMC_VALUES};
// FP32 copy for the FP32 contractions (no double-to-float conversion in
// their inner loops; the values are exact in FP32 up to t = 11 and rounded
// to FP32 beyond)
#if defined(__CUDACC__)
static __device__ const float kHermC32Dev[17 * 17] = {NX_HERMC_VALUES};
#endif
static const float kHermC32Host[17 * 17] = {NX_HERMC_VALUES};
#undef NX_HERMC_VALUES
NX_HD double hermc(int t, int i) {
#if defined(__CUDA_ARCH__)
  return __ldg(&kHermCDev[t * 17 + i]);
#else
  return kHermCHost[t * 17 + i];
#endif
}
NX_HD float hermc32(int t, int i) {
#if defined(__CUDA_ARCH__)
  return __ldg(&kHermC32Dev[t * 17 + i]);
#else
  return kHermC32Host[t * 17 + i];
#endif
}

// F_m(T_g), m = 0..22, and exp(-T_g) on the grid T_g = g/16, g = 0..320
// (boys_table.inc, written by gen_boys_table.py from the integral definition
// at 40 digits).
constexpr int kBoysCols = 24, kBoysRows = 321;
#if defined(__CUDACC__)
static __device__ const double kBoysTabDev[kBoysRows * kBoysCols] = {
#include "boys_table.inc"
};
#endif
static const double kBoysTabHost[kBoysRows * kBoysCols] = {
#include "boys_table.inc"
};
NX_HD double boys_tab(int i) {
#if defined(__CUDA_ARCH__)
  return __ldg(&kBoysTabDev[i]);
#else
  return kBoysTabHost[i];
#endif
}

// F[0..M](T) in FP64 for both instances (M <= 16).  T > 20 (and NaN): the
// asymptotic branch of XGAMMAF (common.f:327-333), F_0 = sqrt(pi/T)/2 and
// F_L = F_(L-1) (L - 1/2) / T.  T <= 20: F_M from the Taylor expansion about
// the nearest grid point, F_M(T) = sum_{k<=6} F_(M+k)(T_g) d^k / k!,
// d = T_g - T (|d| <= 1/32, truncation < 1e-14 relative), exp(-T) likewise
// from exp(-T_g), then the downward recursion F_L = (2T F_(L+1) + exp(-T)) /
// (2L + 1) as in XGAMMAF (common.f:336-346).
NX_BIG void boys(int M, double T, double* F) {
  if (!(T <= 20.0)) {
    const double rT = 1.0 / T;
    double f = 0.88622692545275801365 / sqrt(T);
    F[0] = f;
    for (int L = 1; L <= M; L++) {
      f = f * (1.0 * L - 0.5) * rT;
      F[L] = f;
    }
    return;
  }
  int g = (int)(T * 16.0 + 0.5);
  g = g < 0 ? 0 : (g > kBoysRows - 1 ? kBoysRows - 1 : g);
  const double d = (double)g * 0.0625 - T;
  const int row = g * kBoysCols;
  // e_k = d^k / k!, shared by F_M and exp(d)
  double e[7];
  e[0] = 1.0;
  e[1] = d;
  e[2] = e[1] * d * 0.5;
  e[3] = e[2] * d * (1.0 / 3.0);
  e[4] = e[3] * d * 0.25;
  e[5] = e[4] * d * 0.2;
  e[6] = e[5] * d * (1.0 / 6.0);
  double f = boys_tab(row + M + 6) * e[6];
  for (int k = 5; k >= 0; k--) f = fma(boys_tab(row + M + k), e[k], f);
  F[M] = f;
  if (M == 0) return;
  const double ex =
      boys_tab(row + kBoysCols - 1) * (((((e[6] + e[5]) + e[4]) + e[3]) + e[2]) + e[1] + 1.0);
  const double t2 = 2.0 * T;
  for (int L = M - 1; L >= 0; L--) {
    f = fma(f, t2, ex) * boys_rinv(L);   // (2T F_(L+1) + e^-T) / (2L + 1)
    F[L] = f;
  }
}

// sum_{m=0..L} (-alpha)^m F_m(T) b(m) in FP64 (L <= 16), with boys()'s
// Boys function evaluated inside the sum and no F table: for T <= 20 the
// downward recursion from F_L runs alongside a Horner evaluation in
// (-alpha) (s <- s (-alpha) + F_m b(m)), F_L and exp(d) by Horner in d;
// for T > 20 (and NaN) the asymptotic upward recursion runs alongside the
// ascending sum.  b(m) is called once per m, from m = L down (T <= 20) or
// from m = 0 up.  Equal to boys() followed by the sum to rounding.  For an
// FP32 argument the grid index and the offset d = T_g - T are formed in
// FP32: T_g and T then lie within 1/32 of each other, so the subtraction is
// exact (Sterbenz) and gives the same d as in FP64 with fewer FP64
// instructions.
template <class TT, class BF>
NX_HD double boys_sum(int L, TT Tin, double alpha, BF&& b) {
  const double T = (double)Tin;
  const double ma = -alpha;
  if (!(T <= 20.0)) {
    const double rT = 1.0 / T;
    double f = 0.88622692545275801365 / sqrt(T);
    double s = f * (double)b(0), pw = 1.0;
    for (int m = 1; m <= L; m++) {
      f = f * ((double)m - 0.5) * rT;
      pw *= ma;
      s = fma(pw * f, (double)b(m), s);
    }
    return s;
  }
  int g;
  double d;
  if constexpr (sizeof(TT) == sizeof(float)) {
    const float tf = (float)Tin;
    g = (int)(tf * 16.0f + 0.5f);
    g = g < 0 ? 0 : (g > kBoysRows - 1 ? kBoysRows - 1 : g);
    d = (double)((float)g * 0.0625f - tf);
  } else {
    g = (int)(T * 16.0 + 0.5);
    g = g < 0 ? 0 : (g > kBoysRows - 1 ? kBoysRows - 1 : g);
    d = (double)g * 0.0625 - T;
  }
  const int row = g * kBoysCols;
  const double d2 = d * 0.5, d3 = d * (1.0 / 3.0), d4 = d * 0.25, d5 = d * 0.2,
               d6 = d * (1.0 / 6.0);
  // F_L(T) = sum_k F_(L+k)(T_g) d^k / k!
  double f = boys_tab(row + L + 6);
  f = fma(f, d6, boys_tab(row + L + 5));
  f = fma(f, d5, boys_tab(row + L + 4));
  f = fma(f, d4, boys_tab(row + L + 3));
  f = fma(f, d3, boys_tab(row + L + 2));
  f = fma(f, d2, boys_tab(row + L + 1));
  f = fma(f, d, boys_tab(row + L));
  double s = f * (double)b(L);
  if (L == 0) return s;
  double ep = 1.0 + d6;   // exp(d), the same seven terms
  ep = fma(ep, d5, 1.0);
  ep = fma(ep, d4, 1.0);
  ep = fma(ep, d3, 1.0);
  ep = fma(ep, d2, 1.0);
  ep = fma(ep, d, 1.0);
  const double ex = boys_tab(row + kBoysCols - 1) * ep;
  const double t2 = 2.0 * T;
  for (int m = L - 1; m >= 0; m--) {
    f = fma(f, t2, ex) * boys_rinv(m);
    s = fma(s, ma, f * (double)b(m));
  }
  return s;
}
}  // namespace neoxc
#endif

namespace neoxc {
namespace MD_NS {

using real = MD_REAL;
#define R_(x) static_cast<real>(x)

constexpr real kPiT = R_(3.14159265358979e+00);   // truncated (MD kernels)
constexpr real kPi = R_(3.14159265358979323846);   // acos(-1) (AC kernels)

// Supported primitives: Cartesian s, p, d (total l <= 2, hence l <= 2 in
// every direction).  The host rejects anything larger.
constexpr int LP = 2;              // max l per Cartesian direction / primitive
constexpr int LSUM = 2;            // max total l per primitive
constexpr int TMX = 2 * LP + 2;    // max t per particle (ket shifted by +2 in KE)
constexpr int TD = TMX + 1;
constexpr int LTOT = 4 * 2 * LSUM; // max total Hermite order (4 particles)

struct Prim {
  real a;
  real c[3];
  int l[3];
};

// ------------------------------------------------------- Hermite E^{ij}_t
// out[t], t = 0..i+j (XC1_int_tools.f:136-227 ghec; common.f hecod)
NX_BIG void hermite_e(int i, int j, real K, real a, real b, real p,
                     real q, real Qx, real* out) {
  real e[2 * TMX + 3], f[2 * TMX + 3];
  const real x1 = R_(1.0) / (R_(2.0) * p);
  real x2 = -q * Qx / a;
  for (int t = 0; t <= i + j + 1; t++) e[t] = R_(0.0);
  e[0] = K;
  for (int ii = 1; ii <= i; ii++) {          // E(ii,0,t) from E(ii-1,0,t)
    for (int t = 0; t <= ii + 1; t++) f[t] = R_(0.0);
    f[0] = x2 * e[0] + e[1];
    for (int t = 1; t <= ii; t++)
      f[t] = x1 * e[t - 1] + x2 * e[t] + (real)(t + 1) * e[t + 1];
    for (int t = 0; t <= ii + 1; t++) e[t] = f[t];
  }
  x2 = q * Qx / b;
  for (int jj = 1; jj <= j; jj++) {          // E(i,jj,t) from E(i,jj-1,t)
    for (int t = 0; t <= i + jj + 1; t++) f[t] = R_(0.0);
    f[0] = x2 * e[0] + e[1];
    for (int t = 1; t <= i + jj; t++)
      f[t] = x1 * e[t - 1] + x2 * e[t] + (real)(t + 1) * e[t + 1];
    for (int t = 0; t <= i + jj + 1; t++) e[t] = f[t];
  }
  for (int t = 0; t <= i + j; t++) out[t] = e[t];
}

// Gaussian product of one primitive pair (XC1_int_tools.f:2-46).
struct Pair {
  real p, q;
  real P[3], Q[3], K[3];
};
NX_HD void gauss_pair(const Prim& A, const Prim& B, Pair& r) {
  r.q = A.a * B.a / (A.a + B.a);
  r.p = A.a + B.a;
  for (int d = 0; d < 3; d++) {
    r.Q[d] = A.c[d] - B.c[d];
    r.K[d] = exp(-r.q * r.Q[d] * r.Q[d]);
    r.P[d] = (A.a * A.c[d] + B.a * B.c[d]) / (A.a + B.a);
  }
}

// ------------------------------------- derivatives of a Gaussian product
// D[n1][n2][n3] = d^n1/dx1 d^n2/dx2 d^n3/dx3 prod_k exp(-xi_k u_k^2),
// u_k = f_k x1 + g_k x2 + h_k x3, at x = X.  NK Gaussians, 3 variables.
struct GK3 {
  int nk;
  real xi[3], c[3][3];   // c[k] = (f,g,h)
};
NX_BIG void dgauss3(const GK3& g, const real* X, int N1, int N2, int N3,
                   real* D /* [TD][TD][TD] */) {
  if ((N1 | N2 | N3) == 0) {   // s shells: the base value only
    real expo = R_(0.0);
    for (int k = 0; k < g.nk; k++) {
      const real u = g.c[k][0] * X[0] + g.c[k][1] * X[1] + g.c[k][2] * X[2];
      expo -= g.xi[k] * u * u;
    }
    D[0] = exp(expo);
    return;
  }
  real grad[3] = {0, 0, 0}, H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  real expo = R_(0.0);   // prod_k exp(-xi_k u_k^2) as one exponential
  for (int k = 0; k < g.nk; k++) {
    real u = g.c[k][0] * X[0] + g.c[k][1] * X[1] + g.c[k][2] * X[2];
    expo -= g.xi[k] * u * u;
    for (int i = 0; i < 3; i++) {
      grad[i] += R_(2.0) * g.xi[k] * u * g.c[k][i];
      for (int j = 0; j < 3; j++) H[i][j] += R_(2.0) * g.xi[k] * g.c[k][i] * g.c[k][j];
    }
  }
  const real base = exp(expo);
#define D3(a, b, c) D[((a) * (N2 + 1) + (b)) * (N3 + 1) + (c)]
  for (int n1 = 0; n1 <= N1; n1++)
    for (int n2 = 0; n2 <= N2; n2++)
      for (int n3 = 0; n3 <= N3; n3++) {
        if (n1 == 0 && n2 == 0 && n3 == 0) { D3(0, 0, 0) = base; continue; }
        int m[3] = {n1, n2, n3};
        int i = n1 > 0 ? 0 : (n2 > 0 ? 1 : 2);
        m[i] -= 1;                                   // n = m + e_i
        real v = -grad[i] * D3(m[0], m[1], m[2]);
        for (int j = 0; j < 3; j++)
          if (m[j] > 0) {
            int r[3] = {m[0], m[1], m[2]};
            r[j] -= 1;
            v -= H[i][j] * (real)m[j] * D3(r[0], r[1], r[2]);
          }
        D3(n1, n2, n3) = v;
      }
#undef D3
}

struct GK4 {
  int nk;
  real xi[3], c[3][4];   // c[k] = (e,f,g,h)
};
// D[n1][n2][n3][n4], extents T4D each
constexpr int T4D = 2 * LP + 1;
NX_BIG void dgauss4(const GK4& g, const real* X, const int* N, real* D) {
  if ((N[0] | N[1] | N[2] | N[3]) == 0) {   // s shells: the base value only
    real expo = R_(0.0);
    for (int k = 0; k < g.nk; k++) {
      const real u = g.c[k][0] * X[0] + g.c[k][1] * X[1] + g.c[k][2] * X[2] +
                     g.c[k][3] * X[3];
      expo -= g.xi[k] * u * u;
    }
    D[0] = exp(expo);
    return;
  }
  real grad[4] = {0, 0, 0, 0}, H[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) H[i][j] = R_(0.0);
  real expo = R_(0.0);   // prod_k exp(-xi_k u_k^2) as one exponential
  for (int k = 0; k < g.nk; k++) {
    real u = g.c[k][0] * X[0] + g.c[k][1] * X[1] + g.c[k][2] * X[2] +
               g.c[k][3] * X[3];
    expo -= g.xi[k] * u * u;
    for (int i = 0; i < 4; i++) {
      grad[i] += R_(2.0) * g.xi[k] * u * g.c[k][i];
      for (int j = 0; j < 4; j++) H[i][j] += R_(2.0) * g.xi[k] * g.c[k][i] * g.c[k][j];
    }
  }
  const real base = exp(expo);
#define D4(a, b, c, e) D[(((a) * T4D + (b)) * T4D + (c)) * T4D + (e)]
  for (int n1 = 0; n1 <= N[0]; n1++)
    for (int n2 = 0; n2 <= N[1]; n2++)
      for (int n3 = 0; n3 <= N[2]; n3++)
        for (int n4 = 0; n4 <= N[3]; n4++) {
          if (n1 + n2 + n3 + n4 == 0) { D4(0, 0, 0, 0) = base; continue; }
          int m[4] = {n1, n2, n3, n4};
          int i = n1 > 0 ? 0 : (n2 > 0 ? 1 : (n3 > 0 ? 2 : 3));
          m[i] -= 1;
          real v = -grad[i] * D4(m[0], m[1], m[2], m[3]);
          for (int j = 0; j < 4; j++)
            if (m[j] > 0) {
              int r[4] = {m[0], m[1], m[2], m[3]};
              r[j] -= 1;
              v -= H[i][j] * (real)m[j] * D4(r[0], r[1], r[2], r[3]);
            }
          D4(n1, n2, n3, n4) = v;
        }
#undef D4
}

// ------------------------------------------------------------- R_tuv
NX_HD int tet_size(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
NX_HD int tet(int t, int u, int v) {
  int n = t + u + v;               // entries with t+u+v < n precede
  int k = u + v;                   // within shell n: order by (u+v), then v
  return n * (n + 1) * (n + 2) / 6 + k * (k + 1) / 2 + v;
}
NX_HD real binom(int n, int k) {
  real r = R_(1.0);
  for (int i = 1; i <= k; i++) r = r * (real)(n - k + i) / (real)i;
  return r;
}

// ======================================================================
// 3-particle kernels (XC1_G3_MD.f): Boys' lemma on particle 3.
// gam[6] = {A12, A13, A23, B12, B13, B23}.
struct G3 {
  Prim A[3], B[3];
  Pair pr[3];
  real gam12, gam13, gam23, xsum;
  real C1, C2, S1, S2, Sm1[3], Sm2[3];
  GK3 gk;
  int T[3][3];                 // [particle][dim] max t incl. KE shift
  real D[3][TD * TD * TD];   // per dimension, compact [T[0]+1][T[1]+1][T[2]+1]
};

// pairs: the Gaussian products of (A[i], B[i]), which do not depend on the
// geminal exponents; callers that set up many geminal terms for the same
// primitives compute them once (g3_setup below computes them itself).
NX_BIG void g3_setup_pairs(G3& s, const Prim* A, const Prim* B,
                          const Pair* pairs, const real* gam, int ke_shift) {
  for (int i = 0; i < 3; i++) {
    s.A[i] = A[i];
    s.B[i] = B[i];
    s.pr[i] = pairs[i];
  }
  s.gam13 = gam[1] + gam[4];
  s.gam23 = gam[2] + gam[5];
  const real P1 = s.pr[0].p, P2 = s.pr[1].p, P3 = s.pr[2].p;
  s.xsum = P3 + s.gam13 + s.gam23;
  s.C1 = (P3 * s.gam13) / s.xsum;
  s.C2 = (P3 * s.gam23) / s.xsum;
  const real C12 = (s.gam13 * s.gam23) / s.xsum;
  s.gam12 = (gam[0] + gam[3]) + C12;
  s.S1 = P1 + s.C1;
  s.S2 = P2 + s.C2;
  for (int d = 0; d < 3; d++) {
    s.Sm1[d] = (P1 * s.pr[0].P[d] + s.C1 * s.pr[2].P[d]) / (P1 + s.C1);
    s.Sm2[d] = (P2 * s.pr[1].P[d] + s.C2 * s.pr[2].P[d]) / (P2 + s.C2);
  }
  const real c1 = s.C1, c2 = s.C2, s1 = s.S1, s2 = s.S2, g12 = s.gam12;
  s.gk.nk = 3;
  s.gk.xi[0] = (P1 * c1) / (P1 + c1);
  s.gk.c[0][0] = R_(1.0); s.gk.c[0][1] = R_(0.0); s.gk.c[0][2] = -R_(1.0);
  s.gk.xi[1] = (P2 * c2) / (P2 + c2);
  s.gk.c[1][0] = R_(0.0); s.gk.c[1][1] = R_(1.0); s.gk.c[1][2] = -R_(1.0);
  s.gk.xi[2] = (s1 * s2 * g12) / (s1 * s2 + s1 * g12 + s2 * g12);
  s.gk.c[2][0] = P1 / (P1 + c1);
  s.gk.c[2][1] = -P2 / (P2 + c2);
  s.gk.c[2][2] = (c1 / (P1 + c1)) - (c2 / (P2 + c2));
  for (int d = 0; d < 3; d++) {
    for (int i = 0; i < 3; i++) s.T[i][d] = A[i].l[d] + B[i].l[d];
    s.T[0][d] += ke_shift;
    s.T[2][d] += ke_shift;
    const real X[3] = {s.pr[0].P[d], s.pr[1].P[d], s.pr[2].P[d]};
    dgauss3(s.gk, X, s.T[0][d], s.T[1][d], s.T[2][d], s.D[d]);
  }
}

NX_BIG void g3_setup(G3& s, const Prim* A, const Prim* B, const real* gam,
                    int ke_shift) {
  Pair pr[3];
  for (int i = 0; i < 3; i++) gauss_pair(A[i], B[i], pr[i]);
  g3_setup_pairs(s, A, B, pr, gam, ke_shift);
}

// 1-D overlap factor with ket momenta (L1, L3) of particles 1 and 3
// (G3_MD_xggs1D, XC1_G3_MD.f:90-293), without the C0*C3 prefactor.
NX_BIG real g3_ovl1d(const G3& s, int d, int L1, int L3) {
  const Pair* pr = s.pr;
  real E1[2 * TMX + 1], E2[2 * TMX + 1], E3[2 * TMX + 1];
  const int I1 = s.A[0].l[d], I2 = s.A[1].l[d], I3 = s.A[2].l[d];
  const int L2 = s.B[1].l[d];
  hermite_e(I1, L1, pr[0].K[d], s.A[0].a, s.B[0].a, pr[0].p, pr[0].q, pr[0].Q[d], E1);
  hermite_e(I2, L2, pr[1].K[d], s.A[1].a, s.B[1].a, pr[1].p, pr[1].q, pr[1].Q[d], E2);
  hermite_e(I3, L3, pr[2].K[d], s.A[2].a, s.B[2].a, pr[2].p, pr[2].q, pr[2].Q[d], E3);
  const int X1 = s.T[1][d] + 1, X2 = s.T[2][d] + 1;   // D's compact extents
  real acc = R_(0.0);
  for (int t1 = 0; t1 <= I1 + L1; t1++)
    for (int t2 = 0; t2 <= I2 + L2; t2++)
      for (int t3 = 0; t3 <= I3 + L3; t3++)
        acc += E1[t1] * E2[t2] * E3[t3] * s.D[d][(t1 * X1 + t2) * X2 + t3];
  return acc;
}

NX_HD real g3_ovl_pref1d(const G3& s) {
  const real tv1 = s.S1 * s.S2 + s.S1 * s.gam12 + s.S2 * s.gam12;
  return sqrt(kPiT / s.xsum) * sqrt(kPiT * kPiT / tv1);
}

// G3_MD_xggs (XC1_G3_MD.f:2-87)
NX_BIG real g3_overlap(const G3& s) {
  const real pf = g3_ovl_pref1d(s);
  real r = R_(1.0);
  for (int d = 0; d < 3; d++) r *= pf * g3_ovl1d(s, d, s.B[0].l[d], s.B[2].l[d]);
  return r;
}

// G3_MD_KE (XC1_G3_MD.f:2546-2677) with G3_MD_T1d (:2680-2866); needs a
// setup with ke_shift = 2.  Kinetic operator on particle 1; the ket
// geminal coupling particle 1 is gamB13 (gam[4]).
NX_BIG real g3_ke(const G3& s, real gB13, real xmass) {
  const real pf = g3_ovl_pref1d(s);
  real S[3], Tk[3];
  for (int d = 0; d < 3; d++) {
    const int L1 = s.B[0].l[d], L3 = s.B[2].l[d];
    const real b1 = s.B[0].a, XB = s.B[0].c[d] - s.B[2].c[d];
    real x[10];
    for (int i = 0; i < 10; i++) x[i] = R_(0.0);
    if (L1 > 0) {
      if (L1 > 1) x[1] = pf * g3_ovl1d(s, d, L1 - 2, L3);
      x[2] = pf * g3_ovl1d(s, d, L1 - 1, L3);
      x[3] = pf * g3_ovl1d(s, d, L1 - 1, L3 + 1);
    }
    x[4] = pf * g3_ovl1d(s, d, L1, L3);
    x[5] = pf * g3_ovl1d(s, d, L1, L3 + 1);
    x[6] = pf * g3_ovl1d(s, d, L1, L3 + 2);
    x[7] = pf * g3_ovl1d(s, d, L1 + 1, L3);
    x[8] = pf * g3_ovl1d(s, d, L1 + 1, L3 + 1);
    x[9] = pf * g3_ovl1d(s, d, L1 + 2, L3);
    const real g = gB13, dl = (real)L1;
    real t = (real)(L1 * (L1 - 1)) * x[1] - R_(4.0) * g * XB * dl * x[2] +
               R_(4.0) * g * dl * x[3] - R_(2.0) * b1 * (R_(2.0) * dl + R_(1.0)) * x[4] -
               R_(4.0) * g * dl * x[4] + R_(4.0) * g * g * XB * XB * x[4] -
               R_(2.0) * g * x[4] - R_(8.0) * g * g * XB * x[5] + R_(4.0) * g * g * x[6] +
               R_(8.0) * b1 * g * XB * x[7] + R_(8.0) * g * g * XB * x[7] -
               R_(8.0) * b1 * g * x[8] - R_(8.0) * g * g * x[8] +
               (R_(4.0) * b1 * b1 + R_(8.0) * b1 * g + R_(4.0) * g * g) * x[9];
    S[d] = x[4];
    Tk[d] = t;
  }
  real r = Tk[0] * S[1] * S[2] + S[0] * Tk[1] * S[2] + S[0] * S[1] * Tk[2];
  return -R_(0.5) * r / xmass;
}

// W_d[n] for the 3-particle Coulomb kernels.
NX_BIG void g3_wvec(const G3& s, int d, real bf, real bg, real bh,
                   real* W, int* nmax) {
  const Pair* pr = s.pr;
  real E[3][2 * TMX + 1];
  int tl[3];
  for (int i = 0; i < 3; i++) {
    tl[i] = s.A[i].l[d] + s.B[i].l[d];
    hermite_e(s.A[i].l[d], s.B[i].l[d], pr[i].K[d], s.A[i].a, s.B[i].a,
              pr[i].p, pr[i].q, pr[i].Q[d], E[i]);
  }
  const int N = tl[0] + tl[1] + tl[2];
  const int X1 = s.T[1][d] + 1, X2 = s.T[2][d] + 1;   // D's compact extents
  for (int n = 0; n <= N; n++) W[n] = R_(0.0);
  real pf[TD], pg[TD], ph[TD];
  pf[0] = pg[0] = ph[0] = R_(1.0);
  for (int k = 1; k < TD; k++) {
    pf[k] = pf[k - 1] * bf;
    pg[k] = pg[k - 1] * bg;
    ph[k] = ph[k - 1] * bh;
  }
  for (int t1 = 0; t1 <= tl[0]; t1++)
    for (int t2 = 0; t2 <= tl[1]; t2++)
      for (int t3 = 0; t3 <= tl[2]; t3++) {
        const real e = E[0][t1] * E[1][t2] * E[2][t3];
        for (int x1 = 0; x1 <= t1; x1++)
          for (int x2 = 0; x2 <= t2; x2++)
            for (int x3 = 0; x3 <= t3; x3++) {
              real c = binom(t1, x1) * binom(t2, x2) * binom(t3, x3) *
                         pf[x1] * pg[x2] * ph[x3] *
                         s.D[d][((t1 - x1) * X1 + (t2 - x2)) * X2 + (t3 - x3)];
              W[x1 + x2 + x3] += e * c;
            }
      }
  *nmax = N;
}

// I = sum_{t,u,v} Wx[t] Wy[u] Wz[v] R_tuv(alpha, R3) in factorised form:
// R_tuv = d^t/dX^t d^u/dY^u d^v/dZ^v F_0(alpha |R|^2), and because F_0's
// argument is additive over directions the derivatives factorise,
//   I = sum_m (-alpha)^m F_m(T) sum_{i+j+k=m} A_x[i] A_y[j] A_z[k],
//   A_d[i] = sum_t W_d[t] C(t,i) 2^(2i-t) R_d^(2i-t)  (hermc),
// O(L^2) work and no R_tuv table; equal to the MD recursion of the
// reference's RTUV (XC1_int_tools.f:341-464) to rounding.  The seeds
// (-alpha)^m F_m(T) and the final sum are FP64 in both instances.
NX_BIG real contract_wr(const real* Wx, int nx, const real* Wy, int ny,
                        const real* Wz, int nz, real T, real alpha,
                        const real* R3) {
  constexpr bool k32 = sizeof(real) == sizeof(float);
  const real* W[3] = {Wx, Wy, Wz};
  const int n[3] = {nx, ny, nz};
  real A[3][LTOT + 1];
  for (int d = 0; d < 3; d++) {
    real xp[LTOT + 1];
    xp[0] = R_(1.0);
    for (int k = 1; k <= n[d]; k++) xp[k] = xp[k - 1] * R3[d];
    for (int i = 0; i <= n[d]; i++) A[d][i] = R_(0.0);
    for (int t = 0; t <= n[d]; t++)
      for (int i = (t + 1) / 2; i <= t; i++)
        A[d][i] += W[d][t] * (k32 ? (real)hermc32(t, i) : (real)hermc(t, i)) * xp[2 * i - t];
  }
  real Bxy[2 * LTOT + 1];
  for (int m = 0; m <= nx + ny; m++) Bxy[m] = R_(0.0);
  for (int i = 0; i <= nx; i++)
    for (int j = 0; j <= ny; j++) Bxy[i + j] += A[0][i] * A[1][j];
  const int L = nx + ny + nz;
  const double s = boys_sum(L, T, (double)alpha, [&](int m) {
    real bm = R_(0.0);
    const int lo = m - nz > 0 ? m - nz : 0, hi = m < nx + ny ? m : nx + ny;
    for (int i = lo; i <= hi; i++) bm += Bxy[i] * A[2][m - i];
    return bm;
  });
  return (real)s;
}

// G3_MD_xgVxCg (XC1_G3_MD.f:711-1088): attraction of particle 1 to C
// Coulomb factor of a G3 kernel, C0 C3 sum W_x W_y W_z R_tuv: for s shells
// every Hermite expansion is E_0 = K, so W_d = K1 K2 K3 D_d(0,0,0) and only
// R_000 = F_0(T) enters -- the same products in the same order as the
// general contraction, without its tables.
NX_BIG real g3_coulomb(const G3& s, real C0, real C3, real bf, real bg, real bh, real T,
                       real alpha, const real* Rv) {
  bool all_s = true;
  for (int i = 0; i < 3; i++)
    for (int d = 0; d < 3; d++) all_s = all_s && s.T[i][d] == 0;
  if (all_s) {
    real w = R_(1.0);
    for (int d = 0; d < 3; d++) {
      const real wd = ((s.pr[0].K[d] * s.pr[1].K[d]) * s.pr[2].K[d]) * s.D[d][0];
      w = d == 0 ? wd : w * wd;
    }
    return C0 * C3 * (w * (real)boys_sum(0, T, 0.0, [](int) { return 1.0; }));
  }
  real W[3][LTOT + 1];
  int n[3];
  for (int d = 0; d < 3; d++) g3_wvec(s, d, bf, bg, bh, W[d], &n[d]);
  return C0 * C3 * contract_wr(W[0], n[0], W[1], n[1], W[2], n[2], T, alpha, Rv);
}

NX_BIG real g3_vxc(const G3& s, const real* C) {
  const real s1 = s.S1, s2 = s.S2, g = s.gam12;
  const real p1 = s.pr[0].p, p2 = s.pr[1].p, c1 = s.C1, c2 = s.C2;
  const real tv1 = s2 + g;
  const real tv2 = s1 * s2 + s1 * g + s2 * g;
  const real tv3 = tv2 / tv1;
  const real x = kPiT / tv1;
  const real C3 = sqrt(x * x * x) * (R_(2.0) * kPiT / tv3);
  const real C0 = pow(kPiT / s.xsum, R_(1.5));
  const real bf = (s1 * s2 + s1 * g) / tv2 * (p1 / (p1 + c1));
  const real bg = (s2 * g) / tv2 * (p2 / (p2 + c2));
  const real bh = (s1 * s2 + s1 * g) / tv2 * (c1 / (p1 + c1)) +
                    (s2 * g) / tv2 * (c2 / (p2 + c2));
  real Rv[3], R2 = R_(0.0);
  for (int d = 0; d < 3; d++) {
    real sm = ((s1 * s2 + s1 * g) / tv2) * s.Sm1[d] + ((s2 * g) / tv2) * s.Sm2[d];
    Rv[d] = sm - C[d];
    R2 += Rv[d] * Rv[d];
  }
  const real alpha = tv3, T = alpha * R2;
  return g3_coulomb(s, C0, C3, bf, bg, bh, T, alpha, Rv);
}

// G3_MD_xgVxCg for nat classical centres at once (cat: 3 x nat bohr):
// the Hermite vectors W_d do not depend on the attracting centre, so they
// are folded once and only the Coulomb sum runs per centre; out[ia] equals
// g3_vxc(s, C_ia).
NX_BIG void g3_vxc_multi(const G3& s, int nat, const double* cat, real* out) {
  const real s1 = s.S1, s2 = s.S2, g = s.gam12;
  const real p1 = s.pr[0].p, p2 = s.pr[1].p, c1 = s.C1, c2 = s.C2;
  const real tv1 = s2 + g;
  const real tv2 = s1 * s2 + s1 * g + s2 * g;
  const real tv3 = tv2 / tv1;
  const real x = kPiT / tv1;
  const real C3 = sqrt(x * x * x) * (R_(2.0) * kPiT / tv3);
  const real C0 = pow(kPiT / s.xsum, R_(1.5));
  const real bf = (s1 * s2 + s1 * g) / tv2 * (p1 / (p1 + c1));
  const real bg = (s2 * g) / tv2 * (p2 / (p2 + c2));
  const real bh = (s1 * s2 + s1 * g) / tv2 * (c1 / (p1 + c1)) +
                    (s2 * g) / tv2 * (c2 / (p2 + c2));
  const real alpha = tv3;
  bool all_s = true;
  for (int i = 0; i < 3; i++)
    for (int d = 0; d < 3; d++) all_s = all_s && s.T[i][d] == 0;
  real W[3][LTOT + 1];
  int n[3] = {0, 0, 0};
  real w = R_(1.0);
  if (all_s) {
    for (int d = 0; d < 3; d++) {
      const real wd = ((s.pr[0].K[d] * s.pr[1].K[d]) * s.pr[2].K[d]) * s.D[d][0];
      w = d == 0 ? wd : w * wd;
    }
  } else {
    for (int d = 0; d < 3; d++) g3_wvec(s, d, bf, bg, bh, W[d], &n[d]);
  }
  for (int ia = 0; ia < nat; ia++) {
    real Rv[3], R2 = R_(0.0);
    for (int d = 0; d < 3; d++) {
      real sm = ((s1 * s2 + s1 * g) / tv2) * s.Sm1[d] + ((s2 * g) / tv2) * s.Sm2[d];
      Rv[d] = sm - (real)cat[3 * ia + d];
      R2 += Rv[d] * Rv[d];
    }
    const real T = alpha * R2;
    if (all_s) {
      out[ia] = C0 * C3 * (w * (real)boys_sum(0, T, 0.0, [](int) { return 1.0; }));
    } else {
      out[ia] = C0 * C3 * contract_wr(W[0], n[0], W[1], n[1], W[2], n[2], T, alpha, Rv);
    }
  }
}

// G3_MD_xgVeeg (XC1_G3_MD.f:1376-1675): 1/|r1 - r2|
NX_BIG real g3_vee(const G3& s) {
  const real s1 = s.S1, s2 = s.S2, g = s.gam12;
  const real tv2 = s1 * s2 + s1 * g + s2 * g;
  const real tv1 = tv2 * sqrt(s1 + s2);
  const real tv3 = tv2 * (s1 + s2);
  const real C3 = (R_(2.0) * sqrt(kPiT * kPiT * kPiT * kPiT * kPiT)) / tv1;
  const real C0 = pow(kPiT / s.xsum, R_(1.5));
  const real alpha = (s1 * s1 * s2 * s2) / tv3;
  real Rv[3], R2 = R_(0.0);
  for (int d = 0; d < 3; d++) {
    Rv[d] = s.gk.c[2][0] * s.pr[0].P[d] + s.gk.c[2][1] * s.pr[1].P[d] +
            s.gk.c[2][2] * s.pr[2].P[d];
    real dd = s.Sm1[d] - s.Sm2[d];
    R2 += dd * dd;
  }
  const real T = alpha * R2;
  return g3_coulomb(s, C0, C3, s.gk.c[2][0], s.gk.c[2][1], s.gk.c[2][2], T, alpha, Rv);
}

// ======================================================================
// G2_MD_xggs (XC1_G2_MD.f:3-187): particles (A1,B1), (A2,B2), geminal
// exp(-(gamma1+gamma2) r12^2).
NX_BIG real g2_xggs(const Prim& A1, const Prim& A2, const Prim& B1,
                     const Prim& B2, real gamma1, real gamma2) {
  const real G = gamma1 + gamma2;
  Pair p1, p2;
  gauss_pair(A1, B1, p1);
  gauss_pair(A2, B2, p2);
  const real P1 = p1.p, P2 = p2.p;
  const real qP = (P1 * P2 * G) / (P1 * P2 + P1 * G + P2 * G);
  const real c1 = pow(kPiT * kPiT / (P1 * P2 + P1 * G + P2 * G), R_(1.5));
  real r = c1;
  for (int d = 0; d < 3; d++) {
    real E1[2 * LP + 1], E2[2 * LP + 1];
    const int l1 = A1.l[d] + B1.l[d], l2 = A2.l[d] + B2.l[d];
    hermite_e(A1.l[d], B1.l[d], p1.K[d], A1.a, B1.a, P1, p1.q, p1.Q[d], E1);
    hermite_e(A2.l[d], B2.l[d], p2.K[d], A2.a, B2.a, P2, p2.q, p2.Q[d], E2);
    // g[N] = d^N/dx^N exp(-qP (x - Pm2)^2) at x = Pm1
    real gd[4 * LP + 1];
    const real u = p1.P[d] - p2.P[d];
    gd[0] = exp(-qP * u * u);
    for (int N = 1; N <= l1 + l2; N++)
      gd[N] = -R_(2.0) * qP * u * gd[N - 1] - (N > 1 ? R_(2.0) * qP * (N - 1) * gd[N - 2] : R_(0.0));
    real acc = R_(0.0);
    for (int t1 = 0; t1 <= l1; t1++)
      for (int t2 = 0; t2 <= l2; t2++)
        acc += E1[t1] * E2[t2] * ((t2 & 1) ? -R_(1.0) : R_(1.0)) * gd[t1 + t2];
    r *= acc;
  }
  return r;
}

// ======================================================================
// 4-particle kernels (XC1_G4_MD.f)
struct G4 {
  Prim A[4], B[4];
  Pair pr[4];
};

NX_HD void g4_pairs(G4& s, const Prim* A, const Prim* B) {
  for (int i = 0; i < 4; i++) {
    s.A[i] = A[i];
    s.B[i] = B[i];
    gauss_pair(A[i], B[i], s.pr[i]);
  }
}

NX_BIG real g4_coulomb(const G4& s, const GK4& gk, const real* cof,
                        real pref, real T, real alpha,
                        const real* Rv) {
  bool all_s = true;
  for (int i = 0; i < 4; i++)
    for (int d = 0; d < 3; d++) all_s = all_s && (s.A[i].l[d] + s.B[i].l[d] == 0);
  if (all_s) {
    // s shells: every Hermite expansion is E_0 = K, the derivative table is
    // its base value and the Coulomb factor is R_000 = F_0(T)
    real w = R_(1.0), expo = R_(0.0);
    for (int d = 0; d < 3; d++) {
      for (int k = 0; k < gk.nk; k++) {
        const real u = gk.c[k][0] * s.pr[0].P[d] + gk.c[k][1] * s.pr[1].P[d] +
                       gk.c[k][2] * s.pr[2].P[d] + gk.c[k][3] * s.pr[3].P[d];
        expo -= gk.xi[k] * u * u;
      }
      w *= s.pr[0].K[d] * s.pr[1].K[d] * s.pr[2].K[d] * s.pr[3].K[d];
    }
    w *= exp(expo);
    return pref * (w * (real)boys_sum(0, T, 0.0, [](int) { return 1.0; }));
  }
  real W[3][LTOT + 1];
  int nmax[3];
  real D[T4D * T4D * T4D * T4D];
  for (int d = 0; d < 3; d++) {
    real E[4][2 * LP + 1];
    int tl[4];
    real X[4];
    for (int i = 0; i < 4; i++) {
      tl[i] = s.A[i].l[d] + s.B[i].l[d];
      X[i] = s.pr[i].P[d];
      hermite_e(s.A[i].l[d], s.B[i].l[d], s.pr[i].K[d], s.A[i].a, s.B[i].a,
                s.pr[i].p, s.pr[i].q, s.pr[i].Q[d], E[i]);
    }
    dgauss4(gk, X, tl, D);
    const int N = tl[0] + tl[1] + tl[2] + tl[3];
    for (int n = 0; n <= N; n++) W[d][n] = R_(0.0);
    real pw[4][2 * LP + 1];
    for (int i = 0; i < 4; i++) {
      pw[i][0] = R_(1.0);
      for (int k = 1; k <= 2 * LP; k++) pw[i][k] = pw[i][k - 1] * cof[i];
    }
    for (int t1 = 0; t1 <= tl[0]; t1++)
    for (int t2 = 0; t2 <= tl[1]; t2++)
    for (int t3 = 0; t3 <= tl[2]; t3++)
    for (int t4 = 0; t4 <= tl[3]; t4++) {
      const real e = E[0][t1] * E[1][t2] * E[2][t3] * E[3][t4];
      for (int x1 = 0; x1 <= t1; x1++)
      for (int x2 = 0; x2 <= t2; x2++)
      for (int x3 = 0; x3 <= t3; x3++)
      for (int x4 = 0; x4 <= t4; x4++) {
        real c = binom(t1, x1) * binom(t2, x2) * binom(t3, x3) *
                   binom(t4, x4) * pw[0][x1] * pw[1][x2] * pw[2][x3] *
                   pw[3][x4] *
                   D[(((t1 - x1) * T4D + (t2 - x2)) * T4D + (t3 - x3)) * T4D + (t4 - x4)];
        W[d][x1 + x2 + x3 + x4] += e * c;
      }
    }
    nmax[d] = N;
  }
  return pref * contract_wr(W[0], nmax[0], W[1], nmax[1], W[2], nmax[2], T,
                            alpha, Rv);
}

// G4_MD_xgVeeg (XC1_G4_MD.f:796-1125): geminals (1,4) bra, (3,4) ket,
// Coulomb between particles 1 and 2.
NX_BIG real g4_vee(const G4& s, real gam14, real gam34) {
  const real P1 = s.pr[0].p, P2 = s.pr[1].p, P3 = s.pr[2].p, P4 = s.pr[3].p;
  const real xsum = P4 + gam14 + gam34;
  const real C0 = pow(kPiT / xsum, R_(1.5));
  const real C1 = (P4 * gam14) / xsum, C3 = (P4 * gam34) / xsum;
  const real C13 = (gam14 * gam34) / xsum;
  const real S1 = P1 + C1, S3 = P3 + C3;
  const real CB0 = (kPiT / (S3 + C13)) * sqrt(kPiT / (S3 + C13));
  const real CB1 = (S3 * C13) / (S3 + C13);
  const real W1 = S1 + CB1;
  real cof[4];
  cof[0] = P1 / (S1 + CB1);
  cof[1] = -R_(1.0);
  cof[2] = (CB1 / (S1 + CB1)) * (P3 / (P3 + C3));
  cof[3] = (C1 / (S1 + CB1)) + (CB1 / (S1 + CB1)) * (C3 / (P3 + C3));
  real Rv[3], R2 = R_(0.0);
  for (int d = 0; d < 3; d++) {
    Rv[d] = cof[0] * s.pr[0].P[d] + cof[1] * s.pr[1].P[d] +
            cof[2] * s.pr[2].P[d] + cof[3] * s.pr[3].P[d];
    R2 += Rv[d] * Rv[d];
  }
  const real C4 = (R_(2.0) * kPiT * kPiT * sqrt(kPiT)) / (W1 * P2 * sqrt(W1 + P2));
  const real alpha = (W1 * P2) / (W1 + P2);
  GK4 gk;
  gk.nk = 3;
  gk.xi[0] = P1 * C1 / (P1 + C1);
  gk.xi[1] = P3 * C3 / (P3 + C3);
  gk.xi[2] = S1 * CB1 / (S1 + CB1);
  const real c0[4] = {R_(1.0), R_(0.0), R_(0.0), -R_(1.0)}, cc1[4] = {R_(0.0), R_(0.0), R_(1.0), -R_(1.0)};
  const real cc2[4] = {P1 / (P1 + C1), R_(0.0), -P3 / (P3 + C3),
                         C1 / (P1 + C1) - C3 / (P3 + C3)};
  for (int i = 0; i < 4; i++) {
    gk.c[0][i] = c0[i];
    gk.c[1][i] = cc1[i];
    gk.c[2][i] = cc2[i];
  }
  return g4_coulomb(s, gk, cof, C0 * CB0 * C4, alpha * R2, alpha, Rv);
}

// G4_MD_xgVepg (XC1_G4_MD.f:1559-1978): geminals (1,4) bra, (2,4) ket,
// Coulomb between particles 3 and 4.
NX_BIG real g4_vep(const G4& s, real gam14, real gam24) {
  const real P1 = s.pr[0].p, P2 = s.pr[1].p, P3 = s.pr[2].p, P4 = s.pr[3].p;
  const real C0 = (kPiT / (P1 + gam14)) * sqrt(kPiT / (P1 + gam14));
  const real C1 = (P1 * gam14) / (P1 + gam14);
  const real S4 = C1 + P4;
  const real CB0 = (kPiT / (P2 + gam24)) * sqrt(kPiT / (P2 + gam24));
  const real CB1 = (P2 * gam24) / (P2 + gam24);
  const real Tx4 = S4 + CB1;
  const real xcof = (S4 + CB1) * (C1 + P4);
  real cof[4] = {S4 * C1 / xcof, CB1 / (S4 + CB1), -R_(1.0), S4 * P4 / xcof};
  real Rv[3], R2 = R_(0.0);
  for (int d = 0; d < 3; d++) {
    const real sm4 = (C1 * s.pr[0].P[d] + P4 * s.pr[3].P[d]) / (C1 + P4);
    const real tm4 = (S4 * sm4 + CB1 * s.pr[1].P[d]) / (S4 + CB1);
    Rv[d] = tm4 - s.pr[2].P[d];
    R2 += Rv[d] * Rv[d];
  }
  const real C4 = (R_(2.0) * kPiT * kPiT * sqrt(kPiT)) / (P3 * Tx4 * sqrt(P3 + Tx4));
  const real alpha = (P3 * Tx4) / (P3 + Tx4);
  GK4 gk;
  gk.nk = 2;
  gk.xi[0] = (P4 * C1) / (P4 + C1);
  gk.xi[1] = (S4 * CB1) / (S4 + CB1);
  const real c0[4] = {R_(1.0), R_(0.0), R_(0.0), -R_(1.0)};
  const real cc1[4] = {C1 / (C1 + P4), -R_(1.0), R_(0.0), P4 / (C1 + P4)};
  for (int i = 0; i < 4; i++) {
    gk.c[0][i] = c0[i];
    gk.c[1][i] = cc1[i];
    gk.c[2][i] = R_(0.0);
  }
  gk.xi[2] = R_(0.0);
  return g4_coulomb(s, gk, cof, C0 * CB0 * C4, alpha * R2, alpha, Rv);
}

// ======================================================================
// two-centre integrals (AC_Integrals): full-precision pi.
NX_BIG real ovl1d(int I, real a, real A, int L, real b, real B) {
  const real p = a + b, q = (a * b) / (a + b), Q = A - B;
  real E[2 * TMX + 1];
  hermite_e(I, L, exp(-q * Q * Q), a, b, p, q, Q, E);
  return E[0] * sqrt(kPi / p);
}

// gfke (ke.f:2-59) with Lapx1 (:62-120)
NX_BIG real gfke(const Prim& A, const Prim& B, real xmass) {
  real S[3], Tk[3];
  for (int d = 0; d < 3; d++) {
    const int I = A.l[d], L = B.l[d];
    S[d] = ovl1d(I, A.a, A.c[d], L, B.a, B.c[d]);
    real d1 = (L - 1 >= 0) ? (real)(L * (L - 1)) : R_(0.0);
    real d2 = -R_(2.0) * B.a * (real)(2 * L + 1);
    real d3 = R_(4.0) * B.a * B.a;
    real p1 = (L - 2 >= 0) ? ovl1d(I, A.a, A.c[d], L - 2, B.a, B.c[d]) : R_(0.0);
    real p3 = ovl1d(I, A.a, A.c[d], L + 2, B.a, B.c[d]);
    real w = (d1 * p1) + (d2 * S[d]) + (d3 * p3);
    Tk[d] = -w * R_(0.5) / xmass;
  }
  return Tk[0] * S[1] * S[2] + S[0] * Tk[1] * S[2] + S[0] * S[1] * Tk[2];
}

// gfvec (vec.f:2-94): positive-sign nuclear attraction to C
NX_BIG real gfvec(const Prim& A, const Prim& B, const real* C) {
  Pair pr;
  gauss_pair(A, B, pr);
  real E[3][2 * LP + 1];
  real PC[3], R2 = R_(0.0);
  for (int d = 0; d < 3; d++) {
    hermite_e(A.l[d], B.l[d], pr.K[d], A.a, B.a, pr.p, pr.q, pr.Q[d], E[d]);
    PC[d] = pr.P[d] - C[d];
    R2 += PC[d] * PC[d];
  }
  const int nx = A.l[0] + B.l[0], ny = A.l[1] + B.l[1], nz = A.l[2] + B.l[2];
  return (R_(2.0) * kPi / pr.p) *
         contract_wr(E[0], nx, E[1], ny, E[2], nz, pr.p * R2, pr.p, PC);
}

// gfvee (vee.f:3-78): (A1 B1 | A2 B2) electron repulsion
NX_BIG real gfvee(const Prim& A1, const Prim& A2, const Prim& B1,
                   const Prim& B2) {
  Pair p1, p2;
  gauss_pair(A1, B1, p1);
  gauss_pair(A2, B2, p2);
  const real coe2 = (R_(2.0) * sqrt(kPi * kPi * kPi * kPi * kPi)) /
                      ((p1.p * p2.p) * sqrt(p1.p + p2.p));
  const real beta = ((p1.p * p2.p) * (p1.p * p2.p)) /
                      ((p1.p * p2.p) * (p1.p + p2.p));
  real Rv[3], R2 = R_(0.0);
  real W[3][LTOT + 1];
  int n[3];
  for (int d = 0; d < 3; d++) {
    Rv[d] = p1.P[d] - p2.P[d];
    R2 += Rv[d] * Rv[d];
    real E1[2 * LP + 1], E2[2 * LP + 1];
    const int l1 = A1.l[d] + B1.l[d], l2 = A2.l[d] + B2.l[d];
    hermite_e(A1.l[d], B1.l[d], p1.K[d], A1.a, B1.a, p1.p, p1.q, p1.Q[d], E1);
    hermite_e(A2.l[d], B2.l[d], p2.K[d], A2.a, B2.a, p2.p, p2.q, p2.Q[d], E2);
    for (int k = 0; k <= l1 + l2; k++) W[d][k] = R_(0.0);
    for (int t1 = 0; t1 <= l1; t1++)
      for (int t2 = 0; t2 <= l2; t2++)
        W[d][t1 + t2] += E1[t1] * E2[t2] * ((t2 & 1) ? -R_(1.0) : R_(1.0));
    n[d] = l1 + l2;
  }
  return coe2 * contract_wr(W[0], n[0], W[1], n[1], W[2], n[2], beta * R2,
                            beta, Rv);
}

// ======================================================================
// two-particle geminal kernels of gam_1 (XC1_G2_MD.f, g2.f)

// d^N/dx^N exp(-q (x - B)^2) at x = A for N = 0..nmax (common.f gdel_x)
NX_HD void gauss_derivs(int nmax, real q, real u /* A - B */, real* g) {
  g[0] = exp(-q * u * u);
  for (int N = 1; N <= nmax; N++)
    g[N] = -R_(2.0) * q * u * g[N - 1] - (N > 1 ? R_(2.0) * q * (N - 1) * g[N - 2] : R_(0.0));
}

// G2_MD_xggvec (XC1_G2_MD.f:190-624): attraction of particle 1 to the point
// C for the pairs (A1,B1), (A2,B2) coupled by exp(-(gamma1+gamma2) r12^2).
// Per direction W[n] folds the Hermite coefficients, the binomial split
// between the Gaussian and Coulomb parts and the powers of -DC1 / -DC2 of
// g2_dhermite_vec; R_tuv is taken about C - S as in g2_vec_prefactors.
NX_BIG real g2_xggvec(const Prim& A1, const Prim& A2, const Prim& B1,
                       const Prim& B2, real gamma1, real gamma2,
                       const real* C) {
  const real G = gamma1 + gamma2;
  Pair p1, p2;
  gauss_pair(A1, B1, p1);
  gauss_pair(A2, B2, p2);
  const real P1 = p1.p, P2 = p2.p;
  const real s = (P1 * P2 + P1 * G + P2 * G) / (P2 + G);
  const real alpha = s;
  const real x = kPiT / (P2 + G);
  const real c1 = pow(x, R_(1.5)) * R_(2.0) * kPiT / s;
  const real xx = P1 * P2 + P1 * G + P2 * G;
  const real qP = (P1 * P2 * G) / xx;
  const real DC1 = (P1 * P2 + P1 * G) / xx, DC2 = (P2 * G) / xx;
  real RCS[3], R2 = R_(0.0);
  real W[3][LTOT + 1];
  int n[3];
  for (int d = 0; d < 3; d++) {
    const real Sm = ((P1 * P2 + P1 * G) * p1.P[d] + P2 * G * p2.P[d]) / xx;
    RCS[d] = C[d] - Sm;
    R2 += RCS[d] * RCS[d];
    real E1[2 * LP + 1], E2[2 * LP + 1], gd[4 * LP + 1];
    const int l1 = A1.l[d] + B1.l[d], l2 = A2.l[d] + B2.l[d];
    hermite_e(A1.l[d], B1.l[d], p1.K[d], A1.a, B1.a, P1, p1.q, p1.Q[d], E1);
    hermite_e(A2.l[d], B2.l[d], p2.K[d], A2.a, B2.a, P2, p2.q, p2.Q[d], E2);
    gauss_derivs(l1 + l2, qP, p1.P[d] - p2.P[d], gd);
    real pw1[2 * LP + 1], pw2[2 * LP + 1];
    pw1[0] = pw2[0] = R_(1.0);
    for (int k = 1; k <= 2 * LP; k++) {
      pw1[k] = pw1[k - 1] * -DC1;
      pw2[k] = pw2[k - 1] * -DC2;
    }
    for (int k = 0; k <= l1 + l2; k++) W[d][k] = R_(0.0);
    for (int t1 = 0; t1 <= l1; t1++)
      for (int t2 = 0; t2 <= l2; t2++) {
        const real e = E1[t1] * E2[t2];
        for (int b1 = 0; b1 <= t1; b1++)
          for (int b2 = 0; b2 <= t2; b2++) {
            const real sg = ((t2 - b2) & 1) ? -R_(1.0) : R_(1.0);
            W[d][b1 + b2] += e * binom(t1, b1) * binom(t2, b2) * sg * pw1[b1] *
                             pw2[b2] * gd[(t1 - b1) + (t2 - b2)];
          }
      }
    n[d] = l1 + l2;
  }
  return c1 * contract_wr(W[0], n[0], W[1], n[1], W[2], n[2], alpha * R2,
                          alpha, RCS);
}

// G2_MD_xggvee (XC1_G2_MD.f:630-960): 1/|r1 - r2| between the two
// geminal-coupled particles (g2_ee_prefactors, g2_dhermite_vee).
NX_BIG real g2_xggvee(const Prim& A1, const Prim& A2, const Prim& B1,
                       const Prim& B2, real gamma1, real gamma2) {
  const real G = gamma1 + gamma2;
  Pair p1, p2;
  gauss_pair(A1, B1, p1);
  gauss_pair(A2, B2, p2);
  const real P1 = p1.p, P2 = p2.p;
  const real xx = P1 * P2 + P1 * G + P2 * G;
  const real c0 = (R_(2.0) * pow(kPiT, R_(2.5))) / (xx * sqrt(P1 + P2));
  const real qP = (P1 * P2 * G) / xx;
  const real alpha = (P1 * P1 * P2 * P2) / (xx * (P1 + P2));
  real X[3], R2 = R_(0.0);
  real W[3][LTOT + 1];
  int n[3];
  for (int d = 0; d < 3; d++) {
    X[d] = p1.P[d] - p2.P[d];
    R2 += X[d] * X[d];
    real E1[2 * LP + 1], E2[2 * LP + 1], gd[4 * LP + 1];
    const int l1 = A1.l[d] + B1.l[d], l2 = A2.l[d] + B2.l[d];
    hermite_e(A1.l[d], B1.l[d], p1.K[d], A1.a, B1.a, P1, p1.q, p1.Q[d], E1);
    hermite_e(A2.l[d], B2.l[d], p2.K[d], A2.a, B2.a, P2, p2.q, p2.Q[d], E2);
    gauss_derivs(l1 + l2, qP, X[d], gd);
    for (int k = 0; k <= l1 + l2; k++) W[d][k] = R_(0.0);
    for (int t1 = 0; t1 <= l1; t1++)
      for (int t2 = 0; t2 <= l2; t2++) {
        const real e = E1[t1] * E2[t2] * ((t2 & 1) ? -R_(1.0) : R_(1.0));
        const int N = t1 + t2;
        for (int b = 0; b <= N; b++) W[d][b] += e * binom(N, b) * gd[N - b];
      }
    n[d] = l1 + l2;
  }
  return c0 * contract_wr(W[0], n[0], W[1], n[1], W[2], n[2], alpha * R2,
                          alpha, X);
}

// pgiovlap_1D (g2.f:915-1009) with pgi_hint0_1D (:200-234, whose pi is
// 3.141592650): 1-D overlap of two particles coupled by
// exp(-(gamA+gamB) x12^2).
NX_BIG real pgi_ovl1d(int I1, real a1, real A1, int I2, real a2,
                       real A2, int L1, real b1, real B1, int L2,
                       real b2, real B2, real gam) {
  const real p1 = a1 + b1, q1 = (a1 * b1) / (a1 + b1), Q1 = A1 - B1;
  const real p2 = a2 + b2, q2 = (a2 * b2) / (a2 + b2), Q2 = A2 - B2;
  const real Pm1 = (a1 * A1 + b1 * B1) / (a1 + b1);
  const real Pm2 = (a2 * A2 + b2 * B2) / (a2 + b2);
  real E1[2 * TMX + 1], E2[2 * TMX + 1], gd[2 * TMX + 1];
  hermite_e(I1, L1, exp(-q1 * Q1 * Q1), a1, b1, p1, q1, Q1, E1);
  hermite_e(I2, L2, exp(-q2 * Q2 * Q2), a2, b2, p2, q2, Q2, E2);
  const real s = (p1 * p2) + (p1 * gam) + (p2 * gam);
  const real q = (p1 * p2 * gam) / s;
  const real PI = R_(3.141592650);
  const real pre = sqrt(PI * PI / s);
  gauss_derivs(I1 + L1 + I2 + L2, q, Pm1 - Pm2, gd);
  real acc = R_(0.0);
  for (int t1 = 0; t1 <= I1 + L1; t1++)
    for (int t2 = 0; t2 <= I2 + L2; t2++)
      acc += E1[t1] * E2[t2] * (((t2 & 1) ? -R_(1.0) : R_(1.0)) * pre * gd[t1 + t2]);
  return acc;
}

// pgi_Lapx1 (g2.f:655-765) with pgi_calcS2 / pgi_calcS3 (:768-911)
NX_BIG real pgi_lapx1(int I1, real a1, real A1, int I2, real a2,
                       real A2, int L1, real b1, real B1, int L2,
                       real b2, real B2, real gA, real gB) {
  const real g = gA + gB;
#define OV(l1s, l2s) pgi_ovl1d(I1, a1, A1, I2, a2, A2, (l1s), b1, B1, (l2s), b2, B2, g)
  const real X12 = B1 - B2;
  const real d1 = (L1 - 1 >= 0) ? (real)(L1 * (L1 - 1)) : R_(0.0);
  const real d2 = -R_(2.0) * b1 * (real)((2 * L1) + 1);
  const real d3 = R_(4.0) * b1 * b1;
  const real c1 = (real)L1, c2 = -R_(2.0) * b1;
  const real p1 = (L1 - 2 >= 0) ? OV(L1 - 2, L2) : R_(0.0);
  const real p2 = OV(L1, L2);
  const real p3 = OV(L1 + 2, L2);
  const real W1 = (d1 * p1) + (d2 * p2) + (d3 * p3);
  // calcS2(L) = OV(L+1, L2) - OV(L, L2+1) + X12 OV(L, L2)
  const real q1 = (L1 - 1 >= 0) ? OV(L1, L2) - OV(L1 - 1, L2 + 1) + (X12 * OV(L1 - 1, L2)) : R_(0.0);
  const real q2 = OV(L1 + 2, L2) - OV(L1 + 1, L2 + 1) + (X12 * OV(L1 + 1, L2));
  const real W2 = -R_(2.0) * gB * ((c1 * q1) + (c2 * q2));
  const real t1 = p2;
  const real t2 = OV(L1 + 2, L2) + OV(L1, L2 + 2) + (X12 * X12 * p2) -
                    (R_(2.0) * OV(L1 + 1, L2 + 1)) - (R_(2.0) * X12 * OV(L1, L2 + 1)) +
                    (R_(2.0) * X12 * OV(L1 + 1, L2));
  const real W3 = (-R_(2.0) * gB * t1) + (R_(4.0) * gB * gB * t2);
#undef OV
  return W1 + (R_(2.0) * W2) + W3;
}

// pgike1 (g2.f:545-651): kinetic energy of particle 1 (mass xmass) for the
// geminal-coupled pairs (A1,B1), (A2,B2); geminal exponents gA (bra), gB (ket).
NX_BIG real pgike1(const Prim& A1, const Prim& A2, const Prim& B1,
                    const Prim& B2, real gA, real gB, real xmass) {
  real S[3], T[3];
  for (int d = 0; d < 3; d++) {
    S[d] = pgi_ovl1d(A1.l[d], A1.a, A1.c[d], A2.l[d], A2.a, A2.c[d], B1.l[d],
                     B1.a, B1.c[d], B2.l[d], B2.a, B2.c[d], gA + gB);
    const real dd = pgi_lapx1(A1.l[d], A1.a, A1.c[d], A2.l[d], A2.a,
                                A2.c[d], B1.l[d], B1.a, B1.c[d], B2.l[d],
                                B2.a, B2.c[d], gA, gB);
    T[d] = -dd * R_(0.50) / xmass;
  }
  return (T[0] * S[1] * S[2]) + (S[0] * T[1] * S[2]) + (S[0] * S[1] * T[2]);
}

// |x| < 1e-100 -> 0 (underflow.f:2-11); below FP32's range in the md32 instance
NX_HD real underflow(real x) { return fabs((double)x) < 1.0e-100 ? R_(0.0) : x; }

#undef R_
}  // namespace MD_NS
}  // namespace neoxc
