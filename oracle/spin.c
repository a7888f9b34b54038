/*
 * spin.c -- ORACLE (test infrastructure only): the open-shell XCUHF
 * contractions of NEO-RXCHF restated on the CPU.  Only the tests and the
 * CPU-baseline leg of the benchmark load it.
 *
 *   FAE_OMG1 / UFP_OMG1    xcuhf/xcuhf_omg1.f:2-163
 *   FAE_OMG2 / UFP_OMG2    xcuhf/xcuhf_omg2.f:2-612
 *   FAE_OMG3 / UFP_OMG3    xcuhf/xcuhf_omg3.f:2-588
 *   FAE_OMG4 / UFP_OMG4    xcuhf/xcuhf_omg4.f:2-1078
 *   OMG4_ICR               xcuhf/xcuhf_omg4.f:1080-1315 (raw
 *                          calc_GAM_4_integral values, gam_4_OMP.f:964)
 *
 * Every routine loops over the same tuples as the reference (ip, jp, then
 * the electron pairs with the last ket index fastest) and evaluates the same
 * flag-gated spin terms.  The FAE routines compute the Fock matrix of the
 * spin whose density is passed first (the reference calls FAE_* a second
 * time with the arguments swapped for beta).  Fock matrices accumulate
 * (add2fock); SAE*, SP* and the energies are overwritten, as in the
 * reference.  Matrices are column-major, D(i,j) = D[(i-1) + n (j-1)].
 */
#include <stdlib.h>

#include "neoxc_oracle.h"

#define M2(D, n, i, j) (D)[((i) - 1) + (n) * ((j) - 1)]

/* ---- OMG1 ------------------------------------------------------------- */
/* GAM_1 / GAM_1s[pack_4D(ne,ne,np, je1,ie1,jp,ip) - 1] */
static int64_t g1_index(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                        int64_t ie1, int64_t je1) {
  return orc_pack_4d(ne, ne, np, je1, ie1, jp, ip) - 1;
}

void orc_fae_omg1(int64_t ne, int64_t np, const double *DAE, const double *DP,
                  const double *G1, const double *G1s, double *FAE,
                  double *SAE1, double *E, double *S) {
  double *xf = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double e = 0.0, sv = 0.0;
  for (int64_t k = 0; k < ne * ne; k++) SAE1[k] = 0.0;
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++)
      for (int64_t ie1 = 1; ie1 <= ne; ie1++)
        for (int64_t je1 = 1; je1 <= ne; je1++) {
          const int64_t ia = g1_index(ne, np, ip, jp, ie1, je1);
          const double dp = M2(DP, np, ip, jp);
          M2(xf, ne, ie1, je1) += dp * G1[ia];
          M2(SAE1, ne, ie1, je1) += dp * G1s[ia];
          e += dp * M2(DAE, ne, ie1, je1) * G1[ia];
          sv += dp * M2(DAE, ne, ie1, je1) * G1s[ia];
        }
  for (int64_t k = 0; k < ne * ne; k++) FAE[k] += xf[k];
  *E = e;
  *S = sv;
  free(xf);
}

void orc_ufp_omg1(int64_t ne, int64_t np, const double *DETOT,
                  const double *DP, const double *G1, const double *G1s,
                  double *FP, double *SP1, double *E, double *S) {
  double *xf = (double *)calloc((size_t)(np * np), sizeof(double));
  double e = 0.0, sv = 0.0;
  for (int64_t k = 0; k < np * np; k++) SP1[k] = 0.0;
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++)
      for (int64_t ie1 = 1; ie1 <= ne; ie1++)
        for (int64_t je1 = 1; je1 <= ne; je1++) {
          const int64_t ia = g1_index(ne, np, ip, jp, ie1, je1);
          const double d = M2(DETOT, ne, ie1, je1);
          M2(xf, np, ip, jp) += d * G1[ia];
          M2(SP1, np, ip, jp) += d * G1s[ia];
          e += M2(DP, np, ip, jp) * d * G1[ia];
          sv += M2(DP, np, ip, jp) * d * G1s[ia];
        }
  for (int64_t k = 0; k < np * np; k++) FP[k] += xf[k];
  *E = e;
  *S = sv;
  free(xf);
}

/* ---- OMG2 ------------------------------------------------------------- */
void orc_fae_omg2(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G2, const double *G2s, double *FAE,
                  double *SAE2, double *E, double *S) {
  const int LAA = NAE >= 2, LAB = NAE >= 1 && NBE >= 1;
  const double EFAC = 2.0;
  double *xf = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double e = 0.0, sv = 0.0;
  for (int64_t k = 0; k < ne * ne; k++) SAE2[k] = 0.0;
  for (int64_t ip = 1; ip <= np; ip++)
  for (int64_t jp = 1; jp <= np; jp++)
  for (int64_t i1 = 1; i1 <= ne; i1++)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++) {
    const int64_t a12 = orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2) - 1;
    const int64_t a21 = orc_index_gam_2pk(ne, np, ip, jp, i1, j2, i2, j1) - 1;
    const double o12 = G2[a12], o21 = G2[a21], s12 = G2s[a12], s21 = G2s[a21];
    const double c1 = LAA ? M2(DAE, ne, i2, j2) * M2(DP, np, ip, jp) : 0.0;
    const double c2 = LAB ? M2(DBE, ne, i2, j2) * M2(DP, np, ip, jp) : 0.0;
    const double f = c1 * (o12 - o21) + c2 * o12;
    const double fs = c1 * (s12 - s21) + c2 * s12;
    M2(xf, ne, i1, j1) += EFAC * f;
    M2(SAE2, ne, i1, j1) += EFAC * fs;
    e += M2(DAE, ne, i1, j1) * f;
    sv += M2(DAE, ne, i1, j1) * fs;
  }
  for (int64_t k = 0; k < ne * ne; k++) FAE[k] += xf[k];
  *E = e;
  *S = sv;
  free(xf);
}

void orc_ufp_omg2(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G2, const double *G2s, double *FP,
                  double *SP2, double *E, double *S) {
  const int LAB = NAE >= 1 && NBE >= 1, LAA = NAE >= 2, LBB = NBE >= 2;
  double *xf = (double *)calloc((size_t)(np * np), sizeof(double));
  double e = 0.0, sv = 0.0;
  for (int64_t k = 0; k < np * np; k++) SP2[k] = 0.0;
  for (int64_t ip = 1; ip <= np; ip++)
  for (int64_t jp = 1; jp <= np; jp++)
  for (int64_t i1 = 1; i1 <= ne; i1++)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++) {
    const int64_t a12 = orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2) - 1;
    const int64_t a21 = orc_index_gam_2pk(ne, np, ip, jp, i1, j2, i2, j1) - 1;
    const double o12 = G2[a12], o21 = G2[a21], s12 = G2s[a12], s21 = G2s[a21];
    const double a1 = M2(DAE, ne, i1, j1), b1 = M2(DBE, ne, i1, j1);
    const double a2 = M2(DAE, ne, i2, j2), b2 = M2(DBE, ne, i2, j2);
    const double c1 = LAB ? a1 * b2 + b1 * a2 : 0.0;
    const double c2 = LAA ? a1 * a2 : 0.0;
    const double c3 = LBB ? b1 * b2 : 0.0;
    const double f = c1 * o12 + (c2 + c3) * (o12 - o21);
    const double fs = c1 * s12 + (c2 + c3) * (s12 - s21);
    M2(xf, np, ip, jp) += f;
    M2(SP2, np, ip, jp) += fs;
    e += M2(DP, np, ip, jp) * f;
    sv += M2(DP, np, ip, jp) * fs;
  }
  for (int64_t k = 0; k < np * np; k++) FP[k] += xf[k];
  *E = e;
  *S = sv;
  free(xf);
}

/* ---- OMG3 ------------------------------------------------------------- */
typedef struct { double o6, o23, o12, o13; } omg3_set;

static omg3_set omg3_values(int64_t ne, int64_t np, const double *G3,
                            int64_t ip, int64_t jp, int64_t i1, int64_t j1,
                            int64_t i2, int64_t j2, int64_t i3, int64_t j3) {
#define G(a, b, c) G3[orc_index_gam_3pk(ne, np, ip, jp, i1, a, i2, b, i3, c) - 1]
  const double g123 = G(j1, j2, j3), g213 = G(j2, j1, j3), g312 = G(j3, j1, j2);
  const double g132 = G(j1, j3, j2), g231 = G(j2, j3, j1), g321 = G(j3, j2, j1);
#undef G
  omg3_set r;
  r.o6 = g123 - g213 + g312 - g132 + g231 - g321;
  r.o23 = g123 - g132;
  r.o12 = g123 - g213;
  r.o13 = g123 - g321;
  return r;
}

/* per-thread partial sums over the (ip,jp,i1) outer loops */
#define OUTER_BEGIN(nout)                                                    \
  int nt = orc_num_threads();                                                \
  double *xp = (double *)calloc((size_t)((nout) * nt), sizeof(double));      \
  double *ep = (double *)calloc((size_t)nt, sizeof(double));                 \
  _Pragma("omp parallel for schedule(static)")                               \
  for (int c = 0; c < nt; c++) {                                             \
    double *xf = xp + (size_t)(nout) * c;                                    \
    double e = 0.0;                                                          \
    for (int64_t o = c; o < np * np * ne; o += nt) {                         \
      const int64_t ip = o / (np * ne) + 1, jp = (o / ne) % np + 1;          \
      const int64_t i1 = o % ne + 1;
#define OUTER_END(nout, F)                                                   \
    }                                                                        \
    ep[c] = e;                                                               \
  }                                                                          \
  double etot = 0.0;                                                         \
  for (int c = 0; c < nt; c++) {                                             \
    etot += ep[c];                                                           \
    for (int64_t k = 0; k < (nout); k++) (F)[k] += xp[(size_t)(nout) * c + k]; \
  }                                                                          \
  *E = etot;                                                                 \
  free(xp);                                                                  \
  free(ep);

void orc_fae_omg3(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G3, double *FAE, double *E) {
  const int LAB = NBE >= 1 && NAE >= 2, LBB = NBE >= 2, LAA = NAE >= 3;
  const double EFAC = 3.0;
  OUTER_BEGIN(ne * ne)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++)
  for (int64_t i3 = 1; i3 <= ne; i3++)
  for (int64_t j3 = 1; j3 <= ne; j3++) {
    const omg3_set o = omg3_values(ne, np, G3, ip, jp, i1, j1, i2, j2, i3, j3);
    const double a2 = M2(DAE, ne, i2, j2), b2 = M2(DBE, ne, i2, j2);
    const double a3 = M2(DAE, ne, i3, j3), b3 = M2(DBE, ne, i3, j3);
    const double xaa = a2 * a3 * (LAA ? o.o6 : 0.0);
    const double xbb = b2 * b3 * (LBB ? o.o23 : 0.0);
    const double xab = a2 * b3 * (LAB ? o.o12 : 0.0);
    const double xba = b2 * a3 * (LAB ? o.o13 : 0.0);
    const double dp = M2(DP, np, ip, jp);
    M2(xf, ne, i1, j1) += EFAC * dp * (xaa + xbb + xab + xba);
    e += dp * M2(DAE, ne, i1, j1) * (xaa + xbb + xab + xba);
  }
  OUTER_END(ne * ne, FAE)
}

void orc_ufp_omg3(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G3, double *FP, double *E) {
  const int LAAA = NAE >= 3, LBBB = NBE >= 3;
  const int LAAB = NAE >= 2 && NBE >= 1, LBBA = NBE >= 2 && NAE >= 1;
  OUTER_BEGIN(np * np)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++)
  for (int64_t i3 = 1; i3 <= ne; i3++)
  for (int64_t j3 = 1; j3 <= ne; j3++) {
    const omg3_set o = omg3_values(ne, np, G3, ip, jp, i1, j1, i2, j2, i3, j3);
    const double a1 = M2(DAE, ne, i1, j1), b1 = M2(DBE, ne, i1, j1);
    const double a2 = M2(DAE, ne, i2, j2), b2 = M2(DBE, ne, i2, j2);
    const double a3 = M2(DAE, ne, i3, j3), b3 = M2(DBE, ne, i3, j3);
    const double caaa = LAAA ? a1 * a2 * a3 : 0.0, cbbb = LBBB ? b1 * b2 * b3 : 0.0;
    const double caab = LAAB ? a1 * a2 * b3 : 0.0, caba = LAAB ? a1 * b2 * a3 : 0.0;
    const double cbaa = LAAB ? b1 * a2 * a3 : 0.0;
    const double cbba = LBBA ? b1 * b2 * a3 : 0.0, cbab = LBBA ? b1 * a2 * b3 : 0.0;
    const double cabb = LBBA ? a1 * b2 * b3 : 0.0;
    const double f = (caaa + cbbb) * o.o6 + (caab + cbba) * o.o12 +
                     (caba + cbab) * o.o13 + (cabb + cbaa) * o.o23;
    M2(xf, np, ip, jp) += f;
    e += M2(DP, np, ip, jp) * f;
  }
  OUTER_END(np * np, FP)
}

/* ---- OMG4 ------------------------------------------------------------- */
/* value source: the stored OMG4_ICR tensor, or calc_GAM_4_integral computed
 * on the fly from GAM_2s / GAM_ee (same numbers). */
typedef struct {
  int64_t ne, np;
  const double *G4, *G2s, *Gee;
} g4src;

static double g4v(const g4src *s, int64_t ip, int64_t jp, int64_t i1,
                  int64_t k1, int64_t i2, int64_t k2, int64_t i3, int64_t k3,
                  int64_t i4, int64_t k4) {
  if (s->G4)
    return s->G4[orc_index_gam_4pk2(s->ne, s->np, ip, jp, i1, k1, i2, k2, i3, k3,
                                    i4, k4) - 1];
  return orc_gam4_raw(s->ne, s->np, s->G2s, s->Gee, ip, jp, i1, k1, i2, k2, i3,
                      k3, i4, k4);
}

/* the 8 antisymmetrised combinations of calc_FAEOMG4 / calc_UFPOMG4 (the
 * names follow FAE_OMG4: AAA = 24-term, then the 6-term and 4-term sets),
 * each evaluated only when `need` has its bit set. */
typedef struct { double aaa, aab, aba, baa, abb, bab, bba, bbb; } omg4_set;

static omg4_set omg4_values(const g4src *s, unsigned need, int64_t ip,
                            int64_t jp, int64_t i1, int64_t i2, int64_t i3,
                            int64_t i4, int64_t j1, int64_t j2, int64_t j3,
                            int64_t j4) {
#define V(a, b, c, d) g4v(s, ip, jp, i1, a, i2, b, i3, c, i4, d)
  const double OMG = V(j1, j2, j3, j4);
  const double O23 = V(j1, j3, j2, j4), O12 = V(j2, j1, j3, j4);
  const double O13 = V(j3, j2, j1, j4), O24 = V(j1, j4, j3, j2);
  const double O14 = V(j4, j2, j3, j1), O34 = V(j1, j2, j4, j3);
  omg4_set r = {0, 0, 0, 0, 0, 0, 0, 0};
  if (need & 1u) {
    r.aaa = OMG - O23 - O12 - O13 - O24 - O14 - O34
          + V(j2, j3, j1, j4) + V(j3, j1, j2, j4) + V(j2, j4, j3, j1)
          + V(j4, j1, j3, j2) + V(j2, j1, j4, j3) + V(j3, j2, j4, j1)
          + V(j4, j2, j1, j3) + V(j3, j4, j1, j2) + V(j4, j3, j2, j1)
          + V(j1, j3, j4, j2) + V(j1, j4, j2, j3)
          - V(j2, j3, j4, j1) - V(j2, j4, j1, j3) - V(j3, j1, j4, j2)
          - V(j3, j4, j2, j1) - V(j4, j1, j2, j3) - V(j4, j3, j1, j2);
  }
  if (need & 2u) {
    r.aab = OMG - O23 - O12 + V(j2, j3, j1, j4) + V(j3, j1, j2, j4) - O13;
    r.aba = OMG - O24 - O12 + V(j2, j4, j3, j1) + V(j4, j1, j3, j2) - O14;
    r.baa = OMG - O34 - O13 + V(j3, j2, j4, j1) + V(j4, j2, j1, j3) - O14;
  }
  if (need & 4u) {
    r.abb = OMG - O34 - O12 + V(j2, j1, j4, j3);
    r.bab = OMG - O24 - O13 + V(j3, j4, j1, j2);
    r.bba = OMG - O23 - O14 + V(j4, j3, j2, j1);
  }
  if (need & 8u)
    r.bbb = OMG - O34 - O23 + V(j1, j3, j4, j2) + V(j1, j4, j2, j3) - O24;
#undef V
  return r;
}

static void fae_omg4(const g4src *src, int64_t NAE, int64_t NBE,
                     const double *DAE, const double *DBE, const double *DP,
                     double *FAE, double *E) {
  const int64_t ne = src->ne, np = src->np;
  const int LAAA = NAE >= 4, LBBB = NBE >= 3;
  const int LAAB = NAE >= 3 && NBE >= 1, LBBA = NBE >= 2 && NAE >= 2;
  const unsigned need = (LAAA ? 1u : 0u) | (LAAB ? 2u : 0u) | (LBBA ? 4u : 0u) |
                        (LBBB ? 8u : 0u);
  const double four = 4.0;
  OUTER_BEGIN(ne * ne)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++)
  for (int64_t i3 = 1; i3 <= ne; i3++)
  for (int64_t j3 = 1; j3 <= ne; j3++)
  for (int64_t i4 = 1; i4 <= ne; i4++)
  for (int64_t j4 = 1; j4 <= ne; j4++) {
    const omg4_set o = omg4_values(src, need, ip, jp, i1, i2, i3, i4, j1, j2, j3, j4);
    const double a2 = M2(DAE, ne, i2, j2), b2 = M2(DBE, ne, i2, j2);
    const double a3 = M2(DAE, ne, i3, j3), b3 = M2(DBE, ne, i3, j3);
    const double a4 = M2(DAE, ne, i4, j4), b4 = M2(DBE, ne, i4, j4);
    double x = 0.0;
    if (LAAA) x += a2 * a3 * a4 * o.aaa;
    if (LAAB) x += a2 * a3 * b4 * o.aab + a2 * b3 * a4 * o.aba + b2 * a3 * a4 * o.baa;
    if (LBBA) x += a2 * b3 * b4 * o.abb + b2 * a3 * b4 * o.bab + b2 * b3 * a4 * o.bba;
    if (LBBB) x += b2 * b3 * b4 * o.bbb;
    const double ans = M2(DP, np, ip, jp) * x;
    M2(xf, ne, i1, j1) += four * ans;
    e += M2(DAE, ne, i1, j1) * ans;
  }
  OUTER_END(ne * ne, FAE)
}

static void ufp_omg4(const g4src *src, int64_t NAE, int64_t NBE,
                     const double *DAE, const double *DBE, const double *DP,
                     double *FP, double *E) {
  const int64_t ne = src->ne, np = src->np;
  const int L4A = NAE >= 4, L4B = NBE >= 4;
  const int L3A1B = NAE >= 3 && NBE >= 1, L1A3B = NAE >= 1 && NBE >= 3;
  const int L2A2B = NAE >= 2 && NBE >= 2;
  const unsigned need = ((L4A || L4B) ? 1u : 0u) | ((L3A1B || L1A3B) ? 2u | 8u : 0u) |
                        (L2A2B ? 4u : 0u);
  OUTER_BEGIN(np * np)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++)
  for (int64_t i3 = 1; i3 <= ne; i3++)
  for (int64_t j3 = 1; j3 <= ne; j3++)
  for (int64_t i4 = 1; i4 <= ne; i4++)
  for (int64_t j4 = 1; j4 <= ne; j4++) {
    const omg4_set o = omg4_values(src, need, ip, jp, i1, i2, i3, i4, j1, j2, j3, j4);
    const double a1 = M2(DAE, ne, i1, j1), b1 = M2(DBE, ne, i1, j1);
    const double a2 = M2(DAE, ne, i2, j2), b2 = M2(DBE, ne, i2, j2);
    const double a3 = M2(DAE, ne, i3, j3), b3 = M2(DBE, ne, i3, j3);
    const double a4 = M2(DAE, ne, i4, j4), b4 = M2(DBE, ne, i4, j4);
    double x = 0.0;
    /* XAAAA + XAAAB + XAABA + XABAA + XAABB + XABAB + XABBA + XABBB
     * + XBBBB + XBBBA + XBBAB + XBABB + XBBAA + XBABA + XBAAB + XBAAA */
    if (L4A) x += a1 * a2 * a3 * a4 * o.aaa;
    if (L3A1B) x += a1 * a2 * a3 * b4 * o.aab + a1 * a2 * b3 * a4 * o.aba +
                    a1 * b2 * a3 * a4 * o.baa;
    if (L2A2B) x += a1 * a2 * b3 * b4 * o.abb + a1 * b2 * a3 * b4 * o.bab +
                    a1 * b2 * b3 * a4 * o.bba;
    if (L1A3B) x += a1 * b2 * b3 * b4 * o.bbb;
    if (L4B) x += b1 * b2 * b3 * b4 * o.aaa;
    if (L1A3B) x += b1 * b2 * b3 * a4 * o.aab + b1 * b2 * a3 * b4 * o.aba +
                    b1 * a2 * b3 * b4 * o.baa;
    if (L2A2B) x += b1 * b2 * a3 * a4 * o.abb + b1 * a2 * b3 * a4 * o.bab +
                    b1 * a2 * a3 * b4 * o.bba;
    if (L3A1B) x += b1 * a2 * a3 * a4 * o.bbb;
    M2(xf, np, ip, jp) += x;
    e += M2(DP, np, ip, jp) * x;
  }
  OUTER_END(np * np, FP)
}

void orc_fae_omg4(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G4, double *FAE, double *E) {
  const g4src s = {ne, np, G4, 0, 0};
  fae_omg4(&s, NAE, NBE, DAE, DBE, DP, FAE, E);
}

void orc_ufp_omg4(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G4, double *FP, double *E) {
  const g4src s = {ne, np, G4, 0, 0};
  ufp_omg4(&s, NAE, NBE, DAE, DBE, DP, FP, E);
}

/* the same contractions with the OMG4_ICR values computed on the fly */
void orc_fae_omg4_direct(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                         const double *DAE, const double *DBE, const double *DP,
                         const double *G2s, const double *Gee, double *FAE,
                         double *E) {
  const g4src s = {ne, np, 0, G2s, Gee};
  fae_omg4(&s, NAE, NBE, DAE, DBE, DP, FAE, E);
}

void orc_ufp_omg4_direct(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                         const double *DAE, const double *DBE, const double *DP,
                         const double *G2s, const double *Gee, double *FP,
                         double *E) {
  const g4src s = {ne, np, 0, G2s, Gee};
  ufp_omg4(&s, NAE, NBE, DAE, DBE, DP, FP, E);
}

/* xcuhf_omg4.f:1080-1315 OMG4_ICR: GAM_4(index_GAM_4PK2) = i10 */
void orc_omg4_icr(int64_t ne, int64_t np, const double *G2s, const double *Gee,
                  double *G4) {
  const int64_t n2 = ne * ne, n4 = n2 * n2, n8 = n4 * n4;
  const int64_t ng4 = n8 * np * np;
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < ng4; t++) {
    int64_t r = t;
    const int64_t je4 = r % ne + 1; r /= ne;
    const int64_t ie4 = r % ne + 1; r /= ne;
    const int64_t je3 = r % ne + 1; r /= ne;
    const int64_t ie3 = r % ne + 1; r /= ne;
    const int64_t je2 = r % ne + 1; r /= ne;
    const int64_t ie2 = r % ne + 1; r /= ne;
    const int64_t je1 = r % ne + 1; r /= ne;
    const int64_t ie1 = r % ne + 1; r /= ne;
    const int64_t jp = r % np + 1; r /= np;
    const int64_t ip = r + 1;
    const int64_t ia = orc_index_gam_4pk2(ne, np, ip, jp, ie1, je1, ie2, je2, ie3,
                                          je3, ie4, je4);
    G4[ia - 1] = orc_gam4_raw(ne, np, G2s, Gee, ip, jp, ie1, je1, ie2, je2, ie3,
                              je3, ie4, je4);
  }
}
