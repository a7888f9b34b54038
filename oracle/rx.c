/*
 * rx.c -- ORACLE (test infrastructure only): the in-core special-electron
 * contractions of NEO-RXCHF restated on the CPU.  Only the tests load it.
 *
 *   RXCUHFne_FE/FP/FBE_OMG2   rxchfne/rxcuhfne_omg2.f:2-651   (RXCUHF-ae)
 *   RXCHF_FAE/FP/FBE_OMG2     rxchf/rxchf_omg2.f:2-667        (RXCHF-fe)
 *   RXCHF_FAE/FP/FBE_OMG3     rxchf/rxchf_omg3.f:2-708
 *   RXCHF_FAE/FP/FBE_OMG4     rxchf/rxchf_omg4.f:2-663
 *   RXCUHF_FE/FP/FBE_OMG2     rxchf/rxcuhf_omg2.f:2-694       (RXCUHF-fe)
 *   RXCUHF_FE/FP/FBE_OMG3     rxchf/rxcuhf_omg3.f:2-728
 *
 * Each routine runs the reference's loop nest (ip, jp, iec1, jec1, iec2,
 * jec2, ... with the last index fastest), reads the tensors through the
 * reference's packed-index functions (1-based arguments) and accumulates
 * its private matrices into the caller's (add2fock); energies are
 * overwritten.  Matrices are column-major, D(i,j) = D[(i-1) + n (j-1)].
 */
#include <stdlib.h>

#include "neoxc_oracle.h"

#define D2(D, n, i, j) (D)[((i) - 1) + (n) * ((j) - 1)]
#define I2(a1, b1, a2, b2) (orc_index_gam_2pk(ne, np, ip, jp, a1, b1, a2, b2) - 1)
#define I3(a1, b1, a2, b2, a3, b3) \
  (orc_index_gam_3pk(ne, np, ip, jp, a1, b1, a2, b2, a3, b3) - 1)
#define I4(a1, b1, a2, b2, a3, b3, a4, b4) \
  (orc_index_gam_4pk2(ne, np, ip, jp, a1, b1, a2, b2, a3, b3, a4, b4) - 1)

static double *zeros(int64_t n) { return (double *)calloc((size_t)n, sizeof(double)); }
static void add_into(int64_t n, const double *x, double *F) {
  for (int64_t k = 0; k < n; k++) F[k] += x[k];
}

#define LOOP2                                                   \
  for (int64_t ip = 1; ip <= np; ip++)                          \
  for (int64_t jp = 1; jp <= np; jp++)                          \
  for (int64_t i1 = 1; i1 <= ne; i1++)                          \
  for (int64_t j1 = 1; j1 <= ne; j1++)                          \
  for (int64_t i2 = 1; i2 <= ne; i2++)                          \
  for (int64_t j2 = 1; j2 <= ne; j2++)
#define LOOP3 LOOP2                                             \
  for (int64_t i3 = 1; i3 <= ne; i3++)                          \
  for (int64_t j3 = 1; j3 <= ne; j3++)
#define LOOP4 LOOP3                                             \
  for (int64_t i4 = 1; i4 <= ne; i4++)                          \
  for (int64_t j4 = 1; j4 <= ne; j4++)

/* ---- RXCUHF-ae: rxcuhfne_omg2.f ------------------------------------------ */
void orc_rxcuhfne_fe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                          const double *DAtotE, const double *DBE, const double *DP,
                          const double *G, const double *Gx, double *FAalpE,
                          double *FAbetE, double *E) {
  double *xa = zeros(ne * ne), *xb = zeros(ne * ne), e = 0.0;
  LOOP2 {
    const double val12 = G[I2(i1, j1, i2, j2)], val21 = Gx[I2(i1, j2, i2, j1)];
    D2(xa, ne, i2, j2) += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * (val12 - val21);
    D2(xb, ne, i2, j2) += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * (val12);
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) *
         (D2(DAtotE, ne, i2, j2) * val12 - D2(DAalpE, ne, i2, j2) * val21);
  }
  add_into(ne * ne, xa, FAalpE);
  add_into(ne * ne, xb, FAbetE);
  *E = e;
  free(xa); free(xb);
}

void orc_rxcuhfne_fp_omg2(int64_t ne, int64_t np, const double *DAalpE,
                          const double *DAtotE, const double *DBE, const double *DP,
                          const double *G, const double *Gx, double *FP, double *E) {
  double *xf = zeros(np * np), e = 0.0;
  LOOP2 {
    const double val12 = G[I2(i1, j1, i2, j2)], val21 = Gx[I2(i1, j2, i2, j1)];
    D2(xf, np, ip, jp) += D2(DBE, ne, i1, j1) *
        (D2(DAtotE, ne, i2, j2) * val12 - D2(DAalpE, ne, i2, j2) * val21);
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) *
         (D2(DAtotE, ne, i2, j2) * val12 - D2(DAalpE, ne, i2, j2) * val21);
  }
  add_into(np * np, xf, FP);
  *E = e;
  free(xf);
}

void orc_rxcuhfne_fbe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                           const double *DAtotE, const double *DBE, const double *DP,
                           const double *G, const double *Gx, double *FBE, double *E) {
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP2 {
    const double val12 = G[I2(i1, j1, i2, j2)], val21 = Gx[I2(i1, j2, i2, j1)];
    D2(xf, ne, i1, j1) += D2(DP, np, ip, jp) *
        (D2(DAtotE, ne, i2, j2) * val12 - D2(DAalpE, ne, i2, j2) * val21);
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) *
         (D2(DAtotE, ne, i2, j2) * val12 - D2(DAalpE, ne, i2, j2) * val21);
  }
  add_into(ne * ne, xf, FBE);
  *E = e;
  free(xf);
}

/* ---- RXCHF-fe rank 2: rxchf_omg2.f ---------------------------------------- */
void orc_rxchf_fae_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        const double *Gs, double *FAE, double *SAE, double *E,
                        double *S) {
  const double half = 0.5, two = 2.0;
  double *xf = zeros(ne * ne), *xs = zeros(ne * ne), e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    D2(xf, ne, i2, j2) += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * (two * val1 - val2);
    D2(xs, ne, i2, j2) += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * Sval;
    e += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) *
         (val1 - half * val2);
    sv += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) * (-half) * Sval;
  }
  add_into(ne * ne, xf, FAE);
  add_into(ne * ne, xs, SAE);
  *E = e;
  *S = sv;
  free(xf); free(xs);
}

void orc_rxchf_fp_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G1, const double *G2,
                       const double *Gs, double *FP, double *SP, double *E, double *S) {
  const double half = 0.5;
  double *xf = zeros(np * np), *xs = zeros(np * np), e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    D2(xf, np, ip, jp) += D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) * (val1 - half * val2);
    D2(xs, np, ip, jp) -= half * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) * Sval;
    e += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) *
         (val1 - half * val2);
    sv += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) * (-half) * Sval;
  }
  add_into(np * np, xf, FP);
  add_into(np * np, xs, SP);
  *E = e;
  *S = sv;
  free(xf); free(xs);
}

void orc_rxchf_fbe_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        const double *Gs, double *FBE, double *SBE, double *E,
                        double *S) {
  const double half = 0.5;
  double *xf = zeros(ne * ne), *xs = zeros(ne * ne), e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    D2(xf, ne, i1, j1) += D2(DAE, ne, i2, j2) * D2(DP, np, ip, jp) * (val1 - half * val2);
    D2(xs, ne, i1, j1) -= half * D2(DAE, ne, i2, j2) * D2(DP, np, ip, jp) * Sval;
    e += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) *
         (val1 - half * val2);
    sv += D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) * D2(DBE, ne, i1, j1) * (-half) * Sval;
  }
  add_into(ne * ne, xf, FBE);
  add_into(ne * ne, xs, SBE);
  *E = e;
  *S = sv;
  free(xf); free(xs);
}

/* ---- RXCHF-fe rank 3: rxchf_omg3.f ---------------------------------------- */
void orc_rxchf_fae_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        double *FAE, double *E) {
  const double half = 0.5, two = 2.0;
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP3 {
    const int64_t ia_123_123 = I3(i1, j1, i2, j2, i3, j3);
    const int64_t ia_123_213 = I3(i1, j2, i2, j1, i3, j3);
    const int64_t ia_123_312 = I3(i1, j3, i2, j1, i3, j2);
    const int64_t ia_123_132 = I3(i1, j1, i2, j3, i3, j2);
    const double val1 = G1[ia_123_123] - half * G1[ia_123_132];
    const int64_t ib_123_213 = I3(i1, i2, j2, j1, i3, j3);
    const int64_t ib_123_312 = I3(i1, j3, j2, j1, i3, i2);
    const int64_t ia_132_312 = I3(i1, j3, i3, j1, i2, j2);
    const int64_t ia_132_213 = I3(i1, j2, i3, j1, i2, j3);
    const int64_t ib_132_312 = I3(i1, j3, i3, j1, j2, i2);
    const int64_t ib_132_213 = I3(i1, i2, i3, j1, j2, j3);
    const double val2 = (G2[ia_123_213] + G2[ib_123_213]) -
                        half * (G2[ia_123_312] + G2[ib_123_312]);
    const double val3 = (G2[ia_132_312] + G2[ib_132_312]) -
                        half * (G2[ia_132_213] + G2[ib_132_213]);
    D2(xf, ne, i2, j2) += D2(DAE, ne, i3, j3) * D2(DBE, ne, i1, j1) * D2(DP, np, ip, jp) *
                          (two * val1 - half * (val2 + val3));
    e += half * D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * (val1 - half * val2);
  }
  add_into(ne * ne, xf, FAE);
  *E = e;
  free(xf);
}

/* val1 - val2 of RXCHF_thread_FPOMG3 / FBEOMG3 */
static double rx3_pb(int64_t ne, int64_t np, int64_t ip, int64_t jp, const double *G1,
                     const double *G2, int64_t i1, int64_t j1, int64_t i2, int64_t j2,
                     int64_t i3, int64_t j3) {
  const double half = 0.5;
  const double val1 = G1[I3(i1, j1, i2, j2, i3, j3)] - half * G1[I3(i1, j1, i2, j3, i3, j2)];
  const double val2 = G2[I3(i1, j2, i2, j1, i3, j3)] - half * G2[I3(i1, j3, i2, j1, i3, j2)];
  return val1 - val2;
}

void orc_rxchf_fp_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G1, const double *G2, double *FP,
                       double *E) {
  const double half = 0.5;
  double *xf = zeros(np * np), e = 0.0;
  LOOP3 {
    const double c = rx3_pb(ne, np, ip, jp, G1, G2, i1, j1, i2, j2, i3, j3);
    D2(xf, np, ip, jp) += half * D2(DAE, ne, i2, j2) * D2(DAE, ne, i3, j3) *
                          D2(DBE, ne, i1, j1) * c;
    e += half * D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * c;
  }
  add_into(np * np, xf, FP);
  *E = e;
  free(xf);
}

void orc_rxchf_fbe_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2, double *FBE,
                        double *E) {
  const double half = 0.5;
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP3 {
    const double c = rx3_pb(ne, np, ip, jp, G1, G2, i1, j1, i2, j2, i3, j3);
    D2(xf, ne, i1, j1) += half * D2(DAE, ne, i2, j2) * D2(DAE, ne, i3, j3) *
                          D2(DP, np, ip, jp) * c;
    e += half * D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * c;
  }
  add_into(ne * ne, xf, FBE);
  *E = e;
  free(xf);
}

/* ---- RXCHF-fe rank 4: rxchf_omg4.f ---------------------------------------- */
static double rx4_c(int64_t ne, int64_t np, int64_t ip, int64_t jp, const double *G,
                    int64_t ie1, int64_t je1, int64_t ie2, int64_t je2, int64_t ie3,
                    int64_t je3, int64_t ie4, int64_t je4) {
  const double half = 0.5;
  const double val1 = G[I4(ie1, je3, ie2, je1, ie3, je2, ie4, je4)];
  const double val2 = G[I4(ie1, je3, ie2, je1, ie3, je4, ie4, je2)];
  const double val3 = G[I4(ie1, je2, ie2, je1, ie3, je3, ie4, je4)];
  const double val4 = G[I4(ie1, je2, ie2, je1, ie3, je4, ie4, je3)];
  return val1 - half * val2 - val3 + half * val4;
}

void orc_rxchf_fae_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G, double *FAE, double *E) {
  const double half = 0.5;
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP4 {
    const double c = rx4_c(ne, np, ip, jp, G, i1, j1, i2, j2, i3, j3, i4, j4);
    D2(xf, ne, i2, j2) += half * D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) *
                          D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
    e += half * half * D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
  }
  add_into(ne * ne, xf, FAE);
  *E = e;
  free(xf);
}

void orc_rxchf_fp_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G, double *FP, double *E) {
  const double half = 0.5;
  double *xf = zeros(np * np), e = 0.0;
  LOOP4 {
    const double c = rx4_c(ne, np, ip, jp, G, i1, j1, i2, j2, i3, j3, i4, j4);
    D2(xf, np, ip, jp) += half * half * D2(DBE, ne, i1, j1) * D2(DAE, ne, i2, j2) *
                          D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
    e += half * half * D2(DBE, ne, i1, j1) * D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
  }
  add_into(np * np, xf, FP);
  *E = e;
  free(xf);
}

void orc_rxchf_fbe_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G, double *FBE, double *E) {
  const double half = 0.5;
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP4 {
    const double c = rx4_c(ne, np, ip, jp, G, i1, j1, i2, j2, i3, j3, i4, j4);
    D2(xf, ne, i1, j1) += half * half * D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) *
                          D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
    e += half * half * D2(DBE, ne, i1, j1) * D2(DP, np, ip, jp) * D2(DAE, ne, i2, j2) *
         D2(DAE, ne, i3, j3) * D2(DAE, ne, i4, j4) * c;
  }
  add_into(ne * ne, xf, FBE);
  *E = e;
  free(xf);
}

/* ---- RXCUHF-fe rank 2: rxcuhf_omg2.f -------------------------------------- */
void orc_rxcuhf_fe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAtotE, const double *DBE, const double *DP,
                        const double *G1, const double *G2, const double *Gs,
                        double *FAalpE, double *FAbetE, double *SAalpE, double *E,
                        double *S) {
  double *xa = zeros(ne * ne), *xb = zeros(ne * ne), *xs = zeros(ne * ne);
  double e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    const double w = D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1);
    D2(xa, ne, i2, j2) += w * (val1 - val2);
    D2(xs, ne, i2, j2) += w * (Sval);
    D2(xb, ne, i2, j2) += w * (val1);
    e += w * (D2(DAtotE, ne, i2, j2) * val1 - D2(DAalpE, ne, i2, j2) * val2);
    sv += w * (-D2(DAalpE, ne, i2, j2) * Sval);
  }
  add_into(ne * ne, xa, FAalpE);
  add_into(ne * ne, xb, FAbetE);
  add_into(ne * ne, xs, SAalpE);
  *E = e;
  *S = sv;
  free(xa); free(xb); free(xs);
}

void orc_rxcuhf_fp_omg2(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAtotE, const double *DBE, const double *DP,
                        const double *G1, const double *G2, const double *Gs,
                        double *FP, double *SP, double *E, double *S) {
  double *xf = zeros(np * np), *xs = zeros(np * np), e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    const double f = D2(DBE, ne, i1, j1) *
        (D2(DAtotE, ne, i2, j2) * val1 - D2(DAalpE, ne, i2, j2) * val2);
    const double g = D2(DBE, ne, i1, j1) * (-D2(DAalpE, ne, i2, j2) * Sval);
    D2(xf, np, ip, jp) += f;
    D2(xs, np, ip, jp) += g;
    e += D2(DP, np, ip, jp) * f;
    sv += D2(DP, np, ip, jp) * g;
  }
  add_into(np * np, xf, FP);
  add_into(np * np, xs, SP);
  *E = e;
  *S = sv;
  free(xf); free(xs);
}

void orc_rxcuhf_fbe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                         const double *DAtotE, const double *DBE, const double *DP,
                         const double *G1, const double *G2, const double *Gs,
                         double *FBE, double *SBE, double *E, double *S) {
  double *xf = zeros(ne * ne), *xs = zeros(ne * ne), e = 0.0, sv = 0.0;
  LOOP2 {
    const double val1 = G1[I2(i1, j1, i2, j2)], val2 = G2[I2(i1, j2, i2, j1)];
    const double Sval = Gs[I2(i1, j2, i2, j1)];
    const double f = D2(DP, np, ip, jp) *
        (D2(DAtotE, ne, i2, j2) * val1 - D2(DAalpE, ne, i2, j2) * val2);
    const double g = D2(DP, np, ip, jp) * (-D2(DAalpE, ne, i2, j2) * Sval);
    D2(xf, ne, i1, j1) += f;
    D2(xs, ne, i1, j1) += g;
    e += D2(DBE, ne, i1, j1) * f;
    sv += D2(DBE, ne, i1, j1) * g;
  }
  add_into(ne * ne, xf, FBE);
  add_into(ne * ne, xs, SBE);
  *E = e;
  *S = sv;
  free(xf); free(xs);
}

/* ---- RXCUHF-fe rank 3: rxcuhf_omg3.f -------------------------------------- */
void orc_rxcuhf_fe_omg3(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAbetE, const double *DAtotE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        double *FAalpE, double *FAbetE, double *E) {
  const double half = 0.5;
  double *xa = zeros(ne * ne), *xb = zeros(ne * ne), e = 0.0;
  LOOP3 {
    const int64_t ia_123_123 = I3(i1, j1, i2, j2, i3, j3);
    const int64_t ia_123_213 = I3(i1, j2, i2, j1, i3, j3);
    const int64_t ia_123_312 = I3(i1, j3, i2, j1, i3, j2);
    const int64_t ia_123_132 = I3(i1, j1, i2, j3, i3, j2);
    const int64_t ib_123_213 = I3(i1, i2, j2, j1, i3, j3);
    const int64_t ib_123_312 = I3(i1, j3, j2, j1, i3, i2);
    const int64_t ia_132_312 = I3(i1, j3, i3, j1, i2, j2);
    const int64_t ia_132_213 = I3(i1, j2, i3, j1, i2, j3);
    const int64_t ib_132_312 = I3(i1, j3, i3, j1, j2, i2);
    const int64_t ib_132_213 = I3(i1, i2, i3, j1, j2, j3);
    const double val1a = G1[ia_123_123], val1b = G1[ia_123_132];
    const double val2a = (G2[ia_123_213] + G2[ib_123_213]) * half;
    const double val2b = (G2[ia_123_312] + G2[ib_123_312]) * half;
    const double val2c = (G2[ia_132_312] + G2[ib_132_312]) * half;
    const double val2d = (G2[ia_132_213] + G2[ib_132_213]) * half;
    const double w = D2(DBE, ne, i1, j1) * D2(DP, np, ip, jp);
    D2(xa, ne, i2, j2) += w * (D2(DAtotE, ne, i3, j3) * val1a
                               - D2(DAalpE, ne, i3, j3) * val1b
                               - D2(DAtotE, ne, i3, j3) * val2a
                               + D2(DAalpE, ne, i3, j3) * val2b
                               - D2(DAalpE, ne, i3, j3) * val2c
                               + D2(DAalpE, ne, i3, j3) * val2d);
    D2(xb, ne, i2, j2) += w * (D2(DAtotE, ne, i3, j3) * val1a
                               - D2(DAbetE, ne, i3, j3) * val1b
                               - D2(DAalpE, ne, i3, j3) * val2c);
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) *
         (half * D2(DAtotE, ne, i2, j2) * D2(DAtotE, ne, i3, j3) * val1a
          - half * (D2(DAalpE, ne, i2, j2) * D2(DAalpE, ne, i3, j3) +
                    D2(DAbetE, ne, i2, j2) * D2(DAbetE, ne, i3, j3)) * val1b
          - D2(DAalpE, ne, i2, j2) * D2(DAtotE, ne, i3, j3) * G2[ia_123_213]
          + D2(DAalpE, ne, i2, j2) * D2(DAalpE, ne, i3, j3) * G2[ia_123_312]);
  }
  add_into(ne * ne, xa, FAalpE);
  add_into(ne * ne, xb, FAbetE);
  *E = e;
  free(xa); free(xb);
}

/* the bracket of RXCUHF_thread_FPOMG3 / FBEOMG3 */
static double cu3_pb(int64_t ne, int64_t np, int64_t ip, int64_t jp, const double *G1,
                     const double *G2, const double *DAalpE, const double *DAbetE,
                     const double *DAtotE, int64_t i1, int64_t j1, int64_t i2, int64_t j2,
                     int64_t i3, int64_t j3) {
  const double half = 0.5;
  const double val1a = G1[I3(i1, j1, i2, j2, i3, j3)];
  const double val1b = G1[I3(i1, j1, i2, j3, i3, j2)];
  const double val2a = G2[I3(i1, j2, i2, j1, i3, j3)];
  const double val2b = G2[I3(i1, j3, i2, j1, i3, j2)];
  return half * D2(DAtotE, ne, i2, j2) * D2(DAtotE, ne, i3, j3) * val1a
       - half * (D2(DAalpE, ne, i2, j2) * D2(DAalpE, ne, i3, j3) +
                 D2(DAbetE, ne, i2, j2) * D2(DAbetE, ne, i3, j3)) * val1b
       - D2(DAalpE, ne, i2, j2) * D2(DAtotE, ne, i3, j3) * val2a
       + D2(DAalpE, ne, i2, j2) * D2(DAalpE, ne, i3, j3) * val2b;
}

void orc_rxcuhf_fp_omg3(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAbetE, const double *DAtotE, const double *DBE,
                        const double *DP, const double *G1, const double *G2, double *FP,
                        double *E) {
  double *xf = zeros(np * np), e = 0.0;
  LOOP3 {
    const double c = cu3_pb(ne, np, ip, jp, G1, G2, DAalpE, DAbetE, DAtotE, i1, j1, i2,
                            j2, i3, j3);
    D2(xf, np, ip, jp) += D2(DBE, ne, i1, j1) * c;
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * c;
  }
  add_into(np * np, xf, FP);
  *E = e;
  free(xf);
}

void orc_rxcuhf_fbe_omg3(int64_t ne, int64_t np, const double *DAalpE,
                         const double *DAbetE, const double *DAtotE, const double *DBE,
                         const double *DP, const double *G1, const double *G2,
                         double *FBE, double *E) {
  double *xf = zeros(ne * ne), e = 0.0;
  LOOP3 {
    const double c = cu3_pb(ne, np, ip, jp, G1, G2, DAalpE, DAbetE, DAtotE, i1, j1, i2,
                            j2, i3, j3);
    D2(xf, ne, i1, j1) += D2(DP, np, ip, jp) * c;
    e += D2(DP, np, ip, jp) * D2(DBE, ne, i1, j1) * c;
  }
  add_into(ne * ne, xf, FBE);
  *E = e;
  free(xf);
}
