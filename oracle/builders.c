/*
 * builders.c -- ORACLE (test infrastructure only; never linked by the
 * product).
 *
 * CPU restatement of the NEO-RXCHF contracted-integral builders (gam_2,
 * gam_3, RXCHF-ne gam_2, GAM_ee), the gam_4 assembly, the in-core and
 * direct Fock/energy contractions and the index maps.  Loops visit the
 * flattened tuple space in the reference's loop_map order so that
 * accumulation order matches a single-threaded run of the reference.
 */
#include "neoxc_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- index maps: CS_Integrals/Spot_Check/pack_GAM.f ------------------- */
/* pack_GAM.f:29-69 pack_4D */
int64_t orc_pack_4d(int64_t n1, int64_t n2, int64_t n3, int64_t i1,
                    int64_t i2, int64_t i3, int64_t i4) {
  return 1 + (i1 - 1) + n1 * ((i2 - 1) + n2 * ((i3 - 1) + n3 * (i4 - 1)));
}
/* pack_GAM.f:72-105 index_GAM_2PK */
int64_t orc_index_gam_2pk(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                          int64_t ie1, int64_t je1, int64_t ie2,
                          int64_t je2) {
  return 1 + (je2 - 1) +
         ne * ((ie2 - 1) +
               ne * ((je1 - 1) + ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))));
}
/* pack_GAM.f:108-147 index_GAM_3PK */
int64_t orc_index_gam_3pk(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                          int64_t ie1, int64_t je1, int64_t ie2, int64_t je2,
                          int64_t ie3, int64_t je3) {
  return 1 + (je3 - 1) +
         ne * ((ie3 - 1) +
         ne * ((je2 - 1) +
         ne * ((ie2 - 1) +
         ne * ((je1 - 1) +
         ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))))));
}
/* pack_GAM.f:196-239 index_GAM_4PK2 (integer*8 result) */
int64_t orc_index_gam_4pk2(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                           int64_t ie1, int64_t je1, int64_t ie2, int64_t je2,
                           int64_t ie3, int64_t je3, int64_t ie4,
                           int64_t je4) {
  return 1 + (je4 - 1) +
         ne * ((ie4 - 1) +
         ne * ((je3 - 1) +
         ne * ((ie3 - 1) +
         ne * ((je2 - 1) +
         ne * ((ie2 - 1) +
         ne * ((je1 - 1) +
         ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))))))));
}
/* gam_2_OMP.f:1080-1095 loop_size */
void orc_loop_size(int64_t L1, int64_t L2, int64_t nproc, int64_t myrank,
                   int64_t *istart, int64_t *iend) {
  int64_t w1 = (L2 - L1 + 1) / nproc;
  int64_t w2 = (L2 - L1 + 1) % nproc;
  *istart = myrank * w1 + L1 + (myrank < w2 ? myrank : w2);
  *iend = *istart + w1 - 1;
  if (w2 > myrank) *iend = *iend + 1;
}

/* ---- basis set-up ------------------------------------------------------ */
/* xcneo_HYBRID.f:1269-1307 make_KPE */
void orc_make_kpe(int64_t nebf, int64_t npebf, const int64_t *AMPEB2C,
                  int64_t *KPESTR, int64_t *KPEEND) {
  int64_t ichk = 1, ist = 1, iend;
  (void)nebf;
  for (int64_t iep = 1; iep <= npebf; iep++) {
    int64_t iec = AMPEB2C[iep - 1];
    if (iec != ichk) {
      ichk = ichk + 1;
      iend = iep - 1;
      KPESTR[iec - 2] = ist;
      KPEEND[iec - 2] = iend;
      ist = iep;
    }
    if (iep == npebf) {
      iend = iep;
      KPESTR[iec - 1] = ist;
      KPEEND[iec - 1] = iend;
    }
  }
}

static void get_prim(int64_t n, const int64_t *AM, const double *EX,
                     const double *BFC, int64_t i /*0-based*/, orc_prim *p) {
  for (int d = 0; d < 3; d++) {
    p->l[d] = (int)AM[i + n * d];
    p->c[d] = BFC[i + n * d];
  }
  p->a = EX[i];
}

/* xchf1_independent/pure_ovlap.f:245-362 ELCNORM3 */
void orc_elcnorm3(int64_t npebf, int64_t nebf, const int64_t *AMPEB2C,
                  double *AGEBFCC, const double *ELCEX, const int64_t *ELCAM,
                  const double *ELCBFC) {
  for (int64_t i = 0; i < npebf; i++) {
    orc_prim A;
    get_prim(npebf, ELCAM, ELCEX, ELCBFC, i, &A);
    double ans = orc_gfovlap(&A, &A);
    AGEBFCC[i] = AGEBFCC[i] / sqrt(ans);
  }
  double *kappa = (double *)calloc((size_t)nebf, sizeof(double));
  for (int64_t i = 0; i < npebf; i++)
    for (int64_t j = 0; j < npebf; j++) {
      int64_t ic = AMPEB2C[i], jc = AMPEB2C[j];
      if (ic == jc) {
        orc_prim A, B;
        get_prim(npebf, ELCAM, ELCEX, ELCBFC, i, &A);
        get_prim(npebf, ELCAM, ELCEX, ELCBFC, j, &B);
        double ans = orc_gfovlap(&A, &B);
        kappa[ic - 1] = kappa[ic - 1] + ans * AGEBFCC[i] * AGEBFCC[j];
      }
    }
  for (int64_t i = 0; i < npebf; i++) {
    double nf = 1.0 / sqrt(kappa[AMPEB2C[i] - 1]);
    AGEBFCC[i] = AGEBFCC[i] * nf;
  }
  free(kappa);
}

/* xcneo_HYBRID.f:1309-1347 NUCNORM (centre placed at the origin) */
void orc_nucnorm(int64_t npbf, double *AGNBFCC, const double *NUCEX,
                 const int64_t *NUCAM, const double *NUCBFC) {
  (void)NUCBFC;
  for (int64_t i = 0; i < npbf; i++) {
    orc_prim A;
    for (int d = 0; d < 3; d++) { A.l[d] = (int)NUCAM[i + npbf * d]; A.c[d] = 0.0; }
    A.a = NUCEX[i];
    double ans = orc_gfovlap(&A, &A);
    ans = 1.0 / sqrt(ans);
    AGNBFCC[i] = AGNBFCC[i] * ans;
  }
}

static void e_prim(const orc_system *s, int64_t i1 /*1-based*/, orc_prim *p) {
  get_prim(s->npebf, s->ELCAM, s->ELCEX, s->ELCBFC, i1 - 1, p);
}
static void p_prim(const orc_system *s, int64_t i1 /*1-based*/, orc_prim *p) {
  get_prim(s->npbf, s->NUCAM, s->NUCEX, s->NUCBFC, i1 - 1, p);
}

static void zero6(double *g) { for (int i = 0; i < 6; i++) g[i] = 0.0; }
enum { A12 = 0, A13, A23, B12, B13, B23 };

/* gam_2_OMP.f:546-1077 xcalc_GAM2_MD.  A/B: particles (e1, e2, p). */
void orc_xcalc_gam2(const orc_prim *A, const orc_prim *B,
                    const orc_system *s, double *ansE, double *ansS) {
  const double zero = 0.0, half = 0.5, two = 2.0, four = 4.0;
  const int ng = (int)s->ngtg, nat = (int)s->nat;
  const double *b = s->bgem, *gm = s->ggem;
  double g[6];
  /* reordered particle sets used by the kernels */
  orc_prim A132[3] = {A[0], A[2], A[1]}, B132[3] = {B[0], B[2], B[1]};
  orc_prim A312[3] = {A[2], A[0], A[1]}, B312[3] = {B[2], B[0], B[1]};
  double gTE = zero, gVEC = zero, gVEE = zero, gVEP = zero;
  for (int ik = 0; ik < ng; ik++) {
    zero6(g);
    g[A23] = gm[ik];
    double xgTE = orc_g3_ke(A, B, g, 1.0);
    double xgVEC = zero;
    for (int ia = 0; ia < nat; ia++) {
      const double *C = s->cat + 3 * ia;
      double ZNUC = s->zan[ia];
      double v = orc_underflow(orc_g3_xgvxcg(A, B, g, C));
      xgVEC = xgVEC - ZNUC * v;
    }
    double xgVEP = orc_underflow(orc_g3_xgveeg(A132, B132, g));
    xgVEP = -xgVEP;
    double xgVEE = orc_underflow(orc_g3_xgveeg(A, B, g));
    gTE = gTE + b[ik] * xgTE;
    gVEC = gVEC + b[ik] * xgVEC;
    gVEP = gVEP + b[ik] * xgVEP;
    gVEE = gVEE + b[ik] * xgVEE;
  }
  double gTPg = zero, gTEg1 = zero, gTEg2 = zero, gTEg3 = zero;
  double gVPCg = zero, gVECg1 = zero, gVECg2 = zero;
  double gVEPg1 = zero, gVEPg2 = zero, gVEEg1 = zero, gVEEg2 = zero;
  double gsg = zero;
  for (int ik = 0; ik < ng; ik++)
    for (int il = 0; il < ng; il++) {
      zero6(g); g[A12] = gm[ik]; g[B13] = gm[il];
      double xgTPg = orc_g3_ke(A312, B312, g, s->pmass);
      zero6(g); g[A13] = gm[ik]; g[B23] = gm[il];
      double xgTEg1 = orc_g3_ke(A, B, g, 1.0);
      zero6(g); g[A23] = gm[ik]; g[B13] = gm[il];
      double xgTEg2 = orc_g3_ke(A, B, g, 1.0);
      zero6(g); g[A23] = gm[ik]; g[B23] = gm[il];
      double xgTEg3 = orc_g3_ke(A, B, g, 1.0);
      double xgVPCg = zero, xgVECg1 = zero, xgVECg2 = zero;
      for (int ia = 0; ia < nat; ia++) {
        const double *C = s->cat + 3 * ia;
        double ZNUC = s->zan[ia];
        zero6(g); g[A12] = gm[ik]; g[B13] = gm[il];
        double v = orc_underflow(orc_g3_xgvxcg(A312, B312, g, C));
        xgVPCg = xgVPCg + ZNUC * v;
        zero6(g); g[A13] = gm[ik]; g[B23] = gm[il];
        v = orc_underflow(orc_g3_xgvxcg(A, B, g, C));
        xgVECg1 = xgVECg1 - ZNUC * v;
        zero6(g); g[A23] = gm[ik]; g[B23] = gm[il];
        v = orc_underflow(orc_g3_xgvxcg(A, B, g, C));
        xgVECg2 = xgVECg2 - ZNUC * v;
      }
      zero6(g); g[A12] = gm[ik]; g[B23] = gm[il];
      double xgVEPg1 = -orc_underflow(orc_g3_xgveeg(A132, B132, g));
      zero6(g); g[A23] = gm[ik]; g[B23] = gm[il];
      double xgVEPg2 = -orc_underflow(orc_g3_xgveeg(A132, B132, g));
      zero6(g); g[A13] = gm[ik]; g[B13] = gm[il];
      double xgVEEg1 = orc_underflow(orc_g3_xgveeg(A, B, g));
      zero6(g); g[A13] = gm[ik]; g[B23] = gm[il];
      double xgVEEg2 = orc_underflow(orc_g3_xgveeg(A, B, g));
      zero6(g); g[A13] = gm[ik]; g[B23] = gm[il];
      double xgsg = orc_g3_xggs(A, B, g);
      double bb = b[ik] * b[il];
      gTPg = gTPg + bb * xgTPg;
      gTEg1 = gTEg1 + bb * xgTEg1;
      gTEg2 = gTEg2 + bb * xgTEg2;
      gTEg3 = gTEg3 + bb * xgTEg3;
      gVPCg = gVPCg + bb * xgVPCg;
      gVECg1 = gVECg1 + bb * xgVECg1;
      gVECg2 = gVECg2 + bb * xgVECg2;
      gVEPg1 = gVEPg1 + bb * xgVEPg1;
      gVEPg2 = gVEPg2 + bb * xgVEPg2;
      gVEEg1 = gVEEg1 + bb * xgVEEg1;
      gVEEg2 = gVEEg2 + bb * xgVEEg2;
      gsg = gsg + bb * xgsg;
    }
  *ansE = two * (gTE + gVEC + gVEP) + four * gVEE * half + gTPg + gVPCg +
          gTEg1 + gTEg3 + two * (gVEPg1 + gVECg1) + gTEg2 + gVEPg2 + gVECg2 +
          two * gVEEg1 * half + two * gVEEg2 * half;
  *ansS = gsg;
}

/* rxchfne/rxchfne_gam_2_OMP.f:2-530 RXCHFne_xcalc_GAM2_MD (live terms
 * :409-456) */
void orc_xcalc_gam2_rxchfne(const orc_prim *A, const orc_prim *B,
                            const orc_system *s, double *ansE1,
                            double *ansE2) {
  const int ng = (int)s->ngtg;
  const double *b = s->bgem, *gm = s->ggem;
  orc_prim A321[3] = {A[2], A[1], A[0]}, B321[3] = {B[2], B[1], B[0]};
  double gVEPg2 = 0.0, gVEEg1 = 0.0, gVEEg2 = 0.0, g[6];
  for (int ik = 0; ik < ng; ik++)
    for (int il = 0; il < ng; il++) {
      zero6(g); g[A13] = gm[ik]; g[B13] = gm[il];
      double xgVEPg2 = -orc_underflow(orc_g3_xgveeg(A321, B321, g));
      zero6(g); g[A13] = gm[ik]; g[B13] = gm[il];
      double xgVEEg1 = orc_underflow(orc_g3_xgveeg(A, B, g));
      zero6(g); g[A13] = gm[ik]; g[B23] = gm[il];
      double xgVEEg2 = orc_underflow(orc_g3_xgveeg(A, B, g));
      gVEPg2 = gVEPg2 + b[ik] * b[il] * xgVEPg2;
      gVEEg1 = gVEEg1 + b[ik] * b[il] * xgVEEg1;
      gVEEg2 = gVEEg2 + b[ik] * b[il] * xgVEEg2;
    }
  *ansE1 = gVEPg2 + gVEEg1;
  *ansE2 = gVEEg2;
}

/* gam_3_OMP.f:617-984 xcalc_GAM3_MD.  A/B: particles (e1, e2, e3, p). */
double orc_xcalc_gam3(const orc_prim *A, const orc_prim *B,
                      const orc_system *s) {
  const double zero = 0.0, one = 1.0, two = 2.0, four = 4.0, half = 0.5;
  const int ng = (int)s->ngtg, nat = (int)s->nat;
  const double *b = s->bgem, *gm = s->ggem;
  double gVEE = zero;
  for (int ik = 0; ik < ng; ik++) {
    double xx = orc_g2_xggs(&A[0], &A[3], &B[0], &B[3], gm[ik], zero);
    double yy = orc_gfvee(&A[1], &A[2], &B[1], &B[2]);
    xx = orc_underflow(xx);
    yy = orc_underflow(yy);
    gVEE = gVEE + (b[ik] * (xx * yy));
  }
  orc_prim A124[3] = {A[0], A[1], A[3]}, B124[3] = {B[0], B[1], B[3]};
  double gHEg = zero, gVEEg1 = zero, gVEEg2 = zero;
  for (int ik = 0; ik < ng; ik++)
    for (int il = 0; il < ng; il++) {
      double csign = -one;
      double xke = orc_gfke(&A[2], &B[2], one);
      double Vc = zero;
      for (int ia = 0; ia < nat; ia++) {
        double vv = orc_gfvec(&A[2], &B[2], s->cat + 3 * ia);
        Vc = Vc + (s->zan[ia] * vv);
      }
      double xx = xke + (Vc * csign);
      double g[6] = {zero, gm[ik], zero, zero, zero, gm[il]};
      double yy = orc_g3_xggs(A124, B124, g);
      double zz = orc_g4_xgvepg(A, B, gm[ik], gm[il]);
      xx = orc_underflow(xx);
      yy = orc_underflow(yy);
      zz = orc_underflow(zz);
      double xgHEg = ((xx * yy) + (zz * csign));
      xx = orc_g2_xggs(&A[0], &A[3], &B[0], &B[3], gm[ik], gm[il]);
      yy = orc_gfvee(&A[1], &A[2], &B[1], &B[2]);
      xx = orc_underflow(xx);
      yy = orc_underflow(yy);
      double xgVEEg1 = xx * yy;
      double xgVEEg2 = orc_g4_xgveeg(A, B, gm[ik], gm[il]);
      gHEg = gHEg + (b[ik] * b[il] * xgHEg);
      gVEEg1 = gVEEg1 + (b[ik] * b[il] * xgVEEg1);
      gVEEg2 = gVEEg2 + (b[ik] * b[il] * xgVEEg2);
    }
  return two * gVEE * half + gHEg + gVEEg1 * half + four * gVEEg2 * half;
}

/* decode a flattened tuple (loop_map order, last index fastest) */
static void decode(int64_t t, int n, const int64_t *dims, int64_t *idx) {
  for (int k = n - 1; k >= 0; k--) {
    idx[k] = t % dims[k] + 1;
    t /= dims[k];
  }
}

/* gam2_CONV_OMP.f:388-579 contract_omega2_conv (and the RXCHF-ne twin,
 * rxchfne_gam2_CONV_OMP.f:2-196): sum over primitive quartets. */
static void contract2(const orc_system *s, int64_t ip, int64_t jp,
                      int64_t iec1, int64_t jec1, int64_t iec2, int64_t jec2,
                      int rx, double *O1, double *O2) {
  double o1 = 0.0, o2 = 0.0;
  orc_prim A[3], B[3];
  p_prim(s, ip, &A[2]);
  p_prim(s, jp, &B[2]);
  double cip = s->AGNBFCC[ip - 1], cjp = s->AGNBFCC[jp - 1];
  for (int64_t ie1 = s->KPESTR[iec1 - 1]; ie1 <= s->KPEEND[iec1 - 1]; ie1++)
  for (int64_t je1 = s->KPESTR[jec1 - 1]; je1 <= s->KPEEND[jec1 - 1]; je1++)
  for (int64_t ie2 = s->KPESTR[iec2 - 1]; ie2 <= s->KPEEND[iec2 - 1]; ie2++)
  for (int64_t je2 = s->KPESTR[jec2 - 1]; je2 <= s->KPEEND[jec2 - 1]; je2++) {
    e_prim(s, ie1, &A[0]); e_prim(s, ie2, &A[1]);
    e_prim(s, je1, &B[0]); e_prim(s, je2, &B[1]);
    double c1 = s->AGEBFCC[ie1 - 1], c2 = s->AGEBFCC[ie2 - 1];
    double d1 = s->AGEBFCC[je1 - 1], d2 = s->AGEBFCC[je2 - 1];
    double a1, a2;
    if (rx) orc_xcalc_gam2_rxchfne(A, B, s, &a1, &a2);
    else orc_xcalc_gam2(A, B, s, &a1, &a2);
    o1 = o1 + a1 * cip * cjp * c1 * d1 * c2 * d2;
    o2 = o2 + a2 * cip * cjp * c1 * d1 * c2 * d2;
  }
  *O1 = o1;
  *O2 = o2;
}

/* gam2_IC1_OMP.f:214-337 thread_gam2_IC1 over tuples [t0,t1) */
void orc_gam2_raw(const orc_system *s, int64_t t0, int64_t t1, double *XG2,
                  double *XG2s) {
  const int64_t ne = s->nebf, np = s->npbf;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = t0; t < t1; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    double o, os;
    contract2(s, x[0], x[1], x[2], x[3], x[4], x[5], 0, &o, &os);
    int64_t ia = orc_index_gam_2pk(ne, np, x[0], x[1], x[2], x[3], x[4], x[5]);
    XG2[ia - 1] = o;
    XG2s[ia - 1] = os;
  }
}

/* gam2_IC1_OMP.f:136-185 pair symmetrisation */
void orc_gam2_symmetrize(int64_t ne, int64_t np, const double *XG2,
                         const double *XG2s, double *GM2, double *GM2s) {
  for (int64_t ip = 1; ip <= np; ip++)
  for (int64_t jp = 1; jp <= np; jp++)
  for (int64_t i1 = 1; i1 <= ne; i1++)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++) {
    int64_t a = orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2);
    int64_t b = orc_index_gam_2pk(ne, np, ip, jp, i2, j2, i1, j1);
    GM2[a - 1] = (XG2[a - 1] + XG2[b - 1]) / 2.0;
    GM2s[a - 1] = (XG2s[a - 1] + XG2s[b - 1]) / 2.0;
  }
}

/* gam2_IC1_OMP.f:2-212 GAM2_IC1 */
void orc_gam2_ic1(const orc_system *s, double *GM2ICR, double *GM2sICR) {
  int64_t ng2 = s->nebf * s->nebf * s->nebf * s->nebf * s->npbf * s->npbf;
  double *X = (double *)malloc(sizeof(double) * ng2);
  double *Xs = (double *)malloc(sizeof(double) * ng2);
  orc_gam2_raw(s, 0, ng2, X, Xs);
  orc_gam2_symmetrize(s->nebf, s->npbf, X, Xs, GM2ICR, GM2sICR);
  free(X);
  free(Xs);
}

/* rxchfne_gam2_IC1_OMP.f:245-340 raw tuples */
void orc_rxchfne_gam2_raw(const orc_system *s, int64_t t0, int64_t t1,
                          double *XG2, double *XG2ex) {
  const int64_t ne = s->nebf, np = s->npbf;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = t0; t < t1; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    double o, ox;
    contract2(s, x[0], x[1], x[2], x[3], x[4], x[5], 1, &o, &ox);
    int64_t ia = orc_index_gam_2pk(ne, np, x[0], x[1], x[2], x[3], x[4], x[5]);
    XG2[ia - 1] = o;
    XG2ex[ia - 1] = ox;
  }
}

/* rxchfne_gam2_IC1_OMP.f:2-243 RXCHFne_GAM2_IC1: GM2ICR raw, GM2exICR
 * pair-averaged (:184-201) */
void orc_rxchfne_gam2_ic1(const orc_system *s, double *GM2ICR,
                          double *GM2exICR) {
  const int64_t ne = s->nebf, np = s->npbf;
  int64_t ng2 = ne * ne * ne * ne * np * np;
  double *X = (double *)malloc(sizeof(double) * ng2);
  double *Xx = (double *)malloc(sizeof(double) * ng2);
  orc_rxchfne_gam2_raw(s, 0, ng2, X, Xx);
  for (int64_t ip = 1; ip <= np; ip++)
  for (int64_t jp = 1; jp <= np; jp++)
  for (int64_t i1 = 1; i1 <= ne; i1++)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++) {
    int64_t a = orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2);
    int64_t b = orc_index_gam_2pk(ne, np, ip, jp, i2, j2, i1, j1);
    GM2ICR[a - 1] = X[a - 1];
    GM2exICR[a - 1] = (Xx[a - 1] + Xx[b - 1]) / 2.0;
  }
  free(X);
  free(Xx);
}

/* gam3_CONV_OMP.f:479-705 contract_omega3_conv */
double orc_contract_omega3(const orc_system *s, int64_t ip, int64_t jp,
                           int64_t iec1, int64_t jec1, int64_t iec2,
                           int64_t jec2, int64_t iec3, int64_t jec3) {
  double o = 0.0;
  orc_prim A[4], B[4];
  p_prim(s, ip, &A[3]);
  p_prim(s, jp, &B[3]);
  double cip = s->AGNBFCC[ip - 1], cjp = s->AGNBFCC[jp - 1];
  const int64_t *KS = s->KPESTR, *KE = s->KPEEND;
  for (int64_t ie1 = KS[iec1 - 1]; ie1 <= KE[iec1 - 1]; ie1++)
  for (int64_t je1 = KS[jec1 - 1]; je1 <= KE[jec1 - 1]; je1++)
  for (int64_t ie2 = KS[iec2 - 1]; ie2 <= KE[iec2 - 1]; ie2++)
  for (int64_t je2 = KS[jec2 - 1]; je2 <= KE[jec2 - 1]; je2++)
  for (int64_t ie3 = KS[iec3 - 1]; ie3 <= KE[iec3 - 1]; ie3++)
  for (int64_t je3 = KS[jec3 - 1]; je3 <= KE[jec3 - 1]; je3++) {
    e_prim(s, ie1, &A[0]); e_prim(s, ie2, &A[1]); e_prim(s, ie3, &A[2]);
    e_prim(s, je1, &B[0]); e_prim(s, je2, &B[1]); e_prim(s, je3, &B[2]);
    const double *C = s->AGEBFCC;
    double ans = orc_xcalc_gam3(A, B, s);
    o = o + ans * cip * cjp * C[ie1 - 1] * C[je1 - 1] * C[ie2 - 1] *
                C[je2 - 1] * C[ie3 - 1] * C[je3 - 1];
  }
  return o;
}

/* gam3_IC1_OMP.f:299-431 thread_gam3_IC1 over tuples [t0,t1) */
void orc_gam3_raw(const orc_system *s, int64_t t0, int64_t t1, double *XG3) {
  const int64_t ne = s->nebf, np = s->npbf;
  const int64_t dims[8] = {np, np, ne, ne, ne, ne, ne, ne};
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = t0; t < t1; t++) {
    int64_t x[8];
    decode(t, 8, dims, x);
    double o = orc_contract_omega3(s, x[0], x[1], x[2], x[3], x[4], x[5],
                                   x[6], x[7]);
    int64_t ia = orc_index_gam_3pk(ne, np, x[0], x[1], x[2], x[3], x[4],
                                   x[5], x[6], x[7]);
    XG3[ia - 1] = o;
  }
}

/* gam3_IC1_OMP.f:143-262 six-permutation symmetrisation; every visited
 * tuple rewrites its whole orbit, so the stored value is the one computed
 * at the orbit's last visit in loop order. */
void orc_gam3_symmetrize(int64_t ne, int64_t np, const double *X,
                         double *G) {
  for (int64_t ip = 1; ip <= np; ip++)
  for (int64_t jp = 1; jp <= np; jp++)
  for (int64_t i1 = 1; i1 <= ne; i1++)
  for (int64_t j1 = 1; j1 <= ne; j1++)
  for (int64_t i2 = 1; i2 <= ne; i2++)
  for (int64_t j2 = 1; j2 <= ne; j2++)
  for (int64_t i3 = 1; i3 <= ne; i3++)
  for (int64_t j3 = 1; j3 <= ne; j3++) {
    int64_t a123 = orc_index_gam_3pk(ne, np, ip, jp, i1, j1, i2, j2, i3, j3);
    int64_t a132 = orc_index_gam_3pk(ne, np, ip, jp, i1, j1, i3, j3, i2, j2);
    int64_t a213 = orc_index_gam_3pk(ne, np, ip, jp, i2, j2, i1, j1, i3, j3);
    int64_t a231 = orc_index_gam_3pk(ne, np, ip, jp, i2, j2, i3, j3, i1, j1);
    int64_t a312 = orc_index_gam_3pk(ne, np, ip, jp, i3, j3, i1, j1, i2, j2);
    int64_t a321 = orc_index_gam_3pk(ne, np, ip, jp, i3, j3, i2, j2, i1, j1);
    double xx = (X[a123 - 1] + X[a132 - 1] + X[a213 - 1] + X[a231 - 1] +
                 X[a312 - 1] + X[a321 - 1]) / 6.0;
    G[a123 - 1] = xx; G[a132 - 1] = xx; G[a213 - 1] = xx;
    G[a231 - 1] = xx; G[a312 - 1] = xx; G[a321 - 1] = xx;
  }
}

/* gam3_IC1_OMP.f:2-297 GAM3_IC1 */
void orc_gam3_ic1(const orc_system *s, double *GM3ICR) {
  const int64_t ne = s->nebf, np = s->npbf;
  int64_t ng3 = ne * ne * ne * ne * ne * ne * np * np;
  double *X = (double *)malloc(sizeof(double) * ng3);
  orc_gam3_raw(s, 0, ng3, X);
  orc_gam3_symmetrize(ne, np, X, GM3ICR);
  free(X);
}

/* gam_ee.f:2-169 calc_GAM_ee (primitive loops, contracted accumulation) */
void orc_calc_gam_ee(const orc_system *s, double *GAM_ee) {
  const int64_t ne = s->nebf, npe = s->npebf;
  memset(GAM_ee, 0, sizeof(double) * (size_t)(ne * ne * ne * ne));
  const double *C = s->AGEBFCC;
  for (int64_t ie1 = 1; ie1 <= npe; ie1++)
  for (int64_t je1 = 1; je1 <= npe; je1++)
  for (int64_t ie2 = 1; ie2 <= npe; ie2++)
  for (int64_t je2 = 1; je2 <= npe; je2++) {
    int64_t ic1 = s->AMPEB2C[ie1 - 1], ic2 = s->AMPEB2C[ie2 - 1];
    int64_t jc1 = s->AMPEB2C[je1 - 1], jc2 = s->AMPEB2C[je2 - 1];
    int64_t ia = orc_pack_4d(ne, ne, ne, jc2, ic2, jc1, ic1);
    orc_prim A1, A2, B1, B2;
    e_prim(s, ie1, &A1); e_prim(s, ie2, &A2);
    e_prim(s, je1, &B1); e_prim(s, je2, &B2);
    double ans = orc_gfvee(&A1, &A2, &B1, &B2);
    GAM_ee[ia - 1] = GAM_ee[ia - 1] + ans * C[ie1 - 1] * C[je1 - 1] *
                                          C[ie2 - 1] * C[je2 - 1];
  }
}

/* ---- gam_4 ------------------------------------------------------------- */
/* gam_4_OMP.f:964-1192 calc_GAM_4_integral */
static double gam4_x(int64_t ne, int64_t np, const double *G2s,
                     const double *Gee, int64_t ip, int64_t jp, int64_t ie1,
                     int64_t je1, int64_t ie2, int64_t je2, int64_t ie3,
                     int64_t je3, int64_t ie4, int64_t je4) {
  const double half = 0.5, six = 6.0;
  double ee34 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je4, ie4, je3, ie3) - 1]);
  double ee24 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je4, ie4, je2, ie2) - 1]);
  double ee23 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je3, ie3, je2, ie2) - 1]);
  double ee14 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je4, ie4, je1, ie1) - 1]);
  double ee13 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je3, ie3, je1, ie1) - 1]);
  double ee12 = orc_underflow(Gee[orc_pack_4d(ne, ne, ne, je2, ie2, je1, ie1) - 1]);
  double gs12 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie1, je1, ie2, je2) - 1]);
  double gs13 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie1, je1, ie3, je3) - 1]);
  double gs14 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie1, je1, ie4, je4) - 1]);
  double gs23 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie2, je2, ie3, je3) - 1]);
  double gs24 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie2, je2, ie4, je4) - 1]);
  double gs34 = orc_underflow(G2s[orc_index_gam_2pk(ne, np, ip, jp, ie3, je3, ie4, je4) - 1]);
  double x1 = half * ee34 * gs12, x2 = half * ee24 * gs13;
  double x3 = half * ee23 * gs14, x4 = half * ee14 * gs23;
  double x5 = half * ee13 * gs24, x6 = half * ee12 * gs34;
  return (x1 + x2 + x3 + x4 + x5 + x6) / six;
}

/* calc_GAM_4_integral for callers outside this file (OMG4_ICR) */
double orc_gam4_raw(int64_t ne, int64_t np, const double *G2s, const double *Gee,
                    int64_t ip, int64_t jp, int64_t ie1, int64_t je1, int64_t ie2,
                    int64_t je2, int64_t ie3, int64_t je3, int64_t ie4, int64_t je4) {
  return gam4_x(ne, np, G2s, Gee, ip, jp, ie1, je1, ie2, je2, ie3, je3, ie4, je4);
}

/* gam_4_OMP.f:921-960 i10: argument order (ie1..ie4, je1..je4) */
static double i10(int64_t ne, int64_t np, const double *G2s, const double *Gee,
                  int64_t ip, int64_t jp, int64_t ie1, int64_t ie2,
                  int64_t ie3, int64_t ie4, int64_t je1, int64_t je2,
                  int64_t je3, int64_t je4) {
  return gam4_x(ne, np, G2s, Gee, ip, jp, ie1, je1, ie2, je2, ie3, je3, ie4,
                je4);
}

/* gam_4_OMP.f:712-918 symm_gam4, then /16 as in GAM4_ICR / GAM4_DSCF */
double orc_gam4_element(int64_t ne, int64_t np, const double *G2s,
                        const double *Gee, int64_t ip, int64_t jp,
                        int64_t ii, int64_t i, int64_t jj, int64_t j,
                        int64_t kk, int64_t k, int64_t ll, int64_t l) {
  const double TWO = 2.0, FOUR = 4.0, EIGHT = FOUR * TWO;
#define X(a, b, c, d) i10(ne, np, G2s, Gee, ip, jp, ii, jj, kk, ll, a, b, c, d)
  double x1 = X(i, j, k, l), x2 = X(j, i, k, l), x3 = X(k, i, j, l);
  double x4 = X(i, k, j, l), x5 = X(j, k, i, l), x6 = X(k, j, i, l);
  double x7 = X(l, j, i, k), x8 = X(j, l, i, k), x9 = X(i, l, j, k);
  double x10 = X(l, i, j, k), x11 = X(j, i, l, k), x12 = X(i, j, l, k);
  double x13 = X(i, k, l, j), x14 = X(k, i, l, j), x15 = X(l, i, k, j);
  double x16 = X(i, l, k, j), x17 = X(k, l, i, j), x18 = X(l, k, i, j);
  double x19 = X(l, k, j, i), x20 = X(k, l, j, i), x21 = X(j, l, k, i);
  double x22 = X(l, j, k, i), x23 = X(k, j, l, i), x24 = X(j, k, l, i);
#undef X
  double ans = (FOUR * FOUR * x1) - (EIGHT * x2) + (FOUR * x3) -
               (EIGHT * x4) + (FOUR * x5) - (EIGHT * x6) + (FOUR * x7) -
               (TWO * x8) + (FOUR * x9) - (TWO * x10) + (FOUR * x11) -
               (EIGHT * x12) + (FOUR * x13) - (TWO * x14) + (FOUR * x15) -
               (EIGHT * x16) + (FOUR * x17) - (TWO * x18) + (FOUR * x19) -
               (TWO * x20) + (FOUR * x21) - (EIGHT * x22) + (FOUR * x23) -
               (TWO * x24);
  return ans / (FOUR * FOUR);
}

/* gam4_ICR_OMP.f:2-271 GAM4_ICR */
void orc_gam4_icr(int64_t ne, int64_t np, const double *G2s,
                  const double *Gee, double *G4) {
  const int64_t dims[10] = {np, np, ne, ne, ne, ne, ne, ne, ne, ne};
  int64_t ng4 = ne * ne * ne * ne * ne * ne * ne * ne * np * np;
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < ng4; t++) {
    int64_t x[10];
    decode(t, 10, dims, x);
    int64_t ia = orc_index_gam_4pk2(ne, np, x[0], x[1], x[2], x[3], x[4],
                                    x[5], x[6], x[7], x[8], x[9]);
    G4[ia - 1] = orc_gam4_element(ne, np, G2s, Gee, x[0], x[1], x[2], x[3],
                                  x[4], x[5], x[6], x[7], x[8], x[9]);
  }
}

#define DE_(i, j) DE[((i) - 1) + ne * ((j) - 1)]
#define DP_(i, j) DP[((i) - 1) + np * ((j) - 1)]

/* gam4_DSCF_OMP.f:141-320 thread_gam4_DSCF over tuples [t0,t1): adds into
 * xfocke/xfockp/E (sequential, loop_map order). */
void orc_gam4_dscf_range(int64_t ne, int64_t np, const double *Gee,
                         const double *G2s, const double *DE,
                         const double *DP, int64_t t0, int64_t t1,
                         double *xfe, double *xfp, double *E) {
  const double four = 4.0;
  const int64_t dims[10] = {np, np, ne, ne, ne, ne, ne, ne, ne, ne};
  for (int64_t t = t0; t < t1; t++) {
    int64_t x[10];
    decode(t, 10, dims, x);
    int64_t ip = x[0], jp = x[1], ie1 = x[2], je1 = x[3], ie2 = x[4],
            je2 = x[5], ie3 = x[6], je3 = x[7], ie4 = x[8], je4 = x[9];
    double ans = orc_gam4_element(ne, np, G2s, Gee, ip, jp, ie1, je1, ie2,
                                  je2, ie3, je3, ie4, je4);
    xfe[(ie1 - 1) + ne * (je1 - 1)] +=
        DP_(ip, jp) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) * four * ans;
    xfp[(ip - 1) + np * (jp - 1)] +=
        DE_(ie1, je1) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) * ans;
    *E = *E + DE_(ie1, je1) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) *
                  DP_(ip, jp) * ans;
  }
}

/* gam4_DSCF_OMP.f:2-139 GAM4_DSCF */
void orc_gam4_dscf(int64_t ne, int64_t np, const double *Gee,
                   const double *G2s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *E_gam4) {
  int64_t ng4 = ne * ne * ne * ne * ne * ne * ne * ne * np * np;
  int nt = orc_num_threads();
  double *xfe = (double *)calloc((size_t)(ne * ne * nt), sizeof(double));
  double *xfp = (double *)calloc((size_t)(np * np * nt), sizeof(double));
  double *Ep = (double *)calloc((size_t)nt, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nt; c++) {
    int64_t a, b;
    orc_loop_size(0, ng4 - 1, nt, c, &a, &b);
    orc_gam4_dscf_range(ne, np, Gee, G2s, DE, DP, a, b + 1, xfe + ne * ne * c,
                        xfp + np * np * c, Ep + c);
  }
  double E = 0.0;
  for (int c = 0; c < nt; c++) {
    E += Ep[c];
    for (int64_t k = 0; k < ne * ne; k++) focke[k] += xfe[ne * ne * c + k];
    for (int64_t k = 0; k < np * np; k++) fockp[k] += xfp[np * np * c + k];
  }
  *E_gam4 = E;
  free(xfe); free(xfp); free(Ep);
}

/* gam4_ICR_OMP.f:273-490 EG4ICR */
void orc_eg4icr(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *GM4, double *focke, double *fockp, double *E) {
  const double four = 4.0;
  int64_t ng4 = ne * ne * ne * ne * ne * ne * ne * ne * np * np;
  const int64_t dims[10] = {np, np, ne, ne, ne, ne, ne, ne, ne, ne};
  double *xfe = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double *xfp = (double *)calloc((size_t)(np * np), sizeof(double));
  double e = 0.0;
  for (int64_t t = 0; t < ng4; t++) {
    int64_t x[10];
    decode(t, 10, dims, x);
    int64_t ip = x[0], jp = x[1], ie1 = x[2], je1 = x[3], ie2 = x[4],
            je2 = x[5], ie3 = x[6], je3 = x[7], ie4 = x[8], je4 = x[9];
    double ans = GM4[orc_index_gam_4pk2(ne, np, ip, jp, ie1, je1, ie2, je2,
                                        ie3, je3, ie4, je4) - 1];
    xfe[(ie1 - 1) + ne * (je1 - 1)] +=
        DP_(ip, jp) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) * four * ans;
    xfp[(ip - 1) + np * (jp - 1)] +=
        DE_(ie1, je1) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) * ans;
    e = e + DE_(ie1, je1) * DE_(ie2, je2) * DE_(ie3, je3) * DE_(ie4, je4) *
                DP_(ip, jp) * ans;
  }
  for (int64_t k = 0; k < ne * ne; k++) focke[k] += xfe[k];
  for (int64_t k = 0; k < np * np; k++) fockp[k] += xfp[k];
  *E = e;
  free(xfe); free(xfp);
}

/* gam3_IC1_OMP.f:433-725 EG3IC1 / thread_EG3ICR */
void orc_eg3ic1(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *G, double *focke, double *fockp, double *E) {
  int64_t ng3 = ne * ne * ne * ne * ne * ne * np * np;
  const int64_t dims[8] = {np, np, ne, ne, ne, ne, ne, ne};
  double *xfe = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double *xfp = (double *)calloc((size_t)(np * np), sizeof(double));
  double e = 0.0;
  for (int64_t t = 0; t < ng3; t++) {
    int64_t x[8];
    decode(t, 8, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5],
            i3 = x[6], j3 = x[7];
#define G3(a, b, c, d, e_, f) G[orc_index_gam_3pk(ne, np, ip, jp, a, b, c, d, e_, f) - 1]
    double o123 = G3(i1, j1, i2, j2, i3, j3);
    double o213 = G3(i1, j2, i2, j1, i3, j3);
    double o312 = G3(i1, j3, i2, j1, i3, j2);
    double o132 = G3(i1, j1, i2, j3, i3, j2);
    double o231 = G3(i1, j2, i2, j3, i3, j1);
    double o321 = G3(i1, j3, i2, j2, i3, j1);
#undef G3
    double g3 = 8.0 * o123 - 4.0 * o213 + 2.0 * o312 - 4.0 * o132 +
                2.0 * o231 - 4.0 * o321;
    g3 = g3 / 8.0;
    xfe[(i1 - 1) + ne * (j1 - 1)] +=
        DP_(ip, jp) * DE_(i2, j2) * DE_(i3, j3) * 3.0 * g3;
    xfp[(ip - 1) + np * (jp - 1)] += DE_(i1, j1) * DE_(i2, j2) * DE_(i3, j3) * g3;
    e = e + DE_(i1, j1) * DE_(i2, j2) * DE_(i3, j3) * DP_(ip, jp) * g3;
  }
  for (int64_t k = 0; k < ne * ne; k++) focke[k] += xfe[k];
  for (int64_t k = 0; k < np * np; k++) fockp[k] += xfp[k];
  *E = e;
  free(xfe); free(xfp);
}

/* gam2_IC1_OMP.f:339-570 EG2IC1 / thread_EG2ICR: FE, FP accumulate;
 * SE, SP are overwritten (zeroed at :379-381). */
void orc_eg2ic1(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *GM2, const double *GM2s, double *FE, double *SE,
                double *FP, double *SP, double *E_gam2, double *S_gam2) {
  const double half = 0.5, two = 2.0;
  int64_t ng2 = ne * ne * ne * ne * np * np;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
  double *xfe = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double *xfp = (double *)calloc((size_t)(np * np), sizeof(double));
  memset(SE, 0, sizeof(double) * (size_t)(ne * ne));
  memset(SP, 0, sizeof(double) * (size_t)(np * np));
  double e = 0.0, s = 0.0;
  for (int64_t t = 0; t < ng2; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5];
    int64_t a12 = orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2);
    int64_t a21 = orc_index_gam_2pk(ne, np, ip, jp, i1, j2, i2, j1);
    double v = GM2[a12 - 1] - half * GM2[a21 - 1];
    double vs = GM2s[a12 - 1] - half * GM2s[a21 - 1];
    xfe[(i1 - 1) + ne * (j1 - 1)] += DP_(ip, jp) * DE_(i2, j2) * two * v;
    SE[(i1 - 1) + ne * (j1 - 1)] += DP_(ip, jp) * DE_(i2, j2) * vs;
    xfp[(ip - 1) + np * (jp - 1)] += DE_(i1, j1) * DE_(i2, j2) * v;
    SP[(ip - 1) + np * (jp - 1)] += DE_(i1, j1) * DE_(i2, j2) * vs;
    e = e + DE_(i1, j1) * DE_(i2, j2) * DP_(ip, jp) * v;
    s = s + DE_(i1, j1) * DE_(i2, j2) * DP_(ip, jp) * vs;
  }
  for (int64_t k = 0; k < ne * ne; k++) FE[k] += xfe[k];
  for (int64_t k = 0; k < np * np; k++) FP[k] += xfp[k];
  *E_gam2 = e;
  *S_gam2 = s;
  free(xfe); free(xfp);
}

#undef DE_
#define DA_(i, j) DAE[((i) - 1) + ne * ((j) - 1)]
#define DB_(i, j) DBE[((i) - 1) + ne * ((j) - 1)]

/* rxchfne/rxchfne_omg2.f:2-210 RXCHFne_FAE_OMG2 (+ thread :118) */
void orc_rxchfne_fae_omg2(int64_t ne, int64_t np, const double *DAE,
                          const double *DBE, const double *DP,
                          const double *GM2, double *FAE, double *E) {
  int64_t ng2 = ne * ne * ne * ne * np * np;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
  double *xf = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double e = 0.0;
  for (int64_t t = 0; t < ng2; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5];
    double v = GM2[orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2) - 1];
    xf[(i2 - 1) + ne * (j2 - 1)] += DP_(ip, jp) * DB_(i1, j1) * v;
    e = e + DP_(ip, jp) * DA_(i2, j2) * DB_(i1, j1) * v;
  }
  for (int64_t k = 0; k < ne * ne; k++) FAE[k] += xf[k];
  *E = e;
  free(xf);
}

/* rxchfne/rxchfne_omg2.f:212-407 RXCHFne_FP_OMG2 */
void orc_rxchfne_fp_omg2(int64_t ne, int64_t np, const double *DAE,
                         const double *DBE, const double *DP,
                         const double *GM2, double *FP, double *E) {
  int64_t ng2 = ne * ne * ne * ne * np * np;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
  double *xf = (double *)calloc((size_t)(np * np), sizeof(double));
  double e = 0.0;
  for (int64_t t = 0; t < ng2; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5];
    double v = GM2[orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2) - 1];
    xf[(ip - 1) + np * (jp - 1)] += DA_(i2, j2) * DB_(i1, j1) * v;
    e = e + DP_(ip, jp) * DA_(i2, j2) * DB_(i1, j1) * v;
  }
  for (int64_t k = 0; k < np * np; k++) FP[k] += xf[k];
  *E = e;
  free(xf);
}

/* rxchfne/rxchfne_omg2.f:409-600 RXCHFne_FBE_OMG2 */
void orc_rxchfne_fbe_omg2(int64_t ne, int64_t np, const double *DAE,
                          const double *DBE, const double *DP,
                          const double *GM2, double *FBE, double *E) {
  int64_t ng2 = ne * ne * ne * ne * np * np;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
  double *xf = (double *)calloc((size_t)(ne * ne), sizeof(double));
  double e = 0.0;
  for (int64_t t = 0; t < ng2; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5];
    double v = GM2[orc_index_gam_2pk(ne, np, ip, jp, i1, j1, i2, j2) - 1];
    xf[(i1 - 1) + ne * (j1 - 1)] += DA_(i2, j2) * DP_(ip, jp) * v;
    e = e + DP_(ip, jp) * DA_(i2, j2) * DB_(i1, j1) * v;
  }
  for (int64_t k = 0; k < ne * ne; k++) FBE[k] += xf[k];
  *E = e;
  free(xf);
}
#undef DA_
#undef DB_
#undef DP_

/* xchf1_independent/xchf1_fock.f:728-783 XCfock_correction */
void orc_xcfock_correction(int64_t ne, int64_t np, double S_total,
                           double H_expect, const double *se1,
                           const double *sp1, const double *se2,
                           const double *sp2, double *focke, double *fockp) {
  const double one = 1.0, two = 2.0;
  for (int64_t i = 0; i < ne; i++)
    for (int64_t j = 0; j < ne; j++) {
      int64_t k = i + ne * j;
      focke[k] = (one / S_total) * focke[k] - H_expect * (se1[k] + two * se2[k]);
    }
  for (int64_t i = 0; i < np; i++)
    for (int64_t j = 0; j < np; j++) {
      int64_t k = i + np * j;
      fockp[k] = (one / S_total) * fockp[k] - H_expect * (sp1[k] + sp2[k]);
    }
}

/* xchf1_independent/GAM_IO.f:247-345 read_elec_density (density part) */
void orc_density(int64_t nbf, int64_t nocc, double prefac, const double *C,
                 double *D) {
  for (int64_t i = 0; i < nbf; i++)
    for (int64_t j = 0; j < nbf; j++) {
      double d = 0.0;
      for (int64_t k = 0; k < nocc; k++)
        d = d + prefac * C[i + nbf * k] * C[j + nbf * k];
      D[i + nbf * j] = d;
    }
}

/* Bounded sample of GAM4_DSCF work: tuples [t0,t1) split over the OpenMP
 * threads (thread_gam4_DSCF's parallel loop, gam4_DSCF_OMP.f:230-309);
 * partial Fock matrices and energy are summed into the outputs.  Used as the
 * timed CPU baseline. */
void orc_gam4_dscf_sample(int64_t ne, int64_t np, const double *Gee,
                          const double *G2s, const double *DE,
                          const double *DP, int64_t t0, int64_t t1,
                          double *focke, double *fockp, double *E) {
  int nt = orc_num_threads();
  double *xfe = (double *)calloc((size_t)(ne * ne * nt), sizeof(double));
  double *xfp = (double *)calloc((size_t)(np * np * nt), sizeof(double));
  double *Ep = (double *)calloc((size_t)nt, sizeof(double));
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nt; c++) {
    int64_t a, b;
    orc_loop_size(t0, t1 - 1, nt, c, &a, &b);
    orc_gam4_dscf_range(ne, np, Gee, G2s, DE, DP, a, b + 1, xfe + ne * ne * c,
                        xfp + np * np * c, Ep + c);
  }
  for (int c = 0; c < nt; c++) {
    *E += Ep[c];
    for (int64_t k = 0; k < ne * ne; k++) focke[k] += xfe[ne * ne * c + k];
    for (int64_t k = 0; k < np * np; k++) fockp[k] += xfp[np * np * c + k];
  }
  free(xfe); free(xfp); free(Ep);
}

/* ---- direct-SCF builders ------------------------------------------------ */
#define DEo(i, j) DE[((i) - 1) + ne * ((j) - 1)]
#define DPo(i, j) DP[((i) - 1) + np * ((j) - 1)]

/* gam2_DSCF_OMP.f:330-559 contract_omega2 (direct): the pair-symmetrised
 * OMG2/OMG2s of one contracted tuple, half*(OMG2_12 + OMG2_21). */
static void contract_omega2_direct(const orc_system *s, int64_t ip, int64_t jp,
                                   int64_t iec1, int64_t jec1, int64_t iec2,
                                   int64_t jec2, double *O, double *Os) {
  double o12 = 0.0, o21 = 0.0, s12 = 0.0, s21 = 0.0;
  orc_prim A[3], B[3], A2[3], B2[3];
  p_prim(s, ip, &A[2]);
  p_prim(s, jp, &B[2]);
  double cip = s->AGNBFCC[ip - 1], cjp = s->AGNBFCC[jp - 1];
  for (int64_t ie1 = s->KPESTR[iec1 - 1]; ie1 <= s->KPEEND[iec1 - 1]; ie1++)
  for (int64_t je1 = s->KPESTR[jec1 - 1]; je1 <= s->KPEEND[jec1 - 1]; je1++)
  for (int64_t ie2 = s->KPESTR[iec2 - 1]; ie2 <= s->KPEEND[iec2 - 1]; ie2++)
  for (int64_t je2 = s->KPESTR[jec2 - 1]; je2 <= s->KPEEND[jec2 - 1]; je2++) {
    e_prim(s, ie1, &A[0]); e_prim(s, ie2, &A[1]);
    e_prim(s, je1, &B[0]); e_prim(s, je2, &B[1]);
    A2[0] = A[1]; A2[1] = A[0]; A2[2] = A[2];
    B2[0] = B[1]; B2[1] = B[0]; B2[2] = B[2];
    double c = cip * cjp * s->AGEBFCC[ie1 - 1] * s->AGEBFCC[je1 - 1] *
               s->AGEBFCC[ie2 - 1] * s->AGEBFCC[je2 - 1];
    double aE, aS;
    orc_xcalc_gam2(A, B, s, &aE, &aS);
    o12 = o12 + aE * c;
    s12 = s12 + aS * c;
    orc_xcalc_gam2(A2, B2, s, &aE, &aS);
    o21 = o21 + aE * c;
    s21 = s21 + aS * c;
  }
  *O = 0.5 * (o12 + o21);
  *Os = 0.5 * (s12 + s21);
}

/* gam2_DSCF_OMP.f:2-140 GAM2_DSCF and :143-327 thread_gam2: focke, fockp,
 * se2, sp2 accumulate (add2fock); E_gam2, S_gam2 overwritten.  Threads
 * split the tuples like the reference's OpenMP loop (array reductions). */
void orc_gam2_dscf(const orc_system *s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *se2, double *sp2,
                   double *E_gam2, double *S_gam2) {
  const int64_t ne = s->nebf, np = s->npbf;
  const int64_t dims[6] = {np, np, ne, ne, ne, ne};
  int64_t ng2 = ne * ne * ne * ne * np * np;
  double e = 0.0, sg = 0.0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : e, sg) \
    reduction(+ : focke[0 : ne * ne], se2[0 : ne * ne])             \
    reduction(+ : fockp[0 : np * np], sp2[0 : np * np])
  for (int64_t t = 0; t < ng2; t++) {
    int64_t x[6];
    decode(t, 6, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5];
    double o12, s12, o21, s21;
    contract_omega2_direct(s, ip, jp, i1, j1, i2, j2, &o12, &s12);
    contract_omega2_direct(s, ip, jp, i1, j2, i2, j1, &o21, &s21);
    double g = o12 - 0.5 * o21, gs = s12 - 0.5 * s21;
    focke[(i1 - 1) + ne * (j1 - 1)] += DPo(ip, jp) * DEo(i2, j2) * 2.0 * g;
    fockp[(ip - 1) + np * (jp - 1)] += DEo(i1, j1) * DEo(i2, j2) * g;
    e = e + DEo(i1, j1) * DEo(i2, j2) * DPo(ip, jp) * g;
    se2[(i1 - 1) + ne * (j1 - 1)] += DPo(ip, jp) * DEo(i2, j2) * gs;
    sp2[(ip - 1) + np * (jp - 1)] += DEo(i1, j1) * DEo(i2, j2) * gs;
    sg = sg + DEo(i1, j1) * DEo(i2, j2) * DPo(ip, jp) * gs;
  }
  *E_gam2 = e;
  *S_gam2 = sg;
}

/* gam3_DSCF_OMP.f:367-717 contract_omega3 (direct): the six particle
 * orderings of one contracted tuple evaluated and averaged. */
static double contract_omega3_direct(const orc_system *s, int64_t ip,
                                     int64_t jp, int64_t iec1, int64_t jec1,
                                     int64_t iec2, int64_t jec2, int64_t iec3,
                                     int64_t jec3) {
  static const int ord[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  double o[6] = {0, 0, 0, 0, 0, 0};
  orc_prim A[4], B[4], PA[4], PB[4];
  p_prim(s, ip, &A[3]);
  p_prim(s, jp, &B[3]);
  double cip = s->AGNBFCC[ip - 1], cjp = s->AGNBFCC[jp - 1];
  const int64_t *KS = s->KPESTR, *KE = s->KPEEND;
  const double *C = s->AGEBFCC;
  for (int64_t ie1 = KS[iec1 - 1]; ie1 <= KE[iec1 - 1]; ie1++)
  for (int64_t je1 = KS[jec1 - 1]; je1 <= KE[jec1 - 1]; je1++)
  for (int64_t ie2 = KS[iec2 - 1]; ie2 <= KE[iec2 - 1]; ie2++)
  for (int64_t je2 = KS[jec2 - 1]; je2 <= KE[jec2 - 1]; je2++)
  for (int64_t ie3 = KS[iec3 - 1]; ie3 <= KE[iec3 - 1]; ie3++)
  for (int64_t je3 = KS[jec3 - 1]; je3 <= KE[jec3 - 1]; je3++) {
    e_prim(s, ie1, &A[0]); e_prim(s, ie2, &A[1]); e_prim(s, ie3, &A[2]);
    e_prim(s, je1, &B[0]); e_prim(s, je2, &B[1]); e_prim(s, je3, &B[2]);
    double c = cip * cjp * C[ie1 - 1] * C[je1 - 1] * C[ie2 - 1] * C[je2 - 1] *
               C[ie3 - 1] * C[je3 - 1];
    for (int k = 0; k < 6; k++) {
      for (int m = 0; m < 3; m++) { PA[m] = A[ord[k][m]]; PB[m] = B[ord[k][m]]; }
      PA[3] = A[3];
      PB[3] = B[3];
      o[k] = o[k] + orc_xcalc_gam3(PA, PB, s) * c;
    }
  }
  return (o[0] + o[1] + o[2] + o[3] + o[4] + o[5]) / 6.0;
}

/* gam3_DSCF_OMP.f:2-137 GAM3_DSCF and :140-364 thread_gam3: Fock
 * accumulate, E overwritten (OpenMP array reductions over the tuples). */
void orc_gam3_dscf(const orc_system *s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *E_gam3) {
  const int64_t ne = s->nebf, np = s->npbf;
  const int64_t dims[8] = {np, np, ne, ne, ne, ne, ne, ne};
  int64_t ng3 = ne * ne * ne * ne * ne * ne * np * np;
  double e = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : e) \
    reduction(+ : focke[0 : ne * ne], fockp[0 : np * np])
  for (int64_t t = 0; t < ng3; t++) {
    int64_t x[8];
    decode(t, 8, dims, x);
    int64_t ip = x[0], jp = x[1], i1 = x[2], j1 = x[3], i2 = x[4], j2 = x[5],
            i3 = x[6], j3 = x[7];
    double o123 = contract_omega3_direct(s, ip, jp, i1, j1, i2, j2, i3, j3);
    double o213 = contract_omega3_direct(s, ip, jp, i1, j2, i2, j1, i3, j3);
    double o312 = contract_omega3_direct(s, ip, jp, i1, j3, i2, j1, i3, j2);
    double o132 = contract_omega3_direct(s, ip, jp, i1, j1, i2, j3, i3, j2);
    double o231 = contract_omega3_direct(s, ip, jp, i1, j2, i2, j3, i3, j1);
    double o321 = contract_omega3_direct(s, ip, jp, i1, j3, i2, j2, i3, j1);
    double g = 8.0 * o123 - 4.0 * o213 + 2.0 * o312 - 4.0 * o132 +
               2.0 * o231 - 4.0 * o321;
    g = g / 8.0;
    focke[(i1 - 1) + ne * (j1 - 1)] += DPo(ip, jp) * DEo(i2, j2) * DEo(i3, j3) * 3.0 * g;
    fockp[(ip - 1) + np * (jp - 1)] += DEo(i1, j1) * DEo(i2, j2) * DEo(i3, j3) * g;
    e = e + DEo(i1, j1) * DEo(i2, j2) * DEo(i3, j3) * DPo(ip, jp) * g;
  }
  *E_gam3 = e;
}
#undef DEo
#undef DPo
