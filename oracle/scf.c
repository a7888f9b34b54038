/*
 * scf.c -- ORACLE (test infrastructure only; never linked by the product).
 *
 * CPU restatement of the one- and two-particle integrals the XCHF SCF
 * driver needs besides gam_2/3/4: contracted overlaps (pure_ovlap.f),
 * electronic / nuclear core Hamiltonians (gam_epcore.f), electron-proton
 * Coulomb (gam_ep.f), the geminal gam_1 / gam_1s tensors (gam_1_OMP.f) and
 * the classical nuclear repulsion (class_nuc_rep.f).  Loop order, packing
 * and accumulation order follow the cited routines.
 */
#include "neoxc_oracle.h"
#include <math.h>
#include <string.h>

static void get_prim(int64_t n, const int64_t *AM, const double *EX,
                     const double *BFC, int64_t i, orc_prim *p) {
  for (int d = 0; d < 3; d++) {
    p->l[d] = (int)AM[i + n * d];
    p->c[d] = BFC[i + n * d];
  }
  p->a = EX[i];
}
static void e_prim(const orc_system *s, int64_t i1, orc_prim *p) {
  get_prim(s->npebf, s->ELCAM, s->ELCEX, s->ELCBFC, i1 - 1, p);
}
static void p_prim(const orc_system *s, int64_t i1, orc_prim *p) {
  get_prim(s->npbf, s->NUCAM, s->NUCEX, s->NUCBFC, i1 - 1, p);
}

/* pack_GAM.f pack_2D(n, j, i) = j + n*(i-1) */
static int64_t pack_2d(int64_t n, int64_t j, int64_t i) { return j + n * (i - 1); }

/* xchf1_independent/pure_ovlap.f:2-104 elec_ovlap, :107-202 nuc_ovlap */
void orc_overlaps(const orc_system *s, double *Se, double *Sp) {
  const int64_t ne = s->nebf, npe = s->npebf, np = s->npbf;
  memset(Se, 0, sizeof(double) * (size_t)(ne * ne));
  for (int64_t ie1 = 1; ie1 <= npe; ie1++)
    for (int64_t je1 = 1; je1 <= npe; je1++) {
      int64_t ia = pack_2d(ne, s->AMPEB2C[je1 - 1], s->AMPEB2C[ie1 - 1]);
      orc_prim A, B;
      e_prim(s, ie1, &A);
      e_prim(s, je1, &B);
      double ans = orc_gfovlap(&A, &B);
      Se[ia - 1] = Se[ia - 1] + ans * s->AGEBFCC[ie1 - 1] * s->AGEBFCC[je1 - 1];
    }
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++) {
      orc_prim A, B;
      p_prim(s, ip, &A);
      p_prim(s, jp, &B);
      double ans = orc_gfovlap(&A, &B);
      Sp[pack_2d(np, jp, ip) - 1] = ans * s->AGNBFCC[ip - 1] * s->AGNBFCC[jp - 1];
    }
}

/* gam_epcore.f:200-270 xcalc_GAM_epcore: kinetic + Coulomb to the classical
 * nuclei with sign coul_sign */
static double xcalc_epcore(const orc_prim *A, const orc_prim *B,
                           const orc_system *s, double xmass,
                           double coul_sign) {
  double ans_ke = orc_gfke(A, B, xmass);
  double ans_vec = 0.0;
  for (int64_t k = 0; k < s->nat; k++) {
    const double C[3] = {s->cat[3 * k], s->cat[3 * k + 1], s->cat[3 * k + 2]};
    double xans = orc_gfvec(A, B, C);
    ans_vec = ans_vec + coul_sign * s->zan[k] * xans;
  }
  return ans_ke + ans_vec;
}

/* gam_epcore.f:2-197 calc_GAM_epcore -> GAM_ecore(nebf^2), GAM_pcore(npbf^2),
 * packed by pack_2D(n, j, i) */
void orc_gam_epcore(const orc_system *s, double *Gecore, double *Gpcore) {
  const int64_t ne = s->nebf, npe = s->npebf, np = s->npbf;
  memset(Gecore, 0, sizeof(double) * (size_t)(ne * ne));
  for (int64_t ie1 = 1; ie1 <= npe; ie1++)
    for (int64_t je1 = 1; je1 <= npe; je1++) {
      int64_t ia = pack_2d(ne, s->AMPEB2C[je1 - 1], s->AMPEB2C[ie1 - 1]);
      orc_prim A, B;
      e_prim(s, ie1, &A);
      e_prim(s, je1, &B);
      double ans = xcalc_epcore(&A, &B, s, 1.0, -1.0);
      Gecore[ia - 1] = Gecore[ia - 1] + ans * s->AGEBFCC[ie1 - 1] * s->AGEBFCC[je1 - 1];
    }
  memset(Gpcore, 0, sizeof(double) * (size_t)(np * np));
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++) {
      int64_t ia = pack_2d(np, jp, ip);
      orc_prim A, B;
      p_prim(s, ip, &A);
      p_prim(s, jp, &B);
      double ans = xcalc_epcore(&A, &B, s, s->pmass, 1.0);
      Gpcore[ia - 1] = Gpcore[ia - 1] + ans * s->AGNBFCC[ip - 1] * s->AGNBFCC[jp - 1];
    }
}

/* gam_ep.f:2-164 calc_GAM_ep and :167-219 xcalc_GAM_ep -> GAM_ep(ng1),
 * packed by pack_4D(nebf,nebf,npbf, jec1,iec1,jp,ip) */
void orc_gam_ep(const orc_system *s, double *Gep) {
  const int64_t ne = s->nebf, npe = s->npebf, np = s->npbf;
  memset(Gep, 0, sizeof(double) * (size_t)(ne * ne * np * np));
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++)
      for (int64_t ie1 = 1; ie1 <= npe; ie1++)
        for (int64_t je1 = 1; je1 <= npe; je1++) {
          int64_t iec1 = s->AMPEB2C[ie1 - 1], jec1 = s->AMPEB2C[je1 - 1];
          int64_t ia = orc_pack_4d(ne, ne, np, jec1, iec1, jp, ip);
          orc_prim A1, A2, B1, B2;
          e_prim(s, ie1, &A1);
          p_prim(s, ip, &A2);
          e_prim(s, je1, &B1);
          p_prim(s, jp, &B2);
          double ans = orc_gfvee(&A1, &A2, &B1, &B2);
          ans = ans * -1.0;
          Gep[ia - 1] = Gep[ia - 1] + ans * s->AGNBFCC[ip - 1] * s->AGNBFCC[jp - 1] *
                                          s->AGEBFCC[ie1 - 1] * s->AGEBFCC[je1 - 1];
        }
}

/* gam_1_OMP.f:398-836 xcalc_GAM1_MD: A = (e1, p), B = (e1', p').
 * with_single = 0 is rxchf/rxchf_gam_1_OMP.f RXCHF_xcalc_GAM1_MD: the same
 * sums without the single-geminal terms (tegx, texg, VCEGX, ..., OGX stay
 * zero), only the geminal-pair loop. */
static void xcalc_gam1(const orc_prim *A, const orc_prim *B, const orc_system *s,
                       int with_single, double *ansE, double *ansS) {
  const double zero = 0.0, one = 1.0;
  const int ng = (int)s->ngtg;
  const double pmass = s->pmass;
  double tegx = zero, tpgx = zero, texg = zero, tpxg = zero, tegg = zero,
         tpgg = zero, VCEGX = zero, VCEGG = zero, VCPGX = zero, VCPGG = zero,
         VMGX = zero, VMGG = zero, sval;
  for (int k = 0; k < ng; k++) {
    double GV = s->ggem[k], BCFV = s->bgem[k];
    if (with_single) {
      double tegxi = orc_pgike1(&A[0], &A[1], &B[0], &B[1], GV, zero, one, &sval);
      double tpgxi = orc_pgike1(&A[1], &A[0], &B[1], &B[0], GV, zero, pmass, &sval);
      tegx = tegx + BCFV * tegxi;
      tpgx = tpgx + BCFV * tpgxi;
      double VCEGXI = zero, VCPGXI = zero;
      for (int64_t c = 0; c < s->nat; c++) {
        const double C[3] = {s->cat[3 * c], s->cat[3 * c + 1], s->cat[3 * c + 2]};
        double ZNUC = s->zan[c];
        double a = orc_g2_xggvec(&A[0], &A[1], &B[0], &B[1], GV, zero, C);
        VCEGXI = a * ZNUC + VCEGXI;
        double b = orc_g2_xggvec(&A[1], &A[0], &B[1], &B[0], GV, zero, C);
        VCPGXI = b * ZNUC + VCPGXI;
      }
      double VMGXI = orc_g2_xggvee(&A[0], &A[1], &B[0], &B[1], GV, zero);
      VCEGX = VCEGX + BCFV * VCEGXI;
      VCPGX = VCPGX + BCFV * VCPGXI;
      VMGX = VMGX + BCFV * VMGXI;
      double texgi = orc_pgike1(&A[0], &A[1], &B[0], &B[1], zero, GV, one, &sval);
      double tpxgi = orc_pgike1(&A[1], &A[0], &B[1], &B[0], zero, GV, pmass, &sval);
      texg = texg + BCFV * texgi;
      tpxg = tpxg + BCFV * tpxgi;
    }
    for (int l = 0; l < ng; l++) {
      double GW = s->ggem[l], BCFW = s->bgem[l];
      double teggi = orc_pgike1(&A[0], &A[1], &B[0], &B[1], GV, GW, one, &sval);
      double tpggi = orc_pgike1(&A[1], &A[0], &B[1], &B[0], GV, GW, pmass, &sval);
      tegg = tegg + BCFV * BCFW * teggi;
      tpgg = tpgg + BCFV * BCFW * tpggi;
      double VCEGGI = zero, VCPGGI = zero;
      for (int64_t c = 0; c < s->nat; c++) {
        const double C[3] = {s->cat[3 * c], s->cat[3 * c + 1], s->cat[3 * c + 2]};
        double ZNUC = s->zan[c];
        double a = orc_g2_xggvec(&A[0], &A[1], &B[0], &B[1], GV, GW, C);
        VCEGGI = a * ZNUC + VCEGGI;
        double b = orc_g2_xggvec(&A[1], &A[0], &B[1], &B[0], GV, GW, C);
        VCPGGI = b * ZNUC + VCPGGI;
      }
      double VMGGI = orc_g2_xggvee(&A[0], &A[1], &B[0], &B[1], GV, GW);
      VCEGG = VCEGG + BCFV * BCFW * VCEGGI;
      VCPGG = VCPGG + BCFV * BCFW * VCPGGI;
      VMGG = VMGG + BCFV * BCFW * VMGGI;
    }
  }
  double TE = tegx + texg + tegg;
  double TP = tpgx + tpxg + tpgg;
  double VCE = 2.0 * VCEGX + VCEGG;
  double VCP = 2.0 * VCPGX + VCPGG;
  double VMX = 2.0 * VMGX + VMGG;
  *ansE = TE + TP - VCE + VCP - VMX;
  double OXX = zero, OGX = zero, OGG = zero;
  for (int k = 0; k < ng; k++) {
    double GV = s->ggem[k], BCFV = s->bgem[k];
    if (with_single) {
      double ogxix = orc_g2_xggs(&A[0], &A[1], &B[0], &B[1], GV, zero);
      OGX = OGX + BCFV * ogxix;
    }
    for (int l = 0; l < ng; l++) {
      double GW = s->ggem[l], BCFW = s->bgem[l];
      double oggix = orc_g2_xggs(&A[0], &A[1], &B[0], &B[1], GV, GW);
      OGG = OGG + BCFV * BCFW * oggix;
    }
  }
  *ansS = OXX + 2.0 * OGX + OGG;
}

void orc_xcalc_gam1(const orc_prim *A, const orc_prim *B, const orc_system *s,
                    double *ansE, double *ansS) {
  xcalc_gam1(A, B, s, 1, ansE, ansS);
}

/* gam_1_OMP.f:2-395 GAM1_OMP_MD -> GAM_1, GAM_1s (ng1 = nebf^2 npbf^2),
 * packed by pack_4D(nebf,nebf,npbf, jec1,iec1,jp,ip) */
static void gam1_tables(const orc_system *s, int with_single, double *G1,
                        double *G1s) {
  const int64_t ne = s->nebf, npe = s->npebf, np = s->npbf;
  memset(G1, 0, sizeof(double) * (size_t)(ne * ne * np * np));
  memset(G1s, 0, sizeof(double) * (size_t)(ne * ne * np * np));
  for (int64_t ip = 1; ip <= np; ip++)
    for (int64_t jp = 1; jp <= np; jp++)
      for (int64_t ie1 = 1; ie1 <= npe; ie1++)
        for (int64_t je1 = 1; je1 <= npe; je1++) {
          orc_prim A[2], B[2];
          e_prim(s, ie1, &A[0]);
          p_prim(s, ip, &A[1]);
          e_prim(s, je1, &B[0]);
          p_prim(s, jp, &B[1]);
          double ansE, ansS;
          xcalc_gam1(A, B, s, with_single, &ansE, &ansS);
          int64_t iec1 = s->AMPEB2C[ie1 - 1], jec1 = s->AMPEB2C[je1 - 1];
          double cip = s->AGNBFCC[ip - 1], cjp = s->AGNBFCC[jp - 1];
          double cie = s->AGEBFCC[ie1 - 1], cje = s->AGEBFCC[je1 - 1];
          int64_t ia = orc_pack_4d(ne, ne, np, jec1, iec1, jp, ip);
          G1[ia - 1] = G1[ia - 1] + ansE * cip * cjp * cie * cje;
          G1s[ia - 1] = G1s[ia - 1] + ansS * cip * cjp * cie * cje;
        }
}

void orc_gam1(const orc_system *s, double *G1, double *G1s) {
  gam1_tables(s, 1, G1, G1s);
}

/* rxchf/rxchf_gam_1_OMP.f:2-175 RXCHF_GAM1_OMP_MD (the special electron and
 * the proton share every geminal factor) */
void orc_rxchf_gam1(const orc_system *s, double *G1, double *G1s) {
  gam1_tables(s, 0, G1, G1s);
}

/* class_nuc_rep.f:2-45 class_nuc_rep */
double orc_nuc_rep(const orc_system *s) {
  double E = 0.0;
  if (s->nat < 2) return E;
  for (int64_t i = 2; i <= s->nat; i++)
    for (int64_t j = 1; j <= i - 1; j++) {
      double R2 = 0.0;
      for (int k = 0; k < 3; k++) {
        double d = s->cat[3 * (i - 1) + k] - s->cat[3 * (j - 1) + k];
        R2 = R2 + d * d;
      }
      if (R2 != 0.0) E = E + s->zan[i - 1] * s->zan[j - 1] / sqrt(R2);
    }
  return E;
}
