/*
 * neoxc_oracle.h -- CPU restatement of the NEO-RXCHF geminal-integral hot
 * path.  TEST INFRASTRUCTURE ONLY: this library is the checker that the
 * CUDA path is compared against (and the timed CPU baseline).  Nothing in
 * the product links it.
 *
 * Conventions follow the Fortran reference exactly:
 *   - every multi-index array is column-major with the reference's
 *     dimension order (e.g. ELCAM(npebf,3) -> ELCAM[i + npebf*d]);
 *   - index VALUES stored in arrays (AMPEB2C, KPESTR, KPEEND) are 1-based;
 *   - packed integral tensors use the reference's packed index minus one
 *     (pack_GAM.f), so T[ia-1] is the Fortran T(ia).
 * Each function names the reference routine (file:line) it restates.
 */
#ifndef NEOXC_ORACLE_H
#define NEOXC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Basis / system description: the reference's flat argument arrays. */
typedef struct {
  int64_t nebf, npebf, npbf, nat, ngtg;
  const int64_t *ELCAM;    /* (npebf,3)  angular momenta of e primitives */
  const double  *ELCEX;    /* (npebf)    exponents                       */
  const double  *ELCBFC;   /* (npebf,3)  centres (bohr)                  */
  const int64_t *AMPEB2C;  /* (npebf)    primitive -> contracted (1-based)*/
  const double  *AGEBFCC;  /* (npebf)    contraction coefficients        */
  const int64_t *KPESTR;   /* (nebf)     first primitive (1-based)       */
  const int64_t *KPEEND;   /* (nebf)     last primitive (1-based)        */
  const int64_t *NUCAM;    /* (npbf,3)                                   */
  const double  *NUCEX;    /* (npbf)                                     */
  const double  *NUCBFC;   /* (npbf,3)                                   */
  const double  *AGNBFCC;  /* (npbf)                                     */
  const double  *zan;      /* (nat)                                      */
  const double  *cat;      /* (3,nat)                                    */
  const double  *bgem;     /* (ngtg)  geminal b_k                        */
  const double  *ggem;     /* (ngtg)  geminal gamma_k                    */
  double pmass;
} orc_system;

/* ---- L1 math utilities ------------------------------------------------ */
void   orc_xgammaf(double *F, double T, int M);
double orc_iboys2(int m, double x);
double orc_underflow(double x);
double orc_rtuv(int tLim, int uLim, int vLim, int nLim, double expt,
                double alpha, double XPC, double YPC, double ZPC);
double orc_auxR2(int NMAX, int LMAX, int MMAX, double alp, double a,
                 double b, double c);
void   orc_ghec(int iLim, int jLim, double KAB, double a, double b, double p,
                double q, double Qx, double *EOUT);
double orc_gdel_x(int N, double x, double alp, double Ax);

/* ---- primitive integrals (L2) ----------------------------------------- */
/* One Cartesian Gaussian primitive: (l,m,n), exponent, centre. */
typedef struct { int l[3]; double a; double c[3]; } orc_prim;

double orc_gfovlap(const orc_prim *A, const orc_prim *B);
double orc_gfke(const orc_prim *A, const orc_prim *B, double xmass);
double orc_gfvec(const orc_prim *A, const orc_prim *B, const double *C);
double orc_gfvee(const orc_prim *A1, const orc_prim *A2,
                 const orc_prim *B1, const orc_prim *B2);
double orc_g2_xggs(const orc_prim *A1, const orc_prim *A2,
                   const orc_prim *B1, const orc_prim *B2,
                   double gamma1, double gamma2);
/* gam[6] = {gamA12,gamA13,gamA23,gamB12,gamB13,gamB23} */
double orc_g3_xggs(const orc_prim *A, const orc_prim *B, const double *gam);
double orc_g3_ke(const orc_prim *A, const orc_prim *B, const double *gam,
                 double xmass);
double orc_g3_xgvxcg(const orc_prim *A, const orc_prim *B, const double *gam,
                     const double *C);
double orc_g3_xgveeg(const orc_prim *A, const orc_prim *B, const double *gam);
double orc_g4_xgveeg(const orc_prim *A, const orc_prim *B, double gam14,
                     double gam34);
double orc_g4_xgvepg(const orc_prim *A, const orc_prim *B, double gam14,
                     double gam24);

/* ---- per-primitive-tuple integrands (L3 inner) ------------------------ */
void   orc_xcalc_gam2(const orc_prim *A, const orc_prim *B,
                      const orc_system *s, double *ansE, double *ansS);
double orc_xcalc_gam3(const orc_prim *A, const orc_prim *B,
                      const orc_system *s);
void   orc_xcalc_gam2_rxchfne(const orc_prim *A, const orc_prim *B,
                              const orc_system *s, double *ansE1,
                              double *ansE2);

/* ---- index maps (pack_GAM.f) ------------------------------------------ */
int64_t orc_pack_4d(int64_t n1, int64_t n2, int64_t n3, int64_t i1,
                    int64_t i2, int64_t i3, int64_t i4);
int64_t orc_index_gam_2pk(int64_t nebf, int64_t npbf, int64_t ip, int64_t jp,
                          int64_t ie1, int64_t je1, int64_t ie2, int64_t je2);
int64_t orc_index_gam_3pk(int64_t nebf, int64_t npbf, int64_t ip, int64_t jp,
                          int64_t ie1, int64_t je1, int64_t ie2, int64_t je2,
                          int64_t ie3, int64_t je3);
int64_t orc_index_gam_4pk2(int64_t nebf, int64_t npbf, int64_t ip,
                           int64_t jp, int64_t ie1, int64_t je1, int64_t ie2,
                           int64_t je2, int64_t ie3, int64_t je3, int64_t ie4,
                           int64_t je4);
void    orc_loop_size(int64_t L1, int64_t L2, int64_t nproc, int64_t myrank,
                      int64_t *istart, int64_t *iend);

/* ---- basis set-up ------------------------------------------------------ */
void orc_make_kpe(int64_t nebf, int64_t npebf, const int64_t *AMPEB2C,
                  int64_t *KPESTR, int64_t *KPEEND);
void orc_elcnorm3(int64_t npebf, int64_t nebf, const int64_t *AMPEB2C,
                  double *AGEBFCC, const double *ELCEX, const int64_t *ELCAM,
                  const double *ELCBFC);
void orc_nucnorm(int64_t npbf, double *AGNBFCC, const double *NUCEX,
                 const int64_t *NUCAM, const double *NUCBFC);

/* ---- contracted builders (L3) ----------------------------------------- */
/* Tensor builders compute tuples [t0, t1) of the flattened loop space
 * (ip,jp,iec1,jec1,... with the last ket index fastest) into the RAW
 * (unsymmetrised) array, then *_symmetrize writes the final arrays. */
void orc_gam2_raw(const orc_system *s, int64_t t0, int64_t t1,
                  double *XG2, double *XG2s);
void orc_gam2_symmetrize(int64_t nebf, int64_t npbf, const double *XG2,
                         const double *XG2s, double *GM2, double *GM2s);
void orc_gam2_ic1(const orc_system *s, double *GM2ICR, double *GM2sICR);

void orc_gam3_raw(const orc_system *s, int64_t t0, int64_t t1, double *XG3);
void orc_gam3_symmetrize(int64_t nebf, int64_t npbf, const double *XG3,
                         double *GM3);
void orc_gam3_ic1(const orc_system *s, double *GM3ICR);
/* one contracted OMG3 element (contract_omega3_conv) */
double orc_contract_omega3(const orc_system *s, int64_t ip, int64_t jp,
                           int64_t iec1, int64_t jec1, int64_t iec2,
                           int64_t jec2, int64_t iec3, int64_t jec3);

void orc_rxchfne_gam2_raw(const orc_system *s, int64_t t0, int64_t t1,
                          double *XG2, double *XG2ex);
void orc_rxchfne_gam2_ic1(const orc_system *s, double *GM2ICR,
                          double *GM2exICR);

void orc_calc_gam_ee(const orc_system *s, double *GAM_ee);

/* gam_4_OMP.f:964-1192 calc_GAM_4_integral (one raw product element) */
double orc_gam4_raw(int64_t ne, int64_t np, const double *G2s, const double *Gee,
                    int64_t ip, int64_t jp, int64_t ie1, int64_t je1, int64_t ie2,
                    int64_t je2, int64_t ie3, int64_t je3, int64_t ie4, int64_t je4);

/* ---- open-shell XCUHF contractions (spin.c, xcuhf/xcuhf_omg{1..4}.f) ---- */
void orc_fae_omg1(int64_t ne, int64_t np, const double *DAE, const double *DP,
                  const double *G1, const double *G1s, double *FAE,
                  double *SAE1, double *E, double *S);
void orc_ufp_omg1(int64_t ne, int64_t np, const double *DETOT,
                  const double *DP, const double *G1, const double *G1s,
                  double *FP, double *SP1, double *E, double *S);
void orc_fae_omg2(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G2, const double *G2s, double *FAE,
                  double *SAE2, double *E, double *S);
void orc_ufp_omg2(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G2, const double *G2s, double *FP,
                  double *SP2, double *E, double *S);
void orc_fae_omg3(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G3, double *FAE, double *E);
void orc_ufp_omg3(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G3, double *FP, double *E);
void orc_fae_omg4(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G4, double *FAE, double *E);
void orc_ufp_omg4(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                  const double *DAE, const double *DBE, const double *DP,
                  const double *G4, double *FP, double *E);
void orc_fae_omg4_direct(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                         const double *DAE, const double *DBE, const double *DP,
                         const double *G2s, const double *Gee, double *FAE,
                         double *E);
void orc_ufp_omg4_direct(int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
                         const double *DAE, const double *DBE, const double *DP,
                         const double *G2s, const double *Gee, double *FP,
                         double *E);
void orc_omg4_icr(int64_t ne, int64_t np, const double *G2s, const double *Gee,
                  double *G4);

/* ---- special-electron contractions (rx.c: rxchf/, rxchfne/) ------------ */
void orc_rxcuhfne_fe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                          const double *DAtotE, const double *DBE, const double *DP,
                          const double *G, const double *Gx, double *FAalpE,
                          double *FAbetE, double *E);
void orc_rxcuhfne_fp_omg2(int64_t ne, int64_t np, const double *DAalpE,
                          const double *DAtotE, const double *DBE, const double *DP,
                          const double *G, const double *Gx, double *FP, double *E);
void orc_rxcuhfne_fbe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                           const double *DAtotE, const double *DBE, const double *DP,
                           const double *G, const double *Gx, double *FBE, double *E);
void orc_rxchf_fae_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        const double *Gs, double *FAE, double *SAE, double *E, double *S);
void orc_rxchf_fp_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G1, const double *G2,
                       const double *Gs, double *FP, double *SP, double *E, double *S);
void orc_rxchf_fbe_omg2(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        const double *Gs, double *FBE, double *SBE, double *E, double *S);
void orc_rxchf_fae_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        double *FAE, double *E);
void orc_rxchf_fp_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G1, const double *G2, double *FP,
                       double *E);
void orc_rxchf_fbe_omg3(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G1, const double *G2, double *FBE,
                        double *E);
void orc_rxchf_fae_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G, double *FAE, double *E);
void orc_rxchf_fp_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                       const double *DP, const double *G, double *FP, double *E);
void orc_rxchf_fbe_omg4(int64_t ne, int64_t np, const double *DAE, const double *DBE,
                        const double *DP, const double *G, double *FBE, double *E);
void orc_rxcuhf_fe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAtotE, const double *DBE, const double *DP,
                        const double *G1, const double *G2, const double *Gs,
                        double *FAalpE, double *FAbetE, double *SAalpE, double *E,
                        double *S);
void orc_rxcuhf_fp_omg2(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAtotE, const double *DBE, const double *DP,
                        const double *G1, const double *G2, const double *Gs,
                        double *FP, double *SP, double *E, double *S);
void orc_rxcuhf_fbe_omg2(int64_t ne, int64_t np, const double *DAalpE,
                         const double *DAtotE, const double *DBE, const double *DP,
                         const double *G1, const double *G2, const double *Gs,
                         double *FBE, double *SBE, double *E, double *S);
void orc_rxcuhf_fe_omg3(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAbetE, const double *DAtotE, const double *DBE,
                        const double *DP, const double *G1, const double *G2,
                        double *FAalpE, double *FAbetE, double *E);
void orc_rxcuhf_fp_omg3(int64_t ne, int64_t np, const double *DAalpE,
                        const double *DAbetE, const double *DAtotE, const double *DBE,
                        const double *DP, const double *G1, const double *G2, double *FP,
                        double *E);
void orc_rxcuhf_fbe_omg3(int64_t ne, int64_t np, const double *DAalpE,
                         const double *DAbetE, const double *DAtotE, const double *DBE,
                         const double *DP, const double *G1, const double *G2,
                         double *FBE, double *E);

/* gam_4 element assembly (gam_4_OMP.f symm_gam4 / calc_GAM_4_integral),
 * returned already divided by 16 as stored by GAM4_ICR. */
double orc_gam4_element(int64_t ne, int64_t np, const double *GAM_2s,
                        const double *GAM_ee, int64_t ip, int64_t jp,
                        int64_t ie1, int64_t je1, int64_t ie2, int64_t je2,
                        int64_t ie3, int64_t je3, int64_t ie4, int64_t je4);
void orc_gam4_icr(int64_t ne, int64_t np, const double *GAM_2s,
                  const double *GAM_ee, double *GAM_4);

/* ---- Fock / energy contractions (L4) ---------------------------------- */
/* ACCUMULATE into focke/fockp (add2fock); overwrite energies and SE/SP. */
void orc_gam4_dscf(int64_t ne, int64_t np, const double *GAM_ee,
                   const double *GAM_2s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *E_gam4);
void orc_gam4_dscf_range(int64_t ne, int64_t np, const double *GAM_ee,
                         const double *GAM_2s, const double *DE,
                         const double *DP, int64_t t0, int64_t t1,
                         double *xfocke, double *xfockp, double *E_gam4);
void orc_gam4_dscf_sample(int64_t ne, int64_t np, const double *GAM_ee,
                          const double *GAM_2s, const double *DE,
                          const double *DP, int64_t t0, int64_t t1,
                          double *focke, double *fockp, double *E);
void orc_eg4icr(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *GM4, double *focke, double *fockp,
                double *E_gam4);
void orc_eg3ic1(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *GM3, double *focke, double *fockp,
                double *E_gam3);
void orc_eg2ic1(int64_t ne, int64_t np, const double *DE, const double *DP,
                const double *GM2, const double *GM2s, double *FE, double *SE,
                double *FP, double *SP, double *E_gam2, double *S_gam2);
void orc_rxchfne_fae_omg2(int64_t ne, int64_t np, const double *DAE,
                          const double *DBE, const double *DP,
                          const double *GM2, double *FAE, double *E);
void orc_rxchfne_fp_omg2(int64_t ne, int64_t np, const double *DAE,
                         const double *DBE, const double *DP,
                         const double *GM2, double *FP, double *E);
void orc_rxchfne_fbe_omg2(int64_t ne, int64_t np, const double *DAE,
                          const double *DBE, const double *DP,
                          const double *GM2, double *FBE, double *E);
void orc_xcfock_correction(int64_t ne, int64_t np, double S_total,
                           double H_expect, const double *se1,
                           const double *sp1, const double *se2,
                           const double *sp2, double *focke, double *fockp);

/* direct-SCF variants (gam2_DSCF_OMP.f, gam3_DSCF_OMP.f) */
void orc_gam2_dscf(const orc_system *s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *se2, double *sp2,
                   double *E_gam2, double *S_gam2);
void orc_gam3_dscf(const orc_system *s, const double *DE, const double *DP,
                   double *focke, double *fockp, double *E_gam3);

/* two-particle geminal kernels of gam_1 (XC1_G2_MD.f, g2.f) */
double orc_g2_xggvec(const orc_prim *A1, const orc_prim *A2,
                     const orc_prim *B1, const orc_prim *B2, double gamma1,
                     double gamma2, const double *C);
double orc_g2_xggvee(const orc_prim *A1, const orc_prim *A2,
                     const orc_prim *B1, const orc_prim *B2, double gamma1,
                     double gamma2);
double orc_pgike1(const orc_prim *A1, const orc_prim *A2, const orc_prim *B1,
                  const orc_prim *B2, double gamA, double gamB, double xmass1,
                  double *sval);

/* XCHF SCF integrals (scf.c) */
void orc_overlaps(const orc_system *s, double *Se, double *Sp);
void orc_gam_epcore(const orc_system *s, double *Gecore, double *Gpcore);
void orc_gam_ep(const orc_system *s, double *Gep);
void orc_xcalc_gam1(const orc_prim *A, const orc_prim *B, const orc_system *s,
                    double *ansE, double *ansS);
void orc_gam1(const orc_system *s, double *G1, double *G1s);
void orc_rxchf_gam1(const orc_system *s, double *G1, double *G1s);
double orc_nuc_rep(const orc_system *s);

/* density from MO coefficients (GAM_IO.f read_elec_density) */
void orc_density(int64_t nbf, int64_t nocc, double prefac, const double *C,
                 double *D);

int  orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
