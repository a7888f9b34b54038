/*
 * neoxc.h -- C-ABI of the GB300 engine for the NEO-RXCHF geminal-integral
 * hot path (libneoxc_gb300.so).
 *
 * Every entry point replaces one reference Fortran routine and keeps its
 * argument list, array layouts (column-major, packed indices of
 * CS_Integrals/Spot_Check/pack_GAM.f) and output semantics (builders
 * overwrite, Fock contractions accumulate into the caller's matrices,
 * energies are overwritten).  Integers are int64_t (the reference is built
 * with -integer-size 64), reals are double.  Array arguments are HOST
 * memory unless the name starts with neoxc_dev_ (device pointers, work
 * enqueued on `stream`, a cudaStream_t or NULL for the legacy stream).
 *
 * Return value: NEOXC_OK (0) or an error code; neoxc_last_error() gives a
 * message.  No entry point aborts the process and none falls back to the
 * CPU: without a usable GB300 device every compute call returns
 * NEOXC_ERR_CUDA.
 *
 * Fortran callers can bind the neoxc_* symbols with ISO_C_BINDING
 * interfaces (integer(c_int64_t), value, real(c_double)), or link the
 * by-reference shims (gam2_ic1_, eg3ic1_, ...) which have exactly the
 * reference's external-subroutine signatures.
 */
#ifndef NEOXC_H
#define NEOXC_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NEOXC_OK 0
#define NEOXC_ERR_ARG 1          /* inconsistent sizes / bad pointer     */
#define NEOXC_ERR_CUDA 2         /* CUDA runtime error or no device      */
#define NEOXC_ERR_NOMEM 3        /* device allocation failed             */
#define NEOXC_ERR_UNSUPPORTED 4  /* shape outside the supported range    */
#define NEOXC_ERR_IO 5           /* integral file could not be read      */
#define NEOXC_ERR_TIMEOUT 6      /* server wait ran out (job still runs) */
#define NEOXC_ERR_NUMERIC 7      /* non-finite energy or Fock matrix     */

const char* neoxc_last_error(void);
int neoxc_version(void);
/* 1 when a CUDA device of compute capability 10.3 is current, else 0. */
int neoxc_device_ok(void);

/* ---- packed index maps: CS_Integrals/Spot_Check/pack_GAM.f ------------ */
/* pack_GAM.f:29-69 pack_4D */
int64_t neoxc_pack_4d(int64_t n1, int64_t n2, int64_t n3, int64_t i1,
                      int64_t i2, int64_t i3, int64_t i4);
/* pack_GAM.f:72-105 index_GAM_2PK */
int64_t neoxc_index_gam_2pk(int64_t nebf, int64_t npbf, int64_t ip,
                            int64_t jp, int64_t ie1, int64_t je1,
                            int64_t ie2, int64_t je2);
/* pack_GAM.f:108-147 index_GAM_3PK */
int64_t neoxc_index_gam_3pk(int64_t nebf, int64_t npbf, int64_t ip,
                            int64_t jp, int64_t ie1, int64_t je1,
                            int64_t ie2, int64_t je2, int64_t ie3,
                            int64_t je3);
/* pack_GAM.f:150-193 index_GAM_4PK and :196-239 index_GAM_4PK2 */
int64_t neoxc_index_gam_4pk2(int64_t nebf, int64_t npbf, int64_t ip,
                             int64_t jp, int64_t ie1, int64_t je1,
                             int64_t ie2, int64_t je2, int64_t ie3,
                             int64_t je3, int64_t ie4, int64_t je4);
/* Device evaluation of a whole map in the reference's loop order
 * (kind 0: GAM_ee pack_4D, 2/3/4: index_GAM_2PK/3PK/4PK2); out[count]. */
int neoxc_index_map(int64_t kind, int64_t nebf, int64_t npbf, int64_t count,
                    int64_t* out);

/* ---- basis set-up done by the driver (xcneo_HYBRID.f) ----------------- */
/* xcneo_HYBRID.f:1269-1307 make_KPE */
int neoxc_make_kpe(int64_t nebf, int64_t npebf, const int64_t* AMPEB2C,
                   int64_t* KPESTR, int64_t* KPEEND);

/* ---- integral builders (overwrite their outputs) ---------------------- */
/* gam_ee.f:2-169 calc_GAM_ee: GAM_ee(ngee) packed by pack_4D(je2,ie2,je1,ie1).
 * The reference also writes GAM_ee.ufm; this call only fills the array. */
int neoxc_calc_gam_ee(int64_t nebf, int64_t npebf, int64_t ngee,
                      const int64_t* AMPEB2C, const double* AGEBFCC,
                      const double* ELCEX, const int64_t* ELCAM,
                      const double* ELCBFC, double* GAM_ee);

/* gam2_IC1_OMP.f:2-212 GAM2_IC1 -> GM2ICR, GM2sICR (pair-symmetrised) */
int neoxc_gam2_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                   int64_t ng2, int64_t ng2prm, int64_t nat, int64_t ngtg1,
                   double pmass, const double* cat, const double* zan,
                   const double* bcoef1, const double* gamma1,
                   const int64_t* KPESTR, const int64_t* KPEEND,
                   const int64_t* AMPEB2C, const double* AGEBFCC,
                   const double* AGNBFCC, const double* ELCEX,
                   const double* NUCEX, const int64_t* ELCAM,
                   const int64_t* NUCAM, const double* ELCBFC,
                   const double* NUCBFC, double* GM2ICR, double* GM2sICR);

/* gam3_IC1_OMP.f:2-297 GAM3_IC1 -> GM3ICR (six-permutation symmetrised) */
int neoxc_gam3_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                   int64_t ng3, int64_t ng3prm, int64_t nat, int64_t ngtg1,
                   double pmass, const double* cat, const double* zan,
                   const double* bcoef1, const double* gamma1,
                   const int64_t* KPESTR, const int64_t* KPEEND,
                   const int64_t* AMPEB2C, const double* AGEBFCC,
                   const double* AGNBFCC, const double* ELCEX,
                   const double* NUCEX, const int64_t* ELCAM,
                   const int64_t* NUCAM, const double* ELCBFC,
                   const double* NUCBFC, double* GM3ICR);
/* GAM3_IC1 with options (no reference counterpart for the options):
 * NEOXC_SCF_MIXED computes the four-particle terms with FP32 tables and
 * FP64 Boys function, seeds and sums; NEOXC_SCF_SCREEN skips primitive
 * (bra, ket) pairs whose Schwarz-type estimate is below 1e-12.  seconds
 * (optional) receives the device time of the build (CUDA events, the copy
 * to GM3ICR excluded). */
int neoxc_gam3_ic1_opts(int64_t options, int64_t Nchunks, int64_t nebf, int64_t npebf,
                        int64_t npbf, int64_t ng3, int64_t ng3prm, int64_t nat,
                        int64_t ngtg1, double pmass, const double* cat, const double* zan,
                        const double* bcoef1, const double* gamma1,
                        const int64_t* KPESTR, const int64_t* KPEEND,
                        const int64_t* AMPEB2C, const double* AGEBFCC,
                        const double* AGNBFCC, const double* ELCEX,
                        const double* NUCEX, const int64_t* ELCAM,
                        const int64_t* NUCAM, const double* ELCBFC,
                        const double* NUCBFC, double* GM3ICR, double* seconds);


/* gam3_DSCF_OMP.f:2-137 GAM3_DSCF: builds gam_3 one proton pair at a time
 * and contracts it on the fly; focke, fockp accumulate (add2fock), E_gam3
 * overwritten.  Limit: nebf <= 20. */
int neoxc_gam3_dscf(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                    int64_t ng3, int64_t ng3prm, int64_t nat, int64_t ngtg1,
                    double pmass, const double* cat, const double* zan,
                    const double* bcoef1, const double* gamma1,
                    const int64_t* KPESTR, const int64_t* KPEEND,
                    const int64_t* AMPEB2C, const double* AGEBFCC,
                    const double* AGNBFCC, const double* ELCEX,
                    const double* NUCEX, const int64_t* ELCAM,
                    const int64_t* NUCAM, const double* ELCBFC,
                    const double* NUCBFC, const double* DE, const double* DP,
                    double* focke, double* fockp, double* E_gam3);

/* gam2_DSCF_OMP.f:2-140 GAM2_DSCF: builds gam_2 / gam_2s one proton pair at
 * a time; focke, fockp, se2, sp2 accumulate (add2fock), E_gam2 and S_gam2
 * overwritten. */
int neoxc_gam2_dscf(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                    int64_t ng2, int64_t ng2prm, int64_t nat, int64_t ngtg1,
                    double pmass, const double* cat, const double* zan,
                    const double* bcoef1, const double* gamma1,
                    const int64_t* KPESTR, const int64_t* KPEEND,
                    const int64_t* AMPEB2C, const double* AGEBFCC,
                    const double* AGNBFCC, const double* ELCEX,
                    const double* NUCEX, const int64_t* ELCAM,
                    const int64_t* NUCAM, const double* ELCBFC,
                    const double* NUCBFC, const double* DE, const double* DP,
                    double* focke, double* fockp, double* se2, double* sp2,
                    double* E_gam2, double* S_gam2);

/* rxchfne/rxchfne_gam2_IC1_OMP.f:2-243 RXCHFne_GAM2_IC1 -> GM2ICR (raw),
 * GM2exICR (pair-averaged exchange term) */
int neoxc_rxchfne_gam2_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf,
                           int64_t npbf, int64_t ng2, int64_t ng2prm,
                           int64_t nat, int64_t ngtg1, double pmass,
                           const double* cat, const double* zan,
                           const double* bcoef1, const double* gamma1,
                           const int64_t* KPESTR, const int64_t* KPEEND,
                           const int64_t* AMPEB2C, const double* AGEBFCC,
                           const double* AGNBFCC, const double* ELCEX,
                           const double* NUCEX, const int64_t* ELCAM,
                           const int64_t* NUCAM, const double* ELCBFC,
                           const double* NUCBFC, double* GM2ICR,
                           double* GM2exICR);

/* gam4_ICR_OMP.f:2-138 GAM4_ICR -> GAM_4(ng4) = gam_4/16.  The reference
 * reads GAM_ee from GAM_ee.ufm; here it is an explicit argument. */
int neoxc_gam4_icr(int64_t Nchunks, int64_t ne, int64_t np, int64_t ngee,
                   int64_t ng2, int64_t ng4, const double* GAM_2s,
                   const double* GAM_ee, double* GAM_4);

/* ---- Fock / energy contractions (accumulate Fock, overwrite E) -------- */
/* gam4_DSCF_OMP.f:2-139 GAM4_DSCF: fused gam_4 assembly + contraction, the
 * gam_4 tensor is never stored.  GAM_ee / GAM_2s explicit (the reference
 * reads GAM_ee.ufm / GAM_2s.ufm). */
int neoxc_gam4_dscf(int64_t NG4CHK, int64_t ne, int64_t np, int64_t ngee,
                    int64_t ng2, int64_t ng4, const double* GAM_ee,
                    const double* GAM_2s, const double* DE, const double* DP,
                    double* focke, double* fockp, double* E_gam4);

/* gam4_ICR_OMP.f:273-376 EG4ICR */
int neoxc_eg4icr(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                 const double* DE, const double* DP, const double* GM4ICR,
                 double* focke, double* fockp, double* E_gam4);

/* gam3_IC1_OMP.f:433-535 EG3IC1 */
int neoxc_eg3ic1(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                 const double* DE, const double* DP, const double* GM3ICR,
                 double* focke, double* fockp, double* E_gam3);

/* gam2_IC1_OMP.f:339-443 EG2IC1: FE, FP accumulate; SE, SP, E, S
 * overwritten. */
int neoxc_eg2ic1(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                 const double* DE, const double* DP, const double* GM2ICR,
                 const double* GM2SICR, double* FE, double* SE, double* FP,
                 double* SP, double* E_gam2, double* S_gam2);

/* rxchfne/rxchfne_omg2.f:2-116 RXCHFne_FAE_OMG2 */
int neoxc_rxchfne_fae_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf,
                           int64_t ng2, const double* DAE, const double* DBE,
                           const double* DP, const double* GM2ICR,
                           double* FAE, double* E_AE_OMG2);
/* rxchfne/rxchfne_omg2.f:212-314 RXCHFne_FP_OMG2 */
int neoxc_rxchfne_fp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf,
                          int64_t ng2, int64_t NAE, int64_t NBE,
                          const double* DAE, const double* DBE,
                          const double* DP, const double* GM2ICR, double* FP,
                          double* E_P_OMG2);
/* rxchfne/rxchfne_omg2.f:409-511 RXCHFne_FBE_OMG2 */
int neoxc_rxchfne_fbe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf,
                           int64_t ng2, int64_t NAE, int64_t NBE,
                           const double* DAE, const double* DBE,
                           const double* DP, const double* GM2ICR,
                           double* FBE, double* E_BE_OMG2);
/* One pass over GM2ICR producing all three (no reference counterpart:
 * the three routines above re-read the tensor once each). */
int neoxc_rxchfne_omg2_fused(int64_t nebf, int64_t npbf, const double* DAE,
                             const double* DBE, const double* DP,
                             const double* GM2ICR, double* FAE, double* FP,
                             double* FBE, double* E_OMG2);

/* xchf1_independent/xchf1_fock.f:728-783 XCfock_correction */
int neoxc_xcfock_correction(int64_t nebf, int64_t npbf, double E_total,
                            double S_total, double H_expect,
                            const double* se1, const double* sp1,
                            const double* se2, const double* sp2,
                            double* focke, double* fockp);

/* ---- one-body tables and the whole XCHF Fock build ---------------------- */
/* The integrals xcneo_driver computes before the geminal ones
 * (xcneo_HYBRID.f:665-690,761): pure_ovlap.f:2-105 elec_ovlap -> Se,
 * :107-203 nuc_ovlap -> Sp, gam_epcore.f:2-198 calc_GAM_epcore -> GAM_ecore,
 * GAM_pcore, gam_ep.f:2-165 calc_GAM_ep -> GAM_ep, gam_1_OMP.f:2-396
 * GAM1_OMP_MD -> GAM_1, GAM_1s.  Each output holds the records of the
 * reference's file in order: Se, GAM_ecore pack_2D(nebf,je,ie) (eovlap.ufm,
 * GAM_ecr.ufm); Sp, GAM_pcore pack_2D(npbf,jp,ip) (novlap.ufm, GAM_pcr.ufm);
 * GAM_ep, GAM_1, GAM_1s pack_4D(je,ie,jp,ip) (GAM_ep.ufm, GAM_1.ufm,
 * GAM_1s.ufm).  A NULL output is skipped, and the inputs only it needs may
 * be NULL: the electronic basis (AMPEB2C, AGEBFCC, ELCEX, ELCAM, ELCBFC)
 * serves all but Sp/GAM_pcore, the nuclear basis (AGNBFCC, NUCEX, NUCAM,
 * NUCBFC) all but Se/GAM_ecore, the classical nuclei (nat, zan, cat) the
 * core and GAM_1 tables, the geminal (ngtg1 >= 1, bcoef1, gamma1) GAM_1. */
int neoxc_onebody_integrals(int64_t nebf, int64_t npebf, int64_t npbf,
                            int64_t nat, int64_t ngtg1, double pmass,
                            const double* cat, const double* zan,
                            const double* bcoef1, const double* gamma1,
                            const int64_t* AMPEB2C, const double* AGEBFCC,
                            const double* AGNBFCC, const double* ELCEX,
                            const double* NUCEX, const int64_t* ELCAM,
                            const int64_t* NUCAM, const double* ELCBFC,
                            const double* NUCBFC, double* Se, double* Sp,
                            double* GAM_ecore, double* GAM_pcore,
                            double* GAM_ep, double* GAM_1, double* GAM_1s);
/* rxchf/rxchf_gam_1_OMP.f:2-175 RXCHF_GAM1_OMP_MD: GAM_1 / GAM_1s of the
 * special electron and the proton, which share every geminal factor (the
 * geminal-pair terms of GAM1_OMP_MD only); same layout as GAM_1 above. */
int neoxc_rxchf_gam1(int64_t nebf, int64_t npebf, int64_t npbf, int64_t ng1,
                     int64_t ng1prm, int64_t nat, int64_t ngtg1, double pmass,
                     const double* cat, const double* zan, const double* bcoef1,
                     const double* gamma1, const int64_t* AMPEB2C,
                     const double* AGEBFCC, const double* AGNBFCC,
                     const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                     const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC,
                     double* GAM_1, double* GAM_1s);
/* class_nuc_rep.f:2-45: E_nuc = sum_{i<j} Z_i Z_j / |R_i - R_j| (host
 * arithmetic, O(nat^2)). */
int neoxc_class_nuc_rep(int64_t nat, const double* zan, const double* cat,
                        double* E_nuc);

/* The LOGICAL switches of xchf1_fock as bits of `modes`.  A geminal term
 * with neither its DSCF nor its IC bit is the reference's disk branch
 * (S_from_GAM_2s / E_from_GAM_2 / E_from_GAM_3 / E_from_GAM_4): its tables
 * come in the IC arguments (GM2ICR = GAM_2.ufm, GM2SICR = GAM_2s.ufm,
 * GM3IC1 = GAM_3.ufm, GM4ICR = GAM_4.ufm / 16, the scale E_from_GAM_4
 * applies; xchf1_fock_ reads the files). */
#define NEOXC_FOCK_NEOHF    1   /* LNEOHF: NEO-HF terms only */
#define NEOXC_FOCK_GAM4     2   /* LGAM4: include gam_4 */
#define NEOXC_FOCK_G4DSCF   4   /* LG4DSCF: gam_4 from GAM_ee, GAM_2s */
#define NEOXC_FOCK_G4IC     8   /* LG4IC: gam_4 from GM4ICR */
#define NEOXC_FOCK_G3DSCF  16   /* LG3DSCF: gam_3 rebuilt from the basis */
#define NEOXC_FOCK_G3IC1   32   /* LG3IC1: gam_3 from GM3IC1 */
#define NEOXC_FOCK_G2DSCF  64   /* LG2DSCF: gam_2 rebuilt from the basis */
#define NEOXC_FOCK_G2IC1  128   /* LG2IC1: gam_2 from GM2ICR, GM2SICR */
#define NEOXC_FOCK_GAM4_FACTORED 256  /* direct gam_4 by the factorised build
                                         (same result for pair-symmetric tables) */

/* xchf1_independent/xchf1_fock.f:2-361 xchf1_fock, the XCHF Fock build the
 * SCF runs twice per iteration (xcscf.f:364,428), in one device pass:
 * E_from_GAM_ecore/pcore/ep/ee, S_from_GAM_1s/E_from_GAM_1 (GAM_1, GAM_1s
 * are arguments; the reference reads GAM_1.ufm, GAM_1s.ufm), the gam_2,
 * gam_3, gam_4 terms in the branch `modes` selects, S_total/E_total and
 * XCfock_correction.  Same arguments as the reference, with E_nuc read
 * (not written) and GAM_2s added for the direct gam_4 (GAM4_DSCF reads
 * GAM_2s.ufm; NULL takes GM2SICR).  Outputs overwritten: focke, fockp,
 * Xfocke, Xfockp (the NEO-HF part, :218-219) and the energies.  LCMF's
 * printed checks are not reproduced.  Limits: nebf <= 24 for gam_4,
 * nebf <= 20 for the direct gam_3. */
int neoxc_xchf1_fock(int64_t modes, int64_t NG4CHK, int64_t NG3CHK,
                     int64_t NG2CHK, int64_t npebf, int64_t nebf, int64_t npbf,
                     int64_t nelec, int64_t ngee, int64_t ng1, int64_t ng2,
                     int64_t ng3, int64_t ng4, const double* DE,
                     const double* DP, const double* GAM_ecore,
                     const double* GAM_pcore, const double* GAM_ep,
                     const double* GAM_ee, const double* GAM_1,
                     const double* GAM_1s, const double* GM4ICR,
                     const double* GM3IC1, const double* GM2ICR,
                     const double* GM2SICR, const double* GAM_2s,
                     int64_t ng2prm, int64_t ngtg1, int64_t ng3prm,
                     int64_t nat, double pmass, const double* cat,
                     const double* zan, const double* bcoef1,
                     const double* gamma1, const int64_t* KPESTR,
                     const int64_t* KPEEND, const int64_t* AMPEB2C,
                     const double* AGEBFCC, const double* AGNBFCC,
                     const double* ELCEX, const double* NUCEX,
                     const int64_t* ELCAM, const int64_t* NUCAM,
                     const double* ELCBFC, const double* NUCBFC,
                     double* focke, double* fockp, double* Xfocke,
                     double* Xfockp, double* E_total, const double* E_nuc,
                     double* E_ecore, double* E_pcore, double* E_ep,
                     double* E_ee, double* E_gam1, double* E_gam2,
                     double* E_gam3, double* E_gam4, double* S_total,
                     double* S_gam1, double* S_gam2);

/* ---- device-resident variants (no host copies; for SCF loops) --------- */
int neoxc_dev_gam4_dscf(void* stream, int64_t ne, int64_t np,
                        const double* d_GAM_ee, const double* d_GAM_2s,
                        const double* d_DE, const double* d_DP,
                        double* d_focke, double* d_fockp, double* d_E_gam4);
/* No counterpart in the reference.  Same computation as
 * neoxc_dev_gam4_dscf, for callers that cannot allocate device memory
 * (all of it handed to their own pool allocator, or a strict memory budget
 * where a transient allocation could fail in the middle of an SCF
 * iteration): the call allocates nothing and uses a scratch array built
 * into the library (264,192 doubles per GPU, held until the process exits).
 * Limit: npbf^2*nebf^3 + npbf^2 <= 264,192 (e.g. nebf=12/npbf=8 or
 * nebf=16/npbf=8); larger systems return NEOXC_ERR_UNSUPPORTED.  The
 * stream must belong to the current device (else NEOXC_ERR_ARG).  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the one array, so calls whose
 * work overlaps on the GPU (e.g. on two streams at once) race; serialise
 * them on one stream. */
int neoxc_dev_gam4_dscf_noalloc(void* stream, int64_t ne, int64_t np,
                                const double* d_GAM_ee,
                                const double* d_GAM_2s, const double* d_DE,
                                const double* d_DP, double* d_focke,
                                double* d_fockp, double* d_E_gam4);
int neoxc_dev_eg3ic1(void* stream, int64_t ne, int64_t np,
                     const double* d_DE, const double* d_DP,
                     const double* d_GM3ICR, double* d_focke,
                     double* d_fockp, double* d_E_gam3);
int neoxc_dev_eg2ic1(void* stream, int64_t ne, int64_t np,
                     const double* d_DE, const double* d_DP,
                     const double* d_GM2ICR, const double* d_GM2SICR,
                     double* d_FE, double* d_SE, double* d_FP, double* d_SP,
                     double* d_E_gam2, double* d_S_gam2);
int neoxc_dev_rxchfne_omg2(void* stream, int64_t ne, int64_t np,
                           const double* d_DAE, const double* d_DBE,
                           const double* d_DP, const double* d_GM2ICR,
                           double* d_FAE, double* d_FP, double* d_FBE,
                           double* d_E);

/* ---- factorised gam_4 Fock build (no routine of its own in the reference) --
 * Same focke, fockp (accumulated) and E_gam4 (overwritten) as GAM4_DSCF
 * (gam4_DSCF_OMP.f:2-320, element gam_4_OMP.f:712-1192) for pair-symmetric
 * tables: gs(p;ab;cd) = gs(p;cd;ab) and (ab|cd) = (cd|ab), which the
 * reference's GAM2_IC1 (gam2_IC1_OMP.f:141-176) and calc_GAM_ee produce.
 * Work O(ne^4 np^2 + ne^5) instead of O(ne^8 np^2).  Limits: ne <= 64,
 * np <= 255.  The host-array entry checks the symmetry (relative 1e-12)
 * and returns NEOXC_ERR_ARG without computing when it fails; the device
 * entry does not check.  gam4_dscf_ uses this path when the environment
 * variable NEOXC_GAM4_FACTORED is "1". */
int neoxc_gam4_fock_factored(int64_t ne, int64_t np, int64_t ngee,
                             int64_t ng2, const double* GAM_ee,
                             const double* GAM_2s, const double* DE,
                             const double* DP, double* focke, double* fockp,
                             double* E_gam4);
int neoxc_dev_gam4_fock_factored(void* stream, int64_t ne, int64_t np,
                                 const double* d_GAM_ee,
                                 const double* d_GAM_2s, const double* d_DE,
                                 const double* d_DP, double* d_focke,
                                 double* d_fockp, double* d_E_gam4);
/* Mixed-precision form of neoxc_dev_gam4_fock_factored (gam_4_OMP.f:712-1192
 * element, gam4_DSCF_OMP.f:266-307 contraction; the factorisation is new):
 * the one-index transforms and the focke contraction run on the tensor
 * cores (tcgen05.mma kind::tf32, each FP64 operand narrowed to FP32 and
 * split into two TF32 halves, three products, FP32 accumulation folded into
 * FP64 every 256 K, FP64 results); the two passes over GAM_2s multiply
 * FP32-narrowed elements with FP32 partial sums over 64 terms and FP64
 * beyond; the traces, gradients and final reductions are FP64 (~3e-6
 * relative in E_gam4 at nebf = 60, npbf = 24).  Same accumulate/overwrite
 * contract; returns after the stream has drained (it checks the kernels'
 * bounded-wait flag). */
int neoxc_dev_gam4_fock_factored_tc(void* stream, int64_t ne, int64_t np,
                                    const double* d_GAM_ee,
                                    const double* d_GAM_2s, const double* d_DE,
                                    const double* d_DP, double* d_focke,
                                    double* d_fockp, double* d_E_gam4);

/* ---- XCHF RHF SCF on the device ----------------------------------------------
 * xchf1_independent/xcscf.f:2-658 xcscf (the Roothaan branch, and the
 * second-order branch with NEOXC_SCF_SOSCF) with xchf1_fock.f:2-361 as the
 * Fock build: builds every
 * integral on the GPU (overlaps and core Hamiltonians, pure_ovlap.f and
 * gam_epcore.f; GAM_ep, gam_ep.f; GAM_1/GAM_1s, gam_1_OMP.f; GAM_ee,
 * gam_ee.f; GM2ICR/GM2sICR and GM3ICR in core), then iterates: Fock build
 * -> ROOTHAN for the nucleus (state nucst) -> Fock build -> ROOTHAN for the
 * electrons, until max|dDE| < 1e-6 (and max|dDP| < 1e-4 when npbf > 1), as
 * xcscf does.  gam_4 uses the factorised Fock build unless
 * NEOXC_SCF_GAM4_ELEMENT selects the element-wise GAM4_DSCF.
 * NEOXC_SCF_DIIS (no reference counterpart) extrapolates the electronic Fock
 * matrix over the last 8 iterations (error F DE S - S DE F) before ROOTHAN:
 * same converged state in fewer iterations.
 * NEOXC_SCF_MIXED (no reference counterpart) evaluates the gam_3 primitive
 * integrals with FP32 McMurchie-Davidson recursions (FP64 Boys function,
 * FP64 sums over primitives and geminal pairs); everything else stays FP64.
 * NEOXC_SCF_MIXED_GAM2 does the same for the gam_2 primitive items, with
 * dynamic precision: an item whose FP32 contribution exceeds the threshold
 * of neoxc_set_mixed_threshold is re-evaluated in FP64 (gam_1 is FP64).
 *   DE (in: initial electronic density, e.g. from guessCE; out: converged)
 *   DP (in: initial nuclear density unless NEOXC_SCF_GUESS_PROT; out)
 *   E_init[16], E_final[16]: energy slots 0 E_total 1 E_nuc 2 E_ecore
 *     3 E_pcore 4 E_ep 5 E_ee 6 E_gam1 7 E_gam2 8 E_gam3 9 E_gam4 10 S_total
 *     11 S_gam1 12 S_gam2 13 H_expect 14 max|dDE| 15 max|dDP| of the first
 *     and of the last Fock build ("INITIAL GUESS" / final energetics).
 *   history[4*maxit] (may be NULL): per iteration E_total, its change,
 *     max|dDE|, max|dDP|.
 *   niter, converged: iterations run and 1 when the thresholds were met.
 * Limits: nebf, npbf <= 64; with gam_3 (nelec > 2) nebf <= 20. */
#define NEOXC_SCF_GUESS_PROT 1     /* DP from the nuclear core Hamiltonian */
#define NEOXC_SCF_DIIS 2           /* Pulay DIIS on the electronic Fock (new) */
#define NEOXC_SCF_GAM4_ELEMENT 4   /* element-wise GAM4_DSCF for gam_4     */
#define NEOXC_SCF_MIXED 8          /* gam_3 MD integrals in FP32 (new)     */
#define NEOXC_SCF_MIXED_GAM2 16    /* gam_2 MD integrals in FP32, the large
                                      items in FP64 (new) */
#define NEOXC_SCF_GUESS_ELEC 32    /* DE (XCHF: guess_elec, xcscf.f:660) or
                                      DAE, DBE (XCUHF: guess_A_elec) from the
                                      electronic core Hamiltonian */
#define NEOXC_SCF_SOSCF 128        /* second-order steps on the electronic
                                      orbitals (soscf.f, xcscf.f:459-485)
                                      once the orbital gradient is below 1;
                                      exclusive with NEOXC_SCF_DIIS */
#define NEOXC_SCF_SCREEN 64        /* skip gam_3 (bra, ket) primitive pairs
                                      whose Schwarz-type estimate is below
                                      1e-12 (new; the reference evaluates
                                      every tuple) */
int neoxc_xchf_scf(int64_t nelec, int64_t nucst, int64_t nebf, int64_t npebf,
                   int64_t npbf, int64_t nat, int64_t ngtg1, double pmass,
                   const double* cat, const double* zan, const double* bcoef1,
                   const double* gamma1, const int64_t* KPESTR,
                   const int64_t* KPEEND, const int64_t* AMPEB2C,
                   const double* AGEBFCC, const double* AGNBFCC,
                   const double* ELCEX, const double* NUCEX,
                   const int64_t* ELCAM, const int64_t* NUCAM,
                   const double* ELCBFC, const double* NUCBFC, int64_t options,
                   int64_t maxit, double* DE, double* DP, double* E_init,
                   double* E_final, double* history, int64_t* niter,
                   int64_t* converged);

/* Dynamic-precision threshold of the mixed gam_2 build (NEOXC_SCF_MIXED_GAM2
 * in every entry point that takes it; no reference counterpart).  Each
 * primitive item is first evaluated with the FP32 tables (FP64 Boys
 * function, seeds and sums); an item whose contribution to a contracted
 * gam_2 element exceeds tau in magnitude is re-evaluated entirely in FP64.
 * tau = 0 re-evaluates every item, INFINITY none.  Default 1e-5.
 * Process-wide; NEOXC_ERR_ARG for tau < 0 or NaN.  neoxc_get_mixed_threshold
 * returns the current value. */
int neoxc_set_mixed_threshold(double tau);
double neoxc_get_mixed_threshold(void);

/* ---- batched XCHF solves (no reference counterpart) ----------------------------
 * One job = the arguments of neoxc_xchf_scf for one system; the outputs are
 * written into the job.  neoxc_xchf_scf_batch runs the jobs on nworkers
 * host threads, each with its own CUDA stream: a worker takes the next job
 * as soon as it is free, and a job starts when neoxc_admit (below) starts
 * it, with the device's free memory re-read at each admission; a job that
 * can never fit ends with NEOXC_ERR_NOMEM, unstarted, and the others go on.
 * Each job's result equals a separate neoxc_xchf_scf call.
 * Returns NEOXC_OK, or the first failing job's code (every job's own code is
 * in its status field). */
typedef struct neoxc_xchf_job {
  int64_t nelec, nucst, nebf, npebf, npbf, nat, ngtg1;
  double pmass;
  const double *cat, *zan, *bcoef1, *gamma1;
  const int64_t *KPESTR, *KPEEND, *AMPEB2C;
  const double *AGEBFCC, *AGNBFCC, *ELCEX, *NUCEX;
  const int64_t *ELCAM, *NUCAM;
  const double *ELCBFC, *NUCBFC;
  double *DE, *DP;           /* in: start densities; out: converged */
  double *E_init, *E_final;  /* [16] each, slots as neoxc_xchf_scf */
  double *history;           /* [4*maxit] or NULL */
  double *CE, *CP;           /* out, or NULL: final MO coefficients
                                (column-major, ROOTHAN's VECE / VECP,
                                orbitals by ascending energy) */
  double *EE, *EP;           /* out, or NULL: orbital energies */
  int64_t niter, converged;  /* out */
  int32_t status;            /* out: NEOXC_OK or an error code */
  int32_t reserved;
  double t_submit, t_start, t_end;  /* out (server): seconds since start */
} neoxc_xchf_job;
int64_t neoxc_xchf_job_size(void);   /* sizeof(neoxc_xchf_job), for bindings */
/* One job on the library stream (neoxc_xchf_scf with the job's arrays, plus
 * the optional MO outputs); returns the job's status. */
int neoxc_xchf_scf_job(neoxc_xchf_job* job, int64_t options, int64_t maxit);
int neoxc_xchf_scf_batch(neoxc_xchf_job* jobs, int64_t njobs, int64_t nworkers,
                         int64_t options, int64_t maxit);
/* GAM3_IC1 for many systems at once (no reference counterpart; the batched
 * form of the reference's per-system call, for proton-position or geometry
 * scans): each job's basis arrays are read from a neoxc_xchf_job (its other
 * fields are unused) and GM3ICR[k] receives job k's tensor.  The
 * four-particle terms of all systems of one angular class run in ONE
 * persistent launch over a device work queue (an atomic counter over every
 * system's work items, so uneven systems balance across the SMs); the
 * persistent grid (CTAs per SM, items per grab) is chosen per class and
 * precision by a built-in autotuner on the first call (timed samples of the
 * real work), whose choices neoxc_gam3_batch_tuning reports.  options:
 * NEOXC_SCF_MIXED, NEOXC_SCF_SCREEN as neoxc_gam3_ic1_opts.  seconds
 * (optional): device time of the build (copies excluded).  Every system's
 * tensor equals its neoxc_gam3_ic1 result.  nebf <= 20 per job. */
int neoxc_gam3_ic1_batch(const neoxc_xchf_job* jobs, int64_t njobs, int64_t options,
                         double* const* GM3ICR, double* seconds);
/* The autotuner's choices so far as a JSON array (written into buf up to len
 * bytes, NUL-terminated); returns the full length. */
int64_t neoxc_gam3_batch_tuning(char* buf, int64_t len);

/* Admission by device memory (no reference counterpart), the rule the
 * batch driver and the server apply each time a job is about to start,
 * with free_bytes re-read from the device at that moment:
 *   limit = 0.8 * (free_bytes + in_use_bytes), lowered to cap_bytes if
 *           cap_bytes > 0 (in_use_bytes: footprints of the jobs running);
 *   need > limit                                -> NEOXC_ADMIT_REFUSE (the
 *            job can never fit; it ends with NEOXC_ERR_NOMEM, unstarted);
 *   in_use + need <= limit, need <= 0.9 free    -> NEOXC_ADMIT_START;
 *   otherwise                                   -> NEOXC_ADMIT_WAIT (until
 *            a running job ends).  With nothing running a job never waits.
 * Pure host arithmetic; negative arguments -> NEOXC_ADMIT_REFUSE. */
#define NEOXC_ADMIT_START 0
#define NEOXC_ADMIT_WAIT 1
#define NEOXC_ADMIT_REFUSE 2
int neoxc_admit(int64_t need_bytes, int64_t free_bytes, int64_t in_use_bytes,
                int64_t cap_bytes);
/* Device bytes one XCHF solve holds at its peak (integral tensors, SCF
 * state, contraction scratch): the footprint neoxc_admit weighs. */
int64_t neoxc_xchf_job_bytes(const neoxc_xchf_job* job, int64_t options);

/* ---- serving loop for XCHF solves (no reference counterpart) -------------------
 * Continuous batching: requests are queued with submit (non-blocking) and
 * taken by nworkers threads, each with its own CUDA stream, as soon as a
 * worker is free and neoxc_admit starts the request (free memory re-read at
 * each admission; set_budget caps the bytes the server's running jobs may
 * hold together, 0 = no cap); a request may arrive while others run and its
 * work overlaps theirs on the GPU.  A request that can never fit ends with
 * status NEOXC_ERR_NOMEM without starting; one whose energy or Fock matrix
 * turns non-finite ends with NEOXC_ERR_NUMERIC; one that reaches maxit ends
 * with status NEOXC_OK and converged = 0.  The job struct and its arrays
 * must stay valid until wait() reports it done; the job's t_submit /
 * t_start / t_end record the request's life.  wait() returns the job's
 * status, or NEOXC_ERR_TIMEOUT after timeout_s seconds (the job stays
 * queued or running; wait again).  stop() drains the queue and joins the
 * workers. */
typedef struct neoxc_xchf_server neoxc_xchf_server;
neoxc_xchf_server* neoxc_xchf_server_start(int64_t nworkers, int64_t options,
                                           int64_t maxit);
int neoxc_xchf_server_set_budget(neoxc_xchf_server* srv, int64_t cap_bytes);
int neoxc_xchf_server_submit(neoxc_xchf_server* srv, neoxc_xchf_job* job);
int neoxc_xchf_server_wait(neoxc_xchf_server* srv, neoxc_xchf_job* job,
                           double timeout_s);
int neoxc_xchf_server_stop(neoxc_xchf_server* srv);

/* xcuhf/xcuhf_scf.f:2-582 (Roothaan branch; SOSCF not ported) with
 * UHF_FOCK (xcuhf_fock.f:2-427) on the device: builds every integral
 * (overlaps, core Hamiltonians, GAM_ep, GAM_1/GAM_1s, GAM_ee, GM2ICR /
 * GM2sICR, GM3ICR, OMG4_ICR) and iterates UHF_FOCK / UROOTHAN (proton,
 * alpha, beta from one Fock build) / DENDIF until the alpha and beta
 * densities move less than 1e-6 (and the proton's less than 1e-4 when
 * npbf > 1).  NAE + NBE = nelec.  DAE, DBE in: start densities unless
 * NEOXC_SCF_GUESS_ELEC; DP as in neoxc_xchf_scf; all three out.
 * E_init / E_final [16]: 0 E_total, 1 E_nuc, 2 E_ecore, 3 E_pcore, 4 E_ep,
 * 5 E_ee, 6 E_OMG1, 7 E_OMG2, 8 E_OMG3, 9 E_OMG4 (2..9 divided by S_total,
 * as the log prints them), 10 S_total, 11 S_OMG1, 12 S_OMG2 (raw),
 * 13 / 14 / 15 last alpha / beta / proton density change.  history
 * [4*maxit]: E_total, its change, max(alpha, beta) density change, proton
 * density change.  Options: NEOXC_SCF_GUESS_ELEC, NEOXC_SCF_GUESS_PROT,
 * NEOXC_SCF_DIIS (alpha and beta Fock matrices, separately, once both
 * densities move less than 0.1 per iteration),
 * NEOXC_SCF_MIXED, NEOXC_SCF_MIXED_GAM2.  Limits: nebf, npbf <= 64,
 * nebf <= 20 with gam_3, nebf <= 12 with OMG4. */
int neoxc_xcuhf_scf(int64_t nelec, int64_t NAE, int64_t NBE, int64_t nucst,
                    int64_t nebf, int64_t npebf, int64_t npbf, int64_t nat,
                    int64_t ngtg1, double pmass, const double* cat, const double* zan,
                    const double* bcoef1, const double* gamma1, const int64_t* KPESTR,
                    const int64_t* KPEEND, const int64_t* AMPEB2C,
                    const double* AGEBFCC, const double* AGNBFCC, const double* ELCEX,
                    const double* NUCEX, const int64_t* ELCAM, const int64_t* NUCAM,
                    const double* ELCBFC, const double* NUCBFC, int64_t options,
                    int64_t maxit, double* DAE, double* DBE, double* DP, double* E_init,
                    double* E_final, double* history, int64_t* niter,
                    int64_t* converged);

/* One-special-electron RXCHF SCF on the device (NBE = 1), `kind`:
 *   NEOXC_RX_NE     rxchfne/rxchfne_scf.f xcrxchfne: RXCHF-ne, NAE
 *                   closed-shell regular electrons (NAalpE, NAbetE unused);
 *   NEOXC_RX_CU_NE  rxchfne/rxcuhfne_scf.f xcrxcuhfne, EXCHLEV 0: NAalpE
 *                   alpha and NAbetE beta regular electrons (NAE unused);
 *   NEOXC_RX_CU_AE  the same with EXCHLEV 1 (LADDEXCH: RXCUHFne_*_OMG2).
 * Builds Se, Sp, GAM_ecore, GAM_pcore, GAM_ee, GAM_1 / GAM_1s of
 * RXCHF_GAM1_OMP_MD (rxchf/rxchf_gam_1_OMP.f) and GM2ICR / GM2exICR of
 * RXCHFne_GAM2_IC1; guesses as RXCHF_guess_elec / RXCUHF_guess_elec
 * (rxchf/rxchf_scf.f:785-844, rxchf/rxcuhf_scf.f:863-934) and guess_prot2;
 * then the LOCBSE2 iteration: per iteration a Fock build (RXCHFne_FOCK,
 * rxchfne_fock.f:2-250, or RXCUHFne_FOCK) and the proton's UROOTHAN, then
 * micro-iterations (at most 200) of regular-electron UROOTHAN and
 * RXCHF_OCBSE2 / RXCUHF_OCBSE2 (rxchf/rxchf_scf.f:1124-1330) for the
 * special electron, each followed by a Fock build, until the regular and
 * special densities move less than 1e-6; converged when the proton density
 * of an iteration moved less than 1e-4.  The second-order steps the
 * reference takes for the regular electrons (LSOSCF) are not ported: they
 * change the path, not the converged state.
 * Out: DA (DAE, or DAalpE), DAbet (DAbetE, open shell only), DBE, DP;
 * E_init / E_final [16]: 0 E_TOTAL (with E_nuc), 1 E_NUC, 2 E_ECORE, 3 E_EE,
 * 4 E_OMG1, 5 E_OMG2, 6 S_TOTAL (the components the logs print), 7 E_P_OMG1,
 * 8 E_P_OMG2, 9 S_P_OMG1, 10 E_BE_OMG1, 11 S_BE_OMG1, 12 / 13 / 14 last
 * regular / special / proton density change, 15 micro-iterations of the
 * last iteration; history [3*maxit]: E_TOTAL, micro-iterations, proton
 * density change per iteration.  Limits: nebf, npbf <= 64. */
/* rxchfne/rxchfne_fock.f:2-250 RXCHFne_FOCK (open_shell = 0: DA = DAE of
 * NAE closed-shell regular electrons, FA = FAE) or rxchfne/rxcuhfne_fock.f
 * RXCUHFne_FOCK (open_shell = 1: DA / DAbet = DAalpE / DAbetE with NAalpE /
 * NAbetE electrons, FA / FAbet = FAalpE / FAbetE; addexch = LADDEXCH adds
 * the RXCUHFne_*_OMG2 exchange terms from GM2exICR) in one device pass.
 * GAM_1 / GAM_1s are arguments (the reference's RXCHF_FP_OMG1 and
 * RXCHF_FBE_OMG1 read GAM_1.ufm / GAM_1s.ufm); GM2exICR is read only with
 * addexch.  Outputs overwritten: FP, FA, FAbet (open shell), FBE and the
 * routine's energies (E_total without E_nuc, as the routine returns it).
 * Limits: nebf, npbf <= 64. */
int neoxc_rxchfne_fock(int64_t open_shell, int64_t addexch, int64_t NAE,
                       int64_t NAalpE, int64_t NAbetE, int64_t nebf, int64_t npbf,
                       const double* DA, const double* DAbet, const double* DBE,
                       const double* DP, const double* GAM_ecore, const double* GAM_ee,
                       const double* GAM_1, const double* GAM_1s, const double* GM2ICR,
                       const double* GM2exICR, double* FP, double* FA, double* FAbet,
                       double* FBE, double* E_ecore, double* E_GAMee, double* E_OMG1,
                       double* E_OMG2, double* E_total, double* S_total);

#define NEOXC_RX_NE 0
#define NEOXC_RX_CU_NE 1
#define NEOXC_RX_CU_AE 2
#define NEOXC_RX_NO_OCBSE 16   /* or-ed into kind: the reference's LOCBSE =
   .false. branch -- RXCHF_guess_A/B_elec (rxchf/rxchf_scf.f:733-784), a Fock
   build at the top of every micro-iteration and UROOTHAN of FBE for the
   special electron's lowest orbital instead of RXCHF_OCBSE2 */
int neoxc_rx_scf(int64_t kind, int64_t NAE, int64_t NAalpE, int64_t NAbetE,
                 int64_t nucst, int64_t nebf, int64_t npebf, int64_t npbf,
                 int64_t nat, int64_t ngtg1, double pmass, const double* cat,
                 const double* zan, const double* bcoef1, const double* gamma1,
                 const int64_t* KPESTR, const int64_t* KPEEND,
                 const int64_t* AMPEB2C, const double* AGEBFCC,
                 const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                 const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                 const double* NUCBFC, int64_t maxit, double* DA, double* DAbet,
                 double* DBE, double* DP, double* E_init, double* E_final,
                 double* history, int64_t* niter, int64_t* converged);

/* ---- open-shell XCUHF contractions: xcuhf/xcuhf_omg{1..4}.f ------------ */
/* Same arguments, packed layouts and semantics as the reference: the Fock
 * matrix (FAE or FP) accumulates (add2fock), the SAE / SP matrices and the energies are
 * overwritten.  FAE_* computes the Fock matrix of the spin whose density
 * and count come first; the reference's beta call swaps (NAE,DAE) with
 * (NBE,DBE).  The spin-term flags (LAA, LAB, ..., L4A, L3A1B, ...) are
 * derived from NAE/NBE exactly as in the reference.  Limits: nebf <= 256
 * (OMG1/OMG2), 28 (OMG3), 12 (OMG4); beyond them NEOXC_ERR_UNSUPPORTED. */
/* xcuhf_omg1.f:2-81 FAE_OMG1; GAM_1 / GAM_1s (pack_4D(je,ie,jp,ip)) are
 * arguments here (the reference reads GAM_1.ufm / GAM_1s.ufm). */
int neoxc_fae_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DAE,
                   const double* DP, const double* GAM_1, const double* GAM_1s,
                   double* FAE, double* SAE1, double* E_AE_OMG1, double* S_AE_OMG1);
/* xcuhf_omg1.f:83-163 UFP_OMG1 */
int neoxc_ufp_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DETOT,
                   const double* DP, const double* GAM_1, const double* GAM_1s,
                   double* FP, double* SP1, double* E_P_OMG1, double* S_P_OMG1);
/* xcuhf_omg2.f:2-300 FAE_OMG2 (DETOT is unused, as in the reference) */
int neoxc_fae_omg2(int64_t Nchunks, int64_t NAE, int64_t NBE, int64_t nebf,
                   int64_t npbf, int64_t ng2, const double* DAE, const double* DBE,
                   const double* DETOT, const double* DP, const double* GM2ICR,
                   const double* GM2SICR, double* FAE, double* SAE2,
                   double* E_AE_OMG2, double* S_AE_OMG2);
/* xcuhf_omg2.f:302-612 UFP_OMG2 */
int neoxc_ufp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DETOT, const double* DP, const double* GM2ICR,
                   const double* GM2SICR, double* FP, double* SP2, double* E_P_OMG2,
                   double* S_P_OMG2);
/* xcuhf_omg3.f:2-282 FAE_OMG3 */
int neoxc_fae_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM3ICR, double* FAE,
                   double* E_AE_OMG3);
/* xcuhf_omg3.f:284-588 UFP_OMG3 */
int neoxc_ufp_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM3ICR, double* FP,
                   double* E_P_OMG3);
/* xcuhf_omg4.f:2-510 FAE_OMG4 (GM4ICR from OMG4_ICR) */
int neoxc_fae_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM4ICR, double* FAE,
                   double* E_AE_OMG4);
/* xcuhf_omg4.f:512-1078 UFP_OMG4 */
int neoxc_ufp_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM4ICR, double* FP,
                   double* E_P_OMG4);
/* xcuhf_omg4.f:1080-1315 OMG4_ICR: the raw 5-particle tensor
 * (calc_GAM_4_integral, no permutational symmetrisation) at index_GAM_4PK2;
 * GAM_ee is an argument (the reference reads GAM_ee.ufm). */
int neoxc_omg4_icr(int64_t Nchunks, int64_t ne, int64_t np, int64_t ngee, int64_t ng2,
                   int64_t ng4, const double* GAM_2s, const double* GAM_ee,
                   double* GAM_4);
/* Device pointers, on `stream`: FAE_OMGk, FAE_OMGk for beta (spins
 * exchanged) and UFP_OMGk of one rank K (2: G = GM2ICR, Gs = GM2SICR;
 * 3: GM3ICR; 4: OMG4_ICR, Gs = NULL) from one pass over the tensor.  Any
 * output may be NULL.  Fock matrices accumulate, S* are overwritten,
 * d_E[6] = {E_AE, E_BE, E_P, S_AE, S_BE, S_P} is overwritten. */
int neoxc_dev_xcuhf_omg(void* stream, int64_t K, int64_t ne, int64_t np, int64_t NAE,
                        int64_t NBE, const double* d_G, const double* d_Gs,
                        const double* d_DAE, const double* d_DBE, const double* d_DP,
                        double* d_FAE, double* d_FBE, double* d_FP, double* d_SAE,
                        double* d_SBE, double* d_SP, double* d_E);
int neoxc_dev_omg4_icr(void* stream, int64_t ne, int64_t np, const double* d_gee,
                       const double* d_g2s, double* d_g4);

/* ---- RXCHF-fe / RXCUHF-fe / RXCUHF-ae contractions: rxchf/, rxchfne/ --- */
/* Same argument lists, packed layouts and semantics as the reference: every
 * output matrix (Fock and overlap-Fock alike) accumulates (add2fock), the
 * energies are overwritten.  The in-core tensors are arguments (GM2_1ICR,
 * GM2_2ICR, GM2sICR from RXCHF_GAM2_IC1; GM3_1ICR, GM3_2ICR from
 * RXCHF_GAM3_IC1; GM4ICR; GM2ICR, GM2exICR from RXCHFne_GAM2_IC1). */
/* rxchfne/rxcuhfne_omg2.f:2-130 RXCUHFne_FE_OMG2 (DAbetE unused, as there) */
int neoxc_rxcuhfne_fe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                           const double* DAalpE, const double* DAbetE, const double* DAtotE,
                           const double* DBE, const double* DP, const double* GM2ICR,
                           const double* GM2exICR, double* FAalpE, double* FAbetE,
                           double* E_AE_OMG2);
/* rxcuhfne_omg2.f:239-345 RXCUHFne_FP_OMG2 */
int neoxc_rxcuhfne_fp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                           int64_t NAalpE, int64_t NBE, const double* DAalpE,
                           const double* DAtotE, const double* DBE, const double* DP,
                           const double* GM2ICR, const double* GM2exICR, double* FP,
                           double* E_P_OMG2);
/* rxcuhfne_omg2.f:445-551 RXCUHFne_FBE_OMG2 */
int neoxc_rxcuhfne_fbe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                            int64_t NAalpE, int64_t NBE, const double* DAalpE,
                            const double* DAtotE, const double* DBE, const double* DP,
                            const double* GM2ICR, const double* GM2exICR, double* FBE,
                            double* E_BE_OMG2);
/* rxchf/rxchf_omg2.f:2-114 RXCHF_FAE_OMG2 (F = FAE, S = SAE), :231-334
 * RXCHF_FP_OMG2 (FP, SP), :449-552 RXCHF_FBE_OMG2 (FBE, SBE) */
int neoxc_rxchf_fae_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM2_1ICR, const double* GM2_2ICR,
                         const double* GM2sICR, double* FAE, double* SAE,
                         double* E_AE_OMG2, double* S_AE_OMG2);
int neoxc_rxchf_fp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                        const double* DAE, const double* DBE, const double* DP,
                        const double* GM2_1ICR, const double* GM2_2ICR,
                        const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2,
                        double* S_P_OMG2);
int neoxc_rxchf_fbe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM2_1ICR, const double* GM2_2ICR,
                         const double* GM2sICR, double* FBE, double* SBE,
                         double* E_BE_OMG2, double* S_BE_OMG2);
/* rxchf/rxchf_omg3.f:2-105 RXCHF_FAE_OMG3, :263-366 RXCHF_FP_OMG3,
 * :486-589 RXCHF_FBE_OMG3 */
int neoxc_rxchf_fae_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM3_1ICR, const double* GM3_2ICR, double* FAE,
                         double* E_AE_OMG3);
int neoxc_rxchf_fp_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                        const double* DAE, const double* DBE, const double* DP,
                        const double* GM3_1ICR, const double* GM3_2ICR, double* FP,
                        double* E_P_OMG3);
int neoxc_rxchf_fbe_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM3_1ICR, const double* GM3_2ICR, double* FBE,
                         double* E_BE_OMG3);
/* rxchf/rxchf_omg4.f:2-105 RXCHF_FAE_OMG4, :223-326 RXCHF_FP_OMG4,
 * :444-547 RXCHF_FBE_OMG4 */
int neoxc_rxchf_fae_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM4ICR, double* FAE, double* E_AE_OMG4);
int neoxc_rxchf_fp_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                        const double* DAE, const double* DBE, const double* DP,
                        const double* GM4ICR, double* FP, double* E_P_OMG4);
int neoxc_rxchf_fbe_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                         const double* DAE, const double* DBE, const double* DP,
                         const double* GM4ICR, double* FBE, double* E_BE_OMG4);
/* rxchf/rxcuhf_omg2.f:2-126 RXCUHF_FE_OMG2 (DAbetE unused, as there) */
int neoxc_rxcuhf_fe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                         const double* DAalpE, const double* DAbetE, const double* DAtotE,
                         const double* DBE, const double* DP, const double* GM2_1ICR,
                         const double* GM2_2ICR, const double* GM2sICR, double* FAalpE,
                         double* FAbetE, double* SAalpE, double* E_AE_OMG2,
                         double* S_AE_OMG2);
/* rxcuhf_omg2.f:253-352 RXCUHF_FP_OMG2, :469-576 RXCUHF_FBE_OMG2 */
int neoxc_rxcuhf_fp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                         int64_t NAalpE, int64_t NBE, const double* DAalpE,
                         const double* DAtotE, const double* DBE, const double* DP,
                         const double* GM2_1ICR, const double* GM2_2ICR,
                         const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2,
                         double* S_P_OMG2);
int neoxc_rxcuhf_fbe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                          int64_t NAalpE, int64_t NBE, const double* DAalpE,
                          const double* DAtotE, const double* DBE, const double* DP,
                          const double* GM2_1ICR, const double* GM2_2ICR,
                          const double* GM2sICR, double* FBE, double* SBE,
                          double* E_BE_OMG2, double* S_BE_OMG2);
/* rxchf/rxcuhf_omg3.f:2-107 RXCUHF_FE_OMG3, :270-371 RXCUHF_FP_OMG3,
 * :499-600 RXCUHF_FBE_OMG3 */
int neoxc_rxcuhf_fe_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                         const double* DAalpE, const double* DAbetE, const double* DAtotE,
                         const double* DBE, const double* DP, const double* GM3_1ICR,
                         const double* GM3_2ICR, double* FAalpE, double* FAbetE,
                         double* E_AE_OMG3);
int neoxc_rxcuhf_fp_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                         const double* DAalpE, const double* DAbetE, const double* DAtotE,
                         const double* DBE, const double* DP, const double* GM3_1ICR,
                         const double* GM3_2ICR, double* FP, double* E_P_OMG3);
int neoxc_rxcuhf_fbe_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                          const double* DAalpE, const double* DAbetE, const double* DAtotE,
                          const double* DBE, const double* DP, const double* GM3_1ICR,
                          const double* GM3_2ICR, double* FBE, double* E_BE_OMG3);
/* rxchf/rxchf_omg1.f:2-82 RXCHF_FP_OMG1 and :84-165 RXCHF_FBE_OMG1 (GAM_1 /
 * GAM_1s as arguments; the special electron's density DBE) */
int neoxc_rxchf_fp_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DBE,
                        const double* DP, const double* GAM_1, const double* GAM_1s,
                        double* FP, double* SP, double* E_P_OMG1, double* S_P_OMG1);
int neoxc_rxchf_fbe_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DBE,
                         const double* DP, const double* GAM_1, const double* GAM_1s,
                         double* FBE, double* SBE, double* E_BE_OMG1, double* S_BE_OMG1);

/* ---- on-disk formats: xchf1_independent/GAM_IO.f (host only, no GPU) --- */
/* Direct-access integral files (*.ufm, GAM_IO.f:1-245): record ia (1-based)
 * holds the FP64 at packed index ia, records `recl` bytes long with the value
 * first (RECL=8 counted in bytes = 8; ifort's default 4-byte units = 32).
 * recl <= 0 takes NEOXC_UFM_RECL from the environment, default 8.
 * Replaces the read loops of read_GAM_ee/ep/ecore/pcore and the writes in
 * gam_ee.f:143-155, gam_ep.f:141, gam_4_OMP.f:263. */
int neoxc_ufm_read(const char* path, int64_t n, int64_t recl, double* out);
int neoxc_ufm_write(const char* path, const double* v, int64_t n, int64_t recl);
/* GAM_IO.f:471-518 PUSQLF: nmo MOs of nbf coefficients (V column-major,
 * V[:,j] = MO j) as FORMAT(I2,I3,1P,5E15.8) rows labelled MOD(j,100),
 * MOD(row,1000) -- the FinalC*.dat files. */
int neoxc_mo_write(const char* path, int64_t nbf, int64_t nmo, const double* V);
/* GAM_IO.f:275-303 (read_elec_density's VEC group, FORMAT(I2,I3,5E15.8)):
 * the guessC*.inp / FinalC*.dat layout back into V; a label that does not
 * match returns NEOXC_ERR_IO (the reference prints 9060 and STOPs). */
int neoxc_mo_read(const char* path, int64_t nbf, int64_t nmo, double* V);
/* GAM_IO.f:306-339: D = prefac * sum_{k=kstart..klast} C(:,k) C(:,k)^T
 * (1-based MO indices; read_elec_density: 1..nelec/2, prefac 2;
 * read_nuc_density: NUCST..NUCST, prefac 1). */
int neoxc_mo_density(int64_t nbf, int64_t kstart, int64_t klast, double prefac,
                     const double* C, double* D);
/* ENUCRP.dat (class_nuc_rep.f:39-41 write, xcscf.f:248-250 read): one
 * list-directed real, the classical nuclear repulsion energy. */
int neoxc_enuc_write(const char* path, double E_nuc);
int neoxc_enuc_read(const char* path, double* E_nuc);

/* ---- diagnostics (no reference counterpart) --------------------------- */
/* Sustained FP64 FMA throughput of the current device in TFLOP/s (2 FLOP
 * per FMA), the denominator of the FP64 rooflines. */
int neoxc_probe_fp64(double* tflops);

/* ---- Fortran external-subroutine shims (all arguments by reference) --- */
/* Same argument lists as the reference subroutines; on error they print a
 * message to stderr and record it for neoxc_last_error().  gam4_icr_ and
 * gam4_dscf_ read GAM_ee.ufm (and GAM_2s.ufm) from the working directory
 * like the reference; NEOXC_UFM_RECL sets the record length in bytes
 * (default 8: RECL counted in bytes; 32 for ifort without byterecl). */
void gam4_dscf_(const int64_t* NG4CHK, const int64_t* ne, const int64_t* np,
                const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
                const double* DE, const double* DP, double* focke,
                double* fockp, double* E_gam4);
void gam4_icr_(const int64_t* Nchunks, const int64_t* ne, const int64_t* np,
               const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
               const double* GAM_2s, double* GAM_4);
void eg4icr_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng4, const double* DE, const double* DP,
             const double* GM4ICR, double* focke, double* fockp,
             double* E_gam4);
void eg3ic1_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng3, const double* DE, const double* DP,
             const double* GM3ICR, double* focke, double* fockp,
             double* E_gam3);
void eg2ic1_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng2, const double* DE, const double* DP,
             const double* GM2ICR, const double* GM2SICR, double* FE,
             double* SE, double* FP, double* SP, double* E_gam2,
             double* S_gam2);
void gam2_ic1_(const int64_t* Nchunks, const int64_t* nebf,
               const int64_t* npebf, const int64_t* npbf, const int64_t* ng2,
               const int64_t* ng2prm, const int64_t* nat,
               const int64_t* ngtg1, const double* pmass, const double* cat,
               const double* zan, const double* bcoef1, const double* gamma1,
               const int64_t* KPESTR, const int64_t* KPEEND,
               const int64_t* AMPEB2C, const double* AGEBFCC,
               const double* AGNBFCC, const double* ELCEX,
               const double* NUCEX, const int64_t* ELCAM,
               const int64_t* NUCAM, const double* ELCBFC,
               const double* NUCBFC, double* GM2ICR, double* GM2sICR);
void gam3_ic1_(const int64_t* Nchunks, const int64_t* nebf,
               const int64_t* npebf, const int64_t* npbf, const int64_t* ng3,
               const int64_t* ng3prm, const int64_t* nat,
               const int64_t* ngtg1, const double* pmass, const double* cat,
               const double* zan, const double* bcoef1, const double* gamma1,
               const int64_t* KPESTR, const int64_t* KPEEND,
               const int64_t* AMPEB2C, const double* AGEBFCC,
               const double* AGNBFCC, const double* ELCEX,
               const double* NUCEX, const int64_t* ELCAM,
               const int64_t* NUCAM, const double* ELCBFC,
               const double* NUCBFC, double* GM3ICR);
void gam3_dscf_(const int64_t* Nchunks, const int64_t* nebf,
                const int64_t* npebf, const int64_t* npbf, const int64_t* ng3,
                const int64_t* ng3prm, const int64_t* nat,
                const int64_t* ngtg1, const double* pmass, const double* cat,
                const double* zan, const double* bcoef1, const double* gamma1,
                const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC,
                const double* AGNBFCC, const double* ELCEX,
                const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC,
                const double* NUCBFC, const double* DE, const double* DP,
                double* focke, double* fockp, double* E_gam3);
void gam2_dscf_(const int64_t* Nchunks, const int64_t* nebf,
                const int64_t* npebf, const int64_t* npbf, const int64_t* ng2,
                const int64_t* ng2prm, const int64_t* nat,
                const int64_t* ngtg1, const double* pmass, const double* cat,
                const double* zan, const double* bcoef1, const double* gamma1,
                const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC,
                const double* AGNBFCC, const double* ELCEX,
                const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC,
                const double* NUCBFC, const double* DE, const double* DP,
                double* focke, double* fockp, double* se2, double* sp2,
                double* E_gam2, double* S_gam2);
void rxchfne_gam2_ic1_(const int64_t* Nchunks, const int64_t* nebf,
                       const int64_t* npebf, const int64_t* npbf,
                       const int64_t* ng2, const int64_t* ng2prm,
                       const int64_t* nat, const int64_t* ngtg1,
                       const double* pmass, const double* cat,
                       const double* zan, const double* bcoef1,
                       const double* gamma1, const int64_t* KPESTR,
                       const int64_t* KPEEND, const int64_t* AMPEB2C,
                       const double* AGEBFCC, const double* AGNBFCC,
                       const double* ELCEX, const double* NUCEX,
                       const int64_t* ELCAM, const int64_t* NUCAM,
                       const double* ELCBFC, const double* NUCBFC,
                       double* GM2ICR, double* GM2exICR);
void rxchfne_fae_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                       const int64_t* npbf, const int64_t* ng2,
                       const double* DAE, const double* DBE, const double* DP,
                       const double* GM2ICR, double* FAE, double* E_AE_OMG2);
void rxchfne_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                      const int64_t* npbf, const int64_t* ng2,
                      const int64_t* NAE, const int64_t* NBE,
                      const double* DAE, const double* DBE, const double* DP,
                      const double* GM2ICR, double* FP, double* E_P_OMG2);
void rxchfne_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                       const int64_t* npbf, const int64_t* ng2,
                       const int64_t* NAE, const int64_t* NBE,
                       const double* DAE, const double* DBE, const double* DP,
                       const double* GM2ICR, double* FBE, double* E_BE_OMG2);
void calc_gam_ee_(const int64_t* nebf, const int64_t* npebf,
                  const int64_t* ngee, const int64_t* AMPEB2C,
                  const double* AGEBFCC, const double* ELCEX,
                  const int64_t* ELCAM, const double* ELCBFC);
/* GAM_IO.f readers and writer, same names, arguments and files as the
 * reference (GAM_ee.ufm, GAM_ep.ufm, GAM_ecr.ufm, GAM_pcr.ufm, novlap.ufm,
 * eovlap.ufm, guessCE.inp, guessCP.inp; write_MOs units 852/853/860/861/
 * 870/871 -> FinalCE/FinalCP/FinalCAE/FinalCBE/FinalCAalpE/FinalCAbetE.dat).
 * A failed read prints a message and leaves the output partly filled. */
void read_gam_ee_(const int64_t* ne, const int64_t* ngee, double* GAM_ee);
void read_gam_ep_(const int64_t* ne, const int64_t* np, const int64_t* ng1,
                  double* GAM_ep);
void read_gam_ecore_(const int64_t* ne, const int64_t* ne2, double* GAM_ecore);
void read_gam_pcore_(const int64_t* np, const int64_t* np2, double* GAM_pcore);
void read_nuc_ovlap_(const int64_t* np, double* GS);
void read_elec_ovlap_(const int64_t* ne, double* GS);
void read_elec_density_(const int64_t* nebf, const int64_t* n_particle, double* DE);
void read_nuc_density_(const int64_t* npbf, const int64_t* n_particle,
                       const int64_t* NUCST, double* DP);
void write_mos_(const int64_t* IFIL, const int64_t* nbf, const double* VEC);
/* xcuhf_omg{1..4}.f with the reference's argument lists; fae_omg1_ /
 * ufp_omg1_ read GAM_1.ufm and GAM_1s.ufm, omg4_icr_ reads GAM_ee.ufm, from
 * the working directory like the reference. */
void fae_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
               const double* DAE, const double* DP, double* FAE, double* SAE1,
               double* E_AE_OMG1, double* S_AE_OMG1);
void ufp_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
               const double* DETOT, const double* DP, double* FP, double* SP1,
               double* E_P_OMG1, double* S_P_OMG1);
void fae_omg2_(const int64_t* Nchunks, const int64_t* NAE, const int64_t* NBE,
               const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
               const double* DAE, const double* DBE, const double* DETOT,
               const double* DP, const double* GM2ICR, const double* GM2SICR,
               double* FAE, double* SAE2, double* E_AE_OMG2, double* S_AE_OMG2);
void ufp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng2, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DETOT,
               const double* DP, const double* GM2ICR, const double* GM2SICR,
               double* FP, double* SP2, double* E_P_OMG2, double* S_P_OMG2);
void fae_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng3, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM3ICR, double* FAE, double* E_AE_OMG3);
void ufp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng3, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM3ICR, double* FP, double* E_P_OMG3);
void fae_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng4, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM4ICR, double* FAE, double* E_AE_OMG4);
void ufp_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng4, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM4ICR, double* FP, double* E_P_OMG4);
void omg4_icr_(const int64_t* Nchunks, const int64_t* ne, const int64_t* np,
               const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
               const double* GAM_2s, double* GAM_4);
/* rxchf/rxchf_omg{1..4}.f, rxcuhf_omg{2,3}.f and rxchfne/rxcuhfne_omg2.f with
 * the reference's argument lists; rxchf_fp_omg1_ / rxchf_fbe_omg1_ read
 * GAM_1.ufm and GAM_1s.ufm from the working directory. */
void rxcuhfne_fe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                       const int64_t* ng2, const double* DAalpE, const double* DAbetE,
                       const double* DAtotE, const double* DBE, const double* DP,
                       const double* GM2ICR, const double* GM2exICR, double* FAalpE,
                       double* FAbetE, double* E_AE_OMG2);
void rxcuhfne_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                       const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE,
                       const double* DAalpE, const double* DAtotE, const double* DBE,
                       const double* DP, const double* GM2ICR, const double* GM2exICR,
                       double* FP, double* E_P_OMG2);
void rxcuhfne_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                        const int64_t* npbf, const int64_t* ng2, const int64_t* NAalpE,
                        const int64_t* NBE, const double* DAalpE, const double* DAtotE,
                        const double* DBE, const double* DP, const double* GM2ICR,
                        const double* GM2exICR, double* FBE, double* E_BE_OMG2);
void rxchf_fae_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng2, const double* DAE, const double* DBE,
                     const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,
                     const double* GM2sICR, double* FAE, double* SAE, double* E_AE_OMG2,
                     double* S_AE_OMG2);
void rxchf_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                    const int64_t* ng2, const double* DAE, const double* DBE,
                    const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,
                    const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2,
                    double* S_P_OMG2);
void rxchf_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng2, const double* DAE, const double* DBE,
                     const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,
                     const double* GM2sICR, double* FBE, double* SBE, double* E_BE_OMG2,
                     double* S_BE_OMG2);
void rxchf_fae_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng3, const double* DAE, const double* DBE,
                     const double* DP, const double* GM3_1ICR, const double* GM3_2ICR,
                     double* FAE, double* E_AE_OMG3);
void rxchf_fp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                    const int64_t* ng3, const double* DAE, const double* DBE,
                    const double* DP, const double* GM3_1ICR, const double* GM3_2ICR,
                    double* FP, double* E_P_OMG3);
void rxchf_fbe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng3, const double* DAE, const double* DBE,
                     const double* DP, const double* GM3_1ICR, const double* GM3_2ICR,
                     double* FBE, double* E_BE_OMG3);
void rxchf_fae_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng4, const double* DAE, const double* DBE,
                     const double* DP, const double* GM4ICR, double* FAE,
                     double* E_AE_OMG4);
void rxchf_fp_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                    const int64_t* ng4, const double* DAE, const double* DBE,
                    const double* DP, const double* GM4ICR, double* FP,
                    double* E_P_OMG4);
void rxchf_fbe_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng4, const double* DAE, const double* DBE,
                     const double* DP, const double* GM4ICR, double* FBE,
                     double* E_BE_OMG4);
void rxcuhf_fe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng2, const double* DAalpE, const double* DAbetE,
                     const double* DAtotE, const double* DBE, const double* DP,
                     const double* GM2_1ICR, const double* GM2_2ICR,
                     const double* GM2sICR, double* FAalpE, double* FAbetE,
                     double* SAalpE, double* E_AE_OMG2, double* S_AE_OMG2);
void rxcuhf_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE,
                     const double* DAalpE, const double* DAtotE, const double* DBE,
                     const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,
                     const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2,
                     double* S_P_OMG2);
void rxcuhf_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                      const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE,
                      const double* DAalpE, const double* DAtotE, const double* DBE,
                      const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,
                      const double* GM2sICR, double* FBE, double* SBE,
                      double* E_BE_OMG2, double* S_BE_OMG2);
void rxcuhf_fe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng3, const double* DAalpE, const double* DAbetE,
                     const double* DAtotE, const double* DBE, const double* DP,
                     const double* GM3_1ICR, const double* GM3_2ICR, double* FAalpE,
                     double* FAbetE, double* E_AE_OMG3);
void rxcuhf_fp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                     const int64_t* ng3, const double* DAalpE, const double* DAbetE,
                     const double* DAtotE, const double* DBE, const double* DP,
                     const double* GM3_1ICR, const double* GM3_2ICR, double* FP,
                     double* E_P_OMG3);
void rxcuhf_fbe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
                      const int64_t* ng3, const double* DAalpE, const double* DAbetE,
                      const double* DAtotE, const double* DBE, const double* DP,
                      const double* GM3_1ICR, const double* GM3_2ICR, double* FBE,
                      double* E_BE_OMG3);
void rxchf_fp_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
                    const double* DBE, const double* DP, double* FP, double* SP,
                    double* E_P_OMG1, double* S_P_OMG1);
void rxchf_fbe_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
                     const double* DBE, const double* DP, double* FBE, double* SBE,
                     double* E_BE_OMG1, double* S_BE_OMG1);
/* Integral phase of xcneo_driver with the reference's file outputs:
 * class_nuc_rep_ -> ENUCRP.dat, elec_ovlap_ -> eovlap.ufm, nuc_ovlap_ ->
 * novlap.ufm, calc_gam_epcore_ -> GAM_ecr.ufm + GAM_pcr.ufm, calc_gam_ep_ ->
 * GAM_ep.ufm, gam1_omp_md_ -> GAM_1.ufm + GAM_1s.ufm, gam2_conv_
 * (gam2_CONV_OMP.f GAM2_CONV) -> GAM_2.ufm + GAM_2s.ufm, gam3_conv_
 * (gam3_CONV_OMP.f GAM3_CONV) -> GAM_3.ufm.  The CONV routines' unsymmetrised
 * scratch files (GAM_2X.ufm, GAM_2sX.ufm, GAM_3X.ufm) are not written. */
void class_nuc_rep_(const int64_t* nat, const double* zan, const double* cat);
void elec_ovlap_(const int64_t* npebf, const int64_t* nebf, const int64_t* nebf2,
                 const int64_t* AMPEB2C, const double* AGEBFCC,
                 const double* ELCEX, const int64_t* ELCAM, const double* ELCBFC);
void nuc_ovlap_(const int64_t* npbf, const int64_t* npbf2, const double* AGNBFCC,
                const double* NUCEX, const int64_t* NUCAM, const double* NUCBFC);
void calc_gam_epcore_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                      const int64_t* nebf2, const int64_t* npbf2, const int64_t* nat,
                      const double* pmass, const double* zan, const double* cat,
                      const int64_t* AMPEB2C, const double* AGEBFCC,
                      const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                      const int64_t* ELCAM, const int64_t* NUCAM,
                      const double* ELCBFC, const double* NUCBFC);
void calc_gam_ep_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                  const int64_t* ng1, const int64_t* AMPEB2C, const double* AGEBFCC,
                  const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                  const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                  const double* NUCBFC);
void gam1_omp_md_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                  const int64_t* ng1, const int64_t* ng1prm, const int64_t* nat,
                  const int64_t* ngtg1, const double* pmass, const double* cat,
                  const double* zan, const double* bcoef1, const double* gamma1,
                  const int64_t* AMPEB2C, const double* AGEBFCC,
                  const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                  const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                  const double* NUCBFC);
void rxchf_gam1_omp_md_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                        const int64_t* ng1, const int64_t* ng1prm, const int64_t* nat,
                        const int64_t* ngtg1, const double* pmass, const double* cat,
                        const double* zan, const double* bcoef1, const double* gamma1,
                        const int64_t* AMPEB2C, const double* AGEBFCC,
                        const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                        const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                        const double* NUCBFC);
void gam2_conv_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npebf,
                const int64_t* npbf, const int64_t* ng2, const int64_t* ng2prm,
                const int64_t* nat, const int64_t* ngtg1, const double* pmass,
                const double* cat, const double* zan, const double* bcoef1,
                const double* gamma1, const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC, const double* AGNBFCC,
                const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC);
void gam3_conv_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npebf,
                const int64_t* npbf, const int64_t* ng3, const int64_t* ng3prm,
                const int64_t* nat, const int64_t* ngtg1, const double* pmass,
                const double* cat, const double* zan, const double* bcoef1,
                const double* gamma1, const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC, const double* AGNBFCC,
                const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC);
/* xchf1_fock.f disk contractions: E_from_GAM_2 (:1152-1281, GAM_2.ufm; focke,
 * fockp accumulate, E_gam2 overwritten), S_from_GAM_2s (:1283-1388, GAM_2s.ufm; se2,
 * sp2, S_gam2 overwritten), E_from_GAM_3 (:1390-1550, GAM_3.ufm),
 * E_from_GAM_4 (:1552-1710, GAM_4.ufm, values / 16). */
void e_from_gam_2_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam2);
void s_from_gam_2s_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
                    const double* DE, const double* DP, double* se2, double* sp2,
                    double* S_gam2);
void e_from_gam_3_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng3,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam3);
void e_from_gam_4_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng4,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam4);
/* xchf1_fock.f:2-361 with the reference's argument list; the LOGICAL*8
 * switches are read by their low bit (ifort .TRUE. = -1, gfortran 1).  The
 * disk branches read GAM_1.ufm, GAM_1s.ufm (always, as the reference does
 * outside NEO-HF), GAM_2.ufm, GAM_2s.ufm, GAM_3.ufm, GAM_4.ufm, and the
 * direct gam_4 reads GAM_2s.ufm. */
void xchf1_fock_(const int64_t* LNEOHF, const int64_t* LGAM4, const int64_t* LG4DSCF,
                 const int64_t* LG4IC, const int64_t* LG3DSCF, const int64_t* LG3IC1,
                 const int64_t* LG2DSCF, const int64_t* LG2IC1, const int64_t* LCMF,
                 const int64_t* NG4CHK, const int64_t* NG3CHK, const int64_t* NG2CHK,
                 const int64_t* SZG4IC, const int64_t* SZG3IC1, const int64_t* SZG2ICR,
                 const int64_t* npebf, const int64_t* nebf, const int64_t* nebf2,
                 const int64_t* npbf, const int64_t* npbf2, const int64_t* nelec,
                 const int64_t* ngee, const int64_t* ng1, const int64_t* ng2,
                 const int64_t* ng3, const int64_t* ng4, const double* DE,
                 const double* DP, const double* GAM_ecore, const double* GAM_pcore,
                 const double* GAM_ep, const double* GAM_ee, const double* GM4ICR,
                 const double* GM3IC1, const double* GM2ICR, const double* GM2SICR,
                 const int64_t* ng2prm, const int64_t* ngtg1, const int64_t* ng3prm,
                 const int64_t* nat, const double* pmass, const double* cat,
                 const double* zan, const double* bcoef1, const double* gamma1,
                 const int64_t* KPESTR, const int64_t* KPEEND, const int64_t* AMPEB2C,
                 const double* AGEBFCC, const double* AGNBFCC, const double* ELCEX,
                 const double* NUCEX, const int64_t* ELCAM, const int64_t* NUCAM,
                 const double* ELCBFC, const double* NUCBFC, double* focke,
                 double* fockp, double* Xfocke, double* Xfockp, double* E_total,
                 const double* E_nuc, double* E_ecore, double* E_pcore, double* E_ep,
                 double* E_ee, double* E_gam1, double* E_gam2, double* E_gam3,
                 double* E_gam4, double* S_total, double* S_gam1, double* S_gam2);
/* RXCHFne_FOCK / RXCUHFne_FOCK with the reference's argument lists;
 * GAM_1.ufm and GAM_1s.ufm are read from the working directory as
 * RXCHF_FP_OMG1 does, LOGICAL*8 switches by their low bit; LCMF's printed
 * checks are not reproduced. */
void rxchfne_fock_(const int64_t* LCMF, const int64_t* LNEOHF, const int64_t* nelec,
                   const int64_t* NAE, const int64_t* NBE, const int64_t* nebf,
                   const int64_t* nebf2, const int64_t* npbf, const int64_t* npbf2,
                   const int64_t* ngee, const int64_t* ng1, const int64_t* ng2,
                   const int64_t* ng3, const int64_t* ng4, const int64_t* SZG2ICR,
                   const int64_t* NG2CHK, const double* DAE, const double* DBE,
                   const double* DP, const double* GAM_ecore, const double* GAM_pcore,
                   const double* GAM_ep, const double* GAM_ee, const double* GM2ICR,
                   double* FP, double* FAE, double* FBE, double* E_ecore,
                   double* E_GAMee, double* E_OMG1, double* E_OMG2, double* E_total,
                   double* S_total);
void rxcuhfne_fock_(const int64_t* LCMF, const int64_t* LNEOHF, const int64_t* LADDEXCH,
                    const int64_t* nelec, const int64_t* NBE, const int64_t* NAalpE,
                    const int64_t* NAbetE, const int64_t* nebf, const int64_t* nebf2,
                    const int64_t* npbf, const int64_t* npbf2, const int64_t* ngee,
                    const int64_t* ng1, const int64_t* ng2, const int64_t* ng3,
                    const int64_t* ng4, const int64_t* SZG2ICR, const int64_t* NG2CHK,
                    const double* DAalpE, const double* DAbetE, const double* DBE,
                    const double* DP, const double* GAM_ecore, const double* GAM_pcore,
                    const double* GAM_ep, const double* GAM_ee, const double* GM2ICR,
                    const double* GM2exICR, double* FP, double* FAalpE, double* FAbetE,
                    double* FBE, double* E_ecore, double* E_GAMee, double* E_OMG1,
                    double* E_OMG2, double* E_total, double* S_total);
#ifdef __cplusplus
}
#endif
#endif /* NEOXC_H */
