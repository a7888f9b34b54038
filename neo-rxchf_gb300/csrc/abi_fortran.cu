// abi_fortran.cu -- by-reference shims with the reference's external
// subroutine signatures, so an unmodified Fortran SCF driver can link this
// library in place of the reference's object files.
//
// INTEGER arguments are INTEGER*8 (the reference builds with
// -integer-size 64); every argument is passed by address.  Failures are
// printed to stderr and kept for neoxc_last_error(); the subroutines never
// abort the caller.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/neoxc.h"

namespace {

void report(const char* who, int rc) {
  if (rc != NEOXC_OK)
    std::fprintf(stderr, "neoxc: %s failed (%d): %s\n", who, rc,
                 neoxc_last_error());
}

// Direct-access integral files (GAM_IO.f: OPEN(...,ACCESS='direct',
// RECL=8)): record length from NEOXC_UFM_RECL (bytes, default 8).
bool read_ufm(const char* name, long long n, std::vector<double>& out) {
  out.assign((size_t)n, 0.0);
  return neoxc_ufm_read(name, n, 0, out.data()) == NEOXC_OK;
}

bool write_ufm(const char* name, const double* v, long long n) {
  return neoxc_ufm_write(name, v, n, 0) == NEOXC_OK;
}

// File names of the reference's MO units (GAM_IO.f:450-500); other units
// get ifort's default name fort.<unit>.
std::string mo_unit_file(int64_t unit) {
  switch (unit) {
    case 850: return "guessCE.inp";
    case 851: return "guessCP.inp";
    case 852: return "FinalCE.dat";
    case 853: return "FinalCP.dat";
    case 860: return "FinalCAE.dat";
    case 861: return "FinalCBE.dat";
    case 870: return "FinalCAalpE.dat";
    case 871: return "FinalCAbetE.dat";
    default: return "fort." + std::to_string((long long)unit);
  }
}

// read_elec_density / read_nuc_density: MOs from a guess file, then
// D = prefac * sum_{k=kstart..klast} C(:,k) C(:,k)^T.
void read_density(const char* who, const char* file, int64_t nbf, int64_t kstart,
                  int64_t klast, double prefac, double* D) {
  std::vector<double> C((size_t)(nbf * nbf));
  int rc = neoxc_mo_read(file, nbf, nbf, C.data());
  if (rc == NEOXC_OK) rc = neoxc_mo_density(nbf, kstart, klast, prefac, C.data(), D);
  report(who, rc);
}

// read_GAM_ecore-style readers: records 1..n in packed order.
void read_packed(const char* who, const char* file, int64_t n, double* out) {
  report(who, neoxc_ufm_read(file, n, 0, out));
}

// read_nuc_ovlap / read_elec_ovlap: GS(i,j) = record pack_2D(n,j,i), the
// transpose of the file's column-major order.
void read_ovlap(const char* who, const char* file, int64_t n, double* GS) {
  std::vector<double> r((size_t)(n * n));
  const int rc = neoxc_ufm_read(file, n * n, 0, r.data());
  report(who, rc);
  if (rc != NEOXC_OK) return;
  for (int64_t i = 0; i < n; i++)
    for (int64_t j = 0; j < n; j++) GS[i + n * j] = r[(size_t)(j + n * i)];
}

}  // namespace

extern "C" {

// gam4_DSCF_OMP.f:2-3 GAM4_DSCF(NG4CHK,ne,np,ngee,ng2,ng4,DE,DP,focke,
// fockp,E_gam4); GAM_ee.ufm / GAM_2s.ufm read as in :46-47.
// NEOXC_GAM4_FACTORED=1 selects the factorised Fock build (same results for
// the pair-symmetric tables the reference writes, O(ne^4 np^2 + ne^5)).
void gam4_dscf_(const int64_t* NG4CHK, const int64_t* ne, const int64_t* np,
                const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
                const double* DE, const double* DP, double* focke,
                double* fockp, double* E_gam4) {
  std::vector<double> gee, g2s;
  if (!read_ufm("GAM_ee.ufm", *ngee, gee) || !read_ufm("GAM_2s.ufm", *ng2, g2s)) {
    std::fprintf(stderr, "neoxc: gam4_dscf: cannot read GAM_ee.ufm/GAM_2s.ufm\n");
    return;
  }
  const char* fac = std::getenv("NEOXC_GAM4_FACTORED");
  if (fac && std::strcmp(fac, "1") == 0) {
    report("gam4_dscf (factorised)",
           neoxc_gam4_fock_factored(*ne, *np, *ngee, *ng2, gee.data(),
                                    g2s.data(), DE, DP, focke, fockp, E_gam4));
    return;
  }
  report("gam4_dscf", neoxc_gam4_dscf(*NG4CHK, *ne, *np, *ngee, *ng2, *ng4,
                                      gee.data(), g2s.data(), DE, DP, focke,
                                      fockp, E_gam4));
}

// gam4_ICR_OMP.f:2-3 GAM4_ICR(Nchunks,ne,np,ngee,ng2,ng4,GAM_2s,GAM_4);
// GAM_ee.ufm read as in :32.
void gam4_icr_(const int64_t* Nchunks, const int64_t* ne, const int64_t* np,
               const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
               const double* GAM_2s, double* GAM_4) {
  std::vector<double> gee;
  if (!read_ufm("GAM_ee.ufm", *ngee, gee)) {
    std::fprintf(stderr, "neoxc: gam4_icr: cannot read GAM_ee.ufm\n");
    return;
  }
  report("gam4_icr", neoxc_gam4_icr(*Nchunks, *ne, *np, *ngee, *ng2, *ng4,
                                    GAM_2s, gee.data(), GAM_4));
}

void eg4icr_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng4, const double* DE, const double* DP,
             const double* GM4ICR, double* focke, double* fockp,
             double* E_gam4) {
  report("eg4icr", neoxc_eg4icr(*Nchunks, *nebf, *npbf, *ng4, DE, DP, GM4ICR,
                                focke, fockp, E_gam4));
}

void eg3ic1_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng3, const double* DE, const double* DP,
             const double* GM3ICR, double* focke, double* fockp,
             double* E_gam3) {
  report("eg3ic1", neoxc_eg3ic1(*Nchunks, *nebf, *npbf, *ng3, DE, DP, GM3ICR,
                                focke, fockp, E_gam3));
}

void eg2ic1_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
             const int64_t* ng2, const double* DE, const double* DP,
             const double* GM2ICR, const double* GM2SICR, double* FE,
             double* SE, double* FP, double* SP, double* E_gam2,
             double* S_gam2) {
  report("eg2ic1", neoxc_eg2ic1(*Nchunks, *nebf, *npbf, *ng2, DE, DP, GM2ICR,
                                GM2SICR, FE, SE, FP, SP, E_gam2, S_gam2));
}

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
               const double* NUCBFC, double* GM2ICR, double* GM2sICR) {
  report("gam2_ic1",
         neoxc_gam2_ic1(*Nchunks, *nebf, *npebf, *npbf, *ng2, *ng2prm, *nat,
                        *ngtg1, *pmass, cat, zan, bcoef1, gamma1, KPESTR,
                        KPEEND, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                        NUCAM, ELCBFC, NUCBFC, GM2ICR, GM2sICR));
}

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
               const double* NUCBFC, double* GM3ICR) {
  report("gam3_ic1",
         neoxc_gam3_ic1(*Nchunks, *nebf, *npebf, *npbf, *ng3, *ng3prm, *nat,
                        *ngtg1, *pmass, cat, zan, bcoef1, gamma1, KPESTR,
                        KPEEND, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                        NUCAM, ELCBFC, NUCBFC, GM3ICR));
}

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
                double* focke, double* fockp, double* E_gam3) {
  report("gam3_dscf",
         neoxc_gam3_dscf(*Nchunks, *nebf, *npebf, *npbf, *ng3, *ng3prm, *nat,
                         *ngtg1, *pmass, cat, zan, bcoef1, gamma1, KPESTR,
                         KPEEND, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX,
                         ELCAM, NUCAM, ELCBFC, NUCBFC, DE, DP, focke, fockp,
                         E_gam3));
}

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
                double* E_gam2, double* S_gam2) {
  report("gam2_dscf",
         neoxc_gam2_dscf(*Nchunks, *nebf, *npebf, *npbf, *ng2, *ng2prm, *nat,
                         *ngtg1, *pmass, cat, zan, bcoef1, gamma1, KPESTR,
                         KPEEND, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX,
                         ELCAM, NUCAM, ELCBFC, NUCBFC, DE, DP, focke, fockp,
                         se2, sp2, E_gam2, S_gam2));
}

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
                       double* GM2ICR, double* GM2exICR) {
  report("rxchfne_gam2_ic1",
         neoxc_rxchfne_gam2_ic1(*Nchunks, *nebf, *npebf, *npbf, *ng2, *ng2prm,
                                *nat, *ngtg1, *pmass, cat, zan, bcoef1, gamma1,
                                KPESTR, KPEEND, AMPEB2C, AGEBFCC, AGNBFCC,
                                ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                                GM2ICR, GM2exICR));
}

void rxchfne_fae_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                       const int64_t* npbf, const int64_t* ng2,
                       const double* DAE, const double* DBE, const double* DP,
                       const double* GM2ICR, double* FAE, double* E_AE_OMG2) {
  report("rxchfne_fae_omg2",
         neoxc_rxchfne_fae_omg2(*Nchunks, *nebf, *npbf, *ng2, DAE, DBE, DP,
                                GM2ICR, FAE, E_AE_OMG2));
}

void rxchfne_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                      const int64_t* npbf, const int64_t* ng2,
                      const int64_t* NAE, const int64_t* NBE,
                      const double* DAE, const double* DBE, const double* DP,
                      const double* GM2ICR, double* FP, double* E_P_OMG2) {
  report("rxchfne_fp_omg2",
         neoxc_rxchfne_fp_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAE, *NBE, DAE,
                               DBE, DP, GM2ICR, FP, E_P_OMG2));
}

void rxchfne_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf,
                       const int64_t* npbf, const int64_t* ng2,
                       const int64_t* NAE, const int64_t* NBE,
                       const double* DAE, const double* DBE, const double* DP,
                       const double* GM2ICR, double* FBE, double* E_BE_OMG2) {
  report("rxchfne_fbe_omg2",
         neoxc_rxchfne_fbe_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAE, *NBE, DAE,
                                DBE, DP, GM2ICR, FBE, E_BE_OMG2));
}

// gam_ee.f:2-169 calc_GAM_ee: computes GAM_ee and writes GAM_ee.ufm
// (records in pack_4D order, gam_ee.f:143-155).
void calc_gam_ee_(const int64_t* nebf, const int64_t* npebf,
                  const int64_t* ngee, const int64_t* AMPEB2C,
                  const double* AGEBFCC, const double* ELCEX,
                  const int64_t* ELCAM, const double* ELCBFC) {
  std::vector<double> gee((size_t)*ngee);
  int rc = neoxc_calc_gam_ee(*nebf, *npebf, *ngee, AMPEB2C, AGEBFCC, ELCEX,
                             ELCAM, ELCBFC, gee.data());
  report("calc_gam_ee", rc);
  if (rc == NEOXC_OK && !write_ufm("GAM_ee.ufm", gee.data(), *ngee))
    std::fprintf(stderr, "neoxc: calc_gam_ee: cannot write GAM_ee.ufm\n");
}

// ---- GAM_IO.f: integral files and MO files -------------------------------

// GAM_IO.f:28-67 read_GAM_ee (GAM_ee.ufm, pack_4D order = record order)
void read_gam_ee_(const int64_t* ne, const int64_t* ngee, double* GAM_ee) {
  (void)ne;
  read_packed("read_GAM_ee", "GAM_ee.ufm", *ngee, GAM_ee);
}
// GAM_IO.f:69-108 read_GAM_ep (GAM_ep.ufm)
void read_gam_ep_(const int64_t* ne, const int64_t* np, const int64_t* ng1,
                  double* GAM_ep) {
  (void)ne; (void)np;
  read_packed("read_GAM_ep", "GAM_ep.ufm", *ng1, GAM_ep);
}
// GAM_IO.f:110-142 read_GAM_ecore (GAM_ecr.ufm)
void read_gam_ecore_(const int64_t* ne, const int64_t* ne2, double* GAM_ecore) {
  (void)ne;
  read_packed("read_GAM_ecore", "GAM_ecr.ufm", *ne2, GAM_ecore);
}
// GAM_IO.f:144-176 read_GAM_pcore (GAM_pcr.ufm)
void read_gam_pcore_(const int64_t* np, const int64_t* np2, double* GAM_pcore) {
  (void)np;
  read_packed("read_GAM_pcore", "GAM_pcr.ufm", *np2, GAM_pcore);
}
// GAM_IO.f:178-211 read_nuc_ovlap (novlap.ufm)
void read_nuc_ovlap_(const int64_t* np, double* GS) {
  read_ovlap("read_nuc_ovlap", "novlap.ufm", *np, GS);
}
// GAM_IO.f:213-245 read_elec_ovlap (eovlap.ufm)
void read_elec_ovlap_(const int64_t* ne, double* GS) {
  read_ovlap("read_elec_ovlap", "eovlap.ufm", *ne, GS);
}
// GAM_IO.f:247-347 read_elec_density: guessCE.inp; nocc = n/2 doubly
// occupied orbitals (prefac 2), or orbital 1 (prefac 1) for one particle.
void read_elec_density_(const int64_t* nebf, const int64_t* n_particle, double* DE) {
  const bool many = *n_particle > 1;
  read_density("read_elec_density", "guessCE.inp", *nebf, 1,
               many ? *n_particle / 2 : 1, many ? 2.0 : 1.0, DE);
}
// GAM_IO.f:349-448 read_nuc_density: guessCP.inp; orbital NUCST, prefac 1.
void read_nuc_density_(const int64_t* npbf, const int64_t* n_particle,
                       const int64_t* NUCST, double* DP) {
  (void)n_particle;
  read_density("read_nuc_density", "guessCP.inp", *npbf, *NUCST, *NUCST, 1.0, DP);
}
// GAM_IO.f:450-468 write_MOs -> PUSQLF :471-518 (unit -> file name map)
void write_mos_(const int64_t* IFIL, const int64_t* nbf, const double* VEC) {
  report("write_MOs", neoxc_mo_write(mo_unit_file(*IFIL).c_str(), *nbf, *nbf, VEC));
}

// ---- xcuhf/xcuhf_omg{1..4}.f ---------------------------------------------

// xcuhf_omg1.f:2-81 FAE_OMG1 (GAM_1.ufm, GAM_1s.ufm read as in :20-23)
void fae_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
               const double* DAE, const double* DP, double* FAE, double* SAE1,
               double* E_AE_OMG1, double* S_AE_OMG1) {
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: fae_omg1: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  report("fae_omg1", neoxc_fae_omg1(*nebf, *npbf, *ng1, DAE, DP, g1.data(), g1s.data(),
                                    FAE, SAE1, E_AE_OMG1, S_AE_OMG1));
}
// xcuhf_omg1.f:83-163 UFP_OMG1
void ufp_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
               const double* DETOT, const double* DP, double* FP, double* SP1,
               double* E_P_OMG1, double* S_P_OMG1) {
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: ufp_omg1: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  report("ufp_omg1", neoxc_ufp_omg1(*nebf, *npbf, *ng1, DETOT, DP, g1.data(), g1s.data(),
                                    FP, SP1, E_P_OMG1, S_P_OMG1));
}
// xcuhf_omg2.f:2-4 FAE_OMG2
void fae_omg2_(const int64_t* Nchunks, const int64_t* NAE, const int64_t* NBE,
               const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
               const double* DAE, const double* DBE, const double* DETOT,
               const double* DP, const double* GM2ICR, const double* GM2SICR,
               double* FAE, double* SAE2, double* E_AE_OMG2, double* S_AE_OMG2) {
  report("fae_omg2", neoxc_fae_omg2(*Nchunks, *NAE, *NBE, *nebf, *npbf, *ng2, DAE, DBE,
                                    DETOT, DP, GM2ICR, GM2SICR, FAE, SAE2, E_AE_OMG2,
                                    S_AE_OMG2));
}
// xcuhf_omg2.f:302-304 UFP_OMG2
void ufp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng2, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DETOT,
               const double* DP, const double* GM2ICR, const double* GM2SICR,
               double* FP, double* SP2, double* E_P_OMG2, double* S_P_OMG2) {
  report("ufp_omg2", neoxc_ufp_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAE, *NBE, DAE, DBE,
                                    DETOT, DP, GM2ICR, GM2SICR, FP, SP2, E_P_OMG2,
                                    S_P_OMG2));
}
// xcuhf_omg3.f:2-3 FAE_OMG3
void fae_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng3, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM3ICR, double* FAE, double* E_AE_OMG3) {
  report("fae_omg3", neoxc_fae_omg3(*Nchunks, *nebf, *npbf, *ng3, *NAE, *NBE, DAE, DBE,
                                    DP, GM3ICR, FAE, E_AE_OMG3));
}
// xcuhf_omg3.f:284-285 UFP_OMG3
void ufp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng3, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM3ICR, double* FP, double* E_P_OMG3) {
  report("ufp_omg3", neoxc_ufp_omg3(*Nchunks, *nebf, *npbf, *ng3, *NAE, *NBE, DAE, DBE,
                                    DP, GM3ICR, FP, E_P_OMG3));
}
// xcuhf_omg4.f:2-3 FAE_OMG4
void fae_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng4, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM4ICR, double* FAE, double* E_AE_OMG4) {
  report("fae_omg4", neoxc_fae_omg4(*Nchunks, *nebf, *npbf, *ng4, *NAE, *NBE, DAE, DBE,
                                    DP, GM4ICR, FAE, E_AE_OMG4));
}
// xcuhf_omg4.f:512-513 UFP_OMG4
void ufp_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf,
               const int64_t* ng4, const int64_t* NAE, const int64_t* NBE,
               const double* DAE, const double* DBE, const double* DP,
               const double* GM4ICR, double* FP, double* E_P_OMG4) {
  report("ufp_omg4", neoxc_ufp_omg4(*Nchunks, *nebf, *npbf, *ng4, *NAE, *NBE, DAE, DBE,
                                    DP, GM4ICR, FP, E_P_OMG4));
}
// xcuhf_omg4.f:1080-1081 OMG4_ICR (GAM_ee.ufm read as in read_GAM_ee)
void omg4_icr_(const int64_t* Nchunks, const int64_t* ne, const int64_t* np,
               const int64_t* ngee, const int64_t* ng2, const int64_t* ng4,
               const double* GAM_2s, double* GAM_4) {
  std::vector<double> gee;
  if (!read_ufm("GAM_ee.ufm", *ngee, gee)) {
    std::fprintf(stderr, "neoxc: omg4_icr: cannot read GAM_ee.ufm\n");
    return;
  }
  report("omg4_icr", neoxc_omg4_icr(*Nchunks, *ne, *np, *ngee, *ng2, *ng4, GAM_2s,
                                    gee.data(), GAM_4));
}

// ---- rxchf/rxchf_omg{1..4}.f, rxcuhf_omg{2,3}.f, rxchfne/rxcuhfne_omg2.f -----
// Same names and argument lists as the reference subroutines.
void rxcuhfne_fe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const double* DAalpE, const double* DAbetE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2ICR, const double* GM2exICR, double* FAalpE, double* FAbetE, double* E_AE_OMG2) {
  report("rxcuhfne_fe_omg2", neoxc_rxcuhfne_fe_omg2(*Nchunks, *nebf, *npbf, *ng2, DAalpE, DAbetE, DAtotE, DBE, DP, GM2ICR, GM2exICR, FAalpE, FAbetE, E_AE_OMG2));
}
void rxcuhfne_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE, const double* DAalpE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2ICR, const double* GM2exICR, double* FP, double* E_P_OMG2) {
  report("rxcuhfne_fp_omg2", neoxc_rxcuhfne_fp_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAalpE, *NBE, DAalpE, DAtotE, DBE, DP, GM2ICR, GM2exICR, FP, E_P_OMG2));
}
void rxcuhfne_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE, const double* DAalpE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2ICR, const double* GM2exICR, double* FBE, double* E_BE_OMG2) {
  report("rxcuhfne_fbe_omg2", neoxc_rxcuhfne_fbe_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAalpE, *NBE, DAalpE, DAtotE, DBE, DP, GM2ICR, GM2exICR, FBE, E_BE_OMG2));
}
void rxchf_fae_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const double* DAE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FAE, double* SAE, double* E_AE_OMG2, double* S_AE_OMG2) {
  report("rxchf_fae_omg2", neoxc_rxchf_fae_omg2(*Nchunks, *nebf, *npbf, *ng2, DAE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FAE, SAE, E_AE_OMG2, S_AE_OMG2));
}
void rxchf_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const double* DAE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2, double* S_P_OMG2) {
  report("rxchf_fp_omg2", neoxc_rxchf_fp_omg2(*Nchunks, *nebf, *npbf, *ng2, DAE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FP, SP, E_P_OMG2, S_P_OMG2));
}
void rxchf_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const double* DAE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FBE, double* SBE, double* E_BE_OMG2, double* S_BE_OMG2) {
  report("rxchf_fbe_omg2", neoxc_rxchf_fbe_omg2(*Nchunks, *nebf, *npbf, *ng2, DAE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FBE, SBE, E_BE_OMG2, S_BE_OMG2));
}
void rxchf_fae_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FAE, double* E_AE_OMG3) {
  report("rxchf_fae_omg3", neoxc_rxchf_fae_omg3(*Nchunks, *nebf, *npbf, *ng3, DAE, DBE, DP, GM3_1ICR, GM3_2ICR, FAE, E_AE_OMG3));
}
void rxchf_fp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FP, double* E_P_OMG3) {
  report("rxchf_fp_omg3", neoxc_rxchf_fp_omg3(*Nchunks, *nebf, *npbf, *ng3, DAE, DBE, DP, GM3_1ICR, GM3_2ICR, FP, E_P_OMG3));
}
void rxchf_fbe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FBE, double* E_BE_OMG3) {
  report("rxchf_fbe_omg3", neoxc_rxchf_fbe_omg3(*Nchunks, *nebf, *npbf, *ng3, DAE, DBE, DP, GM3_1ICR, GM3_2ICR, FBE, E_BE_OMG3));
}
void rxchf_fae_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng4, const double* DAE, const double* DBE, const double* DP, const double* GM4ICR, double* FAE, double* E_AE_OMG4) {
  report("rxchf_fae_omg4", neoxc_rxchf_fae_omg4(*Nchunks, *nebf, *npbf, *ng4, DAE, DBE, DP, GM4ICR, FAE, E_AE_OMG4));
}
void rxchf_fp_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng4, const double* DAE, const double* DBE, const double* DP, const double* GM4ICR, double* FP, double* E_P_OMG4) {
  report("rxchf_fp_omg4", neoxc_rxchf_fp_omg4(*Nchunks, *nebf, *npbf, *ng4, DAE, DBE, DP, GM4ICR, FP, E_P_OMG4));
}
void rxchf_fbe_omg4_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng4, const double* DAE, const double* DBE, const double* DP, const double* GM4ICR, double* FBE, double* E_BE_OMG4) {
  report("rxchf_fbe_omg4", neoxc_rxchf_fbe_omg4(*Nchunks, *nebf, *npbf, *ng4, DAE, DBE, DP, GM4ICR, FBE, E_BE_OMG4));
}
void rxcuhf_fe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const double* DAalpE, const double* DAbetE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FAalpE, double* FAbetE, double* SAalpE, double* E_AE_OMG2, double* S_AE_OMG2) {
  report("rxcuhf_fe_omg2", neoxc_rxcuhf_fe_omg2(*Nchunks, *nebf, *npbf, *ng2, DAalpE, DAbetE, DAtotE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FAalpE, FAbetE, SAalpE, E_AE_OMG2, S_AE_OMG2));
}
void rxcuhf_fp_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE, const double* DAalpE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FP, double* SP, double* E_P_OMG2, double* S_P_OMG2) {
  report("rxcuhf_fp_omg2", neoxc_rxcuhf_fp_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAalpE, *NBE, DAalpE, DAtotE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FP, SP, E_P_OMG2, S_P_OMG2));
}
void rxcuhf_fbe_omg2_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng2, const int64_t* NAalpE, const int64_t* NBE, const double* DAalpE, const double* DAtotE, const double* DBE, const double* DP, const double* GM2_1ICR, const double* GM2_2ICR, const double* GM2sICR, double* FBE, double* SBE, double* E_BE_OMG2, double* S_BE_OMG2) {
  report("rxcuhf_fbe_omg2", neoxc_rxcuhf_fbe_omg2(*Nchunks, *nebf, *npbf, *ng2, *NAalpE, *NBE, DAalpE, DAtotE, DBE, DP, GM2_1ICR, GM2_2ICR, GM2sICR, FBE, SBE, E_BE_OMG2, S_BE_OMG2));
}
void rxcuhf_fe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAalpE, const double* DAbetE, const double* DAtotE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FAalpE, double* FAbetE, double* E_AE_OMG3) {
  report("rxcuhf_fe_omg3", neoxc_rxcuhf_fe_omg3(*Nchunks, *nebf, *npbf, *ng3, DAalpE, DAbetE, DAtotE, DBE, DP, GM3_1ICR, GM3_2ICR, FAalpE, FAbetE, E_AE_OMG3));
}
void rxcuhf_fp_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAalpE, const double* DAbetE, const double* DAtotE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FP, double* E_P_OMG3) {
  report("rxcuhf_fp_omg3", neoxc_rxcuhf_fp_omg3(*Nchunks, *nebf, *npbf, *ng3, DAalpE, DAbetE, DAtotE, DBE, DP, GM3_1ICR, GM3_2ICR, FP, E_P_OMG3));
}
void rxcuhf_fbe_omg3_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npbf, const int64_t* ng3, const double* DAalpE, const double* DAbetE, const double* DAtotE, const double* DBE, const double* DP, const double* GM3_1ICR, const double* GM3_2ICR, double* FBE, double* E_BE_OMG3) {
  report("rxcuhf_fbe_omg3", neoxc_rxcuhf_fbe_omg3(*Nchunks, *nebf, *npbf, *ng3, DAalpE, DAbetE, DAtotE, DBE, DP, GM3_1ICR, GM3_2ICR, FBE, E_BE_OMG3));
}
// rxchf/rxchf_omg1.f:2-82 RXCHF_FP_OMG1, :84-165 RXCHF_FBE_OMG1 (GAM_1.ufm,
// GAM_1s.ufm read as in :20-23)
void rxchf_fp_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
                    const double* DBE, const double* DP, double* FP, double* SP,
                    double* E_P_OMG1, double* S_P_OMG1) {
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: rxchf_fp_omg1: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  report("rxchf_fp_omg1", neoxc_rxchf_fp_omg1(*nebf, *npbf, *ng1, DBE, DP, g1.data(),
                                              g1s.data(), FP, SP, E_P_OMG1, S_P_OMG1));
}
void rxchf_fbe_omg1_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng1,
                     const double* DBE, const double* DP, double* FBE, double* SBE,
                     double* E_BE_OMG1, double* S_BE_OMG1) {
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: rxchf_fbe_omg1: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  report("rxchf_fbe_omg1", neoxc_rxchf_fbe_omg1(*nebf, *npbf, *ng1, DBE, DP, g1.data(),
                                                g1s.data(), FBE, SBE, E_BE_OMG1, S_BE_OMG1));
}

}  // extern "C"
