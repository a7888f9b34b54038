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

// GAM_4.ufm holds gam_4 (gam_4_OMP.f:263-293); E_from_GAM_4 (xchf1_fock.f:1552-1710)
// divides each record by 16, which makes it the GM4ICR EG4ICR contracts.
bool read_gam4_over16(int64_t ng4, std::vector<double>& g) {
  if (!read_ufm("GAM_4.ufm", ng4, g)) return false;
  for (double& v : g) v = v / 16.0;
  return true;
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

// ---- integral phase of xcneo_driver (xcneo_HYBRID.f:661-690,761,874,964) ----
// class_nuc_rep.f:2-45 -> ENUCRP.dat (:39-41)
void class_nuc_rep_(const int64_t* nat, const double* zan, const double* cat) {
  double E = 0.0;
  int rc = neoxc_class_nuc_rep(*nat, zan, cat, &E);
  if (rc == NEOXC_OK) rc = neoxc_enuc_write("ENUCRP.dat", E);
  report("class_nuc_rep", rc);
}

// pure_ovlap.f:2-105 elec_ovlap -> eovlap.ufm (:86)
void elec_ovlap_(const int64_t* npebf, const int64_t* nebf, const int64_t* nebf2,
                 const int64_t* AMPEB2C, const double* AGEBFCC,
                 const double* ELCEX, const int64_t* ELCAM, const double* ELCBFC) {
  std::vector<double> S((size_t)*nebf2);
  int rc = *nebf2 == *nebf * *nebf ? NEOXC_OK : NEOXC_ERR_ARG;
  if (rc == NEOXC_OK)
    rc = neoxc_onebody_integrals(*nebf, *npebf, 1, 0, 0, 1.0, nullptr, nullptr, nullptr,
                                 nullptr, AMPEB2C, AGEBFCC, nullptr, ELCEX, nullptr,
                                 ELCAM, nullptr, ELCBFC, nullptr, S.data(), nullptr,
                                 nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc == NEOXC_OK && !write_ufm("eovlap.ufm", S.data(), *nebf2)) rc = NEOXC_ERR_IO;
  report("elec_ovlap", rc);
}

// pure_ovlap.f:107-203 nuc_ovlap -> novlap.ufm (:184)
void nuc_ovlap_(const int64_t* npbf, const int64_t* npbf2, const double* AGNBFCC,
                const double* NUCEX, const int64_t* NUCAM, const double* NUCBFC) {
  std::vector<double> S((size_t)*npbf2);
  int rc = *npbf2 == *npbf * *npbf ? NEOXC_OK : NEOXC_ERR_ARG;
  if (rc == NEOXC_OK)
    rc = neoxc_onebody_integrals(1, 1, *npbf, 0, 0, 1.0, nullptr, nullptr, nullptr,
                                 nullptr, nullptr, nullptr, AGNBFCC, nullptr, NUCEX,
                                 nullptr, NUCAM, nullptr, NUCBFC, nullptr, S.data(),
                                 nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc == NEOXC_OK && !write_ufm("novlap.ufm", S.data(), *npbf2)) rc = NEOXC_ERR_IO;
  report("nuc_ovlap", rc);
}

// gam_epcore.f:2-198 calc_GAM_epcore -> GAM_ecr.ufm (:161), GAM_pcr.ufm (:178)
void calc_gam_epcore_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                      const int64_t* nebf2, const int64_t* npbf2, const int64_t* nat,
                      const double* pmass, const double* zan, const double* cat,
                      const int64_t* AMPEB2C, const double* AGEBFCC,
                      const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                      const int64_t* ELCAM, const int64_t* NUCAM,
                      const double* ELCBFC, const double* NUCBFC) {
  std::vector<double> he((size_t)*nebf2), hp((size_t)*npbf2);
  int rc = (*nebf2 == *nebf * *nebf && *npbf2 == *npbf * *npbf) ? NEOXC_OK : NEOXC_ERR_ARG;
  if (rc == NEOXC_OK)
    rc = neoxc_onebody_integrals(*nebf, *npebf, *npbf, *nat, 0, *pmass, cat, zan,
                                 nullptr, nullptr, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX,
                                 NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, nullptr, nullptr,
                                 he.data(), hp.data(), nullptr, nullptr, nullptr);
  if (rc == NEOXC_OK && !(write_ufm("GAM_ecr.ufm", he.data(), *nebf2) &&
                          write_ufm("GAM_pcr.ufm", hp.data(), *npbf2)))
    rc = NEOXC_ERR_IO;
  report("calc_GAM_epcore", rc);
}

// gam_ep.f:2-165 calc_GAM_ep -> GAM_ep.ufm (:141)
void calc_gam_ep_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                  const int64_t* ng1, const int64_t* AMPEB2C, const double* AGEBFCC,
                  const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                  const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                  const double* NUCBFC) {
  std::vector<double> g((size_t)*ng1);
  int rc = *ng1 == *nebf * *nebf * *npbf * *npbf ? NEOXC_OK : NEOXC_ERR_ARG;
  if (rc == NEOXC_OK)
    rc = neoxc_onebody_integrals(*nebf, *npebf, *npbf, 0, 0, 1.0, nullptr, nullptr,
                                 nullptr, nullptr, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX,
                                 NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, nullptr, nullptr,
                                 nullptr, nullptr, g.data(), nullptr, nullptr);
  if (rc == NEOXC_OK && !write_ufm("GAM_ep.ufm", g.data(), *ng1)) rc = NEOXC_ERR_IO;
  report("calc_GAM_ep", rc);
}

// gam_1_OMP.f:2-396 GAM1_OMP_MD -> GAM_1.ufm, GAM_1s.ufm (:358-361)
void gam1_omp_md_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                  const int64_t* ng1, const int64_t* ng1prm, const int64_t* nat,
                  const int64_t* ngtg1, const double* pmass, const double* cat,
                  const double* zan, const double* bcoef1, const double* gamma1,
                  const int64_t* AMPEB2C, const double* AGEBFCC,
                  const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                  const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                  const double* NUCBFC) {
  std::vector<double> g((size_t)*ng1), gs((size_t)*ng1);
  int rc = (*ng1 == *nebf * *nebf * *npbf * *npbf &&
            *ng1prm == *npebf * *npebf * *npbf * *npbf) ? NEOXC_OK : NEOXC_ERR_ARG;
  if (rc == NEOXC_OK)
    rc = neoxc_onebody_integrals(*nebf, *npebf, *npbf, *nat, *ngtg1, *pmass, cat, zan,
                                 bcoef1, gamma1, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX,
                                 NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, nullptr, nullptr,
                                 nullptr, nullptr, nullptr, g.data(), gs.data());
  if (rc == NEOXC_OK && !(write_ufm("GAM_1.ufm", g.data(), *ng1) &&
                          write_ufm("GAM_1s.ufm", gs.data(), *ng1)))
    rc = NEOXC_ERR_IO;
  report("GAM1_OMP_MD", rc);
}

// rxchf/rxchf_gam_1_OMP.f:2-175 RXCHF_GAM1_OMP_MD -> GAM_1.ufm, GAM_1s.ufm
void rxchf_gam1_omp_md_(const int64_t* nebf, const int64_t* npebf, const int64_t* npbf,
                        const int64_t* ng1, const int64_t* ng1prm, const int64_t* nat,
                        const int64_t* ngtg1, const double* pmass, const double* cat,
                        const double* zan, const double* bcoef1, const double* gamma1,
                        const int64_t* AMPEB2C, const double* AGEBFCC,
                        const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                        const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                        const double* NUCBFC) {
  std::vector<double> g((size_t)*ng1), gs((size_t)*ng1);
  int rc = neoxc_rxchf_gam1(*nebf, *npebf, *npbf, *ng1, *ng1prm, *nat, *ngtg1, *pmass, cat,
                            zan, bcoef1, gamma1, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX,
                            ELCAM, NUCAM, ELCBFC, NUCBFC, g.data(), gs.data());
  if (rc == NEOXC_OK && !(write_ufm("GAM_1.ufm", g.data(), *ng1) &&
                          write_ufm("GAM_1s.ufm", gs.data(), *ng1)))
    rc = NEOXC_ERR_IO;
  report("RXCHF_GAM1_OMP_MD", rc);
}

// gam2_CONV_OMP.f GAM2_CONV: the symmetrised gam_2 / gam_2s into GAM_2.ufm,
// GAM_2s.ufm (the in-core GAM2_IC1 result, written by record)
void gam2_conv_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npebf,
                const int64_t* npbf, const int64_t* ng2, const int64_t* ng2prm,
                const int64_t* nat, const int64_t* ngtg1, const double* pmass,
                const double* cat, const double* zan, const double* bcoef1,
                const double* gamma1, const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC, const double* AGNBFCC,
                const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC) {
  std::vector<double> g((size_t)*ng2), gs((size_t)*ng2);
  int rc = neoxc_gam2_ic1(*Nchunks, *nebf, *npebf, *npbf, *ng2, *ng2prm, *nat, *ngtg1,
                          *pmass, cat, zan, bcoef1, gamma1, KPESTR, KPEEND, AMPEB2C,
                          AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                          g.data(), gs.data());
  if (rc == NEOXC_OK && !(write_ufm("GAM_2.ufm", g.data(), *ng2) &&
                          write_ufm("GAM_2s.ufm", gs.data(), *ng2)))
    rc = NEOXC_ERR_IO;
  report("GAM2_CONV", rc);
}

// gam3_CONV_OMP.f GAM3_CONV: the six-permutation symmetrised gam_3 into
// GAM_3.ufm (:180-253)
void gam3_conv_(const int64_t* Nchunks, const int64_t* nebf, const int64_t* npebf,
                const int64_t* npbf, const int64_t* ng3, const int64_t* ng3prm,
                const int64_t* nat, const int64_t* ngtg1, const double* pmass,
                const double* cat, const double* zan, const double* bcoef1,
                const double* gamma1, const int64_t* KPESTR, const int64_t* KPEEND,
                const int64_t* AMPEB2C, const double* AGEBFCC, const double* AGNBFCC,
                const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC) {
  std::vector<double> g((size_t)*ng3);
  int rc = neoxc_gam3_ic1(*Nchunks, *nebf, *npebf, *npbf, *ng3, *ng3prm, *nat, *ngtg1,
                          *pmass, cat, zan, bcoef1, gamma1, KPESTR, KPEEND, AMPEB2C,
                          AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                          g.data());
  if (rc == NEOXC_OK && !write_ufm("GAM_3.ufm", g.data(), *ng3)) rc = NEOXC_ERR_IO;
  report("GAM3_CONV", rc);
}

// ---- xchf1_fock.f disk contractions ---------------------------------------
// E_from_GAM_2 (xchf1_fock.f:1152-1281): focke, fockp accumulate, E_gam2 overwritten.
// The device contraction also forms the overlap terms; they are discarded.
void e_from_gam_2_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam2) {
  std::vector<double> g;
  if (!read_ufm("GAM_2.ufm", *ng2, g)) {
    std::fprintf(stderr, "neoxc: E_from_GAM_2: cannot read GAM_2.ufm\n");
    return;
  }
  std::vector<double> se((size_t)(*nebf * *nebf)), sp((size_t)(*npbf * *npbf));
  double S = 0.0;
  report("E_from_GAM_2", neoxc_eg2ic1(1, *nebf, *npbf, *ng2, DE, DP, g.data(), g.data(),
                                      focke, se.data(), fockp, sp.data(), E_gam2, &S));
}

// S_from_GAM_2s (xchf1_fock.f:1283-1388): se2, sp2, S_gam2 overwritten.
void s_from_gam_2s_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng2,
                    const double* DE, const double* DP, double* se2, double* sp2,
                    double* S_gam2) {
  std::vector<double> g;
  if (!read_ufm("GAM_2s.ufm", *ng2, g)) {
    std::fprintf(stderr, "neoxc: S_from_GAM_2s: cannot read GAM_2s.ufm\n");
    return;
  }
  std::vector<double> fe((size_t)(*nebf * *nebf), 0.0), fp((size_t)(*npbf * *npbf), 0.0);
  double E = 0.0;
  report("S_from_GAM_2s", neoxc_eg2ic1(1, *nebf, *npbf, *ng2, DE, DP, g.data(), g.data(),
                                       fe.data(), se2, fp.data(), sp2, &E, S_gam2));
}

// E_from_GAM_3 (xchf1_fock.f:1390-1550)
void e_from_gam_3_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng3,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam3) {
  std::vector<double> g;
  if (!read_ufm("GAM_3.ufm", *ng3, g)) {
    std::fprintf(stderr, "neoxc: E_from_GAM_3: cannot read GAM_3.ufm\n");
    return;
  }
  report("E_from_GAM_3", neoxc_eg3ic1(1, *nebf, *npbf, *ng3, DE, DP, g.data(), focke,
                                      fockp, E_gam3));
}

void e_from_gam_4_(const int64_t* nebf, const int64_t* npbf, const int64_t* ng4,
                   const double* DE, const double* DP, double* focke, double* fockp,
                   double* E_gam4) {
  std::vector<double> g;
  if (!read_gam4_over16(*ng4, g)) {
    std::fprintf(stderr, "neoxc: E_from_GAM_4: cannot read GAM_4.ufm\n");
    return;
  }
  report("E_from_GAM_4", neoxc_eg4icr(1, *nebf, *npbf, *ng4, DE, DP, g.data(), focke,
                                      fockp, E_gam4));
}

// xchf1_fock.f:2-361.  LOGICAL*8 arguments are tested by their low bit.
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
                 double* E_gam4, double* S_total, double* S_gam1, double* S_gam2) {
  (void)LCMF;
  (void)nebf2;
  (void)npbf2;
  auto on = [](const int64_t* l) { return (*l & 1) != 0; };
  int64_t modes = 0;
  if (on(LNEOHF)) modes |= NEOXC_FOCK_NEOHF;
  if (on(LGAM4)) modes |= NEOXC_FOCK_GAM4;
  if (on(LG4DSCF)) modes |= NEOXC_FOCK_G4DSCF;
  if (on(LG4IC)) modes |= NEOXC_FOCK_G4IC;
  if (on(LG3DSCF)) modes |= NEOXC_FOCK_G3DSCF;
  if (on(LG3IC1)) modes |= NEOXC_FOCK_G3IC1;
  if (on(LG2DSCF)) modes |= NEOXC_FOCK_G2DSCF;
  if (on(LG2IC1)) modes |= NEOXC_FOCK_G2IC1;
  const char* fac = std::getenv("NEOXC_GAM4_FACTORED");
  if (fac && std::strcmp(fac, "1") == 0) modes |= NEOXC_FOCK_GAM4_FACTORED;
  const bool neohf = (modes & NEOXC_FOCK_NEOHF) != 0;
  const bool t2 = !neohf && *nelec > 1, t3 = !neohf && *nelec > 2;
  const bool t4 = t3 && (modes & NEOXC_FOCK_GAM4);
  // the tables the reference reads from the working directory
  std::vector<double> g1, g1s, g2, g2s, g3, g4, g2s4;
  bool ok = true;
  if (!neohf) ok = read_ufm("GAM_1.ufm", *ng1, g1) && read_ufm("GAM_1s.ufm", *ng1, g1s);
  const double *p2 = GM2ICR, *p2s = GM2SICR, *p3 = GM3IC1, *p4 = GM4ICR, *p2s4 = nullptr;
  if (ok && t2 && !(modes & (NEOXC_FOCK_G2DSCF | NEOXC_FOCK_G2IC1))) {
    ok = read_ufm("GAM_2.ufm", *ng2, g2) && read_ufm("GAM_2s.ufm", *ng2, g2s);
    p2 = g2.data();
    p2s = g2s.data();
  }
  if (ok && t3 && !(modes & (NEOXC_FOCK_G3DSCF | NEOXC_FOCK_G3IC1))) {
    ok = read_ufm("GAM_3.ufm", *ng3, g3);
    p3 = g3.data();
  }
  if (ok && t4 && (modes & NEOXC_FOCK_G4DSCF)) {
    ok = read_ufm("GAM_2s.ufm", *ng2, g2s4);   // gam4_DSCF_OMP.f:46-47
    p2s4 = g2s4.data();
  } else if (ok && t4 && !(modes & NEOXC_FOCK_G4IC)) {
    ok = read_gam4_over16(*ng4, g4);
    p4 = g4.data();
  }
  if (!ok) {
    std::fprintf(stderr, "neoxc: xchf1_fock: cannot read an integral file\n");
    return;
  }
  (void)SZG4IC;
  (void)SZG3IC1;
  (void)SZG2ICR;
  report("xchf1_fock",
         neoxc_xchf1_fock(modes, *NG4CHK, *NG3CHK, *NG2CHK, *npebf, *nebf, *npbf, *nelec,
                          *ngee, *ng1, *ng2, *ng3, *ng4, DE, DP, GAM_ecore, GAM_pcore,
                          GAM_ep, GAM_ee, g1.empty() ? nullptr : g1.data(),
                          g1s.empty() ? nullptr : g1s.data(), p4, p3, p2, p2s, p2s4,
                          *ng2prm, *ngtg1, *ng3prm, *nat, *pmass, cat, zan, bcoef1,
                          gamma1, KPESTR, KPEEND, AMPEB2C, AGEBFCC, AGNBFCC, ELCEX,
                          NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, focke, fockp, Xfocke,
                          Xfockp, E_total, E_nuc, E_ecore, E_pcore, E_ep, E_ee, E_gam1,
                          E_gam2, E_gam3, E_gam4, S_total, S_gam1, S_gam2));
}

// rxchfne/rxchfne_fock.f:2-250 RXCHFne_FOCK
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
                   double* S_total) {
  (void)LCMF; (void)LNEOHF; (void)nelec; (void)NBE; (void)nebf2; (void)npbf2; (void)ngee;
  (void)ng2; (void)ng3; (void)ng4; (void)SZG2ICR; (void)NG2CHK; (void)GAM_pcore;
  (void)GAM_ep;
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: RXCHFne_FOCK: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  report("RXCHFne_FOCK",
         neoxc_rxchfne_fock(0, 0, *NAE, 0, 0, *nebf, *npbf, DAE, nullptr, DBE, DP, GAM_ecore,
                            GAM_ee, g1.data(), g1s.data(), GM2ICR, nullptr, FP, FAE, nullptr,
                            FBE, E_ecore, E_GAMee, E_OMG1, E_OMG2, E_total, S_total));
}

// rxchfne/rxcuhfne_fock.f RXCUHFne_FOCK
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
                    double* E_OMG2, double* E_total, double* S_total) {
  (void)LCMF; (void)LNEOHF; (void)nelec; (void)NBE; (void)nebf2; (void)npbf2; (void)ngee;
  (void)ng2; (void)ng3; (void)ng4; (void)SZG2ICR; (void)NG2CHK; (void)GAM_pcore;
  (void)GAM_ep;
  std::vector<double> g1, g1s;
  if (!read_ufm("GAM_1.ufm", *ng1, g1) || !read_ufm("GAM_1s.ufm", *ng1, g1s)) {
    std::fprintf(stderr, "neoxc: RXCUHFne_FOCK: cannot read GAM_1.ufm/GAM_1s.ufm\n");
    return;
  }
  const int64_t exch = (*LADDEXCH & 1) ? 1 : 0;
  report("RXCUHFne_FOCK",
         neoxc_rxchfne_fock(1, exch, 0, *NAalpE, *NAbetE, *nebf, *npbf, DAalpE, DAbetE, DBE,
                            DP, GAM_ecore, GAM_ee, g1.data(), g1s.data(), GM2ICR,
                            exch ? GM2exICR : nullptr, FP, FAalpE, FAbetE, FBE, E_ecore,
                            E_GAMee, E_OMG1, E_OMG2, E_total, S_total));
}

}  // extern "C"
