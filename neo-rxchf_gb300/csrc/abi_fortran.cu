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

// Record length, in bytes, of the reference's direct-access integral files
// (GAM_IO.f: OPEN(...,ACCESS='direct',RECL=8)).  gfortran counts RECL in
// bytes; ifort without -assume byterecl counts 4-byte units (32 bytes).
long ufm_recl() {
  const char* e = std::getenv("NEOXC_UFM_RECL");
  long v = e ? std::atol(e) : 8;
  return v >= 8 ? v : 8;
}

// Read records 1..n (one FP64 each, at the start of every record).
bool read_ufm(const char* name, long long n, std::vector<double>& out) {
  out.assign((size_t)n, 0.0);
  std::FILE* f = std::fopen(name, "rb");
  if (!f) return false;
  const long recl = ufm_recl();
  std::vector<unsigned char> buf((size_t)recl);
  bool ok = true;
  for (long long i = 0; i < n && ok; i++) {
    if (std::fread(buf.data(), 1, (size_t)recl, f) != (size_t)recl) ok = false;
    else std::memcpy(&out[(size_t)i], buf.data(), sizeof(double));
  }
  std::fclose(f);
  return ok;
}

bool write_ufm(const char* name, const double* v, long long n) {
  std::FILE* f = std::fopen(name, "wb");
  if (!f) return false;
  const long recl = ufm_recl();
  std::vector<unsigned char> buf((size_t)recl, 0);
  bool ok = true;
  for (long long i = 0; i < n && ok; i++) {
    std::memcpy(buf.data(), &v[i], sizeof(double));
    ok = std::fwrite(buf.data(), 1, (size_t)recl, f) == (size_t)recl;
  }
  std::fclose(f);
  return ok;
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

}  // extern "C"
