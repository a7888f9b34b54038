// neoxc_internal.h -- internal launch interface of the GB300 engine.
//
// Every launcher takes DEVICE pointers, enqueues on the given stream and
// returns a cudaError_t from the launch; none of them synchronises.
// Index conventions follow the reference's packed arrays (pack_GAM.f):
// a 0-based offset equals the Fortran packed index minus one.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace neoxc {

// ---- device copy of the basis (driver arrays of xcneo_HYBRID.f) --------
struct DevPrim {      // one primitive Cartesian Gaussian
  double a;           // exponent
  double c[3];        // centre (bohr)
  double coef;        // contraction coefficient (AGEBFCC / AGNBFCC)
  int l[3];           // (l,m,n)
  int pad;
};

struct DevSystem {
  int nebf, npebf, npbf, nat, ngtg;
  double pmass;
  const DevPrim* eprim;     // [npebf]
  const DevPrim* pprim;     // [npbf]
  const int* kpestr;        // [nebf] 0-based first primitive
  const int* kpeend;        // [nebf] 0-based last primitive (inclusive)
  const double* zan;        // [nat]
  const double* cat;        // [3*nat]
  const double* bgem;       // [ngtg]
  const double* ggem;       // [ngtg]
  int lmax_e, lmax_p;       // largest total l of an electronic / nuclear primitive
  // gam_3 pair tables (k_gam3.cu), built by stage_system: g3i holds
  // ket_ab[2 nket] (primitive pairs of the canonical contracted pairs, in
  // canonical order), kofs[nPe+1], tile_k[ntile+1], tile_P[ntile+1],
  // kperm[nket] (kets of each tile ordered by angular class); g3rec the
  // FP64 pair records of the kets and of the canonical nuclear pairs.
  int g3_nket, g3_ntile;
  const int* g3i;
  const double* g3rec;
};

// Largest per-Cartesian angular momentum supported by the MD kernels.
constexpr int kMaxL = 2;
constexpr int kMaxNG = 8;     // geminal terms
constexpr int kMaxNat = 64;   // classical nuclei

// Record an error message for neoxc_last_error(); returns `code`.
int set_last_error(int code, const char* fmt, ...);

// Deterministic reduction of per-CTA Fock partials
//   part[((ipjp*ne + i1)*nsub + s)*ne + j1]:
//   fe(i1,j1) (+)= fe_scale * sum_ipjp DP * sum_s part,
//   fp(ipjp)  (+)= sum_{i1,j1} DE * sum_s part,  E = sum_ipjp DP * fp-part.
cudaError_t launch_fock_reduce(int ne, int np, int nsub, const double* part,
                               const double* DE, const double* DP,
                               double fe_scale, int accumulate, double* fe,
                               double* fp, double* fp_tmp, double* E,
                               cudaStream_t s);

// ---- open-shell XCUHF contractions (k_spin.cu, xcuhf/xcuhf_omg*.f) ------
// Rank K = 2 (GM2ICR, optional GM2sICR as Gs), 3 (GM3ICR) or 4 (OMG4_ICR).
// Flag bits per class (A = alpha-led, B = beta-led), in the order of the
// reference's flag sets (FAE_OMG2: LAA, LAB; FAE_OMG3: LAA, LAB, LBB;
// FAE_OMG4: LAAA, LAAB, LBBA, LBBB; UFP_*: the class-A subset of L4A,
// L3A1B, L2A2B, L1A3B ...).  Outputs, device, overwritten:
//   fe_out[a][i + ne*j] = sum_{ipjp} DP * (sum over the other electrons of
//                         class/tensor a = 2*tensor + class),
//   fp_out[t][ip + np*jp] = sum_{i1,j1} (DA part_A + DB part_B) of tensor t.
size_t spin_scratch_doubles(int K, int ne, int np);
// Ranks 3 and 4 stage a bra's ne^K kets in shared memory (up to nebf = 28
// and 12); rank 2 falls back to global-memory gathers beyond that.
bool spin_smem_fits(int K, int ne);
cudaError_t launch_spin_omg(int K, int ne, int np, const double* G, const double* Gs,
                            const double* DA, const double* DB, const double* DP,
                            unsigned fa, unsigned fb, double* scratch,
                            double* fe_out, double* fp_out, cudaStream_t s);
// GAM_1 / GAM_1s: fe_out[t] = sum_ipjp DP G_t, fp_out[t] = sum W G_t.
cudaError_t launch_omg1(int ne, int np, const double* G1, const double* G1s,
                        const double* W, const double* DP, double* fe_out,
                        double* fp_out, cudaStream_t s);
// F (+)= scale x (if F), S = scale xs (if S and xs), E = <W,x>, Es = <W,xs>.
cudaError_t launch_spin_finish(int n, const double* x, const double* xs,
                               const double* W, double scale, double* F, double* S,
                               double* E, double* Es, cudaStream_t s);
// OMG4_ICR: raw calc_GAM_4_integral tensor (ne^8 np^2, index_GAM_4PK2).
cudaError_t launch_omg4_icr(int ne, int np, const double* gee, const double* g2s,
                            double* g4, cudaStream_t s);

// ---- RXCHF / RXCUHF special-electron contractions (k_rx.cu) -------------
// One routine of rxchf_omg{2,3,4}.f, rxcuhf_omg{2,3}.f or rxcuhfne_omg2.f.
// Tensors T1/T2/Ts and densities A (alpha / DAE), Abet, Atot, B (DBE), P as
// the routine needs them; F0..F2 (device, accumulate) are the routine's
// output matrices in the reference's argument order, E[0..1] its energies
// (overwritten).
enum class RxRoutine {
  CuhfneFE2, CuhfneFP2, CuhfneFBE2,          // RXCUHFne_FE/FP/FBE_OMG2
  FAE2, FP2, FBE2, FAE3, FP3, FBE3, FAE4, FP4, FBE4,   // RXCHF_FAE/FP/FBE_OMGk
  CuFE2, CuFP2, CuFBE2, CuFE3, CuFP3, CuFBE3  // RXCUHF_FE/FP/FBE_OMGk
};
size_t rx_scratch_doubles(int ne, int np);
cudaError_t launch_rx(RxRoutine r, int ne, int np, const double* T1, const double* T2,
                      const double* Ts, const double* A, const double* Abet,
                      const double* Atot, const double* B, const double* P,
                      double* scratch, double* F0, double* F1, double* F2, double* E,
                      cudaStream_t s);

// ---- gam_4 (gam_4_OMP.f, gam4_DSCF_OMP.f, gam4_ICR_OMP.f) --------------
constexpr int kGam4MaxNE = 24;   // shared-memory tables: 25*ne^2 doubles
constexpr int64_t kGam4MaxNP = 4096;   // npbf bound checked before any int cast
size_t gam4_partial_doubles(int ne, int np);   // scratch the DSCF path uses
cudaError_t launch_gam4_dscf(int ne, int np, const double* gee,
                             const double* g2s, const double* DE,
                             const double* DP, double* scratch,
                             double* focke, double* fockp, double* E,
                             cudaStream_t s);
cudaError_t launch_gam4_icr(int ne, int np, const double* gee,
                            const double* g2s, double* g4, cudaStream_t s);
size_t eg4_partial_doubles(int ne, int np);
cudaError_t launch_eg4icr(int ne, int np, const double* DE, const double* DP,
                          const double* g4, double* scratch, double* focke,
                          double* fockp, double* E, cudaStream_t s);

// Factorised gam_4 Fock build (k_gam4f.cu): same focke/fockp/E as
// launch_gam4_dscf for pair-symmetric GAM_ee / GAM_2s, at O(ne^4 np^2 + ne^5).
// accumulate = 1 adds into focke/fockp; E is always overwritten.
constexpr int kGam4FactMaxNE = 64;
size_t gam4f_scratch_doubles(int ne, int np);
cudaError_t launch_gam4_factored(int ne, int np, const double* gee,
                                 const double* g2s, const double* DE,
                                 const double* DP, double* scratch,
                                 double* focke, double* fockp, double* E,
                                 int accumulate, cudaStream_t s);
// The same build with the one-index transforms and the focke contraction on
// the tensor cores (tcgen05, 3xTF32 products with FP32 accumulation, FP64
// results); the passes over GAM_2s, traces and gradients stay FP64.
size_t gam4f_tc_scratch_doubles(int ne, int np);
cudaError_t launch_gam4_factored_tc(int ne, int np, const double* gee,
                                    const double* g2s, const double* DE,
                                    const double* DP, double* scratch,
                                    double* focke, double* fockp, double* E,
                                    int accumulate, cudaStream_t s);
// Largest |T - T^swap| and |T| over GAM_ee (t=0) and GAM_2s (t=1), where
// ^swap exchanges the two electron pairs; per-CTA maxima in out[4*grid],
// returns the grid size used in *grid.
cudaError_t launch_pair_symmetry_check(int ne, int np, const double* gee,
                                       const double* g2s, double* out,
                                       int* grid, cudaStream_t s);

// ---- in-core contractions (gam2_IC1_OMP.f, gam3_IC1_OMP.f, rxchfne) ----
size_t eg3_partial_doubles(int ne, int np);
cudaError_t launch_eg3ic1(int ne, int np, const double* DE, const double* DP,
                          const double* g3, double* scratch, double* focke,
                          double* fockp, double* E, cudaStream_t s);
size_t eg2_partial_doubles(int ne, int np);
cudaError_t launch_eg2ic1(int ne, int np, const double* DE, const double* DP,
                          const double* g2, const double* g2s,
                          double* scratch, double* FE, double* SE, double* FP,
                          double* SP, double* E, double* S, cudaStream_t s);
size_t omg2_partial_doubles(int ne, int np);
// FAE / FP / FBE may be null (that output is skipped); E always written
cudaError_t launch_rxchfne_omg2(int ne, int np, const double* DAE,
                                const double* DBE, const double* DP,
                                const double* g2, double* scratch, double* FAE,
                                double* FP, double* FBE, double* E,
                                cudaStream_t s);
cudaError_t launch_xcfock_correction(int ne, int np, double S_total,
                                     double H_expect, const double* se1,
                                     const double* sp1, const double* se2,
                                     const double* sp2, double* focke,
                                     double* fockp, cudaStream_t s);

// Partial sums of one proton-pair slice [ipjp0, ipjp0+nipjp) of the
// contraction; the slice pointer addresses the slice's first element and the
// partials land at their global positions (direct-SCF slicing).
cudaError_t launch_eg3_partials(int ne, int np, long long ipjp0,
                                long long nipjp, const double* DE,
                                const double* g3_slice, double* part,
                                cudaStream_t s);
cudaError_t launch_eg2_partials(int ne, int np, long long ipjp0,
                                long long nipjp, const double* DE,
                                const double* g2_slice,
                                const double* g2s_slice, double* pv,
                                double* ps, cudaStream_t s);

// ---- integral builders (MD kernels) ------------------------------------
cudaError_t launch_gam_ee(const DevSystem& sys, double* gee, cudaStream_t s);
// tuples [t0, t0+ntup) of the packed index space, written from x[0]
cudaError_t launch_gam2_raw_range(const DevSystem& sys, int rx, long long t0,
                                  long long ntup, double* x1, double* x2,
                                  cudaStream_t s, int fp32 = 0);
// gam_3 raw tensor = W1(p,e1) GAM_ee(e2,e3) + W3(p,e1,e2) Hcore(e3) + R4,
// R4 the contracted primitive sum of the four-particle terms, stored once
// per pair-canonical tuple (k_gam3.cu).  aux (gam3_aux_doubles) holds
// GAM_ee, Hcore, W1, W3 (launch_gam3_aux, FP64) and R4 (launch_gam3_pairs).
size_t gam3_aux_doubles(int ne, int np);
size_t gam3_r4_doubles(int ne, int np);
// gee_in / hc_in (optional, device): GAM_ee and Hcore already built by the
// caller (C-order [i][j][k][l] and [i][j]); copied instead of recomputed.
cudaError_t launch_gam3_aux(const DevSystem& sys, double* aux, cudaStream_t s,
                            const double* gee_in = nullptr,
                            const double* hc_in = nullptr);
// R4 into aux.  fp32 = 1: the four-particle integrals in FP32 with FP64
// Boys function, seeds and sums (mixed path).  screen > 0: (bra, ket)
// pairs whose Schwarz-type estimate is below it are skipped.
cudaError_t launch_gam3_pairs(const DevSystem& sys, double* aux, cudaStream_t s,
                              int fp32, double screen);
// raw tensor of packed tuples [t0, t0+ntup) into x3, after launch_gam3_pairs
cudaError_t launch_gam3_raw_range(const DevSystem& sys, const double* aux,
                                  long long t0, long long ntup, double* x3,
                                  cudaStream_t s);
// pair records of the gam_3 builder (sys.g3i must be set)
size_t g3_record_doubles(int nket, int np);
cudaError_t launch_g3_records(const DevSystem& sys, double* rec, cudaStream_t s);
constexpr int kG3MaxTileKets = 1024;
constexpr double kScreenThreshold = 1.0e-12;   // NEOXC_SCF_SCREEN
cudaError_t launch_gam2_raw(const DevSystem& sys, int rxchfne, double* x1,
                            double* x2, cudaStream_t s, int fp32 = 0);
// Dynamic precision of the mixed gam_2 build (process-wide): a primitive
// item whose FP32 contribution to a contracted element exceeds this
// magnitude is re-evaluated in FP64.
constexpr double kMixedTauGam2 = 1.0e-5;
void set_mixed_recompute_tau(double tau);
double mixed_recompute_tau();
cudaError_t launch_gam2_symmetrize(int ne, int np, int rxchfne, double* x1,
                                   double* x2, cudaStream_t s);
// Many systems of one angular class in one persistent launch: both passes of
// the four-particle terms of every system go through one device work queue
// (an atomic counter over items numbered system by system), each CTA taking
// `chunk` items at a time; r4a receives the G4Vep pass, r4b the G4Vee pass
// (launch_gam3_add adds them).  Grid: ctas_per_sm CTAs per SM.  limit caps
// the items processed (the autotuner's samples; < 0: all).  scratch:
// gam3_batch_scratch_bytes(nsys) of device memory for the system table,
// the item prefix sums and the counter.
struct G3BatchSys {
  DevSystem S;
  const double* erec;
  const double* prec;
  double* r4a;
  double* r4b;
};
size_t gam3_batch_scratch_bytes(int nsys);
cudaError_t launch_gam3_batch_pairs(const G3BatchSys* h_sys, int nsys, int fp32, double screen,
                                    void* scratch, int ctas_per_sm, int chunk, long long limit,
                                    long long* total_items, cudaStream_t s);
cudaError_t launch_gam3_add(long long n, double* a, const double* b, cudaStream_t s);
// launch_gam3_pairs + launch_gam3_raw_range over every tuple
cudaError_t launch_gam3_raw(const DevSystem& sys, double* aux, double* x3,
                            cudaStream_t s, int fp32 = 0, double screen = 0.0);
cudaError_t launch_gam3_symmetrize(int ne, int np, double* g3,
                                   cudaStream_t s);

// ---- XCHF SCF (k_scf.cu): xcscf.f, xchf1_fock.f ---------------------------
// Device energy slots: 0 E_total 1 E_nuc 2 E_ecore 3 E_pcore 4 E_ep 5 E_ee
// 6 E_gam1 7 E_gam2 8 E_gam3 9 E_gam4 10 S_total 11 S_gam1 12 S_gam2
// 13 H_expect 14 max|dDE| 15 max|dDP|.
constexpr int kScfMaxN = 64;   // one-CTA Jacobi eigensolver (3 n^2 doubles)
constexpr int kScfSlots = 16;
cudaError_t launch_scf_onebody(const DevSystem& sys, double* Se, double* Sp,
                               double* Hce, double* Hcp, cudaStream_t s);
cudaError_t launch_gam_ep(const DevSystem& sys, double* Gep, cudaStream_t s);
// pairs_only = 1: RXCHF_GAM1_OMP_MD (rxchf/rxchf_gam_1_OMP.f), the
// geminal-pair terms only.
cudaError_t launch_gam1(const DevSystem& sys, double* G1, double* G1s,
                        cudaStream_t s, int fp32 = 0, int pairs_only = 0);
size_t scf_fock1_part_doubles(int ne, int np);
cudaError_t launch_scf_fock1(int ne, int np, int nelec, const double* Hce,
                             const double* Hcp, const double* Gep,
                             const double* G1, const double* G1s,
                             const double* Gee, const double* DE,
                             const double* DP, double* focke, double* fockp,
                             double* se1, double* sp1, double* part, double* en,
                             cudaStream_t s, double* xfocke = nullptr,
                             double* xfockp = nullptr);
cudaError_t launch_scf_assemble(int ne, int np, double* en, const double* se1,
                                const double* sp1, const double* se2,
                                const double* sp2, double* focke,
                                double* fockp, cudaStream_t s);
cudaError_t launch_inv_sqrt(int n, const double* S, double* X, int* status,
                            cudaStream_t s);
cudaError_t launch_roothan(int n, const double* F, const double* X, int first,
                           int nocc, double prefac, double* D, double* evals,
                           double* C, int* status, cudaStream_t s,
                           const int* skip = nullptr);
// One second-order SCF step on the electronic orbitals (soscf.f, as xcscf.f
// drives it); state[1] = 1 when it replaced the diagonalisation (pass
// state + 1 as launch_roothan's skip).  work = soscf_doubles(n, na, maxit).
size_t soscf_doubles(int n, int na, int maxit);
cudaError_t launch_soscf(int n, int na, const double* F, double* C, const double* EE,
                         double prefac, double* D, int* state, double* work, int maxit,
                         cudaStream_t s);
// XCUHF (UHF_FOCK): one-body / HF terms of both spins and the proton
// (energies into en[2..6], en[11]; en[7..9], en[12] zeroed), the
// normalisation + UHF_Fock_correction, and DENDIF of alpha, beta, proton
// into en[13..15].
cudaError_t launch_uhf_fock1(int ne, int np, const double* Hce, const double* Hcp,
                             const double* Gep, const double* G1, const double* G1s,
                             const double* Gee, const double* DAE, const double* DBE,
                             const double* DP, double* FAE, double* FBE, double* FP,
                             double* SAE1, double* SBE1, double* SP1, double* part,
                             double* en, cudaStream_t s);
cudaError_t launch_uhf_assemble(int ne, int np, double* en, const double* sae1,
                                const double* sbe1, const double* sp1,
                                const double* sae2, const double* sbe2,
                                const double* sp2, double* FAE, double* FBE, double* FP,
                                cudaStream_t s);
cudaError_t launch_uhf_dendif(int ne, int np, const double* DA, double* DA0,
                              const double* DB, double* DB0, const double* DP,
                              double* DP0, double* en, cudaStream_t s);
cudaError_t launch_dendif(int ne, int np, const double* DE, double* DE0,
                          const double* DP, double* DP0, double* en,
                          cudaStream_t s);
// Pulay DIIS on F (in place) with error F D S - S D F; work = diis_doubles(n)
// (zeroed before the first call), state[2] = {0, 0} initially.
size_t diis_doubles(int n);
cudaError_t launch_diis(int n, double* F, const double* D, const double* S,
                        double* work, int* state, double* err, cudaStream_t s);

// ---- one-special-electron RXCHF SCF pieces (k_rxscf.cu) ------------------
// Device energy slots of the RX Fock build: 0 E_total (with E_nuc) 1 E_nuc
// 2 E_ecore 3 E_ee 4 E_OMG1 5 E_OMG2 6 S_total 7 E_P_OMG1 8 E_P_OMG2
// 9 S_P_OMG1 10 E_BE_OMG1 11 S_BE_OMG1 12-15 density changes.
constexpr int kRxSlots = 16;
size_t rx_fock1_part_doubles(int ne);
// Regular electrons' FAE_ecore + GAMee terms: closed (open = 0: FA1 from DA)
// or open shell (FA1 / FB1 per spin, DT = DA + DB); en[2], en[3].
cudaError_t launch_rx_fock1(int ne, int open, int with_ee, const double* Hce,
                            const double* Gee, const double* DA, const double* DB,
                            double* FA1, double* FB1, double* DT, double* part,
                            double* en, cudaStream_t s);
cudaError_t launch_rx_assemble(int ne, int np, double* en, const double* XFA1,
                               const double* XFA2, const double* XFB1,
                               const double* XFB2, const double* XFP,
                               const double* XSP, const double* XFBE,
                               const double* XSBE, double* FA, double* FB, double* FP,
                               double* FBE, cudaStream_t s);
cudaError_t launch_rx_dendif(int n, const double* D, double* D0, double* out,
                             cudaStream_t s);
// RXCHF_OCBSE2: new special-electron orbitals CB (column-major n x n) and
// DB from the regular orbitals CA (nocca occupied), the previous special
// orbital cb0 and FBE.  info[2] = {discarded orbital, projected norm},
// status[2] of the subspace eigensolver.
size_t ocbse_scratch_doubles(int n);
cudaError_t launch_ocbse2(int n, int nocca, const double* CA, const double* cb0,
                          const double* F, const double* S, double* scratch,
                          double* CB, double* DB, double* info, int* status,
                          cudaStream_t s);

// ---- index maps on the device (pack_GAM.f) -----------------------------
cudaError_t launch_index_fill(int kind, int ne, int np, int64_t count,
                              int64_t* out, cudaStream_t s);

}  // namespace neoxc
