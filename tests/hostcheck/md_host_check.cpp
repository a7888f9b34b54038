// md_host_check.cpp -- test helper: compiles the device integral math
// (neo-rxchf_gb300/csrc/md_math.cuh) as plain C++ so the factorised MD
// algorithm the GPU kernels run can be compared with the CPU oracle on any
// machine.  Only the tests load this library.
#include "../../neo-rxchf_gb300/csrc/md_math.cuh"
#include "../../neo-rxchf_gb300/csrc/md_math32.cuh"
#include "../../neo-rxchf_gb300/csrc/g3_fatbra.cuh"
#include "../../neo-rxchf_gb300/csrc/narrow.cuh"

using namespace neoxc::md;

extern "C" {
// same layout as the oracle's orc_prim
struct HP { int l[3]; double a; double c[3]; };

static Prim cv(const HP& h) {
  Prim p;
  p.a = h.a;
  for (int d = 0; d < 3; d++) { p.l[d] = h.l[d]; p.c[d] = h.c[d]; }
  return p;
}

double hc_g3(int kind, const HP* A, const HP* B, const double* gam,
             const double* C, double xmass) {
  Prim a[3], b[3];
  for (int i = 0; i < 3; i++) { a[i] = cv(A[i]); b[i] = cv(B[i]); }
  static thread_local G3 s;
  g3_setup(s, a, b, gam, kind == 1 ? 2 : 0);
  switch (kind) {
    case 0: return g3_overlap(s);
    case 1: return g3_ke(s, gam[4], xmass);
    case 2: return g3_vxc(s, C);
    default: return g3_vee(s);
  }
}

double hc_g4(int kind, const HP* A, const HP* B, double g1, double g2) {
  G4 s;
  Prim a[4], b[4];
  for (int i = 0; i < 4; i++) { a[i] = cv(A[i]); b[i] = cv(B[i]); }
  g4_pairs(s, a, b);
  return kind == 0 ? g4_vee(s, g1, g2) : g4_vep(s, g1, g2);
}

double hc_g2_xggs(const HP* A1, const HP* A2, const HP* B1, const HP* B2,
                  double g1, double g2) {
  return g2_xggs(cv(*A1), cv(*A2), cv(*B1), cv(*B2), g1, g2);
}
double hc_g2_xggvec(const HP* A1, const HP* A2, const HP* B1, const HP* B2,
                    double g1, double g2, const double* C) {
  return g2_xggvec(cv(*A1), cv(*A2), cv(*B1), cv(*B2), g1, g2, C);
}
double hc_g2_xggvee(const HP* A1, const HP* A2, const HP* B1, const HP* B2,
                    double g1, double g2) {
  return g2_xggvee(cv(*A1), cv(*A2), cv(*B1), cv(*B2), g1, g2);
}
double hc_pgike1(const HP* A1, const HP* A2, const HP* B1, const HP* B2,
                 double gA, double gB, double m) {
  return pgike1(cv(*A1), cv(*A2), cv(*B1), cv(*B2), gA, gB, m);
}
double hc_gfvee(const HP* A1, const HP* A2, const HP* B1, const HP* B2) {
  return gfvee(cv(*A1), cv(*A2), cv(*B1), cv(*B2));
}
double hc_gfke(const HP* A, const HP* B, double m) { return gfke(cv(*A), cv(*B), m); }
double hc_gfvec(const HP* A, const HP* B, const double* C) { return gfvec(cv(*A), cv(*B), C); }
double hc_boys(int m, double T) { double F[64]; neoxc::boys(m, T, F); return F[m]; }
// the tensor-core path's integer-pipe FP64 -> FP32 narrowing
float hc_narrow(double v) { return neoxc::tc::narrow_f64(v); }
// sum_m (-alpha)^m F_m(T) b[m] by the fused recursion, with T passed as FP64
// or (f32 = 1) as FP32
double hc_boys_sum(int L, double T, double alpha, const double* b, int f32) {
  auto bf = [&](int m) { return b[m]; };
  return f32 ? neoxc::boys_sum(L, (float)T, alpha, bf) : neoxc::boys_sum(L, T, alpha, bf);
}

// the FP32 instance (mixed path): same integrals, FP32 tables, FP64 Boys
static neoxc::md32::Prim cv32(const HP& h) {
  neoxc::md32::Prim p;
  p.a = (float)h.a;
  for (int d = 0; d < 3; d++) { p.l[d] = h.l[d]; p.c[d] = (float)h.c[d]; }
  return p;
}
double hc32_g4(int kind, const HP* A, const HP* B, double g1, double g2) {
  neoxc::md32::G4 s;
  neoxc::md32::Prim a[4], b[4];
  for (int i = 0; i < 4; i++) { a[i] = cv32(A[i]); b[i] = cv32(B[i]); }
  neoxc::md32::g4_pairs(s, a, b);
  return kind == 0 ? neoxc::md32::g4_vee(s, (float)g1, (float)g2)
                   : neoxc::md32::g4_vep(s, (float)g1, (float)g2);
}
double hc32_g3(int kind, const HP* A, const HP* B, const double* gam,
               const double* C, double xmass) {
  neoxc::md32::Prim a[3], b[3];
  for (int i = 0; i < 3; i++) { a[i] = cv32(A[i]); b[i] = cv32(B[i]); }
  float g[6], c[3] = {(float)C[0], (float)C[1], (float)C[2]};
  for (int k = 0; k < 6; k++) g[k] = (float)gam[k];
  static thread_local neoxc::md32::G3 s;
  neoxc::md32::g3_setup(s, a, b, g, kind == 1 ? 2 : 0);
  switch (kind) {
    case 0: return neoxc::md32::g3_overlap(s);
    case 1: return neoxc::md32::g3_ke(s, g[4], (float)xmass);
    case 2: return neoxc::md32::g3_vxc(s, c);
    default: return neoxc::md32::g3_vee(s);
  }
}
}  // extern "C"

// the gam_3 builder's composite-bra form (g3_fatbra.cuh) of G4_MD_xgVeeg
// (kind 0: bra e1, e3, p / ket e2) and G4_MD_xgVepg (kind 1: bra e1, e2, p /
// ket e3), in precision R, for the general s/p/d class
template <class R>
static double fb_one(int kind, const HP* A, const HP* B, double g1, double g2) {
  namespace g3 = neoxc::g3;
  double rec[4][g3::kRLen];
  for (int i = 0; i < 4; i++) g3::fill_pair_record(cv(A[i]), cv(B[i]), 1.0, 1.0, rec[i]);
  g3::Bra<R, 12> b;
  int ket;
  if (kind == 1) {
    g3::build_bra_vep<R, 2, 2, 12>(rec[0], rec[1], rec[3], (R)g1, (R)g2, b);
    ket = 2;
  } else {
    g3::build_bra_vee<R, 2, 2, 12>(rec[0], rec[2], rec[3], (R)g1, (R)g2, b);
    ket = 1;
  }
  const double* rk = rec[ket];
  R Xk[3], Ek[3][5];
  int tk[3];
  for (int d = 0; d < 3; d++) {
    Xk[d] = (R)rk[g3::kRX + d];
    tk[d] = (int)rk[g3::kRT + d];
    for (int t = 0; t < 5; t++)
      Ek[d][t] = (t & 1) ? -(R)rk[g3::kRE + 5 * d + t] : (R)rk[g3::kRE + 5 * d + t];
  }
  return g3::fb_eval<R, 12, 4>(b, (R)rk[g3::kRP], Xk, Ek, tk);
}

extern "C" {
double hc_fb(int kind, const HP* A, const HP* B, double g1, double g2) {
  return fb_one<double>(kind, A, B, g1, g2);
}
double hc32_fb(int kind, const HP* A, const HP* B, double g1, double g2) {
  return fb_one<float>(kind, A, B, g1, g2);
}
}
