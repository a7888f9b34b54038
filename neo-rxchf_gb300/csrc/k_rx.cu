// k_rx.cu -- in-core RXCHF / RXCUHF contractions (special-electron
// families) for sm_103a.
//
// Reference: rxchf/rxchf_omg2.f, rxchf_omg3.f, rxchf_omg4.f (RXCHF-fe:
// RXCHF_FAE/FP/FBE_OMGk), rxchf/rxcuhf_omg2.f, rxcuhf_omg3.f (RXCUHF-fe:
// RXCUHF_FE/FP/FBE_OMGk) and rxchfne/rxcuhfne_omg2.f (RXCUHF-ae:
// RXCUHFne_FE/FP/FBE_OMG2).
//
// These routines read several stored tensors at index patterns that mix
// bra and ket positions (e.g. index_GAM_3PK(ip,jp,ie1,ie2,je2,je1,...)), so
// one bra's kets are not a closed block as in the XCUHF contractions.  The
// layout here is output-stationary instead: a CTA owns one element of the
// output matrix (F(i_r,j_r) of the slot the routine's Fock matrix belongs
// to, or FP(ip,jp)) and a slice of the remaining index space; its threads
// evaluate the routine's element formula with gathers that hit L2 (the
// in-core tensors of these methods are tens of MB), and the per-CTA sums
// are reduced in a fixed order by a second kernel.  Each routine is one
// functor with the reference's formula; up to three output matrices and
// two energies per routine, all accumulated as the reference's add2fock.
#include "neoxc_internal.h"

namespace neoxc {
namespace {

constexpr int kRxThreads = 256;
constexpr int kRxCh = 5;   // 3 matrices + 2 energies per CTA partial

// index_GAM_2PK / 3PK / 4PK2 - 1 for pair-slot arguments (bra_m, ket_m)
__device__ __forceinline__ long long x2(int ne, long long ipjp, int a1, int b1, int a2,
                                        int b2) {
  return b2 + ne * (a2 + ne * (b1 + (long long)ne * (a1 + ne * ipjp)));
}
__device__ __forceinline__ long long x3(int ne, long long ipjp, int a1, int b1, int a2,
                                        int b2, int a3, int b3) {
  return b3 + ne * (a3 + (long long)ne * x2(ne, ipjp, a1, b1, a2, b2));
}
__device__ __forceinline__ long long x4(int ne, long long ipjp, int a1, int b1, int a2,
                                        int b2, int a3, int b3, int a4, int b4) {
  return b4 + ne * (a4 + (long long)ne * x3(ne, ipjp, a1, b1, a2, b2, a3, b3));
}

struct RxView {
  int ne, np;
  const double *T1, *T2, *Ts;                    // tensors of the routine
  const double *A, *Abet, *Atot, *B, *P;         // densities (column-major)
  __device__ double a(int i, int j) const { return __ldg(A + i + ne * j); }
  __device__ double ab(int i, int j) const { return __ldg(Abet + i + ne * j); }
  __device__ double at(int i, int j) const { return __ldg(Atot + i + ne * j); }
  __device__ double b(int i, int j) const { return __ldg(B + i + ne * j); }
  __device__ double p(int ip, int jp) const { return __ldg(P + ip + np * jp); }
};

// ---- RXCUHF-ae (rxcuhfne_omg2.f), tensors T1 = GM2ICR, T2 = GM2exICR ----
// val12 = GM2ICR(ia_12), val21 = GM2exICR(ia_21)
struct CuhfneFE2 {   // :131-237, F = (FAalpE, FAbetE), E_AE_OMG2
  static constexpr int K = 2, SLOT = 2, NF = 2, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double v12 = __ldg(v.T1 + x2(v.ne, pq, i[0], j[0], i[1], j[1]));
    const double v21 = __ldg(v.T2 + x2(v.ne, pq, i[0], j[1], i[1], j[0]));
    const double w = v.p(ip, jp) * v.b(i[0], j[0]);
    f[0] += w * (v12 - v21);
    f[1] += w * v12;
    e[0] += w * (v.at(i[1], j[1]) * v12 - v.a(i[1], j[1]) * v21);
  }
};
struct CuhfneFP2 {   // :347-443
  static constexpr int K = 2, SLOT = 0, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double v12 = __ldg(v.T1 + x2(v.ne, pq, i[0], j[0], i[1], j[1]));
    const double v21 = __ldg(v.T2 + x2(v.ne, pq, i[0], j[1], i[1], j[0]));
    const double x = v.b(i[0], j[0]) * (v.at(i[1], j[1]) * v12 - v.a(i[1], j[1]) * v21);
    f[0] += x;
    e[0] += v.p(ip, jp) * x;
  }
};
struct CuhfneFBE2 {  // :553-651
  static constexpr int K = 2, SLOT = 1, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double v12 = __ldg(v.T1 + x2(v.ne, pq, i[0], j[0], i[1], j[1]));
    const double v21 = __ldg(v.T2 + x2(v.ne, pq, i[0], j[1], i[1], j[0]));
    const double x = v.p(ip, jp) * (v.at(i[1], j[1]) * v12 - v.a(i[1], j[1]) * v21);
    f[0] += x;
    e[0] += v.b(i[0], j[0]) * x;
  }
};

// ---- RXCHF-fe, rank 2 (rxchf_omg2.f): T1 = GM2_1ICR, T2 = GM2_2ICR, Ts = GM2sICR
struct Rx2 {
  double val1, val2, sv;
  __device__ Rx2(const RxView& v, long long pq, const int* i, const int* j) {
    val1 = __ldg(v.T1 + x2(v.ne, pq, i[0], j[0], i[1], j[1]));
    val2 = __ldg(v.T2 + x2(v.ne, pq, i[0], j[1], i[1], j[0]));
    sv = __ldg(v.Ts + x2(v.ne, pq, i[0], j[1], i[1], j[0]));
  }
};
struct RxFAE2 {   // :116-229, F = (FAE, SAE), (E_AE_OMG2, S_AE_OMG2)
  static constexpr int K = 2, SLOT = 2, NF = 2, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double w = v.p(ip, jp) * v.b(i[0], j[0]);
    f[0] += w * (2.0 * r.val1 - r.val2);
    f[1] += w * r.sv;
    const double wa = w * v.a(i[1], j[1]);
    e[0] += wa * (r.val1 - 0.5 * r.val2);
    e[1] += wa * (-0.5) * r.sv;
  }
};
struct RxFP2 {    // :336-447
  static constexpr int K = 2, SLOT = 0, NF = 2, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double w = v.a(i[1], j[1]) * v.b(i[0], j[0]);
    const double x = w * (r.val1 - 0.5 * r.val2), y = -0.5 * w * r.sv;
    f[0] += x;
    f[1] += y;
    e[0] += v.p(ip, jp) * x;
    e[1] += v.p(ip, jp) * y;
  }
};
struct RxFBE2 {   // :554-667
  static constexpr int K = 2, SLOT = 1, NF = 2, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double w = v.a(i[1], j[1]) * v.p(ip, jp);
    const double x = w * (r.val1 - 0.5 * r.val2), y = -0.5 * w * r.sv;
    f[0] += x;
    f[1] += y;
    e[0] += v.b(i[0], j[0]) * x;
    e[1] += v.b(i[0], j[0]) * y;
  }
};

// ---- rank 3 (rxchf_omg3.f, rxcuhf_omg3.f): T1 = GM3_1ICR, T2 = GM3_2ICR ---
// The six ket permutations at the plain bra, named as the reference's ia_*.
struct P3 {
  long long i123, i213, i312, i132, i231, i321;
  __device__ P3(int ne, long long pq, const int* i, const int* j) {
    i123 = x3(ne, pq, i[0], j[0], i[1], j[1], i[2], j[2]);
    i213 = x3(ne, pq, i[0], j[1], i[1], j[0], i[2], j[2]);
    i312 = x3(ne, pq, i[0], j[2], i[1], j[0], i[2], j[1]);
    i132 = x3(ne, pq, i[0], j[0], i[1], j[2], i[2], j[1]);
    i231 = x3(ne, pq, i[0], j[1], i[1], j[2], i[2], j[0]);
    i321 = x3(ne, pq, i[0], j[2], i[1], j[1], i[2], j[0]);
  }
};
// The bra/ket-mixed partners of RXCHF_thread_FAEOMG3 / RXCUHF_thread_FEOMG3:
// ib_123_213, ib_123_312, ia_132_312, ia_132_213, ib_132_312, ib_132_213.
struct Q3 {
  long long b123_213, b123_312, a132_312, a132_213, b132_312, b132_213;
  __device__ Q3(int ne, long long pq, const int* i, const int* j) {
    b123_213 = x3(ne, pq, i[0], i[1], j[1], j[0], i[2], j[2]);
    b123_312 = x3(ne, pq, i[0], j[2], j[1], j[0], i[2], i[1]);
    a132_312 = x3(ne, pq, i[0], j[2], i[2], j[0], i[1], j[1]);
    a132_213 = x3(ne, pq, i[0], j[1], i[2], j[0], i[1], j[2]);
    b132_312 = x3(ne, pq, i[0], j[2], i[2], j[0], j[1], i[1]);
    b132_213 = x3(ne, pq, i[0], i[1], i[2], j[0], j[1], j[2]);
  }
};

struct RxFAE3 {   // rxchf_omg3.f:107-261
  static constexpr int K = 3, SLOT = 2, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const P3 a(v.ne, pq, i, j);
    const Q3 q(v.ne, pq, i, j);
    const double* G1 = v.T1;
    const double* G2 = v.T2;
    const double val1 = __ldg(G1 + a.i123) - 0.5 * __ldg(G1 + a.i132);
    const double val2 = (__ldg(G2 + a.i213) + __ldg(G2 + q.b123_213)) -
                        0.5 * (__ldg(G2 + a.i312) + __ldg(G2 + q.b123_312));
    const double val3 = (__ldg(G2 + q.a132_312) + __ldg(G2 + q.b132_312)) -
                        0.5 * (__ldg(G2 + q.a132_213) + __ldg(G2 + q.b132_213));
    const double dp = v.p(ip, jp), db = v.b(i[0], j[0]), a3 = v.a(i[2], j[2]);
    f[0] += a3 * db * dp * (2.0 * val1 - 0.5 * (val2 + val3));
    e[0] += 0.5 * dp * db * v.a(i[1], j[1]) * a3 * (val1 - 0.5 * val2);
  }
};
struct Rx3PB {   // val1 - val2 of RXCHF_thread_FPOMG3 / FBEOMG3
  __device__ static double c(const RxView& v, long long pq, const int* i, const int* j) {
    const P3 a(v.ne, pq, i, j);
    const double val1 = __ldg(v.T1 + a.i123) - 0.5 * __ldg(v.T1 + a.i132);
    const double val2 = __ldg(v.T2 + a.i213) - 0.5 * __ldg(v.T2 + a.i312);
    return val1 - val2;
  }
};
struct RxFP3 {    // rxchf_omg3.f:368-484
  static constexpr int K = 3, SLOT = 0, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = 0.5 * v.a(i[1], j[1]) * v.a(i[2], j[2]) * v.b(i[0], j[0]) *
                     Rx3PB::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.p(ip, jp) * x;
  }
};
struct RxFBE3 {   // rxchf_omg3.f:591-708
  static constexpr int K = 3, SLOT = 1, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = 0.5 * v.a(i[1], j[1]) * v.a(i[2], j[2]) * v.p(ip, jp) *
                     Rx3PB::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.b(i[0], j[0]) * x;
  }
};

// ---- rank 4 (rxchf_omg4.f): T1 = GM4ICR ----------------------------------
struct Rx4C {   // val1 - val2/2 - val3 + val4/2 with ia_3124, ia_3142, ia_2134, ia_2143
  __device__ static double c(const RxView& v, long long pq, const int* i, const int* j) {
    const int ne = v.ne;
    const double v1 = __ldg(v.T1 + x4(ne, pq, i[0], j[2], i[1], j[0], i[2], j[1], i[3], j[3]));
    const double v2 = __ldg(v.T1 + x4(ne, pq, i[0], j[2], i[1], j[0], i[2], j[3], i[3], j[1]));
    const double v3 = __ldg(v.T1 + x4(ne, pq, i[0], j[1], i[1], j[0], i[2], j[2], i[3], j[3]));
    const double v4 = __ldg(v.T1 + x4(ne, pq, i[0], j[1], i[1], j[0], i[2], j[3], i[3], j[2]));
    return v1 - 0.5 * v2 - v3 + 0.5 * v4;
  }
};
struct RxFAE4 {   // :107-221
  static constexpr int K = 4, SLOT = 2, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double c = Rx4C::c(v, pq, i, j);
    const double w = v.p(ip, jp) * v.b(i[0], j[0]) * v.a(i[2], j[2]) * v.a(i[3], j[3]);
    f[0] += 0.5 * w * c;
    e[0] += 0.25 * w * v.a(i[1], j[1]) * c;
  }
};
struct RxFP4 {    // :328-442
  static constexpr int K = 4, SLOT = 0, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = 0.25 * v.b(i[0], j[0]) * v.a(i[1], j[1]) * v.a(i[2], j[2]) *
                     v.a(i[3], j[3]) * Rx4C::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.p(ip, jp) * x;
  }
};
struct RxFBE4 {   // :549-663
  static constexpr int K = 4, SLOT = 1, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = 0.25 * v.p(ip, jp) * v.a(i[1], j[1]) * v.a(i[2], j[2]) *
                     v.a(i[3], j[3]) * Rx4C::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.b(i[0], j[0]) * x;
  }
};

// ---- RXCUHF-fe (rxcuhf_omg2.f, rxcuhf_omg3.f) -------------------------------
struct CuFE2 {    // rxcuhf_omg2.f:128-251, F = (FAalpE, FAbetE, SAalpE)
  static constexpr int K = 2, SLOT = 2, NF = 3, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double w = v.p(ip, jp) * v.b(i[0], j[0]);
    f[0] += w * (r.val1 - r.val2);
    f[1] += w * r.val1;
    f[2] += w * r.sv;
    e[0] += w * (v.at(i[1], j[1]) * r.val1 - v.a(i[1], j[1]) * r.val2);
    e[1] += w * (-v.a(i[1], j[1]) * r.sv);
  }
};
struct CuFP2 {    // rxcuhf_omg2.f:354-467
  static constexpr int K = 2, SLOT = 0, NF = 2, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double db = v.b(i[0], j[0]);
    const double x = db * (v.at(i[1], j[1]) * r.val1 - v.a(i[1], j[1]) * r.val2);
    const double y = db * (-v.a(i[1], j[1]) * r.sv);
    f[0] += x;
    f[1] += y;
    e[0] += v.p(ip, jp) * x;
    e[1] += v.p(ip, jp) * y;
  }
};
struct CuFBE2 {   // rxcuhf_omg2.f:578-694
  static constexpr int K = 2, SLOT = 1, NF = 2, NE = 2;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const Rx2 r(v, pq, i, j);
    const double dp = v.p(ip, jp);
    const double x = dp * (v.at(i[1], j[1]) * r.val1 - v.a(i[1], j[1]) * r.val2);
    const double y = dp * (-v.a(i[1], j[1]) * r.sv);
    f[0] += x;
    f[1] += y;
    e[0] += v.b(i[0], j[0]) * x;
    e[1] += v.b(i[0], j[0]) * y;
  }
};
struct CuFE3 {    // rxcuhf_omg3.f:109-268, F = (FAalpE, FAbetE)
  static constexpr int K = 3, SLOT = 2, NF = 2, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const P3 a(v.ne, pq, i, j);
    const Q3 q(v.ne, pq, i, j);
    const double* G1 = v.T1;
    const double* G2 = v.T2;
    const double val1a = __ldg(G1 + a.i123), val1b = __ldg(G1 + a.i132);
    const double g213 = __ldg(G2 + a.i213), g312 = __ldg(G2 + a.i312);
    const double val2a = (g213 + __ldg(G2 + q.b123_213)) * 0.5;
    const double val2b = (g312 + __ldg(G2 + q.b123_312)) * 0.5;
    const double val2c = (__ldg(G2 + q.a132_312) + __ldg(G2 + q.b132_312)) * 0.5;
    const double val2d = (__ldg(G2 + q.a132_213) + __ldg(G2 + q.b132_213)) * 0.5;
    const double w = v.b(i[0], j[0]) * v.p(ip, jp);
    const double t3 = v.at(i[2], j[2]), a3 = v.a(i[2], j[2]), b3 = v.ab(i[2], j[2]);
    f[0] += w * (t3 * val1a - a3 * val1b - t3 * val2a + a3 * val2b - a3 * val2c +
                 a3 * val2d);
    f[1] += w * (t3 * val1a - b3 * val1b - a3 * val2c);
    const double t2 = v.at(i[1], j[1]), a2 = v.a(i[1], j[1]), b2 = v.ab(i[1], j[1]);
    e[0] += v.p(ip, jp) * v.b(i[0], j[0]) *
            (0.5 * t2 * t3 * val1a - 0.5 * (a2 * a3 + b2 * b3) * val1b - a2 * t3 * g213 +
             a2 * a3 * g312);
  }
};
struct Cu3PB {   // the bracket of RXCUHF_thread_FPOMG3 / FBEOMG3
  __device__ static double c(const RxView& v, long long pq, const int* i, const int* j) {
    const P3 a(v.ne, pq, i, j);
    const double val1a = __ldg(v.T1 + a.i123), val1b = __ldg(v.T1 + a.i132);
    const double val2a = __ldg(v.T2 + a.i213), val2b = __ldg(v.T2 + a.i312);
    const double t2 = v.at(i[1], j[1]), a2 = v.a(i[1], j[1]), b2 = v.ab(i[1], j[1]);
    const double t3 = v.at(i[2], j[2]), a3 = v.a(i[2], j[2]), b3 = v.ab(i[2], j[2]);
    return 0.5 * t2 * t3 * val1a - 0.5 * (a2 * a3 + b2 * b3) * val1b - a2 * t3 * val2a +
           a2 * a3 * val2b;
  }
};
struct CuFP3 {    // rxcuhf_omg3.f:373-497
  static constexpr int K = 3, SLOT = 0, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = v.b(i[0], j[0]) * Cu3PB::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.p(ip, jp) * x;
  }
};
struct CuFBE3 {   // rxcuhf_omg3.f:602-728
  static constexpr int K = 3, SLOT = 1, NF = 1, NE = 1;
  __device__ static void eval(const RxView& v, long long pq, int ip, int jp, const int* i,
                              const int* j, double* f, double* e) {
    const double x = v.p(ip, jp) * Cu3PB::c(v, pq, i, j);
    f[0] += x;
    e[0] += v.b(i[0], j[0]) * x;
  }
};

// ---- the output-stationary kernel and its reducer ---------------------------
// CTA (o, split): o = io + n jo is the output element (n = np for the proton
// matrix, else ne), split a strided slice of the remaining index space.
template <class R>
__global__ void __launch_bounds__(kRxThreads)
rx_kernel(RxView v, int nsplit, double* __restrict__ part) {
  constexpr int K = R::K;
  const int ne = v.ne, np = v.np;
  const int n = R::SLOT == 0 ? np : ne;
  const int nout = n * n;
  const int o = blockIdx.x % nout, split = blockIdx.x / nout;
  const int io = o % n, jo = o / n;
  long long total = 1;
  for (int m = 0; m < 2 * K - (R::SLOT == 0 ? 0 : 2); m++) total *= ne;
  if (R::SLOT != 0) total *= (long long)np * np;
  double f[3] = {0.0, 0.0, 0.0}, e[2] = {0.0, 0.0};
  for (long long t = (long long)split * blockDim.x + threadIdx.x; t < total;
       t += (long long)nsplit * blockDim.x) {
    int i[4] = {0, 0, 0, 0}, j[4] = {0, 0, 0, 0};
    int ip, jp;
    long long r = t;
    for (int m = K - 1; m >= 0; m--) {
      if (m == R::SLOT - 1) continue;
      j[m] = (int)(r % ne); r /= ne;
      i[m] = (int)(r % ne); r /= ne;
    }
    if (R::SLOT == 0) {
      ip = io;
      jp = jo;
    } else {
      i[R::SLOT - 1] = io;
      j[R::SLOT - 1] = jo;
      jp = (int)(r % np); r /= np;
      ip = (int)r;
    }
    const long long pq = (long long)ip * np + jp;
    R::eval(v, pq, ip, jp, i, j, f, e);
  }
  __shared__ double red[kRxCh][kRxThreads];
  for (int c = 0; c < 3; c++) red[c][threadIdx.x] = f[c];
  for (int c = 0; c < 2; c++) red[3 + c][threadIdx.x] = e[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < kRxCh; c++) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if ((int)threadIdx.x < kRxCh)
    part[((size_t)o * nsplit + split) * kRxCh + threadIdx.x] = red[threadIdx.x][0];
}

// One CTA: F_c[o] += sum over splits (c < nf), E_c = sum over o and splits.
__global__ void rx_finish_kernel(int nout, int nsplit, int nf, int nen,
                                 const double* __restrict__ part, double* F0, double* F1,
                                 double* F2, double* E) {
  __shared__ double red[2][256];
  double e0 = 0.0, e1 = 0.0;
  for (int o = threadIdx.x; o < nout; o += blockDim.x) {
    double s[kRxCh] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < nsplit; k++)
      for (int c = 0; c < kRxCh; c++) s[c] += part[((size_t)o * nsplit + k) * kRxCh + c];
    if (nf > 0 && F0) F0[o] += s[0];
    if (nf > 1 && F1) F1[o] += s[1];
    if (nf > 2 && F2) F2[o] += s[2];
    e0 += s[3];
    e1 += s[4];
  }
  red[0][threadIdx.x] = e0;
  red[1][threadIdx.x] = e1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (nen > 0) E[0] = red[0][0];
    if (nen > 1) E[1] = red[1][0];
  }
}

constexpr long long kRxTargetCtas = 2 * 152 * 4;

int rx_nsplit(long long total, int nout) {
  // enough CTAs to fill the GPU a few times over, no more splits than blocks
  long long want = (kRxTargetCtas + nout - 1) / nout;
  long long cap = (total + kRxThreads - 1) / kRxThreads;
  long long s = want < cap ? want : cap;
  if (s < 1) s = 1;
  return (int)s;
}

template <class R>
cudaError_t launch_rx_t(const RxView& v, double* scratch, double* F0, double* F1,
                        double* F2, double* E, cudaStream_t s) {
  const int n = R::SLOT == 0 ? v.np : v.ne;
  const int nout = n * n;
  long long total = 1;
  for (int m = 0; m < 2 * R::K - (R::SLOT == 0 ? 0 : 2); m++) total *= v.ne;
  if (R::SLOT != 0) total *= (long long)v.np * v.np;
  const int nsplit = rx_nsplit(total, nout);
  rx_kernel<R><<<(unsigned)((long long)nout * nsplit), kRxThreads, 0, s>>>(v, nsplit,
                                                                            scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  rx_finish_kernel<<<1, 256, 0, s>>>(nout, nsplit, R::NF, R::NE, scratch, F0, F1, F2, E);
  return cudaGetLastError();
}

}  // namespace

size_t rx_scratch_doubles(int ne, int np) {
  // nout * nsplit <= kRxTargetCtas + nout - 1
  const long long nout = ne * ne > np * np ? (long long)ne * ne : (long long)np * np;
  return (size_t)(kRxTargetCtas + nout) * kRxCh;
}

cudaError_t launch_rx(RxRoutine r, int ne, int np, const double* T1, const double* T2,
                      const double* Ts, const double* A, const double* Abet,
                      const double* Atot, const double* B, const double* P,
                      double* scratch, double* F0, double* F1, double* F2, double* E,
                      cudaStream_t s) {
  const RxView v{ne, np, T1, T2, Ts, A, Abet, Atot, B, P};
  switch (r) {
    case RxRoutine::CuhfneFE2: return launch_rx_t<CuhfneFE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuhfneFP2: return launch_rx_t<CuhfneFP2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuhfneFBE2: return launch_rx_t<CuhfneFBE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FAE2: return launch_rx_t<RxFAE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FP2: return launch_rx_t<RxFP2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FBE2: return launch_rx_t<RxFBE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FAE3: return launch_rx_t<RxFAE3>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FP3: return launch_rx_t<RxFP3>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FBE3: return launch_rx_t<RxFBE3>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FAE4: return launch_rx_t<RxFAE4>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FP4: return launch_rx_t<RxFP4>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::FBE4: return launch_rx_t<RxFBE4>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFE2: return launch_rx_t<CuFE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFP2: return launch_rx_t<CuFP2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFBE2: return launch_rx_t<CuFBE2>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFE3: return launch_rx_t<CuFE3>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFP3: return launch_rx_t<CuFP3>(v, scratch, F0, F1, F2, E, s);
    case RxRoutine::CuFBE3: return launch_rx_t<CuFBE3>(v, scratch, F0, F1, F2, E, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace neoxc
