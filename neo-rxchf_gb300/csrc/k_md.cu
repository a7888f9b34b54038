// k_md.cu -- contracted geminal-integral builders on sm_103a (FP64).
//
// Reference:
//   gam_ee.f:2-169 (calc_GAM_ee)                 -> gam_ee_kernel
//   gam_2_OMP.f:546-1077 (xcalc_GAM2_MD),
//   gam2_CONV_OMP.f:388-579 (contract_omega2_conv),
//   gam2_IC1_OMP.f:214-337 (thread_gam2_IC1)     -> gam2_raw_kernel
//   rxchfne/rxchfne_gam_2_OMP.f:2-530,
//   rxchfne/rxchfne_gam2_IC1_OMP.f:245-340       -> gam2_raw_kernel<RX, F32>
//   gam2_IC1_OMP.f:136-185, rxchfne_gam2_IC1_OMP.f:184-201
//                                                -> gam2_sym_kernel
//   gam_3_OMP.f:617-984 (xcalc_GAM3_MD) separable terms
//                                                -> gam3_w1/w3/hcore_kernel
//     (the four-particle terms: k_gam3.cu)
//   gam3_IC1_OMP.f:143-262                       -> gam3_sym_kernel
//
// Work decomposition: one warp per contracted tuple (its packed index is
// the warp id, since the reference's loop order equals the packing order);
// the lanes split the tuple's primitive combinations and the contraction
// is a warp-shuffle reduction.  Each lane evaluates the reference's
// per-primitive integrand with the factorised MD kernels of md_math.cuh,
// re-using one Boys'-lemma/derivative setup for every integral that shares
// a particle order and geminal assignment.
#include <atomic>
#include <type_traits>

#include "md_math.cuh"
#include "md_math32.cuh"
#include "neoxc_internal.h"

namespace neoxc {
namespace {

using md::G3;
using md::G4;
using md::Prim;

__device__ __forceinline__ Prim to_prim(const DevPrim& d) {
  Prim p;
  p.a = d.a;
  for (int k = 0; k < 3; k++) {
    p.c[k] = d.c[k];
    p.l[k] = d.l[k];
  }
  return p;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <class R>
__device__ __forceinline__ void gam6(R* g, int slot_a, R va, int slot_b, R vb) {
  for (int k = 0; k < 6; k++) g[k] = R(0.0);
  if (slot_a >= 0) g[slot_a] = va;
  if (slot_b >= 0) g[slot_b] = vb;
}
enum { A12 = 0, A13, A23, B12, B13, B23 };

template <class P>
__device__ __forceinline__ void perm3(const P* X, int a, int b, int c, P* Y) {
  Y[0] = X[a];
  Y[1] = X[b];
  Y[2] = X[c];
}

// gam_2_OMP.f:546-1077 xcalc_GAM2_MD.  Particles (e1, e2, p).  P is md::Prim
// (FP64 integrals) or md32::Prim (FP32 integrals of the mixed path); the
// integral calls resolve to md:: / md32:: by argument-dependent lookup and
// every sum over geminal terms is FP64 in both.
//
// The reference's result is a linear combination over geminal terms,
//   ansE = sum_k b_k T1(k) + sum_kl b_k b_l T2(k,l),  ansS = sum_kl b_k b_l S2(k,l),
// so one primitive tuple is split into ng + ng^2 independent work items
// (gi < ng: single-geminal term k = gi; else the pair (k,l)) that the lanes
// of a warp share.
//
// Four of the terms have no geminal on electron 1 -- xgTE and xgVEC (bra
// geminal e2-p), xgTEg3 and xgVECg2 (both geminals e2-p) -- so they factor
// exactly into electron 1's core Hamiltonian times a two-particle geminal
// overlap of (e2, p): their contracted sum is H1(i1,j1) W2(i2,j2,ip,jp) with
//   W2 = sum c^4 [2 sum_k b_k G2xggs(g_k, 0) + sum_kl b_k b_l G2xggs(g_k, g_l)],
// which gam2_raw_kernel adds once per contracted tuple, in FP64 on both
// paths (separable_gam2); the per-primitive items below omit them.
template <class P, class G3T>
__device__ void xcalc_gam2_item(const P* A, const P* B, const DevSystem& S,
                                G3T& st, int gi, double& ansE, double& ansS) {
  using R = typename std::remove_cv<decltype(P::a)>::type;
  const int ng = S.ngtg, nat = S.nat;
  const double* b = S.bgem;
  const double* gm = S.ggem;
  P A132[3], B132[3], A312[3], B312[3];
  perm3(A, 0, 2, 1, A132);
  perm3(B, 0, 2, 1, B132);
  perm3(A, 2, 0, 1, A312);
  perm3(B, 2, 0, 1, B312);
  // Gaussian products of the three particle pairs, shared by every setup
  using PairT = typename std::remove_all_extents<decltype(G3T::pr)>::type;
  PairT pr[3], pr132[3], pr312[3];
  for (int i = 0; i < 3; i++) gauss_pair(A[i], B[i], pr[i]);
  perm3(pr, 0, 2, 1, pr132);
  perm3(pr, 2, 0, 1, pr312);
  R g[6];
  const R zero = R(0.0), one = R(1.0);
  // sum over the classical nuclei of sign * zan * underflow(G3_MD_xgVxCg),
  // in the reference's order; the Hermite fold is shared by all nuclei
  R vx[kMaxNat];
  auto vxc_sum = [&](double sign) {
    g3_vxc_multi(st, nat, S.cat, vx);
    double acc = 0.0;
    for (int ia = 0; ia < nat; ia++) {
      const double v = md::underflow((double)vx[ia]);
      acc = sign < 0.0 ? acc - S.zan[ia] * v : acc + S.zan[ia] * v;
    }
    return acc;
  };
  if (gi < ng) {
    const int ik = gi;
    gam6(g, A23, (R)gm[ik], -1, zero);
    g3_setup_pairs(st, A, B, pr, g, 0);
    double xgVEE = md::underflow((double)g3_vee(st));
    g3_setup_pairs(st, A132, B132, pr132, g, 0);
    double xgVEP = -md::underflow((double)g3_vee(st));
    // 2 (gTE + gVEC + gVEP) + 4 gVEE / 2, gTE and gVEC in separable_gam2
    ansE = 2.0 * (b[ik] * xgVEP) + 4.0 * (b[ik] * xgVEE) * 0.5;
    ansS = 0.0;
    return;
  }
  const int ik = (gi - ng) / ng, il = (gi - ng) - ik * ng;
  const R gk = (R)gm[ik], gl = (R)gm[il];
  const double bb = b[ik] * b[il];
  // order (p, e1, e2): gA12 = g(p,e1), gB13 = g(p,e2)
  gam6(g, A12, gk, B13, gl);
  g3_setup_pairs(st, A312, B312, pr312, g, 2);
  double xgTPg = (double)g3_ke(st, gl, (R)S.pmass);
  double xgVPCg = vxc_sum(1.0);
  // order (e1, e2, p): A13, B23
  gam6(g, A13, gk, B23, gl);
  g3_setup_pairs(st, A, B, pr, g, 2);
  double xgTEg1 = (double)g3_ke(st, zero, one);
  double xgVECg1 = vxc_sum(-1.0);
  double xgVEEg2 = md::underflow((double)g3_vee(st));
  double xgsg = (double)g3_overlap(st);
  // A23, B13
  gam6(g, A23, gk, B13, gl);
  g3_setup_pairs(st, A, B, pr, g, 2);
  double xgTEg2 = (double)g3_ke(st, gl, one);
  // A23, B23: xgTEg3 and xgVECg2 are separable (separable_gam2)
  // A13, B13
  gam6(g, A13, gk, B13, gl);
  g3_setup_pairs(st, A, B, pr, g, 0);
  double xgVEEg1 = md::underflow((double)g3_vee(st));
  // order (e1, p, e2): A12 B23 and A23 B23
  gam6(g, A12, gk, B23, gl);
  g3_setup_pairs(st, A132, B132, pr132, g, 0);
  double xgVEPg1 = -md::underflow((double)g3_vee(st));
  gam6(g, A23, gk, B23, gl);
  g3_setup_pairs(st, A132, B132, pr132, g, 0);
  double xgVEPg2 = -md::underflow((double)g3_vee(st));
  // gTPg + gVPCg + gTEg1 + gTEg3 + 2 (gVEPg1 + gVECg1) + gTEg2 + gVEPg2 +
  // gVECg2 + 2 gVEEg1 / 2 + 2 gVEEg2 / 2, gTEg3 and gVECg2 in separable_gam2
  ansE = bb * xgTPg + bb * xgVPCg + bb * xgTEg1 +
         2.0 * (bb * xgVEPg1 + bb * xgVECg1) + bb * xgTEg2 + bb * xgVEPg2 +
         2.0 * (bb * xgVEEg1) * 0.5 + 2.0 * (bb * xgVEEg2) * 0.5;
  ansS = bb * xgsg;
}

// rxchfne/rxchfne_gam_2_OMP.f:2-530 (live terms :409-456): one geminal pair
// (ik, il) = (gi / ng, gi % ng) per work item:
//   ansE1 = bb (xgVEPg2 + xgVEEg1), ansE2 = bb xgVEEg2.
__device__ void xcalc_gam2_rx_item(const Prim* A, const Prim* B, const DevSystem& S,
                                   G3& st, int gi, double& ansE1, double& ansE2) {
  const int ng = S.ngtg;
  const double* b = S.bgem;
  const double* gm = S.ggem;
  Prim A321[3], B321[3];
  perm3(A, 2, 1, 0, A321);
  perm3(B, 2, 1, 0, B321);
  md::Pair pr[3], pr321[3];
  for (int i = 0; i < 3; i++) md::gauss_pair(A[i], B[i], pr[i]);
  perm3(pr, 2, 1, 0, pr321);
  double g[6];
  const int ik = gi / ng, il = gi - ik * ng;
  const double gk = gm[ik], gl = gm[il], bb = b[ik] * b[il];
  gam6(g, A13, gk, B13, gl);
  md::g3_setup_pairs(st, A321, B321, pr321, g, 0);
  double xgVEPg2 = -md::underflow(md::g3_vee(st));
  md::g3_setup_pairs(st, A, B, pr, g, 0);
  double xgVEEg1 = md::underflow(md::g3_vee(st));
  gam6(g, A13, gk, B23, gl);
  md::g3_setup_pairs(st, A, B, pr, g, 0);
  double xgVEEg2 = md::underflow(md::g3_vee(st));
  ansE1 = bb * xgVEPg2 + bb * xgVEEg1;
  ansE2 = bb * xgVEEg2;
}

__device__ __forceinline__ md32::Prim to_prim32(const DevPrim& d) {
  md32::Prim p;
  p.a = (float)d.a;
  for (int k = 0; k < 3; k++) {
    p.c[k] = (float)d.c[k];
    p.l[k] = d.l[k];
  }
  return p;
}

// The separable part of one contracted XCHF gam_2 tuple (see
// xcalc_gam2_item): H1(i1,j1) W2(i2,j2,ip,jp), FP64, summed by the warp.
// H1 = sum c c [T - sum_C Z V_C] (gfke, gfvec), W2 as above (G2_MD_xggs).
__device__ double separable_gam2(const DevSystem& S, int ic1, int jc1, int ic2, int jc2,
                                 int ip, int jp, int lane) {
  const int s1 = S.kpestr[ic1], n1 = S.kpeend[ic1] - s1 + 1;
  const int t1 = S.kpestr[jc1], m1 = S.kpeend[jc1] - t1 + 1;
  const int s2 = S.kpestr[ic2], n2 = S.kpeend[ic2] - s2 + 1;
  const int t2 = S.kpestr[jc2], m2 = S.kpeend[jc2] - t2 + 1;
  const int ng = S.ngtg;
  double h = 0.0, w = 0.0;
  for (int q = lane; q < n1 * m1; q += 32) {
    const int a = s1 + q / m1, bq = t1 + q % m1;
    const Prim A = to_prim(S.eprim[a]), B = to_prim(S.eprim[bq]);
    double v = md::gfke(A, B, 1.0);
    for (int ia = 0; ia < S.nat; ia++) v = v - S.zan[ia] * md::gfvec(A, B, S.cat + 3 * ia);
    h = h + v * (S.eprim[a].coef * S.eprim[bq].coef);
  }
  const Prim Pa = to_prim(S.pprim[ip]), Pb = to_prim(S.pprim[jp]);
  const int nit = ng + ng * ng;
  for (int q = lane; q < n2 * m2 * nit; q += 32) {
    const int it = q / (n2 * m2), u = q - it * (n2 * m2);
    const int a = s2 + u / m2, bq = t2 + u % m2;
    const Prim A = to_prim(S.eprim[a]), B = to_prim(S.eprim[bq]);
    double v;
    if (it < ng) {
      v = 2.0 * S.bgem[it] * md::g2_xggs(A, Pa, B, Pb, S.ggem[it], 0.0);
    } else {
      const int k = (it - ng) / ng, l = (it - ng) - k * ng;
      v = S.bgem[k] * S.bgem[l] * md::g2_xggs(A, Pa, B, Pb, S.ggem[k], S.ggem[l]);
    }
    w = w + v * (S.eprim[a].coef * S.eprim[bq].coef);
  }
  h = warp_sum(h);
  w = warp_sum(w);
  return h * w * (S.pprim[ip].coef * S.pprim[jp].coef);
}

// ---- GAM_ee: warp per contracted (iec1,jec1,iec2,jec2) ----------------------
// lanes share the primitive quartets; warp-shuffle contraction.
__global__ void __launch_bounds__(128)
gam_ee_kernel(DevSystem S, double* __restrict__ gee) {
  const int ne = S.nebf;
  const long long n4 = (long long)ne * ne * ne * ne;
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * blockDim.x / 32;
  for (long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32; t < n4;
       t += nw) {
    // pack_4D(jec2, iec2, jec1, iec1) - 1 == t
    long long r = t;
    const int jc2 = (int)(r % ne); r /= ne;
    const int ic2 = (int)(r % ne); r /= ne;
    const int jc1 = (int)(r % ne); r /= ne;
    const int ic1 = (int)r;
    const int s1 = S.kpestr[ic1], n1 = S.kpeend[ic1] - s1 + 1;
    const int t1 = S.kpestr[jc1], m1 = S.kpeend[jc1] - t1 + 1;
    const int s2 = S.kpestr[ic2], n2 = S.kpeend[ic2] - s2 + 1;
    const int t2 = S.kpestr[jc2], m2 = S.kpeend[jc2] - t2 + 1;
    const int nq = n1 * m1 * n2 * m2;
    double acc = 0.0;
    for (int q = lane; q < nq; q += 32) {
      int qq = q;
      const int j2 = t2 + qq % m2; qq /= m2;
      const int i2 = s2 + qq % n2; qq /= n2;
      const int j1 = t1 + qq % m1; qq /= m1;
      const int i1 = s1 + qq;
      const DevPrim &a1 = S.eprim[i1], &a2 = S.eprim[i2];
      const DevPrim &b1 = S.eprim[j1], &b2 = S.eprim[j2];
      double v = md::gfvee(to_prim(a1), to_prim(a2), to_prim(b1), to_prim(b2));
      acc = acc + v * a1.coef * b1.coef * a2.coef * b2.coef;
    }
    acc = warp_sum(acc);
    if (lane == 0) gee[t] = acc;
  }
}

// ---- gam_2 raw tensors: warp per contracted tuple --------------------------
// One primitive work item q2 of a tuple (geminal item fastest-varying over
// the primitive combination, see below): its FP64 contribution to x1, x2.
struct Gam2Tuple {
  int s_i1, n_i1, s_j1, n_j1, s_i2, n_i2, s_j2, n_j2, nq;
};

template <bool F32>
__device__ __forceinline__ void gam2_item(const DevSystem& S, const Gam2Tuple& t,
                                          const DevPrim& pa, const DevPrim& pb, double cp,
                                          int q2, double& v1, double& v2) {
  const int gi = q2 / t.nq;
  int qq = q2 - gi * t.nq;
  const int j2 = t.s_j2 + qq % t.n_j2; qq /= t.n_j2;
  const int i2 = t.s_i2 + qq % t.n_i2; qq /= t.n_i2;
  const int j1 = t.s_j1 + qq % t.n_j1; qq /= t.n_j1;
  const int i1 = t.s_i1 + qq;
  double a1, a2;
  if constexpr (F32) {
    md32::G3 st;
    md32::Prim A[3] = {to_prim32(S.eprim[i1]), to_prim32(S.eprim[i2]), to_prim32(pa)};
    md32::Prim B[3] = {to_prim32(S.eprim[j1]), to_prim32(S.eprim[j2]), to_prim32(pb)};
    xcalc_gam2_item(A, B, S, st, gi, a1, a2);
  } else {
    G3 st;
    Prim A[3] = {to_prim(S.eprim[i1]), to_prim(S.eprim[i2]), to_prim(pa)};
    Prim B[3] = {to_prim(S.eprim[j1]), to_prim(S.eprim[j2]), to_prim(pb)};
    xcalc_gam2_item(A, B, S, st, gi, a1, a2);
  }
  const double c = cp * S.eprim[i1].coef * S.eprim[j1].coef *
                   S.eprim[i2].coef * S.eprim[j2].coef;
  v1 = a1 * c;
  v2 = a2 * c;
}

// The FP64 re-evaluation of the mixed path, kept out of line so that it
// does not change the register allocation of the FP32 loop.
__device__ __noinline__ void gam2_item64(const DevSystem& S, const Gam2Tuple& t,
                                         const DevPrim& pa, const DevPrim& pb, double cp,
                                         int q2, double& v1, double& v2) {
  gam2_item<false>(S, t, pa, pb, cp, q2, v1, v2);
}

// F32 (the mixed path) evaluates every item in FP32 first and uses that
// value as its own magnitude estimate: an item whose contribution exceeds
// `tau` in magnitude is discarded and re-evaluated in FP64 (dynamic
// precision per primitive item, in the spirit of Luehr, Ufimtsev and
// Martinez, J. Chem. Theory Comput. 7, 949 (2011), which selects the
// precision per shell quartet from a Schwarz bound).  The FP32 error left
// in the sum is that of the small items only; how much FP64 work that takes
// depends on the basis (at tau = 1e-5 about a quarter of the items of a
// 12-function s/p basis with exponents up to 20, most items of a basis
// with tight s primitives, where the mixed build costs more than the FP64
// one).  Each warp queues its large items in shared memory and
// re-evaluates them 32 at a time, so that the FP64 work runs on full warps.
// The result is deterministic (fixed lane order, fixed queue order).
template <int RX, bool F32>
__global__ void __launch_bounds__(64, F32 ? 16 : 8)
gam2_raw_kernel(DevSystem S, double* __restrict__ x1,
                double* __restrict__ x2, long long t0, long long ntup, double tau) {
  const int ne = S.nebf, np = S.npbf;
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (w >= ntup) return;
  long long r = w + t0;   // packed index - 1 of the tuple; outputs from t0
  const int jc2 = (int)(r % ne); r /= ne;
  const int ic2 = (int)(r % ne); r /= ne;
  const int jc1 = (int)(r % ne); r /= ne;
  const int ic1 = (int)(r % ne); r /= ne;
  const int jp = (int)(r % np);
  const int ip = (int)(r / np);
  Gam2Tuple t;
  t.s_i1 = S.kpestr[ic1]; t.n_i1 = S.kpeend[ic1] - t.s_i1 + 1;
  t.s_j1 = S.kpestr[jc1]; t.n_j1 = S.kpeend[jc1] - t.s_j1 + 1;
  t.s_i2 = S.kpestr[ic2]; t.n_i2 = S.kpeend[ic2] - t.s_i2 + 1;
  t.s_j2 = S.kpestr[jc2]; t.n_j2 = S.kpeend[jc2] - t.s_j2 + 1;
  t.nq = t.n_i1 * t.n_j1 * t.n_i2 * t.n_j2;
  const int ng = S.ngtg;
  const int nitem = RX ? ng * ng : ng + ng * ng;   // geminal work items
  const int total = t.nq * nitem;
  const DevPrim& pa = S.pprim[ip];
  const DevPrim& pb = S.pprim[jp];
  const double cp = pa.coef * pb.coef;
  double o1 = 0.0, o2 = 0.0;
  // lanes take (geminal item, primitive combination) pairs, the primitive
  // combination fastest so that neighbouring lanes share the geminal item
  if constexpr (RX) {
    for (int q2 = lane; q2 < total; q2 += 32) {
      const int gi = q2 / t.nq;
      int qq = q2 - gi * t.nq;
      const int j2 = t.s_j2 + qq % t.n_j2; qq /= t.n_j2;
      const int i2 = t.s_i2 + qq % t.n_i2; qq /= t.n_i2;
      const int j1 = t.s_j1 + qq % t.n_j1; qq /= t.n_j1;
      const int i1 = t.s_i1 + qq;
      G3 st;
      Prim A[3] = {to_prim(S.eprim[i1]), to_prim(S.eprim[i2]), to_prim(pa)};
      Prim B[3] = {to_prim(S.eprim[j1]), to_prim(S.eprim[j2]), to_prim(pb)};
      double a1, a2;
      xcalc_gam2_rx_item(A, B, S, st, gi, a1, a2);
      const double c = cp * S.eprim[i1].coef * S.eprim[j1].coef *
                       S.eprim[i2].coef * S.eprim[j2].coef;
      o1 = o1 + a1 * c;
      o2 = o2 + a2 * c;
    }
  } else if constexpr (!F32) {
    for (int q2 = lane; q2 < total; q2 += 32) {
      double v1, v2;
      gam2_item<false>(S, t, pa, pb, cp, q2, v1, v2);
      o1 = o1 + v1;
      o2 = o2 + v2;
    }
  } else {
    __shared__ int queue[2][64];   // per warp of the 64-thread CTA
    int* qw = queue[threadIdx.x >> 5];
    int qn = 0;
    for (int base = 0; base < total; base += 32) {
      const int q2 = base + lane;
      bool big = false;
      if (q2 < total) {
        double v1, v2;
        gam2_item<true>(S, t, pa, pb, cp, q2, v1, v2);
        if (fabs(v1) > tau || fabs(v2) > tau || !(v1 == v1) || !(v2 == v2)) {
          big = true;
        } else {
          o1 = o1 + v1;
          o2 = o2 + v2;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, big);
      if (big) qw[qn + __popc(m & ((1u << lane) - 1u))] = q2;
      qn += __popc(m);
      __syncwarp();
      if (qn >= 32) {   // 32 queued items: one full-warp FP64 pass
        double v1, v2;
        gam2_item64(S, t, pa, pb, cp, qw[lane], v1, v2);
        o1 = o1 + v1;
        o2 = o2 + v2;
        __syncwarp();
        if (lane < qn - 32) qw[lane] = qw[lane + 32];
        __syncwarp();
        qn -= 32;
      }
    }
    if (lane < qn) {
      double v1, v2;
      gam2_item64(S, t, pa, pb, cp, qw[lane], v1, v2);
      o1 = o1 + v1;
      o2 = o2 + v2;
    }
  }
  o1 = warp_sum(o1);
  o2 = warp_sum(o2);
  if (!RX) o1 += separable_gam2(S, ic1, jc1, ic2, jc2, ip, jp, lane);
  if (lane == 0) {
    x1[w] = o1;
    x2[w] = o2;
  }
}

// In-place pair symmetrisation; the thread of the smaller packed index of
// each {12, 21} pair writes both elements.
__global__ void gam2_sym_kernel(int ne, int np, int rx, double* __restrict__ x1,
                                double* __restrict__ x2, long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    long long r = t;
    const int j2 = (int)(r % ne); r /= ne;
    const int i2 = (int)(r % ne); r /= ne;
    const int j1 = (int)(r % ne); r /= ne;
    const int i1 = (int)(r % ne); r /= ne;
    const long long pp = r;  // jp + np*ip
    const long long u = j1 + (long long)ne * (i1 + (long long)ne * (j2 + (long long)ne * (i2 + (long long)ne * pp)));
    if (u < t) continue;
    const double a2 = x2[t], b2 = x2[u];
    x2[t] = (a2 + b2) / 2.0;
    x2[u] = (b2 + a2) / 2.0;
    if (!rx) {
      const double a1 = x1[t], b1 = x1[u];
      x1[t] = (a1 + b1) / 2.0;
      x1[u] = (b1 + a1) / 2.0;
    }
  }
}

// ---- separable gam_3 factors (contracted, FP64) ---------------------------
// W1[ip][jp][i1][j1] = sum_prims c c c_p c_p' [sum_k b_k G2xggs(g_k,0)
//                       + 1/2 sum_kl b_k b_l G2xggs(g_k,g_l)]       (e1, p)
__global__ void gam3_w1_kernel(DevSystem S, double* __restrict__ W1) {
  const int ne = S.nebf, np = S.npbf;
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (w >= (long long)np * np * ne * ne) return;
  long long r = w;
  const int j1 = (int)(r % ne); r /= ne;
  const int i1 = (int)(r % ne); r /= ne;
  const int jp = (int)(r % np);
  const int ip = (int)(r / np);
  const int s1 = S.kpestr[i1], n1 = S.kpeend[i1] - s1 + 1;
  const int s2 = S.kpestr[j1], n2 = S.kpeend[j1] - s2 + 1;
  const Prim P1 = to_prim(S.pprim[ip]), P2 = to_prim(S.pprim[jp]);
  double o = 0.0;
  for (int q = lane; q < n1 * n2; q += 32) {
    const int a = s1 + q / n2, bq = s2 + q % n2;
    const Prim A = to_prim(S.eprim[a]), B = to_prim(S.eprim[bq]);
    double v = 0.0;
    for (int k = 0; k < S.ngtg; k++)
      v = v + S.bgem[k] * md::underflow(md::g2_xggs(A, P1, B, P2, S.ggem[k], 0.0));
    double v2 = 0.0;
    for (int k = 0; k < S.ngtg; k++)
      for (int l = 0; l < S.ngtg; l++)
        v2 = v2 + S.bgem[k] * S.bgem[l] *
                      md::underflow(md::g2_xggs(A, P1, B, P2, S.ggem[k], S.ggem[l]));
    o = o + (v + 0.5 * v2) * (S.eprim[a].coef * S.eprim[bq].coef *
                              S.pprim[ip].coef * S.pprim[jp].coef);
  }
  o = warp_sum(o);
  if (lane == 0) W1[w] = o;
}

// W3[ip][jp][i1][j1][i2][j2] = sum_prims c^6 sum_kl b_k b_l
//                              G3xggs(e1,e2,p; A13 = g_k, B23 = g_l)
__global__ void __launch_bounds__(64)
gam3_w3_kernel(DevSystem S, double* __restrict__ W3) {
  const int ne = S.nebf, np = S.npbf;
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (w >= (long long)np * np * ne * ne * ne * ne) return;
  long long r = w;
  int c[4];
  for (int k = 3; k >= 0; k--) {
    c[k] = (int)(r % ne);
    r /= ne;
  }
  const int jp = (int)(r % np);
  const int ip = (int)(r / np);
  int st0[4], cnt[4], nq = 1;
  for (int k = 0; k < 4; k++) {
    st0[k] = S.kpestr[c[k]];
    cnt[k] = S.kpeend[c[k]] - st0[k] + 1;
    nq *= cnt[k];
  }
  G3 st;
  double o = 0.0, g[6];
  for (int q = lane; q < nq; q += 32) {
    int qq = q, idx[4];
    for (int k = 3; k >= 0; k--) {
      idx[k] = st0[k] + qq % cnt[k];
      qq /= cnt[k];
    }
    const Prim A[3] = {to_prim(S.eprim[idx[0]]), to_prim(S.eprim[idx[2]]),
                       to_prim(S.pprim[ip])};
    const Prim B[3] = {to_prim(S.eprim[idx[1]]), to_prim(S.eprim[idx[3]]),
                       to_prim(S.pprim[jp])};
    md::Pair pr[3];
    for (int i = 0; i < 3; i++) md::gauss_pair(A[i], B[i], pr[i]);
    double v = 0.0;
    for (int k = 0; k < S.ngtg; k++)
      for (int l = 0; l < S.ngtg; l++) {
        gam6(g, A13, S.ggem[k], B23, S.ggem[l]);
        md::g3_setup_pairs(st, A, B, pr, g, 0);
        v = v + S.bgem[k] * S.bgem[l] * md::underflow(md::g3_overlap(st));
      }
    double cc = S.pprim[ip].coef * S.pprim[jp].coef;
    for (int k = 0; k < 4; k++) cc = cc * S.eprim[idx[k]].coef;
    o = o + v * cc;
  }
  o = warp_sum(o);
  if (lane == 0) W3[w] = o;
}

// Hcore[i][j] = sum_prims c c [T - sum_C Z V_C]  (xcalc_GAM3_MD's h(e3))
__global__ void gam3_hcore_kernel(DevSystem S, double* __restrict__ Hc) {
  const int ne = S.nebf;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ne * ne) return;
  const int i = t / ne, j = t - i * ne;
  double h = 0.0;
  for (int a = S.kpestr[i]; a <= S.kpeend[i]; a++)
    for (int bq = S.kpestr[j]; bq <= S.kpeend[j]; bq++) {
      const Prim A = to_prim(S.eprim[a]), B = to_prim(S.eprim[bq]);
      const double xke = md::gfke(A, B, 1.0);
      double Vc = 0.0;
      for (int ia = 0; ia < S.nat; ia++)
        Vc = Vc + (S.zan[ia] * md::gfvec(A, B, S.cat + 3 * ia));
      h = h + (xke + (Vc * -1.0)) * (S.eprim[a].coef * S.eprim[bq].coef);
    }
  Hc[t] = h;
}

// Six-permutation symmetrisation in place: each orbit is handled by the
// tuple with the largest packed index (the reference's last writer), which
// averages in its own permutation order and writes the whole orbit.
__global__ void gam3_sym_kernel(int ne, int np, double* __restrict__ g,
                                long long n) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    long long r = t;
    const int j3 = (int)(r % ne); r /= ne;
    const int i3 = (int)(r % ne); r /= ne;
    const int j2 = (int)(r % ne); r /= ne;
    const int i2 = (int)(r % ne); r /= ne;
    const int j1 = (int)(r % ne); r /= ne;
    const int i1 = (int)(r % ne); r /= ne;
    const long long pp = r;
    auto idx = [&](int a, int b, int c, int d, int e, int f) -> long long {
      return f + (long long)ne * (e + (long long)ne * (d + (long long)ne * (c +
             (long long)ne * (b + (long long)ne * (a + (long long)ne * pp)))));
    };
    const long long a132 = idx(i1, j1, i3, j3, i2, j2);
    const long long a213 = idx(i2, j2, i1, j1, i3, j3);
    const long long a231 = idx(i2, j2, i3, j3, i1, j1);
    const long long a312 = idx(i3, j3, i1, j1, i2, j2);
    const long long a321 = idx(i3, j3, i2, j2, i1, j1);
    if (a132 > t || a213 > t || a231 > t || a312 > t || a321 > t) continue;
    const double xx = (g[t] + g[a132] + g[a213] + g[a231] + g[a312] + g[a321]) / 6.0;
    g[t] = xx;
    g[a132] = xx;
    g[a213] = xx;
    g[a231] = xx;
    g[a312] = xx;
    g[a321] = xx;
  }
}

}  // namespace

cudaError_t launch_gam_ee(const DevSystem& sys, double* gee, cudaStream_t s) {
  const long long n4 = (long long)sys.nebf * sys.nebf * sys.nebf * sys.nebf;
  long long blocks = (n4 * 32 + 127) / 128;   // a warp per contracted quartet
  if (blocks > 152 * 64) blocks = 152 * 64;
  gam_ee_kernel<<<(unsigned)blocks, 128, 0, s>>>(sys, gee);
  return cudaGetLastError();
}

cudaError_t launch_gam2_raw_range(const DevSystem& sys, int rx, long long t0,
                                  long long ntup, double* x1, double* x2,
                                  cudaStream_t s, int fp32) {
  const long long threads = ntup * 32;
  const unsigned blocks = (unsigned)((threads + 63) / 64);
  if (ntup <= 0) return cudaSuccess;
  if (rx && fp32) return cudaErrorInvalidValue;   // FP32 path: XCHF gam_2 only
  const double tau = mixed_recompute_tau();
  // the builders keep their integral set-ups in local memory: prefer the
  // largest L1 share of the unified L1 / shared-memory array (a hint)
  if (rx) cudaFuncSetAttribute(gam2_raw_kernel<1, false>,
                               cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  else if (fp32) cudaFuncSetAttribute(gam2_raw_kernel<0, true>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  else cudaFuncSetAttribute(gam2_raw_kernel<0, false>,
                            cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  if (rx) gam2_raw_kernel<1, false><<<blocks, 64, 0, s>>>(sys, x1, x2, t0, ntup, tau);
  else if (fp32) gam2_raw_kernel<0, true><<<blocks, 64, 0, s>>>(sys, x1, x2, t0, ntup, tau);
  else gam2_raw_kernel<0, false><<<blocks, 64, 0, s>>>(sys, x1, x2, t0, ntup, tau);
  return cudaGetLastError();
}

namespace {
std::atomic<double> g_tau_gam2{kMixedTauGam2};
}
void set_mixed_recompute_tau(double tau) { g_tau_gam2.store(tau); }
double mixed_recompute_tau() { return g_tau_gam2.load(); }

cudaError_t launch_gam2_raw(const DevSystem& sys, int rx, double* x1,
                            double* x2, cudaStream_t s, int fp32) {
  const long long ntup = (long long)sys.nebf * sys.nebf * sys.nebf * sys.nebf *
                         sys.npbf * sys.npbf;
  return launch_gam2_raw_range(sys, rx, 0, ntup, x1, x2, s, fp32);
}

cudaError_t launch_gam2_symmetrize(int ne, int np, int rx, double* x1,
                                   double* x2, cudaStream_t s) {
  const long long n = (long long)ne * ne * ne * ne * np * np;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  gam2_sym_kernel<<<(unsigned)blocks, 256, 0, s>>>(ne, np, rx, x1, x2, n);
  return cudaGetLastError();
}

cudaError_t launch_gam3_aux(const DevSystem& sys, double* aux, cudaStream_t s,
                            const double* gee_in, const double* hc_in) {
  const int ne = sys.nebf, np = sys.npbf;
  const long long n2 = (long long)ne * ne, n4 = n2 * n2;
  double* gee = aux;
  double* hc = gee + n4;
  double* W1 = hc + n2;
  double* W3 = W1 + (long long)np * np * n2;
  cudaError_t e = gee_in ? cudaMemcpyAsync(gee, gee_in, sizeof(double) * n4,
                                           cudaMemcpyDeviceToDevice, s)
                         : launch_gam_ee(sys, gee, s);
  if (e != cudaSuccess) return e;
  if (hc_in)
    e = cudaMemcpyAsync(hc, hc_in, sizeof(double) * n2, cudaMemcpyDeviceToDevice, s);
  else
    gam3_hcore_kernel<<<(unsigned)((n2 + 127) / 128), 128, 0, s>>>(sys, hc);
  if (e != cudaSuccess) return e;
  const long long w1 = (long long)np * np * n2, w3 = w1 * n2;
  gam3_w1_kernel<<<(unsigned)((w1 * 32 + 127) / 128), 128, 0, s>>>(sys, W1);
  gam3_w3_kernel<<<(unsigned)((w3 * 32 + 63) / 64), 64, 0, s>>>(sys, W3);
  return cudaGetLastError();
}

cudaError_t launch_gam3_symmetrize(int ne, int np, double* g3,
                                   cudaStream_t s) {
  const long long n = (long long)ne * ne * ne * ne * ne * ne * np * np;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  gam3_sym_kernel<<<(unsigned)blocks, 256, 0, s>>>(ne, np, g3, n);
  return cudaGetLastError();
}

}  // namespace neoxc
