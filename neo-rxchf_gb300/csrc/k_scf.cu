// k_scf.cu -- device side of the XCHF RHF SCF (xchf1_independent/xcscf.f,
// xchf1_fock.f) for sm_103a: the one- and two-particle integrals besides
// gam_2/3/4, the Fock/energy assembly, ROOTHAN with a block-parallel Jacobi
// eigensolver, and the density-change check.  Every kernel takes device
// pointers; energies and convergence scalars live in a device array so an
// SCF iteration needs no host round trip except the final 3-scalar read.
//
// Device energy slots (en[]):
//   0 E_total 1 E_nuc 2 E_ecore 3 E_pcore 4 E_ep 5 E_ee 6 E_gam1 7 E_gam2
//   8 E_gam3 9 E_gam4 10 S_total 11 S_gam1 12 S_gam2 13 H_expect
//   14 max|DE-DE0| 15 max|DP-DP0|
// Matrices (DE, DP, focke, fockp, se*, sp*, S, X) are column-major like the
// reference's Fortran arrays; the core matrices keep pack_2D order
// ([i][j] = GAM_ecore(pack_2D(n,j,i))) and GAM_ep / GAM_1 / GAM_1s keep
// pack_4D(nebf,nebf,npbf, je,ie,jp,ip) order, i.e. C-order [ip][jp][ie][je].
#include <type_traits>

#include "md_math.cuh"
#include "md_math32.cuh"
#include "neoxc_internal.h"

namespace neoxc {
namespace {

using md::Prim;

__device__ __forceinline__ Prim to_prim(const DevPrim& p) {
  Prim r;
  r.a = p.a;
  for (int d = 0; d < 3; d++) {
    r.c[d] = p.c[d];
    r.l[d] = p.l[d];
  }
  return r;
}

__device__ __forceinline__ double gfovlap(const Prim& A, const Prim& B) {
  double s = 1.0;
  for (int d = 0; d < 3; d++) s *= md::ovl1d(A.l[d], A.a, A.c[d], B.l[d], B.a, B.c[d]);
  return s;
}

// gam_epcore.f:200-270 xcalc_GAM_epcore
__device__ __noinline__ double xcalc_epcore(const Prim& A, const Prim& B,
                                            const DevSystem& S, double xmass,
                                            double coul_sign) {
  const double ke = md::gfke(A, B, xmass);
  double v = 0.0;
  for (int k = 0; k < S.nat; k++) {
    const double C[3] = {S.cat[3 * k], S.cat[3 * k + 1], S.cat[3 * k + 2]};
    v = v + coul_sign * S.zan[k] * md::gfvec(A, B, C);
  }
  return ke + v;
}

// ---- overlaps and core Hamiltonians (pure_ovlap.f, gam_epcore.f) ----------
// t < ne^2: electronic pair (i,j); then np^2 nuclear pairs.  Sums over the
// primitive pairs in the reference's order (bra primitive outer).
__global__ void onebody_kernel(DevSystem S, double* __restrict__ Se,
                               double* __restrict__ Sp, double* __restrict__ Hce,
                               double* __restrict__ Hcp) {
  const int ne = S.nebf, np = S.npbf;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ne * ne) {
    const int i = t / ne, j = t - i * ne;
    double so = 0.0, h = 0.0;
    for (int a = S.kpestr[i]; a <= S.kpeend[i]; a++)
      for (int b = S.kpestr[j]; b <= S.kpeend[j]; b++) {
        const Prim A = to_prim(S.eprim[a]), B = to_prim(S.eprim[b]);
        const double c = S.eprim[a].coef, d = S.eprim[b].coef;
        so = so + gfovlap(A, B) * c * d;
        h = h + xcalc_epcore(A, B, S, 1.0, -1.0) * c * d;
      }
    Se[i * ne + j] = so;   // pack_2D(ne, j, i) order; symmetric
    Hce[i * ne + j] = h;
  } else if (t < ne * ne + np * np) {
    const int k = t - ne * ne, p = k / np, q = k - p * np;
    const Prim A = to_prim(S.pprim[p]), B = to_prim(S.pprim[q]);
    const double c = S.pprim[p].coef, d = S.pprim[q].coef;
    Sp[p * np + q] = gfovlap(A, B) * c * d;
    Hcp[p * np + q] = xcalc_epcore(A, B, S, S.pmass, 1.0) * c * d;
  }
}

// ---- GAM_ep (gam_ep.f:2-219): -(e p | e' p'), C-order [ip][jp][ie][je] ----
__global__ void gam_ep_kernel(DevSystem S, double* __restrict__ Gep) {
  const int ne = S.nebf, np = S.npbf;
  const int total = np * np * ne * ne;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int r = t;
  const int je = r % ne; r /= ne;
  const int ie = r % ne; r /= ne;
  const int jp = r % np; r /= np;
  const int ip = r;
  const Prim P1 = to_prim(S.pprim[ip]), P2 = to_prim(S.pprim[jp]);
  const double cp = S.pprim[ip].coef, cq = S.pprim[jp].coef;
  double acc = 0.0;
  for (int a = S.kpestr[ie]; a <= S.kpeend[ie]; a++)
    for (int b = S.kpestr[je]; b <= S.kpeend[je]; b++) {
      const double v = -md::gfvee(to_prim(S.eprim[a]), P1, to_prim(S.eprim[b]), P2);
      acc = acc + v * cp * cq * S.eprim[a].coef * S.eprim[b].coef;
    }
  Gep[t] = acc;
}

// ---- gam_1 (gam_1_OMP.f:398-836 xcalc_GAM1_MD) -----------------------------
// A = (e, p), B = (e', p'); one geminal work item of the reference's
// result (gi < ng: the single-geminal terms of k = gi; else the pair
// (k, l)): ansE = TE + TP - VCE + VCP - VMX and ansS = 2 OGX + OGG are
// linear in these items, so the lanes of a warp share them.  P is md::Prim
// (FP64) or md32::Prim (FP32 integrals, mixed path); the integral calls
// resolve by argument-dependent lookup and every geminal/atom sum is FP64.
template <class P>
__device__ __noinline__ void xcalc_gam1_item(const P* A, const P* B, const DevSystem& S,
                                             int gi, double* ansE, double* ansS) {
  using R = typename std::remove_cv<decltype(P::a)>::type;
  const R zero = R(0.0), one = R(1.0), pmass = (R)S.pmass;
  const int ng = S.ngtg;
  if (gi < ng) {
    const R GV = (R)S.ggem[gi];
    const double BV = S.bgem[gi];
    const double tegx = BV * (double)pgike1(A[0], A[1], B[0], B[1], GV, zero, one);
    const double tpgx = BV * (double)pgike1(A[1], A[0], B[1], B[0], GV, zero, pmass);
    double ve = 0.0, vp = 0.0;
    for (int c = 0; c < S.nat; c++) {
      const R C[3] = {(R)S.cat[3 * c], (R)S.cat[3 * c + 1], (R)S.cat[3 * c + 2]};
      ve = (double)g2_xggvec(A[0], A[1], B[0], B[1], GV, zero, C) * S.zan[c] + ve;
      vp = (double)g2_xggvec(A[1], A[0], B[1], B[0], GV, zero, C) * S.zan[c] + vp;
    }
    const double vm = (double)g2_xggvee(A[0], A[1], B[0], B[1], GV, zero);
    const double texg = BV * (double)pgike1(A[0], A[1], B[0], B[1], zero, GV, one);
    const double tpxg = BV * (double)pgike1(A[1], A[0], B[1], B[0], zero, GV, pmass);
    // TE + TP - 2 VCEGX + 2 VCPGX - 2 VMGX (this k's share)
    *ansE = (tegx + texg) + (tpgx + tpxg) - 2.0 * (BV * ve) + 2.0 * (BV * vp) -
            2.0 * (BV * vm);
    *ansS = 2.0 * (BV * (double)g2_xggs(A[0], A[1], B[0], B[1], GV, zero));
    return;
  }
  const int k = (gi - ng) / ng, l = (gi - ng) - k * ng;
  const R GV = (R)S.ggem[k], GW = (R)S.ggem[l];
  const double BB = S.bgem[k] * S.bgem[l];
  const double tegg = BB * (double)pgike1(A[0], A[1], B[0], B[1], GV, GW, one);
  const double tpgg = BB * (double)pgike1(A[1], A[0], B[1], B[0], GV, GW, pmass);
  double vee = 0.0, vpp = 0.0;
  for (int c = 0; c < S.nat; c++) {
    const R C[3] = {(R)S.cat[3 * c], (R)S.cat[3 * c + 1], (R)S.cat[3 * c + 2]};
    vee = (double)g2_xggvec(A[0], A[1], B[0], B[1], GV, GW, C) * S.zan[c] + vee;
    vpp = (double)g2_xggvec(A[1], A[0], B[1], B[0], GV, GW, C) * S.zan[c] + vpp;
  }
  const double vmm = (double)g2_xggvee(A[0], A[1], B[0], B[1], GV, GW);
  *ansE = tegg + tpgg - BB * vee + BB * vpp - BB * vmm;
  *ansS = BB * (double)g2_xggs(A[0], A[1], B[0], B[1], GV, GW);
}

__device__ __forceinline__ md32::Prim to_prim32(const DevPrim& p) {
  md32::Prim r;
  r.a = (float)p.a;
  for (int d = 0; d < 3; d++) {
    r.c[d] = (float)p.c[d];
    r.l[d] = p.l[d];
  }
  return r;
}

// One warp per contracted (ip, jp, ie, je); lanes take primitive pairs and
// the warp sums them in a fixed shuffle order (deterministic).
template <bool F32>
__global__ void gam1_kernel(DevSystem S, double* __restrict__ G1,
                            double* __restrict__ G1s, int pairs_only) {
  const int ne = S.nebf, np = S.npbf;
  const int total = np * np * ne * ne;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (w >= total) return;
  int r = w;
  const int je = r % ne; r /= ne;
  const int ie = r % ne; r /= ne;
  const int jp = r % np; r /= np;
  const int ip = r;
  const int na = S.kpeend[ie] - S.kpestr[ie] + 1;
  const int nb = S.kpeend[je] - S.kpestr[je] + 1;
  const int nq = na * nb, ng = S.ngtg;
  const int g0 = pairs_only ? ng : 0, nit = pairs_only ? ng * ng : ng + ng * ng;
  double e = 0.0, sv = 0.0;
  // lanes take (geminal item, primitive pair), the pair fastest
  for (int q2 = lane; q2 < nq * nit; q2 += 32) {
    const int gq = q2 / nq, k = q2 - gq * nq, gi = g0 + gq;
    const int a = S.kpestr[ie] + k / nb, b = S.kpestr[je] + k % nb;
    double aE, aS;
    if constexpr (F32) {
      md32::Prim A[2] = {to_prim32(S.eprim[a]), to_prim32(S.pprim[ip])};
      md32::Prim B[2] = {to_prim32(S.eprim[b]), to_prim32(S.pprim[jp])};
      xcalc_gam1_item(A, B, S, gi, &aE, &aS);
    } else {
      Prim A[2] = {to_prim(S.eprim[a]), to_prim(S.pprim[ip])};
      Prim B[2] = {to_prim(S.eprim[b]), to_prim(S.pprim[jp])};
      xcalc_gam1_item(A, B, S, gi, &aE, &aS);
    }
    const double cip = S.pprim[ip].coef, cjp = S.pprim[jp].coef;
    const double cie = S.eprim[a].coef, cje = S.eprim[b].coef;
    e = e + aE * cip * cjp * cie * cje;
    sv = sv + aS * cip * cjp * cie * cje;
  }
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, o);
    sv += __shfl_down_sync(0xffffffffu, sv, o);
  }
  if (lane == 0) {
    G1[w] = e;
    G1s[w] = sv;
  }
}

// ---- one-body part of xchf1_fock (E_from_GAM_ecore/pcore/ep/ee/1, S_from_GAM_1s)
// t < ne^2 : electronic (i,j);  ne^2 <= t < ne^2+np^2 : nuclear (p,q).
// part[c*nt + t]: c = 0 E_ecore, 1 E_pcore, 2 E_ep, 3 E_ee, 4 E_gam1, 5 S_gam1.
// xfocke / xfockp (optional): the NEO-HF part without GAM_1 (xchf1_fock.f's
// Xfocke / Xfockp, :218-219).
__global__ void fock1_kernel(int ne, int np, int nelec,
                             const double* __restrict__ Hce,
                             const double* __restrict__ Hcp,
                             const double* __restrict__ Gep,
                             const double* __restrict__ G1,
                             const double* __restrict__ G1s,
                             const double* __restrict__ Gee,
                             const double* __restrict__ DE,
                             const double* __restrict__ DP,
                             double* __restrict__ focke, double* __restrict__ fockp,
                             double* __restrict__ se1, double* __restrict__ sp1,
                             double* __restrict__ part,
                             double* __restrict__ xfocke,
                             double* __restrict__ xfockp) {
  const int nt = ne * ne + np * np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int n2 = ne * ne;
  double e[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (t < n2) {
    const int i = t / ne, j = t - i * ne;
    const double fc = Hce[i * ne + j];
    double fep = 0.0, fg1 = 0.0, s1 = 0.0;
    for (int p = 0; p < np; p++)
      for (int q = 0; q < np; q++) {
        const double dp = DP[p + np * q];
        const long long o = ((long long)(p * np + q) * ne + i) * ne + j;
        fep = fep + dp * Gep[o];
        fg1 = fg1 + dp * G1[o];
        s1 = s1 + dp * G1s[o];
      }
    double fee = 0.0;
    if (nelec > 1) {
      for (int k = 0; k < ne; k++)
        for (int l = 0; l < ne; l++) {
          const double v1 = Gee[(((long long)i * ne + j) * ne + k) * ne + l];
          const double v2 = Gee[(((long long)i * ne + l) * ne + k) * ne + j];
          fee = fee + 2.0 * DE[k + ne * l] * ((v1 - 0.5 * v2) * 0.5);
        }
    }
    focke[i + ne * j] = fc + fep + fee + fg1;
    if (xfocke) xfocke[i + ne * j] = fc + fep + fee;
    se1[i + ne * j] = s1;
    const double d = DE[i + ne * j];
    e[0] = d * fc;
    e[2] = d * fep;
    e[3] = d * (0.5 * fee);
    e[4] = d * fg1;
    e[5] = d * s1;
  } else {
    const int k = t - n2, p = k / np, q = k - p * np;
    const double fc = Hcp[p * np + q];
    double fep = 0.0, fg1 = 0.0, s1 = 0.0;
    for (int i = 0; i < ne; i++)
      for (int j = 0; j < ne; j++) {
        const double de = DE[i + ne * j];
        const long long o = ((long long)(p * np + q) * ne + i) * ne + j;
        fep = fep + de * Gep[o];
        fg1 = fg1 + de * G1[o];
        s1 = s1 + de * G1s[o];
      }
    fockp[p + np * q] = fc + fep + fg1;
    if (xfockp) xfockp[p + np * q] = fc + fep;
    sp1[p + np * q] = s1;
    e[1] = DP[p + np * q] * fc;
  }
  for (int c = 0; c < 6; c++) part[(long long)c * nt + t] = e[c];
}

__device__ double block_sum(double v, double* sw) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sw[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r += sw[k];
  return r;   // every thread gets the same value
}

// en[2..6], en[11] from the partials; the later slots (gam_2..4) are zeroed
// here and filled by their contractions when the electron count has them.
__global__ void fock1_energy_kernel(int nt, const double* __restrict__ part,
                                    double* __restrict__ en) {
  __shared__ double sw[32];
  const int slot[6] = {2, 3, 4, 5, 6, 11};
  for (int c = 0; c < 6; c++) {
    double v = 0.0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) v += part[(long long)c * nt + t];
    const double s = block_sum(v, sw);
    if (threadIdx.x == 0) en[slot[c]] = s;
    __syncthreads();
  }
  if (threadIdx.x == 0) en[7] = en[8] = en[9] = en[12] = 0.0;
}

// S_total, E_total, H_expect (xchf1_fock.f:311-319) and XCfock_correction
// (:728-783), from the device energy slots.
__global__ void assemble_kernel(int ne, int np, double* __restrict__ en,
                                const double* __restrict__ se1,
                                const double* __restrict__ sp1,
                                const double* __restrict__ se2,
                                const double* __restrict__ sp2,
                                double* __restrict__ focke,
                                double* __restrict__ fockp) {
  __shared__ double sS, sH;
  if (threadIdx.x == 0) {
    const double S_total = 1.0 + en[11] + en[12];
    const double psi = (en[2] + en[3] + en[4] + en[5] + en[6] + en[7] + en[8] + en[9]) / S_total;
    en[0] = psi + en[1];
    en[10] = S_total;
    en[13] = psi / S_total;
    sS = S_total;
    sH = psi / S_total;
  }
  __syncthreads();
  const double one = 1.0, two = 2.0, S = sS, H = sH;
  for (int k = threadIdx.x; k < ne * ne; k += blockDim.x)
    focke[k] = (one / S) * focke[k] - H * (se1[k] + two * se2[k]);
  for (int k = threadIdx.x; k < np * np; k += blockDim.x)
    fockp[k] = (one / S) * fockp[k] - H * (sp1[k] + sp2[k]);
}

// ---- XCUHF (xcuhf/xcuhf_fock.f UHF_FOCK) ----------------------------------
// One-body and HF terms of IC_construct_FAE / IC_construct_FP for both spins
// (xcuhf_hfterms.f FAE_ecore, FAE_GAMep, FAE_GAMee; xcuhf_omg1.f FAE_OMG1;
// FP_pcore, FP_GAMep, UFP_OMG1).  t < ne^2: electron (i,j) of both spins;
// then proton (p,q).  Energy channels (as fock1_kernel, so
// fock1_energy_kernel files them into en[2..6], en[11]):
//   0 E_AE_ecore + E_BE_ecore, 1 E_P_pcore, 2 E_P_GAMep,
//   3 E_AE_GAMee + E_BE_GAMee, 4 E_P_OMG1, 5 S_P_OMG1.
__global__ void uhf_fock1_kernel(int ne, int np, const double* __restrict__ Hce,
                                 const double* __restrict__ Hcp,
                                 const double* __restrict__ Gep,
                                 const double* __restrict__ G1,
                                 const double* __restrict__ G1s,
                                 const double* __restrict__ Gee,
                                 const double* __restrict__ DAE,
                                 const double* __restrict__ DBE,
                                 const double* __restrict__ DP,
                                 double* __restrict__ FAE, double* __restrict__ FBE,
                                 double* __restrict__ FP, double* __restrict__ SAE1,
                                 double* __restrict__ SBE1, double* __restrict__ SP1,
                                 double* __restrict__ part) {
  const int nt = ne * ne + np * np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int n2 = ne * ne;
  double e[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (t < n2) {
    const int i = t / ne, j = t - i * ne;
    const double fc = Hce[i * ne + j];   // GAM_ecore(pack_2D(ne,je,ie))
    double fep = 0.0, fg1 = 0.0, s1 = 0.0;
    for (int p = 0; p < np; p++)
      for (int q = 0; q < np; q++) {
        const double dp = DP[p + np * q];
        const long long o = ((long long)(p * np + q) * ne + i) * ne + j;
        fep = fep + dp * Gep[o];
        fg1 = fg1 + dp * G1[o];
        s1 = s1 + dp * G1s[o];
      }
    // FAE_GAMee: DETOT (i j|k l) - D_spin (i l|k j)
    double J = 0.0, KA = 0.0, KB = 0.0;
    for (int k = 0; k < ne; k++)
      for (int l = 0; l < ne; l++) {
        const double v12 = Gee[(((long long)i * ne + j) * ne + k) * ne + l];
        const double v21 = Gee[(((long long)i * ne + l) * ne + k) * ne + j];
        const double da = DAE[k + ne * l], db = DBE[k + ne * l];
        J = J + (da + db) * v12;
        KA = KA + da * v21;
        KB = KB + db * v21;
      }
    const int c = i + ne * j;
    FAE[c] = fc + fep + (J - KA) + fg1;
    FBE[c] = fc + fep + (J - KB) + fg1;
    SAE1[c] = s1;
    SBE1[c] = s1;
    const double da = DAE[c], db = DBE[c];
    e[0] = (da + db) * fc;
    e[3] = 0.5 * (da * (J - KA) + db * (J - KB));
  } else {
    const int k = t - n2, p = k / np, q = k - p * np;
    const double fc = Hcp[p * np + q];
    double fep = 0.0, fg1 = 0.0, s1 = 0.0;
    for (int i = 0; i < ne; i++)
      for (int j = 0; j < ne; j++) {
        const double dt = DAE[i + ne * j] + DBE[i + ne * j];
        const long long o = ((long long)(p * np + q) * ne + i) * ne + j;
        fep = fep + dt * Gep[o];
        fg1 = fg1 + dt * G1[o];
        s1 = s1 + dt * G1s[o];
      }
    const int c = p + np * q;
    FP[c] = fc + fep + fg1;
    SP1[c] = s1;
    const double dp = DP[c];
    e[1] = dp * fc;
    e[2] = dp * fep;
    e[4] = dp * fg1;
    e[5] = dp * s1;
  }
  for (int c = 0; c < 6; c++) part[(long long)c * nt + t] = e[c];
}

// UHF_FOCK tail (xcuhf_fock.f:318-371) and UHF_Fock_correction (:742-780):
// S_total = 1 + S_OMG1 + S_OMG2, Psi_H_Psi = the raw components, printed
// components divided by S_total, F = XF / S_total - Psi_H_Psi / S_total^2
// (XS1 + XS2) for FP, FAE, FBE.
__global__ void uhf_assemble_kernel(int ne, int np, double* __restrict__ en,
                                    const double* __restrict__ sae1,
                                    const double* __restrict__ sbe1,
                                    const double* __restrict__ sp1,
                                    const double* __restrict__ sae2,
                                    const double* __restrict__ sbe2,
                                    const double* __restrict__ sp2,
                                    double* __restrict__ FAE, double* __restrict__ FBE,
                                    double* __restrict__ FP) {
  __shared__ double sS, sPsi;
  __syncthreads();
  if (threadIdx.x == 0) {
    const double S_total = 1.0 + en[11] + en[12];
    const double psi = en[3] + en[2] + en[5] + en[4] + en[6] + en[7] + en[8] + en[9];
    for (int k = 2; k <= 9; k++) en[k] = en[k] / S_total;
    en[0] = (en[3] + en[2] + en[4] + en[5]) + en[6] + en[7] + en[8] + en[9] + en[1];
    en[10] = S_total;
    sS = S_total;
    sPsi = psi;
  }
  __syncthreads();
  const double c1 = 1.0 / sS, c2 = sPsi / (sS * sS);
  for (int k = threadIdx.x; k < np * np; k += blockDim.x)
    FP[k] = c1 * FP[k] - c2 * (sp1[k] + sp2[k]);
  for (int k = threadIdx.x; k < ne * ne; k += blockDim.x) {
    FAE[k] = c1 * FAE[k] - c2 * (sae1[k] + sae2[k]);
    FBE[k] = c1 * FBE[k] - c2 * (sbe1[k] + sbe2[k]);
  }
}

// DENDIF + COPYDEN for alpha, beta and the proton (xcuhf_scf.f:512-523):
// en[13], en[14], en[15].
__global__ void uhf_dendif_kernel(int ne, int np, const double* __restrict__ DA,
                                  double* __restrict__ DA0, const double* __restrict__ DB,
                                  double* __restrict__ DB0, const double* __restrict__ DP,
                                  double* __restrict__ DP0, double* __restrict__ en) {
  __shared__ double sw[32];
  for (int which = 0; which < 3; which++) {
    const int n = which == 2 ? np : ne;
    const double* D = which == 0 ? DA : (which == 1 ? DB : DP);
    double* D0 = which == 0 ? DA0 : (which == 1 ? DB0 : DP0);
    double mx = 0.0;
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
      mx = fmax(mx, fabs(D0[k] - D[k]));
      D0[k] = D[k];
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sw[w] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0;
      for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r = fmax(r, sw[k]);
      en[13 + which] = r;
    }
    __syncthreads();
  }
}

// ---- symmetric eigensolver: cyclic Jacobi with round-robin pairing ------------
// A (row-major n x n, symmetric) and V in shared memory; on return A is
// diagonal to working precision and V holds the eigenvectors as columns.
// Sweeps are bounded; *sweeps_out = sweeps used (kJacobiMaxSweeps + 1 when
// the off-diagonal norm did not converge).
constexpr int kJacobiMaxSweeps = 40;

__device__ int jacobi_eig(int n, double* A, double* V, double* rc, double* rs,
                          int* rp, int* rq, double* sw) {
  const int m = (n + 1) & ~1;   // pad to even with a dummy index n
  for (int k = threadIdx.x; k < n * n; k += blockDim.x)
    V[k] = (k / n == k % n) ? 1.0 : 0.0;
  __syncthreads();
  int sweep = 0;
  double prev_off = 0.0;
  for (; sweep < kJacobiMaxSweeps; sweep++) {
    // convergence: off-diagonal vs diagonal squared norms
    double off = 0.0, dia = 0.0;
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
      const double a = A[k];
      if (k / n == k % n) dia += a * a;
      else off += a * a;
    }
    off = block_sum(off, sw);
    __syncthreads();
    dia = block_sum(dia, sw);
    __syncthreads();
    if (!(off == off) || !(dia == dia)) return kJacobiMaxSweeps + 2;   // NaN input
    if (off <= 1e-30 * dia || off == 0.0) break;
    // at the rounding floor (n^2 eps^2 of the diagonal mass can exceed
    // 1e-30 for n >= 5 when the eigenvalues span several decades) a sweep
    // no longer shrinks the off-diagonal mass: stop there once it is below
    // 1e-24 of the diagonal (off-diagonal norm 1e-12 relative)
    if (sweep > 0 && off <= 1e-24 * dia && off >= 0.25 * prev_off) break;
    if (sweep >= 8 && off <= 1e-24 * dia) break;
    prev_off = off;
    for (int step = 0; step < m - 1; step++) {
      // round robin: slot 0 fixed, the other m-1 rotate
      for (int k = threadIdx.x; k < m / 2; k += blockDim.x) {
        const int a = (k == 0) ? 0 : 1 + (k - 1 + step) % (m - 1);
        const int b = 1 + (m - 2 - k + step) % (m - 1);
        int p = a < b ? a : b, q = a < b ? b : a;
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p * n + q];
          if (apq != 0.0) {
            const double th = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
            const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
          }
        } else {
          p = q = -1;   // pair with the dummy index: no rotation
        }
        rp[k] = p;
        rq[k] = q;
        rc[k] = c;
        rs[k] = s;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int e = threadIdx.x; e < (m / 2) * n; e += blockDim.x) {
        const int k = e / n, j = e - k * n, p = rp[k], q = rq[k];
        if (p < 0) continue;
        const double c = rc[k], s = rs[k];
        const double apj = A[p * n + j], aqj = A[q * n + j];
        A[p * n + j] = c * apj - s * aqj;
        A[q * n + j] = s * apj + c * aqj;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int e = threadIdx.x; e < (m / 2) * n; e += blockDim.x) {
        const int k = e / n, i = e - k * n, p = rp[k], q = rq[k];
        if (p < 0) continue;
        const double c = rc[k], s = rs[k];
        const double aip = A[i * n + p], aiq = A[i * n + q];
        A[i * n + p] = c * aip - s * aiq;
        A[i * n + q] = s * aip + c * aiq;
        const double vip = V[i * n + p], viq = V[i * n + q];
        V[i * n + p] = c * vip - s * viq;
        V[i * n + q] = s * vip + c * viq;
      }
      __syncthreads();
    }
  }
  return sweep < kJacobiMaxSweeps ? sweep : kJacobiMaxSweeps + 1;
}

struct EigSmem {
  double *A, *V, *T, *rc, *rs, *sw;
  int *rp, *rq, *rank;
};
__device__ EigSmem carve(int n, double* base) {
  EigSmem m;
  m.A = base;
  m.V = m.A + n * n;
  m.T = m.V + n * n;
  m.rc = m.T + n * n;
  m.rs = m.rc + 64;
  m.sw = m.rs + 64;
  m.rp = (int*)(m.sw + 32);
  m.rq = m.rp + 64;
  m.rank = m.rq + 64;
  return m;
}
size_t eig_smem_bytes(int n) {
  return sizeof(double) * (3 * (size_t)n * n + 64 + 64 + 32) + sizeof(int) * (64 * 3);
}

// X = S^{-1/2} = U diag(1/sqrt(w)) U^T (xcscf.f:766-838 in ROOTHAN).
// S, X column-major (symmetric).  status[0] = Jacobi sweeps (> max: failed).
__global__ void inv_sqrt_kernel(int n, const double* __restrict__ S,
                                double* __restrict__ X, int* status) {
  extern __shared__ double smem[];
  EigSmem m = carve(n, smem);
  // RS reads the lower triangle: use it for both halves
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    m.A[k] = i >= j ? S[i + n * j] : S[j + n * i];
  }
  __syncthreads();
  const int sw = jacobi_eig(n, m.A, m.V, m.rc, m.rs, m.rp, m.rq, m.sw);
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    double acc = 0.0;
    for (int l = 0; l < n; l++)
      acc += m.V[i * n + l] * (1.0 / sqrt(m.A[l * n + l])) * m.V[j * n + l];
    X[i + n * j] = acc;
  }
  if (threadIdx.x == 0) status[0] = sw;
}

// ROOTHAN (xcscf.f:766-953): F' = X^T F X, eigenvectors V (ascending
// eigenvalues), C = X V, D = prefac sum_{k=first}^{first+nocc-1} C_k C_k^T.
// evals[n] (ascending) and C (column-major, sorted) written when non-null.
__global__ void roothan_kernel(int n, const double* __restrict__ F,
                               const double* __restrict__ X, int first, int nocc,
                               double prefac, double* __restrict__ D,
                               double* __restrict__ evals,
                               double* __restrict__ Cout, int* status,
                               const int* __restrict__ skip) {
  if (skip && *skip) return;   // a second-order step already gave D (soscf_kernel)
  extern __shared__ double smem[];
  EigSmem m = carve(n, smem);
  // T = F X  (row-major T[i][j])
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    double acc = 0.0;
    for (int l = 0; l < n; l++) acc += F[i + n * l] * X[l + n * j];
    m.T[k] = acc;
  }
  __syncthreads();
  // A = X^T T, lower triangle mirrored (RS reads the lower triangle)
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    const int r = i >= j ? i : j, c = i >= j ? j : i;
    double acc = 0.0;
    for (int l = 0; l < n; l++) acc += X[l + n * r] * m.T[l * n + c];
    m.A[k] = acc;
  }
  __syncthreads();
  const int sw = jacobi_eig(n, m.A, m.V, m.rc, m.rs, m.rp, m.rq, m.sw);
  // ascending order: rank of each eigenvalue (ties by index).  The order is
  // total even for NaN eigenvalues (a NaN Fock matrix, reported through
  // status): NaNs sort last, among themselves by index, so the ranks are a
  // permutation and every rank slot is written.
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double w = m.A[i * n + i];
    const bool wn = isnan(w);
    int r = 0;
    for (int j = 0; j < n; j++) {
      const double v = m.A[j * n + j];
      const bool vn = isnan(v);
      r += (vn || wn) ? ((!vn && wn) || (vn && wn && j < i))
                      : ((v < w) || (v == w && j < i));
    }
    m.rank[r < n ? r : n - 1] = i;   // rank -> eigen index
  }
  __syncthreads();
  // C = X V in sorted order (T reused, row-major T[i][k])
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, k = e - i * n;
    const int col = min(max(m.rank[k], 0), n - 1);
    double acc = 0.0;
    for (int l = 0; l < n; l++) acc += X[i + n * l] * m.V[l * n + col];
    m.T[e] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    double acc = 0.0;
    for (int k = first; k < first + nocc; k++) acc += prefac * m.T[i * n + k] * m.T[j * n + k];
    D[i + n * j] = acc;
    if (Cout) Cout[i + n * j] = m.T[e];
  }
  if (evals)
    for (int k = threadIdx.x; k < n; k += blockDim.x)
      evals[k] = m.A[min(max(m.rank[k], 0), n - 1) * (n + 1)];
  if (threadIdx.x == 0) status[0] = sw;
}

// DENDIF + COPYDEN (xcscf.f:719-764) for both particles: en[14], en[15].
__global__ void dendif_kernel(int ne, int np, const double* __restrict__ DE,
                              double* __restrict__ DE0,
                              const double* __restrict__ DP,
                              double* __restrict__ DP0, double* __restrict__ en) {
  __shared__ double sw[32];
  for (int which = 0; which < 2; which++) {
    const int n = which ? np : ne;
    const double* D = which ? DP : DE;
    double* D0 = which ? DP0 : DE0;
    double mx = 0.0;
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
      mx = fmax(mx, fabs(D0[k] - D[k]));
      D0[k] = D[k];
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sw[w] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0;
      for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r = fmax(r, sw[k]);
      en[14 + which] = r;
    }
    __syncthreads();
  }
}

// ---- DIIS (Pulay) extrapolation of the electronic Fock matrix ------------------
// Not in the reference (xcscf.f iterates plain Roothaan or SOSCF).  One CTA:
// error e = F D S - S D F (= M - M^T with M = F D S for symmetric F, D, S),
// stored with F in a ring of kDiisMax slots; B_ij = <e_i, e_j>; the Pulay
// system [B -1; -1 0][c; l] = [0; -1] is solved by Gaussian elimination with
// partial pivoting; F <- sum_i c_i F_i.  state[0] = vectors held, state[1] =
// next slot.  With fewer than two vectors, or a singular system, F is left
// unchanged.  err_out (optional) receives max|e|.
constexpr int kDiisMax = 8;

__global__ void diis_kernel(int n, double* __restrict__ F,
                            const double* __restrict__ D,
                            const double* __restrict__ S, double* __restrict__ Fh,
                            double* __restrict__ Eh, double* __restrict__ B,
                            int* __restrict__ state, double* __restrict__ err_out) {
  extern __shared__ double sm[];
  double* T = sm;            // F D
  double* M = sm + n * n;    // F D S
  __shared__ double sw[32];
  __shared__ double coef[kDiisMax + 1];
  __shared__ int s_cnt, s_slot, s_ok;
  const int nn = n * n;
  if (threadIdx.x == 0) {
    s_cnt = state[0];
    s_slot = state[1];
  }
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const int i = k / n, j = k - i * n;   // T[i][j]
    double acc = 0.0;
    for (int l = 0; l < n; l++) acc += F[i + n * l] * D[l + n * j];
    T[k] = acc;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    double acc = 0.0;
    for (int l = 0; l < n; l++) acc += T[i * n + l] * S[l + n * j];
    M[k] = acc;
  }
  __syncthreads();
  const int slot = s_slot;
  double* e = Eh + (size_t)slot * nn;
  double* f = Fh + (size_t)slot * nn;
  double emax = 0.0;
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const int i = k / n, j = k - i * n;
    const double v = M[i * n + j] - M[j * n + i];
    e[i + n * j] = v;
    f[k] = F[k];
    emax = fmax(emax, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) emax = fmax(emax, __shfl_down_sync(0xffffffffu, emax, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x / 32] = emax;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r = fmax(r, sw[k]);
    if (err_out) *err_out = r;
  }
  __syncthreads();
  const int cnt = s_cnt + 1 < kDiisMax ? s_cnt + 1 : kDiisMax;
  // new row of B: <e_slot, e_j> for the occupied slots
  for (int j = 0; j < cnt; j++) {
    const double* ej = Eh + (size_t)j * nn;
    double acc = 0.0;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) acc += e[k] * ej[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x / 32] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0;
      for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r += sw[k];
      B[slot * kDiisMax + j] = r;
      B[j * kDiisMax + slot] = r;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    state[0] = cnt;
    state[1] = (slot + 1) % kDiisMax;
    s_ok = 0;
    if (cnt >= 2) {
      const int m = cnt + 1;
      double A[(kDiisMax + 1) * (kDiisMax + 2)];
      const int w = m + 1;
      for (int i = 0; i < cnt; i++) {
        for (int j = 0; j < cnt; j++) A[i * w + j] = B[i * kDiisMax + j];
        A[i * w + cnt] = -1.0;
        A[i * w + m] = 0.0;
      }
      for (int j = 0; j < cnt; j++) A[cnt * w + j] = -1.0;
      A[cnt * w + cnt] = 0.0;
      A[cnt * w + m] = -1.0;
      double scale = 0.0;
      for (int i = 0; i < cnt; i++) scale = fmax(scale, fabs(B[i * kDiisMax + i]));
      bool ok = scale > 0.0;
      for (int c = 0; c < m && ok; c++) {
        int piv = c;
        for (int r = c + 1; r < m; r++)
          if (fabs(A[r * w + c]) > fabs(A[piv * w + c])) piv = r;
        if (fabs(A[piv * w + c]) < 1e-14 * fmax(scale, 1.0)) { ok = false; break; }
        if (piv != c)
          for (int k = 0; k <= m; k++) {
            const double t = A[c * w + k];
            A[c * w + k] = A[piv * w + k];
            A[piv * w + k] = t;
          }
        for (int r = 0; r < m; r++) {
          if (r == c) continue;
          const double fct = A[r * w + c] / A[c * w + c];
          for (int k = c; k <= m; k++) A[r * w + k] -= fct * A[c * w + k];
        }
      }
      if (ok) {
        for (int i = 0; i < cnt; i++) coef[i] = A[i * w + m] / A[i * w + i];
        s_ok = 1;
      }
    }
  }
  __syncthreads();
  if (s_ok) {
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
      double acc = 0.0;
      for (int i = 0; i < cnt; i++) acc += coef[i] * Fh[(size_t)i * nn + k];
      F[k] = acc;
    }
  }
}

// ---- second-order SCF step (soscf.f SOGRAD / SOHESS / SONEWT / SOTRAN,
// driven as in xcscf.f:459-485) ---------------------------------------------
// One CTA.  F: electronic Fock matrix (column-major; its lower triangle is
// used, as pack_LT does), C: the current MO coefficients (column-major,
// orbitals by ascending energy; rotated in place), EE: the orbital energies
// of the last diagonalisation.  state[0] = ITSO (second-order steps taken
// since the last reset), state[1] = 1 when this call replaced the
// diagonalisation (D then holds prefac C_occ C_occ^T), else 0.  work:
// GRAD, PGRAD, DISPLI, HSTART, DISPLN, DGRADI, UPDTI (NPR each) and the
// (DISPL, DGRAD, UPDT) history the reference keeps on unit 15.
__device__ double block_dot(const double* a, const double* b, int n, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += a[i] * b[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) t += red[w];
  __syncthreads();
  return t;   // every thread
}

__global__ void soscf_kernel(int n, int na, const double* __restrict__ F,
                             double* __restrict__ C, const double* __restrict__ EE,
                             double prefac, double* __restrict__ D, int* __restrict__ state,
                             double* __restrict__ work, int maxit) {
  extern __shared__ double sm[];
  double* G = sm;                  // [n][n] rotation, G[i*n + j] = G(i,j)
  double* T = G + n * n;           // [n][n] scratch
  double* FC = T + n * n;          // [n][na] F C_occ
  double* red = FC + n * na;       // 64 reduction slots
  const int nv = n - na, npr = na * nv;
  double* grad = work;
  double* pgrad = grad + npr;
  double* displ = pgrad + npr;     // DISPLI
  double* hst = displ + npr;       // HSTART
  double* dn = hst + npr;          // DISPLN
  double* dg = dn + npr;           // DGRADI
  double* up = dg + npr;           // UPDTI
  double* hist = up + npr;         // [k][3][npr]
  const int tid = threadIdx.x;
  auto Fs = [&](int i, int k) { return i >= k ? F[i + n * k] : F[k + n * i]; };
  // SOGRAD: GRAD(jo, jv) = -C_jv^T F C_jo, ORBGRD = max |GRAD|
  for (int e = tid; e < n * na; e += blockDim.x) {
    const int i = e / na, jo = e - i * na;
    double acc = 0.0;
    for (int k = 0; k < n; k++) acc += Fs(i, k) * C[k + n * jo];
    FC[e] = acc;
  }
  __syncthreads();
  double gmax = 0.0;
  for (int q = tid; q < npr; q += blockDim.x) {
    const int jo = q / nv, jv = na + (q - jo * nv);
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc += FC[i * na + jo] * C[i + n * jv];
    grad[q] = -acc;
    gmax = fmax(gmax, fabs(acc));
  }
  for (int o = 16; o > 0; o >>= 1) gmax = fmax(gmax, __shfl_down_sync(0xffffffffu, gmax, o));
  __syncthreads();
  if ((tid & 31) == 0) red[tid >> 5] = gmax;
  __syncthreads();
  double orbgrd = 0.0;
  for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) orbgrd = fmax(orbgrd, red[w]);
  __syncthreads();
  int itso = state[0];
  const double sogtol = 1.0;        // xcscf.f:330
  if (!(orbgrd < sogtol || itso > 0)) {
    if (tid == 0) state[1] = 0;
    return;
  }
  // SOHESS on the first step: HSTART = 1/(e_v - e_o), capped at 200
  if (itso == 0)
    for (int q = tid; q < npr; q += blockDim.x) {
      const int jo = q / nv, jv = na + (q - jo * nv);
      const double de = EE[jv] - EE[jo];
      hst[q] = de > 0.5e-2 ? 1.0 / de : 200.0;
    }
  itso += 1;
  __syncthreads();
  // SONEWT
  for (int q = tid; q < npr; q += blockDim.x) dn[q] = hst[q] * grad[q];
  __syncthreads();
  const double small = 1.0e-3 * 1.0e-5;
  bool update = itso != 1;
  if (update && orbgrd < small) {
    itso -= 1;
    update = false;
  }
  if (update) {
    for (int q = tid; q < npr; q += blockDim.x) {
      dg[q] = grad[q] - pgrad[q];
      up[q] = hst[q] * dg[q];
    }
    __syncthreads();
    for (int k = 0; k < itso - 2 && k < maxit; k++) {
      const double* Dk = hist + (size_t)k * 3 * npr;
      const double* Gk = Dk + npr;
      const double* Uk = Gk + npr;
      double s1 = block_dot(Dk, Gk, npr, red), s2 = block_dot(Gk, Uk, npr, red);
      const double s3 = block_dot(Dk, grad, npr, red), s4 = block_dot(Uk, grad, npr, red);
      const double s5 = block_dot(Dk, dg, npr, red), s6 = block_dot(Uk, dg, npr, red);
      s1 = 1.0 / s1;
      s2 = 1.0 / s2;
      const double t = 1.0 + s1 / s2, t2 = s1 * s3, t4 = s1 * s5;
      const double t1 = t * t2 - s1 * s4, t3 = t * t4 - s1 * s6;
      for (int q = tid; q < npr; q += blockDim.x) {
        dn[q] += t1 * Dk[q] - t2 * Uk[q];
        up[q] += t3 * Dk[q] - t4 * Uk[q];
      }
      __syncthreads();
    }
    double s1 = block_dot(displ, dg, npr, red), s2 = block_dot(dg, up, npr, red);
    const double s3 = block_dot(displ, grad, npr, red), s4 = block_dot(up, grad, npr, red);
    s1 = 1.0 / s1;
    s2 = 1.0 / s2;
    const double t = 1.0 + s1 / s2, t2 = s1 * s3, t1 = t * t2 - s1 * s4;
    for (int q = tid; q < npr; q += blockDim.x) dn[q] += t1 * displ[q] - t2 * up[q];
    // the history entry of this step: the previous displacement, the
    // gradient change and its Hessian-updated image
    const int slot = itso - 2;
    if (slot >= 0 && slot <= maxit) {
      double* Hk = hist + (size_t)slot * 3 * npr;
      for (int q = tid; q < npr; q += blockDim.x) {
        Hk[q] = displ[q];
        Hk[npr + q] = dg[q];
        Hk[2 * npr + q] = up[q];
      }
    }
    __syncthreads();
  }
  for (int q = tid; q < npr; q += blockDim.x) displ[q] = -dn[q];
  __syncthreads();
  const double sqcdf = sqrt(block_dot(displ, displ, npr, red) / npr);
  if (sqcdf > 1.0 && itso > 5) itso = 0;     // reset on a huge rotation
  if (sqcdf > 0.1) {
    const double scal = sqrt(0.1 / sqcdf);
    for (int q = tid; q < npr; q += blockDim.x) displ[q] *= scal;
  }
  __syncthreads();
  // SOTRAN: G = 1 + X (X antisymmetric from the displacement), columns
  // orthonormalised in order, C <- C G
  for (int e = tid; e < n * n; e += blockDim.x) G[e] = 0.0;
  __syncthreads();
  for (int q = tid; q < npr; q += blockDim.x) {
    const int j = q / nv, i = na + (q - j * nv);
    G[j * n + i] = displ[q];
    G[i * n + j] = -displ[q];
  }
  __syncthreads();
  if (orbgrd <= 1.0e-20) {   // second-order term of the exponential (SOTRAN)
    for (int e = tid; e < na * na; e += blockDim.x) {
      const int i = e / na, j = e - i * na;
      if (j < i) continue;
      double dum = 0.0;
      for (int k = 0; k < nv; k++) dum += displ[nv * i + k] * displ[nv * j + k];
      dum *= -0.5;
      G[i * n + j] += dum;   // G(I,J) and G(J,I): twice on the diagonal, as SOTRAN
      G[j * n + i] += dum;
    }
    for (int e = tid; e < nv * nv; e += blockDim.x) {
      const int i = e / nv, j = e - i * nv;
      if (j < i) continue;
      double dum = 0.0;
      for (int k = 0; k < na; k++) dum += displ[nv * k + i] * displ[nv * k + j];
      dum *= -0.5;
      G[(na + i) * n + na + j] += dum;
      G[(na + j) * n + na + i] += dum;
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) G[i * n + i] += 1.0;
  __syncthreads();
  for (int i = 0; i < n; i++) {   // Gram-Schmidt on the columns G(:, i)
    if (tid == 0) {
      double d = 0.0;
      for (int k = 0; k < n; k++) d += G[k * n + i] * G[k * n + i];
      red[0] = 1.0 / sqrt(d);
    }
    __syncthreads();
    const double sc = red[0];
    for (int k = tid; k < n; k += blockDim.x) G[k * n + i] *= sc;
    __syncthreads();
    for (int j = i + 1 + tid; j < n; j += blockDim.x) {
      double d = 0.0;
      for (int k = 0; k < n; k++) d += G[k * n + i] * G[k * n + j];
      for (int k = 0; k < n; k++) G[k * n + j] -= d * G[k * n + i];
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;    // T(i,j) = sum_k C(i,k) G(k,j)
    double acc = 0.0;
    for (int k = 0; k < n; k++) acc += C[i + n * k] * G[k * n + j];
    T[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    C[i + n * j] = T[e];
  }
  for (int q = tid; q < npr; q += blockDim.x) pgrad[q] = grad[q];
  __syncthreads();
  // make_density: D = prefac sum_occ C_o C_o^T
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    double acc = 0.0;
    for (int o = 0; o < na; o++) acc += prefac * T[i * n + o] * T[j * n + o];
    D[i + n * j] = acc;
  }
  if (tid == 0) {
    state[0] = itso;
    state[1] = 1;
  }
}

}  // namespace

cudaError_t launch_scf_onebody(const DevSystem& S, double* Se, double* Sp,
                               double* Hce, double* Hcp, cudaStream_t s) {
  const int n = S.nebf * S.nebf + S.npbf * S.npbf;
  onebody_kernel<<<(n + 127) / 128, 128, 0, s>>>(S, Se, Sp, Hce, Hcp);
  return cudaGetLastError();
}

cudaError_t launch_gam_ep(const DevSystem& S, double* Gep, cudaStream_t s) {
  const int n = S.npbf * S.npbf * S.nebf * S.nebf;
  gam_ep_kernel<<<(n + 127) / 128, 128, 0, s>>>(S, Gep);
  return cudaGetLastError();
}

cudaError_t launch_gam1(const DevSystem& S, double* G1, double* G1s,
                        cudaStream_t s, int fp32, int pairs_only) {
  const long long warps = (long long)S.npbf * S.npbf * S.nebf * S.nebf;
  const long long blocks = (warps * 32 + 127) / 128;
  if (fp32) gam1_kernel<true><<<(unsigned)blocks, 128, 0, s>>>(S, G1, G1s, pairs_only);
  else gam1_kernel<false><<<(unsigned)blocks, 128, 0, s>>>(S, G1, G1s, pairs_only);
  return cudaGetLastError();
}

size_t scf_fock1_part_doubles(int ne, int np) {
  return 6 * ((size_t)ne * ne + (size_t)np * np);
}

cudaError_t launch_scf_fock1(int ne, int np, int nelec, const double* Hce,
                             const double* Hcp, const double* Gep,
                             const double* G1, const double* G1s,
                             const double* Gee, const double* DE,
                             const double* DP, double* focke, double* fockp,
                             double* se1, double* sp1, double* part, double* en,
                             cudaStream_t s, double* xfocke, double* xfockp) {
  const int nt = ne * ne + np * np;
  fock1_kernel<<<(nt + 127) / 128, 128, 0, s>>>(ne, np, nelec, Hce, Hcp, Gep, G1,
                                                G1s, Gee, DE, DP, focke, fockp,
                                                se1, sp1, part, xfocke, xfockp);
  fock1_energy_kernel<<<1, 256, 0, s>>>(nt, part, en);
  return cudaGetLastError();
}

cudaError_t launch_scf_assemble(int ne, int np, double* en, const double* se1,
                                const double* sp1, const double* se2,
                                const double* sp2, double* focke,
                                double* fockp, cudaStream_t s) {
  assemble_kernel<<<1, 256, 0, s>>>(ne, np, en, se1, sp1, se2, sp2, focke, fockp);
  return cudaGetLastError();
}

static cudaError_t eig_attr(const void* fn, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

cudaError_t launch_inv_sqrt(int n, const double* S, double* X, int* status,
                            cudaStream_t s) {
  if (n < 1 || n > kScfMaxN) return cudaErrorInvalidValue;
  const size_t smem = eig_smem_bytes(n);
  cudaError_t e = eig_attr((const void*)inv_sqrt_kernel, smem);
  if (e != cudaSuccess) return e;
  inv_sqrt_kernel<<<1, 256, smem, s>>>(n, S, X, status);
  return cudaGetLastError();
}

cudaError_t launch_roothan(int n, const double* F, const double* X, int first,
                           int nocc, double prefac, double* D, double* evals,
                           double* C, int* status, cudaStream_t s, const int* skip) {
  if (n < 1 || n > kScfMaxN || first < 0 || nocc < 1 || first + nocc > n)
    return cudaErrorInvalidValue;
  const size_t smem = eig_smem_bytes(n);
  cudaError_t e = eig_attr((const void*)roothan_kernel, smem);
  if (e != cudaSuccess) return e;
  roothan_kernel<<<1, 256, smem, s>>>(n, F, X, first, nocc, prefac, D, evals, C,
                                      status, skip);
  return cudaGetLastError();
}

size_t soscf_doubles(int n, int na, int maxit) {
  const size_t npr = (size_t)na * (n - na);
  return 7 * npr + 3 * npr * (size_t)(maxit + 1);
}

cudaError_t launch_soscf(int n, int na, const double* F, double* C, const double* EE,
                         double prefac, double* D, int* state, double* work, int maxit,
                         cudaStream_t s) {
  if (n < 2 || n > kScfMaxN || na < 1 || na >= n) return cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (2 * (size_t)n * n + (size_t)n * na) + 64 * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(soscf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  soscf_kernel<<<1, 256, smem, s>>>(n, na, F, C, EE, prefac, D, state, work, maxit);
  return cudaGetLastError();
}

size_t diis_doubles(int n) {
  return 2 * (size_t)kDiisMax * n * n + (size_t)kDiisMax * kDiisMax;
}

cudaError_t launch_diis(int n, double* F, const double* D, const double* S,
                        double* work, int* state, double* err, cudaStream_t s) {
  if (n < 1 || n > kScfMaxN) return cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * 2 * (size_t)n * n;
  cudaError_t e = eig_attr((const void*)diis_kernel, smem);
  if (e != cudaSuccess) return e;
  double* Fh = work;
  double* Eh = Fh + (size_t)kDiisMax * n * n;
  double* B = Eh + (size_t)kDiisMax * n * n;
  diis_kernel<<<1, 256, smem, s>>>(n, F, D, S, Fh, Eh, B, state, err);
  return cudaGetLastError();
}

cudaError_t launch_dendif(int ne, int np, const double* DE, double* DE0,
                          const double* DP, double* DP0, double* en,
                          cudaStream_t s) {
  dendif_kernel<<<1, 256, 0, s>>>(ne, np, DE, DE0, DP, DP0, en);
  return cudaGetLastError();
}

cudaError_t launch_uhf_fock1(int ne, int np, const double* Hce, const double* Hcp,
                             const double* Gep, const double* G1, const double* G1s,
                             const double* Gee, const double* DAE, const double* DBE,
                             const double* DP, double* FAE, double* FBE, double* FP,
                             double* SAE1, double* SBE1, double* SP1, double* part,
                             double* en, cudaStream_t s) {
  const int nt = ne * ne + np * np;
  uhf_fock1_kernel<<<(nt + 127) / 128, 128, 0, s>>>(ne, np, Hce, Hcp, Gep, G1, G1s, Gee,
                                                    DAE, DBE, DP, FAE, FBE, FP, SAE1,
                                                    SBE1, SP1, part);
  fock1_energy_kernel<<<1, 256, 0, s>>>(nt, part, en);
  return cudaGetLastError();
}

cudaError_t launch_uhf_assemble(int ne, int np, double* en, const double* sae1,
                                const double* sbe1, const double* sp1,
                                const double* sae2, const double* sbe2,
                                const double* sp2, double* FAE, double* FBE, double* FP,
                                cudaStream_t s) {
  uhf_assemble_kernel<<<1, 256, 0, s>>>(ne, np, en, sae1, sbe1, sp1, sae2, sbe2, sp2,
                                        FAE, FBE, FP);
  return cudaGetLastError();
}

cudaError_t launch_uhf_dendif(int ne, int np, const double* DA, double* DA0,
                              const double* DB, double* DB0, const double* DP,
                              double* DP0, double* en, cudaStream_t s) {
  uhf_dendif_kernel<<<1, 256, 0, s>>>(ne, np, DA, DA0, DB, DB0, DP, DP0, en);
  return cudaGetLastError();
}

}  // namespace neoxc
