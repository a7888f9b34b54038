// k_gam4.cu -- gam_4 (5-particle) element assembly, fused direct-SCF Fock
// contraction, in-core storage and in-core contraction for sm_103a.
//
// Reference: gam_4_OMP.f:712-1192 (symm_gam4 / i10 / calc_GAM_4_integral),
// gam4_DSCF_OMP.f:141-320 (thread_gam4_DSCF), gam4_ICR_OMP.f:140-271
// (thread_gam4_IC) and :378-490 (thread_EG4ICR).
//
// Element (ip,jp; ie1..ie4; je1..je4):
//   gam4 = 1/16 * sum_{sigma in S4} c_sigma * x_sigma,
//   x_sigma = 1/6 * sum_{6 pair splits (ab|cd)} 1/2 ee(ie_c k_c|ie_d k_d)
//                                               * gs(p; ie_a k_a; ie_b k_b),
// with k_m = je_{sigma(m)} and c_sigma in {16,-8,4,-2} as in symm_gam4.
//
// Layout: one CTA per (ip,jp,ie1,ie2).  For each (ie3,ie4) the CTA stages
// the twelve ne x ne slices of GAM_2s / GAM_ee that the 24 permutations of
// that bra can touch, plus their transformed copies (see gam4_elem_f), in
// shared memory; every thread then evaluates ket tuples (je1 fixed per
// thread, je2..je4 strided) with 42 FP64 products per element.  The Fock/energy
// contraction is fused (the direct-SCF path never writes gam_4), and
// per-CTA partial sums are reduced deterministically by a second kernel.
#include "neoxc_internal.h"

namespace neoxc {
namespace {

// pair splits: GS(a,b) * EE(c,d) (calc_GAM_4_integral x1..x6); split q
// packs (a,b,c,d) in 2-bit fields.
__device__ __forceinline__ int split_of(int q, int f) {
  int code = 0;
  switch (q) {
    case 0: code = 228; break;
    case 1: code = 216; break;
    case 2: code = 156; break;
    case 3: code = 201; break;
    case 4: code = 141; break;
    case 5: code = 78; break;
    default: break;
  }
  return (code >> (2 * f)) & 3;
}

// table slot of pair (a,b), a<b : 01 02 03 12 13 23 -> 0..5
__host__ __device__ constexpr int pair_slot(int a, int b) {
  return a == 0 ? b - 1 : (a == 1 ? b + 1 : 5);
}

__device__ __forceinline__ double flush(double x) {
  return fabs(x) < 1.0e-100 ? 0.0 : x;   // underflow.f:2-11
}

// Stage the 12 tables for bra (i[0..3]) of proton pair (ip,jp).
// GS[s][x*ne+y] = GAM_2s(ip,jp; i_a,x; i_b,y);  EE[s][x*ne+y] = (i_a x|i_b y).
__device__ void stage_tables(int ne, int np, int ip, int jp, const int* i,
                             const double* __restrict__ gee,
                             const double* __restrict__ g2s, double* sGS,
                             double* sEE) {
  const int n2 = ne * ne;
  const long long pbase = (long long)(jp + np * ip);
  for (int k = threadIdx.x; k < 6 * n2; k += blockDim.x) {
    int s = k / n2, r = k - s * n2, x = r / ne, y = r - x * ne;
    int a = s < 3 ? 0 : (s < 5 ? 1 : 2);
    int b = s < 3 ? s + 1 : (s < 5 ? s - 1 : 3);
    // index_GAM_2PK(ip,jp,ie_a,x,ie_b,y) - 1
    long long og = y + (long long)ne * (i[b] + (long long)ne * (x + (long long)ne * (i[a] + (long long)ne * pbase)));
    // pack_4D(ne,ne,ne, y, ie_b, x, ie_a) - 1
    long long oe = y + (long long)ne * (i[b] + (long long)ne * (x + (long long)ne * i[a]));
    sGS[k] = flush(__ldg(g2s + og));
    sEE[k] = flush(__ldg(gee + oe));
  }
}

// ---- factored element (42 products instead of 144) ------------------------
// For each pair split q = (ab|cd) and each choice of the two kets that land
// on the Coulomb pair (c,d), the four ket orderings of the two pairs carry
// coefficients c_sigma that form a 2x2 block.  With T = X - X^T/2 applied to
// the split's GAM_ee slice (X = EE_q) and GAM_2s slice (X = GS_q), 30 of
// the 36 blocks are one product T_E * T_G times -8, 4 or 16, and the
// remaining 6 (the kets of the pair (a,b) sent to (c,d) and vice versa)
// need one extra raw product E * G times 3.  The element is then
//   gam4 = (-8 A + 4 B + 16 C + 3 D) / 192,
// the same value as the sum over the 24 permutations of symm_gam4 up to
// rounding.  Term t packs (split q, raw flag, ket slots of the E factor,
// ket slots of the G factor, coefficient class).
__device__ __forceinline__ int fterm(int t) {
  switch (t) {
    case 0: return 7744;  // split 0 T E(J0,J1) G(J2,J3) class 1
    case 1: return 15128;  // split 0 raw E(J1,J0) G(J3,J2) class 3
    case 2: return 1824;  // split 0 T E(J2,J0) G(J3,J1) class 0
    case 3: return 1728;  // split 0 T E(J0,J3) G(J2,J1) class 0
    case 4: return 3168;  // split 0 T E(J2,J1) G(J0,J3) class 0
    case 5: return 2256;  // split 0 T E(J1,J3) G(J0,J2) class 0
    case 6: return 9440;  // split 0 T E(J2,J3) G(J0,J1) class 2
    case 7: return 2833;  // split 1 T E(J1,J0) G(J3,J2) class 0
    case 8: return 7553;  // split 1 T E(J0,J2) G(J1,J3) class 1
    case 9: return 14121;  // split 1 raw E(J2,J0) G(J3,J1) class 3
    case 10: return 2497;  // split 1 T E(J0,J3) G(J1,J2) class 0
    case 11: return 3217;  // split 1 T E(J1,J2) G(J0,J3) class 0
    case 12: return 10449;  // split 1 T E(J1,J3) G(J0,J2) class 2
    case 13: return 1249;  // split 1 T E(J2,J3) G(J0,J1) class 0
    case 14: return 3602;  // split 2 T E(J1,J0) G(J2,J3) class 0
    case 15: return 3458;  // split 2 T E(J0,J2) G(J1,J3) class 0
    case 16: return 6594;  // split 2 T E(J0,J3) G(J1,J2) class 1
    case 17: return 13882;  // split 2 raw E(J3,J0) G(J2,J1) class 3
    case 18: return 11410;  // split 2 T E(J1,J2) G(J0,J3) class 2
    case 19: return 2258;  // split 2 T E(J1,J3) G(J0,J2) class 0
    case 20: return 1202;  // split 2 T E(J3,J2) G(J0,J1) class 0
    case 21: return 2883;  // split 3 T E(J0,J1) G(J3,J2) class 0
    case 22: return 3459;  // split 3 T E(J0,J2) G(J1,J3) class 0
    case 23: return 10691;  // split 3 T E(J0,J3) G(J1,J2) class 2
    case 24: return 7315;  // split 3 T E(J1,J2) G(J0,J3) class 1
    case 25: return 13163;  // split 3 raw E(J2,J1) G(J3,J0) class 3
    case 26: return 2259;  // split 3 T E(J1,J3) G(J0,J2) class 0
    case 27: return 483;  // split 3 T E(J2,J3) G(J1,J0) class 0
    case 28: return 3652;  // split 4 T E(J0,J1) G(J2,J3) class 0
    case 29: return 11652;  // split 4 T E(J0,J2) G(J1,J3) class 2
    case 30: return 2500;  // split 4 T E(J0,J3) G(J1,J2) class 0
    case 31: return 3220;  // split 4 T E(J1,J2) G(J0,J3) class 0
    case 32: return 6356;  // split 4 T E(J1,J3) G(J0,J2) class 1
    case 33: return 12924;  // split 4 raw E(J3,J1) G(J2,J0) class 3
    case 34: return 436;  // split 4 T E(J3,J2) G(J1,J0) class 0
    case 35: return 11845;  // split 5 T E(J0,J1) G(J2,J3) class 2
    case 36: return 3461;  // split 5 T E(J0,J2) G(J1,J3) class 0
    case 37: return 1733;  // split 5 T E(J0,J3) G(J2,J1) class 0
    case 38: return 3173;  // split 5 T E(J2,J1) G(J0,J3) class 0
    case 39: return 629;  // split 5 T E(J3,J1) G(J2,J0) class 0
    case 40: return 5349;  // split 5 T E(J2,J3) G(J0,J1) class 1
    case 41: return 12733;  // split 5 raw E(J3,J2) G(J1,J0) class 3
    default: return 0;
  }
}

// Per-split tables from the staged slot tables: TE_q = E_q - E_q^T/2 and
// TG_q = G_q - G_q^T/2 (E_q = EE slot (c,d), G_q = GS slot (a,b) of split q).
__device__ void stage_transformed(int ne, const double* __restrict__ sGS,
                                  const double* __restrict__ sEE, double* sTG,
                                  double* sTE) {
  const int n2 = ne * ne;
  for (int k = threadIdx.x; k < 6 * n2; k += blockDim.x) {
    const int q = k / n2, r = k - q * n2, x = r / ne, y = r - x * ne;
    const int sg = pair_slot(split_of(q, 0), split_of(q, 1));
    const int se = pair_slot(split_of(q, 2), split_of(q, 3));
    sTG[k] = fma(-0.5, sGS[sg * n2 + y * ne + x], sGS[sg * n2 + r]);
    sTE[k] = fma(-0.5, sEE[se * n2 + y * ne + x], sEE[se * n2 + r]);
  }
}

__device__ __forceinline__ double gam4_elem_f(const double* __restrict__ sGS,
                                              const double* __restrict__ sEE,
                                              const double* __restrict__ sTG,
                                              const double* __restrict__ sTE,
                                              const int* jn, const int* jv,
                                              int n2) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
  for (int t = 0; t < 42; t++) {
    const int code = fterm(t);
    const int q = code & 7, raw = (code >> 3) & 1;
    const int e0 = (code >> 4) & 3, e1 = (code >> 6) & 3;
    const int g0 = (code >> 8) & 3, g1 = (code >> 10) & 3;
    const int cl = (code >> 12) & 3;
    const double* Et = raw ? sEE + pair_slot(split_of(q, 2), split_of(q, 3)) * n2
                           : sTE + q * n2;
    const double* Gt = raw ? sGS + pair_slot(split_of(q, 0), split_of(q, 1)) * n2
                           : sTG + q * n2;
    const double x = Et[jn[e0] + jv[e1]];
    const double y = Gt[jn[g0] + jv[g1]];
    if (cl == 0) a0 = fma(x, y, a0);
    else if (cl == 1) a1 = fma(x, y, a1);
    else if (cl == 2) a2 = fma(x, y, a2);
    else a3 = fma(x, y, a3);
  }
  return (-8.0 * a0 + 4.0 * a1 + 16.0 * a2 + 3.0 * a3) * (1.0 / 192.0);
}

// mode 0: fused DSCF contraction; mode 1: store gam4 (GAM4_ICR)
template <int MODE>
__global__ void __launch_bounds__(256)
gam4_kernel(int ne, int np, const double* __restrict__ gee,
            const double* __restrict__ g2s, const double* __restrict__ DE,
            const double* __restrict__ DP, double* __restrict__ part,
            double* __restrict__ g4) {
  extern __shared__ double smem[];
  const int n2 = ne * ne;
  double* sGS = smem;
  double* sEE = smem + 6 * n2;
  double* sTG = smem + 12 * n2;
  double* sTE = smem + 18 * n2;
  double* sDE = smem + 24 * n2;
  double* sred = sDE + n2;
  int cta = blockIdx.x;
  const int i2 = cta % ne; cta /= ne;
  const int i1 = cta % ne; cta /= ne;
  const int jp = cta % np;
  const int ip = cta / np;
  if (MODE == 0)  // the store mode (GAM4_ICR) has no density
    for (int k = threadIdx.x; k < n2; k += blockDim.x) sDE[k] = DE[k];
  const int lanes_per_j1 = blockDim.x / ne;       // blockDim = ne*lanes
  const int j1 = threadIdx.x % ne;
  const int q0 = threadIdx.x / ne;
  const int n3 = n2 * ne;
  double acc = 0.0;
  int ibra[4] = {i1, i2, 0, 0};
  for (int i3 = 0; i3 < ne; i3++)
    for (int i4 = 0; i4 < ne; i4++) {
      ibra[2] = i3;
      ibra[3] = i4;
      __syncthreads();
      stage_tables(ne, np, ip, jp, ibra, gee, g2s, sGS, sEE);
      __syncthreads();
      stage_transformed(ne, sGS, sEE, sTG, sTE);
      __syncthreads();
      for (int q = q0; q < n3; q += lanes_per_j1) {
        const int j2 = q / n2, r = q - j2 * n2, j3 = r / ne, j4 = r - j3 * ne;
        int jv[4] = {j1, j2, j3, j4};
        int jn[4] = {j1 * ne, j2 * ne, j3 * ne, j4 * ne};
        double g = gam4_elem_f(sGS, sEE, sTG, sTE, jn, jv, n2);
        if (MODE == 0) {
          // DE is column-major DE(i,j) = DE[i + ne*j]
          double w = sDE[i2 + ne * j2] * sDE[i3 + ne * j3] * sDE[i4 + ne * j4];
          acc = fma(w, g, acc);
        } else {
          // index_GAM_4PK2 - 1
          long long o = j4 + (long long)ne * (i4 + (long long)ne * (j3 + (long long)ne * (i3 +
              (long long)ne * (j2 + (long long)ne * (i2 + (long long)ne * (j1 + (long long)ne * (i1 +
              (long long)ne * (jp + (long long)np * ip))))))));
          g4[o] = g;
        }
      }
    }
  if (MODE == 0) {
    __syncthreads();
    sred[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < ne) {
      double s = 0.0;
      for (int t = threadIdx.x; t < blockDim.x; t += ne) s += sred[t];
      // per-CTA partials: [cta][j1] = sum_w g  (scaled in the reducer)
      part[(size_t)blockIdx.x * ne + threadIdx.x] = s;
    }
  }
}

int gam4_block(int ne) { return ne * (256 / ne); }
size_t gam4_smem(int ne, int bs) {
  return sizeof(double) * (size_t)(25 * ne * ne + bs);
}

template <int MODE>
cudaError_t launch_gam4_kernel(int ne, int np, const double* gee,
                               const double* g2s, const double* DE,
                               const double* DP, double* part, double* g4,
                               cudaStream_t s) {
  const int bs = gam4_block(ne);
  const size_t smem = gam4_smem(ne, bs);
  cudaError_t e = cudaFuncSetAttribute(gam4_kernel<MODE>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  gam4_kernel<MODE><<<(unsigned)(np * np * ne * ne), bs, smem, s>>>(
      ne, np, gee, g2s, DE, DP, part, g4);
  return cudaGetLastError();
}

}  // namespace

size_t gam4_partial_doubles(int ne, int np) {
  return (size_t)np * np * ne * ne * ne + (size_t)np * np;
}

cudaError_t launch_gam4_dscf(int ne, int np, const double* gee,
                             const double* g2s, const double* DE,
                             const double* DP, double* scratch, double* focke,
                             double* fockp, double* E, cudaStream_t s) {
  if (ne < 1 || ne > kGam4MaxNE || np < 1) return cudaErrorInvalidValue;
  cudaError_t e = launch_gam4_kernel<0>(ne, np, gee, g2s, DE, DP, scratch,
                                        nullptr, s);
  if (e != cudaSuccess) return e;
  double* fp_tmp = scratch + (size_t)np * np * ne * ne * ne;
  return launch_fock_reduce(ne, np, ne, scratch, DE, DP, 4.0, 1, focke, fockp,
                            fp_tmp, E, s);
}

cudaError_t launch_gam4_icr(int ne, int np, const double* gee,
                            const double* g2s, double* g4, cudaStream_t s) {
  if (ne < 1 || ne > kGam4MaxNE || np < 1) return cudaErrorInvalidValue;
  return launch_gam4_kernel<1>(ne, np, gee, g2s, nullptr, nullptr, nullptr,
                               g4, s);
}

// ---- EG4ICR: stream GM4ICR once (HBM-bound) ----------------------------
// CTA per (ip,jp,ie1,je1): the ne^6 elements (ie2,je2,ie3,je3,ie4,je4) of
// that block are contiguous in the packed layout (je4 fastest).
namespace {
__global__ void __launch_bounds__(256)
eg4_kernel(int ne, int np, const double* __restrict__ DE,
           const double* __restrict__ g4, double* __restrict__ part) {
  __shared__ double sDE[kGam4MaxNE * kGam4MaxNE];
  __shared__ double sred[256];
  const int n2 = ne * ne;
  for (int k = threadIdx.x; k < n2; k += blockDim.x) sDE[k] = DE[k];
  __syncthreads();
  const long long n6 = (long long)n2 * n2 * n2;
  const double* blk = g4 + (long long)blockIdx.x * n6;
  double acc = 0.0;
  for (long long q = threadIdx.x; q < n6; q += blockDim.x) {
    long long r = q;
    int j4 = (int)(r % ne); r /= ne;
    int i4 = (int)(r % ne); r /= ne;
    int j3 = (int)(r % ne); r /= ne;
    int i3 = (int)(r % ne); r /= ne;
    int j2 = (int)(r % ne); r /= ne;
    int i2 = (int)r;
    double w = sDE[i2 + ne * j2] * sDE[i3 + ne * j3] * sDE[i4 + ne * j4];
    acc = fma(w, __ldg(blk + q), acc);
  }
  sred[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sred[threadIdx.x] += sred[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sred[0];
}
}  // namespace

size_t eg4_partial_doubles(int ne, int np) {
  return (size_t)np * np * ne * ne + (size_t)np * np;
}

cudaError_t launch_eg4icr(int ne, int np, const double* DE, const double* DP,
                          const double* g4, double* scratch, double* focke,
                          double* fockp, double* E, cudaStream_t s) {
  if (ne < 1 || ne > kGam4MaxNE || np < 1) return cudaErrorInvalidValue;
  eg4_kernel<<<(unsigned)(np * np * ne * ne), 256, 0, s>>>(ne, np, DE, g4,
                                                           scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // part layout [ipjp][i1][j1] == gam4 reducer layout with nsub = 1
  double* fp_tmp = scratch + (size_t)np * np * ne * ne;
  return launch_fock_reduce(ne, np, 1, scratch, DE, DP, 4.0, 1, focke, fockp,
                            fp_tmp, E, s);
}

}  // namespace neoxc
