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
// that bra can touch in shared memory, then every thread evaluates ket
// tuples (je1 fixed per thread, je2..je4 strided).  The Fock/energy
// contraction is fused (the direct-SCF path never writes gam_4), and
// per-CTA partial sums are reduced deterministically by a second kernel.
#include "neoxc_internal.h"

namespace neoxc {
namespace {

// Permutations of symm_gam4 (gam_4_OMP.f:756-803): ket slot feeding bra
// position m (2 bits per position), and the coefficients of :833-856.
// Written as switch functions so that, once the element loops are
// unrolled, every lookup folds to an immediate.
__device__ __forceinline__ int perm_code(int p) {
  switch (p) {
    case 0: return 228;
    case 1: return 225;
    case 2: return 210;
    case 3: return 216;
    case 4: return 201;
    case 5: return 198;
    case 6: return 135;
    case 7: return 141;
    case 8: return 156;
    case 9: return 147;
    case 10: return 177;
    case 11: return 180;
    case 12: return 120;
    case 13: return 114;
    case 14: return 99;
    case 15: return 108;
    case 16: return 78;
    case 17: return 75;
    case 18: return 27;
    case 19: return 30;
    case 20: return 45;
    case 21: return 39;
    case 22: return 54;
    case 23: return 57;
    default: return 0;
  }
}
__device__ __forceinline__ int perm_of(int p, int m) {
  return (perm_code(p) >> (2 * m)) & 3;
}
__device__ __forceinline__ double coef_of(int p) {
  switch (p) {
    case 0: return 16.0;
    case 1: return -8.0;
    case 2: return 4.0;
    case 3: return -8.0;
    case 4: return 4.0;
    case 5: return -8.0;
    case 6: return 4.0;
    case 7: return -2.0;
    case 8: return 4.0;
    case 9: return -2.0;
    case 10: return 4.0;
    case 11: return -8.0;
    case 12: return 4.0;
    case 13: return -2.0;
    case 14: return 4.0;
    case 15: return -8.0;
    case 16: return 4.0;
    case 17: return -2.0;
    case 18: return 4.0;
    case 19: return -2.0;
    case 20: return 4.0;
    case 21: return -8.0;
    case 22: return 4.0;
    case 23: return -2.0;
    default: return 0.0;
  }
}
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

// gam_4 element for ket offsets jn[m] = je_m*ne, jv[m] = je_m.
__device__ __forceinline__ double gam4_elem(const double* __restrict__ sGS,
                                            const double* __restrict__ sEE,
                                            const int* jn, const int* jv,
                                            int n2) {
  double acc = 0.0;
#pragma unroll
  for (int p = 0; p < 24; p++) {
    double x = 0.0;
#pragma unroll
    for (int q = 0; q < 6; q++) {
      const int a = split_of(q, 0), b = split_of(q, 1);
      const int c = split_of(q, 2), d = split_of(q, 3);
      const int sg = pair_slot(a, b), se = pair_slot(c, d);
      const int ka = perm_of(p, a), kb = perm_of(p, b);
      const int kc = perm_of(p, c), kd = perm_of(p, d);
      double gs = sGS[sg * n2 + jn[ka] + jv[kb]];
      double ee = sEE[se * n2 + jn[kc] + jv[kd]];
      x = fma(ee, gs, x);
    }
    acc = fma(coef_of(p), x, acc);
  }
  return acc * (1.0 / 192.0);   // 1/16 * 1/6 * 1/2
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
  double* sDE = smem + 12 * n2;
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
      for (int q = q0; q < n3; q += lanes_per_j1) {
        const int j2 = q / n2, r = q - j2 * n2, j3 = r / ne, j4 = r - j3 * ne;
        int jv[4] = {j1, j2, j3, j4};
        int jn[4] = {j1 * ne, j2 * ne, j3 * ne, j4 * ne};
        double g = gam4_elem(sGS, sEE, jn, jv, n2);
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
  return sizeof(double) * (size_t)(13 * ne * ne + bs);
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
  const int bs = gam4_block(ne);
  const size_t smem = gam4_smem(ne, bs);
  cudaError_t e = cudaFuncSetAttribute(gam4_kernel<0>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)(np * np * ne * ne);
  gam4_kernel<0><<<grid, bs, smem, s>>>(ne, np, gee, g2s, DE, DP, scratch,
                                        nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double* fp_tmp = scratch + (size_t)np * np * ne * ne * ne;
  return launch_fock_reduce(ne, np, ne, scratch, DE, DP, 4.0, 1, focke, fockp,
                            fp_tmp, E, s);
}

cudaError_t launch_gam4_icr(int ne, int np, const double* gee,
                            const double* g2s, double* g4, cudaStream_t s) {
  if (ne < 1 || ne > kGam4MaxNE || np < 1) return cudaErrorInvalidValue;
  const int bs = gam4_block(ne);
  const size_t smem = gam4_smem(ne, bs);
  cudaError_t e = cudaFuncSetAttribute(gam4_kernel<1>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  gam4_kernel<1><<<(unsigned)(np * np * ne * ne), bs, smem, s>>>(
      ne, np, gee, g2s, nullptr, nullptr, nullptr, g4);
  return cudaGetLastError();
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
