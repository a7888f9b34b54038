// k_gam4f.cu -- factorised gam_4 Fock build for sm_103a.
//
// Same results as the fused element-wise GAM4_DSCF (gam4_DSCF_OMP.f:2-320,
// element from gam_4_OMP.f:712-1192) at O(nebf^4 npbf^2 + nebf^5) work
// instead of O(nebf^8 npbf^2), for the reference's actual inputs: GAM_2s
// pair-symmetric, gs(p; ab; cd) = gs(p; cd; ab) (GAM2_IC1 stores
// (x12+x21)/2, gam2_IC1_OMP.f:141-176), and GAM_ee symmetric under pair
// exchange, (ab|cd) = (cd|ab) (an ERI tensor).
//
// Derivation.  With k_m = je_sigma(m) the element is
//   gam4 = 1/16 sum_sigma c_sigma 1/6 sum_{splits (ab|cd)} 1/2
//          ee(ie_c k_c | ie_d k_d) gs(p; ie_a k_a; ie_b k_b),
// c_sigma = 16 (-1/2)^(4 - cycles(sigma)).  Summed against
// DP(p) DE(ie1,je1)..DE(ie4,je4), relabelling the four electrons maps every
// split onto (12|34) without changing c_sigma (a class function), so
//   E = 1/32 sum_sigma c_sigma sum_{i1..i4} G'(i1,i_s1,i2,i_s2) E'(i3,i_s3,i4,i_s4)
// with G = sum_p DP(p) gs(p) and the ket legs carried to bra labels by DE:
//   T'(a,x,c,y) = sum_{b,d} T(a,b,c,d) DE(x,b) DE(y,d).
// E is linear in DP and quartic in DE, and the same relabelling symmetry
// makes the reference's Fock contractions (4 DP DE^3 gam4 into focke(ie1,je1),
// DE^4 gam4 into fockp) exactly its gradients:
//   fockp(p)  = <gs(p), W>,   W = back-transform of W' = dE/dG',
//   focke(x,b)= sum_{a,c,y} [W'+W'^swap](a,x,c,y) H_G(a,b,c,y)
//             + [V'+V'^swap](a,x,c,y) H_E(a,b,c,y),   V' = dE/dE',
// H_T(a,b,c,y) = sum_d T(a,b,c,d) DE(y,d) the half-transformed tensor and
// ^swap the pair exchange (a,x,c,y) -> (c,y,a,x).  E = sum_p DP(p) fockp(p).
//
// dE/dG' at (a,x,c,y) is, per sigma, either a gather of E' with permuted
// legs, a Kronecker delta times a partial trace (one index pair of E'
// contracted), or two deltas times a full double trace; the 24 cases are the
// switch table sig_code below (the same table serves dE/dE' with G').
//
// Every 4-index tensor is stored C-order [l0][l1][l2][l3] (the layout of
// GAM_ee = pack_4D(je2,ie2,je1,ie1) and of one proton pair of GAM_2s =
// index_GAM_2PK), so a table read is a linear offset.  All arithmetic is
// FP64; table reads pass through the reference's underflow (|x|<1e-100 -> 0).
#include "neoxc_internal.h"
#include "tc_gemm.cuh"

namespace neoxc {
namespace {

__device__ __forceinline__ double flush(double x) {
  return fabs(x) < 1.0e-100 ? 0.0 : x;   // underflow.f:2-11
}

// ---- 1. G = sum_p DP(p) GAM_2s(p) ------------------------------------------
__global__ void dp_contract_kernel(long long n4, int np,
                                   const double* __restrict__ g2s,
                                   const double* __restrict__ DP,
                                   double* __restrict__ G) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n4;
       r += stride) {
    double acc = 0.0;
    for (int ip = 0; ip < np; ip++)
      for (int jp = 0; jp < np; jp++)
        acc = fma(DP[ip + np * jp],
                  flush(__ldg(g2s + (long long)(ip * np + jp) * n4 + r)), acc);
    G[r] = acc;
  }
}

// ---- 2. one-index transforms ------------------------------------------------
// out[row][y] = sum_k in[row][k] * M(y,k),  M(y,k) = M[y*sy + k*sk];
// rows = n^3.  A CTA stages RB rows of `in` and M^T in shared memory.
template <bool FLUSH>
__global__ void xform_last_kernel(int n, long long nrow,
                                  const double* __restrict__ in,
                                  const double* __restrict__ M, int sy, int sk,
                                  double* __restrict__ out) {
  extern __shared__ double sm[];
  double* sMt = sm;            // [k][y]
  double* sIn = sm + n * n;    // [RB][n]
  const int RB = blockDim.x / n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int k = e / n, y = e - k * n;
    sMt[e] = M[(long long)y * sy + (long long)k * sk];
  }
  const int rl = threadIdx.x / n, y = threadIdx.x - rl * n;
  for (long long r0 = (long long)blockIdx.x * RB; r0 < nrow;
       r0 += (long long)gridDim.x * RB) {
    __syncthreads();
    for (int e = threadIdx.x; e < RB * n; e += blockDim.x) {
      const long long row = r0 + e / n;
      double v = row < nrow ? in[row * n + (e % n)] : 0.0;
      sIn[e] = FLUSH ? flush(v) : v;
    }
    __syncthreads();
    const long long row = r0 + rl;
    if (rl < RB && row < nrow) {
      double acc = 0.0;
      for (int k = 0; k < n; k++) acc = fma(sIn[rl * n + k], sMt[k * n + y], acc);
      out[row * n + y] = acc;
    }
  }
}

// out[a][x][j] = sum_b M(x,b) * in[a][b][j],  j < m = n^2,  M(x,b) = M[x*sx + b*sb]
__global__ void xform_second_kernel(int n, int m, const double* __restrict__ in,
                                    const double* __restrict__ M, int sx, int sb,
                                    double* __restrict__ out) {
  extern __shared__ double sM[];   // [x][b]
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int x = e / n, b = e - x * n;
    sM[e] = M[(long long)x * sx + (long long)b * sb];
  }
  __syncthreads();
  const long long total = (long long)n * n * m;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < total;
       o += stride) {
    const long long am = o / m;
    const int j = (int)(o - am * m);
    const int a = (int)(am / n), x = (int)(am - (long long)a * n);
    const double* src = in + (long long)a * n * m + j;
    double acc = 0.0;
    for (int b = 0; b < n; b++) acc = fma(sM[x * n + b], src[(long long)b * m], acc);
    out[o] = acc;
  }
}

// ---- 3. partial and double traces ------------------------------------------
// leg pairs (0,1) (0,2) (0,3) (1,2) (1,3) (2,3) -> 0..5
__host__ __device__ constexpr int pair_leg(int p, int which) {
  return which == 0 ? (p < 3 ? 0 : (p < 5 ? 1 : 2))
                    : (p < 3 ? p + 1 : (p < 5 ? p - 1 : 3));
}

__device__ __forceinline__ long long idx4(int n, int l0, int l1, int l2, int l3) {
  return ((long long)((long long)l0 * n + l1) * n + l2) * n + l3;
}

// PT[t][p][u][v] = sum_z T_t with the legs of pair p at z and the other two
// legs (in leg order) at u, v.  blockIdx.y picks the tensor.
__global__ void traces_kernel(int n, const double* __restrict__ T0,
                              const double* __restrict__ T1,
                              double* __restrict__ PT) {
  const double* T = blockIdx.y ? T1 : T0;
  double* out = PT + (size_t)blockIdx.y * 6 * n * n;
  const int total = 6 * n * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    const int p = e / (n * n), r = e - p * n * n, u = r / n, v = r - u * n;
    const int k = pair_leg(p, 0), m = pair_leg(p, 1);
    int l[4];
    int q = 0;
    double acc = 0.0;
    for (int z = 0; z < n; z++) {
      q = 0;
      for (int g = 0; g < 4; g++) {
        if (g == k || g == m) l[g] = z;
        else l[g] = (q++ == 0) ? u : v;
      }
      acc += T[idx4(n, l[0], l[1], l[2], l[3])];
    }
    out[e] = acc;
  }
}

// ST[t][0..2] = double traces (01)(23), (02)(13), (03)(12) = traces of
// PT[t][0], PT[t][1], PT[t][2].  One warp per tensor.
__global__ void dtraces_kernel(int n, const double* __restrict__ PT,
                               double* __restrict__ ST) {
  const int t = threadIdx.x / 32, lane = threadIdx.x & 31;
  if (t >= 2) return;
  for (int s = 0; s < 3; s++) {
    const double* P = PT + ((size_t)t * 6 + s) * n * n;
    double acc = 0.0;
    for (int u = lane; u < n; u += 32) acc += P[u * n + u];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) ST[t * 4 + s] = acc;
  }
}

// ---- 4. dE/dG' and dE/dE' --------------------------------------------------
// Term t of the 24 permutations, for the gradient with respect to the tensor
// on slots (0,1) at output legs o = (a,x,c,y).  Bits: [0:2) k with
// coefficient 1/2 (-1/2)^k (= c_sigma/32); [2:6) Kronecker deltas between
// output legs (0,1), (2,3), (0,3), (1,2); [6:8) kind (0 gather, 1 partial
// trace, 2 double trace); [8:11) trace id (leg pair, or pairing for kind
// 2); then for legs 0..3 of the other tensor, 3 bits each: the output leg
// that supplies its value, 7 = traced.  Derived by following each label of
// the permutation through the two tensors' legs; by the exchange symmetry of
// slots (0,1) <-> (2,3) the same table gives the gradient with respect to
// the tensor on slots (2,3).
__device__ __forceinline__ int sig_code(int t) {
  switch (t) {
    case 0: return 8386700;   // sigma = id:          +1/2,  d01 d23, (01)(23)
    case 1: return 8387213;   // -1/4, d01 d23, (03)(12)
    case 2: return 8297797;   // -1/4, d01, PT(23) of legs (y,c)
    case 3: return 3136326;   // +1/8, d01, PT(12) of legs (y,c)
    case 4: return 7780934;   // +1/8, d01, PT(03) of legs (c,y)
    case 5: return 2619461;   // -1/4, d01, PT(01) of legs (y,c)
    case 6: return 8386737;   // -1/4, d03 d12, (01)(23)
    case 7: return 8387250;   // +1/8, d03 d12, (03)(12)
    case 8: return 8265058;   // +1/8, d12, PT(23) of legs (y,a)
    case 9: return 1039203;   // -1/16, d12, PT(12) of legs (y,a)
    case 10: return 7748195;  // -1/16, d12, PT(03) of legs (a,y)
    case 11: return 522338;   // +1/8, d12, PT(01) of legs (y,a)
    case 12: return 8293714;  // +1/8, d03, PT(23) of legs (x,c)
    case 13: return 3132243;  // -1/16, d03, PT(12) of legs (x,c)
    case 14: return 8260937;  // -1/4, d23, PT(23) of legs (x,a)
    case 15: return 1035082;  // +1/8, d23, PT(12) of legs (x,a)
    case 16: return 2492418;  // +1/8, gather (x,a,y,c)
    case 17: return 428035;   // -1/16, gather (x,c,y,a)
    case 18: return 7518803;  // -1/16, d03, PT(03) of legs (c,x)
    case 19: return 2357330;  // +1/8, d03, PT(01) of legs (x,c)
    case 20: return 7486026;  // +1/8, d23, PT(03) of legs (a,x)
    case 21: return 260169;   // -1/4, d23, PT(01) of legs (x,a)
    case 22: return 2234371;  // -1/16, gather (y,a,x,c)
    case 23: return 169986;   // +1/8, gather (y,c,x,a)
    default: return 0;
  }
}

__device__ __forceinline__ double sig_coef(int k) {
  return k == 0 ? 0.5 : (k == 1 ? -0.25 : (k == 2 ? 0.125 : -0.0625));
}

// blockIdx.y = 0: Wp = dE/dG' from (E', PT_E, ST_E);
// blockIdx.y = 1: Vp = dE/dE' from (G', PT_G, ST_G).
__global__ void gam4f_grad_kernel(int n, const double* __restrict__ Ep,
                                  const double* __restrict__ Gp,
                                  const double* __restrict__ PT,
                                  const double* __restrict__ ST,
                                  double* __restrict__ Wp,
                                  double* __restrict__ Vp) {
  const int which = blockIdx.y;
  const double* T = which ? Gp : Ep;                       // the other tensor
  const double* P = PT + (size_t)(which ? 0 : 1) * 6 * n * n;
  const double* S = ST + (which ? 0 : 4);
  double* out = which ? Vp : Wp;
  const long long n4 = (long long)n * n * n * n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n4;
       o += stride) {
    int l[4];
    long long r = o;
    l[3] = (int)(r % n); r /= n;
    l[2] = (int)(r % n); r /= n;
    l[1] = (int)(r % n); r /= n;
    l[0] = (int)r;
    double acc = 0.0;
#pragma unroll
    for (int t = 0; t < 24; t++) {
      const int code = sig_code(t);
      const int dm = (code >> 2) & 15;
      if ((dm & 1) && l[0] != l[1]) continue;
      if ((dm & 2) && l[2] != l[3]) continue;
      if ((dm & 4) && l[0] != l[3]) continue;
      if ((dm & 8) && l[1] != l[2]) continue;
      const int kind = (code >> 6) & 3, tid = (code >> 8) & 7;
      const int s0 = (code >> 11) & 7, s1 = (code >> 14) & 7,
                s2 = (code >> 17) & 7, s3 = (code >> 20) & 7;
      double v;
      if (kind == 0) {
        v = T[idx4(n, l[s0], l[s1], l[s2], l[s3])];
      } else if (kind == 1) {
        int uv[2], q = 0;
        if (s0 != 7) uv[q++] = l[s0];
        if (s1 != 7) uv[q++] = l[s1];
        if (s2 != 7) uv[q++] = l[s2];
        if (s3 != 7) uv[q++] = l[s3];
        v = P[((size_t)tid * n + uv[0]) * n + uv[1]];
      } else {
        v = S[tid];
      }
      acc = fma(sig_coef(code & 3), v, acc);
    }
    out[o] = acc;
  }
}

// ---- 5. fockp(p) = <GAM_2s(p), W>;  E = sum_p DP(p) fockp(p) ----------------
constexpr int kDotTB = 256;
constexpr int kDotChunk = 16384;   // elements per CTA

__device__ __forceinline__ double block_sum(double v, double* sw) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sw[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x + 31) / 32 ? sw[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;   // valid in thread 0
}

// grid (nchunk, np*np): part[p*nchunk + chunk]
__global__ void fockp_dot_kernel(long long n4, int nchunk,
                                 const double* __restrict__ g2s,
                                 const double* __restrict__ W,
                                 double* __restrict__ part) {
  __shared__ double sw[32];
  const int p = blockIdx.y;
  const long long base = (long long)blockIdx.x * kDotChunk;
  const long long end = base + kDotChunk < n4 ? base + kDotChunk : n4;
  const double* g = g2s + (long long)p * n4;
  double acc = 0.0;
  for (long long r = base + threadIdx.x; r < end; r += blockDim.x)
    acc = fma(flush(__ldg(g + r)), W[r], acc);
  const double t = block_sum(acc, sw);
  if (threadIdx.x == 0) part[(long long)p * nchunk + blockIdx.x] = t;
}

// One CTA: fockp(ip,jp) (+)= sum_chunk part; E = sum_p DP(p) * (new part).
__global__ void fockp_reduce_kernel(int np, int nchunk,
                                    const double* __restrict__ part,
                                    const double* __restrict__ DP,
                                    int accumulate, double* __restrict__ fockp,
                                    double* __restrict__ E) {
  __shared__ double sw[32];
  double e = 0.0;
  for (int p = threadIdx.x; p < np * np; p += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[(long long)p * nchunk + c];
    const int ip = p / np, jp = p - ip * np;
    const int f = ip + np * jp;                  // column-major fockp(ip,jp)
    fockp[f] = accumulate ? fockp[f] + s : s;
    e = fma(DP[f], s, e);
  }
  const double t = block_sum(e, sw);
  if (threadIdx.x == 0) *E = t;
}

// ---- mixed-precision forms of the two GAM_2s passes (tensor-core build) ----
// The FP64 forms above issue one FP64 FMA per GAM_2s element, which on this
// GPU (FP64 at 1/64 of the FP32 rate) costs more than reading the element
// from HBM.  These narrow each element to FP32 on the integer pipes
// (tc::narrow_f64) and multiply in FP32; partial sums are FP32 over at most
// kMixChunk terms and FP64 beyond, so the result carries ~1e-7 relative
// rounding (the GAM_2s values themselves are FP64 in memory).  GAM_2s is
// read once per pass with evict-first loads (__ldcs), which leaves L2 to
// the re-read operands (DP, the narrowed W).
constexpr int kMixChunk = 64;
constexpr int kDpShared = 12288;   // np^2 up to this: DP staged in shared memory

// G[r] = sum_p DP(p) GAM_2s[p][r]  (DP column-major, p = ip*np + jp as above);
// two consecutive elements per thread (16-byte loads) when every row p * n4
// stays 16-byte aligned, i.e. n4 even.
__global__ void dp_contract_mixed_kernel(long long n4, int np, const double* __restrict__ g2s,
                         const double* __restrict__ DP, double* __restrict__ G) {
  extern __shared__ float sdp[];   // [np*np] in the loop order of g2s, if staged
  const int np2 = np * np;
  const bool staged = np2 <= kDpShared;
  if (staged)
    for (int p = threadIdx.x; p < np2; p += blockDim.x) {
      const int ip = p / np, jp = p - ip * np;
      sdp[p] = tc::narrow_f64(DP[ip + np * jp]);
    }
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long nv = (n4 & 1) ? n4 : n4 / 2;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += stride) {
    double acc0 = 0.0, acc1 = 0.0;
    for (int p0 = 0; p0 < np2; p0 += kMixChunk) {
      const int p1 = p0 + kMixChunk < np2 ? p0 + kMixChunk : np2;
      float a0 = 0.0f, a1 = 0.0f;
      if (n4 & 1) {
#pragma unroll 8
        for (int p = p0; p < p1; p++) {
          const float d = staged ? sdp[p] : tc::narrow_f64(DP[(p / np) + np * (p % np)]);
          a0 = fmaf(d, tc::narrow_f64(__ldcs(g2s + (long long)p * n4 + v)), a0);
        }
      } else {
#pragma unroll 8
        for (int p = p0; p < p1; p++) {
          const float d = staged ? sdp[p] : tc::narrow_f64(DP[(p / np) + np * (p % np)]);
          const double2 g = __ldcs(reinterpret_cast<const double2*>(g2s + (long long)p * n4) + v);
          a0 = fmaf(d, tc::narrow_f64(g.x), a0);
          a1 = fmaf(d, tc::narrow_f64(g.y), a1);
        }
      }
      acc0 += (double)a0;
      acc1 += (double)a1;
    }
    if (n4 & 1) {
      G[v] = acc0;
    } else {
      G[2 * v] = acc0;
      G[2 * v + 1] = acc1;
    }
  }
}

// Wf[r] = narrow_f64(W[r])
__global__ void narrow_kernel(long long n, const double* __restrict__ in,
                              float* __restrict__ out) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x)
    out[r] = tc::narrow_f64(in[r]);
}

// part[p*nchunk + chunk] = sum_{r in chunk} GAM_2s[p][r] Wf[r], FP32
// products; each thread sums its kDotChunk / kDotTB (= kMixChunk) terms in
// FP32, the block in FP64.  Wf: W narrowed once (narrow_kernel), so the
// np^2 re-reads of it come from L2 at half the bytes.
// A CTA takes kDotP consecutive p (grid (nchunk, ceil(np^2 / kDotP))) so
// that each Wf element it loads serves kDotP products.
static_assert(kDotChunk / kDotTB == kMixChunk, "one FP32 partial sum per thread");
constexpr int kDotP = 2;
__global__ void __launch_bounds__(kDotTB)
fockp_dot_mixed_kernel(long long n4, int nchunk, int np2,
                       const double* __restrict__ g2s,
                       const float* __restrict__ Wf,
                       double* __restrict__ part) {
  __shared__ double sw[kDotP][kDotTB / 32];
  const int p0 = blockIdx.y * kDotP;
  const int pn = np2 - p0 < kDotP ? np2 - p0 : kDotP;
  const long long base = (long long)blockIdx.x * kDotChunk;
  const long long end = base + kDotChunk < n4 ? base + kDotChunk : n4;
  float a[kDotP];
#pragma unroll
  for (int j = 0; j < kDotP; j++) a[j] = 0.0f;
  for (long long r = base + threadIdx.x; r < end; r += blockDim.x) {
    const float w = __ldg(Wf + r);
#pragma unroll
    for (int j = 0; j < kDotP; j++)
      if (j < pn) a[j] = fmaf(tc::narrow_f64(__ldcs(g2s + (long long)(p0 + j) * n4 + r)), w, a[j]);
  }
  // kDotP block sums in FP64: warp shuffles, then one warp over the warps
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kDotP; j++) {
    double v = (double)a[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sw[j][warp] = v;
  }
  __syncthreads();
  if (warp < kDotP && warp < pn) {
    double v = lane < kDotTB / 32 ? sw[warp][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) part[(long long)(p0 + warp) * nchunk + blockIdx.x] = v;
  }
}

// ---- 6. focke ---------------------------------------------------------------
// CTA per (a,c): part[(a*n+c)][x*n+b] = sum_y Ws(a,x,c,y) H_G(a,b,c,y)
//                                      + Vs(a,x,c,y) H_E(a,b,c,y),
// Ws(a,x,c,y) = Wp(a,x,c,y) + Wp(c,y,a,x) (likewise Vs).
__global__ void focke_part_kernel(int n, const double* __restrict__ Wp,
                                  const double* __restrict__ HG,
                                  const double* __restrict__ Vp,
                                  const double* __restrict__ HE,
                                  double* __restrict__ part) {
  extern __shared__ double sm[];
  double* sS = sm;           // [x][y]
  double* sH = sm + n * n;   // [b][y]
  const int a = blockIdx.x / n, c = blockIdx.x - a * n;
  const int nn = n * n;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};   // up to 4 outputs per thread (n <= 64, 1024 threads)
  for (int pass = 0; pass < 2; pass++) {
    const double* X = pass ? Vp : Wp;
    const double* H = pass ? HE : HG;
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      const int u = e / n, y = e - u * n;
      sS[e] = X[idx4(n, a, u, c, y)] + X[idx4(n, c, y, a, u)];
      sH[e] = H[idx4(n, a, u, c, y)];
    }
    __syncthreads();
    int q = 0;
    for (int e = threadIdx.x; e < nn; e += blockDim.x, q++) {
      const int x = e / n, b = e - x * n;
      double s = 0.0;
      for (int y = 0; y < n; y++) s = fma(sS[x * n + y], sH[b * n + y], s);
      acc[q] += s;
    }
  }
  int q = 0;
  for (int e = threadIdx.x; e < nn; e += blockDim.x, q++)
    part[(long long)blockIdx.x * nn + e] = acc[q];
}

// focke(x,b) (+)= sum_{(a,c)} part[(a,c)][x*n+b]   (column-major focke)
__global__ void focke_reduce_kernel(int n, const double* __restrict__ part,
                                    int accumulate, double* __restrict__ focke) {
  const int nn = n * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int ac = 0; ac < nn; ac++) s += part[(long long)ac * nn + e];
    const int x = e / n, b = e - x * n;
    const int f = x + n * b;
    focke[f] = accumulate ? focke[f] + s : s;
  }
}

// Per-CTA maxima of |T(l0,l1,l2,l3) - T(l2,l3,l0,l1)| and |T| for GAM_ee
// (n^4) and GAM_2s (np^2 blocks of n^4): out[4*blockIdx.x + {0,1,2,3}].
__global__ void pair_symmetry_kernel(int n, int np, const double* __restrict__ gee,
                                     const double* __restrict__ g2s,
                                     double* __restrict__ out) {
  __shared__ double sw[4][32];
  const long long n4 = (long long)n * n * n * n;
  const long long total = n4 * (1 + (long long)np * np);
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += stride) {
    const long long blk = g / n4, r = g - blk * n4;
    const double* T = blk == 0 ? gee : g2s + (blk - 1) * n4;
    long long q = r;
    const int l3 = (int)(q % n); q /= n;
    const int l2 = (int)(q % n); q /= n;
    const int l1 = (int)(q % n); q /= n;
    const int l0 = (int)q;
    const double v = T[r];
    const double d = fabs(v - T[idx4(n, l2, l3, l0, l1)]);
    const int t = blk == 0 ? 0 : 2;
    m[t] = fmax(m[t], d);
    m[t + 1] = fmax(m[t + 1], fabs(v));
  }
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  for (int k = 0; k < 4; k++) {
    double v = m[k];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sw[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; i++) v = fmax(v, sw[threadIdx.x][i]);
    out[4 * blockIdx.x + threadIdx.x] = v;
  }
}

int grid_for(long long work, int tb) {
  long long g = (work + tb - 1) / tb;
  const long long cap = 152LL * 16;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

// out = underflow(in), element by element
__global__ void flush_copy_kernel(long long n, const double* __restrict__ in,
                                  double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = flush(in[i]);
}

// ---- mixed-precision variant: the transforms and focke on tensor cores -----
// C[m*ldc + n] = alpha sum_{k in split} A[m*lda + k] B[n*ldb + k]
// grid (ceil(M/128), ceil(N/64), nsplit); split z covers K range
// [z*kchunk, min(K, (z+1)*kchunk)) and writes C + z*split_stride.
__global__ void __launch_bounds__(tc::kThreads, 1)
tc_gemm_kernel(const double* __restrict__ A, long long lda, long long M,
               const double* __restrict__ B, long long ldb, long long N, long long K,
               long long kchunk, double alpha, double* __restrict__ C, long long ldc,
               long long split_stride, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_sm[];
  unsigned char* a_hi = tc_sm;
  unsigned char* a_lo = tc_sm + tc::kABytes;
  unsigned char* b_hi = tc_sm + 2 * tc::kABytes;
  unsigned char* b_lo = b_hi + tc::kBBytes;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(b_lo + tc::kBBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(b_lo + tc::kBBytes + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long m0 = (long long)blockIdx.x * tc::kTileM;
  const long long n0 = (long long)blockIdx.y * tc::kTileN;
  const long long kbeg = (long long)blockIdx.z * kchunk;
  const long long kend = kbeg + kchunk < K ? kbeg + kchunk : K;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;"
                 :: "r"(tc::smem_u32(tmem_slot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(tc::smem_u32(mbar))
                 : "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t mb = tc::smem_u32(mbar);
  uint32_t phase = 0;
  bool ok = true;
  const uint32_t idesc = tc::instr_desc();
  // kFoldTiles 64-wide K tiles are accumulated in TMEM (FP32) and then
  // folded into this thread's FP64 row of the result
  double acc[tc::kTileN];
#pragma unroll
  for (int i = 0; i < tc::kTileN; i++) acc[i] = 0.0;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  int tile = 0;
  for (long long kt = kbeg; kt < kend && ok; kt += tc::kTileK, tile++) {
    const bool first = tile % tc::kFoldTiles == 0;
    const bool fold = (tile + 1) % tc::kFoldTiles == 0 || kt + tc::kTileK >= kend;
    for (int e = tid; e < tc::kTileM * tc::kTileK; e += tc::kThreads) {
      const int r = e / tc::kTileK, k = e - r * tc::kTileK;
      const long long gm = m0 + r, gk = kt + k;
      const double v = (gm < M && gk < kend) ? A[gm * lda + gk] : 0.0;
      uint32_t hi, lo;
      tc::split_tf32(v, hi, lo);
      const int off = tc::canon_off(r, k);
      *reinterpret_cast<uint32_t*>(a_hi + off) = hi;
      *reinterpret_cast<uint32_t*>(a_lo + off) = lo;
    }
    for (int e = tid; e < tc::kTileN * tc::kTileK; e += tc::kThreads) {
      const int r = e / tc::kTileK, k = e - r * tc::kTileK;
      const long long gn = n0 + r, gk = kt + k;
      const double v = (gn < N && gk < kend) ? B[gn * ldb + gk] : 0.0;
      uint32_t hi, lo;
      tc::split_tf32(v, hi, lo);
      const int off = tc::canon_off(r, k);
      *reinterpret_cast<uint32_t*>(b_hi + off) = hi;
      *reinterpret_cast<uint32_t*>(b_lo + off) = lo;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = tc::smem_u32(a_hi), al = tc::smem_u32(a_lo);
      const uint32_t bh = tc::smem_u32(b_hi), bl = tc::smem_u32(b_lo);
      for (int st = 0; st < tc::kTileK / 8; st++) {
        const uint32_t o = st * 256;   // two 128-byte core matrices per K step
        tc::mma_tf32(tmem, tc::smem_desc(ah + o), tc::smem_desc(bh + o), idesc,
                     (st > 0 || !first) ? 1 : 0);
        tc::mma_tf32(tmem, tc::smem_desc(ah + o), tc::smem_desc(bl + o), idesc, 1);
        tc::mma_tf32(tmem, tc::smem_desc(al + o), tc::smem_desc(bh + o), idesc, 1);
      }
      tc::mma_commit(mb);
    }
    ok = __syncthreads_and(tc::mbar_wait(mb, phase) ? 1 : 0) != 0;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && fold) {
#pragma unroll
      for (int c = 0; c < tc::kTileN / 16; c++) {
        float v[16];
        tc::tmem_ld16(trow + (uint32_t)(c * 16), v);
#pragma unroll
        for (int i = 0; i < 16; i++) acc[c * 16 + i] += (double)v[i];
      }
    }
    // every lane's reads are done before the next tile's MMA overwrites TMEM
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    // every MMA has completed (last wait) and the operand tiles are dead:
    // stage the 128 x 64 FP64 tile in their shared memory (row stride 65)
    // and write it row-segment by row-segment, coalesced
    double* sc = reinterpret_cast<double*>(tc_sm);
    const int rloc = warp * 32 + lane;
#pragma unroll
    for (int i = 0; i < tc::kTileN; i++) sc[rloc * (tc::kTileN + 1) + i] = alpha * acc[i];
    __syncthreads();
    double* out = C + (long long)blockIdx.z * split_stride;
    for (int e = tid; e < tc::kTileM * tc::kTileN; e += tc::kThreads) {
      const int r = e / tc::kTileN, c = e - r * tc::kTileN;
      const long long row = m0 + r, n = n0 + c;
      if (row < M && n < N) out[row * ldc + n] = sc[r * (tc::kTileN + 1) + c];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" :: "r"(tmem)
                 : "memory");
  }
}

// out(i,j,k,l) = in(k,l,i,j) + beta in(i,j,k,l): a transpose of the
// (n^2 x n^2) matrix view, through 32 x 32 shared-memory tiles.
__global__ void pair_swap_kernel(int n2, const double* __restrict__ in, double beta,
                                 double* __restrict__ out) {
  __shared__ double t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < n2 && c < n2) t[j][threadIdx.x] = in[(long long)r * n2 + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + j, c = by + threadIdx.x;   // out[r][c] = in[c][r]
    if (r < n2 && c < n2) {
      const long long o = (long long)r * n2 + c;
      out[o] = t[threadIdx.x][j] + (beta != 0.0 ? beta * in[o] : 0.0);
    }
  }
}

// out(x,a,c,y) = in(a,x,c,y)
__global__ void swap12_kernel(int n, const double* __restrict__ in, double* __restrict__ out) {
  const long long n2 = (long long)n * n, total = n2 * n2;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < total;
       o += (long long)gridDim.x * blockDim.x) {
    const long long j = o % n2, xa = o / n2;
    const long long a = xa % n, x = xa / n;
    out[o] = in[(a * n + x) * n2 + j];
  }
}

// DEt[y*n + d] = DE(y,d) (column-major DE)
__global__ void transpose_n_kernel(int n, const double* __restrict__ DE, double* __restrict__ t) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
    const int y = e / n, d = e - y * n;
    t[e] = DE[y + n * d];
  }
}

// focke(x,b) (+)= sum_split part[split][x*64 + b]
__global__ void focke_tc_reduce_kernel(int n, int nsplit, const double* __restrict__ part,
                                       int accumulate, double* __restrict__ focke) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
    const int x = e / n, b = e - x * n;
    double s = 0.0;
    for (int z = 0; z < nsplit; z++) s += part[(long long)z * 128 * 64 + x * 64 + b];
    const int f = x + n * b;
    focke[f] = accumulate ? focke[f] + s : s;
  }
}

constexpr long long kFockeKChunk = 1024;

cudaError_t tc_gemm(const double* A, long long lda, long long M, const double* B,
                    long long ldb, long long N, long long K, long long kchunk, double alpha,
                    double* C, long long ldc, long long split_stride, int* err,
                    cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes);
  if (e != cudaSuccess) return e;
  const long long nsplit = (K + kchunk - 1) / kchunk;
  const dim3 grid((unsigned)((M + tc::kTileM - 1) / tc::kTileM),
                  (unsigned)((N + tc::kTileN - 1) / tc::kTileN), (unsigned)(nsplit < 1 ? 1 : nsplit));
  tc_gemm_kernel<<<grid, tc::kThreads, tc::kSmemBytes, s>>>(A, lda, M, B, ldb, N, K, kchunk,
                                                           alpha, C, ldc, split_stride, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pair_symmetry_check(int ne, int np, const double* gee,
                                       const double* g2s, double* out,
                                       int* grid, cudaStream_t s) {
  if (ne < 1 || np < 1) return cudaErrorInvalidValue;
  const long long n4 = (long long)ne * ne * ne * ne;
  const int g = grid_for(n4 * (1 + (long long)np * np), 256);
  *grid = g;
  pair_symmetry_kernel<<<g, 256, 0, s>>>(ne, np, gee, g2s, out);
  return cudaGetLastError();
}

size_t gam4f_scratch_doubles(int ne, int np) {
  const size_t n4 = (size_t)ne * ne * ne * ne;
  const size_t nchunk = (n4 + kDotChunk - 1) / kDotChunk;
  // G, H_G, G', H_E, E', Wp, Vp + PT(2x6 n^2) + ST(8) + fockp partials
  return 7 * n4 + 12 * (size_t)ne * ne + 8 + (size_t)np * np * nchunk;
}

cudaError_t launch_gam4_factored(int ne, int np, const double* gee,
                                 const double* g2s, const double* DE,
                                 const double* DP, double* scratch,
                                 double* focke, double* fockp, double* E,
                                 int accumulate, cudaStream_t s) {
  if (ne < 1 || ne > kGam4FactMaxNE || np < 1 || np > 255)
    return cudaErrorInvalidValue;
  const int n = ne;
  const long long n4 = (long long)n * n * n * n, n3 = (long long)n * n * n;
  const int nchunk = (int)((n4 + kDotChunk - 1) / kDotChunk);
  double* G = scratch;
  double* HG = G + n4;
  double* Gp = HG + n4;
  double* HE = Gp + n4;
  double* Ep = HE + n4;
  double* Wp = Ep + n4;
  double* Vp = Wp + n4;
  double* PT = Vp + n4;
  double* ST = PT + 12 * n * n;
  double* fpart = ST + 8;
  // buffers reused once their contents are dead
  double* Ht = Gp;      // back-transform intermediate (after the gradients)
  double* W = Ep;       // back-transformed dE/dG'
  double* epart = G;    // focke partials (n^2 x n^2 = n^4)

  const int TB = 256;
  const int RB = TB / n;
  const int TBl = RB * n;                       // threads of xform_last
  const size_t sm_last = sizeof(double) * ((size_t)n * n + (size_t)RB * n);
  const size_t sm_second = sizeof(double) * n * n;
  const int g_last = grid_for((n3 + RB - 1) / RB * TB, TB) ;
  const int g_n4 = grid_for(n4, TB);

  // 1. G = DP . GAM_2s
  dp_contract_kernel<<<g_n4, TB, 0, s>>>(n4, np, g2s, DP, G);
  // 2. H_G = G x DE (last index), G' = DE x H_G (second index); same for GAM_ee
  xform_last_kernel<false><<<g_last, TBl, sm_last, s>>>(n, n3, G, DE, 1, n, HG);
  xform_second_kernel<<<g_n4, TB, sm_second, s>>>(n, n * n, HG, DE, 1, n, Gp);
  xform_last_kernel<true><<<g_last, TBl, sm_last, s>>>(n, n3, gee, DE, 1, n, HE);
  xform_second_kernel<<<g_n4, TB, sm_second, s>>>(n, n * n, HE, DE, 1, n, Ep);
  // 3. traces of G' (t=0) and E' (t=1)
  traces_kernel<<<dim3(grid_for(6LL * n * n, TB), 2), TB, 0, s>>>(n, Gp, Ep, PT);
  dtraces_kernel<<<1, 64, 0, s>>>(n, PT, ST);
  // 4. Wp = dE/dG', Vp = dE/dE'
  gam4f_grad_kernel<<<dim3(g_n4, 2), TB, 0, s>>>(n, Ep, Gp, PT, ST, Wp, Vp);
  // 5. W = back-transform of Wp:  W(a,b,c,d) = sum_{x,y} Wp(a,x,c,y) DE(x,b) DE(y,d)
  xform_last_kernel<false><<<g_last, TBl, sm_last, s>>>(n, n3, Wp, DE, n, 1, Ht);
  xform_second_kernel<<<g_n4, TB, sm_second, s>>>(n, n * n, Ht, DE, n, 1, W);
  fockp_dot_kernel<<<dim3(nchunk, np * np), kDotTB, 0, s>>>(n4, nchunk, g2s, W, fpart);
  fockp_reduce_kernel<<<1, 256, 0, s>>>(np, nchunk, fpart, DP, accumulate, fockp, E);
  // 6. focke
  const int tbf = n * n < 1024 ? ((n * n + 31) / 32) * 32 : 1024;
  if (2 * sm_second > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(
        focke_part_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)(2 * sm_second));
    if (e != cudaSuccess) return e;
  }
  focke_part_kernel<<<n * n, tbf, 2 * sm_second, s>>>(n, Wp, HG, Vp, HE, epart);
  focke_reduce_kernel<<<grid_for((long long)n * n, TB), TB, 0, s>>>(n, epart, accumulate, focke);
  return cudaGetLastError();
}

size_t gam4f_tc_scratch_doubles(int ne, int np) {
  const size_t n4 = (size_t)ne * ne * ne * ne;
  const size_t nchunk = (n4 + kDotChunk - 1) / kDotChunk;
  const size_t nsplit = (size_t)((n4 / ne + kFockeKChunk - 1) / kFockeKChunk);
  // 8 n^4 tensors, DE^T, PT(2x6 n^2), ST(8), fockp partials, focke partials,
  // error flag
  return 8 * n4 + (size_t)ne * ne + 12 * (size_t)ne * ne + 8 + (size_t)np * np * nchunk +
         2 * nsplit * 128 * 64 + 2;
}

// Same focke / fockp / E as launch_gam4_factored, with the one-index
// transforms and the focke contraction on the tensor cores (tc_gemm.cuh:
// 3xTF32 products, FP32 accumulation, FP64 results) and everything else
// (the two passes over GAM_2s, traces, gradients, reductions) FP64.  The
// second-index transforms use the pair-exchange symmetry of the tables:
// sum_b T(a,b,c,d) DE(x,b) = H(c,d,a,x) with H the last-index transform, so
// T' = last(swap(last(T))); likewise the back transform of the symmetrised
// gradient.  *err (device int, optional) is set when a tensor-core wait ran
// out; the call then returns cudaErrorLaunchTimeout after the stream drains.
cudaError_t launch_gam4_factored_tc(int ne, int np, const double* gee,
                                    const double* g2s, const double* DE,
                                    const double* DP, double* scratch,
                                    double* focke, double* fockp, double* E,
                                    int accumulate, cudaStream_t s) {
  if (ne < 1 || ne > 64 || np < 1 || np > 255) return cudaErrorInvalidValue;
  const int n = ne;
  const long long n2 = (long long)n * n, n3 = n2 * n, n4 = n2 * n2;
  const int nchunk = (int)((n4 + kDotChunk - 1) / kDotChunk);
  const long long nsplit = (n3 + kFockeKChunk - 1) / kFockeKChunk;
  double* buf[8];
  for (int i = 0; i < 8; i++) buf[i] = scratch + (size_t)i * n4;
  double* DEt = scratch + 8 * n4;
  double* PT = DEt + n2;
  double* ST = PT + 12 * n2;
  double* fpart = ST + 8;
  double* epart = fpart + (size_t)np * np * nchunk;   // [2][nsplit][128*64]
  int* err = reinterpret_cast<int*>(epart + 2 * nsplit * 128 * 64);
  const int TB = 256;
  const int g_n4 = grid_for(n4, TB);
  const dim3 tgrid((unsigned)((n2 + 31) / 32), (unsigned)((n2 + 31) / 32));
  const dim3 tblk(32, 8);
  cudaError_t e;
#define TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
  TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  transpose_n_kernel<<<grid_for(n2, TB), TB, 0, s>>>(n, DE, DEt);
  // last-index transforms: T'(..,y) = sum_d T(..,d) DE(y,d)  [B = DE^T rows]
  auto last_f = [&](const double* in, double* out) {
    return tc_gemm(in, n, n3, DEt, n, n, n, n, 1.0, out, n, 0, err, s);
  };
  // back transforms: T'(..,d) = sum_y T(..,y) DE(y,d)  [B = DE rows]
  auto last_b = [&](const double* in, double* out, double alpha) {
    return tc_gemm(in, n, n3, DE, n, n, n, n, alpha, out, n, 0, err, s);
  };
  // 1. G = DP . GAM_2s (FP32 products, HBM)
  dp_contract_mixed_kernel<<<g_n4, 256, np * np <= kDpShared ? sizeof(float) * np * np : 0, s>>>(
      n4, np, g2s, DP, buf[0]);
  // 2. H_G, G' and H_E, E'
  TRY(last_f(buf[0], buf[1]));                                        // H_G
  pair_swap_kernel<<<tgrid, tblk, 0, s>>>((int)n2, buf[1], 0.0, buf[2]);
  TRY(last_f(buf[2], buf[3]));                                        // G'
  flush_copy_kernel<<<g_n4, TB, 0, s>>>(n4, gee, buf[0]);             // flushed GAM_ee
  TRY(last_f(buf[0], buf[4]));                                        // H_E
  pair_swap_kernel<<<tgrid, tblk, 0, s>>>((int)n2, buf[4], 0.0, buf[2]);
  TRY(last_f(buf[2], buf[5]));                                        // E'
  // 3-4. traces and gradients (FP64)
  traces_kernel<<<dim3(grid_for(6LL * n * n, TB), 2), TB, 0, s>>>(n, buf[3], buf[5], PT);
  dtraces_kernel<<<1, 64, 0, s>>>(n, PT, ST);
  gam4f_grad_kernel<<<dim3(g_n4, 2), TB, 0, s>>>(n, buf[5], buf[3], PT, ST, buf[6], buf[7]);
  // Ws = Wp + Wp^swap, Vs = Vp + Vp^swap
  pair_swap_kernel<<<tgrid, tblk, 0, s>>>((int)n2, buf[6], 1.0, buf[0]);
  pair_swap_kernel<<<tgrid, tblk, 0, s>>>((int)n2, buf[7], 1.0, buf[2]);
  // 5. W = back(Ws / 2), fockp = <GAM_2s, W>, E
  TRY(last_b(buf[0], buf[3], 0.5));
  pair_swap_kernel<<<tgrid, tblk, 0, s>>>((int)n2, buf[3], 0.0, buf[5]);
  TRY(last_b(buf[5], buf[6], 1.0));                                   // W
  float* Wf = reinterpret_cast<float*>(buf[7]);   // free until swap12 below
  narrow_kernel<<<g_n4, TB, 0, s>>>(n4, buf[6], Wf);
  fockp_dot_mixed_kernel<<<dim3(nchunk, (np * np + kDotP - 1) / kDotP), kDotTB, 0, s>>>(
      n4, nchunk, np * np, g2s, Wf, fpart);
  fockp_reduce_kernel<<<1, 256, 0, s>>>(np, nchunk, fpart, DP, accumulate, fockp, E);
  // 6. focke(x,b) = sum_{a,c,y} Ws(a,x,c,y) H_G(a,b,c,y) + Vs(a,x,c,y) H_E(a,b,c,y)
  swap12_kernel<<<g_n4, TB, 0, s>>>(n, buf[0], buf[3]);   // Ws  -> [x][a][c][y]
  swap12_kernel<<<g_n4, TB, 0, s>>>(n, buf[1], buf[5]);   // H_G -> [b][a][c][y]
  swap12_kernel<<<g_n4, TB, 0, s>>>(n, buf[2], buf[7]);   // Vs
  swap12_kernel<<<g_n4, TB, 0, s>>>(n, buf[4], buf[1]);   // H_E
  TRY(tc_gemm(buf[3], n3, n, buf[5], n3, n, n3, kFockeKChunk, 1.0, epart, 64, 128 * 64, err, s));
  TRY(tc_gemm(buf[7], n3, n, buf[1], n3, n, n3, kFockeKChunk, 1.0, epart + nsplit * 128 * 64,
              64, 128 * 64, err, s));
  focke_tc_reduce_kernel<<<grid_for(n2, TB), TB, 0, s>>>(n, (int)(2 * nsplit), epart,
                                                        accumulate, focke);
#undef TRY
  return cudaGetLastError();
}

}  // namespace neoxc
