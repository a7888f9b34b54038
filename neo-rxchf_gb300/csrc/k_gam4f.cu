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

}  // namespace neoxc
