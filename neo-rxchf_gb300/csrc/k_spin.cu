// k_spin.cu -- open-shell (XCUHF) in-core contractions for sm_103a.
//
// Reference: xcuhf/xcuhf_omg1.f (FAE_OMG1 / UFP_OMG1), xcuhf_omg2.f
// (FAE_OMG2 / UFP_OMG2), xcuhf_omg3.f (FAE_OMG3 / UFP_OMG3), xcuhf_omg4.f
// (FAE_OMG4 / UFP_OMG4 and OMG4_ICR).
//
// The reference evaluates, for every stored element, antisymmetrised
// combinations of ket-permuted partners (2, 6 or 24 of them) weighted by
// products of the alpha / beta densities of the other electrons, once per
// routine.  Here one pass over the tensor serves all of them: a CTA owns the
// bra (ip,jp,i1,i2[,i3,i4]) and stages the ne^K ket values of that bra in
// shared memory (one HBM read per element), each thread owns one ket j1 and
// loops over the remaining kets, and two accumulators are kept per thread:
//   class A = the alpha Fock row (FAE) and the alpha-weighted proton term,
//   class B = the same with alpha and beta exchanged (FBE, beta weights).
// The flag sets of the reference (LAA, LAB, ... / L4A, L3A1B, ...) arrive
// as bit masks, so FAE with swapped arguments (the reference's beta call)
// and UFP's class B are the same code.  Per-CTA partials are reduced by a
// second deterministic kernel (no floating-point atomics).
#include <type_traits>

#include "neoxc_internal.h"

namespace neoxc {
namespace {

constexpr int kSpinThreads = 256;

// offset of ket slot m (0-based, of K) in the packed tensor: the packed
// index interleaves (i_m, j_m) with the last ket fastest, so ket m moves by
// ne^(2(K-1-m)) and bra m by ne^(2(K-1-m)+1).
__host__ __device__ inline long long pw(int ne, int e) {
  long long r = 1;
  for (int k = 0; k < e; k++) r *= ne;
  return r;
}

// Ket block of one bra: the shared-memory copy (int strides) or the global
// tensor (64-bit strides).
template <int K, typename I>
struct Slab {
  const double* p;
  I st[K];             // stride of each ket slot
  __device__ double operator()(const int* j) const {
    I o = 0;
#pragma unroll
    for (int m = 0; m < K; m++) o += (I)j[m] * st[m];
    return p[o];
  }
};

// Shared-memory pitches of the ket block: slot K-1 contiguous, every other
// slot's pitch rounded up to an odd number of doubles, so lanes that differ
// in any one ket index hit different banks.  Returns the padded size.
__host__ __device__ inline int ket_pitches(int K, int ne, int* pt) {
  pt[K - 1] = 1;
  for (int m = K - 2; m >= 0; m--) pt[m] = (pt[m + 1] * ne) | 1;
  return pt[0] * ne;
}

// x / d for x < 65536 and 2 <= d <= 256 with one multiply-high:
// m = ceil(2^32 / d) is exact in that range.
struct DivNe {
  unsigned d, m;
  __device__ explicit DivNe(int ne)
      : d((unsigned)ne), m((unsigned)(((1ull << 32) + (unsigned)ne - 1) / (unsigned)ne)) {}
  __device__ unsigned operator()(unsigned x) const { return d == 1 ? x : __umulhi(x, m); }
};

// K = 2: G(j1,j2), G(j2,j1)
template <typename S>
__device__ inline void acc2(const S& g, int j1, int j2, double a2, double b2,
                            unsigned fa, unsigned fb, double& A, double& B) {
  const int k12[2] = {j1, j2}, k21[2] = {j2, j1};
  const double o12 = g(k12), o21 = g(k21);
  // FAE_OMG2: LAA (bit0) DAE2 (o12-o21) + LAB (bit1) DBE2 o12; UFP classes
  if (fa & 1u) A = fma(a2, o12 - o21, A);
  if (fa & 2u) A = fma(b2, o12, A);
  if (fb & 1u) B = fma(b2, o12 - o21, B);
  if (fb & 2u) B = fma(a2, o12, B);
}

// K = 3: OMG6 (bit0), the two mixed pairs OMG12/OMG13 (bit1), OMG23 (bit2)
template <typename S>
__device__ inline void acc3(const S& g, const int* j, double a2, double b2,
                            double a3, double b3, unsigned fa, unsigned fb,
                            double& A, double& B) {
  const int j1 = j[0], j2 = j[1], j3 = j[2];
  const int k123[3] = {j1, j2, j3}, k213[3] = {j2, j1, j3}, k312[3] = {j3, j1, j2};
  const int k132[3] = {j1, j3, j2}, k231[3] = {j2, j3, j1}, k321[3] = {j3, j2, j1};
  const double g123 = g(k123), g213 = g(k213), g132 = g(k132), g321 = g(k321);
  const unsigned f = fa | fb;
  double o6 = 0.0;
  if (f & 1u) o6 = g123 - g213 + g(k312) - g132 + g(k231) - g321;
  const double o23 = g123 - g132, o12 = g123 - g213, o13 = g123 - g321;
  if (fa & 1u) A = fma(a2 * a3, o6, A);
  if (fa & 2u) A = fma(a2 * b3, o12, fma(b2 * a3, o13, A));
  if (fa & 4u) A = fma(b2 * b3, o23, A);
  if (fb & 1u) B = fma(b2 * b3, o6, B);
  if (fb & 2u) B = fma(b2 * a3, o12, fma(a2 * b3, o13, B));
  if (fb & 4u) B = fma(a2 * a3, o23, B);
}

// K = 4: the 24-term set (bit0), the three 6-term sets (bit1), the three
// 4-term sets (bit2) and the last 6-term set (bit3) of calc_FAEOMG4.
template <typename S>
__device__ inline void acc4(const S& g, const int* j, const double* a,
                            const double* b, unsigned fa, unsigned fb, double& A,
                            double& B) {
  const int j1 = j[0], j2 = j[1], j3 = j[2], j4 = j[3];
#define V(w, x, y, z) ([&]() { const int k_[4] = {w, x, y, z}; return g(k_); }())
  const unsigned f = fa | fb;
  const double OMG = V(j1, j2, j3, j4);
  const double O23 = V(j1, j3, j2, j4), O12 = V(j2, j1, j3, j4);
  const double O13 = V(j3, j2, j1, j4), O24 = V(j1, j4, j3, j2);
  const double O14 = V(j4, j2, j3, j1), O34 = V(j1, j2, j4, j3);
  double aaa = 0.0, aab = 0.0, aba = 0.0, baa = 0.0, abb = 0.0, bab = 0.0,
         bba = 0.0, bbb = 0.0;
  if (f & 1u)
    aaa = OMG - O23 - O12 - O13 - O24 - O14 - O34
        + V(j2, j3, j1, j4) + V(j3, j1, j2, j4) + V(j2, j4, j3, j1)
        + V(j4, j1, j3, j2) + V(j2, j1, j4, j3) + V(j3, j2, j4, j1)
        + V(j4, j2, j1, j3) + V(j3, j4, j1, j2) + V(j4, j3, j2, j1)
        + V(j1, j3, j4, j2) + V(j1, j4, j2, j3)
        - V(j2, j3, j4, j1) - V(j2, j4, j1, j3) - V(j3, j1, j4, j2)
        - V(j3, j4, j2, j1) - V(j4, j1, j2, j3) - V(j4, j3, j1, j2);
  if (f & 2u) {
    aab = OMG - O23 - O12 + V(j2, j3, j1, j4) + V(j3, j1, j2, j4) - O13;
    aba = OMG - O24 - O12 + V(j2, j4, j3, j1) + V(j4, j1, j3, j2) - O14;
    baa = OMG - O34 - O13 + V(j3, j2, j4, j1) + V(j4, j2, j1, j3) - O14;
  }
  if (f & 4u) {
    abb = OMG - O34 - O12 + V(j2, j1, j4, j3);
    bab = OMG - O24 - O13 + V(j3, j4, j1, j2);
    bba = OMG - O23 - O14 + V(j4, j3, j2, j1);
  }
  if (f & 8u) bbb = OMG - O34 - O23 + V(j1, j3, j4, j2) + V(j1, j4, j2, j3) - O24;
#undef V
  // a[m], b[m]: alpha / beta density of electron m+2 at (i_m+2, j_m+2)
  if (fa & 1u) A = fma(a[0] * a[1] * a[2], aaa, A);
  if (fa & 2u)
    A += a[0] * a[1] * b[2] * aab + a[0] * b[1] * a[2] * aba + b[0] * a[1] * a[2] * baa;
  if (fa & 4u)
    A += a[0] * b[1] * b[2] * abb + b[0] * a[1] * b[2] * bab + b[0] * b[1] * a[2] * bba;
  if (fa & 8u) A = fma(b[0] * b[1] * b[2], bbb, A);
  if (fb & 1u) B = fma(b[0] * b[1] * b[2], aaa, B);
  if (fb & 2u)
    B += b[0] * b[1] * a[2] * aab + b[0] * a[1] * b[2] * aba + a[0] * b[1] * b[2] * baa;
  if (fb & 4u)
    B += b[0] * a[1] * a[2] * abb + a[0] * b[1] * a[2] * bab + a[0] * a[1] * b[2] * bba;
  if (fb & 8u) B = fma(a[0] * a[1] * a[2], bbb, B);
}

// CTA (ipjp, i1, i2) for rank 2, (ipjp, i1, i2, i3) for ranks 3 and 4 (rank
// 4 loops over i4).  Outputs per CTA: part[(cta*nacc + a)*ne + j1]
// (a = 2*tensor + class; the electron Fock rows) and ppart[cta*2 + t] =
// sum_j1 (DA(i1,j1) A_t[j1] + DB(i1,j1) B_t[j1]) (the proton terms).
template <int K, bool SMEM>
__global__ void __launch_bounds__(kSpinThreads)
spin_kernel(int ne, int np, const double* __restrict__ G,
            const double* __restrict__ Gs, const double* __restrict__ DA,
            const double* __restrict__ DB, unsigned fa, unsigned fb,
            double* __restrict__ part, double* __restrict__ ppart) {
  extern __shared__ double sm[];
  const int n2 = ne * ne;
  const int nten = (K == 2 && Gs) ? 2 : 1;
  const long long slab = pw(ne, K);
  int pt[K];
  const int slabp = ket_pitches(K, ne, pt);      // padded shared-memory block
  double* sDA = sm;
  double* sDB = sm + n2;
  double* sG = sm + 2 * n2;                      // SMEM: nten * slabp
  double* sred = sG + (SMEM ? nten * slabp : 0); // [blockDim]
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    sDA[k] = DA[k];
    sDB[k] = DB[k];
  }
  __syncthreads();
  int cta = blockIdx.x;
  int ib[4] = {0, 0, 0, 0};
  if (K >= 3) { ib[2] = cta % ne; cta /= ne; }
  ib[1] = cta % ne; cta /= ne;
  ib[0] = cta % ne; cta /= ne;
  const long long ipjp = cta;
  const int lanes = blockDim.x / ne;
  const int j1 = threadIdx.x % ne;
  const int q0 = threadIdx.x / ne;
  const bool active = q0 < lanes;
  const int nrest = (int)(slab / ne);
  const DivNe dv(ne);
  using I = typename std::conditional<SMEM, int, long long>::type;
  long long gst[K];    // global stride of ket slot m: ne^(2(K-1-m))
  for (int m = 0; m < K; m++) gst[m] = pw(ne, 2 * (K - 1 - m));
  double accA[2] = {0.0, 0.0}, accB[2] = {0.0, 0.0};
  const int ninner = K == 4 ? ne : 1;
  for (int in = 0; in < ninner; in++) {
    if (K == 4) ib[3] = in;
    long long base = ipjp * pw(ne, 2 * K);
    for (int m = 0; m < K; m++) base += ib[m] * (gst[m] * ne);
    Slab<K, I> g[2];
    for (int t = 0; t < 2; t++) {
      const double* src = t == 0 ? G : Gs;
      if (SMEM) {
        g[t].p = sG + t * slabp;
        for (int m = 0; m < K; m++) g[t].st[m] = (I)pt[m];
      } else {
        g[t].p = src ? src + base : nullptr;
        for (int m = 0; m < K; m++) g[t].st[m] = (I)gst[m];
      }
    }
    if (SMEM) {
      __syncthreads();
      for (int t = 0; t < nten; t++) {
        const double* src = (t == 0 ? G : Gs) + base;
        for (int k = threadIdx.x; k < (int)slab; k += blockDim.x) {
          unsigned r = (unsigned)k;
          long long o = 0;
          int so = 0;
#pragma unroll
          for (int m = K - 1; m >= 0; m--) {
            const unsigned q = dv(r);
            const int x = (int)(r - q * (unsigned)ne);
            o += (long long)x * gst[m];
            so += x * pt[m];
            r = q;
          }
          sG[t * slabp + so] = __ldg(src + o);
        }
      }
      __syncthreads();
    }
    if (active) {
      double a[3], b[3];
      for (int q = q0; q < nrest; q += lanes) {
        int j[4] = {j1, 0, 0, 0};
        unsigned r = (unsigned)q;
#pragma unroll
        for (int m = K - 1; m >= 1; m--) {
          const unsigned qq = dv(r);
          j[m] = (int)(r - qq * (unsigned)ne);
          r = qq;
        }
        for (int m = 1; m < K; m++) {
          a[m - 1] = sDA[ib[m] + ne * j[m]];
          b[m - 1] = sDB[ib[m] + ne * j[m]];
        }
        if constexpr (K == 2) {
          acc2(g[0], j1, j[1], a[0], b[0], fa, fb, accA[0], accB[0]);
          if (nten == 2) acc2(g[1], j1, j[1], a[0], b[0], fa, fb, accA[1], accB[1]);
        } else if constexpr (K == 3) {
          acc3(g[0], j, a[0], b[0], a[1], b[1], fa, fb, accA[0], accB[0]);
        } else {
          acc4(g[0], j, a, b, fa, fb, accA[0], accB[0]);
        }
      }
    }
  }
  // reduce over the lanes of each j1; thread j1 keeps its row sums
  const int nacc = 2 * nten;
  double row[4] = {0.0, 0.0, 0.0, 0.0};
  for (int acc = 0; acc < nacc; acc++) {
    __syncthreads();
    const double v = (acc & 1) ? accB[acc >> 1] : accA[acc >> 1];
    sred[threadIdx.x] = active ? v : 0.0;
    __syncthreads();
    if ((int)threadIdx.x < ne) {
      double s = 0.0;
      for (int t = threadIdx.x; t < lanes * ne; t += ne) s += sred[t];
      part[((size_t)blockIdx.x * nacc + acc) * ne + threadIdx.x] = s;
      row[acc] = s;
    }
  }
  // proton terms of this CTA: sum over j1 in a fixed order
  for (int t = 0; t < nten; t++) {
    __syncthreads();
    if ((int)threadIdx.x < ne) {
      const int j = threadIdx.x;
      sred[j] = sDA[ib[0] + ne * j] * row[2 * t] + sDB[ib[0] + ne * j] * row[2 * t + 1];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int j = 0; j < ne; j++) s += sred[j];
      ppart[(size_t)blockIdx.x * 2 + t] = s;
    }
  }
}

// fe_out[a][i1 + ne*j1] = sum_ipjp DP(ipjp) sum_sub part; thread per
// output, the CTAs of one (ipjp, i1) are nsub consecutive ones.
__global__ void spin_reduce_e_kernel(int ne, int np, int nacc, int nsub,
                                     const double* __restrict__ part,
                                     const double* __restrict__ DP,
                                     double* __restrict__ fe_out) {
  // one warp per output; lanes take the nsub sub-blocks strided, then a
  // fixed-order shuffle tree (deterministic)
  const int n2 = ne * ne, p2 = np * np;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= nacc * n2) return;
  const int a = t / n2, r = t - a * n2, i1 = r / ne, j1 = r - i1 * ne;
  double s = 0.0;
  for (int ipjp = 0; ipjp < p2; ipjp++) {
    const int ip = ipjp / np, jp = ipjp - ip * np;
    const size_t c0 = (size_t)(ipjp * ne + i1) * nsub;
    double ss = 0.0;
    for (int sb = lane; sb < nsub; sb += 32) ss += part[((c0 + sb) * nacc + a) * ne + j1];
    s = fma(DP[ip + np * jp], ss, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) fe_out[(size_t)a * n2 + i1 + ne * j1] = s;
}

// fp_out[t][ip + np*jp] = sum over the ne*nsub CTAs of (ipjp) of ppart;
// one block per (t, ipjp), fixed-order tree reduction.
__global__ void spin_reduce_p_kernel(int ne, int np, int nsub,
                                     const double* __restrict__ ppart,
                                     double* __restrict__ fp_out) {
  __shared__ double red[256];
  const int p2 = np * np;
  const int tn = blockIdx.x / p2, ipjp = blockIdx.x - tn * p2;
  const int ip = ipjp / np, jp = ipjp - ip * np;
  const size_t c0 = (size_t)ipjp * ne * nsub, nc = (size_t)ne * nsub;
  double s = 0.0;
  for (size_t c = threadIdx.x; c < nc; c += blockDim.x) s += ppart[(c0 + c) * 2 + tn];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) fp_out[(size_t)tn * p2 + ip + np * jp] = red[0];
}

// GAM_1 / GAM_1s contractions (FAE_OMG1, UFP_OMG1): GAM_1[ip][jp][ie][je].
//   fe_out[t][ie + ne*je] = sum_ipjp DP G_t;  fp_out[t][ip + np*jp] = sum W G_t
__global__ void omg1_kernel(int ne, int np, const double* __restrict__ G1,
                            const double* __restrict__ G1s,
                            const double* __restrict__ W,
                            const double* __restrict__ DP,
                            double* __restrict__ fe_out,
                            double* __restrict__ fp_out) {
  const int n2 = ne * ne, p2 = np * np;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2 * n2) {
    const int tn = t / n2, r = t - tn * n2, ie = r / ne, je = r - ie * ne;
    const double* g = tn ? G1s : G1;
    double s = 0.0;
    for (int ipjp = 0; ipjp < p2; ipjp++) {
      const int ip = ipjp / np, jp = ipjp - ip * np;
      s = fma(DP[ip + np * jp], g[(size_t)ipjp * n2 + ie * ne + je], s);
    }
    fe_out[(size_t)tn * n2 + ie + ne * je] = s;
  } else if (t < 2 * n2 + 2 * p2) {
    const int u = t - 2 * n2, tn = u / p2, ipjp = u - tn * p2;
    const int ip = ipjp / np, jp = ipjp - ip * np;
    const double* g = (tn ? G1s : G1) + (size_t)ipjp * n2;
    double s = 0.0;
    for (int ie = 0; ie < ne; ie++)
      for (int je = 0; je < ne; je++) s = fma(W[ie + ne * je], g[ie * ne + je], s);
    fp_out[(size_t)tn * p2 + ip + np * jp] = s;
  }
}

// Output stage: F (+)= scale * x, S = scale * xs (when given), E = sum W x,
// Es = sum W xs.  One CTA; deterministic block reduction.
__global__ void spin_finish_kernel(int n, const double* __restrict__ x,
                                   const double* __restrict__ xs,
                                   const double* __restrict__ W, double scale,
                                   double* F, double* S, double* E, double* Es) {
  __shared__ double red[2][256];
  const int n2 = n * n;
  double e = 0.0, es = 0.0;
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    if (F) F[k] += scale * x[k];
    e = fma(W[k], x[k], e);
    if (xs) {
      if (S) S[k] = scale * xs[k];
      es = fma(W[k], xs[k], es);
    }
  }
  red[0][threadIdx.x] = e;
  red[1][threadIdx.x] = es;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (E) *E = red[0][0];
    if (Es) *Es = red[1][0];
  }
}

// OMG4_ICR: GAM_4[index_GAM_4PK2 - 1] = calc_GAM_4_integral (the raw
// product element, gam_4_OMP.f:964-1192); one thread per element, stores
// coalesced along je4.
__device__ __forceinline__ double uflow(double x) {
  return fabs(x) < 1.0e-100 ? 0.0 : x;   // underflow.f:2-11
}

__global__ void __launch_bounds__(256)
omg4_icr_kernel(int ne, int np, long long ng4, const double* __restrict__ gee,
                const double* __restrict__ g2s, double* __restrict__ g4) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ng4) return;
  long long r = t;
  int xi[8];
  for (int m = 7; m >= 0; m--) {   // xi = (i1,j1,i2,j2,i3,j3,i4,j4)
    xi[m] = (int)(r % ne);
    r /= ne;
  }
  const long long ipjp = r;
  const long long n2 = (long long)ne * ne;
  // GAM_ee(pack_4D(je_b,ie_b,je_a,ie_a)) - 1 = je_b + ne (ie_b + ne (je_a + ne ie_a))
  auto ee = [&](int a, int b) {
    return uflow(__ldg(gee + xi[2 * b + 1] + ne * (xi[2 * b] + ne * (xi[2 * a + 1] +
                                                                   (long long)ne * xi[2 * a]))));
  };
  // GAM_2s(index_GAM_2PK(ip,jp,ie_a,je_a,ie_b,je_b)) - 1
  auto gs = [&](int a, int b) {
    return uflow(__ldg(g2s + xi[2 * b + 1] + ne * (xi[2 * b] + ne * (xi[2 * a + 1] +
                 (long long)ne * (xi[2 * a] + ne * ipjp)))));
  };
  (void)n2;
  // rounded products, no fused multiply-add: the same operations in the
  // same order as the reference's x1..x6 and their sum
  auto x = [&](int a, int b, int c, int d) {
    return __dmul_rn(__dmul_rn(0.5, ee(a, b)), gs(c, d));
  };
  const double s1 = __dadd_rn(x(2, 3, 0, 1), x(1, 3, 0, 2));
  const double s2 = __dadd_rn(s1, x(1, 2, 0, 3));
  const double s3 = __dadd_rn(s2, x(0, 3, 1, 2));
  const double s4 = __dadd_rn(s3, x(0, 2, 1, 3));
  g4[t] = __ddiv_rn(__dadd_rn(s4, x(0, 1, 2, 3)), 6.0);
}

}  // namespace

bool spin_smem_fits(int K, int ne) {
  if (ne < 1 || ne > kSpinThreads || pw(ne, K) > 65536) return false;
  int pt[4];
  const long long slab = ket_pitches(K, ne, pt);
  const int nten = K == 2 ? 2 : 1;
  return sizeof(double) * (2 * (size_t)ne * ne + nten * slab + kSpinThreads) <=
         200 * 1024;
}

namespace {

template <int K, bool SMEM>
cudaError_t launch_spin_kernel(int ne, int np, const double* G, const double* Gs,
                               const double* DA, const double* DB, unsigned fa,
                               unsigned fb, double* part, double* ppart, cudaStream_t s) {
  const int nten = (K == 2 && Gs) ? 2 : 1;
  const int lanes = kSpinThreads / ne;
  const int bs = ne * lanes;
  int pt[4];
  const size_t slabp = (size_t)ket_pitches(K, ne, pt);
  const size_t smem = sizeof(double) * (2 * (size_t)ne * ne + (SMEM ? nten * slabp : 0) + bs);
  cudaError_t e = cudaFuncSetAttribute(spin_kernel<K, SMEM>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long grid = (long long)np * np * ne * ne * (K >= 3 ? ne : 1);
  spin_kernel<K, SMEM><<<(unsigned)grid, bs, smem, s>>>(ne, np, G, Gs, DA, DB, fa,
                                                         fb, part, ppart);
  return cudaGetLastError();
}

}  // namespace

size_t spin_scratch_doubles(int K, int ne, int np) {
  const int nacc = K == 2 ? 4 : 2;
  const size_t ncta = (size_t)np * np * ne * ne * (K >= 3 ? ne : 1);
  return ncta * nacc * ne + ncta * 2;
}

cudaError_t launch_spin_omg(int K, int ne, int np, const double* G, const double* Gs,
                            const double* DA, const double* DB, const double* DP,
                            unsigned fa, unsigned fb, double* scratch,
                            double* fe_out, double* fp_out, cudaStream_t s) {
  if (ne < 1 || ne > kSpinThreads || np < 1 || K < 2 || K > 4 || (K != 2 && Gs))
    return cudaErrorInvalidValue;
  const int nacc = (K == 2 && Gs) ? 4 : 2;
  const size_t ncta = (size_t)np * np * ne * ne * (K >= 3 ? ne : 1);
  double* part = scratch;
  double* ppart = scratch + ncta * (K == 2 ? 4 : 2) * ne;
  cudaError_t e;
  const bool fits = spin_smem_fits(K, ne);
  if (K == 2)
    e = fits ? launch_spin_kernel<2, true>(ne, np, G, Gs, DA, DB, fa, fb, part, ppart, s)
             : launch_spin_kernel<2, false>(ne, np, G, Gs, DA, DB, fa, fb, part, ppart, s);
  else if (!fits)   // ranks 3 and 4 stage the whole ket block
    return cudaErrorInvalidValue;
  else if (K == 3)
    e = launch_spin_kernel<3, true>(ne, np, G, nullptr, DA, DB, fa, fb, part, ppart, s);
  else
    e = launch_spin_kernel<4, true>(ne, np, G, nullptr, DA, DB, fa, fb, part, ppart, s);
  if (e != cudaSuccess) return e;
  const int nsub = K == 2 ? ne : ne * ne;
  const int ne_out = nacc * ne * ne;
  spin_reduce_e_kernel<<<(ne_out + 3) / 4, 128, 0, s>>>(ne, np, nacc, nsub, part, DP,
                                                        fe_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  spin_reduce_p_kernel<<<(nacc / 2) * np * np, 256, 0, s>>>(ne, np, nsub, ppart, fp_out);
  return cudaGetLastError();
}

cudaError_t launch_omg1(int ne, int np, const double* G1, const double* G1s,
                        const double* W, const double* DP, double* fe_out,
                        double* fp_out, cudaStream_t s) {
  if (ne < 1 || np < 1) return cudaErrorInvalidValue;
  const int nout = 2 * ne * ne + 2 * np * np;
  omg1_kernel<<<(nout + 127) / 128, 128, 0, s>>>(ne, np, G1, G1s, W, DP, fe_out, fp_out);
  return cudaGetLastError();
}

cudaError_t launch_spin_finish(int n, const double* x, const double* xs,
                               const double* W, double scale, double* F, double* S,
                               double* E, double* Es, cudaStream_t s) {
  spin_finish_kernel<<<1, 256, 0, s>>>(n, x, xs, W, scale, F, S, E, Es);
  return cudaGetLastError();
}

cudaError_t launch_omg4_icr(int ne, int np, const double* gee, const double* g2s,
                            double* g4, cudaStream_t s) {
  if (ne < 1 || np < 1) return cudaErrorInvalidValue;
  const long long ng4 = pw(ne, 8) * np * np;
  const long long grid = (ng4 + 255) / 256;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
  omg4_icr_kernel<<<(unsigned)grid, 256, 0, s>>>(ne, np, ng4, gee, g2s, g4);
  return cudaGetLastError();
}

}  // namespace neoxc
