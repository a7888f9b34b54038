// k_gam3.cu -- the four-particle part of the gam_3 builder on sm_103a.
//
// Reference: gam_3_OMP.f:617-984 (xcalc_GAM3_MD), gam3_CONV_OMP.f:479-705
// (contract_omega3_conv), gam3_IC1_OMP.f:299-431 (thread_gam3_IC1),
// XC1_G4_MD.f:796-1125 (G4_MD_xgVeeg), :1559-1978 (G4_MD_xgVepg).
//
// xcalc_GAM3_MD's integrand is gVEE + gHEg + gVEEg1/2 + 2 gVEEg2 (:964).
// Its separable terms are contracted once per system in k_md.cu (W1 x
// GAM_ee + W3 x Hcore); what remains per primitive 8-tuple is
//   g4part = sum_kl b_k b_l (2 G4Vee(e1,e2,e3,p) - G4Vep(e1,e2,e3,p))
// (:846, :930).  Two structural facts make it cheap on the GPU:
//
//  1. Every operator in g4part is multiplicative (geminals, Coulomb), so it
//     depends on each particle only through its pair density phi_i phi_j:
//     the contracted sum R4 is unchanged when the bra and ket of any one
//     particle are swapped.  R4 is computed once per pair-canonical tuple
//     (i1>=j1, i2>=j2, i3>=j3, ip>=jp) and gam3_expand_kernel gathers it
//     onto the packed index_GAM_3PK order with the separable terms
//     ((n(n+1)/2)^3 m(m+1)/2 tuples instead of n^6 m^2: 11x fewer at
//     nebf=12, npbf=8).
//
//  2. In G4Vep the Coulomb operator joins e3 and p and no geminal touches
//     e3; in G4Vee it joins e1 and e2 and no geminal touches e2.  Each is a
//     two-centre Coulomb integral between a composite "bra" (the other
//     three pair densities with both geminals integrated out by Boys'
//     lemma: one Gaussian times a polynomial, Hermite vectors W'_d per
//     Cartesian direction) and the "ket" pair density of the free electron
//     (Hermite vector E_d): the derivative table of the reference's kernel
//     does not depend on the free electron's centre, so its binomial fold
//     collapses to a 1-D convolution of W'_d with (-1)^t E_d.  The bra does
//     not depend on the ket, so a CTA builds the bras of one canonical
//     (proton pair, electron pair, electron pair) -- every primitive pair and
//     geminal pair -- once in shared memory and sweeps all primitive-pair
//     kets against them.  Per (bra, ket) (g3_fatbra.cuh fb_eval):
//       W_d = W'_d (*) (-1)^t E_d                 (1-D convolutions)
//       S   = sum_{t,u,v} W_x[t] W_y[u] W_z[v] R_tuv(alpha, R)
//           = sum_m (-alpha)^m F_m(T) sum_{i+j+k=m} A_x[i] A_y[j] A_z[k],
//       A_d[i] = sum_t W_d[t] C(t,i) 2^(2i-t) R_d^(2i-t),
//     the Hermite-Coulomb sum in factorised form, O(L^2) work instead of
//     the O(L^4) R_tuv table; the seeds (-alpha)^m F_m(T) and their final
//     sum are FP64 in both precisions.
//
// The prefactors, exponents and centres follow G4_MD_xgVepg / G4_MD_xgVeeg
// (truncated pi, the reference's underflow on every G4Vep value); only the
// summation order differs from the element-wise evaluation.
//
// Kernels are instantiated per angular-momentum class (LE = largest l of an
// electronic primitive, LN of a nuclear one), so every table is sized for
// the class.  Optional screening (screen > 0, new; the reference evaluates
// every tuple): per primitive pair the overlap magnitude S (|c_a c_b|
// (pi/p)^(3/2) K_ab times an angular factor) and the Schwarz factor
// Q = |c_a c_b| sqrt((ab|ab)).  Integrating the geminal-coupled particles
// out bounds their factors by S and the Coulomb pair by Schwarz:
//   |G4Vep| <~ S1 S2 Q3 Qp,   |G4Vee| <~ S3 Sp Q1 Q2
// (a bound for s functions, an estimate for p/d); a (bra, ket) whose
// estimate times sum_kl |b_k b_l| falls below `screen` is skipped.
//
// Many systems (launch_gam3_batch_pairs): the blocks of one angular class
// from every system and both passes form one work space that a persistent
// grid drains through a device counter (gam3_fb_persistent); the per-block
// arithmetic is that of gam3_fb_kernel, so each system's R4 is bit-identical
// to its separate build.
#include <type_traits>
#include <vector>

#include "g3_fatbra.cuh"
#include "neoxc_internal.h"

namespace neoxc {
namespace {

using namespace g3;

__device__ __forceinline__ md::Prim to_md(const DevPrim& d) {
  md::Prim p;
  p.a = d.a;
  for (int k = 0; k < 3; k++) {
    p.c[k] = d.c[k];
    p.l[k] = d.l[k];
  }
  return p;
}

__device__ __forceinline__ void unpair(int P, int& i, int& j) {
  int a = (int)((sqrtf(8.0f * (float)P + 1.0f) - 1.0f) * 0.5f);
  while (a * (a + 1) / 2 > P) a--;
  while ((a + 1) * (a + 2) / 2 <= P) a++;
  i = a;
  j = P - a * (a + 1) / 2;
}

// Records of every canonical electronic primitive pair (ket order) and every
// canonical nuclear pair.
__global__ void g3_records_kernel(DevSystem S, double* __restrict__ erec,
                                  double* __restrict__ prec) {
  const int nket = S.g3_nket;
  const int nPp = S.npbf * (S.npbf + 1) / 2;
  const int* ket_ab = S.g3i;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nket + nPp;
       t += gridDim.x * blockDim.x) {
    const DevPrim* pa;
    const DevPrim* pb;
    double* out;
    if (t < nket) {
      pa = S.eprim + ket_ab[2 * t];
      pb = S.eprim + ket_ab[2 * t + 1];
      out = erec + (size_t)kRLen * t;
    } else {
      int ip, jp;
      unpair(t - nket, ip, jp);
      pa = S.pprim + ip;
      pb = S.pprim + jp;
      out = prec + (size_t)kRLen * (t - nket);
    }
    fill_pair_record(to_md(*pa), to_md(*pb), pa->coef, pb->coef, out);
  }
}

constexpr int kFbThreads = 128;   // threads (and bras per chunk) of a CTA

// One CTA's work: block blk (Pp, Pa, Pb) and ket tile `tile` of one pass.
// MODE 0: G4Vep, (Pp, P1, P2), kets e3 -> R4[Pp][P1][P2][P3]  = -sum
// MODE 1: G4Vee, (Pp, P1, P3), kets e2 -> R4[Pp][P1][P2][P3] += 2 sum
//         (or = 2 sum when store1: the batched launch keeps the two passes
//         in separate arrays and adds them afterwards).
// Each element has one owner CTA per pass, so results are deterministic.
template <bool F32, int LE, int LN, int MODE>
__device__ __forceinline__ void fb_block(const DevSystem& S, const double* __restrict__ erec,
                                         const double* __restrict__ prec, double screen,
                                         double* __restrict__ r4, long long blk, int tile,
                                         unsigned char* smraw, bool store1) {
  using R = typename std::conditional<F32, float, double>::type;
  constexpr int NW = 4 * LE + 2 * LN;   // bra Hermite order per direction
  constexpr int NK = 2 * LE;            // ket Hermite order per direction
  __syncthreads();   // the previous block's reads of the shared tables are done
  Bra<R, NW>* bras = reinterpret_cast<Bra<R, NW>*>(smraw);
  double* acc_s = reinterpret_cast<double*>(smraw + sizeof(Bra<R, NW>) * kFbThreads);

  const int ne = S.nebf;
  const int nPe = ne * (ne + 1) / 2;
  const int* kofs = S.g3i + 2 * S.g3_nket;          // [nPe + 1]
  const int* tile_k = kofs + nPe + 1;               // [ntile + 1]
  const int* tile_P = tile_k + S.g3_ntile + 1;      // [ntile + 1]
  const int* kperm = tile_P + S.g3_ntile + 1;       // [nket]
  long long r = blk;
  const int Pb = (int)(r % nPe); r /= nPe;
  const int Pa = (int)(r % nPe); r /= nPe;
  const int Pp = (int)r;
  const int k0 = tile_k[tile], nkt = tile_k[tile + 1] - k0;
  const int P0 = tile_P[tile], P1t = tile_P[tile + 1];
  const int ka = kofs[Pa], na = kofs[Pa + 1] - ka;
  const int kb = kofs[Pb], nb = kofs[Pb + 1] - kb;
  const int ng = S.ngtg;
  const int nbra = na * nb * ng * ng;
  const double* rp = prec + (size_t)kRLen * Pp;
  double wsum = 0.0;
  if (screen > 0.0)
    for (int k = 0; k < ng; k++)
      for (int l = 0; l < ng; l++) wsum += fabs(S.bgem[k] * S.bgem[l]);

  for (int k = threadIdx.x; k < nkt; k += blockDim.x) acc_s[k] = 0.0;
  for (int c0 = 0; c0 < nbra; c0 += kFbThreads) {
    const int nvalid = nbra - c0 < kFbThreads ? nbra - c0 : kFbThreads;
    __syncthreads();
    if ((int)threadIdx.x < nvalid) {
      int q = c0 + threadIdx.x;
      const int l = q % ng; q /= ng;
      const int k = q % ng; q /= ng;
      const int ub = q % nb;
      const int ua = q / nb;
      const double* ra = erec + (size_t)kRLen * (ka + ua);
      const double* rb = erec + (size_t)kRLen * (kb + ub);
      Bra<R, NW> b;
      if constexpr (MODE == 0)
        build_bra_vep<R, LE, LN, NW>(ra, rb, rp, (R)S.ggem[k], (R)S.ggem[l], b);
      else
        build_bra_vee<R, LE, LN, NW>(ra, rb, rp, (R)S.ggem[k], (R)S.ggem[l], b);
      b.wgt = (MODE == 0 ? -1.0 : 2.0) * (S.bgem[k] * S.bgem[l]) * ra[kRC] * rb[kRC] *
              rp[kRC];
      // Vep: S1 S2 Qp (x Q3 of the ket); Vee: Q1 S3 Sp (x Q2 of the ket)
      b.est = wsum * (MODE == 0 ? ra[kRS] * rb[kRS] * rp[kRQ]
                                : 2.0 * ra[kRQ] * rb[kRS] * rp[kRS]);
      bras[threadIdx.x] = b;
    }
    __syncthreads();
    for (int kk = threadIdx.x; kk < nkt; kk += blockDim.x) {
      const int kid = kperm[k0 + kk];
      const double* rk = erec + (size_t)kRLen * kid;
      const R pk = (R)rk[kRP];
      R Xk[3], Ek[3][NK + 1];
      int tk[3];
      for (int d = 0; d < 3; d++) {
        Xk[d] = (R)rk[kRX + d];
        tk[d] = (int)rk[kRT + d];
        for (int t = 0; t <= NK; t++)
          Ek[d][t] = (t & 1) ? -(R)rk[kRE + 5 * d + t] : (R)rk[kRE + 5 * d + t];
      }
      const double qk = rk[kRQ];
      const double rkc = rk[kRC];
      double part = 0.0;
      for (int bi = 0; bi < nvalid; bi++) {
        const Bra<R, NW>& b = bras[bi];
        if (screen > 0.0 && b.est * qk < screen) continue;
        double v = fb_eval<R, NW, NK>(b, pk, Xk, Ek, tk);
        if (MODE == 0) v = md::underflow(v);   // zz = underflow(G4_MD_xgVepg)
        part += b.wgt * v;
      }
      acc_s[kid - k0] += part * rkc;
    }
  }
  __syncthreads();
  const long long nP = nPe;
  for (int P = P0 + threadIdx.x; P < P1t; P += blockDim.x) {
    double s = 0.0;
    for (int k = kofs[P]; k < kofs[P + 1]; k++) s += acc_s[k - k0];
    if (MODE == 0)
      r4[((Pp * nP + Pa) * nP + Pb) * nP + P] = s;
    else if (store1)
      r4[((Pp * nP + Pa) * nP + P) * nP + Pb] = s;
    else
      r4[((Pp * nP + Pa) * nP + P) * nP + Pb] += s;
  }
}

template <bool F32, int LE, int LN, int MODE>
__global__ void __launch_bounds__(kFbThreads, 4)
gam3_fb_kernel(DevSystem S, const double* __restrict__ erec,
               const double* __restrict__ prec, double screen,
               double* __restrict__ r4) {
  extern __shared__ __align__(16) unsigned char smraw[];
  fb_block<F32, LE, LN, MODE>(S, erec, prec, screen, r4, (long long)blockIdx.x, blockIdx.y,
                              smraw, false);
}

// ---- many systems in one persistent launch ----------------------------------
// Work items are numbered over groups g = 2 s + mode (system s, pass mode):
// group g holds nblk_s x ntile_s items, first item prefix[g].  Each CTA
// takes chunks of `chunk` consecutive items from an atomic counter until
// the items run out (or `limit`, for the autotuner's samples).
template <bool F32, int LE, int LN>
__global__ void __launch_bounds__(kFbThreads, 4)
gam3_fb_persistent(const G3BatchSys* __restrict__ sys, const long long* __restrict__ prefix,
                   int ngroups, int chunk, long long limit, double screen,
                   unsigned long long* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ long long s_item;
  const long long total = prefix[ngroups] < limit ? prefix[ngroups] : limit;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ULL) * chunk;
    __syncthreads();
    const long long first = s_item;
    if (first >= total) break;
    const long long last = first + chunk < total ? first + chunk : total;
    for (long long it = first; it < last; it++) {
      int lo = 0, hi = ngroups - 1;   // the group holding item `it`
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= it) lo = mid; else hi = mid - 1;
      }
      const G3BatchSys& b = sys[lo >> 1];
      const long long local = it - prefix[lo];
      const int tile = (int)(local % b.S.g3_ntile);
      const long long blk = local / b.S.g3_ntile;
      if ((lo & 1) == 0)
        fb_block<F32, LE, LN, 0>(b.S, b.erec, b.prec, screen, b.r4a, blk, tile, smraw, false);
      else
        fb_block<F32, LE, LN, 1>(b.S, b.erec, b.prec, screen, b.r4b, blk, tile, smraw, true);
    }
  }
}

// r4a += r4b (the two passes of the batched launch)
__global__ void add_kernel(long long n, double* __restrict__ a, const double* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] += b[i];
}



// x3[w] = R4(canonical tuple of t0 + w) + W1(p,e1) GAM_ee(e2,e3) + W3(p,e1,e2) Hcore(e3)
__global__ void gam3_expand_kernel(int ne, int np, const double* __restrict__ aux,
                                   double* __restrict__ x3, long long t0, long long n) {
  const long long n2 = (long long)ne * ne, n4 = n2 * n2;
  const double* gee = aux;
  const double* hc = gee + n4;
  const double* W1 = hc + n2;
  const double* W3 = W1 + (long long)np * np * n2;
  const double* R4 = W3 + (long long)np * np * n4;
  const long long nPe = (long long)ne * (ne + 1) / 2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    long long r = t + t0;
    int c[6];
    for (int k = 5; k >= 0; k--) {
      c[k] = (int)(r % ne);
      r /= ne;
    }
    const int jp = (int)(r % np);
    const int ip = (int)(r / np);
    const long long Pp = pair_index(ip, jp);
    const long long cr =
        ((Pp * nPe + pair_index(c[0], c[1])) * nPe + pair_index(c[2], c[3])) * nPe +
        pair_index(c[4], c[5]);
    const long long pp = (long long)ip * np + jp;
    const double w1 = W1[(pp * ne + c[0]) * ne + c[1]];
    const double w3 = W3[(((pp * ne + c[0]) * ne + c[1]) * ne + c[2]) * ne + c[3]];
    const double ee = gee[((c[2] * (long long)ne + c[3]) * ne + c[4]) * ne + c[5]];
    const double h = hc[c[4] * ne + c[5]];
    x3[t] = R4[cr] + w1 * ee + w3 * h;
  }
}

template <bool F32, int LE, int LN>
cudaError_t persistent_t(const G3BatchSys* d_sys, const long long* d_prefix, int ngroups,
                         int chunk, long long limit, double screen,
                         unsigned long long* d_counter, int ctas_per_sm, cudaStream_t s) {
  using R = typename std::conditional<F32, float, double>::type;
  constexpr int NW = 4 * LE + 2 * LN;
  const size_t smem = sizeof(Bra<R, NW>) * kFbThreads + sizeof(double) * kG3MaxTileKets;
  cudaError_t e = cudaFuncSetAttribute(gam3_fb_persistent<F32, LE, LN>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, occ = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gam3_fb_persistent<F32, LE, LN>,
                                                         kFbThreads, smem)) != cudaSuccess)
    return e;
  const int per_sm = ctas_per_sm < 1 ? 1 : (ctas_per_sm > occ ? (occ > 0 ? occ : 1) : ctas_per_sm);
  gam3_fb_persistent<F32, LE, LN><<<nsm * per_sm, kFbThreads, smem, s>>>(
      d_sys, d_prefix, ngroups, chunk, limit, screen, d_counter);
  return cudaGetLastError();
}

template <bool F32>
cudaError_t persistent_dispatch(int le, int lp, const G3BatchSys* d_sys,
                                const long long* d_prefix, int ngroups, int chunk,
                                long long limit, double screen, unsigned long long* d_counter,
                                int ctas_per_sm, cudaStream_t s) {
  const int LN = lp == 0 ? 0 : 2;
#define PD(a, b) persistent_t<F32, a, b>(d_sys, d_prefix, ngroups, chunk, limit, screen, \
                                         d_counter, ctas_per_sm, s)
  switch (le * 3 + LN) {
    case 0: return PD(0, 0);
    case 2: return PD(0, 2);
    case 3: return PD(1, 0);
    case 5: return PD(1, 2);
    case 6: return PD(2, 0);
    case 8: return PD(2, 2);
    default: return cudaErrorInvalidValue;
  }
#undef PD
}

template <bool F32, int LE, int LN>
cudaError_t fb_t(const DevSystem& sys, const double* erec, const double* prec,
                 double screen, double* r4, cudaStream_t s) {
  using R = typename std::conditional<F32, float, double>::type;
  constexpr int NW = 4 * LE + 2 * LN;
  const size_t smem = sizeof(Bra<R, NW>) * kFbThreads + sizeof(double) * kG3MaxTileKets;
  const int nPe = sys.nebf * (sys.nebf + 1) / 2;
  const int nPp = sys.npbf * (sys.npbf + 1) / 2;
  const long long nblk = (long long)nPp * nPe * nPe;
  if (nblk > 0x7fffffffLL || sys.g3_ntile > 65535) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)nblk, (unsigned)sys.g3_ntile);
  cudaError_t e = cudaFuncSetAttribute(gam3_fb_kernel<F32, LE, LN, 0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(gam3_fb_kernel<F32, LE, LN, 1>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  gam3_fb_kernel<F32, LE, LN, 0><<<grid, kFbThreads, smem, s>>>(sys, erec, prec, screen, r4);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  gam3_fb_kernel<F32, LE, LN, 1><<<grid, kFbThreads, smem, s>>>(sys, erec, prec, screen, r4);
  return cudaGetLastError();
}

template <bool F32>
cudaError_t fb_dispatch(const DevSystem& sys, const double* erec, const double* prec,
                        double screen, double* r4, cudaStream_t s) {
  const int LE = sys.lmax_e, LN = sys.lmax_p == 0 ? 0 : 2;
  switch (LE * 3 + LN) {
    case 0: return fb_t<F32, 0, 0>(sys, erec, prec, screen, r4, s);
    case 2: return fb_t<F32, 0, 2>(sys, erec, prec, screen, r4, s);
    case 3: return fb_t<F32, 1, 0>(sys, erec, prec, screen, r4, s);
    case 5: return fb_t<F32, 1, 2>(sys, erec, prec, screen, r4, s);
    case 6: return fb_t<F32, 2, 0>(sys, erec, prec, screen, r4, s);
    case 8: return fb_t<F32, 2, 2>(sys, erec, prec, screen, r4, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

size_t gam3_r4_doubles(int ne, int np) {
  const size_t nPe = (size_t)ne * (ne + 1) / 2, nPp = (size_t)np * (np + 1) / 2;
  return nPp * nPe * nPe * nPe;
}

size_t gam3_aux_doubles(int ne, int np) {
  const size_t n2 = (size_t)ne * ne;
  return n2 * n2 + n2 + (size_t)np * np * n2 + (size_t)np * np * n2 * n2 +
         gam3_r4_doubles(ne, np);
}

size_t gam3_batch_scratch_bytes(int nsys) {
  return sizeof(G3BatchSys) * (size_t)nsys + sizeof(long long) * (2 * (size_t)nsys + 1) + 64;
}

cudaError_t launch_gam3_batch_pairs(const G3BatchSys* h_sys, int nsys, int fp32, double screen,
                                    void* scratch, int ctas_per_sm, int chunk, long long limit,
                                    long long* total_items, cudaStream_t s) {
  if (nsys < 1 || chunk < 1) return cudaErrorInvalidValue;
  const int le = h_sys[0].S.lmax_e, lp = h_sys[0].S.lmax_p;
  std::vector<long long> prefix(2 * (size_t)nsys + 1, 0);
  for (int k = 0; k < nsys; k++) {
    const DevSystem& S = h_sys[k].S;
    if (S.lmax_e != le || (S.lmax_p == 0) != (lp == 0) || S.g3_ntile < 1 || !S.g3i || !S.g3rec)
      return cudaErrorInvalidValue;   // one angular class per launch
    const long long nPe = (long long)S.nebf * (S.nebf + 1) / 2;
    const long long nPp = (long long)S.npbf * (S.npbf + 1) / 2;
    const long long items = nPp * nPe * nPe * S.g3_ntile;
    prefix[2 * k + 1] = prefix[2 * k] + items;
    prefix[2 * k + 2] = prefix[2 * k + 1] + items;
  }
  if (total_items) *total_items = prefix[2 * nsys];
  unsigned char* p = static_cast<unsigned char*>(scratch);
  G3BatchSys* d_sys = reinterpret_cast<G3BatchSys*>(p);
  long long* d_prefix = reinterpret_cast<long long*>(p + sizeof(G3BatchSys) * (size_t)nsys);
  unsigned long long* d_counter =
      reinterpret_cast<unsigned long long*>(d_prefix + 2 * (size_t)nsys + 1);
  cudaError_t e = cudaMemcpyAsync(d_sys, h_sys, sizeof(G3BatchSys) * (size_t)nsys,
                                  cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(d_prefix, prefix.data(), sizeof(long long) * prefix.size(),
                      cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  // the host vectors are released when this returns: make the copies land
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  const long long lim = limit < 0 ? prefix[2 * nsys] : limit;
  return fp32 ? persistent_dispatch<true>(le, lp, d_sys, d_prefix, 2 * nsys, chunk, lim, screen,
                                          d_counter, ctas_per_sm, s)
              : persistent_dispatch<false>(le, lp, d_sys, d_prefix, 2 * nsys, chunk, lim, screen,
                                           d_counter, ctas_per_sm, s);
}

cudaError_t launch_gam3_add(long long n, double* a, const double* b, cudaStream_t s) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  add_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, a, b);
  return cudaGetLastError();
}

size_t g3_record_doubles(int nket, int np) {
  return (size_t)kRLen * ((size_t)nket + (size_t)np * (np + 1) / 2);
}

cudaError_t launch_g3_records(const DevSystem& sys, double* rec, cudaStream_t s) {
  const int n = sys.g3_nket + sys.npbf * (sys.npbf + 1) / 2;
  int blocks = (n + 127) / 128;
  if (blocks > 152 * 8) blocks = 152 * 8;
  g3_records_kernel<<<blocks, 128, 0, s>>>(sys, rec, rec + (size_t)kRLen * sys.g3_nket);
  return cudaGetLastError();
}

cudaError_t launch_gam3_pairs(const DevSystem& sys, double* aux, cudaStream_t s, int fp32,
                              double screen) {
  const int ne = sys.nebf, np = sys.npbf;
  if (sys.lmax_e < 0 || sys.lmax_e > 2 || sys.lmax_p < 0 || sys.lmax_p > 2 ||
      !sys.g3rec || !sys.g3i || sys.g3_ntile < 1)
    return cudaErrorInvalidValue;
  const size_t n2 = (size_t)ne * ne;
  double* r4 = aux + n2 * n2 + n2 + (size_t)np * np * n2 + (size_t)np * np * n2 * n2;
  const double* erec = sys.g3rec;
  const double* prec = sys.g3rec + (size_t)kRLen * sys.g3_nket;
  return fp32 ? fb_dispatch<true>(sys, erec, prec, screen, r4, s)
              : fb_dispatch<false>(sys, erec, prec, screen, r4, s);
}

cudaError_t launch_gam3_raw_range(const DevSystem& sys, const double* aux,
                                  long long t0, long long ntup, double* x3,
                                  cudaStream_t s) {
  if (ntup <= 0) return cudaSuccess;
  long long blocks = (ntup + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  gam3_expand_kernel<<<(unsigned)blocks, 256, 0, s>>>(sys.nebf, sys.npbf, aux, x3, t0, ntup);
  return cudaGetLastError();
}

cudaError_t launch_gam3_raw(const DevSystem& sys, double* aux, double* x3,
                            cudaStream_t s, int fp32, double screen) {
  cudaError_t e = launch_gam3_pairs(sys, aux, s, fp32, screen);
  if (e != cudaSuccess) return e;
  const long long n6 = (long long)sys.nebf * sys.nebf * sys.nebf * sys.nebf *
                       sys.nebf * sys.nebf;
  return launch_gam3_raw_range(sys, aux, 0, n6 * sys.npbf * sys.npbf, x3, s);
}

}  // namespace neoxc
