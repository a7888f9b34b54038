// k_contract.cu -- in-core Fock/energy contractions for sm_103a and the
// deterministic partial-sum reducer shared by every contraction kernel.
//
// Reference: gam2_IC1_OMP.f:339-570 (EG2IC1 / thread_EG2ICR),
// gam3_IC1_OMP.f:433-725 (EG3IC1 / thread_EG3ICR), rxchfne/rxchfne_omg2.f
// (RXCHFne_FAE/FP/FBE_OMG2), xchf1_independent/xchf1_fock.f:728-783
// (XCfock_correction), CS_Integrals/Spot_Check/pack_GAM.f (index maps).
//
// All kernels here are HBM-bound streams over the stored integral tensor:
// every element is read from HBM once, permuted partners are gathered from
// shared memory, and partial sums are written per CTA and reduced by a
// second, deterministic kernel (no floating-point atomics), so repeated
// calls give bit-identical results.
#include "neoxc_internal.h"

namespace neoxc {

// part[((ipjp*ne + i1)*nsub + s)*ne + j1] -> Fock/energy.
//   fe(i1,j1) (+)= fe_scale * sum_{ipjp} DP(ipjp) * sum_s part
//   fp(ipjp)  (+)= sum_{i1,j1} DE(i1,j1) * sum_s part
//   fp_tmp[ipjp] = DP(ipjp) * [that fp contribution]   (energy terms)
__global__ void fock_reduce_kernel(int ne, int np, int nsub,
                                   const double* __restrict__ part,
                                   const double* __restrict__ DE,
                                   const double* __restrict__ DP,
                                   double fe_scale, int accumulate,
                                   double* fe, double* fp, double* fp_tmp) {
  const int n2 = ne * ne, p2 = np * np;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n2) {
    int i1 = t / ne, j1 = t % ne;
    double s = 0.0;
    for (int ipjp = 0; ipjp < p2; ipjp++) {
      int ip = ipjp / np, jp = ipjp % np;
      double ss = 0.0;
      for (int k = 0; k < nsub; k++)
        ss += part[((size_t)(ipjp * ne + i1) * nsub + k) * ne + j1];
      s = fma(DP[ip + np * jp], ss, s);
    }
    if (fe) {
      if (accumulate) fe[i1 + ne * j1] += fe_scale * s;
      else fe[i1 + ne * j1] = fe_scale * s;
    }
  } else if (t < n2 + p2) {
    int ipjp = t - n2, ip = ipjp / np, jp = ipjp % np;
    double s = 0.0;
    for (int i1 = 0; i1 < ne; i1++)
      for (int j1 = 0; j1 < ne; j1++) {
        double ss = 0.0;
        for (int k = 0; k < nsub; k++)
          ss += part[((size_t)(ipjp * ne + i1) * nsub + k) * ne + j1];
        s = fma(DE[i1 + ne * j1], ss, s);
      }
    if (fp) {
      if (accumulate) fp[ip + np * jp] += s;
      else fp[ip + np * jp] = s;
    }
    fp_tmp[ipjp] = s * DP[ip + np * jp];
  }
}

__global__ void sum_vec_kernel(int n, const double* __restrict__ v,
                               double* out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) s += v[k];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

cudaError_t launch_fock_reduce(int ne, int np, int nsub, const double* part,
                               const double* DE, const double* DP,
                               double fe_scale, int accumulate, double* fe,
                               double* fp, double* fp_tmp, double* E,
                               cudaStream_t s) {
  const int nout = ne * ne + np * np;
  fock_reduce_kernel<<<(nout + 127) / 128, 128, 0, s>>>(
      ne, np, nsub, part, DE, DP, fe_scale, accumulate, fe, fp, fp_tmp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_vec_kernel<<<1, 256, 0, s>>>(np * np, fp_tmp, E);
  return cudaGetLastError();
}

namespace {

// ---- EG3IC1 --------------------------------------------------------------
// CTA per (ip,jp,i1,i2,i3): the ne^3 ket values G3(i1,x;i2,y;i3,z) are
// staged in shared memory (one HBM read per element), then each thread
// forms GAM3 for its (j1,j2,j3) from the six ket permutations.
__global__ void __launch_bounds__(256)
eg3_kernel(int ne, int np, const double* __restrict__ DE,
           const double* __restrict__ g3, double* __restrict__ part,
           long long ipjp0) {
  extern __shared__ double sm[];
  const int n2 = ne * ne, n3 = n2 * ne;
  double* sG = sm;           // [x][y][z] = G3(i1,x,i2,y,i3,z)
  double* sDE = sm + n3;
  double* sred = sDE + n2;
  int cta = blockIdx.x;
  const int i3 = cta % ne; cta /= ne;
  const int i2 = cta % ne; cta /= ne;
  const int i1 = cta % ne; cta /= ne;
  const long long ipjp = cta;   // relative to the slice g3 points at
  for (int k = threadIdx.x; k < n2; k += blockDim.x) sDE[k] = DE[k];
  // index_GAM_3PK(ip,jp,i1,x,i2,y,i3,z)-1 = z + ne*(i3 + ne*(y + ne*(i2 +
  //   ne*(x + ne*(i1 + ne*ipjp)))))
  for (int k = threadIdx.x; k < n3; k += blockDim.x) {
    int x = k / n2, r = k - x * n2, y = r / ne, z = r - y * ne;
    long long o = z + (long long)ne * (i3 + (long long)ne * (y + (long long)ne * (i2 +
                  (long long)ne * (x + (long long)ne * (i1 + (long long)ne * ipjp)))));
    sG[k] = __ldg(g3 + o);
  }
  __syncthreads();
  const int lanes = blockDim.x / ne;
  const int j1 = threadIdx.x % ne;
  double acc = 0.0;
  for (int q = threadIdx.x / ne; q < n2; q += lanes) {
    const int j2 = q / ne, j3 = q - j2 * ne;
#define G(a, b, c) sG[(a) * n2 + (b) * ne + (c)]
    double o123 = G(j1, j2, j3), o213 = G(j2, j1, j3), o312 = G(j3, j1, j2);
    double o132 = G(j1, j3, j2), o231 = G(j2, j3, j1), o321 = G(j3, j2, j1);
#undef G
    double g = 8.0 * o123 - 4.0 * o213 + 2.0 * o312 - 4.0 * o132 +
               2.0 * o231 - 4.0 * o321;
    g = g / 8.0;
    acc = fma(sDE[i2 + ne * j2] * sDE[i3 + ne * j3], g, acc);
  }
  sred[threadIdx.x] = acc;
  __syncthreads();
  if ((int)threadIdx.x < ne) {
    double s = 0.0;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += ne) s += sred[t];
    part[((size_t)blockIdx.x + (size_t)ipjp0 * n3) * ne + threadIdx.x] = s;
  }
}

// ---- EG2IC1 --------------------------------------------------------------
// CTA per (ip,jp,i1,i2); thread per j1 (strided), loop over j2.
__global__ void eg2_kernel(int ne, int np, const double* __restrict__ DE,
                           const double* __restrict__ g2,
                           const double* __restrict__ g2s,
                           double* __restrict__ pv, double* __restrict__ ps,
                           long long ipjp0) {
  int cta = blockIdx.x;
  const int i2 = cta % ne; cta /= ne;
  const int i1 = cta % ne; cta /= ne;
  const long long ipjp = cta;
  for (int j1 = threadIdx.x; j1 < ne; j1 += blockDim.x) {
    double av = 0.0, as = 0.0;
    for (int j2 = 0; j2 < ne; j2++) {
      // a12 = (i1,j1,i2,j2), a21 = (i1,j2,i2,j1)
      long long b1 = i1 + (long long)ne * ipjp;
      long long a12 = j2 + (long long)ne * (i2 + (long long)ne * (j1 + (long long)ne * b1));
      long long a21 = j1 + (long long)ne * (i2 + (long long)ne * (j2 + (long long)ne * b1));
      double v = g2[a12] - 0.5 * g2[a21];
      double vs = g2s[a12] - 0.5 * g2s[a21];
      double d = DE[i2 + ne * j2];
      av = fma(d, v, av);
      as = fma(d, vs, as);
    }
    const size_t c = (size_t)blockIdx.x + (size_t)ipjp0 * ne * ne;
    pv[c * ne + j1] = av;
    ps[c * ne + j1] = as;
  }
}

// ---- RXCHF-ne OMG2 (fused FAE / FP / FBE / energy) -----------------------
// GM2ICR viewed as M[r][c], r = (ip,jp,i1,j1), c = (i2,j2) (c fastest).
//   FAE[c]     += sum_r DP(ip,jp) DBE(i1,j1) M[r][c]
//   v[r]        = sum_c DAE[c] M[r][c]
//   FBE(i1,j1) += sum_{ip,jp} DP v[r];  FP(ip,jp) += sum_{i1,j1} DBE v[r]
constexpr int kOmgRows = 8;
__global__ void __launch_bounds__(256)
omg2_kernel(int ne, int np, long long nrows, int rows_per_cta,
            const double* __restrict__ DAE, const double* __restrict__ DBE,
            const double* __restrict__ DP, const double* __restrict__ g2,
            double* __restrict__ fae_part, double* __restrict__ vrow) {
  extern __shared__ double sm[];
  const int n2 = ne * ne;
  double* sDAE = sm;
  double* sFAE = sm + n2;
  double* swarp = sFAE + n2;   // [8 warps][kOmgRows]
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    sDAE[k] = DAE[k];
    sFAE[k] = 0.0;
  }
  __syncthreads();
  const long long r0 = (long long)blockIdx.x * rows_per_cta;
  const long long r1 = min(nrows, r0 + rows_per_cta);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (long long rb = r0; rb < r1; rb += kOmgRows) {
    double dot[kOmgRows], u[kOmgRows];
#pragma unroll
    for (int k = 0; k < kOmgRows; k++) {
      dot[k] = 0.0;
      long long rr = rb + k;
      int j1 = (int)(rr % ne); rr /= ne;
      int i1 = (int)(rr % ne); rr /= ne;
      int jp = (int)(rr % np);
      int ip = (int)((rr / np) % np);
      u[k] = DP[ip + np * jp] * DBE[i1 + ne * j1];
    }
    for (int c = threadIdx.x; c < n2; c += blockDim.x) {
      double fa = 0.0;
      const double dae = sDAE[c];
#pragma unroll
      for (int k = 0; k < kOmgRows; k++) {
        long long r = rb + k;
        if (r < r1) {
          double m = __ldg(g2 + r * n2 + c);
          fa = fma(u[k], m, fa);
          dot[k] = fma(dae, m, dot[k]);
        }
      }
      sFAE[c] += fa;   // column c is owned by exactly one thread
    }
#pragma unroll
    for (int k = 0; k < kOmgRows; k++) {
      double v = dot[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) swarp[warp * kOmgRows + k] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < kOmgRows && rb + threadIdx.x < r1) {
      double v = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++)
        v += swarp[w * kOmgRows + threadIdx.x];
      vrow[rb + threadIdx.x] = v;
    }
    __syncthreads();
  }
  for (int c = threadIdx.x; c < n2; c += blockDim.x)
    fae_part[(size_t)blockIdx.x * n2 + c] = sFAE[c];
}

__global__ void omg2_reduce(int ne, int np, int nparts,
                            const double* __restrict__ fae_part,
                            const double* __restrict__ vrow,
                            const double* __restrict__ DBE,
                            const double* __restrict__ DP, double* FAE,
                            double* FP, double* FBE, double* fp_tmp) {
  const int n2 = ne * ne, p2 = np * np;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n2) {                       // FAE column c = i2*ne + j2
    double s = 0.0;
    for (int k = 0; k < nparts; k++) s += fae_part[(size_t)k * n2 + t];
    int i2 = t / ne, j2 = t % ne;
    if (FAE) FAE[i2 + ne * j2] += s;
  } else if (t < 2 * n2) {            // FBE(i1,j1)
    int c = t - n2, i1 = c / ne, j1 = c % ne;
    double s = 0.0;
    for (int ipjp = 0; ipjp < p2; ipjp++) {
      int ip = ipjp / np, jp = ipjp % np;
      s = fma(DP[ip + np * jp], vrow[(size_t)ipjp * n2 + i1 * ne + j1], s);
    }
    if (FBE) FBE[i1 + ne * j1] += s;
  } else if (t < 2 * n2 + p2) {       // FP(ip,jp)
    int ipjp = t - 2 * n2, ip = ipjp / np, jp = ipjp % np;
    double s = 0.0;
    for (int i1 = 0; i1 < ne; i1++)
      for (int j1 = 0; j1 < ne; j1++)
        s = fma(DBE[i1 + ne * j1], vrow[(size_t)ipjp * n2 + i1 * ne + j1], s);
    if (FP) FP[ip + np * jp] += s;
    fp_tmp[ipjp] = DP[ip + np * jp] * s;
  }
}

int omg2_parts(long long nrows) {
  // a few waves over 152 SMs; each CTA streams a contiguous row range
  long long want = 152LL * 8;
  long long per = (nrows + want - 1) / want;
  per = ((per + kOmgRows - 1) / kOmgRows) * kOmgRows;
  if (per < kOmgRows) per = kOmgRows;
  return (int)((nrows + per - 1) / per);
}

__global__ void xcfock_kernel(int ne, int np, double S_total, double H,
                              const double* se1, const double* sp1,
                              const double* se2, const double* sp2,
                              double* focke, double* fockp) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double one = 1.0, two = 2.0;
  if (t < ne * ne) {
    focke[t] = (one / S_total) * focke[t] - H * (se1[t] + two * se2[t]);
  } else if (t < ne * ne + np * np) {
    int k = t - ne * ne;
    fockp[k] = (one / S_total) * fockp[k] - H * (sp1[k] + sp2[k]);
  }
}

// ---- index maps (pack_GAM.f) on the device ------------------------------
// kind 0: pack_4D(ne,ne,ne) over (i4,i3,i2,i1) loop order  [GAM_ee]
// kind 2: index_GAM_2PK, 3: index_GAM_3PK, 4: index_GAM_4PK2, each over the
// reference's loop order (ip,jp,ie1,je1,... with the last ket fastest).
__global__ void index_fill_kernel(int kind, int ne, int np, long long count,
                                  long long* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       t < count; t += (long long)gridDim.x * blockDim.x) {
    long long r = t;
    int nidx = kind == 0 ? 4 : 2 + 2 * kind;
    int idx[10];
    for (int k = nidx - 1; k >= 0; k--) {
      int dim = (kind != 0 && k < 2) ? np : ne;
      idx[k] = (int)(r % dim) + 1;
      r /= dim;
    }
    long long ia;
    if (kind == 0) {
      // loop (ie1, je1, ie2, je2) -> pack_4D(je2, ie2, je1, ie1)
      ia = 1 + (idx[3] - 1) + (long long)ne * ((idx[2] - 1) + (long long)ne *
           ((idx[1] - 1) + (long long)ne * (idx[0] - 1)));
    } else {
      // innermost ket first: je_k, ie_k, ..., je1, ie1, jp, ip
      long long acc = idx[0] - 1;                 // ip
      acc = (idx[1] - 1) + (long long)np * acc;   // jp
      for (int k = 2; k < nidx; k++) acc = (idx[k] - 1) + (long long)ne * acc;
      ia = 1 + acc;
    }
    out[t] = ia;
  }
}

}  // namespace

size_t eg3_partial_doubles(int ne, int np) {
  return (size_t)np * np * ne * ne * ne * ne + (size_t)np * np;
}

cudaError_t launch_eg3_partials(int ne, int np, long long ipjp0,
                                long long nipjp, const double* DE,
                                const double* g3_slice, double* part,
                                cudaStream_t s) {
  if (ne < 1 || ne > 20 || np < 1) return cudaErrorInvalidValue;
  const int bs = ne * (256 / ne);
  const size_t smem = sizeof(double) * ((size_t)ne * ne * ne + ne * ne + bs);
  cudaError_t e = cudaFuncSetAttribute(eg3_kernel,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long grid = nipjp * ne * ne * ne;
  eg3_kernel<<<(unsigned)grid, bs, smem, s>>>(ne, np, DE, g3_slice, part, ipjp0);
  return cudaGetLastError();
}

cudaError_t launch_eg3ic1(int ne, int np, const double* DE, const double* DP,
                          const double* g3, double* scratch, double* focke,
                          double* fockp, double* E, cudaStream_t s) {
  cudaError_t e = launch_eg3_partials(ne, np, 0, (long long)np * np, DE, g3,
                                      scratch, s);
  if (e != cudaSuccess) return e;
  const long long grid = (long long)np * np * ne * ne * ne;
  double* fp_tmp = scratch + (size_t)grid * ne;
  return launch_fock_reduce(ne, np, ne * ne, scratch, DE, DP, 3.0, 1, focke,
                            fockp, fp_tmp, E, s);
}

size_t eg2_partial_doubles(int ne, int np) {
  return 2 * (size_t)np * np * ne * ne * ne + 2 * (size_t)np * np;
}

cudaError_t launch_eg2ic1(int ne, int np, const double* DE, const double* DP,
                          const double* g2, const double* g2s,
                          double* scratch, double* FE, double* SE, double* FP,
                          double* SP, double* E, double* S, cudaStream_t s) {
  if (ne < 1 || np < 1) return cudaErrorInvalidValue;
  const size_t npart = (size_t)np * np * ne * ne * ne;
  double* pv = scratch;
  double* ps = scratch + npart;
  double* ftmp = scratch + 2 * npart;
  eg2_kernel<<<(unsigned)(np * np * ne * ne), 32, 0, s>>>(ne, np, DE, g2, g2s,
                                                          pv, ps, 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // FE, FP accumulate (add2fock); SE, SP are overwritten (:379-381)
  e = launch_fock_reduce(ne, np, ne, pv, DE, DP, 2.0, 1, FE, FP, ftmp, E, s);
  if (e != cudaSuccess) return e;
  return launch_fock_reduce(ne, np, ne, ps, DE, DP, 1.0, 0, SE, SP,
                            ftmp + np * np, S, s);
}

cudaError_t launch_eg2_partials(int ne, int np, long long ipjp0,
                                long long nipjp, const double* DE,
                                const double* g2_slice,
                                const double* g2s_slice, double* pv,
                                double* ps, cudaStream_t s) {
  if (ne < 1 || np < 1 || nipjp < 1) return cudaErrorInvalidValue;
  eg2_kernel<<<(unsigned)(nipjp * ne * ne), 32, 0, s>>>(
      ne, np, DE, g2_slice, g2s_slice, pv, ps, ipjp0);
  return cudaGetLastError();
}

size_t omg2_partial_doubles(int ne, int np) {
  long long nrows = (long long)np * np * ne * ne;
  return (size_t)omg2_parts(nrows) * ne * ne + (size_t)nrows + np * np;
}

cudaError_t launch_rxchfne_omg2(int ne, int np, const double* DAE,
                                const double* DBE, const double* DP,
                                const double* g2, double* scratch, double* FAE,
                                double* FP, double* FBE, double* E,
                                cudaStream_t s) {
  if (ne < 1 || np < 1 || ne * ne > 16384) return cudaErrorInvalidValue;
  const long long nrows = (long long)np * np * ne * ne;
  const int nparts = omg2_parts(nrows);
  const int per = (int)((nrows + nparts - 1) / nparts);
  const int rows_per_cta = ((per + kOmgRows - 1) / kOmgRows) * kOmgRows;
  const int grid = (int)((nrows + rows_per_cta - 1) / rows_per_cta);
  double* fae_part = scratch;
  double* vrow = scratch + (size_t)nparts * ne * ne;
  double* fp_tmp = vrow + nrows;
  const size_t smem = sizeof(double) * (2 * (size_t)ne * ne + 8 * kOmgRows);
  cudaError_t e = cudaFuncSetAttribute(omg2_kernel,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  omg2_kernel<<<grid, 256, smem, s>>>(ne, np, nrows, rows_per_cta, DAE, DBE,
                                      DP, g2, fae_part, vrow);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int nout = 2 * ne * ne + np * np;
  omg2_reduce<<<(nout + 127) / 128, 128, 0, s>>>(ne, np, grid, fae_part, vrow,
                                                 DBE, DP, FAE, FP, FBE, fp_tmp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_vec_kernel<<<1, 256, 0, s>>>(np * np, fp_tmp, E);
  return cudaGetLastError();
}

cudaError_t launch_xcfock_correction(int ne, int np, double S_total,
                                     double H_expect, const double* se1,
                                     const double* sp1, const double* se2,
                                     const double* sp2, double* focke,
                                     double* fockp, cudaStream_t s) {
  int n = ne * ne + np * np;
  xcfock_kernel<<<(n + 127) / 128, 128, 0, s>>>(ne, np, S_total, H_expect,
                                                se1, sp1, se2, sp2, focke,
                                                fockp);
  return cudaGetLastError();
}

cudaError_t launch_index_fill(int kind, int ne, int np, int64_t count,
                              int64_t* out, cudaStream_t s) {
  if (!(kind == 0 || (kind >= 2 && kind <= 4))) return cudaErrorInvalidValue;
  long long blocks = (count + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  index_fill_kernel<<<(unsigned)blocks, 256, 0, s>>>(
      kind, ne, np, count, reinterpret_cast<long long*>(out));
  return cudaGetLastError();
}

}  // namespace neoxc
