// k_rxscf.cu -- the one-special-electron RXCHF SCF pieces that are not
// contractions: the regular electrons' one-body and Coulomb/exchange terms,
// the RXCHFne_Fock_correction1/2 assembly with the energy components, the
// density-change checks, and the orthogonality-constrained special-electron
// step (RXCHF_OCBSE2).
//
//   rxchfne/rxchfne_fock.f:2-250    RXCHFne_FOCK, RXCHFne_Fock_correction1/2
//   rxchfne/rxchfne_hfterms.f:2-50  RXCHFne_FAE_GAMee (closed shell)
//   xcuhf/xcuhf_hfterms.f:2-43,219-290  FAE_ecore, FAE_GAMee (open shell)
//   rxchfne/rxcuhfne_fock.f          RXCUHFne_FOCK
//   rxchf/rxchf_scf.f:1124-1330      RXCHF_OCBSE2 / RXCHF_OCBSE_driver2
//
// Matrices are column-major n x n (F(i,j) at i + n*j); GAM_ee is C-order
// [ie1][je1][ie2][je2] (pack_4D(je2,ie2,je1,ie1)), the core Hamiltonian
// C-order [i][j] (pack_2D).  Every kernel here is small (n <= 64): one CTA,
// or one thread per matrix element.
#include <cuda_runtime.h>

#include "neoxc_internal.h"

namespace neoxc {
namespace {

__device__ double cta_sum(double v, double* sw) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sw[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r += sw[k];
  __syncthreads();
  return r;
}

__device__ double cta_max(double v, double* sw) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x / 32, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sw[w] = v;
  __syncthreads();
  double r = 0.0;
  for (int k = 0; k < (int)(blockDim.x + 31) / 32; k++) r = fmax(r, sw[k]);
  __syncthreads();
  return r;
}

// Regular-electron terms of RXCHFne_IC_construct_FAE (closed shell) or
// RXCUHFne_IC_construct_FE (open shell), one thread per (i, j):
//   closed: FA1 = ecore + [with_ee] sum_kl DA(k,l) ((ij|kl) - 1/2 (il|kj))
//   open:   F1_s = ecore + [with_ee] sum_kl DAtot(k,l) (ij|kl) - D_s(k,l) (il|kj)
// part[t] = E_ecore share, part[n2 + t] = E_ee share (1/2 D x per spin);
// the open case also writes DAtot = DA + DB.
__global__ void rx_fock1_kernel(int ne, int open, int with_ee,
                                const double* __restrict__ Hce,
                                const double* __restrict__ Gee,
                                const double* __restrict__ DA,
                                const double* __restrict__ DB,
                                double* __restrict__ FA1, double* __restrict__ FB1,
                                double* __restrict__ DT, double* __restrict__ part) {
  const int n2 = ne * ne;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n2) return;
  const int i = t / ne, j = t - i * ne;
  const double fc = Hce[i * ne + j];
  const int o = i + ne * j;
  if (!open) {
    double x = 0.0;
    if (with_ee)
      for (int k = 0; k < ne; k++)
        for (int l = 0; l < ne; l++) {
          const double v1 = Gee[(((long long)i * ne + j) * ne + k) * ne + l];
          const double v2 = Gee[(((long long)i * ne + l) * ne + k) * ne + j];
          x = x + DA[k + ne * l] * (v1 - 0.5 * v2);
        }
    FA1[o] = fc + x;
    part[t] = DA[o] * fc;
    part[n2 + t] = 0.5 * DA[o] * x;
    return;
  }
  double xa = 0.0, xb = 0.0;
  if (with_ee)
    for (int k = 0; k < ne; k++)
      for (int l = 0; l < ne; l++) {
        const double v1 = Gee[(((long long)i * ne + j) * ne + k) * ne + l];
        const double v2 = Gee[(((long long)i * ne + l) * ne + k) * ne + j];
        const double da = DA[k + ne * l], db = DB[k + ne * l], dt = da + db;
        xa = xa + (dt * v1 - da * v2);
        xb = xb + (dt * v1 - db * v2);
      }
  FA1[o] = fc + xa;
  FB1[o] = fc + xb;
  DT[o] = DA[o] + DB[o];
  part[t] = DA[o] * fc + DB[o] * fc;
  part[n2 + t] = 0.5 * (DA[o] * xa) + 0.5 * (DB[o] * xb);
}

// en[2] = E_ecore, en[3] = E_ee from the per-element shares.
__global__ void rx_fock1_energy_kernel(int n2, const double* __restrict__ part,
                                       double* __restrict__ en) {
  __shared__ double sw[32];
  for (int c = 0; c < 2; c++) {
    double v = 0.0;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) v += part[(long long)c * n2 + t];
    const double s = cta_sum(v, sw);
    if (threadIdx.x == 0) en[2 + c] = s;
  }
}

// RXCHFne_FOCK's energy assembly and Fock corrections (rxchfne_fock.f:187-
// 250): S_total = S_P_OMG1, E_OMGk = E_P_OMGk / S_total, E_total =
// E_ecore + E_ee + E_OMG1 + E_OMG2 (+ E_nuc, added by the SCF driver);
// FA = XF1 + XF2 / S, FP = XFP / S - (E_P1 + E_P2) / S^2 XSP, FBE alike.
// The beta pair (XFB1, XFB2 -> FB) is assembled when XFB1 is non-null.
__global__ void rx_assemble_kernel(int ne, int np, double* __restrict__ en,
                                   const double* __restrict__ XFA1,
                                   const double* __restrict__ XFA2,
                                   const double* __restrict__ XFB1,
                                   const double* __restrict__ XFB2,
                                   const double* __restrict__ XFP,
                                   const double* __restrict__ XSP,
                                   const double* __restrict__ XFBE,
                                   const double* __restrict__ XSBE,
                                   double* __restrict__ FA, double* __restrict__ FB,
                                   double* __restrict__ FP, double* __restrict__ FBE) {
  __shared__ double sS, sPsi;
  if (threadIdx.x == 0) {
    const double S = en[9];
    const double psi = en[7] + en[8];
    en[6] = S;
    en[4] = en[7] / S;
    en[5] = en[8] / S;
    en[0] = en[2] + en[3] + en[4] + en[5] + en[1];
    sS = S;
    sPsi = psi;
  }
  __syncthreads();
  const double one = 1.0, S = sS;
  const double c1 = one / S, c2 = sPsi / (S * S);
  const int n2 = ne * ne, p2 = np * np;
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    FA[k] = XFA1[k] + c1 * XFA2[k];
    if (XFB1) FB[k] = XFB1[k] + c1 * XFB2[k];
    FBE[k] = c1 * XFBE[k] - c2 * XSBE[k];
  }
  for (int k = threadIdx.x; k < p2; k += blockDim.x) FP[k] = c1 * XFP[k] - c2 * XSP[k];
}

// DENDIF + COPYDEN for one density: out = max |D0 - D|, D0 = D.
__global__ void rx_dendif_kernel(int n2, const double* __restrict__ D,
                                 double* __restrict__ D0, double* __restrict__ out) {
  __shared__ double sw[32];
  double m = 0.0;
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    m = fmax(m, fabs(D0[k] - D[k]));
  }
  const double r = cta_max(m, sw);
  for (int k = threadIdx.x; k < n2; k += blockDim.x) D0[k] = D[k];
  if (threadIdx.x == 0) *out = r;
}

// RXCHF_OCBSE_driver2, first half: overlaps <CA_k | S | cb0> of every
// regular orbital with the previous special orbital, the orbital of largest
// |overlap| among k >= 1 (0-based) is discarded; W = [CA(:, nocca..ne-2)
// with the discarded column replaced by CA(:, ne-1), projected and
// normalised cb0], m = ne - nocca columns; then AUX = F W, S W and the
// projected matrices wF = W^T F W, wS = W^T S W (m x m, column-major).
// scr: n*m (AUX).  info[0] = discarded orbital (0-based), info[1] = the
// projected norm (<= 0 means the projection vanished).
__global__ void ocbse_prep_kernel(int n, int nocca, const double* __restrict__ CA,
                                  const double* __restrict__ cb0,
                                  const double* __restrict__ F,
                                  const double* __restrict__ S,
                                  double* __restrict__ W, double* __restrict__ aux,
                                  double* __restrict__ wF, double* __restrict__ wS,
                                  double* __restrict__ info) {
  __shared__ double ov[kScfMaxN], proj[kScfMaxN], sb[kScfMaxN], sw[32];
  __shared__ int discard;
  __shared__ double snorm;
  const int m = n - nocca, nvirt = m - 1;
  // S cb0
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += S[i + n * j] * cb0[j];
    sb[i] = acc;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc += CA[i + n * k] * sb[i];
    ov[k] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double best = 0.0;
    int d = 0;
    for (int k = 1; k < n; k++)
      if (fabs(ov[k]) > best) {
        best = fabs(ov[k]);
        d = k;
      }
    discard = d;
  }
  __syncthreads();
  // projected special orbital: cb0 - sum_{k != discard} ov_k CA_k
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double p = cb0[i];
    for (int k = 0; k < n; k++)
      if (k != discard) p = p - ov[k] * CA[i + n * k];
    proj[i] = p;
  }
  __syncthreads();
  double part = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += S[i + n * j] * proj[j];
    part += proj[i] * acc;
  }
  const double nrm = cta_sum(part, sw);
  if (threadIdx.x == 0) snorm = nrm;
  __syncthreads();
  const double inv = snorm > 0.0 ? 1.0 / sqrt(snorm) : 0.0;
  for (int e = threadIdx.x; e < n * m; e += blockDim.x) {
    const int i = e % n, c = e / n;
    double v;
    if (c < nvirt) {
      const int col = nocca + c;
      v = col != discard ? CA[i + n * col] : CA[i + n * (n - 1)];
    } else {
      v = proj[i] * inv;
    }
    W[i + n * c] = v;
  }
  __syncthreads();
  // wF = W^T (F W), then wS = W^T (S W), with aux = F W / S W (n x m)
  for (int pass = 0; pass < 2; pass++) {
    const double* M = pass == 0 ? F : S;
    double* out = pass == 0 ? wF : wS;
    for (int e = threadIdx.x; e < n * m; e += blockDim.x) {
      const int i = e % n, c = e / n;
      double acc = 0.0;
      for (int l = 0; l < n; l++) acc += M[i + n * l] * W[l + n * c];
      aux[i + n * c] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int r = e % m, c = e / m;
      double acc = 0.0;
      for (int l = 0; l < n; l++) acc += W[l + n * r] * aux[l + n * c];
      out[r + m * c] = acc;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    info[0] = (double)discard;
    info[1] = snorm;
  }
}

// Second half: CB(:, c) = W Cx(:, c) for the m subspace orbitals (the rest
// of CB zero), DB = CB(:,0) CB(:,0)^T (RXCHF_construct_DBE, NBE = 1).
__global__ void ocbse_finish_kernel(int n, int m, const double* __restrict__ W,
                                    const double* __restrict__ Cx,
                                    double* __restrict__ CB, double* __restrict__ DB) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, c = e / n;
    double acc = 0.0;
    if (c < m)
      for (int l = 0; l < m; l++) acc += W[i + n * l] * Cx[l + m * c];
    CB[i + n * c] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    DB[i + n * j] = CB[i] * CB[j];
  }
}

}  // namespace

size_t rx_fock1_part_doubles(int ne) { return 2 * (size_t)ne * ne; }

cudaError_t launch_rx_fock1(int ne, int open, int with_ee, const double* Hce,
                            const double* Gee, const double* DA, const double* DB,
                            double* FA1, double* FB1, double* DT, double* part,
                            double* en, cudaStream_t s) {
  if (ne < 1 || ne > kScfMaxN) return cudaErrorInvalidValue;
  const int n2 = ne * ne;
  rx_fock1_kernel<<<(n2 + 127) / 128, 128, 0, s>>>(ne, open, with_ee, Hce, Gee, DA, DB,
                                                   FA1, FB1, DT, part);
  rx_fock1_energy_kernel<<<1, 256, 0, s>>>(n2, part, en);
  return cudaGetLastError();
}

cudaError_t launch_rx_assemble(int ne, int np, double* en, const double* XFA1,
                               const double* XFA2, const double* XFB1,
                               const double* XFB2, const double* XFP,
                               const double* XSP, const double* XFBE,
                               const double* XSBE, double* FA, double* FB, double* FP,
                               double* FBE, cudaStream_t s) {
  rx_assemble_kernel<<<1, 256, 0, s>>>(ne, np, en, XFA1, XFA2, XFB1, XFB2, XFP, XSP, XFBE,
                                       XSBE, FA, FB, FP, FBE);
  return cudaGetLastError();
}

cudaError_t launch_rx_dendif(int n, const double* D, double* D0, double* out,
                             cudaStream_t s) {
  rx_dendif_kernel<<<1, 256, 0, s>>>(n * n, D, D0, out);
  return cudaGetLastError();
}

size_t ocbse_scratch_doubles(int n) { return 6 * (size_t)n * n + 2 * (size_t)n + 8; }

cudaError_t launch_ocbse2(int n, int nocca, const double* CA, const double* cb0,
                          const double* F, const double* S, double* scratch,
                          double* CB, double* DB, double* info, int* status,
                          cudaStream_t s) {
  if (n < 2 || n > kScfMaxN || nocca < 1 || nocca >= n) return cudaErrorInvalidValue;
  const int m = n - nocca;
  double* W = scratch;                       // n*m
  double* aux = W + (size_t)n * n;           // n*m
  double* wF = aux + (size_t)n * n;          // m*m
  double* wS = wF + (size_t)n * n;           // m*m
  double* Xm = wS + (size_t)n * n;           // m*m
  double* Cx = Xm + (size_t)n * n;           // m*m (D of the subspace solve reuses CB)
  ocbse_prep_kernel<<<1, 256, 0, s>>>(n, nocca, CA, cb0, F, S, W, aux, wF, wS, info);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_inv_sqrt(m, wS, Xm, status, s);
  if (e != cudaSuccess) return e;
  // the subspace density is not used; CB (n*n >= m*m) holds it until the
  // finish kernel overwrites CB with the expanded orbitals
  e = launch_roothan(m, wF, Xm, 0, 1, 1.0, CB, nullptr, Cx, status + 1, s);
  if (e != cudaSuccess) return e;
  ocbse_finish_kernel<<<1, 256, 0, s>>>(n, m, W, Cx, CB, DB);
  return cudaGetLastError();
}

}  // namespace neoxc
