// abi.cu -- host side of the C-ABI declared in include/neoxc.h.
//
// Each neoxc_* entry point validates the reference's size arguments,
// stages host arrays into device memory on the library stream, runs the
// sm_103a kernels and copies results back (accumulating into the caller's
// Fock matrices where the reference does add2fock).  There is no CPU
// compute path: if CUDA is unusable the call returns NEOXC_ERR_CUDA.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/neoxc.h"
#include "neoxc_internal.h"

using namespace neoxc;

namespace {

thread_local std::string g_err;

int set_err(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CU(call)                                                           \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess)                                                 \
      return set_err(e_ == cudaErrorMemoryAllocation ? NEOXC_ERR_NOMEM     \
                                                     : NEOXC_ERR_CUDA,     \
                     "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                     __FILE__, __LINE__);                                  \
  } while (0)

struct Ctx {
  cudaStream_t stream = nullptr;
  int device = -1;
};

std::mutex g_mu;
Ctx g_ctx[64];

// library stream of the current device (created on first use)
int get_stream(cudaStream_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_err(NEOXC_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return set_err(NEOXC_ERR_CUDA, "device id %d", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  Ctx& c = g_ctx[dev];
  if (!c.stream) {
    cudaDeviceProp p;
    e = cudaGetDeviceProperties(&p, dev);
    if (e != cudaSuccess)
      return set_err(NEOXC_ERR_CUDA, "cudaGetDeviceProperties: %s",
                     cudaGetErrorString(e));
    if (!(p.major == 10 && p.minor == 3))
      return set_err(NEOXC_ERR_CUDA,
                     "device %d is sm_%d%d; this library is built for sm_103a",
                     dev, p.major, p.minor);
    e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
      return set_err(NEOXC_ERR_CUDA, "cudaStreamCreate: %s",
                     cudaGetErrorString(e));
    c.device = dev;
  }
  *out = c.stream;
  return NEOXC_OK;
}

// Device buffer released on the stream it was allocated on.
struct DBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

int dalloc(DBuf& b, size_t bytes, cudaStream_t s) {
  b.s = s;
  if (bytes == 0) bytes = 8;
  cudaError_t e = cudaMallocAsync(&b.p, bytes, s);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return set_err(NEOXC_ERR_NOMEM, "device allocation of %zu bytes: %s",
                   bytes, cudaGetErrorString(e));
  }
  return NEOXC_OK;
}

int upload(DBuf& b, const void* h, size_t bytes, cudaStream_t s) {
  int rc = dalloc(b, bytes, s);
  if (rc) return rc;
  if (bytes) CU(cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, s));
  return NEOXC_OK;
}

int finish(cudaStream_t s) {
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(s));
  return NEOXC_OK;
}

#define RC(x)               \
  do {                      \
    int rc_ = (x);          \
    if (rc_) return rc_;    \
  } while (0)

int need(bool ok, const char* what) {
  return ok ? NEOXC_OK : set_err(NEOXC_ERR_ARG, "argument check failed: %s", what);
}

// ---- basis staging for the MD builders ------------------------------------
struct SysUpload {
  DevSystem d{};
  DBuf eprim, pprim, kps, kpe, zan, cat, bgem, ggem, g3i, g3rec;
};

int stage_system(SysUpload& u, cudaStream_t s, int64_t nebf, int64_t npebf,
                 int64_t npbf, int64_t nat, int64_t ngtg, double pmass,
                 const double* cat, const double* zan, const double* bcoef1,
                 const double* gamma1, const int64_t* KPESTR,
                 const int64_t* KPEEND, const double* AGEBFCC,
                 const double* AGNBFCC, const double* ELCEX,
                 const double* NUCEX, const int64_t* ELCAM,
                 const int64_t* NUCAM, const double* ELCBFC,
                 const double* NUCBFC) {
  RC(need(nebf >= 1 && npebf >= nebf && npbf >= 1, "basis sizes"));
  RC(need(nat >= 0 && nat <= kMaxNat, "nat within the supported range"));
  RC(need(ngtg >= 1 && ngtg <= kMaxNG, "ngtg within the supported range"));
  std::vector<DevPrim> ep(npebf), pp(npbf);
  for (int64_t i = 0; i < npebf; i++) {
    DevPrim& q = ep[i];
    q.a = ELCEX[i];
    q.coef = AGEBFCC[i];
    for (int d = 0; d < 3; d++) {
      q.c[d] = ELCBFC[i + npebf * d];
      q.l[d] = (int)ELCAM[i + npebf * d];
      if (q.l[d] < 0 || q.l[d] > kMaxL)
        return set_err(NEOXC_ERR_UNSUPPORTED,
                       "electronic primitive %lld has l=%d in one Cartesian "
                       "direction (supported: 0..%d)",
                       (long long)i + 1, q.l[d], kMaxL);
    }
    if (q.l[0] + q.l[1] + q.l[2] > 2)
      return set_err(NEOXC_ERR_UNSUPPORTED,
                     "electronic primitive %lld has total l > 2 (the MD "
                     "kernels support Cartesian s, p, d)", (long long)i + 1);
    q.pad = 0;
  }
  for (int64_t i = 0; i < npbf; i++) {
    DevPrim& q = pp[i];
    q.a = NUCEX[i];
    q.coef = AGNBFCC[i];
    for (int d = 0; d < 3; d++) {
      q.c[d] = NUCBFC[i + npbf * d];
      q.l[d] = (int)NUCAM[i + npbf * d];
      if (q.l[d] < 0 || q.l[d] > kMaxL)
        return set_err(NEOXC_ERR_UNSUPPORTED,
                       "nuclear primitive %lld has l=%d in one Cartesian "
                       "direction (supported: 0..%d)",
                       (long long)i + 1, q.l[d], kMaxL);
    }
    if (q.l[0] + q.l[1] + q.l[2] > 2)
      return set_err(NEOXC_ERR_UNSUPPORTED,
                     "nuclear primitive %lld has total l > 2 (the MD kernels "
                     "support Cartesian s, p, d)", (long long)i + 1);
    q.pad = 0;
  }
  std::vector<int> ks(nebf), ke(nebf);
  for (int64_t i = 0; i < nebf; i++) {
    ks[i] = (int)KPESTR[i] - 1;
    ke[i] = (int)KPEEND[i] - 1;
    if (ks[i] < 0 || ke[i] < ks[i] || ke[i] >= npebf)
      return set_err(NEOXC_ERR_ARG, "KPESTR/KPEEND(%lld) out of range",
                     (long long)i + 1);
  }
  RC(upload(u.eprim, ep.data(), sizeof(DevPrim) * npebf, s));
  RC(upload(u.pprim, pp.data(), sizeof(DevPrim) * npbf, s));
  RC(upload(u.kps, ks.data(), sizeof(int) * nebf, s));
  RC(upload(u.kpe, ke.data(), sizeof(int) * nebf, s));
  RC(upload(u.zan, zan, sizeof(double) * (nat ? nat : 1) * (nat ? 1 : 0), s));
  RC(upload(u.cat, cat, sizeof(double) * 3 * nat, s));
  RC(upload(u.bgem, bcoef1, sizeof(double) * ngtg, s));
  RC(upload(u.ggem, gamma1, sizeof(double) * ngtg, s));
  u.d.nebf = (int)nebf;
  u.d.npebf = (int)npebf;
  u.d.npbf = (int)npbf;
  u.d.nat = (int)nat;
  u.d.ngtg = (int)ngtg;
  u.d.pmass = pmass;
  u.d.eprim = u.eprim.as<DevPrim>();
  u.d.pprim = u.pprim.as<DevPrim>();
  u.d.kpestr = u.kps.as<int>();
  u.d.kpeend = u.kpe.as<int>();
  u.d.zan = u.zan.as<double>();
  u.d.cat = u.cat.as<double>();
  u.d.bgem = u.bgem.as<double>();
  u.d.ggem = u.ggem.as<double>();
  int le = 0, lp = 0;
  for (const DevPrim& q : ep) le = std::max(le, q.l[0] + q.l[1] + q.l[2]);
  for (const DevPrim& q : pp) lp = std::max(lp, q.l[0] + q.l[1] + q.l[2]);
  u.d.lmax_e = le;
  u.d.lmax_p = lp;
  // gam_3 pair tables (k_gam3.cu): the primitive pairs of every canonical
  // contracted pair (i >= j, P = i(i+1)/2 + j) in P order, tiles of whole
  // pairs with at most kG3MaxTileKets kets, and within a tile the kets
  // ordered by angular class (so the lanes of a warp take alike kets)
  {
    const int ne = (int)nebf;
    const int nPe = ne * (ne + 1) / 2;
    std::vector<int> ab, kofs(nPe + 1, 0), tk, tp, perm, cls;
    for (int i = 0; i < ne; i++)
      for (int j = 0; j <= i; j++) {
        const int P = i * (i + 1) / 2 + j;
        kofs[P] = (int)ab.size() / 2;
        for (int a = ks[i]; a <= ke[i]; a++)
          for (int b = ks[j]; b <= ke[j]; b++) {
            ab.push_back(a);
            ab.push_back(b);
            int key = 0;
            for (int d = 0; d < 3; d++) key = key * 8 + ep[a].l[d] + ep[b].l[d];
            cls.push_back(key);
          }
      }
    const int nket = (int)ab.size() / 2;
    kofs[nPe] = nket;
    bool ok = true;
    tk.push_back(0);
    tp.push_back(0);
    for (int P = 0; P < nPe; P++) {
      if (kofs[P + 1] - kofs[P] > kG3MaxTileKets) ok = false;
      if (kofs[P + 1] - tk.back() > kG3MaxTileKets) {
        tk.push_back(kofs[P]);
        tp.push_back(P);
      }
    }
    tk.push_back(nket);
    tp.push_back(nPe);
    const int ntile = (int)tk.size() - 1;
    perm.resize(nket);
    for (int t = 0; t < ntile; t++) {
      std::vector<int> idx;
      for (int k = tk[t]; k < tk[t + 1]; k++) idx.push_back(k);
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int x, int y) { return cls[x] < cls[y]; });
      for (size_t q = 0; q < idx.size(); q++) perm[tk[t] + q] = idx[q];
    }
    std::vector<int> g3i;
    g3i.insert(g3i.end(), ab.begin(), ab.end());
    g3i.insert(g3i.end(), kofs.begin(), kofs.end());
    g3i.insert(g3i.end(), tk.begin(), tk.end());
    g3i.insert(g3i.end(), tp.begin(), tp.end());
    g3i.insert(g3i.end(), perm.begin(), perm.end());
    RC(upload(u.g3i, g3i.data(), sizeof(int) * g3i.size(), s));
    u.d.g3_nket = nket;
    u.d.g3_ntile = ok ? ntile : 0;
    u.d.g3i = u.g3i.as<int>();
    RC(dalloc(u.g3rec, sizeof(double) * g3_record_doubles(nket, (int)npbf), s));
    u.d.g3rec = u.g3rec.as<double>();
    CU(launch_g3_records(u.d, const_cast<double*>(u.d.g3rec), s));
  }
  return NEOXC_OK;
}

// Fock accumulate: device result added to the caller's host matrix.
int accumulate_back(double* host, const double* dev, int64_t n,
                    cudaStream_t s) {
  std::vector<double> tmp(n);
  CU(cudaMemcpyAsync(tmp.data(), dev, sizeof(double) * n,
                     cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  for (int64_t k = 0; k < n; k++) host[k] += tmp[k];
  return NEOXC_OK;
}

}  // namespace

// Records an error for neoxc_last_error() from other translation units.
int neoxc::set_last_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

extern "C" {

const char* neoxc_last_error(void) { return g_err.c_str(); }
int neoxc_version(void) { return 100; }

int neoxc_device_ok(void) {
  cudaStream_t s;
  return get_stream(&s) == NEOXC_OK ? 1 : 0;
}

// ---- index maps --------------------------------------------------------------
int64_t neoxc_pack_4d(int64_t n1, int64_t n2, int64_t n3, int64_t i1,
                      int64_t i2, int64_t i3, int64_t i4) {
  return 1 + (i1 - 1) + n1 * ((i2 - 1) + n2 * ((i3 - 1) + n3 * (i4 - 1)));
}
int64_t neoxc_index_gam_2pk(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                            int64_t ie1, int64_t je1, int64_t ie2,
                            int64_t je2) {
  return 1 + (je2 - 1) +
         ne * ((ie2 - 1) +
               ne * ((je1 - 1) + ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))));
}
int64_t neoxc_index_gam_3pk(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                            int64_t ie1, int64_t je1, int64_t ie2,
                            int64_t je2, int64_t ie3, int64_t je3) {
  return 1 + (je3 - 1) +
         ne * ((ie3 - 1) + ne * ((je2 - 1) + ne * ((ie2 - 1) +
         ne * ((je1 - 1) + ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))))));
}
int64_t neoxc_index_gam_4pk2(int64_t ne, int64_t np, int64_t ip, int64_t jp,
                             int64_t ie1, int64_t je1, int64_t ie2,
                             int64_t je2, int64_t ie3, int64_t je3,
                             int64_t ie4, int64_t je4) {
  return 1 + (je4 - 1) +
         ne * ((ie4 - 1) + ne * ((je3 - 1) + ne * ((ie3 - 1) +
         ne * ((je2 - 1) + ne * ((ie2 - 1) + ne * ((je1 - 1) +
         ne * ((ie1 - 1) + ne * ((jp - 1) + np * (ip - 1)))))))));
}

int neoxc_index_map(int64_t kind, int64_t ne, int64_t np, int64_t count,
                    int64_t* out) {
  RC(need(out != nullptr && count >= 0, "output"));
  int64_t total = kind == 0 ? ne * ne * ne * ne
                : kind == 2 ? ne * ne * ne * ne * np * np
                : kind == 3 ? ne * ne * ne * ne * ne * ne * np * np
                : kind == 4 ? ne * ne * ne * ne * ne * ne * ne * ne * np * np
                            : -1;
  RC(need(total >= 0, "kind in {0,2,3,4}"));
  RC(need(count <= total, "count <= size of the map"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf d;
  RC(dalloc(d, sizeof(int64_t) * count, s));
  CU(launch_index_fill((int)kind, (int)ne, (int)np, count, d.as<int64_t>(), s));
  CU(cudaMemcpyAsync(out, d.p, sizeof(int64_t) * count, cudaMemcpyDeviceToHost,
                     s));
  return finish(s);
}

int neoxc_make_kpe(int64_t nebf, int64_t npebf, const int64_t* AMPEB2C,
                   int64_t* KPESTR, int64_t* KPEEND) {
  RC(need(nebf >= 1 && npebf >= nebf && AMPEB2C && KPESTR && KPEEND, "sizes"));
  int64_t ichk = 1, ist = 1;
  for (int64_t iep = 1; iep <= npebf; iep++) {
    int64_t iec = AMPEB2C[iep - 1];
    if (iec < 1 || iec > nebf)
      return set_err(NEOXC_ERR_ARG, "AMPEB2C(%lld)=%lld out of range",
                     (long long)iep, (long long)iec);
    if (iec != ichk) {
      ichk = ichk + 1;
      if (iec - 2 < 0) return set_err(NEOXC_ERR_ARG, "AMPEB2C not ordered");
      KPESTR[iec - 2] = ist;
      KPEEND[iec - 2] = iep - 1;
      ist = iep;
    }
    if (iep == npebf) {
      KPESTR[iec - 1] = ist;
      KPEEND[iec - 1] = iep;
    }
  }
  return NEOXC_OK;
}

// ---- builders -----------------------------------------------------------------
int neoxc_calc_gam_ee(int64_t nebf, int64_t npebf, int64_t ngee,
                      const int64_t* AMPEB2C, const double* AGEBFCC,
                      const double* ELCEX, const int64_t* ELCAM,
                      const double* ELCBFC, double* GAM_ee) {
  RC(need(ngee == nebf * nebf * nebf * nebf, "ngee == nebf**4"));
  RC(need(GAM_ee && AMPEB2C && AGEBFCC && ELCEX && ELCAM && ELCBFC, "pointers"));
  std::vector<int64_t> kps(nebf), kpe(nebf);
  RC(neoxc_make_kpe(nebf, npebf, AMPEB2C, kps.data(), kpe.data()));
  cudaStream_t s;
  RC(get_stream(&s));
  // GAM_ee needs no nuclear basis or geminal; stage a 1-function stub
  const double one = 1.0, zero3[3] = {0, 0, 0}, g1 = 1.0, b1 = 0.0;
  const int64_t l0[3] = {0, 0, 0};
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, 1, 0, 1, 1.0, zero3, &one, &b1, &g1,
                  kps.data(), kpe.data(), AGEBFCC, &one, ELCEX, &one, ELCAM,
                  l0, ELCBFC, zero3));
  DBuf d;
  RC(dalloc(d, sizeof(double) * ngee, s));
  CU(launch_gam_ee(u.d, d.as<double>(), s));
  CU(cudaMemcpyAsync(GAM_ee, d.p, sizeof(double) * ngee,
                     cudaMemcpyDeviceToHost, s));
  return finish(s);
}

static int gam2_common(int rx, int64_t nebf, int64_t npebf, int64_t npbf,
                       int64_t ng2, int64_t nat, int64_t ngtg1, double pmass,
                       const double* cat, const double* zan,
                       const double* bcoef1, const double* gamma1,
                       const int64_t* KPESTR, const int64_t* KPEEND,
                       const double* AGEBFCC, const double* AGNBFCC,
                       const double* ELCEX, const double* NUCEX,
                       const int64_t* ELCAM, const int64_t* NUCAM,
                       const double* ELCBFC, const double* NUCBFC,
                       double* out1, double* out2) {
  RC(need(ng2 == nebf * nebf * nebf * nebf * npbf * npbf,
          "ng2 == nebf**4 * npbf**2"));
  RC(need(out1 && out2, "output pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan,
                  bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX,
                  NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC));
  DBuf d1, d2;
  RC(dalloc(d1, sizeof(double) * ng2, s));
  RC(dalloc(d2, sizeof(double) * ng2, s));
  CU(launch_gam2_raw(u.d, rx, d1.as<double>(), d2.as<double>(), s));
  CU(launch_gam2_symmetrize((int)nebf, (int)npbf, rx, d1.as<double>(),
                            d2.as<double>(), s));
  CU(cudaMemcpyAsync(out1, d1.p, sizeof(double) * ng2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(out2, d2.p, sizeof(double) * ng2, cudaMemcpyDeviceToHost, s));
  return finish(s);
}

int neoxc_gam2_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                   int64_t ng2, int64_t ng2prm, int64_t nat, int64_t ngtg1,
                   double pmass, const double* cat, const double* zan,
                   const double* bcoef1, const double* gamma1,
                   const int64_t* KPESTR, const int64_t* KPEEND,
                   const int64_t* AMPEB2C, const double* AGEBFCC,
                   const double* AGNBFCC, const double* ELCEX,
                   const double* NUCEX, const int64_t* ELCAM,
                   const int64_t* NUCAM, const double* ELCBFC,
                   const double* NUCBFC, double* GM2ICR, double* GM2sICR) {
  (void)AMPEB2C;
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ng2prm == npebf * npebf * npebf * npebf * npbf * npbf, "ng2prm"));
  return gam2_common(0, nebf, npebf, npbf, ng2, nat, ngtg1, pmass, cat, zan,
                     bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX,
                     NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, GM2ICR, GM2sICR);
}

int neoxc_rxchfne_gam2_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf,
                           int64_t npbf, int64_t ng2, int64_t ng2prm,
                           int64_t nat, int64_t ngtg1, double pmass,
                           const double* cat, const double* zan,
                           const double* bcoef1, const double* gamma1,
                           const int64_t* KPESTR, const int64_t* KPEEND,
                           const int64_t* AMPEB2C, const double* AGEBFCC,
                           const double* AGNBFCC, const double* ELCEX,
                           const double* NUCEX, const int64_t* ELCAM,
                           const int64_t* NUCAM, const double* ELCBFC,
                           const double* NUCBFC, double* GM2ICR,
                           double* GM2exICR) {
  (void)AMPEB2C;
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ng2prm == npebf * npebf * npebf * npebf * npbf * npbf, "ng2prm"));
  return gam2_common(1, nebf, npebf, npbf, ng2, nat, ngtg1, pmass, cat, zan,
                     bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX,
                     NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, GM2ICR, GM2exICR);
}

int neoxc_gam3_ic1_opts(int64_t options, int64_t Nchunks, int64_t nebf, int64_t npebf,
                        int64_t npbf, int64_t ng3, int64_t ng3prm, int64_t nat,
                        int64_t ngtg1, double pmass, const double* cat, const double* zan,
                        const double* bcoef1, const double* gamma1,
                        const int64_t* KPESTR, const int64_t* KPEEND,
                        const int64_t* AMPEB2C, const double* AGEBFCC,
                        const double* AGNBFCC, const double* ELCEX,
                        const double* NUCEX, const int64_t* ELCAM,
                        const int64_t* NUCAM, const double* ELCBFC,
                        const double* NUCBFC, double* GM3ICR, double* seconds) {
  (void)AMPEB2C;
  RC(need((options & ~(int64_t)(NEOXC_SCF_MIXED | NEOXC_SCF_SCREEN)) == 0, "options"));
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  int64_t n6 = nebf * nebf * nebf * nebf * nebf * nebf;
  RC(need(ng3 == n6 * npbf * npbf, "ng3 == nebf**6 * npbf**2"));
  int64_t p6 = npebf * npebf * npebf * npebf * npebf * npebf;
  RC(need(ng3prm == p6 * npbf * npbf, "ng3prm"));
  RC(need(GM3ICR != nullptr, "output pointer"));
  cudaStream_t s;
  RC(get_stream(&s));
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan,
                  bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX,
                  NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC));
  DBuf d, aux;
  RC(dalloc(d, sizeof(double) * ng3, s));
  RC(dalloc(aux, sizeof(double) * gam3_aux_doubles((int)nebf, (int)npbf), s));
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (seconds) {
    CU(cudaEventCreate(&ev[0]));
    CU(cudaEventCreate(&ev[1]));
    CU(cudaEventRecord(ev[0], s));
  }
  CU(launch_gam3_aux(u.d, aux.as<double>(), s));
  CU(launch_gam3_raw(u.d, aux.as<double>(), d.as<double>(), s,
                     (options & NEOXC_SCF_MIXED) ? 1 : 0,
                     (options & NEOXC_SCF_SCREEN) ? kScreenThreshold : 0.0));
  CU(launch_gam3_symmetrize((int)nebf, (int)npbf, d.as<double>(), s));
  if (seconds) CU(cudaEventRecord(ev[1], s));
  CU(cudaMemcpyAsync(GM3ICR, d.p, sizeof(double) * ng3, cudaMemcpyDeviceToHost,
                     s));
  const int rc = finish(s);
  if (seconds) {
    float ms = 0.0f;
    if (rc == NEOXC_OK) cudaEventElapsedTime(&ms, ev[0], ev[1]);
    *seconds = 1e-3 * ms;
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
  }
  return rc;
}

}  // extern "C"

// ---- many systems' gam_3 in persistent launches ----------------------------
// The autotuner's choices per (angular class, precision): CTAs per SM of the
// persistent grid and work items per queue grab, with the sample rate that
// chose them (items/s); read back by neoxc_gam3_batch_tuning.
struct G3Tune {
  int ctas_per_sm = 0, chunk = 0;
  double items_per_s = 0.0;
  std::string trials;
};
static std::mutex g_tune_mu;
static std::map<int, G3Tune> g_tune;   // key: (lmax_e * 3 + lmax_p) * 2 + fp32

static int g3_tune_key(const DevSystem& S, int fp32) {
  return ((S.lmax_e * 3 + (S.lmax_p == 0 ? 0 : 2)) * 2) + fp32;
}

// Time candidate (ctas_per_sm, chunk) pairs on a sample of the batch's work
// items (the first ~8 CTA-waves) and keep the fastest.  The candidates run
// the real kernel on the real inputs; the sample's outputs are overwritten
// by the full launch that follows.
static int g3_autotune(const std::vector<G3BatchSys>& hs, int fp32, double screen,
                       void* scratch, cudaStream_t s, G3Tune* out) {
  static const int kCtas[] = {1, 2, 3, 4};
  static const int kChunks[] = {1, 4, 16};
  int dev = 0, nsm = 0;
  CU(cudaGetDevice(&dev));
  CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  G3Tune best;
  char buf[160];
  for (int c : kCtas)
    for (int ch : kChunks) {
      const long long sample = 8LL * nsm * c * ch;
      long long total = 0;
      CU(cudaEventRecord(a, s));
      CU(launch_gam3_batch_pairs(hs.data(), (int)hs.size(), fp32, screen, scratch, c, ch, sample,
                                 &total, s));
      CU(cudaEventRecord(b, s));
      CU(cudaEventSynchronize(b));
      float ms = 0.0f;
      CU(cudaEventElapsedTime(&ms, a, b));
      const long long done = sample < total ? sample : total;
      const double rate = ms > 0.0f ? done / (1e-3 * ms) : 0.0;
      snprintf(buf, sizeof(buf), "%s{\"ctas_per_sm\":%d,\"chunk\":%d,\"items_per_s\":%.4g}",
               best.trials.empty() ? "" : ",", c, ch, rate);
      best.trials += buf;
      if (rate > best.items_per_s) {
        best.items_per_s = rate;
        best.ctas_per_sm = c;
        best.chunk = ch;
      }
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *out = best;
  return NEOXC_OK;
}

extern "C" {

int neoxc_gam3_ic1_batch(const neoxc_xchf_job* jobs, int64_t njobs, int64_t options,
                         double* const* GM3ICR, double* seconds) {
  RC(need(jobs != nullptr && GM3ICR != nullptr && njobs >= 1, "jobs, GM3ICR, njobs >= 1"));
  RC(need((options & ~(int64_t)(NEOXC_SCF_MIXED | NEOXC_SCF_SCREEN)) == 0, "options"));
  const int fp32 = (options & NEOXC_SCF_MIXED) ? 1 : 0;
  const double screen = (options & NEOXC_SCF_SCREEN) ? kScreenThreshold : 0.0;
  for (int64_t k = 0; k < njobs; k++) {
    RC(need(GM3ICR[k] != nullptr, "GM3ICR[k]"));
    if (jobs[k].nebf > 20)
      return set_err(NEOXC_ERR_UNSUPPORTED, "gam_3 batch: nebf <= 20 (job %lld)", (long long)k);
  }
  cudaStream_t s;
  RC(get_stream(&s));
  std::vector<SysUpload> up((size_t)njobs);
  std::vector<DBuf> aux((size_t)njobs), r4b((size_t)njobs), g3((size_t)njobs);
  for (int64_t k = 0; k < njobs; k++) {
    const neoxc_xchf_job& j = jobs[k];
    RC(stage_system(up[k], s, j.nebf, j.npebf, j.npbf, j.nat, j.ngtg1, j.pmass, j.cat, j.zan,
                    j.bcoef1, j.gamma1, j.KPESTR, j.KPEEND, j.AGEBFCC, j.AGNBFCC, j.ELCEX,
                    j.NUCEX, j.ELCAM, j.NUCAM, j.ELCBFC, j.NUCBFC));
    if (up[k].d.g3_ntile < 1)
      return set_err(NEOXC_ERR_UNSUPPORTED, "gam_3 batch: a contracted pair has more than %d "
                                            "primitive pairs (job %lld)", kG3MaxTileKets,
                     (long long)k);
    const int ne = (int)j.nebf, np = (int)j.npbf;
    RC(dalloc(aux[k], sizeof(double) * gam3_aux_doubles(ne, np), s));
    RC(dalloc(r4b[k], sizeof(double) * gam3_r4_doubles(ne, np), s));
    const size_t ng3 = (size_t)ne * ne * ne * ne * ne * ne * np * np;
    RC(dalloc(g3[k], sizeof(double) * ng3, s));
  }
  DBuf scr;
  RC(dalloc(scr, gam3_batch_scratch_bytes((int)njobs), s));
  cudaEvent_t ev[2];
  CU(cudaEventCreate(&ev[0]));
  CU(cudaEventCreate(&ev[1]));
  RC(finish(s));
  CU(cudaEventRecord(ev[0], s));
  for (int64_t k = 0; k < njobs; k++) CU(launch_gam3_aux(up[k].d, aux[k].as<double>(), s));
  // one persistent launch per angular class
  std::map<int, std::vector<int64_t>> classes;
  for (int64_t k = 0; k < njobs; k++) classes[g3_tune_key(up[k].d, fp32)].push_back(k);
  for (auto& kv : classes) {
    std::vector<G3BatchSys> hs;
    for (int64_t k : kv.second) {
      G3BatchSys b;
      b.S = up[k].d;
      b.erec = up[k].d.g3rec;
      b.prec = up[k].d.g3rec + (size_t)32 * up[k].d.g3_nket;
      const size_t n2 = (size_t)up[k].d.nebf * up[k].d.nebf;
      const size_t p2 = (size_t)up[k].d.npbf * up[k].d.npbf;
      b.r4a = aux[k].as<double>() + n2 * n2 + n2 + p2 * n2 + p2 * n2 * n2;
      b.r4b = r4b[k].as<double>();
      hs.push_back(b);
    }
    G3Tune t;
    bool have = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(kv.first);
      if (it != g_tune.end()) {
        t = it->second;
        have = true;
      }
    }
    if (!have) {
      RC(g3_autotune(hs, fp32, screen, scr.p, s, &t));
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[kv.first] = t;
    }
    CU(launch_gam3_batch_pairs(hs.data(), (int)hs.size(), fp32, screen, scr.p, t.ctas_per_sm,
                               t.chunk, -1, nullptr, s));
  }
  for (int64_t k = 0; k < njobs; k++) {
    const int ne = up[k].d.nebf, np = up[k].d.npbf;
    const size_t n2 = (size_t)ne * ne, p2 = (size_t)np * np;
    double* r4a = aux[k].as<double>() + n2 * n2 + n2 + p2 * n2 + p2 * n2 * n2;
    CU(launch_gam3_add((long long)gam3_r4_doubles(ne, np), r4a, r4b[k].as<double>(), s));
    const long long ng3 = (long long)(n2 * n2 * n2 * p2);
    CU(launch_gam3_raw_range(up[k].d, aux[k].as<double>(), 0, ng3, g3[k].as<double>(), s));
    CU(launch_gam3_symmetrize(ne, np, g3[k].as<double>(), s));
  }
  CU(cudaEventRecord(ev[1], s));
  for (int64_t k = 0; k < njobs; k++) {
    const int ne = up[k].d.nebf, np = up[k].d.npbf;
    const size_t ng3 = (size_t)ne * ne * ne * ne * ne * ne * np * np;
    CU(cudaMemcpyAsync(GM3ICR[k], g3[k].p, sizeof(double) * ng3, cudaMemcpyDeviceToHost, s));
  }
  const int rc = finish(s);
  if (seconds) {
    float ms = 0.0f;
    if (rc == NEOXC_OK) cudaEventElapsedTime(&ms, ev[0], ev[1]);
    *seconds = 1e-3 * ms;
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  return rc;
}

int neoxc_set_mixed_threshold(double tau) {
  if (!(tau >= 0.0)) return set_err(NEOXC_ERR_ARG, "mixed threshold: tau >= 0");
  set_mixed_recompute_tau(tau);
  return NEOXC_OK;
}

double neoxc_get_mixed_threshold(void) { return mixed_recompute_tau(); }

int64_t neoxc_gam3_batch_tuning(char* buf, int64_t len) {
  std::string out = "[";
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    bool first = true;
    for (auto& kv : g_tune) {
      const int fp32 = kv.first & 1, cls = kv.first >> 1;
      char line[256];
      snprintf(line, sizeof(line),
               "%s{\"lmax_e\":%d,\"lmax_p_class\":%d,\"fp32\":%d,\"ctas_per_sm\":%d,"
               "\"chunk\":%d,\"items_per_s\":%.4g,\"trials\":[",
               first ? "" : ",", cls / 3, cls % 3, fp32, kv.second.ctas_per_sm, kv.second.chunk,
               kv.second.items_per_s);
      out += line;
      out += kv.second.trials + "]}";
      first = false;
    }
  }
  out += "]";
  if (buf && len > 0) {
    const size_t n = out.size() < (size_t)(len - 1) ? out.size() : (size_t)(len - 1);
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return (int64_t)out.size();
}

int neoxc_gam3_ic1(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                   int64_t ng3, int64_t ng3prm, int64_t nat, int64_t ngtg1,
                   double pmass, const double* cat, const double* zan,
                   const double* bcoef1, const double* gamma1,
                   const int64_t* KPESTR, const int64_t* KPEEND,
                   const int64_t* AMPEB2C, const double* AGEBFCC,
                   const double* AGNBFCC, const double* ELCEX,
                   const double* NUCEX, const int64_t* ELCAM,
                   const int64_t* NUCAM, const double* ELCBFC,
                   const double* NUCBFC, double* GM3ICR) {
  return neoxc_gam3_ic1_opts(0, Nchunks, nebf, npebf, npbf, ng3, ng3prm, nat, ngtg1, pmass,
                             cat, zan, bcoef1, gamma1, KPESTR, KPEEND, AMPEB2C, AGEBFCC,
                             AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC, GM3ICR,
                             nullptr);
}

int neoxc_gam4_icr(int64_t Nchunks, int64_t ne, int64_t np, int64_t ngee,
                   int64_t ng2, int64_t ng4, const double* GAM_2s,
                   const double* GAM_ee, double* GAM_4) {
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ngee == ne * ne * ne * ne, "ngee == ne**4"));
  RC(need(ng2 == ngee * np * np, "ng2 == ne**4 np**2"));
  RC(need(ng4 == ngee * ngee * np * np, "ng4 == ne**8 np**2"));
  RC(need(GAM_2s && GAM_ee && GAM_4, "pointers"));
  if (ne > kGam4MaxNE)
    return set_err(NEOXC_ERR_UNSUPPORTED, "gam_4 element kernels: ne <= %d",
                   kGam4MaxNE);
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dg2, dee, d4;
  RC(upload(dg2, GAM_2s, sizeof(double) * ng2, s));
  RC(upload(dee, GAM_ee, sizeof(double) * ngee, s));
  RC(dalloc(d4, sizeof(double) * ng4, s));
  CU(launch_gam4_icr((int)ne, (int)np, dee.as<double>(), dg2.as<double>(),
                     d4.as<double>(), s));
  CU(cudaMemcpyAsync(GAM_4, d4.p, sizeof(double) * ng4, cudaMemcpyDeviceToHost,
                     s));
  return finish(s);
}

// ---- contractions -------------------------------------------------------------
int neoxc_dev_gam4_dscf(void* stream, int64_t ne, int64_t np,
                        const double* d_gee, const double* d_g2s,
                        const double* d_DE, const double* d_DP,
                        double* d_focke, double* d_fockp, double* d_E) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  if (ne > kGam4MaxNE || np > kGam4MaxNP)
    return set_err(NEOXC_ERR_UNSUPPORTED,
                   "gam_4 element kernels: ne <= %d, np <= %lld", kGam4MaxNE,
                   (long long)kGam4MaxNP);
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  RC(dalloc(scr, sizeof(double) * gam4_partial_doubles((int)ne, (int)np), s));
  CU(launch_gam4_dscf((int)ne, (int)np, d_gee, d_g2s, d_DE, d_DP,
                      scr.as<double>(), d_focke, d_fockp, d_E, s));
  return NEOXC_OK;
}

int neoxc_gam4_dscf(int64_t NG4CHK, int64_t ne, int64_t np, int64_t ngee,
                    int64_t ng2, int64_t ng4, const double* GAM_ee,
                    const double* GAM_2s, const double* DE, const double* DP,
                    double* focke, double* fockp, double* E_gam4) {
  RC(need(NG4CHK >= 1, "NG4CHK >= 1"));
  RC(need(ngee == ne * ne * ne * ne, "ngee == ne**4"));
  RC(need(ng2 == ngee * np * np, "ng2 == ne**4 np**2"));
  RC(need(ng4 == ngee * ngee * np * np, "ng4 == ne**8 np**2"));
  RC(need(GAM_ee && GAM_2s && DE && DP && focke && fockp && E_gam4, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dee, dg2, dde, ddp, dfe, dfp, dE;
  RC(upload(dee, GAM_ee, sizeof(double) * ngee, s));
  RC(upload(dg2, GAM_2s, sizeof(double) * ng2, s));
  RC(upload(dde, DE, sizeof(double) * ne * ne, s));
  RC(upload(ddp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfe, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dE, sizeof(double), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  RC(neoxc_dev_gam4_dscf(s, ne, np, dee.as<double>(), dg2.as<double>(),
                         dde.as<double>(), ddp.as<double>(), dfe.as<double>(),
                         dfp.as<double>(), dE.as<double>()));
  RC(accumulate_back(focke, dfe.as<double>(), ne * ne, s));
  RC(accumulate_back(fockp, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(E_gam4, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

// ---- factorised gam_4 Fock build ----------------------------------------------
int neoxc_dev_gam4_fock_factored_tc(void* stream, int64_t ne, int64_t np,
                                    const double* d_gee, const double* d_g2s,
                                    const double* d_DE, const double* d_DP,
                                    double* d_focke, double* d_fockp, double* d_E) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  if (ne > kGam4FactMaxNE || np > 255)
    return set_err(NEOXC_ERR_UNSUPPORTED,
                   "factorised gam_4 Fock build: ne <= %d, np <= 255",
                   kGam4FactMaxNE);
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  const size_t nd = gam4f_tc_scratch_doubles((int)ne, (int)np);
  RC(dalloc(scr, sizeof(double) * nd, s));
  CU(launch_gam4_factored_tc((int)ne, (int)np, d_gee, d_g2s, d_DE, d_DP,
                             scr.as<double>(), d_focke, d_fockp, d_E, 1, s));
  int flag = 0;   // the tensor-core waits' error flag, last word of the scratch
  CU(cudaMemcpyAsync(&flag, scr.as<double>() + nd - 2, sizeof(int),
                     cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  if (flag)
    return set_err(NEOXC_ERR_CUDA, "factorised gam_4 (tensor cores): an MMA completion "
                                   "wait ran out; results not written");
  return NEOXC_OK;
}

int neoxc_dev_gam4_fock_factored(void* stream, int64_t ne, int64_t np,
                                 const double* d_gee, const double* d_g2s,
                                 const double* d_DE, const double* d_DP,
                                 double* d_focke, double* d_fockp,
                                 double* d_E) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  if (ne > kGam4FactMaxNE || np > 255)
    return set_err(NEOXC_ERR_UNSUPPORTED,
                   "factorised gam_4 Fock build: ne <= %d, np <= 255",
                   kGam4FactMaxNE);
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  RC(dalloc(scr, sizeof(double) * gam4f_scratch_doubles((int)ne, (int)np), s));
  CU(launch_gam4_factored((int)ne, (int)np, d_gee, d_g2s, d_DE, d_DP,
                          scr.as<double>(), d_focke, d_fockp, d_E, 1, s));
  return NEOXC_OK;
}

int neoxc_gam4_fock_factored(int64_t ne, int64_t np, int64_t ngee,
                             int64_t ng2, const double* GAM_ee,
                             const double* GAM_2s, const double* DE,
                             const double* DP, double* focke, double* fockp,
                             double* E_gam4) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  if (ne > kGam4FactMaxNE || np > 255)
    return set_err(NEOXC_ERR_UNSUPPORTED,
                   "factorised gam_4 Fock build: ne <= %d, np <= 255",
                   kGam4FactMaxNE);
  RC(need(ngee == ne * ne * ne * ne, "ngee == ne**4"));
  RC(need(ng2 == ngee * np * np, "ng2 == ne**4 np**2"));
  RC(need(GAM_ee && GAM_2s && DE && DP && focke && fockp && E_gam4, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dee, dg2, dde, ddp, dfe, dfp, dE, dchk;
  RC(upload(dee, GAM_ee, sizeof(double) * ngee, s));
  RC(upload(dg2, GAM_2s, sizeof(double) * ng2, s));
  // The factorisation holds for pair-symmetric tables (what GAM2_IC1 and
  // calc_GAM_ee produce); refuse others instead of returning a different sum.
  RC(dalloc(dchk, sizeof(double) * 4 * 152 * 16, s));
  int grid = 0;
  CU(launch_pair_symmetry_check((int)ne, (int)np, dee.as<double>(),
                                dg2.as<double>(), dchk.as<double>(), &grid, s));
  std::vector<double> chk(4 * (size_t)grid);
  CU(cudaMemcpyAsync(chk.data(), dchk.p, sizeof(double) * chk.size(),
                     cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  for (int g = 0; g < grid; g++)
    for (int k = 0; k < 4; k++) m[k] = chk[4 * g + k] > m[k] ? chk[4 * g + k] : m[k];
  if (m[0] > 1e-12 * m[1])
    return set_err(NEOXC_ERR_ARG,
                   "factorised gam_4: GAM_ee is not symmetric under pair exchange "
                   "(max |(ab|cd)-(cd|ab)| = %.3e, max |(ab|cd)| = %.3e)", m[0], m[1]);
  if (m[2] > 1e-12 * m[3])
    return set_err(NEOXC_ERR_ARG,
                   "factorised gam_4: GAM_2s is not pair-symmetric (max "
                   "|gs(p;ab;cd)-gs(p;cd;ab)| = %.3e, max |gs| = %.3e)", m[2], m[3]);
  RC(upload(dde, DE, sizeof(double) * ne * ne, s));
  RC(upload(ddp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfe, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dE, sizeof(double), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  RC(neoxc_dev_gam4_fock_factored(s, ne, np, dee.as<double>(), dg2.as<double>(),
                                  dde.as<double>(), ddp.as<double>(),
                                  dfe.as<double>(), dfp.as<double>(),
                                  dE.as<double>()));
  RC(accumulate_back(focke, dfe.as<double>(), ne * ne, s));
  RC(accumulate_back(fockp, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(E_gam4, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

int neoxc_eg4icr(int64_t Nchunks, int64_t ne, int64_t np, int64_t ng4,
                 const double* DE, const double* DP, const double* GM4ICR,
                 double* focke, double* fockp, double* E_gam4) {
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ng4 == ne * ne * ne * ne * ne * ne * ne * ne * np * np,
          "ng4 == ne**8 np**2"));
  RC(need(DE && DP && GM4ICR && focke && fockp && E_gam4, "pointers"));
  if (ne > kGam4MaxNE)
    return set_err(NEOXC_ERR_UNSUPPORTED, "EG4ICR: ne <= %d", kGam4MaxNE);
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dg, dde, ddp, dfe, dfp, dE, scr;
  RC(upload(dg, GM4ICR, sizeof(double) * ng4, s));
  RC(upload(dde, DE, sizeof(double) * ne * ne, s));
  RC(upload(ddp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfe, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dE, sizeof(double), s));
  RC(dalloc(scr, sizeof(double) * eg4_partial_doubles((int)ne, (int)np), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  CU(launch_eg4icr((int)ne, (int)np, dde.as<double>(), ddp.as<double>(),
                   dg.as<double>(), scr.as<double>(), dfe.as<double>(),
                   dfp.as<double>(), dE.as<double>(), s));
  RC(accumulate_back(focke, dfe.as<double>(), ne * ne, s));
  RC(accumulate_back(fockp, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(E_gam4, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

int neoxc_dev_eg3ic1(void* stream, int64_t ne, int64_t np, const double* d_DE,
                     const double* d_DP, const double* d_g3, double* d_focke,
                     double* d_fockp, double* d_E) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  if (ne > 20) return set_err(NEOXC_ERR_UNSUPPORTED, "EG3IC1: ne <= 20");
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  RC(dalloc(scr, sizeof(double) * eg3_partial_doubles((int)ne, (int)np), s));
  CU(launch_eg3ic1((int)ne, (int)np, d_DE, d_DP, d_g3, scr.as<double>(),
                   d_focke, d_fockp, d_E, s));
  return NEOXC_OK;
}

int neoxc_eg3ic1(int64_t Nchunks, int64_t ne, int64_t np, int64_t ng3,
                 const double* DE, const double* DP, const double* GM3ICR,
                 double* focke, double* fockp, double* E_gam3) {
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ng3 == ne * ne * ne * ne * ne * ne * np * np, "ng3 == ne**6 np**2"));
  RC(need(DE && DP && GM3ICR && focke && fockp && E_gam3, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dg, dde, ddp, dfe, dfp, dE;
  RC(upload(dg, GM3ICR, sizeof(double) * ng3, s));
  RC(upload(dde, DE, sizeof(double) * ne * ne, s));
  RC(upload(ddp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfe, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dE, sizeof(double), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  RC(neoxc_dev_eg3ic1(s, ne, np, dde.as<double>(), ddp.as<double>(),
                      dg.as<double>(), dfe.as<double>(), dfp.as<double>(),
                      dE.as<double>()));
  RC(accumulate_back(focke, dfe.as<double>(), ne * ne, s));
  RC(accumulate_back(fockp, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(E_gam3, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

int neoxc_dev_eg2ic1(void* stream, int64_t ne, int64_t np, const double* d_DE,
                     const double* d_DP, const double* d_g2,
                     const double* d_g2s, double* d_FE, double* d_SE,
                     double* d_FP, double* d_SP, double* d_E, double* d_S) {
  RC(need(ne >= 1 && np >= 1, "sizes"));
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  RC(dalloc(scr, sizeof(double) * eg2_partial_doubles((int)ne, (int)np), s));
  CU(launch_eg2ic1((int)ne, (int)np, d_DE, d_DP, d_g2, d_g2s, scr.as<double>(),
                   d_FE, d_SE, d_FP, d_SP, d_E, d_S, s));
  return NEOXC_OK;
}

int neoxc_eg2ic1(int64_t Nchunks, int64_t ne, int64_t np, int64_t ng2,
                 const double* DE, const double* DP, const double* GM2ICR,
                 const double* GM2SICR, double* FE, double* SE, double* FP,
                 double* SP, double* E_gam2, double* S_gam2) {
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ng2 == ne * ne * ne * ne * np * np, "ng2 == ne**4 np**2"));
  RC(need(DE && DP && GM2ICR && GM2SICR && FE && SE && FP && SP && E_gam2 &&
              S_gam2, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dg, dgs, dde, ddp, dfe, dse, dfp, dsp, dE;
  RC(upload(dg, GM2ICR, sizeof(double) * ng2, s));
  RC(upload(dgs, GM2SICR, sizeof(double) * ng2, s));
  RC(upload(dde, DE, sizeof(double) * ne * ne, s));
  RC(upload(ddp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfe, sizeof(double) * ne * ne, s));
  RC(dalloc(dse, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dsp, sizeof(double) * np * np, s));
  RC(dalloc(dE, 2 * sizeof(double), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  RC(neoxc_dev_eg2ic1(s, ne, np, dde.as<double>(), ddp.as<double>(),
                      dg.as<double>(), dgs.as<double>(), dfe.as<double>(),
                      dse.as<double>(), dfp.as<double>(), dsp.as<double>(),
                      dE.as<double>(), dE.as<double>() + 1));
  RC(accumulate_back(FE, dfe.as<double>(), ne * ne, s));
  RC(accumulate_back(FP, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(SE, dse.p, sizeof(double) * ne * ne, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(SP, dsp.p, sizeof(double) * np * np, cudaMemcpyDeviceToHost, s));
  double e2[2];
  CU(cudaMemcpyAsync(e2, dE.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  *E_gam2 = e2[0];
  *S_gam2 = e2[1];
  return NEOXC_OK;
}

int neoxc_dev_rxchfne_omg2(void* stream, int64_t ne, int64_t np,
                           const double* d_DAE, const double* d_DBE,
                           const double* d_DP, const double* d_g2,
                           double* d_FAE, double* d_FP, double* d_FBE,
                           double* d_E) {
  RC(need(ne >= 1 && np >= 1 && ne * ne <= 16384, "sizes"));
  cudaStream_t s = (cudaStream_t)stream;
  DBuf scr;
  RC(dalloc(scr, sizeof(double) * omg2_partial_doubles((int)ne, (int)np), s));
  CU(launch_rxchfne_omg2((int)ne, (int)np, d_DAE, d_DBE, d_DP, d_g2,
                         scr.as<double>(), d_FAE, d_FP, d_FBE, d_E, s));
  return NEOXC_OK;
}

static int omg2_host(int64_t ne, int64_t np, const double* DAE,
                     const double* DBE, const double* DP, const double* G,
                     double* FAE, double* FP, double* FBE, double* E) {
  RC(need(DAE && DBE && DP && G && E, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  const int64_t ng2 = ne * ne * ne * ne * np * np;
  DBuf dg, da, db, dp, dfa, dfp, dfb, dE;
  RC(upload(dg, G, sizeof(double) * ng2, s));
  RC(upload(da, DAE, sizeof(double) * ne * ne, s));
  RC(upload(db, DBE, sizeof(double) * ne * ne, s));
  RC(upload(dp, DP, sizeof(double) * np * np, s));
  RC(dalloc(dfa, sizeof(double) * ne * ne, s));
  RC(dalloc(dfb, sizeof(double) * ne * ne, s));
  RC(dalloc(dfp, sizeof(double) * np * np, s));
  RC(dalloc(dE, sizeof(double), s));
  CU(cudaMemsetAsync(dfa.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfb.p, 0, sizeof(double) * ne * ne, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * np * np, s));
  RC(neoxc_dev_rxchfne_omg2(s, ne, np, da.as<double>(), db.as<double>(),
                            dp.as<double>(), dg.as<double>(),
                            FAE ? dfa.as<double>() : nullptr,
                            FP ? dfp.as<double>() : nullptr,
                            FBE ? dfb.as<double>() : nullptr, dE.as<double>()));
  if (FAE) RC(accumulate_back(FAE, dfa.as<double>(), ne * ne, s));
  if (FBE) RC(accumulate_back(FBE, dfb.as<double>(), ne * ne, s));
  if (FP) RC(accumulate_back(FP, dfp.as<double>(), np * np, s));
  CU(cudaMemcpyAsync(E, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

int neoxc_rxchfne_fae_omg2(int64_t Nchunks, int64_t ne, int64_t np,
                           int64_t ng2, const double* DAE, const double* DBE,
                           const double* DP, const double* G, double* FAE,
                           double* E) {
  RC(need(Nchunks >= 1 && ng2 == ne * ne * ne * ne * np * np && FAE, "sizes"));
  return omg2_host(ne, np, DAE, DBE, DP, G, FAE, nullptr, nullptr, E);
}
int neoxc_rxchfne_fp_omg2(int64_t Nchunks, int64_t ne, int64_t np,
                          int64_t ng2, int64_t NAE, int64_t NBE,
                          const double* DAE, const double* DBE,
                          const double* DP, const double* G, double* FP,
                          double* E) {
  (void)NAE;
  (void)NBE;
  RC(need(Nchunks >= 1 && ng2 == ne * ne * ne * ne * np * np && FP, "sizes"));
  return omg2_host(ne, np, DAE, DBE, DP, G, nullptr, FP, nullptr, E);
}
int neoxc_rxchfne_fbe_omg2(int64_t Nchunks, int64_t ne, int64_t np,
                           int64_t ng2, int64_t NAE, int64_t NBE,
                           const double* DAE, const double* DBE,
                           const double* DP, const double* G, double* FBE,
                           double* E) {
  (void)NAE;
  (void)NBE;
  RC(need(Nchunks >= 1 && ng2 == ne * ne * ne * ne * np * np && FBE, "sizes"));
  return omg2_host(ne, np, DAE, DBE, DP, G, nullptr, nullptr, FBE, E);
}
int neoxc_rxchfne_omg2_fused(int64_t ne, int64_t np, const double* DAE,
                             const double* DBE, const double* DP,
                             const double* G, double* FAE, double* FP,
                             double* FBE, double* E) {
  RC(need(ne >= 1 && np >= 1 && FAE && FP && FBE, "sizes"));
  return omg2_host(ne, np, DAE, DBE, DP, G, FAE, FP, FBE, E);
}

int neoxc_xcfock_correction(int64_t ne, int64_t np, double E_total,
                            double S_total, double H_expect,
                            const double* se1, const double* sp1,
                            const double* se2, const double* sp2,
                            double* focke, double* fockp) {
  (void)E_total;
  RC(need(ne >= 1 && np >= 1 && se1 && sp1 && se2 && sp2 && focke && fockp,
          "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf a, b, c, d, fe, fp;
  RC(upload(a, se1, sizeof(double) * ne * ne, s));
  RC(upload(b, sp1, sizeof(double) * np * np, s));
  RC(upload(c, se2, sizeof(double) * ne * ne, s));
  RC(upload(d, sp2, sizeof(double) * np * np, s));
  RC(upload(fe, focke, sizeof(double) * ne * ne, s));
  RC(upload(fp, fockp, sizeof(double) * np * np, s));
  CU(launch_xcfock_correction((int)ne, (int)np, S_total, H_expect,
                              a.as<double>(), b.as<double>(), c.as<double>(),
                              d.as<double>(), fe.as<double>(), fp.as<double>(),
                              s));
  CU(cudaMemcpyAsync(focke, fe.p, sizeof(double) * ne * ne,
                     cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(fockp, fp.p, sizeof(double) * np * np,
                     cudaMemcpyDeviceToHost, s));
  return finish(s);
}

// ---- direct-SCF builders: slice by proton pair, never hold the tensor --------
// gam3_DSCF_OMP.f:2-137 GAM3_DSCF.  For each proton pair (ip,jp) the raw
// gam_3 slice (nebf^6 doubles) is built, six-permutation symmetrised in place
// and contracted into per-CTA partials; one reduction gives the Fock
// matrices (accumulated) and E_gam3 (overwritten).  Nchunks (the reference's
// NG3CHK) is accepted and validated; the slicing is by proton pair.
// The direct gam_3 loop on device buffers: dfe, dfp accumulate (one add of
// the finished contraction, like add2fock), dE overwritten.
static int gam3_dscf_dev(const SysUpload& u, cudaStream_t s, const double* dde,
                         const double* ddp, double* dfe, double* dfp,
                         double* dE) {
  const int ne = u.d.nebf, np = u.d.npbf;
  const int64_t n6 = (int64_t)ne * ne * ne * ne * ne * ne;
  DBuf slice, part, aux;
  RC(dalloc(slice, sizeof(double) * n6, s));
  RC(dalloc(part, sizeof(double) * eg3_partial_doubles(ne, np), s));
  RC(dalloc(aux, sizeof(double) * gam3_aux_doubles(ne, np), s));
  CU(launch_gam3_aux(u.d, aux.as<double>(), s));
  CU(launch_gam3_pairs(u.d, aux.as<double>(), s, 0, 0.0));
  for (int64_t pp = 0; pp < (int64_t)np * np; pp++) {
    CU(launch_gam3_raw_range(u.d, aux.as<double>(), pp * n6, n6,
                             slice.as<double>(), s));
    CU(launch_gam3_symmetrize(ne, 1, slice.as<double>(), s));
    CU(launch_eg3_partials(ne, np, pp, 1, dde, slice.as<double>(),
                           part.as<double>(), s));
  }
  const size_t nparts = (size_t)np * np * ne * ne * ne * ne;
  CU(launch_fock_reduce(ne, np, ne * ne, part.as<double>(), dde, ddp, 3.0, 1,
                        dfe, dfp, part.as<double>() + nparts, dE, s));
  return NEOXC_OK;
}

int neoxc_gam3_dscf(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                    int64_t ng3, int64_t ng3prm, int64_t nat, int64_t ngtg1,
                    double pmass, const double* cat, const double* zan,
                    const double* bcoef1, const double* gamma1,
                    const int64_t* KPESTR, const int64_t* KPEEND,
                    const int64_t* AMPEB2C, const double* AGEBFCC,
                    const double* AGNBFCC, const double* ELCEX,
                    const double* NUCEX, const int64_t* ELCAM,
                    const int64_t* NUCAM, const double* ELCBFC,
                    const double* NUCBFC, const double* DE, const double* DP,
                    double* focke, double* fockp, double* E_gam3) {
  (void)AMPEB2C;
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  const int64_t n6 = nebf * nebf * nebf * nebf * nebf * nebf;
  RC(need(ng3 == n6 * npbf * npbf, "ng3 == nebf**6 * npbf**2"));
  RC(need(ng3prm == npebf * npebf * npebf * npebf * npebf * npebf * npbf * npbf,
          "ng3prm"));
  RC(need(DE && DP && focke && fockp && E_gam3, "pointers"));
  if (nebf > 20) return set_err(NEOXC_ERR_UNSUPPORTED, "GAM3_DSCF: nebf <= 20");
  cudaStream_t s;
  RC(get_stream(&s));
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1,
                  gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                  NUCAM, ELCBFC, NUCBFC));
  DBuf dde, ddp, dfe, dfp, dE;
  RC(upload(dde, DE, sizeof(double) * nebf * nebf, s));
  RC(upload(ddp, DP, sizeof(double) * npbf * npbf, s));
  RC(dalloc(dfe, sizeof(double) * nebf * nebf, s));
  RC(dalloc(dfp, sizeof(double) * npbf * npbf, s));
  RC(dalloc(dE, sizeof(double), s));
  CU(cudaMemsetAsync(dfe.p, 0, sizeof(double) * nebf * nebf, s));
  CU(cudaMemsetAsync(dfp.p, 0, sizeof(double) * npbf * npbf, s));
  RC(gam3_dscf_dev(u, s, dde.as<double>(), ddp.as<double>(), dfe.as<double>(),
                   dfp.as<double>(), dE.as<double>()));
  RC(accumulate_back(focke, dfe.as<double>(), nebf * nebf, s));
  RC(accumulate_back(fockp, dfp.as<double>(), npbf * npbf, s));
  CU(cudaMemcpyAsync(E_gam3, dE.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  return finish(s);
}

// gam2_DSCF_OMP.f:2-140 GAM2_DSCF on device buffers: dfe, dfp, dse, dsp
// accumulate (the reference's add2fock); dE[0] = E_gam2, dE[1] = S_gam2.
static int gam2_dscf_dev(const SysUpload& u, cudaStream_t s, const double* dde,
                         const double* ddp, double* dfe, double* dfp,
                         double* dse, double* dsp, double* dE, double* dS) {
  const int ne = u.d.nebf, np = u.d.npbf;
  const int64_t n4 = (int64_t)ne * ne * ne * ne;
  const size_t npart = (size_t)np * np * ne * ne * ne;
  DBuf s1, s2, part;
  RC(dalloc(s1, sizeof(double) * n4, s));
  RC(dalloc(s2, sizeof(double) * n4, s));
  RC(dalloc(part, sizeof(double) * (2 * npart + 2 * np * np), s));
  double* pv = part.as<double>();
  double* ps = pv + npart;
  double* ftmp = ps + npart;
  for (int64_t pp = 0; pp < (int64_t)np * np; pp++) {
    CU(launch_gam2_raw_range(u.d, 0, pp * n4, n4, s1.as<double>(),
                             s2.as<double>(), s));
    CU(launch_gam2_symmetrize(ne, 1, 0, s1.as<double>(), s2.as<double>(), s));
    CU(launch_eg2_partials(ne, np, pp, 1, dde, s1.as<double>(),
                           s2.as<double>(), pv, ps, s));
  }
  CU(launch_fock_reduce(ne, np, ne, pv, dde, ddp, 2.0, 1, dfe, dfp, ftmp, dE, s));
  CU(launch_fock_reduce(ne, np, ne, ps, dde, ddp, 1.0, 1, dse, dsp,
                        ftmp + np * np, dS, s));
  return NEOXC_OK;
}

int neoxc_gam2_dscf(int64_t Nchunks, int64_t nebf, int64_t npebf, int64_t npbf,
                    int64_t ng2, int64_t ng2prm, int64_t nat, int64_t ngtg1,
                    double pmass, const double* cat, const double* zan,
                    const double* bcoef1, const double* gamma1,
                    const int64_t* KPESTR, const int64_t* KPEEND,
                    const int64_t* AMPEB2C, const double* AGEBFCC,
                    const double* AGNBFCC, const double* ELCEX,
                    const double* NUCEX, const int64_t* ELCAM,
                    const int64_t* NUCAM, const double* ELCBFC,
                    const double* NUCBFC, const double* DE, const double* DP,
                    double* focke, double* fockp, double* se2, double* sp2,
                    double* E_gam2, double* S_gam2) {
  (void)AMPEB2C;
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  const int64_t n4 = nebf * nebf * nebf * nebf;
  RC(need(ng2 == n4 * npbf * npbf, "ng2 == nebf**4 * npbf**2"));
  RC(need(ng2prm == npebf * npebf * npebf * npebf * npbf * npbf, "ng2prm"));
  RC(need(DE && DP && focke && fockp && se2 && sp2 && E_gam2 && S_gam2,
          "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1,
                  gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                  NUCAM, ELCBFC, NUCBFC));
  DBuf dde, ddp, dfe, dfp, dse, dsp, dE;
  RC(upload(dde, DE, sizeof(double) * nebf * nebf, s));
  RC(upload(ddp, DP, sizeof(double) * npbf * npbf, s));
  RC(dalloc(dfe, sizeof(double) * nebf * nebf, s));
  RC(dalloc(dfp, sizeof(double) * npbf * npbf, s));
  RC(dalloc(dse, sizeof(double) * nebf * nebf, s));
  RC(dalloc(dsp, sizeof(double) * npbf * npbf, s));
  RC(dalloc(dE, 2 * sizeof(double), s));
  for (DBuf* b : {&dfe, &dse}) CU(cudaMemsetAsync(b->p, 0, sizeof(double) * nebf * nebf, s));
  for (DBuf* b : {&dfp, &dsp}) CU(cudaMemsetAsync(b->p, 0, sizeof(double) * npbf * npbf, s));
  RC(gam2_dscf_dev(u, s, dde.as<double>(), ddp.as<double>(), dfe.as<double>(),
                   dfp.as<double>(), dse.as<double>(), dsp.as<double>(),
                   dE.as<double>(), dE.as<double>() + 1));
  RC(accumulate_back(focke, dfe.as<double>(), nebf * nebf, s));
  RC(accumulate_back(fockp, dfp.as<double>(), npbf * npbf, s));
  RC(accumulate_back(se2, dse.as<double>(), nebf * nebf, s));
  RC(accumulate_back(sp2, dsp.as<double>(), npbf * npbf, s));
  double e2[2];
  CU(cudaMemcpyAsync(e2, dE.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  *E_gam2 = e2[0];
  *S_gam2 = e2[1];
  return NEOXC_OK;
}

// ---- XCHF RHF SCF on the device (xchf1_independent/xcscf.f:2-658) ----------
// class_nuc_rep.f:2-45
static double nuc_rep(int64_t nat, const double* zan, const double* cat) {
  double E = 0.0;
  for (int64_t i = 1; i < nat; i++)
    for (int64_t j = 0; j < i; j++) {
      double R2 = 0.0;
      for (int k = 0; k < 3; k++) {
        const double d = cat[3 * i + k] - cat[3 * j + k];
        R2 = R2 + d * d;
      }
      if (R2 != 0.0) E = E + zan[i] * zan[j] / sqrt(R2);
    }
  return E;
}

int neoxc_class_nuc_rep(int64_t nat, const double* zan, const double* cat,
                        double* E_nuc) {
  RC(need(nat >= 0 && E_nuc && (nat == 0 || (zan && cat)), "nat, zan, cat, E_nuc"));
  *E_nuc = nuc_rep(nat, zan, cat);
  return NEOXC_OK;
}

// ---- one-body tables: pure_ovlap.f, gam_epcore.f, gam_ep.f, gam_1_OMP.f ----
// The same kernels the device SCF builds its tables with; outputs that are
// not asked for are not computed, and the parts of the system only they
// need are replaced by one s function at the origin.
static int onebody_impl(int64_t nebf, int64_t npebf, int64_t npbf, int64_t nat,
                        int64_t ngtg1, double pmass, const double* cat, const double* zan,
                        const double* bcoef1, const double* gamma1,
                        const int64_t* AMPEB2C, const double* AGEBFCC,
                        const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                        const int64_t* ELCAM, const int64_t* NUCAM, const double* ELCBFC,
                        const double* NUCBFC, double* Se, double* Sp, double* GAM_ecore,
                        double* GAM_pcore, double* GAM_ep, double* GAM_1, double* GAM_1s,
                        int gam1_pairs_only) {
  const bool want_g1 = GAM_1 || GAM_1s;
  const bool want_core = GAM_ecore || GAM_pcore;
  const bool want_e = Se || GAM_ecore || GAM_ep || want_g1;
  const bool want_p = Sp || GAM_pcore || GAM_ep || want_g1;
  if (!want_e && !want_p) return NEOXC_OK;
  if (want_e)
    RC(need(nebf >= 1 && npebf >= nebf && AMPEB2C && AGEBFCC && ELCEX && ELCAM &&
                ELCBFC,
            "electronic basis"));
  if (want_p) RC(need(npbf >= 1 && AGNBFCC && NUCEX && NUCAM && NUCBFC, "nuclear basis"));
  const bool nuclei = want_core || want_g1;
  if (nuclei) {
    RC(need(nat >= 0 && (nat == 0 || (zan && cat)), "nat, zan, cat"));
    RC(need(pmass > 0.0, "pmass > 0"));
  }
  if (want_g1) RC(need(ngtg1 >= 1 && bcoef1 && gamma1, "ngtg1 >= 1, bcoef1, gamma1"));
  const double one = 1.0, zero3[3] = {0.0, 0.0, 0.0}, b0 = 0.0;
  const int64_t l0[3] = {0, 0, 0};
  const int64_t ne = want_e ? nebf : 1, npe = want_e ? npebf : 1;
  const int64_t np = want_p ? npbf : 1;
  std::vector<int64_t> kps((size_t)ne, 1), kpe((size_t)ne, 1);
  if (want_e) RC(neoxc_make_kpe(ne, npe, AMPEB2C, kps.data(), kpe.data()));
  const int64_t na = nuclei ? nat : 0;
  cudaStream_t s;
  RC(get_stream(&s));
  SysUpload u;
  RC(stage_system(u, s, ne, npe, np, na, want_g1 ? ngtg1 : 1, nuclei ? pmass : 1.0,
                  na ? cat : zero3, na ? zan : &one, want_g1 ? bcoef1 : &b0,
                  want_g1 ? gamma1 : &one, kps.data(), kpe.data(),
                  want_e ? AGEBFCC : &one, want_p ? AGNBFCC : &one,
                  want_e ? ELCEX : &one, want_p ? NUCEX : &one, want_e ? ELCAM : l0,
                  want_p ? NUCAM : l0, want_e ? ELCBFC : zero3,
                  want_p ? NUCBFC : zero3));
  const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np, n1 = e2 * p2;
  DBuf a, b, c, d, g, g1, g1s;
  auto back = [&](double* host, const DBuf& dev, size_t n) -> int {
    if (host)
      CU(cudaMemcpyAsync(host, dev.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    return NEOXC_OK;
  };
  if (Se || Sp || want_core) {
    RC(dalloc(a, sizeof(double) * e2, s));
    RC(dalloc(b, sizeof(double) * p2, s));
    RC(dalloc(c, sizeof(double) * e2, s));
    RC(dalloc(d, sizeof(double) * p2, s));
    CU(launch_scf_onebody(u.d, a.as<double>(), b.as<double>(), c.as<double>(),
                          d.as<double>(), s));
    RC(back(Se, a, e2));
    RC(back(Sp, b, p2));
    RC(back(GAM_ecore, c, e2));
    RC(back(GAM_pcore, d, p2));
  }
  if (GAM_ep) {
    RC(dalloc(g, sizeof(double) * n1, s));
    CU(launch_gam_ep(u.d, g.as<double>(), s));
    RC(back(GAM_ep, g, n1));
  }
  if (want_g1) {
    RC(dalloc(g1, sizeof(double) * n1, s));
    RC(dalloc(g1s, sizeof(double) * n1, s));
    CU(launch_gam1(u.d, g1.as<double>(), g1s.as<double>(), s, 0, gam1_pairs_only));
    RC(back(GAM_1, g1, n1));
    RC(back(GAM_1s, g1s, n1));
  }
  return finish(s);
}

int neoxc_onebody_integrals(int64_t nebf, int64_t npebf, int64_t npbf,
                            int64_t nat, int64_t ngtg1, double pmass,
                            const double* cat, const double* zan,
                            const double* bcoef1, const double* gamma1,
                            const int64_t* AMPEB2C, const double* AGEBFCC,
                            const double* AGNBFCC, const double* ELCEX,
                            const double* NUCEX, const int64_t* ELCAM,
                            const int64_t* NUCAM, const double* ELCBFC,
                            const double* NUCBFC, double* Se, double* Sp,
                            double* GAM_ecore, double* GAM_pcore,
                            double* GAM_ep, double* GAM_1, double* GAM_1s) {
  return onebody_impl(nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1, gamma1,
                      AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                      Se, Sp, GAM_ecore, GAM_pcore, GAM_ep, GAM_1, GAM_1s, 0);
}

// rxchf/rxchf_gam_1_OMP.f:2-175 RXCHF_GAM1_OMP_MD
int neoxc_rxchf_gam1(int64_t nebf, int64_t npebf, int64_t npbf, int64_t ng1, int64_t ng1prm,
                     int64_t nat, int64_t ngtg1, double pmass, const double* cat,
                     const double* zan, const double* bcoef1, const double* gamma1,
                     const int64_t* AMPEB2C, const double* AGEBFCC, const double* AGNBFCC,
                     const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
                     const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC,
                     double* GAM_1, double* GAM_1s) {
  RC(need(ng1 == nebf * nebf * npbf * npbf && ng1prm == npebf * npebf * npbf * npbf,
          "ng1 == nebf**2 npbf**2, ng1prm == npebf**2 npbf**2"));
  RC(need(GAM_1 && GAM_1s, "GAM_1, GAM_1s"));
  return onebody_impl(nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1, gamma1,
                      AMPEB2C, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                      nullptr, nullptr, nullptr, nullptr, nullptr, GAM_1, GAM_1s, 1);
}

// ---- xchf1_independent/xchf1_fock.f:2-361 xchf1_fock ------------------------
// One stream, every term on the device in the reference's order: the one-body
// and GAM_1 terms (fock1 kernel, which also keeps the NEO-HF part), gam_2,
// gam_3, gam_4 in the branch `modes` selects (each adds its finished
// contraction to the Fock matrices once, as add2fock does), then S_total,
// E_total and XCfock_correction (assemble kernel).
int neoxc_xchf1_fock(int64_t modes, int64_t NG4CHK, int64_t NG3CHK,
                     int64_t NG2CHK, int64_t npebf, int64_t nebf, int64_t npbf,
                     int64_t nelec, int64_t ngee, int64_t ng1, int64_t ng2,
                     int64_t ng3, int64_t ng4, const double* DE,
                     const double* DP, const double* GAM_ecore,
                     const double* GAM_pcore, const double* GAM_ep,
                     const double* GAM_ee, const double* GAM_1,
                     const double* GAM_1s, const double* GM4ICR,
                     const double* GM3IC1, const double* GM2ICR,
                     const double* GM2SICR, const double* GAM_2s,
                     int64_t ng2prm, int64_t ngtg1, int64_t ng3prm,
                     int64_t nat, double pmass, const double* cat,
                     const double* zan, const double* bcoef1,
                     const double* gamma1, const int64_t* KPESTR,
                     const int64_t* KPEEND, const int64_t* AMPEB2C,
                     const double* AGEBFCC, const double* AGNBFCC,
                     const double* ELCEX, const double* NUCEX,
                     const int64_t* ELCAM, const int64_t* NUCAM,
                     const double* ELCBFC, const double* NUCBFC,
                     double* focke, double* fockp, double* Xfocke,
                     double* Xfockp, double* E_total, const double* E_nuc,
                     double* E_ecore, double* E_pcore, double* E_ep,
                     double* E_ee, double* E_gam1, double* E_gam2,
                     double* E_gam3, double* E_gam4, double* S_total,
                     double* S_gam1, double* S_gam2) {
  (void)AMPEB2C;
  RC(need((modes & ~(int64_t)(255 | NEOXC_FOCK_GAM4_FACTORED)) == 0, "modes"));
  RC(need(nebf >= 1 && npbf >= 1 && nelec >= 1, "nebf, npbf, nelec >= 1"));
  RC(need(nebf <= 4096 && npbf <= 4096, "nebf, npbf <= 4096"));
  const int64_t e2 = nebf * nebf, p2 = npbf * npbf, n4 = e2 * e2;
  RC(need(ng1 == e2 * p2, "ng1 == nebf**2 npbf**2"));
  RC(need(DE && DP && GAM_ecore && GAM_pcore && GAM_ep && E_nuc && focke &&
              fockp && Xfocke && Xfockp && E_total && E_ecore && E_pcore &&
              E_ep && E_ee && E_gam1 && E_gam2 && E_gam3 && E_gam4 &&
              S_total && S_gam1 && S_gam2,
          "pointers"));
  const bool neohf = (modes & NEOXC_FOCK_NEOHF) != 0;
  const bool t2 = !neohf && nelec > 1, t3 = !neohf && nelec > 2;
  const bool t4 = t3 && (modes & NEOXC_FOCK_GAM4);
  const bool d2 = t2 && (modes & NEOXC_FOCK_G2DSCF);
  const bool d3 = t3 && (modes & NEOXC_FOCK_G3DSCF);
  const bool d4 = t4 && (modes & NEOXC_FOCK_G4DSCF);
  if (nelec > 1) RC(need(GAM_ee && ngee == n4, "GAM_ee, ngee == nebf**4"));
  if (!neohf) RC(need(GAM_1 && GAM_1s, "GAM_1, GAM_1s"));
  if (t2) {
    RC(need(NG2CHK >= 1 && ng2 == n4 * p2, "NG2CHK >= 1, ng2 == nebf**4 npbf**2"));
    if (d2)
      RC(need(ng2prm == npebf * npebf * npebf * npebf * npbf * npbf, "ng2prm"));
    else
      RC(need(GM2ICR && GM2SICR, "GM2ICR, GM2SICR"));
  }
  if (t3) {
    RC(need(NG3CHK >= 1 && ng3 == n4 * e2 * p2, "NG3CHK >= 1, ng3 == nebf**6 npbf**2"));
    if (d3) {
      RC(need(ng3prm == npebf * npebf * npebf * npebf * npebf * npebf * npbf * npbf,
              "ng3prm"));
      if (nebf > 20) return set_err(NEOXC_ERR_UNSUPPORTED, "GAM3_DSCF: nebf <= 20");
    } else {
      RC(need(GM3IC1 != nullptr, "GM3IC1"));
    }
  }
  const bool fact4 = d4 && (modes & NEOXC_FOCK_GAM4_FACTORED);
  const double* g2s_host = GAM_2s ? GAM_2s : GM2SICR;
  if (t4) {
    RC(need(NG4CHK >= 1 && ng4 == n4 * n4 * p2, "NG4CHK >= 1, ng4 == nebf**8 npbf**2"));
    if (fact4) {
      if (nebf > kGam4FactMaxNE || npbf > 255)
        return set_err(NEOXC_ERR_UNSUPPORTED,
                       "factorised gam_4: nebf <= %d, npbf <= 255", kGam4FactMaxNE);
    } else if (nebf > kGam4MaxNE) {
      return set_err(NEOXC_ERR_UNSUPPORTED, "gam_4: nebf <= %d", kGam4MaxNE);
    }
    if (d4)
      RC(need(g2s_host && ng2 == n4 * p2, "GAM_2s (or GM2SICR), ng2 == nebf**4 npbf**2"));
    else
      RC(need(GM4ICR != nullptr, "GM4ICR"));
  }
  if (d2 || d3)
    RC(need(KPESTR && KPEEND && AGEBFCC && AGNBFCC && ELCEX && NUCEX && ELCAM &&
                NUCAM && ELCBFC && NUCBFC && bcoef1 && gamma1 &&
                (nat == 0 || (cat && zan)),
            "basis arrays"));
  cudaStream_t s;
  RC(get_stream(&s));
  const int ne = (int)nebf, np = (int)npbf;
  SysUpload u;
  if (d2 || d3)
    RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1,
                    gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                    NUCAM, ELCBFC, NUCBFC));
  DBuf dde, ddp, hce, hcp, gep, gee, g1, g1s, fe, fp, xfe, xfp, se1, sp1, se2, sp2,
      en, part, scr, g2, g2s, g3, g4;
  RC(upload(dde, DE, sizeof(double) * e2, s));
  RC(upload(ddp, DP, sizeof(double) * p2, s));
  RC(upload(hce, GAM_ecore, sizeof(double) * e2, s));
  RC(upload(hcp, GAM_pcore, sizeof(double) * p2, s));
  RC(upload(gep, GAM_ep, sizeof(double) * ng1, s));
  if (nelec > 1) RC(upload(gee, GAM_ee, sizeof(double) * n4, s));
  else RC(dalloc(gee, sizeof(double), s));
  if (!neohf) {
    RC(upload(g1, GAM_1, sizeof(double) * ng1, s));
    RC(upload(g1s, GAM_1s, sizeof(double) * ng1, s));
  } else {
    // the NEO-HF branch returns before E_from_GAM_1 (:222-235)
    RC(dalloc(g1, sizeof(double) * ng1, s));
    RC(dalloc(g1s, sizeof(double) * ng1, s));
    CU(cudaMemsetAsync(g1.p, 0, sizeof(double) * ng1, s));
    CU(cudaMemsetAsync(g1s.p, 0, sizeof(double) * ng1, s));
  }
  for (DBuf* b : {&fe, &xfe, &se1, &se2}) RC(dalloc(*b, sizeof(double) * e2, s));
  for (DBuf* b : {&fp, &xfp, &sp1, &sp2}) RC(dalloc(*b, sizeof(double) * p2, s));
  CU(cudaMemsetAsync(se2.p, 0, sizeof(double) * e2, s));
  CU(cudaMemsetAsync(sp2.p, 0, sizeof(double) * p2, s));
  RC(dalloc(en, sizeof(double) * kScfSlots, s));
  CU(cudaMemsetAsync(en.p, 0, sizeof(double) * kScfSlots, s));
  CU(cudaMemcpyAsync(en.as<double>() + 1, E_nuc, sizeof(double),
                     cudaMemcpyHostToDevice, s));
  RC(dalloc(part, sizeof(double) * scf_fock1_part_doubles(ne, np), s));
  size_t nscr = 1;
  if (t2 && !d2) nscr = std::max(nscr, eg2_partial_doubles(ne, np));
  if (t3 && !d3) nscr = std::max(nscr, eg3_partial_doubles(ne, np));
  if (t4)
    nscr = std::max(nscr, fact4 ? gam4f_scratch_doubles(ne, np)
                          : d4  ? gam4_partial_doubles(ne, np)
                                : eg4_partial_doubles(ne, np));
  RC(dalloc(scr, sizeof(double) * nscr, s));
  double* d_en = en.as<double>();
  CU(launch_scf_fock1(ne, np, (int)nelec, hce.as<double>(), hcp.as<double>(),
                      gep.as<double>(), g1.as<double>(), g1s.as<double>(),
                      gee.as<double>(), dde.as<double>(), ddp.as<double>(),
                      fe.as<double>(), fp.as<double>(), se1.as<double>(),
                      sp1.as<double>(), part.as<double>(), d_en, s,
                      xfe.as<double>(), xfp.as<double>()));
  if (t2) {
    if (d2) {
      RC(gam2_dscf_dev(u, s, dde.as<double>(), ddp.as<double>(), fe.as<double>(),
                       fp.as<double>(), se2.as<double>(), sp2.as<double>(),
                       d_en + 7, d_en + 12));
    } else {
      RC(upload(g2, GM2ICR, sizeof(double) * ng2, s));
      RC(upload(g2s, GM2SICR, sizeof(double) * ng2, s));
      CU(launch_eg2ic1(ne, np, dde.as<double>(), ddp.as<double>(), g2.as<double>(),
                       g2s.as<double>(), scr.as<double>(), fe.as<double>(),
                       se2.as<double>(), fp.as<double>(), sp2.as<double>(),
                       d_en + 7, d_en + 12, s));
    }
  }
  if (t3) {
    if (d3) {
      RC(gam3_dscf_dev(u, s, dde.as<double>(), ddp.as<double>(), fe.as<double>(),
                       fp.as<double>(), d_en + 8));
    } else {
      RC(upload(g3, GM3IC1, sizeof(double) * ng3, s));
      CU(launch_eg3ic1(ne, np, dde.as<double>(), ddp.as<double>(), g3.as<double>(),
                       scr.as<double>(), fe.as<double>(), fp.as<double>(),
                       d_en + 8, s));
    }
  }
  if (t4) {
    if (d4) {
      const double* d_g2s = g2s.as<double>();
      if (!(g2s.p && g2s_host == GM2SICR)) {
        RC(upload(g4, g2s_host, sizeof(double) * ng2, s));
        d_g2s = g4.as<double>();
      }
      if (fact4)
        CU(launch_gam4_factored(ne, np, gee.as<double>(), d_g2s, dde.as<double>(),
                                ddp.as<double>(), scr.as<double>(), fe.as<double>(),
                                fp.as<double>(), d_en + 9, 1, s));
      else
        CU(launch_gam4_dscf(ne, np, gee.as<double>(), d_g2s, dde.as<double>(),
                            ddp.as<double>(), scr.as<double>(), fe.as<double>(),
                            fp.as<double>(), d_en + 9, s));
    } else {
      RC(upload(g4, GM4ICR, sizeof(double) * ng4, s));
      CU(launch_eg4icr(ne, np, dde.as<double>(), ddp.as<double>(), g4.as<double>(),
                       scr.as<double>(), fe.as<double>(), fp.as<double>(), d_en + 9, s));
    }
  }
  if (!neohf)
    CU(launch_scf_assemble(ne, np, d_en, se1.as<double>(), sp1.as<double>(),
                           se2.as<double>(), sp2.as<double>(), fe.as<double>(),
                           fp.as<double>(), s));
  double h_en[kScfSlots];
  CU(cudaMemcpyAsync(focke, neohf ? xfe.p : fe.p, sizeof(double) * e2,
                     cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(fockp, neohf ? xfp.p : fp.p, sizeof(double) * p2,
                     cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(Xfocke, xfe.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(Xfockp, xfp.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h_en, d_en, sizeof(h_en), cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  *E_ecore = h_en[2];
  *E_pcore = h_en[3];
  *E_ep = h_en[4];
  *E_ee = h_en[5];
  if (neohf) {
    // :222-235: E_total = E_NEOHF, S_total = 1, the XC terms stay zero
    *E_total = h_en[2] + h_en[3] + h_en[4] + h_en[5] + *E_nuc;
    *S_total = 1.0;
    *E_gam1 = *E_gam2 = *E_gam3 = *E_gam4 = 0.0;
    *S_gam1 = *S_gam2 = 0.0;
    return NEOXC_OK;
  }
  *E_gam1 = h_en[6];
  *E_gam2 = h_en[7];
  *E_gam3 = h_en[8];
  *E_gam4 = h_en[9];
  *S_gam1 = h_en[11];
  *S_gam2 = h_en[12];
  *S_total = h_en[10];
  *E_total = h_en[0];
  return NEOXC_OK;
}

static int xchf_scf_on(cudaStream_t s, int64_t nelec, int64_t nucst, int64_t nebf, int64_t npebf,
                   int64_t npbf, int64_t nat, int64_t ngtg1, double pmass,
                   const double* cat, const double* zan, const double* bcoef1,
                   const double* gamma1, const int64_t* KPESTR,
                   const int64_t* KPEEND, const int64_t* AMPEB2C,
                   const double* AGEBFCC, const double* AGNBFCC,
                   const double* ELCEX, const double* NUCEX,
                   const int64_t* ELCAM, const int64_t* NUCAM,
                   const double* ELCBFC, const double* NUCBFC, int64_t options,
                   int64_t maxit, double* DE, double* DP, double* E_init,
                   double* E_final, double* history, int64_t* niter,
                   int64_t* converged, double* CE = nullptr,
                   double* CP = nullptr, double* EE = nullptr,
                   double* EP = nullptr) {
  (void)AMPEB2C;
  RC(need(nelec >= 1 && maxit >= 1, "nelec >= 1, maxit >= 1"));
  RC(need(nucst >= 1 && nucst <= npbf, "1 <= nucst <= npbf"));
  RC(need(DE && DP && E_init && E_final && niter && converged, "pointers"));
  RC(need((options & ~(int64_t)(NEOXC_SCF_GUESS_PROT | NEOXC_SCF_DIIS |
                                NEOXC_SCF_GAM4_ELEMENT | NEOXC_SCF_MIXED |
                                NEOXC_SCF_MIXED_GAM2 | NEOXC_SCF_GUESS_ELEC |
                                NEOXC_SCF_SCREEN | NEOXC_SCF_SOSCF)) == 0,
          "options"));
  const bool soscf = (options & NEOXC_SCF_SOSCF) != 0 && nelec > 1 && nelec / 2 < nebf;
  RC(need(!((options & NEOXC_SCF_SOSCF) && (options & NEOXC_SCF_DIIS)),
          "NEOXC_SCF_SOSCF and NEOXC_SCF_DIIS are exclusive"));
  const int mixed = (options & NEOXC_SCF_MIXED) ? 1 : 0;
  const int mixed_gam2 = (options & NEOXC_SCF_MIXED_GAM2) ? 1 : 0;
  if (nebf > kScfMaxN || npbf > kScfMaxN)
    return set_err(NEOXC_ERR_UNSUPPORTED, "XCHF SCF: nebf, npbf <= %d", kScfMaxN);
  const bool elem4 = (options & NEOXC_SCF_GAM4_ELEMENT) != 0;
  if (nelec > 2 && nebf > 20)
    return set_err(NEOXC_ERR_UNSUPPORTED, "XCHF SCF with gam_3: nebf <= 20");
  if (nelec > 2 && elem4 && nebf > kGam4MaxNE)
    return set_err(NEOXC_ERR_UNSUPPORTED, "element-wise gam_4: nebf <= %d", kGam4MaxNE);
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1,
                  gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM,
                  NUCAM, ELCBFC, NUCBFC));
  const int ne = (int)nebf, np = (int)npbf;
  const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np;
  const size_t ng1 = e2 * p2, ng2 = e2 * e2 * p2;
  const size_t ng3 = nelec > 2 ? e2 * e2 * e2 * p2 : 0;
  // integrals
  DBuf Se, Sp, Hce, Hcp, Gep, G1, G1s, Gee, G2, G2s, G3;
  RC(dalloc(Se, sizeof(double) * e2, s));
  RC(dalloc(Sp, sizeof(double) * p2, s));
  RC(dalloc(Hce, sizeof(double) * e2, s));
  RC(dalloc(Hcp, sizeof(double) * p2, s));
  RC(dalloc(Gep, sizeof(double) * ng1, s));
  RC(dalloc(G1, sizeof(double) * ng1, s));
  RC(dalloc(G1s, sizeof(double) * ng1, s));
  RC(dalloc(Gee, sizeof(double) * e2 * e2, s));
  RC(dalloc(G2, sizeof(double) * (nelec > 1 ? ng2 : 1), s));
  RC(dalloc(G2s, sizeof(double) * (nelec > 1 ? ng2 : 1), s));
  RC(dalloc(G3, sizeof(double) * (ng3 ? ng3 : 1), s));
  CU(launch_scf_onebody(u.d, Se.as<double>(), Sp.as<double>(), Hce.as<double>(),
                        Hcp.as<double>(), s));
  CU(launch_gam_ep(u.d, Gep.as<double>(), s));
  CU(launch_gam1(u.d, G1.as<double>(), G1s.as<double>(), s, 0));
  CU(launch_gam_ee(u.d, Gee.as<double>(), s));
  if (nelec > 1) {
    CU(launch_gam2_raw(u.d, 0, G2.as<double>(), G2s.as<double>(), s,
                       mixed_gam2));
    CU(launch_gam2_symmetrize(ne, np, 0, G2.as<double>(), G2s.as<double>(), s));
  }
  if (nelec > 2) {
    DBuf aux;
    RC(dalloc(aux, sizeof(double) * gam3_aux_doubles(ne, np), s));
    // GAM_ee and the core Hamiltonian (Hce, pack_2D order) are already built
    CU(launch_gam3_aux(u.d, aux.as<double>(), s, Gee.as<double>(), Hce.as<double>()));
    CU(launch_gam3_raw(u.d, aux.as<double>(), G3.as<double>(), s, mixed,
                       (options & NEOXC_SCF_SCREEN) ? kScreenThreshold : 0.0));
    CU(launch_gam3_symmetrize(ne, np, G3.as<double>(), s));
  }
  // SCF state
  DBuf dDE, dDP, DE0, DP0, fe, fp, se1, sp1, se2, sp2, Xe, Xp, en, part, scr, st;
  RC(upload(dDE, DE, sizeof(double) * e2, s));
  RC(dalloc(dDP, sizeof(double) * p2, s));
  RC(dalloc(DE0, sizeof(double) * e2, s));
  RC(dalloc(DP0, sizeof(double) * p2, s));
  for (DBuf* b : {&fe, &se1, &se2}) RC(dalloc(*b, sizeof(double) * e2, s));
  for (DBuf* b : {&fp, &sp1, &sp2}) RC(dalloc(*b, sizeof(double) * p2, s));
  RC(dalloc(Xe, sizeof(double) * e2, s));
  RC(dalloc(Xp, sizeof(double) * p2, s));
  RC(dalloc(en, sizeof(double) * kScfSlots, s));
  RC(dalloc(part, sizeof(double) * scf_fock1_part_doubles(ne, np), s));
  size_t nscr = 1;
  if (nelec > 1) nscr = std::max(nscr, eg2_partial_doubles(ne, np));
  if (nelec > 2) {
    nscr = std::max(nscr, eg3_partial_doubles(ne, np));
    nscr = std::max(nscr, elem4 ? gam4_partial_doubles(ne, np)
                                : gam4f_scratch_doubles(ne, np));
  }
  RC(dalloc(scr, sizeof(double) * nscr, s));
  RC(dalloc(st, sizeof(int) * 8, s));
  const bool diis = (options & NEOXC_SCF_DIIS) != 0;
  DBuf dwork;
  RC(dalloc(dwork, sizeof(double) * (diis ? diis_doubles(ne) : 1), s));
  if (diis) CU(cudaMemsetAsync(dwork.p, 0, sizeof(double) * diis_doubles(ne), s));
  CU(cudaMemsetAsync(DE0.p, 0, sizeof(double) * e2, s));
  CU(cudaMemsetAsync(DP0.p, 0, sizeof(double) * p2, s));
  CU(cudaMemsetAsync(se2.p, 0, sizeof(double) * e2, s));
  CU(cudaMemsetAsync(sp2.p, 0, sizeof(double) * p2, s));
  CU(cudaMemsetAsync(st.p, 0, sizeof(int) * 8, s));
  CU(cudaMemsetAsync(en.p, 0, sizeof(double) * kScfSlots, s));
  const double Enuc = nuc_rep(nat, zan, cat);
  CU(cudaMemcpyAsync(en.as<double>() + 1, &Enuc, sizeof(double),
                     cudaMemcpyHostToDevice, s));
  int* sts = st.as<int>();
  CU(launch_inv_sqrt(ne, Se.as<double>(), Xe.as<double>(), sts + 0, s));
  CU(launch_inv_sqrt(np, Sp.as<double>(), Xp.as<double>(), sts + 1, s));
  const int noccE = nelec > 1 ? (int)(nelec / 2) : 1;
  const double prefE = nelec > 1 ? 2.0 : 1.0;
  if (options & NEOXC_SCF_GUESS_ELEC)   // guess_elec (xcscf.f:660-670)
    CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), 0, noccE, prefE,
                      dDE.as<double>(), nullptr, nullptr, sts + 2, s));
  if (options & NEOXC_SCF_GUESS_PROT) {
    // guess_prot (xcscf.f:683-716): diagonalise the nuclear core Hamiltonian
    CU(launch_roothan(np, Hcp.as<double>(), Xp.as<double>(), (int)nucst - 1, 1,
                      1.0, dDP.as<double>(), nullptr, nullptr, sts + 3, s));
  } else {
    CU(cudaMemcpyAsync(dDP.p, DP, sizeof(double) * p2, cudaMemcpyHostToDevice, s));
  }
  double* d_en = en.as<double>();
  // final MOs and orbital energies (ROOTHAN's VECE/EE, VECP/EP) when asked,
  // and always for the second-order steps (they rotate VECE)
  const bool want_mo = CE || CP || EE || EP || soscf;
  DBuf dCE, dCP, dEE, dEP;
  DBuf sow, sost;
  if (soscf) {
    RC(dalloc(sow, sizeof(double) * soscf_doubles(ne, (int)(nelec / 2), (int)maxit), s));
    RC(dalloc(sost, sizeof(int) * 4, s));
    CU(cudaMemsetAsync(sost.p, 0, sizeof(int) * 4, s));
  }
  if (want_mo) {
    RC(dalloc(dCE, sizeof(double) * e2, s));
    RC(dalloc(dCP, sizeof(double) * p2, s));
    RC(dalloc(dEE, sizeof(double) * ne, s));
    RC(dalloc(dEP, sizeof(double) * np, s));
  }
  auto fock_build = [&]() -> int {
    CU(launch_scf_fock1(ne, np, (int)nelec, Hce.as<double>(), Hcp.as<double>(),
                        Gep.as<double>(), G1.as<double>(), G1s.as<double>(),
                        Gee.as<double>(), dDE.as<double>(), dDP.as<double>(),
                        fe.as<double>(), fp.as<double>(), se1.as<double>(),
                        sp1.as<double>(), part.as<double>(), d_en, s));
    if (nelec > 1)
      CU(launch_eg2ic1(ne, np, dDE.as<double>(), dDP.as<double>(), G2.as<double>(),
                       G2s.as<double>(), scr.as<double>(), fe.as<double>(),
                       se2.as<double>(), fp.as<double>(), sp2.as<double>(),
                       d_en + 7, d_en + 12, s));
    if (nelec > 2) {
      CU(launch_eg3ic1(ne, np, dDE.as<double>(), dDP.as<double>(), G3.as<double>(),
                       scr.as<double>(), fe.as<double>(), fp.as<double>(),
                       d_en + 8, s));
      if (elem4)
        CU(launch_gam4_dscf(ne, np, Gee.as<double>(), G2s.as<double>(),
                            dDE.as<double>(), dDP.as<double>(), scr.as<double>(),
                            fe.as<double>(), fp.as<double>(), d_en + 9, s));
      else
        CU(launch_gam4_factored(ne, np, Gee.as<double>(), G2s.as<double>(),
                                dDE.as<double>(), dDP.as<double>(),
                                scr.as<double>(), fe.as<double>(),
                                fp.as<double>(), d_en + 9, 1, s));
    }
    CU(launch_scf_assemble(ne, np, d_en, se1.as<double>(), sp1.as<double>(),
                           se2.as<double>(), sp2.as<double>(), fe.as<double>(),
                           fp.as<double>(), s));
    return NEOXC_OK;
  };
  const double tolE = 1.0e-6, tolP = 1.0e-4;   // xcscf.f TOLE, TOLP
  double Eold = 0.0;
  int64_t it = 0;
  bool done = false;
  for (it = 1; it <= maxit && !done; it++) {
    RC(fock_build());
    if (it == 1) {
      CU(cudaMemcpyAsync(E_init, d_en, sizeof(double) * kScfSlots,
                         cudaMemcpyDeviceToHost, s));
    }
    CU(launch_roothan(np, fp.as<double>(), Xp.as<double>(), (int)nucst - 1, 1, 1.0,
                      dDP.as<double>(), want_mo ? dEP.as<double>() : nullptr,
                      want_mo ? dCP.as<double>() : nullptr, sts + 1, s));
    RC(fock_build());
    if (diis)
      CU(launch_diis(ne, fe.as<double>(), dDE.as<double>(), Se.as<double>(),
                     dwork.as<double>(), sts + 4, nullptr, s));
    // second-order step (xcscf.f:459-485) from the second iteration on; when
    // it moves the orbitals, the diagonalisation below is skipped on the
    // device (state[1])
    if (soscf && it > 1)
      CU(launch_soscf(ne, noccE, fe.as<double>(), dCE.as<double>(), dEE.as<double>(), prefE,
                      dDE.as<double>(), sost.as<int>(), sow.as<double>(), (int)maxit, s));
    CU(launch_roothan(ne, fe.as<double>(), Xe.as<double>(), 0, noccE, prefE,
                      dDE.as<double>(), want_mo ? dEE.as<double>() : nullptr,
                      want_mo ? dCE.as<double>() : nullptr, sts + 0, s,
                      soscf ? sost.as<int>() + 1 : nullptr));
    CU(launch_dendif(ne, np, dDE.as<double>(), DE0.as<double>(), dDP.as<double>(),
                     DP0.as<double>(), d_en, s));
    double h[kScfSlots];
    int hs[4];
    CU(cudaMemcpyAsync(h, d_en, sizeof(h), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(hs, st.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
    RC(finish(s));
    for (int k = 0; k < 4; k++)
      if (hs[k] > 40)
        return set_err(hs[k] > 41 ? NEOXC_ERR_NUMERIC : NEOXC_ERR_CUDA,
                       "ROOTHAN: Jacobi eigensolver %s (status slot %d, iteration %lld)",
                       hs[k] > 41 ? "met a NaN" : "did not converge", k, (long long)it);
    if (!std::isfinite(h[0]))
      return set_err(NEOXC_ERR_NUMERIC, "XCHF SCF: non-finite total energy at iteration %lld",
                     (long long)it);
    if (history) {
      history[4 * (it - 1) + 0] = h[0];
      history[4 * (it - 1) + 1] = h[0] - Eold;
      history[4 * (it - 1) + 2] = h[14];
      history[4 * (it - 1) + 3] = h[15];
    }
    Eold = h[0];
    for (int k = 0; k < kScfSlots; k++) E_final[k] = h[k];
    done = npbf > 1 ? (h[14] < tolE && h[15] < tolP) : (h[14] < tolE);
    if (done) *niter = it;
  }
  if (!done) *niter = maxit;
  *converged = done ? 1 : 0;
  CU(cudaMemcpyAsync(DE, dDE.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(DP, dDP.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  if (CE) CU(cudaMemcpyAsync(CE, dCE.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  if (CP) CU(cudaMemcpyAsync(CP, dCP.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  if (EE) CU(cudaMemcpyAsync(EE, dEE.p, sizeof(double) * ne, cudaMemcpyDeviceToHost, s));
  if (EP) CU(cudaMemcpyAsync(EP, dEP.p, sizeof(double) * np, cudaMemcpyDeviceToHost, s));
  return finish(s);
}


int neoxc_xchf_scf(int64_t nelec, int64_t nucst, int64_t nebf, int64_t npebf,
                   int64_t npbf, int64_t nat, int64_t ngtg1, double pmass,
                   const double* cat, const double* zan, const double* bcoef1,
                   const double* gamma1, const int64_t* KPESTR,
                   const int64_t* KPEEND, const int64_t* AMPEB2C,
                   const double* AGEBFCC, const double* AGNBFCC,
                   const double* ELCEX, const double* NUCEX,
                   const int64_t* ELCAM, const int64_t* NUCAM,
                   const double* ELCBFC, const double* NUCBFC, int64_t options,
                   int64_t maxit, double* DE, double* DP, double* E_init,
                   double* E_final, double* history, int64_t* niter,
                   int64_t* converged) {
  cudaStream_t s;
  RC(get_stream(&s));
  return xchf_scf_on(s, nelec, nucst, nebf, npebf, npbf, nat, ngtg1, pmass, cat,
                     zan, bcoef1, gamma1, KPESTR, KPEEND, AMPEB2C, AGEBFCC,
                     AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC, NUCBFC,
                     options, maxit, DE, DP, E_init, E_final, history, niter,
                     converged);
}

int64_t neoxc_xchf_job_size(void) { return (int64_t)sizeof(neoxc_xchf_job); }

int neoxc_xchf_scf_job(neoxc_xchf_job* j, int64_t options, int64_t maxit) {
  RC(need(j != nullptr, "job"));
  cudaStream_t s;
  RC(get_stream(&s));
  j->status = xchf_scf_on(s, j->nelec, j->nucst, j->nebf, j->npebf, j->npbf, j->nat,
                          j->ngtg1, j->pmass, j->cat, j->zan, j->bcoef1, j->gamma1,
                          j->KPESTR, j->KPEEND, j->AMPEB2C, j->AGEBFCC, j->AGNBFCC,
                          j->ELCEX, j->NUCEX, j->ELCAM, j->NUCAM, j->ELCBFC,
                          j->NUCBFC, options, maxit, j->DE, j->DP, j->E_init,
                          j->E_final, j->history, &j->niter, &j->converged, j->CE,
                          j->CP, j->EE, j->EP);
  return j->status;
}

// Device bytes one solve holds at its peak (integral tensors, SCF state and
// contraction scratch), for admission against the memory budget.
static size_t xchf_job_bytes(const neoxc_xchf_job& j, int64_t options) {
  const size_t ne = (size_t)j.nebf, np = (size_t)j.npbf;
  const size_t e2 = ne * ne, p2 = np * np;
  size_t d = 4 * e2 + 4 * p2 + 3 * e2 * p2 + e2 * e2 + 32 * (e2 + p2);
  if (j.nelec > 1) d += 2 * e2 * e2 * p2 + eg2_partial_doubles((int)ne, (int)np);
  if (j.nelec > 2) {
    d += e2 * e2 * e2 * p2 + gam3_aux_doubles((int)ne, (int)np) +
         eg3_partial_doubles((int)ne, (int)np);
    d += (options & NEOXC_SCF_GAM4_ELEMENT) ? gam4_partial_doubles((int)ne, (int)np)
                                            : gam4f_scratch_doubles((int)ne, (int)np);
  }
  return sizeof(double) * d + (1u << 20);
}

int neoxc_admit(int64_t need_b, int64_t free_b, int64_t in_use, int64_t cap) {
  if (need_b < 0 || free_b < 0 || in_use < 0 || cap < 0) return NEOXC_ADMIT_REFUSE;
  double limit = 0.8 * ((double)free_b + (double)in_use);
  if (cap > 0 && (double)cap < limit) limit = (double)cap;
  if ((double)need_b > limit) return NEOXC_ADMIT_REFUSE;
  if ((double)in_use + (double)need_b <= limit && (double)need_b <= 0.9 * (double)free_b)
    return NEOXC_ADMIT_START;
  return NEOXC_ADMIT_WAIT;
}

int64_t neoxc_xchf_job_bytes(const neoxc_xchf_job* j, int64_t options) {
  if (!j || j->nebf < 1 || j->npbf < 1 || j->nebf > kScfMaxN || j->npbf > kScfMaxN) return -1;
  return (int64_t)xchf_job_bytes(*j, options);
}

// One admission decision for a job of need_b bytes: re-reads the device's
// free memory each time and waits (on cv, woken when a job ends, or every
// 50 ms) while neoxc_admit says wait.  Called with mu held by lk; returns
// NEOXC_ADMIT_START (in_use and running updated) or NEOXC_ADMIT_REFUSE.
static int admit_job(std::unique_lock<std::mutex>& lk, std::condition_variable& cv,
                     size_t need_b, size_t& in_use, int& running, int64_t cap) {
  for (;;) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
    const int d = neoxc_admit((int64_t)need_b, (int64_t)free_b, (int64_t)in_use, cap);
    if (d == NEOXC_ADMIT_REFUSE) return d;
    if (d == NEOXC_ADMIT_START) {
      in_use += need_b;
      running++;
      return d;
    }
    cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

// Independent XCHF solves (geometry or proton-position scans, many small
// molecules) on nworkers host threads, each with its own CUDA stream.  Jobs
// are taken in order as workers free up and admitted by neoxc_admit against
// the memory free at that moment; a job that can never fit is refused with
// NEOXC_ERR_NOMEM.  Every job gives the same result as a separate
// neoxc_xchf_scf call (same kernels, same order on its stream).
int neoxc_xchf_scf_batch(neoxc_xchf_job* jobs, int64_t njobs, int64_t nworkers,
                         int64_t options, int64_t maxit) {
  RC(need(jobs != nullptr && njobs >= 0 && nworkers >= 1, "jobs, njobs, nworkers"));
  if (njobs == 0) return NEOXC_OK;
  cudaStream_t s0;
  RC(get_stream(&s0));   // checks the device and fixes it for the workers
  int dev = 0;
  CU(cudaGetDevice(&dev));
  std::mutex mu;
  std::condition_variable cv;
  size_t in_use = 0;
  int running = 0;
  std::atomic<int64_t> next(0);
  const int nw = (int)std::min<int64_t>(nworkers, njobs);
  std::vector<std::thread> pool;
  for (int w = 0; w < nw; w++) {
    pool.emplace_back([&, w]() {
      (void)w;
      cudaSetDevice(dev);
      cudaStream_t st = nullptr;
      if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) st = nullptr;
      for (;;) {
        const int64_t k = next.fetch_add(1);
        if (k >= njobs) break;
        neoxc_xchf_job& j = jobs[k];
        if (!st) {
          j.status = NEOXC_ERR_CUDA;
          continue;
        }
        const size_t need_b = xchf_job_bytes(j, options);
        int decision;
        {
          std::unique_lock<std::mutex> lk(mu);
          decision = admit_job(lk, cv, need_b, in_use, running, 0);
        }
        if (decision == NEOXC_ADMIT_REFUSE) {
          j.status = NEOXC_ERR_NOMEM;
          continue;
        }
        j.status = xchf_scf_on(st, j.nelec, j.nucst, j.nebf, j.npebf, j.npbf, j.nat,
                               j.ngtg1, j.pmass, j.cat, j.zan, j.bcoef1, j.gamma1,
                               j.KPESTR, j.KPEEND, j.AMPEB2C, j.AGEBFCC, j.AGNBFCC,
                               j.ELCEX, j.NUCEX, j.ELCAM, j.NUCAM, j.ELCBFC,
                               j.NUCBFC, options, maxit, j.DE, j.DP, j.E_init,
                               j.E_final, j.history, &j.niter, &j.converged, j.CE,
                               j.CP, j.EE, j.EP);
        {
          std::lock_guard<std::mutex> lk(mu);
          in_use -= need_b;
          running--;
        }
        cv.notify_all();
      }
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
    });
  }
  for (auto& t : pool) t.join();
  for (int64_t k = 0; k < njobs; k++)
    if (jobs[k].status != NEOXC_OK)
      return set_err(jobs[k].status, "XCHF batch: job %lld failed (code %d)",
                     (long long)k, jobs[k].status);
  return NEOXC_OK;
}


// ---- serving loop --------------------------------------------------------------
}  // extern "C"

struct neoxc_xchf_server {
  int dev = 0;
  int64_t options = 0, maxit = 100;
  int64_t cap = 0;   // neoxc_xchf_server_set_budget (0 = none)
  size_t in_use = 0;
  int running = 0;
  bool stopping = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_mem;
  std::deque<neoxc_xchf_job*> queue;
  std::vector<std::thread> workers;
  std::chrono::steady_clock::time_point t0;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

// job completion marker: reserved = 1 once the worker has written the result
static void server_worker(neoxc_xchf_server* S) {
  cudaSetDevice(S->dev);
  cudaStream_t st = nullptr;
  const bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  for (;;) {
    neoxc_xchf_job* j = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stopping || !S->queue.empty(); });
      if (S->queue.empty()) break;   // stopping and drained
      j = S->queue.front();
      S->queue.pop_front();
    }
    const size_t need_b = xchf_job_bytes(*j, S->options);
    int decision;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      decision = admit_job(lk, S->cv_mem, need_b, S->in_use, S->running, S->cap);
      if (decision == NEOXC_ADMIT_REFUSE) {
        j->status = NEOXC_ERR_NOMEM;
        j->t_start = j->t_end = S->now();
        j->reserved = 1;
      }
    }
    if (decision == NEOXC_ADMIT_REFUSE) {
      S->cv_done.notify_all();
      continue;
    }
    j->t_start = S->now();
    j->status = ok ? xchf_scf_on(st, j->nelec, j->nucst, j->nebf, j->npebf, j->npbf,
                                 j->nat, j->ngtg1, j->pmass, j->cat, j->zan, j->bcoef1,
                                 j->gamma1, j->KPESTR, j->KPEEND, j->AMPEB2C,
                                 j->AGEBFCC, j->AGNBFCC, j->ELCEX, j->NUCEX, j->ELCAM,
                                 j->NUCAM, j->ELCBFC, j->NUCBFC, S->options, S->maxit,
                                 j->DE, j->DP, j->E_init, j->E_final, j->history,
                                 &j->niter, &j->converged, j->CE, j->CP, j->EE,
                                 j->EP)
                   : NEOXC_ERR_CUDA;
    j->t_end = S->now();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->in_use -= need_b;
      S->running--;
      j->reserved = 1;
    }
    S->cv_mem.notify_all();
    S->cv_done.notify_all();
  }
  if (ok) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
}

extern "C" {

neoxc_xchf_server* neoxc_xchf_server_start(int64_t nworkers, int64_t options,
                                           int64_t maxit) {
  if (nworkers < 1 || maxit < 1) {
    set_err(NEOXC_ERR_ARG, "server: nworkers >= 1, maxit >= 1");
    return nullptr;
  }
  cudaStream_t s0;
  if (get_stream(&s0) != NEOXC_OK) return nullptr;
  auto* S = new neoxc_xchf_server();
  cudaGetDevice(&S->dev);
  S->options = options;
  S->maxit = maxit;
  S->t0 = std::chrono::steady_clock::now();
  for (int64_t w = 0; w < nworkers; w++) S->workers.emplace_back(server_worker, S);
  return S;
}

int neoxc_xchf_server_set_budget(neoxc_xchf_server* S, int64_t cap_bytes) {
  RC(need(S != nullptr && cap_bytes >= 0, "server, cap_bytes >= 0"));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->cap = cap_bytes;
  }
  S->cv_mem.notify_all();
  return NEOXC_OK;
}

int neoxc_xchf_server_submit(neoxc_xchf_server* S, neoxc_xchf_job* job) {
  RC(need(S != nullptr && job != nullptr, "server, job"));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) return set_err(NEOXC_ERR_ARG, "server is stopping");
    job->reserved = 0;
    job->status = NEOXC_OK;
    job->t_submit = S->now();
    S->queue.push_back(job);
  }
  S->cv_work.notify_one();
  return NEOXC_OK;
}

int neoxc_xchf_server_wait(neoxc_xchf_server* S, neoxc_xchf_job* job,
                           double timeout_s) {
  RC(need(S != nullptr && job != nullptr, "server, job"));
  std::unique_lock<std::mutex> lk(S->mu);
  const bool done = S->cv_done.wait_for(
      lk, std::chrono::duration<double>(timeout_s), [&] { return job->reserved == 1; });
  if (!done) return set_err(NEOXC_ERR_TIMEOUT, "server wait: timeout after %g s", timeout_s);
  return job->status;
}

int neoxc_xchf_server_stop(neoxc_xchf_server* S) {
  RC(need(S != nullptr, "server"));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  delete S;
  return NEOXC_OK;
}

}  // extern "C"

// ---- open-shell XCUHF contractions (xcuhf/xcuhf_omg{1..4}.f) --------------
namespace {

// FAE_OMG2 (LAA, LAB), FAE_OMG3 (LAA, LAB, LBB), FAE_OMG4 (LAAA, LAAB,
// LBBA, LBBB) for the spin with na electrons (nb of the other spin).
unsigned fae_flags(int K, int64_t na, int64_t nb) {
  if (K == 2) return (na >= 2 ? 1u : 0u) | (na >= 1 && nb >= 1 ? 2u : 0u);
  if (K == 3)
    return (na >= 3 ? 1u : 0u) | (nb >= 1 && na >= 2 ? 2u : 0u) | (nb >= 2 ? 4u : 0u);
  return (na >= 4 ? 1u : 0u) | (na >= 3 && nb >= 1 ? 2u : 0u) |
         (nb >= 2 && na >= 2 ? 4u : 0u) | (nb >= 3 ? 8u : 0u);
}

// UFP_OMG2 (LAA, LAB), UFP_OMG3 (LAAA, LAAB, LBBA), UFP_OMG4 (L4A, L3A1B,
// L2A2B, L1A3B): the terms whose first electron has the spin with na.
unsigned ufp_flags(int K, int64_t na, int64_t nb) {
  if (K == 2) return (na >= 2 ? 1u : 0u) | (na >= 1 && nb >= 1 ? 2u : 0u);
  if (K == 3)
    return (na >= 3 ? 1u : 0u) | (na >= 2 && nb >= 1 ? 2u : 0u) |
           (nb >= 2 && na >= 1 ? 4u : 0u);
  return (na >= 4 ? 1u : 0u) | (na >= 3 && nb >= 1 ? 2u : 0u) |
         (na >= 2 && nb >= 2 ? 4u : 0u) | (na >= 1 && nb >= 3 ? 8u : 0u);
}

// One pass (two when the proton flags differ) over the rank-K tensor gives
// FAE_OMGk (alpha), FAE_OMGk with the spins exchanged (beta) and UFP_OMGk.
// Null outputs are skipped.  E[6] = {E_AE, E_BE, E_P, S_AE, S_BE, S_P}.
// Size limits of the rank-K contraction, checked before any array is read.
int spin_limits(int K, int64_t ne, int64_t np) {
  RC(need(ne >= 1 && ne <= 256 && np >= 1, "1 <= nebf <= 256, npbf >= 1"));
  RC(need(K >= 2 && K <= 4, "rank 2..4"));
  if (K > 2 && !spin_smem_fits(K, (int)ne))
    return set_err(NEOXC_ERR_UNSUPPORTED,
                   "rank-%d open-shell contraction: nebf <= %d (one bra's kets "
                   "are staged in shared memory)", K, K == 3 ? 28 : 12);
  return NEOXC_OK;
}

int xcuhf_dev(cudaStream_t s, int K, int64_t ne, int64_t np, int64_t NAE,
              int64_t NBE, const double* G, const double* Gs, const double* DAE,
              const double* DBE, const double* DP, double* FAE, double* FBE,
              double* FP, double* SAE, double* SBE, double* SP, double* E) {
  RC(spin_limits(K, ne, np));
  RC(need(K == 2 || !Gs, "overlap tensor only for rank 2"));
  RC(need(NAE >= 0 && NBE >= 0, "NAE, NBE >= 0"));
  RC(need(G && DAE && DBE && DP && E, "pointers"));
  const int64_t n2 = ne * ne, p2 = np * np;
  const bool want_a = FAE || SAE, want_b = FBE || SBE, want_p = FP || SP;
  const unsigned fa = want_a ? fae_flags(K, NAE, NBE) : 0u;
  const unsigned fb = want_b ? fae_flags(K, NBE, NAE) : 0u;
  const unsigned pa = ufp_flags(K, NAE, NBE), pb = ufp_flags(K, NBE, NAE);
  DBuf scr, fe, fp;
  RC(dalloc(scr, sizeof(double) * spin_scratch_doubles(K, (int)ne, (int)np), s));
  RC(dalloc(fe, sizeof(double) * 4 * n2, s));
  RC(dalloc(fp, sizeof(double) * 2 * p2, s));
  CU(cudaMemsetAsync(E, 0, sizeof(double) * 6, s));
  const double scale = (double)K;   // EFAC = 2, 3, 4
  double* x = fe.as<double>();
  if (want_a || want_b) {
    CU(launch_spin_omg(K, (int)ne, (int)np, G, Gs, DAE, DBE, DP, fa, fb,
                       scr.as<double>(), x, fp.as<double>(), s));
    if (want_a)
      CU(launch_spin_finish((int)ne, x, Gs ? x + 2 * n2 : nullptr, DAE, scale, FAE,
                            SAE, E + 0, E + 3, s));
    if (want_b)
      CU(launch_spin_finish((int)ne, x + n2, Gs ? x + 3 * n2 : nullptr, DBE, scale,
                            FBE, SBE, E + 1, E + 4, s));
  }
  if (want_p) {
    if (!(want_a && want_b && fa == pa && fb == pb))
      CU(launch_spin_omg(K, (int)ne, (int)np, G, Gs, DAE, DBE, DP, pa, pb,
                         scr.as<double>(), x, fp.as<double>(), s));
    CU(launch_spin_finish((int)np, fp.as<double>(), Gs ? fp.as<double>() + p2 : nullptr,
                          DP, 1.0, FP, SP, E + 2, E + 5, s));
  }
  return NEOXC_OK;
}

// Host wrapper of one reference routine: `proton` selects UFP_OMGk, else
// FAE_OMGk for the spin of DAE.  Fock accumulates; S, E, Es overwritten.
int xcuhf_host(int K, int64_t ne, int64_t np, int64_t NAE, int64_t NBE,
               int64_t ng, const double* G, const double* Gs, const double* DAE,
               const double* DBE, const double* DP, bool proton, double* F,
               double* S, double* E, double* Es) {
  RC(spin_limits(K, ne, np));
  RC(need(DAE && DBE && DP && G && F && E, "pointers"));
  RC(need(K == 2 ? (Gs && S && Es) : true, "GM2SICR, SAE2/SP2, S_*_OMG2"));
  cudaStream_t s;
  RC(get_stream(&s));
  const int64_t n2 = ne * ne, p2 = np * np, nf = proton ? p2 : n2;
  DBuf dg, dgs, da, db, dp, dF, dS, dE;
  RC(upload(dg, G, sizeof(double) * ng, s));
  if (Gs) RC(upload(dgs, Gs, sizeof(double) * ng, s));
  RC(upload(da, DAE, sizeof(double) * n2, s));
  RC(upload(db, DBE, sizeof(double) * n2, s));
  RC(upload(dp, DP, sizeof(double) * p2, s));
  RC(dalloc(dF, sizeof(double) * nf, s));
  RC(dalloc(dS, sizeof(double) * nf, s));
  RC(dalloc(dE, sizeof(double) * 6, s));
  CU(cudaMemsetAsync(dF.p, 0, sizeof(double) * nf, s));
  double* f = dF.as<double>();
  double* sv = Gs ? dS.as<double>() : nullptr;
  RC(xcuhf_dev(s, K, ne, np, NAE, NBE, dg.as<double>(), Gs ? dgs.as<double>() : nullptr,
               da.as<double>(), db.as<double>(), dp.as<double>(), proton ? nullptr : f,
               nullptr, proton ? f : nullptr, proton ? nullptr : sv, nullptr,
               proton ? sv : nullptr, dE.as<double>()));
  double e6[6];
  CU(cudaMemcpyAsync(e6, dE.p, sizeof e6, cudaMemcpyDeviceToHost, s));
  if (Gs) CU(cudaMemcpyAsync(S, dS.p, sizeof(double) * nf, cudaMemcpyDeviceToHost, s));
  RC(accumulate_back(F, f, nf, s));   // synchronises the stream
  *E = proton ? e6[2] : e6[0];
  if (Es) *Es = proton ? e6[5] : e6[3];
  return finish(s);
}

// FAE_OMG1 / UFP_OMG1: W = DAE (alpha Fock) or DETOT (proton Fock).
int omg1_host(int64_t ne, int64_t np, int64_t ng1, const double* W, const double* DP,
              const double* G1, const double* G1s, bool proton, double* F,
              double* S, double* E, double* Es) {
  RC(need(ng1 == ne * ne * np * np, "ng1 == nebf**2 npbf**2"));
  RC(need(W && DP && G1 && G1s && F && S && E && Es, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  const int64_t n2 = ne * ne, p2 = np * np, nf = proton ? p2 : n2;
  DBuf dg, dgs, dw, dp, fe, fpo, dF, dS, dE;
  RC(upload(dg, G1, sizeof(double) * ng1, s));
  RC(upload(dgs, G1s, sizeof(double) * ng1, s));
  RC(upload(dw, W, sizeof(double) * n2, s));
  RC(upload(dp, DP, sizeof(double) * p2, s));
  RC(dalloc(fe, sizeof(double) * 2 * n2, s));
  RC(dalloc(fpo, sizeof(double) * 2 * p2, s));
  RC(dalloc(dF, sizeof(double) * nf, s));
  RC(dalloc(dS, sizeof(double) * nf, s));
  RC(dalloc(dE, sizeof(double) * 2, s));
  CU(cudaMemsetAsync(dF.p, 0, sizeof(double) * nf, s));
  CU(launch_omg1((int)ne, (int)np, dg.as<double>(), dgs.as<double>(), dw.as<double>(),
                 dp.as<double>(), fe.as<double>(), fpo.as<double>(), s));
  if (proton)
    CU(launch_spin_finish((int)np, fpo.as<double>(), fpo.as<double>() + p2,
                          dp.as<double>(), 1.0, dF.as<double>(), dS.as<double>(),
                          dE.as<double>(), dE.as<double>() + 1, s));
  else
    CU(launch_spin_finish((int)ne, fe.as<double>(), fe.as<double>() + n2,
                          dw.as<double>(), 1.0, dF.as<double>(), dS.as<double>(),
                          dE.as<double>(), dE.as<double>() + 1, s));
  double e2[2];
  CU(cudaMemcpyAsync(e2, dE.p, sizeof e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(S, dS.p, sizeof(double) * nf, cudaMemcpyDeviceToHost, s));
  RC(accumulate_back(F, dF.as<double>(), nf, s));
  *E = e2[0];
  *Es = e2[1];
  return finish(s);
}

}  // namespace

extern "C" {

int neoxc_fae_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DAE,
                   const double* DP, const double* GAM_1, const double* GAM_1s,
                   double* FAE, double* SAE1, double* E_AE_OMG1, double* S_AE_OMG1) {
  return omg1_host(nebf, npbf, ng1, DAE, DP, GAM_1, GAM_1s, false, FAE, SAE1,
                   E_AE_OMG1, S_AE_OMG1);
}

int neoxc_ufp_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DETOT,
                   const double* DP, const double* GAM_1, const double* GAM_1s,
                   double* FP, double* SP1, double* E_P_OMG1, double* S_P_OMG1) {
  return omg1_host(nebf, npbf, ng1, DETOT, DP, GAM_1, GAM_1s, true, FP, SP1,
                   E_P_OMG1, S_P_OMG1);
}

int neoxc_fae_omg2(int64_t Nchunks, int64_t NAE, int64_t NBE, int64_t nebf,
                   int64_t npbf, int64_t ng2, const double* DAE, const double* DBE,
                   const double* DETOT, const double* DP, const double* GM2ICR,
                   const double* GM2SICR, double* FAE, double* SAE2,
                   double* E_AE_OMG2, double* S_AE_OMG2) {
  (void)DETOT;
  RC(need(Nchunks >= 1 && ng2 == nebf * nebf * nebf * nebf * npbf * npbf,
          "Nchunks >= 1, ng2 == nebf**4 npbf**2"));
  return xcuhf_host(2, nebf, npbf, NAE, NBE, ng2, GM2ICR, GM2SICR, DAE, DBE, DP,
                    false, FAE, SAE2, E_AE_OMG2, S_AE_OMG2);
}

int neoxc_ufp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DETOT, const double* DP, const double* GM2ICR,
                   const double* GM2SICR, double* FP, double* SP2, double* E_P_OMG2,
                   double* S_P_OMG2) {
  (void)DETOT;
  RC(need(Nchunks >= 1 && ng2 == nebf * nebf * nebf * nebf * npbf * npbf,
          "Nchunks >= 1, ng2 == nebf**4 npbf**2"));
  return xcuhf_host(2, nebf, npbf, NAE, NBE, ng2, GM2ICR, GM2SICR, DAE, DBE, DP,
                    true, FP, SP2, E_P_OMG2, S_P_OMG2);
}

int neoxc_fae_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM3ICR, double* FAE,
                   double* E_AE_OMG3) {
  const int64_t n3 = nebf * nebf * nebf;
  RC(need(Nchunks >= 1 && ng3 == n3 * n3 * npbf * npbf, "Nchunks >= 1, ng3 == nebf**6 npbf**2"));
  return xcuhf_host(3, nebf, npbf, NAE, NBE, ng3, GM3ICR, nullptr, DAE, DBE, DP, false,
                    FAE, nullptr, E_AE_OMG3, nullptr);
}

int neoxc_ufp_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM3ICR, double* FP,
                   double* E_P_OMG3) {
  const int64_t n3 = nebf * nebf * nebf;
  RC(need(Nchunks >= 1 && ng3 == n3 * n3 * npbf * npbf, "Nchunks >= 1, ng3 == nebf**6 npbf**2"));
  return xcuhf_host(3, nebf, npbf, NAE, NBE, ng3, GM3ICR, nullptr, DAE, DBE, DP, true,
                    FP, nullptr, E_P_OMG3, nullptr);
}

int neoxc_fae_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM4ICR, double* FAE,
                   double* E_AE_OMG4) {
  const int64_t n4 = nebf * nebf * nebf * nebf;
  RC(need(Nchunks >= 1 && ng4 == n4 * n4 * npbf * npbf, "Nchunks >= 1, ng4 == nebf**8 npbf**2"));
  return xcuhf_host(4, nebf, npbf, NAE, NBE, ng4, GM4ICR, nullptr, DAE, DBE, DP, false,
                    FAE, nullptr, E_AE_OMG4, nullptr);
}

int neoxc_ufp_omg4(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4,
                   int64_t NAE, int64_t NBE, const double* DAE, const double* DBE,
                   const double* DP, const double* GM4ICR, double* FP,
                   double* E_P_OMG4) {
  const int64_t n4 = nebf * nebf * nebf * nebf;
  RC(need(Nchunks >= 1 && ng4 == n4 * n4 * npbf * npbf, "Nchunks >= 1, ng4 == nebf**8 npbf**2"));
  return xcuhf_host(4, nebf, npbf, NAE, NBE, ng4, GM4ICR, nullptr, DAE, DBE, DP, true,
                    FP, nullptr, E_P_OMG4, nullptr);
}

int neoxc_dev_xcuhf_omg(void* stream, int64_t K, int64_t ne, int64_t np, int64_t NAE,
                        int64_t NBE, const double* d_G, const double* d_Gs,
                        const double* d_DAE, const double* d_DBE, const double* d_DP,
                        double* d_FAE, double* d_FBE, double* d_FP, double* d_SAE,
                        double* d_SBE, double* d_SP, double* d_E) {
  return xcuhf_dev((cudaStream_t)stream, (int)K, ne, np, NAE, NBE, d_G, d_Gs, d_DAE,
                   d_DBE, d_DP, d_FAE, d_FBE, d_FP, d_SAE, d_SBE, d_SP, d_E);
}

int neoxc_dev_omg4_icr(void* stream, int64_t ne, int64_t np, const double* d_gee,
                       const double* d_g2s, double* d_g4) {
  RC(need(ne >= 1 && np >= 1 && d_gee && d_g2s && d_g4, "sizes, pointers"));
  CU(launch_omg4_icr((int)ne, (int)np, d_gee, d_g2s, d_g4, (cudaStream_t)stream));
  return NEOXC_OK;
}

int neoxc_omg4_icr(int64_t Nchunks, int64_t ne, int64_t np, int64_t ngee, int64_t ng2,
                   int64_t ng4, const double* GAM_2s, const double* GAM_ee,
                   double* GAM_4) {
  RC(need(Nchunks >= 1, "Nchunks >= 1"));
  RC(need(ngee == ne * ne * ne * ne, "ngee == ne**4"));
  RC(need(ng2 == ngee * np * np, "ng2 == ne**4 np**2"));
  RC(need(ng4 == ngee * ngee * np * np, "ng4 == ne**8 np**2"));
  RC(need(GAM_2s && GAM_ee && GAM_4, "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  DBuf dg2, dee, d4;
  RC(upload(dg2, GAM_2s, sizeof(double) * ng2, s));
  RC(upload(dee, GAM_ee, sizeof(double) * ngee, s));
  RC(dalloc(d4, sizeof(double) * ng4, s));
  CU(launch_omg4_icr((int)ne, (int)np, dee.as<double>(), dg2.as<double>(),
                     d4.as<double>(), s));
  CU(cudaMemcpyAsync(GAM_4, d4.p, sizeof(double) * ng4, cudaMemcpyDeviceToHost, s));
  return finish(s);
}

}  // extern "C"

// ---- RXCHF-fe / RXCUHF-fe / RXCUHF-ae contractions (rxchf/, rxchfne/) -------
namespace {

// One reference routine on host arrays: tensors of ng elements, densities of
// ne x ne (P: np x np), outputs F0..F2 (ne x ne, or np x np for the proton
// routines) accumulated, energies E0 / E1 overwritten.
int rx_host(RxRoutine r, int K, bool proton, int nf, int nen, int64_t ne, int64_t np,
            int64_t ng, const double* T1, const double* T2, const double* Ts,
            const double* A, const double* Abet, const double* Atot, const double* B,
            const double* P, double* F0, double* F1, double* F2, double* E0,
            double* E1) {
  RC(need(ne >= 1 && np >= 1, "nebf, npbf >= 1"));
  int64_t want = np * np;
  for (int m = 0; m < 2 * K; m++) want *= ne;
  RC(need(ng == want, "tensor size == nebf**(2k) npbf**2"));
  RC(need(T1 && B && P && F0 && E0 && (nf < 2 || F1) && (nf < 3 || F2) && (nen < 2 || E1),
          "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  const int64_t n2 = ne * ne, p2 = np * np, nout = proton ? p2 : n2;
  DBuf d1, d2, ds, da, dab, dat, db, dp, scr, f0, f1, f2, dE;
  RC(upload(d1, T1, sizeof(double) * ng, s));
  if (T2) RC(upload(d2, T2, sizeof(double) * ng, s));
  if (Ts) RC(upload(ds, Ts, sizeof(double) * ng, s));
  if (A) RC(upload(da, A, sizeof(double) * n2, s));
  if (Abet) RC(upload(dab, Abet, sizeof(double) * n2, s));
  if (Atot) RC(upload(dat, Atot, sizeof(double) * n2, s));
  RC(upload(db, B, sizeof(double) * n2, s));
  RC(upload(dp, P, sizeof(double) * p2, s));
  RC(dalloc(scr, sizeof(double) * rx_scratch_doubles((int)ne, (int)np), s));
  RC(dalloc(f0, sizeof(double) * 3 * nout, s));
  RC(dalloc(dE, sizeof(double) * 2, s));
  CU(cudaMemsetAsync(f0.p, 0, sizeof(double) * 3 * nout, s));
  double* f = f0.as<double>();
  CU(launch_rx(r, (int)ne, (int)np, d1.as<double>(), T2 ? d2.as<double>() : nullptr,
               Ts ? ds.as<double>() : nullptr, A ? da.as<double>() : nullptr,
               Abet ? dab.as<double>() : nullptr, Atot ? dat.as<double>() : nullptr,
               db.as<double>(), dp.as<double>(), scr.as<double>(), f, f + nout,
               f + 2 * nout, dE.as<double>(), s));
  double e2[2];
  CU(cudaMemcpyAsync(e2, dE.p, sizeof e2, cudaMemcpyDeviceToHost, s));
  RC(accumulate_back(F0, f, nout, s));
  if (nf > 1) RC(accumulate_back(F1, f + nout, nout, s));
  if (nf > 2) RC(accumulate_back(F2, f + 2 * nout, nout, s));
  *E0 = e2[0];
  if (nen > 1) *E1 = e2[1];
  return finish(s);
}

}  // namespace

extern "C" {

// rxchfne/rxcuhfne_omg2.f:2-130 RXCUHFne_FE_OMG2
int neoxc_rxcuhfne_fe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                           const double* DAalpE, const double* DAbetE, const double* DAtotE,
                           const double* DBE, const double* DP, const double* GM2ICR,
                           const double* GM2exICR, double* FAalpE, double* FAbetE,
                           double* E_AE_OMG2) {
  (void)DAbetE;
  RC(need(Nchunks >= 1 && GM2exICR && DAalpE && DAtotE, "Nchunks, pointers"));
  return rx_host(RxRoutine::CuhfneFE2, 2, false, 2, 1, nebf, npbf, ng2, GM2ICR, GM2exICR,
                 nullptr, DAalpE, nullptr, DAtotE, DBE, DP, FAalpE, FAbetE, nullptr,
                 E_AE_OMG2, nullptr);
}
// rxcuhfne_omg2.f:239-345 RXCUHFne_FP_OMG2
int neoxc_rxcuhfne_fp_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                           int64_t NAalpE, int64_t NBE, const double* DAalpE,
                           const double* DAtotE, const double* DBE, const double* DP,
                           const double* GM2ICR, const double* GM2exICR, double* FP,
                           double* E_P_OMG2) {
  (void)NAalpE; (void)NBE;
  RC(need(Nchunks >= 1 && GM2exICR && DAalpE && DAtotE, "Nchunks, pointers"));
  return rx_host(RxRoutine::CuhfneFP2, 2, true, 1, 1, nebf, npbf, ng2, GM2ICR, GM2exICR,
                 nullptr, DAalpE, nullptr, DAtotE, DBE, DP, FP, nullptr, nullptr, E_P_OMG2,
                 nullptr);
}
// rxcuhfne_omg2.f:445-551 RXCUHFne_FBE_OMG2
int neoxc_rxcuhfne_fbe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                            int64_t NAalpE, int64_t NBE, const double* DAalpE,
                            const double* DAtotE, const double* DBE, const double* DP,
                            const double* GM2ICR, const double* GM2exICR, double* FBE,
                            double* E_BE_OMG2) {
  (void)NAalpE; (void)NBE;
  RC(need(Nchunks >= 1 && GM2exICR && DAalpE && DAtotE, "Nchunks, pointers"));
  return rx_host(RxRoutine::CuhfneFBE2, 2, false, 1, 1, nebf, npbf, ng2, GM2ICR, GM2exICR,
                 nullptr, DAalpE, nullptr, DAtotE, DBE, DP, FBE, nullptr, nullptr,
                 E_BE_OMG2, nullptr);
}

// rxchf/rxchf_omg2.f:2-114 RXCHF_FAE_OMG2, :231-334 RXCHF_FP_OMG2,
// :449-552 RXCHF_FBE_OMG2
#define RXCHF_OMG2(name, routine, proton)                                              \
  int name(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2, const double* DAE, \
           const double* DBE, const double* DP, const double* GM2_1ICR,                \
           const double* GM2_2ICR, const double* GM2sICR, double* F, double* S,        \
           double* E, double* Es) {                                                    \
    RC(need(Nchunks >= 1 && DAE && GM2_2ICR && GM2sICR, "Nchunks, pointers"));         \
    return rx_host(routine, 2, proton, 2, 2, nebf, npbf, ng2, GM2_1ICR, GM2_2ICR,      \
                   GM2sICR, DAE, nullptr, nullptr, DBE, DP, F, S, nullptr, E, Es);     \
  }
RXCHF_OMG2(neoxc_rxchf_fae_omg2, RxRoutine::FAE2, false)
RXCHF_OMG2(neoxc_rxchf_fp_omg2, RxRoutine::FP2, true)
RXCHF_OMG2(neoxc_rxchf_fbe_omg2, RxRoutine::FBE2, false)
#undef RXCHF_OMG2

// rxchf_omg3.f:2-105 RXCHF_FAE_OMG3, :263-366 RXCHF_FP_OMG3, :486-589 FBE
#define RXCHF_OMG3(name, routine, proton)                                              \
  int name(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3, const double* DAE, \
           const double* DBE, const double* DP, const double* GM3_1ICR,                \
           const double* GM3_2ICR, double* F, double* E) {                             \
    RC(need(Nchunks >= 1 && DAE && GM3_2ICR, "Nchunks, pointers"));                    \
    return rx_host(routine, 3, proton, 1, 1, nebf, npbf, ng3, GM3_1ICR, GM3_2ICR,      \
                   nullptr, DAE, nullptr, nullptr, DBE, DP, F, nullptr, nullptr, E,    \
                   nullptr);                                                           \
  }
RXCHF_OMG3(neoxc_rxchf_fae_omg3, RxRoutine::FAE3, false)
RXCHF_OMG3(neoxc_rxchf_fp_omg3, RxRoutine::FP3, true)
RXCHF_OMG3(neoxc_rxchf_fbe_omg3, RxRoutine::FBE3, false)
#undef RXCHF_OMG3

// rxchf_omg4.f:2-105 RXCHF_FAE_OMG4, :223-326 RXCHF_FP_OMG4, :444-547 FBE
#define RXCHF_OMG4(name, routine, proton)                                              \
  int name(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng4, const double* DAE, \
           const double* DBE, const double* DP, const double* GM4ICR, double* F,       \
           double* E) {                                                                \
    RC(need(Nchunks >= 1 && DAE, "Nchunks, pointers"));                                \
    return rx_host(routine, 4, proton, 1, 1, nebf, npbf, ng4, GM4ICR, nullptr, nullptr, \
                   DAE, nullptr, nullptr, DBE, DP, F, nullptr, nullptr, E, nullptr);   \
  }
RXCHF_OMG4(neoxc_rxchf_fae_omg4, RxRoutine::FAE4, false)
RXCHF_OMG4(neoxc_rxchf_fp_omg4, RxRoutine::FP4, true)
RXCHF_OMG4(neoxc_rxchf_fbe_omg4, RxRoutine::FBE4, false)
#undef RXCHF_OMG4

// rxchf/rxcuhf_omg2.f:2-126 RXCUHF_FE_OMG2
int neoxc_rxcuhf_fe_omg2(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2,
                         const double* DAalpE, const double* DAbetE, const double* DAtotE,
                         const double* DBE, const double* DP, const double* GM2_1ICR,
                         const double* GM2_2ICR, const double* GM2sICR, double* FAalpE,
                         double* FAbetE, double* SAalpE, double* E_AE_OMG2,
                         double* S_AE_OMG2) {
  (void)DAbetE;
  RC(need(Nchunks >= 1 && DAalpE && DAtotE && GM2_2ICR && GM2sICR, "Nchunks, pointers"));
  return rx_host(RxRoutine::CuFE2, 2, false, 3, 2, nebf, npbf, ng2, GM2_1ICR, GM2_2ICR,
                 GM2sICR, DAalpE, nullptr, DAtotE, DBE, DP, FAalpE, FAbetE, SAalpE,
                 E_AE_OMG2, S_AE_OMG2);
}
// rxcuhf_omg2.f:253-352 RXCUHF_FP_OMG2 and :469-576 RXCUHF_FBE_OMG2
#define RXCUHF_OMG2(name, routine, proton)                                             \
  int name(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng2, int64_t NAalpE,   \
           int64_t NBE, const double* DAalpE, const double* DAtotE, const double* DBE, \
           const double* DP, const double* GM2_1ICR, const double* GM2_2ICR,           \
           const double* GM2sICR, double* F, double* S, double* E, double* Es) {       \
    (void)NAalpE; (void)NBE;                                                           \
    RC(need(Nchunks >= 1 && DAalpE && DAtotE && GM2_2ICR && GM2sICR,                   \
            "Nchunks, pointers"));                                                     \
    return rx_host(routine, 2, proton, 2, 2, nebf, npbf, ng2, GM2_1ICR, GM2_2ICR,      \
                   GM2sICR, DAalpE, nullptr, DAtotE, DBE, DP, F, S, nullptr, E, Es);   \
  }
RXCUHF_OMG2(neoxc_rxcuhf_fp_omg2, RxRoutine::CuFP2, true)
RXCUHF_OMG2(neoxc_rxcuhf_fbe_omg2, RxRoutine::CuFBE2, false)
#undef RXCUHF_OMG2

// rxchf/rxcuhf_omg3.f:2-107 RXCUHF_FE_OMG3
int neoxc_rxcuhf_fe_omg3(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,
                         const double* DAalpE, const double* DAbetE, const double* DAtotE,
                         const double* DBE, const double* DP, const double* GM3_1ICR,
                         const double* GM3_2ICR, double* FAalpE, double* FAbetE,
                         double* E_AE_OMG3) {
  RC(need(Nchunks >= 1 && DAalpE && DAbetE && DAtotE && GM3_2ICR, "Nchunks, pointers"));
  return rx_host(RxRoutine::CuFE3, 3, false, 2, 1, nebf, npbf, ng3, GM3_1ICR, GM3_2ICR,
                 nullptr, DAalpE, DAbetE, DAtotE, DBE, DP, FAalpE, FAbetE, nullptr,
                 E_AE_OMG3, nullptr);
}
// rxcuhf_omg3.f:270-371 RXCUHF_FP_OMG3 and :499-600 RXCUHF_FBE_OMG3
#define RXCUHF_OMG3(name, routine, proton)                                             \
  int name(int64_t Nchunks, int64_t nebf, int64_t npbf, int64_t ng3,                   \
           const double* DAalpE, const double* DAbetE, const double* DAtotE,           \
           const double* DBE, const double* DP, const double* GM3_1ICR,                \
           const double* GM3_2ICR, double* F, double* E) {                             \
    RC(need(Nchunks >= 1 && DAalpE && DAbetE && DAtotE && GM3_2ICR,                    \
            "Nchunks, pointers"));                                                     \
    return rx_host(routine, 3, proton, 1, 1, nebf, npbf, ng3, GM3_1ICR, GM3_2ICR,      \
                   nullptr, DAalpE, DAbetE, DAtotE, DBE, DP, F, nullptr, nullptr, E,   \
                   nullptr);                                                           \
  }
RXCUHF_OMG3(neoxc_rxcuhf_fp_omg3, RxRoutine::CuFP3, true)
RXCUHF_OMG3(neoxc_rxcuhf_fbe_omg3, RxRoutine::CuFBE3, false)
#undef RXCUHF_OMG3

// rxchf/rxchf_omg1.f:2-82 RXCHF_FP_OMG1 (UFP_OMG1 with the special electron's
// density) and :84-165 RXCHF_FBE_OMG1 (FAE_OMG1 with DBE)
int neoxc_rxchf_fp_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DBE,
                        const double* DP, const double* GAM_1, const double* GAM_1s,
                        double* FP, double* SP, double* E_P_OMG1, double* S_P_OMG1) {
  return omg1_host(nebf, npbf, ng1, DBE, DP, GAM_1, GAM_1s, true, FP, SP, E_P_OMG1,
                   S_P_OMG1);
}
int neoxc_rxchf_fbe_omg1(int64_t nebf, int64_t npbf, int64_t ng1, const double* DBE,
                         const double* DP, const double* GAM_1, const double* GAM_1s,
                         double* FBE, double* SBE, double* E_BE_OMG1, double* S_BE_OMG1) {
  return omg1_host(nebf, npbf, ng1, DBE, DP, GAM_1, GAM_1s, false, FBE, SBE, E_BE_OMG1,
                   S_BE_OMG1);
}

}  // extern "C"

// ---- XCUHF SCF on the device (xcuhf/xcuhf_scf.f, Roothaan branch) ----------
namespace {

int xcuhf_scf_on(cudaStream_t s, int64_t nelec, int64_t NAE, int64_t NBE, int64_t nucst,
                 int64_t nebf, int64_t npebf, int64_t npbf, int64_t nat, int64_t ngtg1,
                 double pmass, const double* cat, const double* zan, const double* bcoef1,
                 const double* gamma1, const int64_t* KPESTR, const int64_t* KPEEND,
                 const double* AGEBFCC, const double* AGNBFCC, const double* ELCEX,
                 const double* NUCEX, const int64_t* ELCAM, const int64_t* NUCAM,
                 const double* ELCBFC, const double* NUCBFC, int64_t options,
                 int64_t maxit, double* DAE, double* DBE, double* DP, double* E_init,
                 double* E_final, double* history, int64_t* niter, int64_t* converged) {
  RC(need(nelec >= 1 && NAE >= 0 && NBE >= 0 && NAE + NBE == nelec,
          "nelec >= 1, NAE + NBE == nelec"));
  RC(need(maxit >= 1 && nucst >= 1 && nucst <= npbf, "maxit >= 1, 1 <= nucst <= npbf"));
  RC(need(NAE <= nebf && NBE <= nebf, "NAE, NBE <= nebf"));
  RC(need(DAE && DBE && DP && E_init && E_final && niter && converged, "pointers"));
  RC(need((options & ~(int64_t)(NEOXC_SCF_GUESS_PROT | NEOXC_SCF_GUESS_ELEC |
                                NEOXC_SCF_DIIS | NEOXC_SCF_MIXED |
                                NEOXC_SCF_MIXED_GAM2)) == 0,
          "options"));
  if (nebf > kScfMaxN || npbf > kScfMaxN)
    return set_err(NEOXC_ERR_UNSUPPORTED, "XCUHF SCF: nebf, npbf <= %d", kScfMaxN);
  if (nelec > 2 && nebf > 20)
    return set_err(NEOXC_ERR_UNSUPPORTED, "XCUHF SCF with gam_3: nebf <= 20");
  if (nelec > 3 && !spin_smem_fits(4, (int)nebf))
    return set_err(NEOXC_ERR_UNSUPPORTED, "XCUHF SCF with OMG4: nebf <= 12");
  const int mixed = (options & NEOXC_SCF_MIXED) ? 1 : 0;
  const int mixed_gam2 = (options & NEOXC_SCF_MIXED_GAM2) ? 1 : 0;
  const bool diis = (options & NEOXC_SCF_DIIS) != 0;
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1, gamma1,
                  KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC,
                  NUCBFC));
  const int ne = (int)nebf, np = (int)npbf;
  const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np;
  const size_t ng1 = e2 * p2, ng2 = e2 * e2 * p2;
  const size_t ng3 = nelec > 2 ? e2 * e2 * e2 * p2 : 0;
  const size_t ng4 = nelec > 3 ? e2 * e2 * e2 * e2 * p2 : 0;
  // integrals: as the XCHF SCF, plus the raw OMG4_ICR tensor
  DBuf Se, Sp, Hce, Hcp, Gep, G1, G1s, Gee, G2, G2s, G3, G4;
  RC(dalloc(Se, sizeof(double) * e2, s));
  RC(dalloc(Sp, sizeof(double) * p2, s));
  RC(dalloc(Hce, sizeof(double) * e2, s));
  RC(dalloc(Hcp, sizeof(double) * p2, s));
  RC(dalloc(Gep, sizeof(double) * ng1, s));
  RC(dalloc(G1, sizeof(double) * ng1, s));
  RC(dalloc(G1s, sizeof(double) * ng1, s));
  RC(dalloc(Gee, sizeof(double) * e2 * e2, s));
  RC(dalloc(G2, sizeof(double) * (nelec > 1 ? ng2 : 1), s));
  RC(dalloc(G2s, sizeof(double) * (nelec > 1 ? ng2 : 1), s));
  RC(dalloc(G3, sizeof(double) * (ng3 ? ng3 : 1), s));
  RC(dalloc(G4, sizeof(double) * (ng4 ? ng4 : 1), s));
  CU(launch_scf_onebody(u.d, Se.as<double>(), Sp.as<double>(), Hce.as<double>(),
                        Hcp.as<double>(), s));
  CU(launch_gam_ep(u.d, Gep.as<double>(), s));
  CU(launch_gam1(u.d, G1.as<double>(), G1s.as<double>(), s, 0));
  CU(launch_gam_ee(u.d, Gee.as<double>(), s));
  if (nelec > 1) {
    CU(launch_gam2_raw(u.d, 0, G2.as<double>(), G2s.as<double>(), s, mixed_gam2));
    CU(launch_gam2_symmetrize(ne, np, 0, G2.as<double>(), G2s.as<double>(), s));
  }
  if (nelec > 2) {
    DBuf aux;
    RC(dalloc(aux, sizeof(double) * gam3_aux_doubles(ne, np), s));
    CU(launch_gam3_aux(u.d, aux.as<double>(), s, Gee.as<double>(), Hce.as<double>()));
    CU(launch_gam3_raw(u.d, aux.as<double>(), G3.as<double>(), s, mixed,
                       (options & NEOXC_SCF_SCREEN) ? kScreenThreshold : 0.0));
    CU(launch_gam3_symmetrize(ne, np, G3.as<double>(), s));
  }
  if (nelec > 3)
    CU(launch_omg4_icr(ne, np, Gee.as<double>(), G2s.as<double>(), G4.as<double>(), s));
  // SCF state
  DBuf dA, dB, dP, A0, B0, P0, fa, fb, fp, sa1, sb1, sp1, sa2, sb2, sp2, Xe, Xp, en, part,
      e6, st, wa, wb;
  RC(upload(dA, DAE, sizeof(double) * e2, s));
  RC(upload(dB, DBE, sizeof(double) * e2, s));
  RC(dalloc(dP, sizeof(double) * p2, s));
  for (DBuf* b : {&A0, &B0, &fa, &fb, &sa1, &sb1, &sa2, &sb2, &Xe})
    RC(dalloc(*b, sizeof(double) * e2, s));
  for (DBuf* b : {&P0, &fp, &sp1, &sp2, &Xp}) RC(dalloc(*b, sizeof(double) * p2, s));
  RC(dalloc(en, sizeof(double) * kScfSlots, s));
  RC(dalloc(part, sizeof(double) * scf_fock1_part_doubles(ne, np), s));
  RC(dalloc(e6, sizeof(double) * 18, s));
  // status words: 0..7 eigensolver sweeps, 8..9 / 10..11 alpha / beta DIIS
  RC(dalloc(st, sizeof(int) * 16, s));
  RC(dalloc(wa, sizeof(double) * (diis ? diis_doubles(ne) : 1), s));
  RC(dalloc(wb, sizeof(double) * (diis ? diis_doubles(ne) : 1), s));
  if (diis) {
    CU(cudaMemsetAsync(wa.p, 0, sizeof(double) * diis_doubles(ne), s));
    CU(cudaMemsetAsync(wb.p, 0, sizeof(double) * diis_doubles(ne), s));
  }
  for (DBuf* b : {&A0, &B0, &sa2, &sb2}) CU(cudaMemsetAsync(b->p, 0, sizeof(double) * e2, s));
  for (DBuf* b : {&P0, &sp2}) CU(cudaMemsetAsync(b->p, 0, sizeof(double) * p2, s));
  CU(cudaMemsetAsync(st.p, 0, sizeof(int) * 16, s));
  CU(cudaMemsetAsync(en.p, 0, sizeof(double) * kScfSlots, s));
  const double Enuc = nuc_rep(nat, zan, cat);
  CU(cudaMemcpyAsync(en.as<double>() + 1, &Enuc, sizeof(double), cudaMemcpyHostToDevice, s));
  int* sts = st.as<int>();
  CU(launch_inv_sqrt(ne, Se.as<double>(), Xe.as<double>(), sts + 0, s));
  CU(launch_inv_sqrt(np, Sp.as<double>(), Xp.as<double>(), sts + 1, s));
  if (options & NEOXC_SCF_GUESS_ELEC) {
    // guess_A_elec (xcuhf_scf.f:585-609): lowest NAE / NBE core orbitals
    CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), 0, (int)NAE, 1.0,
                      dA.as<double>(), nullptr, nullptr, sts + 2, s));
    CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), 0, (int)NBE, 1.0,
                      dB.as<double>(), nullptr, nullptr, sts + 2, s));
  }
  if (options & NEOXC_SCF_GUESS_PROT) {
    // guess_prot2 (xcuhf_scf.f:611-640)
    CU(launch_roothan(np, Hcp.as<double>(), Xp.as<double>(), (int)nucst - 1, 1, 1.0,
                      dP.as<double>(), nullptr, nullptr, sts + 3, s));
  } else {
    CU(cudaMemcpyAsync(dP.p, DP, sizeof(double) * p2, cudaMemcpyHostToDevice, s));
  }
  double* d_en = en.as<double>();
  double* d_e6 = e6.as<double>();
  auto fock_build = [&]() -> int {
    CU(launch_uhf_fock1(ne, np, Hce.as<double>(), Hcp.as<double>(), Gep.as<double>(),
                        G1.as<double>(), G1s.as<double>(), Gee.as<double>(),
                        dA.as<double>(), dB.as<double>(), dP.as<double>(), fa.as<double>(),
                        fb.as<double>(), fp.as<double>(), sa1.as<double>(),
                        sb1.as<double>(), sp1.as<double>(), part.as<double>(), d_en, s));
    for (int k = 2; k <= 4 && k <= nelec; k++) {
      const double* G = k == 2 ? G2.as<double>() : (k == 3 ? G3.as<double>() : G4.as<double>());
      double* E = d_e6 + 6 * (k - 2);
      RC(xcuhf_dev(s, k, ne, np, NAE, NBE, G, k == 2 ? G2s.as<double>() : nullptr,
                   dA.as<double>(), dB.as<double>(), dP.as<double>(), fa.as<double>(),
                   fb.as<double>(), fp.as<double>(), k == 2 ? sa2.as<double>() : nullptr,
                   k == 2 ? sb2.as<double>() : nullptr, k == 2 ? sp2.as<double>() : nullptr,
                   E));
      // UHF_FOCK keeps the proton-side energies: E_P_OMGk (and S_P_OMG2)
      CU(cudaMemcpyAsync(d_en + 5 + k, E + 2, sizeof(double), cudaMemcpyDeviceToDevice, s));
      if (k == 2)
        CU(cudaMemcpyAsync(d_en + 12, E + 5, sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    CU(launch_uhf_assemble(ne, np, d_en, sa1.as<double>(), sb1.as<double>(),
                           sp1.as<double>(), sa2.as<double>(), sb2.as<double>(),
                           sp2.as<double>(), fa.as<double>(), fb.as<double>(),
                           fp.as<double>(), s));
    return NEOXC_OK;
  };
  const double tolE = 1.0e-6, tolP = 1.0e-4;   // xcuhf_scf.f TOLE, TOLP
  // DIIS joins once the spin densities move less than this per iteration:
  // extrapolating from the core-Hamiltonian guess onward diverges here.
  const double kDiisStart = 0.1;
  bool diis_on = false;
  double Eold = 0.0;
  int64_t it = 0;
  bool done = false;
  for (it = 1; it <= maxit && !done; it++) {
    RC(fock_build());
    if (it == 1)
      CU(cudaMemcpyAsync(E_init, d_en, sizeof(double) * kScfSlots, cudaMemcpyDeviceToHost,
                         s));
    // UROOTHAN for the proton, alpha and beta from the same Fock build
    CU(launch_roothan(np, fp.as<double>(), Xp.as<double>(), (int)nucst - 1, 1, 1.0,
                      dP.as<double>(), nullptr, nullptr, sts + 1, s));
    if (diis_on) {
      CU(launch_diis(ne, fa.as<double>(), dA.as<double>(), Se.as<double>(),
                     wa.as<double>(), sts + 8, nullptr, s));
      CU(launch_diis(ne, fb.as<double>(), dB.as<double>(), Se.as<double>(),
                     wb.as<double>(), sts + 10, nullptr, s));
    }
    CU(launch_roothan(ne, fa.as<double>(), Xe.as<double>(), 0, (int)NAE, 1.0,
                      dA.as<double>(), nullptr, nullptr, sts + 0, s));
    CU(launch_roothan(ne, fb.as<double>(), Xe.as<double>(), 0, (int)NBE, 1.0,
                      dB.as<double>(), nullptr, nullptr, sts + 6, s));
    CU(launch_uhf_dendif(ne, np, dA.as<double>(), A0.as<double>(), dB.as<double>(),
                         B0.as<double>(), dP.as<double>(), P0.as<double>(), d_en, s));
    double h[kScfSlots];
    int hs[8];
    CU(cudaMemcpyAsync(h, d_en, sizeof(h), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(hs, st.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
    RC(finish(s));
    for (int k : {0, 1, 2, 3, 6})
      if (hs[k] > 40)
        return set_err(NEOXC_ERR_CUDA, "UROOTHAN: Jacobi eigensolver did not converge");
    if (history) {
      history[4 * (it - 1) + 0] = h[0];
      history[4 * (it - 1) + 1] = h[0] - Eold;
      history[4 * (it - 1) + 2] = std::max(h[13], h[14]);
      history[4 * (it - 1) + 3] = h[15];
    }
    Eold = h[0];
    for (int k = 0; k < kScfSlots; k++) E_final[k] = h[k];
    if (diis && std::max(h[13], h[14]) < kDiisStart) diis_on = true;
    const bool de = h[13] < tolE && h[14] < tolE;
    done = npbf > 1 ? (de && h[15] < tolP) : de;
    if (done) *niter = it;
  }
  if (!done) *niter = maxit;
  *converged = done ? 1 : 0;
  CU(cudaMemcpyAsync(DAE, dA.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(DBE, dB.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(DP, dP.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  return finish(s);
}

}  // namespace

extern "C" int neoxc_xcuhf_scf(int64_t nelec, int64_t NAE, int64_t NBE, int64_t nucst,
                               int64_t nebf, int64_t npebf, int64_t npbf, int64_t nat,
                               int64_t ngtg1, double pmass, const double* cat,
                               const double* zan, const double* bcoef1,
                               const double* gamma1, const int64_t* KPESTR,
                               const int64_t* KPEEND, const int64_t* AMPEB2C,
                               const double* AGEBFCC, const double* AGNBFCC,
                               const double* ELCEX, const double* NUCEX,
                               const int64_t* ELCAM, const int64_t* NUCAM,
                               const double* ELCBFC, const double* NUCBFC,
                               int64_t options, int64_t maxit, double* DAE, double* DBE,
                               double* DP, double* E_init, double* E_final,
                               double* history, int64_t* niter, int64_t* converged) {
  (void)AMPEB2C;
  cudaStream_t s;
  RC(get_stream(&s));
  return xcuhf_scf_on(s, nelec, NAE, NBE, nucst, nebf, npebf, npbf, nat, ngtg1, pmass, cat,
                      zan, bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX,
                      ELCAM, NUCAM, ELCBFC, NUCBFC, options, maxit, DAE, DBE, DP, E_init,
                      E_final, history, niter, converged);
}

// ---- one-special-electron RXCHF SCF on the device ---------------------------
// rxchfne/rxchfne_scf.f xcrxchfne (closed-shell regular electrons) and
// rxchfne/rxcuhfne_scf.f xcrxcuhfne (open shell, EXCHLEV 0 or 1), LOCBSE2
// branch with UROOTHAN for the regular electrons.
namespace {

// One RXCHFne_FOCK / RXCUHFne_FOCK on device buffers: the regular
// electrons' one-body and GAMee terms, RXCHF_FP/FBE_OMG1 with the special
// electron's density, the OMG2 contractions (RXCHFne_* in one fused pass,
// or RXCUHFne_* with GM2exICR when exch), then the corrections and energy
// slots (launch_rx_assemble).  Scratch and partial matrices live in the
// struct; `en` holds E_nuc in slot 1 on entry.
struct RxFock {
  int ne = 0, np = 0, open = 0, exch = 0, with_ee = 0;
  const double *Hce = nullptr, *Gee = nullptr, *G1 = nullptr, *G1s = nullptr,
               *G2 = nullptr, *G2x = nullptr;
  DBuf dT, XFA1, XFB1, XFA2, XFB2, XFP, XSP, XFBE, XSBE, feo, fpo, part, scr, dumE;
  int alloc(cudaStream_t s) {
    const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np;
    for (DBuf* b : {&dT, &XFA1, &XFB1, &XFA2, &XFB2, &XFBE, &XSBE})
      RC(dalloc(*b, sizeof(double) * e2, s));
    for (DBuf* b : {&XFP, &XSP}) RC(dalloc(*b, sizeof(double) * p2, s));
    RC(dalloc(feo, sizeof(double) * 2 * e2, s));
    RC(dalloc(fpo, sizeof(double) * 2 * p2, s));
    RC(dalloc(part, sizeof(double) * rx_fock1_part_doubles(ne), s));
    RC(dalloc(scr, sizeof(double) * std::max(omg2_partial_doubles(ne, np),
                                             rx_scratch_doubles(ne, np)), s));
    RC(dalloc(dumE, sizeof(double) * 4, s));
    return NEOXC_OK;
  }
  // DA (closed: DAE; open: DAalpE), DB (open: DAbetE), DBE, DP in; FA, FB
  // (open), FP, FBE out; en[2..11] written, en[0] = E_total + en[1].
  int build(const double* DA, const double* DB, const double* DBE, const double* DP,
            double* FA, double* FB, double* FP, double* FBE, double* en, cudaStream_t s) {
    const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np;
    CU(launch_rx_fock1(ne, open, with_ee, Hce, Gee, DA, open ? DB : nullptr,
                       XFA1.as<double>(), open ? XFB1.as<double>() : nullptr,
                       open ? dT.as<double>() : nullptr, part.as<double>(), en, s));
    for (DBuf* b : {&XFA2, &XFB2, &XFBE}) CU(cudaMemsetAsync(b->p, 0, sizeof(double) * e2, s));
    CU(cudaMemsetAsync(XFP.p, 0, sizeof(double) * p2, s));
    // RXCHF_FP_OMG1 / RXCHF_FBE_OMG1 with the special electron's density
    CU(launch_omg1(ne, np, G1, G1s, DBE, DP, feo.as<double>(), fpo.as<double>(), s));
    CU(launch_spin_finish(np, fpo.as<double>(), fpo.as<double>() + p2, DP, 1.0,
                          XFP.as<double>(), XSP.as<double>(), en + 7, en + 9, s));
    CU(launch_spin_finish(ne, feo.as<double>(), feo.as<double>() + e2, DBE, 1.0,
                          XFBE.as<double>(), XSBE.as<double>(), en + 10, en + 11, s));
    const double* DT = open ? dT.as<double>() : nullptr;
    if (exch) {   // RXCUHFne_FE/FP/FBE_OMG2 (LADDEXCH)
      CU(launch_rx(RxRoutine::CuhfneFE2, ne, np, G2, G2x, nullptr, DA, nullptr, DT, DBE, DP,
                   scr.as<double>(), XFA2.as<double>(), XFB2.as<double>(), nullptr,
                   dumE.as<double>(), s));
      CU(launch_rx(RxRoutine::CuhfneFP2, ne, np, G2, G2x, nullptr, DA, nullptr, DT, DBE, DP,
                   scr.as<double>(), XFP.as<double>(), nullptr, nullptr, en + 8, s));
      CU(launch_rx(RxRoutine::CuhfneFBE2, ne, np, G2, G2x, nullptr, DA, nullptr, DT, DBE, DP,
                   scr.as<double>(), XFBE.as<double>(), nullptr, nullptr, dumE.as<double>(), s));
    } else {
      // RXCHFne_FAE/FP/FBE_OMG2 in one pass; the FAE part depends on DBE and
      // DP only, so the open-shell alpha and beta matrices are the same one
      CU(launch_rxchfne_omg2(ne, np, open ? DT : DA, DBE, DP, G2, scr.as<double>(),
                             XFA2.as<double>(), XFP.as<double>(), XFBE.as<double>(), en + 8,
                             s));
    }
    CU(launch_rx_assemble(ne, np, en, XFA1.as<double>(), XFA2.as<double>(),
                          open ? XFB1.as<double>() : nullptr,
                          open ? (exch ? XFB2.as<double>() : XFA2.as<double>()) : nullptr,
                          XFP.as<double>(), XSP.as<double>(), XFBE.as<double>(),
                          XSBE.as<double>(), FA, FB, FP, FBE, s));
    return NEOXC_OK;
  }
};

int rx_scf_on(cudaStream_t s, int64_t kind, int64_t NAE, int64_t NAalpE, int64_t NAbetE,
              int64_t nucst, int64_t nebf, int64_t npebf, int64_t npbf, int64_t nat,
              int64_t ngtg1, double pmass, const double* cat, const double* zan,
              const double* bcoef1, const double* gamma1, const int64_t* KPESTR,
              const int64_t* KPEEND, const double* AGEBFCC, const double* AGNBFCC,
              const double* ELCEX, const double* NUCEX, const int64_t* ELCAM,
              const int64_t* NUCAM, const double* ELCBFC, const double* NUCBFC,
              int64_t maxit, double* DA, double* DAbet, double* DBE, double* DP,
              double* E_init, double* E_final, double* history, int64_t* niter,
              int64_t* converged) {
  const bool ocbse = (kind & NEOXC_RX_NO_OCBSE) == 0;
  kind &= ~(int64_t)NEOXC_RX_NO_OCBSE;
  RC(need(kind == NEOXC_RX_NE || kind == NEOXC_RX_CU_NE || kind == NEOXC_RX_CU_AE, "kind"));
  const bool open = kind != NEOXC_RX_NE;
  if (open)
    RC(need(NAalpE >= 1 && NAbetE >= 0, "NAalpE >= 1, NAbetE >= 0"));
  else
    RC(need(NAE >= 1, "NAE >= 1"));
  RC(need(maxit >= 1 && nucst >= 1 && nucst <= npbf, "maxit >= 1, 1 <= nucst <= npbf"));
  RC(need(DA && DBE && DP && E_init && E_final && niter && converged && (!open || DAbet),
          "pointers"));
  if (nebf > kScfMaxN || npbf > kScfMaxN)
    return set_err(NEOXC_ERR_UNSUPPORTED, "RXCHF SCF: nebf, npbf <= %d", kScfMaxN);
  const int nocca = open ? (int)NAalpE : (NAE > 1 ? (int)(NAE / 2) : (int)NAE);
  const double prefA = (!open && NAE > 1) ? 2.0 : 1.0;
  const int nreg = open ? (int)(NAalpE + NAbetE) : (int)NAE;
  RC(need(nocca < nebf && (!open || NAbetE < nebf), "regular orbitals < nebf"));
  SysUpload u;
  RC(stage_system(u, s, nebf, npebf, npbf, nat, ngtg1, pmass, cat, zan, bcoef1, gamma1,
                  KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX, ELCAM, NUCAM, ELCBFC,
                  NUCBFC));
  const int ne = (int)nebf, np = (int)npbf;
  const size_t e2 = (size_t)ne * ne, p2 = (size_t)np * np, ng1 = e2 * p2, ng2 = e2 * e2 * p2;
  // integrals: Se, Sp, GAM_ecore/pcore, RXCHF GAM_1, GAM_ee, RXCHFne gam_2
  DBuf Se, Sp, Hce, Hcp, G1, G1s, Gee, G2, G2x, Xe, Xp;
  for (DBuf* b : {&Se, &Hce, &Xe}) RC(dalloc(*b, sizeof(double) * e2, s));
  for (DBuf* b : {&Sp, &Hcp, &Xp}) RC(dalloc(*b, sizeof(double) * p2, s));
  RC(dalloc(G1, sizeof(double) * ng1, s));
  RC(dalloc(G1s, sizeof(double) * ng1, s));
  RC(dalloc(Gee, sizeof(double) * e2 * e2, s));
  RC(dalloc(G2, sizeof(double) * ng2, s));
  RC(dalloc(G2x, sizeof(double) * ng2, s));
  CU(launch_scf_onebody(u.d, Se.as<double>(), Sp.as<double>(), Hce.as<double>(),
                        Hcp.as<double>(), s));
  CU(launch_gam1(u.d, G1.as<double>(), G1s.as<double>(), s, 0, 1));
  CU(launch_gam_ee(u.d, Gee.as<double>(), s));
  CU(launch_gam2_raw(u.d, 1, G2.as<double>(), G2x.as<double>(), s));
  CU(launch_gam2_symmetrize(ne, np, 1, G2.as<double>(), G2x.as<double>(), s));
  // SCF state
  DBuf dA, dB, dBE, dP, A0, B0, BE0, P0, CA, CBE, Ctmp, FA, FB, FP, FBE, ocb, en, info, st;
  for (DBuf* b : {&dA, &dB, &dBE, &A0, &B0, &BE0, &CA, &CBE, &Ctmp, &FA, &FB, &FBE})
    RC(dalloc(*b, sizeof(double) * e2, s));
  for (DBuf* b : {&dP, &P0, &FP}) RC(dalloc(*b, sizeof(double) * p2, s));
  RC(dalloc(ocb, sizeof(double) * ocbse_scratch_doubles(ne), s));
  RC(dalloc(en, sizeof(double) * kRxSlots, s));
  RC(dalloc(info, sizeof(double) * 4, s));
  RC(dalloc(st, sizeof(int) * 16, s));
  RxFock rf;
  rf.ne = ne;
  rf.np = np;
  rf.open = open ? 1 : 0;
  rf.exch = kind == NEOXC_RX_CU_AE ? 1 : 0;
  rf.with_ee = nreg > 1 ? 1 : 0;
  rf.Hce = Hce.as<double>();
  rf.Gee = Gee.as<double>();
  rf.G1 = G1.as<double>();
  rf.G1s = G1s.as<double>();
  rf.G2 = G2.as<double>();
  rf.G2x = G2x.as<double>();
  RC(rf.alloc(s));
  for (DBuf* b : {&A0, &B0, &BE0, &CBE, &dB})
    CU(cudaMemsetAsync(b->p, 0, sizeof(double) * e2, s));
  CU(cudaMemsetAsync(P0.p, 0, sizeof(double) * p2, s));
  CU(cudaMemsetAsync(en.p, 0, sizeof(double) * kRxSlots, s));
  CU(cudaMemsetAsync(st.p, 0, sizeof(int) * 16, s));
  const double Enuc = nuc_rep(nat, zan, cat);
  CU(cudaMemcpyAsync(en.as<double>() + 1, &Enuc, sizeof(double), cudaMemcpyHostToDevice, s));
  int* sts = st.as<int>();
  double* d_en = en.as<double>();
  CU(launch_inv_sqrt(ne, Se.as<double>(), Xe.as<double>(), sts + 0, s));
  CU(launch_inv_sqrt(np, Sp.as<double>(), Xp.as<double>(), sts + 1, s));
  // guesses: RXCHF_guess_elec / RXCUHF_guess_elec (one UROOTHAN of the
  // electronic core Hamiltonian: regular orbitals first, the special
  // electron in the next one), guess_prot2
  CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), 0, nocca, prefA, dA.as<double>(),
                    nullptr, CA.as<double>(), sts + 2, s));
  if (open && NAbetE > 0)
    CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), 0, (int)NAbetE, 1.0,
                      dB.as<double>(), nullptr, nullptr, sts + 3, s));
  // RXCHF_guess_B_elec (plain branch): the lowest core orbital
  CU(launch_roothan(ne, Hce.as<double>(), Xe.as<double>(), ocbse ? nocca : 0, 1, 1.0,
                    dBE.as<double>(), nullptr, Ctmp.as<double>(), sts + 4, s));
  CU(cudaMemcpyAsync(CBE.p, Ctmp.as<double>() + (size_t)ne * nocca, sizeof(double) * ne,
                     cudaMemcpyDeviceToDevice, s));
  CU(launch_roothan(np, Hcp.as<double>(), Xp.as<double>(), (int)nucst - 1, 1, 1.0,
                    dP.as<double>(), nullptr, nullptr, sts + 5, s));
  auto fock = [&]() -> int {
    return rf.build(dA.as<double>(), open ? dB.as<double>() : nullptr, dBE.as<double>(),
                    dP.as<double>(), FA.as<double>(), FB.as<double>(), FP.as<double>(),
                    FBE.as<double>(), d_en, s);
  };
  auto check_eig = [&](int n_status) -> int {
    int hs[16];
    CU(cudaMemcpyAsync(hs, st.p, sizeof(int) * n_status, cudaMemcpyDeviceToHost, s));
    RC(finish(s));
    for (int k = 0; k < n_status; k++)
      if (hs[k] > 40)
        return set_err(NEOXC_ERR_CUDA, "UROOTHAN: Jacobi eigensolver did not converge");
    return NEOXC_OK;
  };
  const double tolE = 1.0e-6, tolP = 1.0e-4;   // rxchfne_scf.f TOLE, TOLP
  const int maxmicro = 200;
  bool done = false;
  double h[kRxSlots];
  double* dBdiff = info.as<double>() + 2;
  for (int64_t it = 1; it <= maxit && !done; it++) {
    RC(fock());
    if (it == 1) {
      CU(cudaMemcpyAsync(E_init, d_en, sizeof(double) * kRxSlots, cudaMemcpyDeviceToHost, s));
      RC(finish(s));
    }
    CU(launch_roothan(np, FP.as<double>(), Xp.as<double>(), (int)nucst - 1, 1, 1.0,
                      dP.as<double>(), nullptr, nullptr, sts + 6, s));
    CU(launch_rx_dendif(np, dP.as<double>(), P0.as<double>(), d_en + 14, s));
    int micro = 0;
    double dreg = 0.0;
    for (micro = 1; micro <= maxmicro; micro++) {
      if (micro == 1 || !ocbse) RC(fock());
      CU(launch_roothan(ne, FA.as<double>(), Xe.as<double>(), 0, nocca, prefA, dA.as<double>(),
                        nullptr, CA.as<double>(), sts + 7, s));
      CU(launch_rx_dendif(ne, dA.as<double>(), A0.as<double>(), d_en + 12, s));
      if (open && NAbetE > 0) {
        CU(launch_roothan(ne, FB.as<double>(), Xe.as<double>(), 0, (int)NAbetE, 1.0,
                          dB.as<double>(), nullptr, nullptr, sts + 8, s));
        CU(launch_rx_dendif(ne, dB.as<double>(), B0.as<double>(), dBdiff, s));
      }
      // RXCHF_OCBSE2 / RXCUHF_OCBSE2 with the Fock matrix of the densities
      // before this micro-iteration's regular update
      if (ocbse)
        CU(launch_ocbse2(ne, nocca, CA.as<double>(), CBE.as<double>(), FBE.as<double>(),
                         Se.as<double>(), ocb.as<double>(), CBE.as<double>(),
                         dBE.as<double>(), info.as<double>(), sts + 9, s));
      else   // UROOTHAN of FBE, the lowest orbital (RXCHF_construct_DBE)
        CU(launch_roothan(ne, FBE.as<double>(), Xe.as<double>(), 0, 1, 1.0, dBE.as<double>(),
                          nullptr, nullptr, sts + 9, s));
      CU(launch_rx_dendif(ne, dBE.as<double>(), BE0.as<double>(), d_en + 13, s));
      if (ocbse) RC(fock());
      double hi[4];
      CU(cudaMemcpyAsync(h, d_en, sizeof(h), cudaMemcpyDeviceToHost, s));
      CU(cudaMemcpyAsync(hi, info.p, sizeof(hi), cudaMemcpyDeviceToHost, s));
      RC(check_eig(11));
      if (ocbse && !(hi[1] > 0.0))
        return set_err(NEOXC_ERR_CUDA, "OCBSE2: the projected special orbital vanished");
      dreg = (open && NAbetE > 0) ? std::max(h[12], hi[2]) : h[12];
      if (dreg < tolE && h[13] < tolE) break;
    }
    if (micro > maxmicro) micro = maxmicro;
    h[12] = dreg;
    h[15] = (double)micro;
    if (history) {
      history[3 * (it - 1) + 0] = h[0];
      history[3 * (it - 1) + 1] = (double)micro;
      history[3 * (it - 1) + 2] = h[14];
    }
    for (int k = 0; k < kRxSlots; k++) E_final[k] = h[k];
    *niter = it;
    done = h[14] < tolP;
  }
  *converged = done ? 1 : 0;
  CU(cudaMemcpyAsync(DA, dA.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  if (open) CU(cudaMemcpyAsync(DAbet, dB.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(DBE, dBE.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(DP, dP.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  return finish(s);
}

}  // namespace

extern "C" int neoxc_rx_scf(int64_t kind, int64_t NAE, int64_t NAalpE, int64_t NAbetE,
                            int64_t nucst, int64_t nebf, int64_t npebf, int64_t npbf,
                            int64_t nat, int64_t ngtg1, double pmass, const double* cat,
                            const double* zan, const double* bcoef1, const double* gamma1,
                            const int64_t* KPESTR, const int64_t* KPEEND,
                            const int64_t* AMPEB2C, const double* AGEBFCC,
                            const double* AGNBFCC, const double* ELCEX, const double* NUCEX,
                            const int64_t* ELCAM, const int64_t* NUCAM,
                            const double* ELCBFC, const double* NUCBFC, int64_t maxit,
                            double* DA, double* DAbet, double* DBE, double* DP,
                            double* E_init, double* E_final, double* history,
                            int64_t* niter, int64_t* converged) {
  (void)AMPEB2C;
  cudaStream_t s;
  RC(get_stream(&s));
  return rx_scf_on(s, kind, NAE, NAalpE, NAbetE, nucst, nebf, npebf, npbf, nat, ngtg1, pmass,
                   cat, zan, bcoef1, gamma1, KPESTR, KPEEND, AGEBFCC, AGNBFCC, ELCEX, NUCEX,
                   ELCAM, NUCAM, ELCBFC, NUCBFC, maxit, DA, DAbet, DBE, DP, E_init, E_final,
                   history, niter, converged);
}

// rxchfne/rxchfne_fock.f:2-250 RXCHFne_FOCK and rxchfne/rxcuhfne_fock.f
// RXCUHFne_FOCK from host arrays: one RxFock::build on uploaded copies.
extern "C" int neoxc_rxchfne_fock(int64_t open_shell, int64_t addexch, int64_t NAE,
                                  int64_t NAalpE, int64_t NAbetE, int64_t nebf,
                                  int64_t npbf, const double* DA, const double* DAbet,
                                  const double* DBE, const double* DP,
                                  const double* GAM_ecore, const double* GAM_ee,
                                  const double* GAM_1, const double* GAM_1s,
                                  const double* GM2ICR, const double* GM2exICR, double* FP,
                                  double* FA, double* FAbet, double* FBE, double* E_ecore,
                                  double* E_GAMee, double* E_OMG1, double* E_OMG2,
                                  double* E_total, double* S_total) {
  RC(need(nebf >= 1 && npbf >= 1 && nebf <= kScfMaxN && npbf <= kScfMaxN,
          "1 <= nebf, npbf <= 64"));
  RC(need(open_shell == 0 || open_shell == 1, "open_shell is 0 or 1"));
  RC(need(addexch == 0 || (open_shell == 1 && addexch == 1), "addexch only with open_shell"));
  const bool open = open_shell == 1;
  const int64_t nreg = open ? NAalpE + NAbetE : NAE;
  RC(need(nreg >= 1 && (!open || (NAalpE >= 0 && NAbetE >= 0)), "regular electron counts"));
  RC(need(DA && DBE && DP && GAM_ecore && GAM_1 && GAM_1s && GM2ICR && FP && FA && FBE &&
              E_ecore && E_GAMee && E_OMG1 && E_OMG2 && E_total && S_total &&
              (!open || (DAbet && FAbet)) && (!addexch || GM2exICR) && (nreg < 2 || GAM_ee),
          "pointers"));
  cudaStream_t s;
  RC(get_stream(&s));
  const size_t e2 = (size_t)nebf * nebf, p2 = (size_t)npbf * npbf;
  const size_t ng1 = e2 * p2, ng2 = e2 * e2 * p2;
  DBuf hce, gee, g1, g1s, g2, g2x, da, db, dbe, dp, fa, fb, fp, fbe, en;
  RC(upload(hce, GAM_ecore, sizeof(double) * e2, s));
  if (nreg > 1) RC(upload(gee, GAM_ee, sizeof(double) * e2 * e2, s));
  RC(upload(g1, GAM_1, sizeof(double) * ng1, s));
  RC(upload(g1s, GAM_1s, sizeof(double) * ng1, s));
  RC(upload(g2, GM2ICR, sizeof(double) * ng2, s));
  if (addexch) RC(upload(g2x, GM2exICR, sizeof(double) * ng2, s));
  RC(upload(da, DA, sizeof(double) * e2, s));
  if (open) RC(upload(db, DAbet, sizeof(double) * e2, s));
  RC(upload(dbe, DBE, sizeof(double) * e2, s));
  RC(upload(dp, DP, sizeof(double) * p2, s));
  for (DBuf* b : {&fa, &fb, &fbe}) RC(dalloc(*b, sizeof(double) * e2, s));
  RC(dalloc(fp, sizeof(double) * p2, s));
  RC(dalloc(en, sizeof(double) * kRxSlots, s));
  CU(cudaMemsetAsync(en.p, 0, sizeof(double) * kRxSlots, s));   // E_nuc = 0
  RxFock rf;
  rf.ne = (int)nebf;
  rf.np = (int)npbf;
  rf.open = open ? 1 : 0;
  rf.exch = addexch ? 1 : 0;
  rf.with_ee = nreg > 1 ? 1 : 0;
  rf.Hce = hce.as<double>();
  rf.Gee = gee.as<double>();
  rf.G1 = g1.as<double>();
  rf.G1s = g1s.as<double>();
  rf.G2 = g2.as<double>();
  rf.G2x = g2x.as<double>();
  RC(rf.alloc(s));
  RC(rf.build(da.as<double>(), db.as<double>(), dbe.as<double>(), dp.as<double>(),
              fa.as<double>(), fb.as<double>(), fp.as<double>(), fbe.as<double>(),
              en.as<double>(), s));
  double h[kRxSlots];
  CU(cudaMemcpyAsync(FA, fa.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  if (open) CU(cudaMemcpyAsync(FAbet, fb.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(FBE, fbe.p, sizeof(double) * e2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(FP, fp.p, sizeof(double) * p2, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(h, en.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  RC(finish(s));
  *E_ecore = h[2];
  *E_GAMee = h[3];
  *E_OMG1 = h[4];
  *E_OMG2 = h[5];
  *S_total = h[6];
  *E_total = h[0];
  return NEOXC_OK;
}
