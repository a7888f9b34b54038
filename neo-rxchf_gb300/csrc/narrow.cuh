// narrow.cuh -- FP64 -> FP32 narrowing by integer operations on the bit
// pattern, for the mixed-precision tensor-core path.  On this GPU an FP64
// conversion instruction costs as much as an FP64 FMA (FP64 runs at 1/64 of
// the FP32 rate), while these run on the integer pipes.  The significand is
// truncated to 23 bits (relative error below 2^-23, toward zero);
// magnitudes below the FP32 normal range become signed zero, above it
// infinity; NaN stays NaN.  Host-compilable so that the tests can check it.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define NX_NARROW_HD __host__ __device__ __forceinline__
#else
#define NX_NARROW_HD inline
#endif

namespace neoxc {
namespace tc {

NX_NARROW_HD float narrow_f64(double v) {
#if defined(__CUDA_ARCH__)
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
#else
  unsigned long long u;
  memcpy(&u, &v, sizeof(u));
#endif
  const unsigned top = (unsigned)(u >> 32);
  const unsigned sign = top & 0x80000000u;
  const int e = (int)((top >> 20) & 0x7ffu);
  const int ef = e - 1023 + 127;
  unsigned r;
  if (e == 0x7ff)
    r = sign | ((u & 0xfffffffffffffULL) ? 0x7fc00000u : 0x7f800000u);
  else if (ef <= 0)
    r = sign;
  else if (ef >= 255)
    r = sign | 0x7f800000u;
  else
    r = sign | ((unsigned)ef << 23) | (unsigned)((u >> 29) & 0x7fffffu);
#if defined(__CUDA_ARCH__)
  return __uint_as_float(r);
#else
  float f;
  memcpy(&f, &r, sizeof(f));
  return f;
#endif
}

}  // namespace tc
}  // namespace neoxc
