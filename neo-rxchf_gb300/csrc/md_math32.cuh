// md_math32.cuh -- FP32 McMurchie-Davidson geminal integrals (namespace
// neoxc::md32) for the mixed-precision builders: Gaussian products, Hermite
// tables, derivative tables, R_tuv recursions and the final contraction in
// FP32; the Boys function and the recursion seeds (-2 alpha)^j F_j(T) in
// FP64, narrowed to FP32 after the seed; callers accumulate the contracted
// sums in FP64.  The code is md_math_body.cuh with real = float.
#pragma once
#include <math.h>
#define MD_REAL float
#define MD_NS md32
#include "md_math_body.cuh"
#undef MD_REAL
#undef MD_NS
