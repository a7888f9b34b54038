// md_math32.cuh -- FP32 McMurchie-Davidson geminal integrals (namespace
// neoxc::md32) for the mixed-precision builders: Gaussian products,
// Hermite tables, derivative tables and the Hermite folds in FP32; the Boys
// function, the seeds (-alpha)^m F_m(T) and the final Hermite-Coulomb sum
// in FP64; callers accumulate the contracted sums in FP64.  The code is
// md_math_body.cuh with real = float.
#pragma once
#include <math.h>
#define MD_REAL float
#define MD_NS md32
#include "md_math_body.cuh"
#undef MD_REAL
#undef MD_NS
