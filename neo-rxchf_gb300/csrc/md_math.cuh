// md_math.cuh -- FP64 McMurchie-Davidson geminal integrals (namespace
// neoxc::md), the precision of the reference's own arithmetic.  The code is in
// md_math_body.cuh, instantiated here with real = double.
#pragma once
#include <math.h>
#define MD_REAL double
#define MD_NS md
#include "md_math_body.cuh"
#undef MD_REAL
#undef MD_NS
