/*
 * Gaussian-atom Radon oracle (test infrastructure only; see oracle_impl.h).
 * Builds the FP64 oracle (suffix _f64) and its FP32 twin (suffix _f32) from
 * one restatement of the reference's per-pixel kernels.
 */
#include <math.h>
#include <stdlib.h>

#define REAL double
#define SFX _f64
#define RX_EXP(v) exp(v)
#define RX_SQRT(v) sqrt(v)
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef RX_EXP
#undef RX_SQRT

#define REAL float
#define SFX _f32
#define RX_EXP(v) expf(v)
#define RX_SQRT(v) sqrtf(v)
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef RX_EXP
#undef RX_SQRT
