/*
 * sph_oracle.c -- instantiates the CPU oracle (sph_oracle_impl.h) in FP32
 * and FP64.  Test infrastructure only: loaded by the tests, by smoke() to
 * check its results and by bench.py's CPU-baseline leg, never by the
 * product.
 *
 * Build: make -C oracle  (gcc -O2 -ffp-contract=off -fopenmp, no fast-math,
 * so every float operation is individually rounded as in the source).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "sph_oracle.h"

#define REAL float
#define SFX _f32
#define R_POW powf
#define R_SQRT sqrtf
#define R_ATAN atanf
#define R_COS cosf
#define R_SIN sinf
#define R_FABS fabsf
#include "sph_oracle_impl.h"
#undef REAL
#undef SFX
#undef R_POW
#undef R_SQRT
#undef R_ATAN
#undef R_COS
#undef R_SIN
#undef R_FABS

#define REAL double
#define SFX _f64
#define R_POW pow
#define R_SQRT sqrt
#define R_ATAN atan
#define R_COS cos
#define R_SIN sin
#define R_FABS fabs
#include "sph_oracle_impl.h"
