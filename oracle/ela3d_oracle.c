/*
 * ela3d_oracle.c -- float32 and float64 instances of the CPU restatement.
 * TEST INFRASTRUCTURE ONLY (the oracle, never the product path).
 * Build: gcc -O2 -ffp-contract=off -shared -fPIC (see oracle/build.py).
 * The instances are named oracle_run_f32 / oracle_run_f64 and
 * oracle_profiles_f32 / oracle_profiles_f64 (FN() pastes the suffix).
 */
#include <math.h>
#include <stdlib.h>
#include "ela3d_oracle.h"

#define REAL float
#define SFX f32
#define POWR powf
#define EXPR expf
#define LOGR logf
#define SINR sinf
#define COSR cosf
#include "ela3d_oracle_impl.h"
#undef REAL
#undef SFX
#undef POWR
#undef EXPR
#undef LOGR
#undef SINR
#undef COSR

#define REAL double
#define SFX f64
#define POWR pow
#define EXPR exp
#define LOGR log
#define SINR sin
#define COSR cos
#include "ela3d_oracle_impl.h"
#undef REAL
#undef SFX
#undef POWR
#undef EXPR
#undef LOGR
#undef SINR
#undef COSR
