/*
 * fsoracle_wgsl.c -- instantiates the restatement of the reference GPU
 * algorithm in float (fsw_f32_*) and double (fsw_f64_*) arithmetic.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "fsoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define REAL float
#define SUF f32
#include "fsoracle_wgsl_impl.h"
#undef REAL
#undef SUF

#define REAL double
#define SUF f64
#include "fsoracle_wgsl_impl.h"
#undef REAL
#undef SUF
