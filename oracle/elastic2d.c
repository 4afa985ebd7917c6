/*
 * Oracle for the 2D elastic path: the body in elastic2d_body.h compiled in
 * float (suffix _f, the reference precision) and double (suffix _d).
 *
 * TEST INFRASTRUCTURE ONLY: called by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg as the checker, never by the product.
 *
 * Build with -ffp-contract=off so that no multiply-add is fused (the
 * reference's Fortran and C were built on x86 without FMA contraction).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* stencil kinds shared by both precisions: P pairs (i+5,i-4)..(i+1,i),
   M pairs (i+4,i-5)..(i,i-1) */
enum { ST_P = 0, ST_M = 1 };

#define R float
#define R_IS_DOUBLE 0
#define FN(n) n##_f
#include "elastic2d_body.h"
#undef R
#undef R_IS_DOUBLE
#undef FN

#define R double
#define R_IS_DOUBLE 1
#define FN(n) n##_d
#include "elastic2d_body.h"
#undef R
#undef R_IS_DOUBLE
#undef FN
