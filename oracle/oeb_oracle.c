/*
 * oeb_oracle.c -- CPU oracle for the ten open-earth-benchmarks stencils (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference algorithm (kernels/*.h of monellz/open-earth-benchmarks),
 * built as liboeb_oracle.so by oracle/build.py with -O3 -fopenmp -ffp-contract=off.  Only the
 * tests, the smoke check and the CPU-baseline leg of bench.py use it, as the checker; the CUDA
 * library neither links nor calls it.
 *
 * Parity of this restatement is pinned two ways: bit-exact agreement with the reference
 * headers themselves, compiled from their own sources into oracle/_ref by oracle/build.py
 * (tests/test_oracle_vs_reference.py), and the golden vectors under tests/golden/, generated
 * from that reference build by tests/golden/make_golden.py.
 *
 * Each function takes the same descriptors, in the same order, as the reference signature
 * (scratch fields included), followed by the scalars and then the interior extents.
 */
#include <math.h>
#include <stdint.h>

#include "../include/oeb_gb300.h"

#define T double
#define SUF f64
#define M3 oeb_memref3d_f64
#define M1 oeb_memref1d_f64
#define SQRT sqrt
#include "oracle_impl.h"
#undef T
#undef SUF
#undef M3
#undef M1
#undef SQRT

#define T float
#define SUF f32
#define M3 oeb_memref3d_f32
#define M1 oeb_memref1d_f32
#define SQRT sqrtf
#include "oracle_impl.h"
#undef T
#undef SUF
#undef M3
#undef M1
#undef SQRT

/* Version tag so the test layer can detect a stale build. */
int oeb_oracle_version(void) { return 1; }
