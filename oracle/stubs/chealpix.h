/* Declarations-only stand-in for chealpix.h so that the reference's source can
 * be compiled as a library for the oracle; the oracle passes ray angles in
 * directly and never calls these. Not part of the product. */
#pragma once
#include <stdint.h>
static inline void pix2ang_ring64(int64_t, int64_t, double* theta, double* phi) { *theta = 0.0; *phi = 0.0; }
static inline void write_healpix_map(const float*, long, const char*, char, const char*) {}
