/*
 * msfem_fields.h -- C-ABI of libmsfem_fields.so: host generators of the
 * synthetic coefficient fields of the benchmark workloads.  No counterpart in
 * the reference (its coefficient is the analytic MatrixCoeff,
 * include/coefficients/matrix_coeff.tpp:66-91); the fields feed the
 * MSFEM_COEF_SPHERES kind of msfem_gpu.h.
 */
#ifndef MSFEM_FIELDS_H_
#define MSFEM_FIELDS_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random sequential addition of non-overlapping spheres (discs for dim = 2)
 * in the unit cube: radius U[rmin, rmax], centre U[0,1)^dim, both drawn from a
 * SplitMix64 stream seeded with `seed`; a sphere overlapping an accepted one
 * is rejected; stops when the summed volume reaches `fraction` or after
 * max_tries draws.  out[n][4] = (cx, cy, cz, r), cz = 0 in 2D.
 * Returns 0 with *n_out spheres written, 1 when capacity < *n_out (nothing
 * written; call again with a larger buffer), -1 on bad arguments. */
int msfem_spheres_rsa(uint64_t seed, double rmin, double rmax, double fraction, int32_t dim,
                      int64_t max_tries, double *out, int64_t capacity, int64_t *n_out);

#ifdef __cplusplus
}
#endif

#endif /* MSFEM_FIELDS_H_ */
