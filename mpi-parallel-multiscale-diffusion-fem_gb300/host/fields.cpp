// fields.cpp -- libmsfem_fields.so: host generators of the synthetic
// coefficient fields (include/msfem_fields.h).
//
// Random sequential addition of non-overlapping spheres: draw a radius and a
// centre from a SplitMix64 stream, accept the sphere when it overlaps no
// accepted one (uniform hash grid of cell width 2 r_max, so only the 3^d
// neighbouring grid cells are searched), until the summed volume reaches the
// target fraction.  The draws, the overlap test and the volume sum use the
// same operations in the same order as the Python restatement in
// workloads.py, so both give the same spheres bit for bit (this file is
// compiled with -ffp-contract=off: no fused multiply-adds).
#include <cmath>
#include <cstdint>
#include <vector>

#include "msfem_fields.h"

namespace {

struct SplitMix64 {
  uint64_t state;
  uint64_t next() {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

extern "C" int msfem_spheres_rsa(uint64_t seed, double rmin, double rmax, double fraction, int32_t dim,
                                 int64_t max_tries, double *out, int64_t capacity, int64_t *n_out) {
  if ((dim != 2 && dim != 3) || !(rmin > 0.0) || !(rmax >= rmin) || !(fraction >= 0.0) || !n_out ||
      (capacity > 0 && !out))
    return -1;
  SplitMix64 rng{seed};
  const double h = 2.0 * rmax;
  const int G = (int)std::ceil(1.0 / h);
  const int64_t ncell = (int64_t)G * G * (dim == 3 ? G : 1);
  std::vector<std::vector<int64_t>> grid((size_t)ncell);
  std::vector<double> sph;  // accepted spheres (cx, cy, cz, r)
  const double unit = dim == 3 ? (4.0 / 3.0) * M_PI : M_PI;
  double vol = 0.0;
  int64_t tries = 0;
  while (vol < fraction && tries < max_tries) {
    ++tries;
    const double r = rmin + (rmax - rmin) * rng.uniform();
    double c[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < dim; ++a) c[a] = rng.uniform();
    int gi[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a) gi[a] = std::min(G - 1, (int)(c[a] / h));
    bool ok = true;
    for (int k = (dim == 3 ? -1 : 0); k <= (dim == 3 ? 1 : 0) && ok; ++k)
      for (int j = -1; j <= 1 && ok; ++j)
        for (int i = -1; i <= 1 && ok; ++i) {
          const int x = gi[0] + i, y = gi[1] + j, z = gi[2] + k;
          if (x < 0 || y < 0 || z < 0 || x >= G || y >= G || z >= G) continue;
          for (int64_t s : grid[(size_t)(x + (int64_t)G * (y + (int64_t)G * z))]) {
            const double *o = &sph[4 * s];
            double d2 = 0.0;
            for (int a = 0; a < dim; ++a) d2 += (c[a] - o[a]) * (c[a] - o[a]);
            const double rs = r + o[3];
            if (d2 < rs * rs) {
              ok = false;
              break;
            }
          }
        }
    if (!ok) continue;
    const int64_t id = (int64_t)(sph.size() / 4);
    grid[(size_t)(gi[0] + (int64_t)G * (gi[1] + (int64_t)G * gi[2]))].push_back(id);
    sph.insert(sph.end(), {c[0], c[1], dim == 3 ? c[2] : 0.0, r});
    vol += unit * std::pow(r, (double)dim);
  }
  const int64_t n = (int64_t)(sph.size() / 4);
  *n_out = n;
  if (n > capacity) return 1;  // call again with capacity >= *n_out
  for (int64_t i = 0; i < 4 * n; ++i) out[i] = sph[(size_t)i];
  return 0;
}
