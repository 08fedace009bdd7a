"""The host mirror's global Q1 system (host/global_q1.hpp: scatter, the
reference's Neumann and Dirichlet data, banded Cholesky) against the
oracle's coarse solve on the same element matrices and loads, on CPU: a
small harness compiled against the header reads M and F, assembles and
solves."""
import os
import subprocess

import numpy as np
import pytest

HARNESS = r'''
#include <cstdio>
#include <vector>
#include "global_q1.hpp"
using namespace DiffusionProblem;
template <int dim> int run(const char *in, const char *out, unsigned K, int bc) {
  constexpr unsigned nv = 1u << dim;
  size_t nc = 1;
  for (int a = 0; a < dim; ++a) nc *= K;
  std::vector<double> buf(nc * (nv * nv + nv));
  FILE *f = std::fopen(in, "rb");
  if (!f || std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) return 2;
  std::fclose(f);
  GlobalQ1System<dim> sys(K, bc);
  for (size_t c = 0; c < nc; ++c) {
    FullMatrix M(nv, nv);
    Vector F(nv);
    for (unsigned i = 0; i < nv; ++i) {
      for (unsigned j = 0; j < nv; ++j) M(i, j) = buf[c * nv * nv + i * nv + j];
      F(i) = buf[nc * nv * nv + c * nv + i];
    }
    sys.add_cell((unsigned)c, M, F);
  }
  const std::vector<double> u = sys.solve();
  FILE *g = std::fopen(out, "wb");
  std::fwrite(u.data(), sizeof(double), u.size(), g);
  std::fclose(g);
  return 0;
}
int main(int argc, char **argv) {
  const int dim = std::atoi(argv[3]);
  const unsigned K = (unsigned)std::atoi(argv[4]);
  const int bc = std::atoi(argv[5]);
  return dim == 2 ? run<2>(argv[1], argv[2], K, bc) : run<3>(argv[1], argv[2], K, bc);
}
'''


@pytest.fixture(scope="module")
def harness(pkg, tmp_path_factory):
    d = tmp_path_factory.mktemp("gq1")
    src = d / "h.cpp"
    src.write_text("#include <cstdlib>\n" + HARNESS)
    exe = d / "h"
    host = os.path.join(os.path.dirname(pkg.build.LIB_DIR), "host")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", host, "-I", pkg.build.INCLUDE, "-o", str(exe), str(src)],
                   check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("dim,n_refine,n_local,bc", [(2, 3, 2, 0), (2, 4, 0, 1), (3, 2, 1, 0), (3, 2, 0, 1)])
def test_banded_solve_equals_oracle(pkg, oracle, harness, tmp_path, dim, n_refine, n_local, bc):
    W = pkg.workloads
    r = oracle.run(W.reference_problem(dim, n_refine, n_local))
    K = 1 << n_refine
    inp, out = tmp_path / "mf.bin", tmp_path / "u.bin"
    np.concatenate([r["M"].ravel(), r["F"].ravel()]).astype(np.float64).tofile(inp)
    subprocess.run([str(harness), str(inp), str(out), str(dim), str(K), str(bc)], check=True)
    u = np.fromfile(out, dtype=np.float64)
    ref = oracle.coarse_solve(dim, K, r["M"], r["F"], bc)
    assert u.shape == ref.shape
    assert np.abs(u - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
