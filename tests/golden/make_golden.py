"""Generate the golden fixtures of tests/golden/ from the CPU FP64 oracle
(banded-Cholesky direct solves, exact to rounding) on seeded workloads.

    python tests/golden/make_golden.py

Each fixture is an .npz holding the coarse element matrices M, loads F, a
few basis functions, the final coarse solution where the case is a whole
coarse problem, and fingerprints of the generated inputs (corners, Fourier
modes) so a test can tell a changed input generator from a changed solver.

Cases:
  sinsin_8x8       2D 8x8 coarse, N = 16, a = 1 + 0.9 sin(2 pi x/eps) sin(2 pi y/eps),
                   eps = 1/64, f = 1; coarse solve with homogeneous Dirichlet data
  reference_2d     the reference's own problem (MatrixCoeff with PI_D, f = 2,
                   Dirichlet ids 0/2, Neumann ids 1/3) at n_refine = 3,
                   n_refine_local = 4 (source/main.cxx), with the coarse solution
  reference_3d     the same in 3D at n_refine = 1, n_refine_local = 2
  fourier_cells    six cells of the random-Fourier tensor field
                   (64x64 coarse, N = 32, seeds 2/20/200)
  uneven_3d        five 3D cells with N in {1, 2, 3, 5, 4}, scalar sin-sin coefficient
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import __graft_entry__ as graft  # noqa: E402

BASIS_CELLS = 3  # basis functions stored for the first cells of each case


def fingerprint(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def cases(W):
    uneven = W.problem(3, W.unit_cube_corners(3, 2)[:5], np.array([1, 2, 3, 5, 4], dtype=np.int32),
                       {"kind": 2, "params": [0.5, 0.25]}, f_value=1.5)
    return {
        "sinsin_8x8": (W.sinsin_square(), (2, 8, 1)),
        "reference_2d": (W.reference_problem(2, 3, 4), (2, 8, 0)),
        "reference_3d": (W.reference_problem(3, 1, 2), (3, 2, 0)),
        "fourier_cells": (W.subset(W.fourier_square(K=64, N=32), [0, 1, 63, 64, 2080, 4095]), None),
        "uneven_3d": (uneven, None),
    }


def basis_prefix(prob, basis, ncells):
    dim = prob["dim"]
    nv = 1 << dim
    if "n_fine_per_cell" in prob:
        sizes = nv * (prob["n_fine_per_cell"].astype(np.int64) + 1) ** dim
    else:
        sizes = np.full(prob["corners"].shape[0], nv * (prob["n_fine"] + 1) ** dim, dtype=np.int64)
    return basis[:int(sizes[:ncells].sum())]


def main():
    pkg = graft.load_package()
    oracle = graft.load_oracle()
    oracle.build()
    W = pkg.workloads
    index = {}
    for name, (prob, coarse) in cases(W).items():
        ref = oracle.run(prob, want_basis=True)
        assert ref["nfail"] == 0
        out = {"M": ref["M"], "F": ref["F"], "basis_prefix": basis_prefix(prob, ref["basis"], BASIS_CELLS),
               "corners": prob["corners"]}
        meta = {"dim": prob["dim"], "n_cells": int(prob["corners"].shape[0]),
                "corners_sha256": fingerprint(prob["corners"]), "basis_cells": BASIS_CELLS}
        if "n_fine_per_cell" in prob:
            out["n_fine_per_cell"] = prob["n_fine_per_cell"]
        else:
            meta["n_fine"] = int(prob["n_fine"])
        if prob["coef"].get("modes") is not None:
            meta["modes_sha256"] = fingerprint(prob["coef"]["modes"])
        if coarse is not None:
            dim, K, bc = coarse
            out["u"] = oracle.coarse_solve(dim, K, ref["M"], ref["F"], bc)
            meta["coarse"] = {"K": K, "bc": bc}
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        index[name] = meta
        print(name, {k: v.shape for k, v in out.items()})
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
