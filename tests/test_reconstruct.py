"""GPU reconstruction of the fine-scale solution, u = sum_i w_i phi_i per
cell (msfem_reconstruct; diffusion_problem_basis.tpp:352-377): against the
oracle's chain (direct-solve basis -> coarse solve of the reference problem
-> weighted sum) and against numpy on an uneven-N 3D batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reference_problem_fine_solution(pkg, oracle, engine):
    W = pkg.workloads
    prob = W.reference_problem(2, 3, 4)  # 8 x 8 coarse cells, N = 16
    got = engine.run(prob, tol=1e-12, want_basis=True)
    assert got["rc"] == 0
    ref = oracle.run(prob, want_basis=True)
    K, n = 8, 17
    u_c = oracle.coarse_solve(2, K, ref["M"], ref["F"], 0)
    w = np.array([[u_c[(c // K + (i >> 1)) * (K + 1) + c % K + (i & 1)] for i in range(4)]
                  for c in range(K * K)])
    u = engine.reconstruct(prob, got["basis"], w).reshape(K * K, n * n)
    u_ref = np.einsum("ci,cik->ck", w, ref["basis"].reshape(K * K, 4, n * n))
    assert np.abs(u - u_ref).max() < 1e-9 * np.abs(u_ref).max()
    # neighbouring cells agree on their shared edge (the fine solution is continuous)
    grid = u.reshape(K, K, n, n)  # [cy][cx][iy][ix]
    assert np.abs(grid[:, :-1, :, -1] - grid[:, 1:, :, 0]).max() < 1e-9 * np.abs(u_ref).max()


def test_uneven_3d_batch_matches_numpy(pkg, engine):
    W = pkg.workloads
    corners = W.unit_cube_corners(3, 4)[[0, 5, 21, 63]]
    nf = np.array([3, 6, 2, 5], dtype=np.int32)
    prob = W.problem(3, corners, nf, {"kind": 2, "params": [0.8, 0.25]})
    got = engine.run(prob, tol=1e-12, want_basis=True)
    assert got["rc"] == 0
    rng = np.random.default_rng(5)
    w = rng.normal(size=(4, 8))
    u = engine.reconstruct(prob, got["basis"], w)
    off = 0
    parts = []
    for c, N in enumerate(nf):
        nn = (N + 1) ** 3
        phi = got["basis"][off:off + 8 * nn].reshape(8, nn)
        parts.append(w[c] @ phi)
        off += 8 * nn
    ref = np.concatenate(parts)
    assert u.shape == ref.shape
    assert np.abs(u - ref).max() <= 1e-14 * np.abs(ref).max()
