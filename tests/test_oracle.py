"""CPU tests of the oracle: analytic known answers, invariants, solver
agreement and an independent numpy restatement of the reference algorithm
(diffusion_problem_basis.tpp:159-285) on small cells."""
import math

import numpy as np
import pytest

GP = (0.5 - 0.5 / math.sqrt(3.0), 0.5 + 0.5 / math.sqrt(3.0))


def q1_element_kat(H, a1, a2):
    """Coarse Q1 stiffness on an axis-aligned H x H square for A = diag(a1, a2):
    the multiscale basis equals the Q1 basis, so M = a1 Kx(x)My + a2 Mx(x)Ky."""
    K1 = np.array([[1.0, -1.0], [-1.0, 1.0]]) / H
    M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) * H / 6.0
    return a1 * np.kron(M1, K1) + a2 * np.kron(K1, M1)


def test_identity_coefficient_gives_q1_stiffness(pkg, oracle):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 8, {"kind": 0, "params": [1.0, 0.0, 1.0]})
    r = oracle.run(prob, want_basis=True)
    exact = np.array([[2, -.5, -.5, -1], [-.5, 2, -1, -.5], [-.5, -1, 2, -.5], [-1, -.5, -.5, 2]]) / 3
    assert np.abs(r["M"] - exact).max() < 1e-13
    assert np.allclose(r["F"], 0.25 ** 2 / 1.0 * 1.0, atol=1e-15)
    # basis = bilinear hat functions at the fine nodes
    n = 9
    x = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(x, x)  # row = y, col = x -> lexicographic x fastest when raveled
    hats = [(1 - X) * (1 - Y), X * (1 - Y), (1 - X) * Y, X * Y]
    b = r["basis"].reshape(4, 4, n * n)
    for i in range(4):
        assert np.abs(b[0, i] - hats[i].ravel()).max() < 1e-13


@pytest.mark.parametrize("a1,a2", [(3.0, 0.5), (1e-3, 1.0)])
def test_constant_diagonal_tensor_kat(pkg, oracle, a1, a2):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 4), 6, {"kind": 0, "params": [a1, 0.0, a2]})
    r = oracle.run(prob)
    assert np.abs(r["M"] - q1_element_kat(0.25, a1, a2)).max() < 1e-13 * max(a1, a2)


def test_constant_diagonal_tensor_kat_3d(pkg, oracle):
    W = pkg.workloads
    a = (2.0, 0.5, 1.5)
    prob = W.problem(3, W.unit_cube_corners(3, 2), 4,
                     {"kind": 0, "params": [a[0], 0, 0, a[1], 0, a[2]]}, f_value=3.0)
    r = oracle.run(prob)
    H = 0.5
    K1 = np.array([[1.0, -1.0], [-1.0, 1.0]]) / H
    M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) * H / 6.0
    exact = (a[0] * np.kron(M1, np.kron(M1, K1)) + a[1] * np.kron(M1, np.kron(K1, M1))
             + a[2] * np.kron(K1, np.kron(M1, M1)))
    assert np.abs(r["M"] - exact).max() < 1e-13
    assert np.allclose(r["F"], 3.0 * H ** 3 / 8, rtol=1e-13)


def test_invariants_reference_problem(pkg, oracle):
    """Partition of unity => zero row sums; symmetry; sum F = int_K f."""
    prob = pkg.workloads.reference_problem(2, 2, 3)
    r = oracle.run(prob)
    M, F = r["M"], r["F"]
    assert np.abs(M.sum(axis=2)).max() < 1e-12
    assert np.abs(M - M.transpose(0, 2, 1)).max() < 1e-12
    assert abs(F.sum() - 2.0) < 1e-12  # f = 2 on the unit square
    ev = np.linalg.eigvalsh(0.5 * (M + M.transpose(0, 2, 1)))
    assert ev.min() > -1e-12


def test_reference_algorithm_matches_direct(pkg, oracle):
    """SSOR(1.6)-CG to absolute 1e-12 (diffusion_problem_basis.tpp:293-317) and the
    Jacobi-PCG restatement agree with the banded Cholesky oracle."""
    prob = pkg.workloads.reference_problem(2, 2, 4)
    rd = oracle.run(prob, solver=oracle.SOLVER_DIRECT, want_basis=True)
    rs = oracle.run(prob, solver=oracle.SOLVER_SSOR_CG, tol=1e-12, tol_absolute=True,
                    ordering=oracle.ORDER_DEALII, want_basis=True)
    rj = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-13, want_basis=True)
    assert rs["nfail"] == 0 and rj["nfail"] == 0
    scale = np.abs(rd["M"]).max()
    assert np.abs(rs["M"] - rd["M"]).max() < 1e-10 * scale
    assert np.abs(rj["M"] - rd["M"]).max() < 1e-10 * scale
    assert np.abs(rs["basis"] - rd["basis"]).max() < 1e-9
    assert rs["iters"].max() < rj["iters"].max()  # SSOR needs fewer iterations
    assert rd["rel_res"].max() < 1e-12


def test_raw_monomials_agree_with_translated(pkg, oracle):
    """BasisQ1 as in basis_q1.tpp (raw monomials) vs the translated form."""
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 16), 4, {"kind": 1}, f_value=2.0)
    for cell in (0, 37, 255):
        x = prob["corners"][cell].mean(axis=0) + 0.01 / 16
        a = oracle.basis_q1(prob, cell, x, raw_monomials=True)
        b = oracle.basis_q1(prob, cell, x, raw_monomials=False)
        assert np.abs(a - b).max() < 1e-10
        assert abs(b.sum() - 1.0) < 1e-14


def numpy_cell(corners, N, coef_fn, f):
    """Independent restatement of one cell (dense algebra): returns M, F, basis."""
    n = N + 1
    nn = n * n

    def X(t):
        w = [(1 - t[0]) * (1 - t[1]), t[0] * (1 - t[1]), (1 - t[0]) * t[1], t[0] * t[1]]
        return sum(w[v] * corners[v] for v in range(4))

    A = np.zeros((nn, nn))
    b = np.zeros(nn)
    for cy in range(N):
        for cx in range(N):
            V = [X(((cx + (k & 1)) / N, (cy + (k >> 1)) / N)) for k in range(4)]
            nodes = [(cy + (k >> 1)) * n + cx + (k & 1) for k in range(4)]
            for qy in range(2):
                for qx in range(2):
                    xi = np.array([GP[qx], GP[qy]])
                    psi = np.array([(1 - xi[0]) * (1 - xi[1]), xi[0] * (1 - xi[1]),
                                    (1 - xi[0]) * xi[1], xi[0] * xi[1]])
                    dpsi = np.array([[-(1 - xi[1]), -(1 - xi[0])], [1 - xi[1], -xi[0]],
                                     [-xi[1], 1 - xi[0]], [xi[1], xi[0]]])
                    J = sum(np.outer(V[k], dpsi[k]) for k in range(4))
                    xq = sum(psi[k] * V[k] for k in range(4))
                    G = dpsi @ np.linalg.inv(J)
                    Aq = coef_fn(xq)
                    Ke = G @ Aq @ G.T * 0.25 * abs(np.linalg.det(J))
                    for i in range(4):
                        b[nodes[i]] += psi[i] * f * 0.25 * abs(np.linalg.det(J))
                        for j in range(4):
                            A[nodes[i], nodes[j]] += Ke[i, j]
    bnd = np.array([(k % n in (0, N)) or (k // n in (0, N)) for k in range(nn)])
    # Q1 interpolant of the corners in physical bilinear space
    P = np.array([[1, c[0], c[1], c[0] * c[1]] for c in corners])
    C = np.linalg.inv(P)
    phi = np.zeros((4, nn))
    for k in range(nn):
        x = X(((k % n) / N, (k // n) / N))
        m = np.array([1, x[0], x[1], x[0] * x[1]])
        if bnd[k]:
            phi[:, k] = m @ C
    I = ~bnd
    for i in range(4):
        rhs = -A[np.ix_(I, bnd)] @ phi[i, bnd]
        phi[i, I] = np.linalg.solve(A[np.ix_(I, I)], rhs)
    M = phi @ A @ phi.T
    F = phi @ b
    return M, F, phi


@pytest.mark.parametrize("geom", ["square", "parallelogram", "bilinear"])
def test_oracle_matches_numpy_restatement(pkg, oracle, geom):
    W = pkg.workloads
    base = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]]) * 0.3 + 0.1
    if geom == "parallelogram":
        base = base + np.array([[0, 0], [0, 0.05], [0.07, 0], [0.07, 0.05]])
    if geom == "bilinear":
        base = base + np.array([[0, 0], [0.04, 0.02], [-0.03, 0.05], [0.06, -0.04]])
    corners = base[None]
    coef = {"kind": 1}  # the reference MatrixCoeff
    prob = W.problem(2, corners, 5, coef, f_value=2.0)
    r = oracle.run(prob, want_basis=True)
    pid = 3.14592653509793218403
    al = pid / 3
    R = np.array([[math.cos(al), math.sin(al)], [-math.sin(al), math.cos(al)]])

    def coef_fn(x):
        c = 1.0 - 0.9999 * (0.5 * math.sin(2 * pid * 57 * x[0]) + 0.5 * math.sin(2 * pid * 57 * x[1]))
        return R @ (c * np.eye(2)) @ R.T

    M, F, phi = numpy_cell(base, 5, coef_fn, 2.0)
    assert np.abs(r["M"][0] - M).max() < 1e-11 * np.abs(M).max()
    assert np.abs(r["F"][0] - F).max() < 1e-13
    assert np.abs(r["basis"].reshape(4, -1) - phi).max() < 1e-11


def test_tabulated_equals_analytic(pkg, oracle):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 4,
                     W.fourier_coef((2, 20, 200), n_modes=8, kmax=16 * math.pi))
    tab = oracle.tabulate(prob, 3)
    tprob = dict(prob)
    tprob["coef"] = {"kind": 5, "ncomp": 3, "qp_values": tab}
    a = oracle.run(prob)
    b = oracle.run(tprob)
    assert np.abs(a["M"] - b["M"]).max() < 1e-14  # a12 vs a21 rounding of R D R^T


def test_coarse_solve_homogeneous_and_reference(pkg, oracle):
    """Coarse MsFEM problem with a = I reduces to standard Q1 FEM."""
    W = pkg.workloads
    K = 4
    prob = W.problem(2, W.unit_cube_corners(2, K), 4, {"kind": 0, "params": [1.0, 0.0, 1.0]})
    r = oracle.run(prob)
    u = oracle.coarse_solve(2, K, r["M"], r["F"], 1)
    assert u.shape == ((K + 1) ** 2,)
    assert np.all(u >= -1e-14) and u.max() > 0  # f = 1 > 0, zero BC
    u0 = oracle.coarse_solve(2, K, r["M"], r["F"], 0)
    x = np.linspace(0, 1, K + 1)
    Xg, Yg = np.meshgrid(x, x)
    dbc = ((Xg - 0.5) ** 2 + (Yg - 0.5) ** 2).ravel()
    on_dir = ((Xg == 0) | (Yg == 0)).ravel()
    assert np.abs(u0[on_dir] - dbc[on_dir]).max() < 1e-15


def test_tabulated_rhs_constant_equals_f_value(pkg, oracle):
    """f tabulated at the Gauss points (RightHandSide::value_list) with a
    constant value gives the constant-f load, on a bilinear cell too."""
    W = pkg.workloads
    corners = W.unit_cube_corners(2, 2).copy()
    corners[3, 3] += [0.05, -0.03]  # a general (non-parallelogram) cell
    prob = W.problem(2, corners, 6, {"kind": 2, "params": [0.5, 0.25]}, f_value=2.0)
    tab = W.with_rhs(prob, lambda x: np.full(x.shape[:-1], 2.0))
    a = oracle.run(prob)
    b = oracle.run(tab)
    assert np.abs(a["F"] - b["F"]).max() <= 1e-15 * np.abs(a["F"]).max() * 10
    assert np.array_equal(a["M"], b["M"])


@pytest.mark.parametrize("dim", [2, 3])
def test_tabulated_rhs_integrates_linear_f_exactly(pkg, oracle, dim):
    """sum_i F_i = int_K f (the basis is a partition of unity and QGauss(2)
    integrates a linear f exactly on affine cells), on uneven N."""
    W = pkg.workloads
    K = 2
    corners = W.unit_cube_corners(dim, K)
    nf = np.array([3, 4, 2, 5, 4, 3, 2, 3][:K ** dim], dtype=np.int32)
    prob = W.problem(dim, corners, nf, {"kind": 2, "params": [0.7, 0.5]})
    w = np.array([1.0, 2.0, 3.0][:dim])
    prob = W.with_rhs(prob, lambda x: 1.0 + x @ w)
    r = oracle.run(prob, tol=1e-13)
    centers = corners.mean(axis=1)
    exact = (1.0 / K) ** dim * (1.0 + centers @ w)
    assert np.abs(r["F"].sum(axis=1) - exact).max() < 1e-12
