"""The parts of the drop-in boundary that follow the reference's own
interfaces beyond a constant f and a relative tolerance:

- a right-hand side given at the Gauss points (RightHandSide<dim>::value_list,
  include/base/diffusion_problem_basis.tpp:204-205, :219-220) against the
  oracle's assembly with the same values;
- the reference's stopping rule, SolverControl(1000, 1e-12): an absolute l2
  residual (diffusion_problem_basis.tpp:297), against the oracle's Jacobi-PCG
  with the same absolute stop (iteration counts) and its direct solve (M, F).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL = 1e-10


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def f_wavy(x):
    """A smooth non-constant f (its mean is about 2)."""
    s = np.sin(7.0 * x[..., 0]) * np.cos(5.0 * x[..., 1])
    if x.shape[-1] == 3:
        s = s * np.cos(3.0 * x[..., 2])
    return 2.0 + s + x[..., 0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tabulated_rhs_2d(pkg, oracle, engine, precision):
    W = pkg.workloads
    base = W.subset(W.fourier_square(K=64, N=32), [0, 65, 2080, 4095])
    corners = base["corners"].copy()
    corners[1, 3] += [0.002, -0.001]  # one general (bilinear) cell
    base["corners"] = corners
    prob = W.with_rhs(base, f_wavy)
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["F"], ref["F"]) < TOL_REL, rel_err(got["F"], ref["F"])
    assert rel_err(got["M"], ref["M"]) < TOL_REL
    assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9
    # a non-constant f changes F and only F
    const = engine.run(base, precision=precision, tol=1e-13)
    assert rel_err(got["F"], const["F"]) > 1e-3
    assert rel_err(got["M"], const["M"]) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tabulated_rhs_3d_uneven(pkg, oracle, engine, precision):
    W = pkg.workloads
    rng = np.random.default_rng(3)
    sp = np.column_stack([rng.uniform(0, 1, (300, 3)), rng.uniform(0.02, 0.05, 300)])
    corners = W.unit_cube_corners(3, 4)[[2, 21, 50]]
    nf = np.array([6, 8, 4], dtype=np.int32)
    prob = W.with_rhs(W.problem(3, corners, nf, {"kind": 4, "params": [1e4], "spheres": sp}), f_wavy)
    got = engine.run(prob, precision=precision, tol=1e-12)
    ref = oracle.run(prob)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["F"], ref["F"]) < TOL_REL, rel_err(got["F"], ref["F"])
    assert rel_err(got["M"], ref["M"]) < TOL_REL


@pytest.mark.parametrize("dim", [2, 3])
def test_absolute_tolerance_matches_oracle(pkg, oracle, engine, dim):
    """FP64 Jacobi-PCG with the reference's absolute stop: the same iteration
    counts as the oracle's Jacobi-PCG with that stop (+-2), and M/F at the
    direct solve's values."""
    W = pkg.workloads
    if dim == 2:
        prob = W.reference_problem(2, 2, 4)  # MatrixCoeff, f = 2, 16 cells, N = 16
    else:
        prob = W.problem(3, W.unit_cube_corners(3, 2), 6, {"kind": 2, "params": [0.8, 0.25]}, f_value=2.0)
    got = engine.run(prob, precision="fp64", tol=1e-12, tol_absolute=True, check_interval=1)
    ref_it = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-12, tol_absolute=True)
    direct = oracle.run(prob)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert np.abs(got["iters"] - ref_it["iters"]).max() <= 2
    assert rel_err(got["M"], direct["M"]) < TOL_REL
    assert rel_err(got["F"], direct["F"]) < TOL_REL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_absolute_tolerance_is_not_relative(pkg, oracle, engine, precision):
    """With A = 0.01 I the Dirichlet lifting has ||b|| well below 1, so the
    absolute stop at 1e-12 is reached with fewer iterations than the relative
    stop at 1e-12, as in the oracle's Jacobi-PCG; M stays at the direct
    solve's value (it is quadratic in the basis error)."""
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 16, {"kind": 0, "params": [0.01, 0.0, 0.01]})
    rel = engine.run(prob, precision=precision, tol=1e-12, check_interval=1)
    ab = engine.run(prob, precision=precision, tol=1e-12, tol_absolute=True, check_interval=1)
    assert rel["rc"] == 0 and ab["rc"] == 0
    if precision == "fp64":
        assert ab["iters"].sum() < rel["iters"].sum()
    else:  # inner FP32 iterations: fewer or equal (whole refinements are saved)
        assert ab["iters"].sum() <= rel["iters"].sum()
    o_rel = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-12)
    o_abs = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-12, tol_absolute=True)
    assert o_abs["iters"].sum() < o_rel["iters"].sum()
    direct = oracle.run(prob)
    assert rel_err(ab["M"], direct["M"]) < TOL_REL
