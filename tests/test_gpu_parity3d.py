"""3D GPU parity against the CPU FP64 oracle: trilinear Q1 assembly, 8
Dirichlet solves per cell, coarse 8x8 matrix and load.  Same tolerances as 2D:
M, F within 1e-10 relative, basis values within 1e-9 absolute."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL = 1e-10


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def check(got, ref, basis=True):
    assert got["rc"] == 0, got["status"]
    assert np.all(got["status"] == 0)
    assert rel_err(got["M"], ref["M"]) < TOL_REL
    assert rel_err(got["F"], ref["F"]) < TOL_REL
    if basis:
        assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9


def test_constant_diagonal_tensor_kat_3d(pkg, engine):
    W = pkg.workloads
    a = (2.0, 0.5, 1.5)
    prob = W.problem(3, W.unit_cube_corners(3, 2), 6, {"kind": 0, "params": [a[0], 0, 0, a[1], 0, a[2]]},
                     f_value=3.0)
    got = engine.run(prob, precision="fp64", tol=1e-13)
    H = 0.5
    K1 = np.array([[1.0, -1.0], [-1.0, 1.0]]) / H
    M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) * H / 6.0
    exact = (a[0] * np.kron(M1, np.kron(M1, K1)) + a[1] * np.kron(M1, np.kron(K1, M1))
             + a[2] * np.kron(K1, np.kron(M1, M1)))
    assert np.abs(got["M"] - exact).max() < 1e-11
    assert np.allclose(got["F"], 3.0 * H ** 3 / 8, rtol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_coefficient_3d(pkg, oracle, engine, precision):
    """The reference MatrixCoeff<3> (ZXZ Euler rotation, PI_D) on a 2^3 coarse mesh."""
    prob = pkg.workloads.reference_problem(3, 1, 3)  # 8 coarse cells, N = 8
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


@pytest.mark.parametrize("N", [1, 2, 3, 5])
def test_ragged_sizes_3d(pkg, oracle, engine, N):
    W = pkg.workloads
    prob = W.problem(3, W.unit_cube_corners(3, 2), N, {"kind": 2, "params": [0.5, 0.5]})
    got = engine.run(prob, precision="fp64", tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_spheres_uneven_one_launch(pkg, oracle, engine, precision):
    """The sphere coefficient (1e4 contrast) with uneven N in one launch."""
    W = pkg.workloads
    rng = np.random.default_rng(5)
    sp = np.column_stack([rng.uniform(0, 1, (600, 3)), rng.uniform(0.02, 0.05, 600)])
    corners = W.unit_cube_corners(3, 4)[[0, 5, 21, 42, 63]]
    nf = np.array([8, 4, 12, 6, 8], dtype=np.int32)
    prob = W.problem(3, corners, nf, {"kind": 4, "params": [1e4], "spheres": sp})
    got = engine.run(prob, precision=precision, tol=1e-12, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    assert got["stats"]["kernel_launches"] == 2  # tabulation + one basis kernel
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["M"], ref["M"]) < TOL_REL
    assert rel_err(got["F"], ref["F"]) < TOL_REL
    assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9


def test_fp64_iterations_match_oracle_jacobi_pcg_3d(pkg, oracle, engine):
    W = pkg.workloads
    prob = W.problem(3, W.unit_cube_corners(3, 2), 6, {"kind": 2, "params": [0.8, 0.25]})
    got = engine.run(prob, precision="fp64", tol=1e-10, check_interval=1)
    ref = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-10)
    assert np.abs(got["iters"] - ref["iters"]).max() <= 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_compiled_launch_shape_gives_the_same_answer_3d(pkg, oracle, engine, precision):
    """Each 3D launch shape the autotuner can pick (threads x CTAs per SM,
    i.e. register caps) keeps parity on an uneven-N, 1e4-contrast batch."""
    W = pkg.workloads
    rng = np.random.default_rng(9)
    sp = np.column_stack([rng.uniform(0, 1, (400, 3)), rng.uniform(0.02, 0.05, 400)])
    corners = W.unit_cube_corners(3, 4)[[1, 22, 40]]
    nf = np.array([6, 9, 4], dtype=np.int32)
    prob = W.problem(3, corners, nf, {"kind": 4, "params": [1e4], "spheres": sp})
    ref = oracle.run(prob, want_basis=True)
    probe = engine.autotune(prob, precision=precision, tol=1e-12, sample_cells=3)
    prec = 0 if precision == "fp64" else 1
    assert probe["n_variants"] >= 2
    for v in range(probe["n_variants"]):
        engine.set_tuning({"dim": 3, "n_max": 9, "precision": prec, "variant": v, "check_interval": 0,
                           "inner_tol": 1e-6})
        got = engine.run(prob, precision=precision, tol=1e-12, want_basis=True)
        assert got["rc"] == 0 and np.all(got["status"] == 0), v
        assert rel_err(got["M"], ref["M"]) < TOL_REL, v
        assert rel_err(got["F"], ref["F"]) < TOL_REL, v
        assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9, v
    engine.set_tuning({"dim": 3, "n_max": 9, "precision": prec, "variant": 0, "check_interval": 0,
                       "inner_tol": 1e-6})


def test_slab_cluster_ragged_and_empty_slabs(pkg, oracle, engine):
    """The mixed form's 8-CTA slab cluster on cells with fewer interior
    planes than CTAs (N = 1, 2, 3, 5: empty slabs, no interior at N = 1)
    next to the largest cell (N = 24) in one launch, against the oracle."""
    W = pkg.workloads
    rng = np.random.default_rng(12)
    sp = np.column_stack([rng.uniform(0, 1, (300, 3)), rng.uniform(0.02, 0.05, 300)])
    corners = W.unit_cube_corners(3, 4)[[3, 17, 30, 44, 60]]
    nf = np.array([1, 2, 3, 5, 24], dtype=np.int32)
    prob = W.problem(3, corners, nf, {"kind": 4, "params": [1e4], "spheres": sp})
    probe = engine.autotune(prob, precision="mixed", tol=1e-12, sample_cells=5)
    slab = probe["n_variants"] - 1  # the slab cluster is the last compiled mixed shape
    engine.set_tuning({"dim": 3, "n_max": 24, "precision": 1, "variant": slab, "check_interval": 0,
                       "inner_tol": 1e-6})
    try:
        got = engine.run(prob, precision="mixed", tol=1e-12, want_basis=True)
    finally:
        engine.set_tuning({"dim": 3, "n_max": 24, "precision": 1, "variant": 0, "check_interval": 0,
                           "inner_tol": 1e-6})
    ref = oracle.run(prob, want_basis=True)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["M"], ref["M"]) < TOL_REL
    assert rel_err(got["F"], ref["F"]) < TOL_REL
    assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9
