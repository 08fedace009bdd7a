"""GPU parity: the CUDA path through the C-ABI against the CPU FP64 oracle
(banded Cholesky, exact to rounding) on the same seeded inputs.

Tolerances: FP64 form solved to 1e-13 relative residual, compared at 1e-10
relative (M, F) and 1e-9 absolute (basis values, which are O(1)); MIXED form
(FP32 inner CG + FP64 refinement) at the same bars; iteration counts of the
FP64 form equal the oracle's Jacobi-PCG restatement within +-2."""
import math

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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sinsin_square_parity(pkg, oracle, engine, precision):
    prob = pkg.workloads.sinsin_square()
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)
    assert got["stats"]["max_rel_residual"] < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_problem_parity(pkg, oracle, engine, precision):
    """The reference's own MatrixCoeff (PI_D), f = 2, n_refine = 3, n_refine_local = 4."""
    prob = pkg.workloads.reference_problem(2, 3, 4)
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


def test_fp64_iterations_match_oracle_jacobi_pcg(pkg, oracle, engine):
    prob = pkg.workloads.reference_problem(2, 2, 5)
    got = engine.run(prob, precision="fp64", tol=1e-10, check_interval=1)
    ref = oracle.run(prob, solver=oracle.SOLVER_JACOBI_CG, tol=1e-10)
    assert np.abs(got["iters"] - ref["iters"]).max() <= 2
    assert rel_err(got["M"], ref["M"]) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_random_fourier_tensor_parity(pkg, oracle, engine, precision):
    """Random-Fourier tensor family on a subset of cells, N = 32, tabulated on the GPU."""
    W = pkg.workloads
    full = W.fourier_square(K=64, N=32)
    prob = W.subset(full, [0, 1, 63, 64, 2080, 4095])
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    # oracle evaluates the same Fourier field itself
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


def test_two_level_shape_cuts_inner_iterations(pkg, oracle, engine):
    """The two-level inner preconditioner (Chebyshev smoothing around the
    Galerkin coarse correction) meets the oracle like every shape, with well
    under half the inner iterations of the degree-5 Chebyshev shape on
    random-Fourier cells (a broken coarse correction would still converge,
    only slowly)."""
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), [0, 1, 63, 64, 700, 2080, 3333, 4095])
    ref = oracle.run(prob)
    key = {"dim": 2, "n_max": 32, "precision": 1}
    n = engine.describe_tuning(dict(key, variant=0))["n_variants"]
    shapes = [dict(engine.describe_tuning(dict(key, variant=v)), variant=v) for v in range(n)]
    two = [t for t in shapes if t["coarse_spacing"] > 0]
    cheb = [t for t in shapes if t["poly_degree"] == 5 and t["coarse_spacing"] == 0 and t["ctas_per_sm"] == 1
            and t["threads"] == 256]
    assert two and cheb
    iters = {}
    try:
        for name, shape, ratio in (("two-level", two[0], 20.0), ("chebyshev", cheb[0], 100.0)):
            engine.set_tuning(dict(key, variant=shape["variant"], check_interval=0, inner_tol=1e-5, cheb_ratio=ratio))
            got = engine.run(prob, precision="mixed", tol=1e-10)
            check(got, ref, basis=False)
            iters[name] = int(got["stats"]["iterations_total"])
    finally:
        engine.set_tuning(dict(key, variant=0, check_interval=0, inner_tol=1e-6))
    assert iters["two-level"] < 0.5 * iters["chebyshev"], iters


def test_two_level_shape_absolute_tolerance(pkg, oracle, engine):
    """The two-level shape under the reference's absolute stopping rule
    (SolverControl(1000, 1e-12) on the residual, diffusion_problem_basis.tpp:297)
    with A = 0.01 I, so ||b|| is well below 1: no more inner iterations than
    the relative stop, M at the direct solve's value (quadratic in the basis
    error), F within what the absolute stop allows (linear in the basis
    error; the stop leaves a relative residual near 1e-12 / ||b||)."""
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 32, {"kind": 0, "params": [0.01, 0.0, 0.01]})
    key = {"dim": 2, "n_max": 32, "precision": 1}
    n = engine.describe_tuning(dict(key, variant=0))["n_variants"]
    v = next(i for i in range(n) if engine.describe_tuning(dict(key, variant=i))["coarse_spacing"] > 0)
    try:
        engine.set_tuning(dict(key, variant=v, check_interval=0, inner_tol=1e-5, cheb_ratio=20.0))
        rel = engine.run(prob, precision="mixed", tol=1e-12)
        ab = engine.run(prob, precision="mixed", tol=1e-12, tol_absolute=True)
    finally:
        engine.set_tuning(dict(key, variant=0, check_interval=0, inner_tol=1e-6))
    assert rel["rc"] == 0 and ab["rc"] == 0 and np.all(ab["status"] == 0)
    assert ab["iters"].sum() <= rel["iters"].sum()
    direct = oracle.run(prob)
    assert rel_err(ab["M"], direct["M"]) < TOL_REL
    assert rel_err(ab["F"], direct["F"]) < 1e-8
    assert rel_err(rel["F"], direct["F"]) < TOL_REL


def test_tabulation_matches_oracle(pkg, oracle, engine):
    """The field generator against the oracle's direct evaluation: affine
    cells take the phase-recurrence path, a bilinear cell the per-point one."""
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), [5, 700, 4095])
    corners = prob["corners"].copy()
    corners[2, 3] += [-0.0011, 0.0007]  # cell 4095 made bilinear
    prob["corners"] = corners
    a = engine.tabulate(prob, 3)
    b = oracle.tabulate(prob, 3)
    assert np.abs(a - b).max() < 1e-12 * np.abs(b).max()


@pytest.mark.parametrize("ncomp", [1, 6])
def test_tabulation_matches_oracle_3d(pkg, oracle, engine, ncomp):
    """3D log-normal Fourier field (a = exp g1) on uneven N up to 24, both
    output layouts (scalar, and the tensor a I)."""
    W = pkg.workloads
    coef = W.fourier_coef((9,), dim=3, n_modes=48, kmax=64 * np.pi)
    prob = W.problem(3, W.unit_cube_corners(3, 4)[[0, 21, 63]], np.array([24, 7, 17], dtype=np.int32), coef)
    a = engine.tabulate(prob, ncomp)
    b = oracle.tabulate(prob, ncomp)
    assert a.shape == b.shape
    assert np.abs(a - b).max() < 1e-12 * np.abs(b).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("geom", ["parallelogram", "bilinear"])
def test_general_geometry(pkg, oracle, engine, geom, precision):
    W = pkg.workloads
    c = W.unit_cube_corners(2, 4) * 0.8 + 0.05
    if geom == "parallelogram":
        c = c + c[:, :, 1:2] * np.array([0.2, 0.0])  # shear
    else:
        rng = np.random.default_rng(7)
        c = c + rng.uniform(-0.01, 0.01, size=c.shape) * np.array([1, 1])
    prob = W.problem(2, c, 12, {"kind": 1}, f_value=2.0)
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


def test_constant_tensor_known_answer(pkg, engine):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 4), 16, {"kind": 0, "params": [3.0, 0.0, 0.5]})
    got = engine.run(prob, precision="fp64", tol=1e-13)
    H = 0.25
    K1 = np.array([[1.0, -1.0], [-1.0, 1.0]]) / H
    M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) * H / 6.0
    exact = 3.0 * np.kron(M1, K1) + 0.5 * np.kron(K1, M1)
    assert np.abs(got["M"] - exact).max() < 1e-11
    assert np.allclose(got["F"], H * H / 4, rtol=1e-12)


@pytest.mark.parametrize("N", [1, 2, 3, 7, 16, 31, 32])
def test_ragged_sizes(pkg, oracle, engine, N):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), N, {"kind": 2, "params": [0.5, 0.25]})
    got = engine.run(prob, precision="fp64", tol=1e-13, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check(got, ref)


def test_uneven_refinement_one_launch(pkg, oracle, engine):
    W = pkg.workloads
    corners = W.unit_cube_corners(2, 4)
    nf = np.array([8, 16, 32, 24, 5, 32, 16, 8, 12, 32, 8, 16, 20, 4, 32, 9], dtype=np.int32)
    prob = W.problem(2, corners, nf, {"kind": 1}, f_value=2.0)
    for precision in ("fp64", "mixed"):
        got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
        ref = oracle.run(prob, want_basis=True)
        check(got, ref)
        assert got["stats"]["kernel_launches"] == 1


def test_warm_start_exact_basis_converges_immediately(pkg, oracle, engine):
    prob = pkg.workloads.sinsin_square()
    ref = oracle.run(prob, want_basis=True)
    got = engine.run(prob, precision="fp64", tol=1e-10, want_basis=True, warm_basis=ref["basis"])
    check(got, ref)
    assert got["iters"].max() <= 1


def test_maxit_reported_per_cell(pkg, engine):
    prob = pkg.workloads.sinsin_square()
    got = engine.run(prob, precision="fp64", tol=1e-13, maxit=3)
    assert got["rc"] != 0
    assert np.all(got["status"] == pkg._abi.CELL_MAXIT)


def test_nan_coefficient_reported(pkg, engine, oracle):
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 8, {"kind": 2, "params": [0.5, 0.25]})
    tab = oracle.tabulate(prob, 1)
    nfc = 64
    tab[1 * 4 * nfc + 17] = np.nan  # cell 1, q 0, fine cell 17
    tprob = dict(prob)
    tprob["coef"] = {"kind": 5, "ncomp": 1, "qp_values": tab}
    got = engine.run(tprob, precision="fp64", tol=1e-12)
    assert got["status"][1] == pkg._abi.CELL_NAN
    assert np.all(got["status"][[0, 2, 3]] == 0)


def test_degenerate_cell_reported(pkg, engine):
    W = pkg.workloads
    c = W.unit_cube_corners(2, 2).copy()
    c[2] = c[2][0]  # all four corners equal
    prob = W.problem(2, c, 8, {"kind": 0, "params": [1, 0, 1]})
    got = engine.run(prob, precision="fp64", tol=1e-12)
    assert got["status"][2] == pkg._abi.CELL_BAD_INPUT
    assert np.all(got["status"][[0, 1, 3]] == 0)


def test_mixed_reaches_tolerance_and_matches_fp64(pkg, engine):
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), list(range(0, 4096, 97)))
    a = engine.run(prob, precision="fp64", tol=1e-10)
    b = engine.run(prob, precision="mixed", tol=1e-10)
    assert a["stats"]["max_rel_residual"] < 1e-10
    assert b["stats"]["max_rel_residual"] < 1e-10
    assert rel_err(b["M"], a["M"]) < 1e-10


@pytest.mark.parametrize("n_max", [32, 16])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_compiled_launch_shape_gives_the_same_answer(pkg, oracle, engine, precision, n_max):
    """Each CTA shape the autotuner can pick (each inner tolerance and, for the
    polynomial-preconditioned shapes, each Chebyshev interval ratio) keeps parity."""
    W = pkg.workloads
    if n_max == 32:
        prob = W.subset(W.fourier_square(K=64, N=32), [3, 1000, 2222, 4000])
    else:
        prob = W.subset(W.sinsin_square(), [0, 9, 36, 63])
    ref = oracle.run(prob, want_basis=True)
    probe = engine.autotune(prob, precision=precision, tol=1e-13, sample_cells=4)
    assert probe["n_variants"] >= 1
    prec = 0 if precision == "fp64" else 1
    for v in range(probe["n_variants"]):
        engine.set_tuning({"dim": 2, "n_max": n_max, "precision": prec, "variant": v, "check_interval": 0,
                           "inner_tol": 1e-6})
        for itol in ((1e-4, 1e-6) if precision == "mixed" else (1e-6,)):
            for ratio in (10.0, 100.0) if precision == "mixed" else (30.0,):
                engine.set_tuning({"dim": 2, "n_max": n_max, "precision": prec, "variant": v,
                                   "check_interval": 0, "inner_tol": itol, "cheb_ratio": ratio})
                got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
                check(got, ref)
    engine.set_tuning({"dim": 2, "n_max": n_max, "precision": prec, "variant": 0, "check_interval": 0,
                       "inner_tol": 1e-6})


@pytest.mark.parametrize("warm", [False, True])
def test_every_mixed_shape_on_ragged_sizes(pkg, oracle, engine, warm):
    """Every compiled mixed launch shape of the N <= 32 class on cells with N
    from 1 to 32 in one launch (partial thread strips, rows shorter than the
    class, cells without interior nodes), cold and warm-started from the
    oracle's basis plus a perturbation."""
    W = pkg.workloads
    nf = np.array([17, 18, 21, 24, 27, 29, 30, 31, 32, 1, 2, 3, 5, 8, 16, 32], dtype=np.int32)
    prob = W.problem(2, W.unit_cube_corners(2, 4), nf, {"kind": 1}, f_value=2.0)
    ref = oracle.run(prob, want_basis=True)
    warm_basis = None
    if warm:
        rng = np.random.default_rng(11)
        warm_basis = ref["basis"] + 1e-3 * rng.standard_normal(ref["basis"].shape)
    probe = engine.autotune(prob, precision="mixed", tol=1e-13, sample_cells=16)
    assert probe["n_variants"] >= 1
    try:
        for v in range(probe["n_variants"]):
            for ratio in (10.0, 100.0):
                engine.set_tuning({"dim": 2, "n_max": 32, "precision": 1, "variant": v, "check_interval": 0,
                                   "inner_tol": 1e-5, "cheb_ratio": ratio})
                got = engine.run(prob, precision="mixed", tol=1e-13, want_basis=True, warm_basis=warm_basis)
                check(got, ref)
    finally:
        engine.set_tuning({"dim": 2, "n_max": 32, "precision": 1, "variant": 0, "check_interval": 0,
                           "inner_tol": 1e-6})


def test_every_mixed_shape_on_ragged_sizes_16(pkg, oracle, engine):
    """The N <= 16 class: every compiled mixed shape on N = 1 ... 16 in one
    launch, on bilinear cells (general geometry in the mixed form)."""
    W = pkg.workloads
    nf = np.array([1, 2, 3, 4, 5, 7, 9, 11, 12, 13, 14, 15, 16, 16, 8, 6], dtype=np.int32)
    c = W.unit_cube_corners(2, 4) * 0.8 + 0.05
    c = c + np.random.default_rng(9).uniform(-0.01, 0.01, size=c.shape)
    prob = W.problem(2, c, nf, {"kind": 1}, f_value=2.0)
    ref = oracle.run(prob, want_basis=True)
    probe = engine.autotune(prob, precision="mixed", tol=1e-13, sample_cells=16)
    try:
        for v in range(probe["n_variants"]):
            for ratio in (10.0, 100.0):
                engine.set_tuning({"dim": 2, "n_max": 16, "precision": 1, "variant": v, "check_interval": 0,
                                   "inner_tol": 1e-5, "cheb_ratio": ratio})
                got = engine.run(prob, precision="mixed", tol=1e-13, want_basis=True)
                check(got, ref)
    finally:
        engine.set_tuning({"dim": 2, "n_max": 16, "precision": 1, "variant": 0, "check_interval": 0,
                           "inner_tol": 1e-6})


@pytest.mark.parametrize("dim", [2, 3])
def test_empty_batch(pkg, engine, dim):
    """No cells: every entry point returns OK without launching work."""
    W = pkg.workloads
    nv = 1 << dim
    prob = W.problem(dim, np.zeros((0, nv, dim)), np.zeros(0, dtype=np.int32),
                     {"kind": 2, "params": [0.5, 0.25]})
    for precision in ("fp64", "mixed"):
        got = engine.run(prob, precision=precision, want_basis=True)
        assert got["rc"] == 0
        assert got["M"].shape == (0, nv, nv) and got["stats"]["solves"] == 0
    assert engine.reconstruct(prob, np.zeros(0), np.zeros((0, nv))).shape == (0,)
