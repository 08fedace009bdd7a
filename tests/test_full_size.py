"""Parity at the benchmark workloads' own sizes.

Cells taken from the full 256x256-cell evaluation Fourier field (N = 32) and
from the full 3D sphere field (112k spheres, N in {8, 16, 24}) against the
oracle's direct solves (1e-10 relative, M and F); and, over whole batches,
the size-independent properties of the coarse element matrices: symmetry,
zero row sums (the basis is a partition of unity), positive
semi-definiteness, and sum_cells sum_i F_i = integral of f over the domain."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def check_invariants(M, F, f_total, tol_rows, tol_f):
    """tol_f: the basis solves stop at a 1e-10 relative residual, so
    sum_i phi_i = 1 holds to the solve error, which grows with the condition
    number (1e4-contrast spheres in 3D)."""
    scale = np.abs(M).max(axis=(-2, -1))
    asym = (np.abs(M - np.swapaxes(M, -1, -2)).max(axis=(-2, -1)) / scale).max()
    rows = (np.abs(M.sum(axis=-1)).max(axis=-1) / scale).max()
    lmin = (np.linalg.eigvalsh(M)[..., 0] / scale).min()
    fsum = abs(F.sum() - f_total) / f_total
    assert asym <= 1e-12, asym
    assert rows <= tol_rows, rows
    assert lmin >= -1e-10, lmin
    assert fsum <= tol_f, fsum


@pytest.fixture(scope="module")
def sphere_field(pkg):
    return pkg.workloads.spheres_cube()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fourier_256_cells_against_oracle(pkg, oracle, engine, precision):
    W = pkg.workloads
    full = W.fourier_square(K=256, N=32, seeds=W.EVAL_SEEDS)
    prob = W.subset(full, [0, 12345, 40000, 65535])
    got = engine.run(prob, precision=precision, tol=1e-12)
    ref = oracle.run(prob)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["M"], ref["M"]) < 1e-10
    assert rel_err(got["F"], ref["F"]) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sphere_cells_against_oracle(pkg, oracle, engine, sphere_field, precision):
    W = pkg.workloads
    nf = sphere_field["n_fine_per_cell"]
    cells = [int(np.flatnonzero(nf == v)[0]) for v in (24, 16, 8)] + [int(np.flatnonzero(nf == 24)[-1])]
    prob = W.subset(sphere_field, cells)
    got = engine.run(prob, precision=precision, tol=1e-12)
    ref = oracle.run(prob)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel_err(got["M"], ref["M"]) < 1e-10
    assert rel_err(got["F"], ref["F"]) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_compiled_3d_shape_at_sphere_field_sizes(pkg, oracle, engine, sphere_field, precision):
    """Every compiled 3D launch shape the autotuner can pick -- one CTA per
    cell at each register cap, and the 8-CTA thread-block cluster per cell --
    on cells of the full sphere field with N = 24, 16 and 8 (the z-pair
    stencil instantiations) in one uneven-N launch, against the oracle."""
    W = pkg.workloads
    nf = sphere_field["n_fine_per_cell"]
    cells = [int(np.flatnonzero(nf == v)[1]) for v in (24, 16, 8)]
    prob = W.subset(sphere_field, cells)
    ref = oracle.run(prob, want_basis=True)
    prec = 0 if precision == "fp64" else 1
    probe = engine.autotune(prob, precision=precision, tol=1e-12, sample_cells=3)
    assert probe["n_variants"] >= 2
    try:
        for v in range(probe["n_variants"]):
            engine.set_tuning({"dim": 3, "n_max": 24, "precision": prec, "variant": v, "check_interval": 0,
                               "inner_tol": 1e-6})
            got = engine.run(prob, precision=precision, tol=1e-12, want_basis=True)
            assert got["rc"] == 0 and np.all(got["status"] == 0), v
            assert got["stats"]["kernel_launches"] == 2, v  # tabulation + one basis kernel
            assert rel_err(got["M"], ref["M"]) < 1e-10, (v, rel_err(got["M"], ref["M"]))
            assert rel_err(got["F"], ref["F"]) < 1e-10, (v, rel_err(got["F"], ref["F"]))
            assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9, v
    finally:
        engine.set_tuning({"dim": 3, "n_max": 24, "precision": prec, "variant": 0, "check_interval": 0,
                           "inner_tol": 1e-6})


def test_fourier_64_full_batch_invariants(pkg, engine):
    prob = pkg.workloads.fourier_square(K=64, N=32)
    got = engine.run(prob, precision="fp64", tol=1e-10)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    check_invariants(got["M"], got["F"], 1.0, 1e-9, 1e-9)  # f = 1 on the unit square
    mixed = engine.run(prob, precision="mixed", tol=1e-10)
    assert mixed["rc"] == 0
    assert rel_err(mixed["M"], got["M"]) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sphere_full_batch_invariants(pkg, engine, sphere_field, precision):
    got = engine.run(sphere_field, precision=precision, tol=1e-10)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    check_invariants(got["M"], got["F"], 1.0, 1e-9, 1e-6)  # f = 1 on the unit cube
