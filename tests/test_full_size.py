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
            # tabulation + one basis kernel; the cluster shape of the mixed
            # form splits the batch by size class (one more launch)
            split = precision == "mixed" and v == probe["n_variants"] - 1
            assert got["stats"]["kernel_launches"] == (3 if split else 2), v
            assert rel_err(got["M"], ref["M"]) < 1e-10, (v, rel_err(got["M"], ref["M"]))
            assert rel_err(got["F"], ref["F"]) < 1e-10, (v, rel_err(got["F"], ref["F"]))
            assert np.abs(got["basis"] - ref["basis"]).max() < 1e-9, v
    finally:
        engine.set_tuning({"dim": 3, "n_max": 24, "precision": prec, "variant": 0, "check_interval": 0,
                           "inner_tol": 1e-6})


@pytest.mark.parametrize("path", ["eager", "graph"])
def test_size_class_split_against_oracle(pkg, oracle, engine, sphere_field, path):
    """The mixed form with the thread-block-cluster shape on an uneven batch
    splits it by size class: the N = 24 cell runs in the cluster launch, the
    N = 16 and 8 cells in a one-CTA-per-cell launch on a second stream beside
    it.  Eagerly (3 launches: tabulation and the two basis kernels), and from
    device buffers through the CUDA graph (captured once, replayed once),
    against the oracle."""
    torch = pytest.importorskip("torch")
    abi = pkg._abi
    W = pkg.workloads
    nf = sphere_field["n_fine_per_cell"]
    cells = [int(np.flatnonzero(nf == v)[2]) for v in (24, 16, 8)]
    prob = W.subset(sphere_field, cells)
    ref = oracle.run(prob)
    probe = engine.autotune(prob, precision="mixed", tol=1e-12, sample_cells=3)
    slab = probe["n_variants"] - 1  # the cluster shape: the last compiled 3D mixed shape
    engine.set_tuning({"dim": 3, "n_max": 24, "precision": 1, "variant": slab, "check_interval": 0,
                       "inner_tol": 1e-6})
    try:
        if path == "eager":
            got = engine.run(prob, precision="mixed", tol=1e-12)
            assert got["rc"] == 0 and np.all(got["status"] == 0)
            assert got["stats"]["kernel_launches"] == 3
            runs = [(got["M"], got["F"])]
        else:
            n = len(cells)
            nf_d = torch.from_numpy(np.ascontiguousarray(prob["n_fine_per_cell"], dtype=np.int32)).cuda()
            corners_d = torch.from_numpy(np.ascontiguousarray(prob["corners"])).cuda()
            tab_d = torch.from_numpy(engine.tabulate(prob, 1)).cuda()
            d = abi.BatchDesc()
            d.dim, d.n_cells, d.n_fine = 3, n, 24
            d.precision = abi.PREC_MIXED
            d.corners, d.n_fine_per_cell = corners_d.data_ptr(), nf_d.data_ptr()
            d.coef.kind, d.coef.ncomp, d.coef.qp_values = abi.COEF_TABULATED, 1, tab_d.data_ptr()
            d.f_value, d.tol, d.maxit, d.memory = prob["f_value"], 1e-12, 1000, abi.MEM_DEVICE
            M = torch.empty((n, 8, 8), dtype=torch.float64, device="cuda")
            F = torch.empty((n, 8), dtype=torch.float64, device="cuda")
            st = torch.empty(n, dtype=torch.int32, device="cuda")
            it = torch.empty((n, 8), dtype=torch.int32, device="cuda")
            engine.set_stream(None)  # the handle's own stream: graphs are used
            cap0, rep0 = engine.graph_info()
            runs = []
            for call in range(2):
                M.fill_(float("nan"))
                F.fill_(float("nan"))
                st.fill_(-7)
                torch.cuda.synchronize()
                rc, s = engine.run_desc(d, M.data_ptr(), F.data_ptr(), None, st.data_ptr(), it.data_ptr(),
                                        stats=False)
                assert rc == abi.OK and s is None
                torch.cuda.synchronize()
                assert np.all(st.cpu().numpy() == abi.CELL_CONVERGED), call
                runs.append((M.cpu().numpy(), F.cpu().numpy()))
            cap, rep = engine.graph_info()
            assert (cap - cap0, rep - rep0) == (1, 2)
        for M, F in runs:
            assert rel_err(M, ref["M"]) < 1e-10, rel_err(M, ref["M"])
            assert rel_err(F, ref["F"]) < 1e-10, rel_err(F, ref["F"])
    finally:
        engine.set_tuning({"dim": 3, "n_max": 24, "precision": 1, "variant": 0, "check_interval": 0,
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
