"""msfem_run_batch_noalloc: the entry point for callers that cannot allocate
device memory -- frameworks that own every device allocation of the process
(a fixed pool or budget, where a hidden cudaMalloc fails or breaks the
accounting) and latency-critical time loops (cudaMalloc and cudaFree
synchronise the whole device).  It must give the same coarse matrices, loads
and basis as msfem_run_batch, and as the oracle's direct solve, call after
call, while using only the library's fixed scratch array.  Collected last on
purpose (file name)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL = 1e-10


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def device_desc(abi, prob, corners_d, precision, tol, qp_d=None, ncomp=0):
    d = abi.BatchDesc()
    d.dim = prob["dim"]
    d.n_cells = prob["corners"].shape[0]
    d.n_fine = prob["n_fine"]
    d.precision = precision
    d.corners = corners_d.data_ptr()
    c = prob["coef"]
    d.coef.kind = c["kind"] if qp_d is None else abi.COEF_TABULATED
    d.coef.ncomp = ncomp
    for i, v in enumerate(c.get("params", [])):
        d.coef.params[i] = float(v)
    if qp_d is not None:
        d.coef.qp_values = qp_d.data_ptr()
    d.f_value = prob["f_value"]
    d.tol = tol
    d.maxit = 1000
    d.memory = abi.MEM_DEVICE
    return d


def run_noalloc(torch, lib, abi, d, n, n_nodes):
    M = torch.full((n, 4, 4), float("nan"), dtype=torch.float64, device="cuda")
    F = torch.full((n, 4), float("nan"), dtype=torch.float64, device="cuda")
    B = torch.full((n * 4 * n_nodes,), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    it = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.msfem_run_batch_noalloc(ctypes.byref(d), M.data_ptr(), F.data_ptr(), B.data_ptr(),
                                     st.data_ptr(), it.data_ptr(), None)
    assert rc == abi.OK, abi.last_error(lib)
    torch.cuda.synchronize()
    return M.cpu().numpy(), F.cpu().numpy(), B.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_run_batch_twice(pkg, oracle, engine, precision):
    torch = pytest.importorskip("torch")
    abi = pkg._abi
    lib = abi.load()
    prob = pkg.workloads.reference_problem(2, 3, 4)  # MatrixCoeff, f = 2, 64 cells, N = 16
    ref = engine.run(prob, precision=precision, tol=1e-12, want_basis=True)
    assert ref["rc"] == abi.OK
    direct = oracle.run(prob, want_basis=True)  # the oracle's banded-Cholesky solve
    n, n_nodes = prob["corners"].shape[0], 17 * 17
    corners_d = torch.from_numpy(prob["corners"]).cuda()
    prec = abi.PREC_FP64 if precision == "fp64" else abi.PREC_MIXED
    d = device_desc(abi, prob, corners_d, prec, 1e-12)
    first = None
    for call in range(2):  # the scratch keeps the previous call's contents
        M, F, B, st = run_noalloc(torch, lib, abi, d, n, n_nodes)
        assert np.all(st == abi.CELL_CONVERGED)
        assert rel_err(M, ref["M"]) < TOL_REL
        assert rel_err(F, ref["F"]) < TOL_REL
        assert np.abs(B - ref["basis"]).max() < 1e-9
        assert rel_err(M, direct["M"]) < TOL_REL
        assert rel_err(F, direct["F"]) < TOL_REL
        assert np.abs(B - direct["basis"]).max() < 1e-9
        if first is not None:
            assert np.array_equal(M, first)
        first = M


def test_noalloc_allocates_nothing(pkg, engine):
    """After the first call on the device (which loads the kernel and looks up
    the scratch address), further calls change neither torch's allocator nor
    the device's free memory."""
    torch = pytest.importorskip("torch")
    abi = pkg._abi
    lib = abi.load()
    prob = pkg.workloads.sinsin_square()  # 64 cells, N = 16
    n = prob["corners"].shape[0]
    corners_d = torch.from_numpy(prob["corners"]).cuda()
    d = device_desc(abi, prob, corners_d, abi.PREC_FP64, 1e-10)
    out = [torch.empty(s, dtype=t, device="cuda") for s, t in
           (((n, 4, 4), torch.float64), ((n, 4), torch.float64), ((n,), torch.int32))]
    args = (ctypes.byref(d), out[0].data_ptr(), out[1].data_ptr(), None, out[2].data_ptr(), None, None)
    assert lib.msfem_run_batch_noalloc(*args) == abi.OK
    torch.cuda.synchronize()
    alloc0 = torch.cuda.memory_allocated()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.msfem_run_batch_noalloc(*args) == abi.OK
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == alloc0
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, (free0, free1)
    assert np.all(out[2].cpu().numpy() == abi.CELL_CONVERGED)


@pytest.mark.parametrize("reference_stop", [False, True])
def test_noalloc_tabulated_coefficient(pkg, engine, reference_stop):
    """Device-resident tabulated random-Fourier tensor, N = 32; with
    reference_stop, also f tabulated at the Gauss points and the absolute
    residual stop of the reference's SolverControl."""
    torch = pytest.importorskip("torch")
    abi = pkg._abi
    lib = abi.load()
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), [0, 17, 300, 1999, 4095])
    tab = engine.tabulate(prob, 3)
    if reference_stop:
        prob = W.with_rhs(prob, lambda x: 2.0 + x[..., 0] * x[..., 1])
    ref = engine.run(prob, precision="fp64", tol=1e-11, want_basis=True, tol_absolute=reference_stop)
    corners_d = torch.from_numpy(prob["corners"]).cuda()
    qp_d = torch.from_numpy(tab).cuda()
    d = device_desc(abi, prob, corners_d, abi.PREC_FP64, 1e-11, qp_d=qp_d, ncomp=3)
    if reference_stop:
        fq_d = torch.from_numpy(prob["f_qp_values"]).cuda()
        d.f_qp_values = fq_d.data_ptr()
        d.tol_absolute = 1
    for _ in range(2):
        M, F, B, st = run_noalloc(torch, lib, abi, d, 5, 33 * 33)
        assert np.all(st == abi.CELL_CONVERGED)
        assert rel_err(M, ref["M"]) < TOL_REL
        assert rel_err(F, ref["F"]) < TOL_REL
        assert np.abs(B - ref["basis"]).max() < 1e-9


def test_noalloc_rejects_what_it_cannot_do(pkg):
    abi = pkg._abi
    lib = abi.load()
    W = pkg.workloads
    prob = W.sinsin_square()
    d = abi.BatchDesc()
    d.dim, d.n_fine, d.precision = 2, 16, abi.PREC_FP64
    corners = np.ascontiguousarray(prob["corners"])
    d.corners = corners.ctypes.data
    d.coef.kind = abi.COEF_SINSIN
    d.coef.params[0], d.coef.params[1] = 0.9, 1 / 64
    d.tol, d.maxit, d.memory = 1e-10, 100, abi.MEM_DEVICE
    d.n_cells = abi.NOALLOC_MAX_CELLS + 1
    rc = lib.msfem_run_batch_noalloc(ctypes.byref(d), 1, 1, None, 1, None, None)
    assert rc == abi.ERR_INVALID_ARG
    assert "MSFEM_NOALLOC_MAX_CELLS" in abi.last_error(lib)
    d.n_cells = 64
    d.memory = abi.MEM_HOST
    rc = lib.msfem_run_batch_noalloc(ctypes.byref(d), 1, 1, None, 1, None, None)
    assert rc == abi.ERR_INVALID_ARG
    d.memory = abi.MEM_DEVICE
    d.warm_start = abi.WARM_SURROGATE  # the network lives in a handle
    rc = lib.msfem_run_batch_noalloc(ctypes.byref(d), 1, 1, None, 1, None, None)
    assert rc == abi.ERR_UNSUPPORTED
    assert "MSFEM_WARM_SURROGATE" in abi.last_error(lib)
