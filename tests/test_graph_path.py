"""The device-resident call without stats: the branch the throughput figures
time.  It replays one CUDA graph (queue reset + persistent basis kernel) per
call and re-captures it when a pointer, size or launch choice changes.

Each case runs the same descriptor twice (capture, then replay) and once more
with a different output pointer (re-capture), with every output poisoned with
NaN before the call, and compares M, F and the basis with the oracle's direct
solves on config-2 random-Fourier cells (N = 32): at the benchmark's own 1e-10
relative residual M and F within 1e-10 relative, and at 1e-13 additionally
the basis values within 1e-9 absolute."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL = 1e-10
CELLS = [0, 1, 63, 64, 2080, 4095]


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def fourier_cells(pkg, oracle, engine):
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), CELLS)
    return prob, oracle.run(prob, want_basis=True), engine.tabulate(prob, 3)


def device_desc(abi, prob, corners_d, qp_d, precision, tol):
    d = abi.BatchDesc()
    d.dim, d.n_cells, d.n_fine = 2, prob["corners"].shape[0], prob["n_fine"]
    d.precision = precision
    d.corners = corners_d.data_ptr()
    d.coef.kind, d.coef.ncomp, d.coef.qp_values = abi.COEF_TABULATED, 3, qp_d.data_ptr()
    d.f_value = prob["f_value"]
    d.tol, d.maxit = tol, 1000
    d.memory = abi.MEM_DEVICE
    return d


@pytest.mark.parametrize("tol", [1e-10, 1e-13])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replayed_path_matches_oracle(pkg, engine, fourier_cells, precision, tol):
    torch = pytest.importorskip("torch")
    abi = pkg._abi
    prob, ref, tab = fourier_cells
    n, nodes = prob["corners"].shape[0], 33 * 33
    corners_d = torch.from_numpy(prob["corners"]).cuda()
    qp_d = torch.from_numpy(tab).cuda()
    prec = abi.PREC_FP64 if precision == "fp64" else abi.PREC_MIXED
    d = device_desc(abi, prob, corners_d, qp_d, prec, tol)
    bufs = [{"M": torch.empty((n, 4, 4), dtype=torch.float64, device="cuda"),
             "F": torch.empty((n, 4), dtype=torch.float64, device="cuda"),
             "B": torch.empty((n, 4, nodes), dtype=torch.float64, device="cuda"),
             "st": torch.empty(n, dtype=torch.int32, device="cuda"),
             "it": torch.empty((n, 4), dtype=torch.int32, device="cuda")} for _ in range(2)]
    engine.set_stream(None)  # the handle's own stream: graphs are used
    cap0, rep0 = engine.graph_info()
    for call, b in enumerate((bufs[0], bufs[0], bufs[1])):
        for k in ("M", "F", "B"):
            b[k].fill_(float("nan"))
        b["st"].fill_(-7)
        torch.cuda.synchronize()
        rc, st = engine.run_desc(d, b["M"].data_ptr(), b["F"].data_ptr(), b["B"].data_ptr(),
                                 b["st"].data_ptr(), b["it"].data_ptr(), stats=False)
        assert rc == abi.OK and st is None
        torch.cuda.synchronize()
        cap, rep = engine.graph_info()
        # call 0 captures, call 1 replays the same graph, call 2 (new pointers) re-captures
        assert rep - rep0 == call + 1, (call, rep - rep0)
        assert cap - cap0 == (1 if call < 2 else 2), (call, cap - cap0)
        assert np.all(b["st"].cpu().numpy() == abi.CELL_CONVERGED), call
        M, F, B = b["M"].cpu().numpy(), b["F"].cpu().numpy(), b["B"].cpu().numpy()
        assert rel_err(M, ref["M"]) < TOL_REL, (call, rel_err(M, ref["M"]))
        assert rel_err(F, ref["F"]) < TOL_REL, (call, rel_err(F, ref["F"]))
        if tol <= 1e-13:
            assert np.abs(B.ravel() - ref["basis"]).max() < 1e-9, call
        assert np.all(np.isfinite(B))


def test_stats_call_does_not_use_the_graph(pkg, engine, fourier_cells):
    """Calls that return stats (or use host memory) run the eager branch."""
    prob, ref, _ = fourier_cells
    engine.set_stream(None)
    cap0, rep0 = engine.graph_info()
    got = engine.run(prob, precision="fp64", tol=1e-10)
    assert engine.graph_info() == (cap0, rep0)
    assert rel_err(got["M"], ref["M"]) < TOL_REL
