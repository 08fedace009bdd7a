"""The MsFEM against the standard fine-scale FEM on the same coefficient
(diffusion_problem.tpp:102-279, run by main.cxx:33-35 beside the MsFEM):
the reference's own problem (MatrixCoeff, f = 2, Dirichlet on ids 0/2,
Neumann on 1/3) on the 8 x 8 coarse mesh with N = 16, against Q1 FEM on the
128 x 128 fine mesh.

The standard FEM needs no separate assembler: the multiscale basis of a cell
with N = 1 is the Q1 basis (no interior nodes), so the same batch call on
the fine mesh's cells with N = 1 returns the standard QGauss(2) element
matrices and loads, and the coarse-level solve with the reference's boundary
data (diffusion_problem_ms.tpp:91-296, the same classes as
diffusion_problem.tpp) is the standard FEM solve.  Checked: the MsFEM's fine
solution (msfem_reconstruct) is within 1% (relative l2 over the fine
nodes; measured 0.53%) of the fine FEM, and over 10x closer than Q1 FEM on
the coarse mesh (14.5%)."""
import ctypes

import numpy as np
import pytest

K, L = 8, 4          # n_refine = 3, n_refine_local = 4
N = 1 << L
KF = K * N


def weights(u_c, k):
    return np.array([[u_c[(c // k + (i >> 1)) * (k + 1) + c % k + (i & 1)] for i in range(4)]
                     for c in range(k * k)])


def fine_grid(cell_values):
    """[cell][(N+1)^2] lexicographic -> the (KF+1)^2 global fine grid."""
    g = np.zeros((KF + 1, KF + 1))
    v = cell_values.reshape(K, K, N + 1, N + 1)
    for cy in range(K):
        for cx in range(K):
            g[cy * N:(cy + 1) * N + 1, cx * N:(cx + 1) * N + 1] = v[cy, cx]
    return g


def coarse_q1_on_fine(u_c):
    """Bilinear interpolation of coarse nodal values to the fine nodes."""
    t = np.arange(KF + 1) / N
    i0 = np.minimum(np.floor(t).astype(int), K - 1)
    s = t - i0
    U = u_c.reshape(K + 1, K + 1)
    a = U[np.ix_(i0, i0)] * np.outer(1 - s, 1 - s) + U[np.ix_(i0, i0 + 1)] * np.outer(1 - s, s)
    b = U[np.ix_(i0 + 1, i0)] * np.outer(s, 1 - s) + U[np.ix_(i0 + 1, i0 + 1)] * np.outer(s, s)
    return a + b


def errors(U_ms, U_q1, U_f):
    nrm = np.linalg.norm(U_f)
    return np.linalg.norm(U_ms - U_f) / nrm, np.linalg.norm(U_q1 - U_f) / nrm


def test_oracle_msfem_against_fine_fem(pkg, oracle):
    """The chain on the oracle alone (CPU)."""
    W = pkg.workloads
    ms = oracle.run(W.reference_problem(2, 3, L), want_basis=True)
    u_c = oracle.coarse_solve(2, K, ms["M"], ms["F"], 0)
    w = weights(u_c, K)
    U_ms = fine_grid(np.einsum("ci,cik->ck", w, ms["basis"].reshape(K * K, 4, (N + 1) ** 2)))
    fine = oracle.run(W.reference_problem(2, 3 + L, 0))
    U_f = oracle.coarse_solve(2, KF, fine["M"], fine["F"], 0).reshape(KF + 1, KF + 1)
    q1 = oracle.run(W.reference_problem(2, 3, 0))
    U_q1 = coarse_q1_on_fine(oracle.coarse_solve(2, K, q1["M"], q1["F"], 0))
    e_ms, e_q1 = errors(U_ms, U_q1, U_f)
    assert e_ms < 0.01, e_ms
    assert e_ms < 0.1 * e_q1, (e_ms, e_q1)


@pytest.mark.gpu
def test_gpu_msfem_against_fine_fem(pkg, oracle, engine):
    """Every per-cell step on the GPU (MsFEM basis and M/F, the fine FEM's
    element matrices, the reconstruction); the two global solves on the host."""
    W = pkg.workloads
    ms = engine.run(W.reference_problem(2, 3, L), tol=1e-12, want_basis=True)
    assert ms["rc"] == 0
    u_c = oracle.coarse_solve(2, K, ms["M"], ms["F"], 0)
    U_ms = fine_grid(engine.reconstruct(W.reference_problem(2, 3, L), ms["basis"], weights(u_c, K)))
    fine = engine.run(W.reference_problem(2, 3 + L, 0), tol=1e-12)
    assert fine["rc"] == 0
    U_f = oracle.coarse_solve(2, KF, fine["M"], fine["F"], 0).reshape(KF + 1, KF + 1)
    q1 = engine.run(W.reference_problem(2, 3, 0), tol=1e-12)
    U_q1 = coarse_q1_on_fine(oracle.coarse_solve(2, K, q1["M"], q1["F"], 0))
    e_ms, e_q1 = errors(U_ms, U_q1, U_f)
    # the same numbers as the oracle's chain
    ref = oracle.run(W.reference_problem(2, 3 + L, 0))
    assert np.abs(fine["M"] - ref["M"]).max() < 1e-12 * np.abs(ref["M"]).max()
    assert e_ms < 0.01, e_ms
    assert e_ms < 0.1 * e_q1, (e_ms, e_q1)


def fem_lib(pkg):
    from test_host_mirror import host_lib

    lib = host_lib(pkg)
    vp = ctypes.c_void_p
    lib.msfem_host_fem_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int]
    lib.msfem_host_fem_run.restype = ctypes.c_int
    return lib


def test_standard_fem_component_is_exported(built):
    lib = fem_lib(built)
    assert hasattr(lib, "msfem_host_fem_run")


@pytest.mark.gpu
def test_host_standard_fem_component(pkg, oracle, tmp_path, monkeypatch):
    """DiffusionProblem<2> of the host library (the standard Q1 FEM the
    reference runs beside the MsFEM, diffusion_problem.tpp:336-377) on the
    128 x 128 fine mesh: its solution equals the oracle's fine FEM, it writes
    solution-std_2d_refinements-7.0000.vtu, and the host MsFEM's fine solution
    is within 1% of it."""
    from test_host_mirror import run_host

    monkeypatch.chdir(tmp_path)
    lib = fem_lib(pkg)
    W = pkg.workloads
    u = np.zeros((KF + 1) ** 2)
    params = np.zeros(8)
    rc = lib.msfem_host_fem_run(2, 3 + L, 0, ctypes.c_void_p(params.ctypes.data), 2.0, 0, 0, 0,
                                ctypes.c_void_p(u.ctypes.data), 1, 0)
    assert rc == 0
    fine = oracle.run(W.reference_problem(2, 3 + L, 0))
    U_f = oracle.coarse_solve(2, KF, fine["M"], fine["F"], 0)
    assert np.abs(u - U_f).max() < 1e-10 * np.abs(U_f).max()
    assert (tmp_path / f"solution-std_2d_refinements-{3 + L}.0000.vtu").exists()
    rc, msg, _, _, _, fine_ms = run_host(lib, 2, 3, L)
    assert rc == 0, msg
    U_ms = fine_grid(fine_ms)
    e_ms = np.linalg.norm(U_ms - u.reshape(KF + 1, KF + 1)) / np.linalg.norm(u)
    assert e_ms < 0.01, e_ms
