"""The C++ mirror of the reference's DiffusionProblemBasis / coefficient
classes, driven by a replay of DiffusionProblemMultiscale::run
(include/base/diffusion_problem_ms.tpp:445-491): the final coarse solution,
the coarse element matrices and the reconstructed fine solution must match
the oracle's restatement of the whole chain."""
import ctypes
import os

import numpy as np
import pytest


def host_lib(pkg):
    lib = ctypes.CDLL(os.path.join(pkg.build.LIB_DIR, "libmsfem_host.so"))
    vp = ctypes.c_void_p
    lib.msfem_host_ms_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      vp, vp, vp, vp, ctypes.c_int, ctypes.c_int]
    lib.msfem_host_ms_run.restype = ctypes.c_int
    lib.msfem_host_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    return lib


OPT_RELATIVE_TOL, OPT_LINEAR_RHS, OPT_OUTPUT_BASIS = 1, 2, 4


def run_host(lib, dim, n_refine, n_refine_local, coef=0, params=(0.0,) * 8, f=2.0, bc=0, precision=0,
             write_vtu=0, options=0):
    K = 1 << n_refine
    N = 1 << n_refine_local
    nv = 1 << dim
    nc = K ** dim
    u = np.zeros((K + 1) ** dim)
    M = np.zeros((nc, nv, nv))
    F = np.zeros((nc, nv))
    fine = np.zeros((nc, (N + 1) ** dim))
    pr = np.ascontiguousarray(params, dtype=np.float64)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = lib.msfem_host_ms_run(dim, n_refine, n_refine_local, coef, p(pr), f, bc, precision, 0,
                               p(u), p(M), p(F), p(fine), write_vtu, options)
    buf = ctypes.create_string_buffer(512)
    lib.msfem_host_last_error(buf, 512)
    return rc, buf.value.decode(), u, M, F, fine


def test_host_library_builds_and_exports(built):
    lib = host_lib(built)
    assert hasattr(lib, "msfem_host_ms_run")


def test_host_library_reports_missing_gpu(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc, msg, *_ = run_host(host_lib(built), 2, 1, 2)
    assert rc != 0 and "msfem_create" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_reference_driver_coarse_solution_parity(pkg, oracle, precision, tmp_path, monkeypatch):
    """The reference's own problem (MatrixCoeff, f = 2, Dirichlet on ids 0/2/4,
    Neumann on 1/3/5) at n_refine = 3, n_refine_local = 4."""
    monkeypatch.chdir(tmp_path)
    lib = host_lib(pkg)
    rc, msg, u, M, F, fine = run_host(lib, 2, 3, 4, precision=precision, write_vtu=1)
    assert rc == 0, msg
    prob = pkg.workloads.reference_problem(2, 3, 4)
    ref = oracle.run(prob, want_basis=True)
    assert np.abs(M - ref["M"]).max() < 1e-10 * np.abs(ref["M"]).max()
    assert np.abs(F - ref["F"]).max() < 1e-10 * np.abs(ref["F"]).max()
    u_ref = oracle.coarse_solve(2, 8, ref["M"], ref["F"], 0)
    assert np.abs(u - u_ref).max() < 1e-10 * np.abs(u_ref).max()
    # fine solution in cell c = sum_i w_i phi_i (set_global_weights)
    K, n = 8, 17
    basis = ref["basis"].reshape(64, 4, n * n)
    for c in (0, 9, 63):
        cx, cy = c % K, c // K
        w = np.array([u_ref[(cy + (i >> 1)) * (K + 1) + cx + (i & 1)] for i in range(4)])
        assert np.abs(fine[c] - w @ basis[c]).max() < 1e-9
    vtu = list(tmp_path.glob("solution-ms_fine-2d.00000.cell-0_0:.vtu"))
    assert vtu and "UnstructuredGrid" in vtu[0].read_text()[:200]


@pytest.mark.gpu
def test_value_list_tabulation_path_homogeneous(pkg, oracle):
    """A coefficient class without a device description goes through
    value_list tabulation; a = diag(3, 0.5) has the closed-form Q1 answer."""
    lib = host_lib(pkg)
    rc, msg, u, M, F, _ = run_host(lib, 2, 2, 3, coef=2, params=(3.0, 0.0, 0.5, 0, 0, 0, 0, 0),
                                   f=1.0, bc=1)
    assert rc == 0, msg
    H = 0.25
    K1 = np.array([[1.0, -1.0], [-1.0, 1.0]]) / H
    M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) * H / 6.0
    exact = 3.0 * np.kron(M1, K1) + 0.5 * np.kron(K1, M1)
    assert np.abs(M - exact).max() < 1e-11
    u_ref = oracle.coarse_solve(2, 4, M, F, 1)
    assert np.abs(u - u_ref).max() < 1e-12


@pytest.mark.gpu
def test_reference_driver_3d(pkg, oracle):
    lib = host_lib(pkg)
    rc, msg, u, M, F, _ = run_host(lib, 3, 1, 2)
    assert rc == 0, msg
    prob = pkg.workloads.reference_problem(3, 1, 2)
    ref = oracle.run(prob)
    assert np.abs(M - ref["M"]).max() < 1e-10 * np.abs(ref["M"]).max()
    u_ref = oracle.coarse_solve(3, 2, ref["M"], ref["F"], 0)
    assert np.abs(u - u_ref).max() < 1e-10 * max(1.0, np.abs(u_ref).max())


@pytest.mark.gpu
def test_output_flag_writes_basis_vtu(pkg, oracle, tmp_path, monkeypatch):
    """set_output_flag(true) writes the cell's basis functions as the
    reference's output_basis does (diffusion_problem_basis.tpp:392-418):
    "2d-basis.<subdomain>.cell-<id>.vtu" with point data basis_0 .. basis_3."""
    monkeypatch.chdir(tmp_path)
    lib = host_lib(pkg)
    rc, msg, *_ = run_host(lib, 2, 2, 3, options=OPT_OUTPUT_BASIS)
    assert rc == 0, msg
    files = sorted(p.name for p in tmp_path.glob("2d-basis.*.vtu"))
    assert files == ["2d-basis.4294967295.cell-0_0:.vtu"], files
    text = (tmp_path / files[0]).read_text()
    ref = oracle.run(pkg.workloads.reference_problem(2, 2, 3), want_basis=True)
    nodes = 9 * 9
    basis0 = ref["basis"].reshape(16, 4, nodes)[0]
    for i in range(4):
        head = f'Name="basis_{i}" format="ascii">'
        assert head in text
        vals = np.array(text.split(head, 1)[1].split("</DataArray>", 1)[0].split(), dtype=float)
        assert vals.shape == (nodes,)
        assert np.abs(vals - basis0[i]).max() < 1e-10


@pytest.mark.gpu
def test_right_hand_side_function_and_tolerance_modes(pkg, oracle):
    """A RightHandSide without a constant value (f = 2 + x) goes through
    value_list at the Gauss points; both stopping rules (the reference's
    absolute 1e-12, and relative 1e-12) give the oracle's coarse solution."""
    lib = host_lib(pkg)
    W = pkg.workloads
    prob = W.with_rhs(W.reference_problem(2, 3, 4), lambda x: 2.0 + x[..., 0])
    ref = oracle.run(prob)
    u_ref = oracle.coarse_solve(2, 8, ref["M"], ref["F"], 0)
    for opts in (OPT_LINEAR_RHS, OPT_LINEAR_RHS | OPT_RELATIVE_TOL):
        rc, msg, u, M, F, _ = run_host(lib, 2, 3, 4, options=opts)
        assert rc == 0, msg
        assert np.abs(F - ref["F"]).max() < 1e-10 * np.abs(ref["F"]).max()
        assert np.abs(M - ref["M"]).max() < 1e-10 * np.abs(ref["M"]).max()
        assert np.abs(u - u_ref).max() < 1e-10 * np.abs(u_ref).max()
