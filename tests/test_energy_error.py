"""Energy-norm error of every basis function (msfem_energy_error) against the
CPU oracle's restatement: ||phi_i - ref_i||_A and ||ref_i||_A with A the
cell's fine stiffness over all nodes.

Bars: the two sides compute the same quadratic form on identical input
vectors, differing only in summation order, so the norms agree to 1e-9
relative (errors) and 1e-12 relative (reference norms); ||ref_i||_A^2 = M_ii
for a converged reference to 1e-12; identical inputs give exactly 0."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def assert_norms_match(got, ref, rtol):
    scale = np.maximum(np.abs(ref), 1e-300)
    assert np.all(np.isfinite(got))
    assert float((np.abs(got - ref) / scale).max()) < rtol


def check_against_oracle(engine, oracle, prob, basis, ref_basis):
    err, nrm = engine.energy_error(prob, basis, ref_basis)
    err_o, nrm_o = oracle.energy_norms(prob, basis, ref_basis)
    assert_norms_match(nrm, nrm_o, 1e-12)
    # errors are tiny differences; compare where they are above rounding of nrm
    live = err_o > 1e-13 * nrm_o
    assert np.all(np.abs(err - err_o) <= 1e-9 * err_o + 1e-14 * nrm_o)
    return err, nrm, live


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_energy_error_2d_against_oracle(pkg, oracle, engine, precision):
    """Random-Fourier tensor (fourier_square family, tabulated path), N = 32: the
    GPU basis solved to 1e-10 against the oracle's direct solve."""
    W = pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), [0, 17, 2080, 4095])
    got = engine.run(prob, precision=precision, tol=1e-10, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    err, nrm, live = check_against_oracle(engine, oracle, prob, got["basis"], ref["basis"])
    assert live.any()
    # 1e-10 relative residual bounds the relative energy error well below 1e-7
    assert float((err / nrm).max()) < 1e-7
    # converged reference: ||ref_i||_A^2 = M_ii
    Mii = np.diagonal(ref["M"], axis1=1, axis2=2)
    assert float(np.abs(nrm ** 2 - Mii).max() / np.abs(Mii).max()) < 1e-12


def test_energy_error_reference_coefficient_and_identity(pkg, oracle, engine):
    prob = pkg.workloads.reference_problem(2, 2, 4)
    ref = oracle.run(prob, want_basis=True)
    err, nrm = engine.energy_error(prob, ref["basis"], ref["basis"])
    assert np.all(err == 0.0)
    Mii = np.diagonal(ref["M"], axis1=1, axis2=2)
    assert float(np.abs(nrm ** 2 - Mii).max() / np.abs(Mii).max()) < 1e-12


def test_energy_error_known_perturbation(pkg, oracle, engine):
    """phi + t * bump: the error is |t| ||bump||_A exactly (same quadratic form)."""
    W = pkg.workloads
    prob = W.problem(2, W.unit_cube_corners(2, 2), 8, {"kind": 0, "params": [2.0, 0.3, 1.0]})
    ref = oracle.run(prob, want_basis=True)
    rng = np.random.default_rng(3)
    bump = rng.standard_normal(ref["basis"].size) * 1e-3
    err, nrm = engine.energy_error(prob, ref["basis"] + bump, ref["basis"])
    err_o, _ = oracle.energy_norms(prob, ref["basis"] + bump, ref["basis"])
    assert_norms_match(err, err_o, 1e-10)


@pytest.mark.parametrize("geom", ["parallelogram", "bilinear"])
def test_energy_error_general_geometry(pkg, oracle, engine, geom):
    W = pkg.workloads
    c = W.unit_cube_corners(2, 2) * 0.8 + 0.05
    if geom == "parallelogram":
        c = c + c[:, :, 1:2] * np.array([0.2, 0.0])
    else:
        c = c + np.random.default_rng(7).uniform(-0.01, 0.01, size=c.shape)
    prob = W.problem(2, c, 10, {"kind": 1}, f_value=2.0)
    got = engine.run(prob, precision="mixed", tol=1e-9, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check_against_oracle(engine, oracle, prob, got["basis"], ref["basis"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_energy_error_3d_uneven_spheres(pkg, oracle, engine, precision):
    """1e4-contrast spheres, uneven N in one call."""
    W = pkg.workloads
    rng = np.random.default_rng(5)
    sp = np.column_stack([rng.uniform(0, 1, (600, 3)), rng.uniform(0.02, 0.05, 600)])
    corners = W.unit_cube_corners(3, 4)[[0, 5, 21, 42]]
    nf = np.array([8, 4, 6, 3], dtype=np.int32)
    prob = W.problem(3, corners, nf, {"kind": 4, "params": [1e4], "spheres": sp})
    got = engine.run(prob, precision=precision, tol=1e-10, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    err, nrm, _ = check_against_oracle(engine, oracle, prob, got["basis"], ref["basis"])
    Mii = np.diagonal(ref["M"], axis1=1, axis2=2)
    assert float(np.abs(nrm ** 2 - Mii).max() / np.abs(Mii).max()) < 1e-11
    assert float((err / nrm).max()) < 1e-6


def test_energy_error_3d_reference_coefficient(pkg, oracle, engine):
    prob = pkg.workloads.reference_problem(3, 1, 2)
    got = engine.run(prob, precision="fp64", tol=1e-10, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    check_against_oracle(engine, oracle, prob, got["basis"], ref["basis"])


def test_energy_error_device_memory(pkg, oracle, engine):
    """DEVICE memory mode: torch device buffers, asynchronous call."""
    import ctypes

    import torch

    W = pkg.workloads
    abi = pkg._abi
    prob = W.subset(W.fourier_square(K=64, N=32), [3, 9])
    got = engine.run(prob, precision="mixed", tol=1e-10, want_basis=True)
    ref = oracle.run(prob, want_basis=True)
    err_h, nrm_h = engine.energy_error(prob, got["basis"], ref["basis"])
    keep = []
    d = engine.make_desc(prob, keep=keep)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (prob["corners"],)]
    d.corners = dev[0].data_ptr()
    # tabulated coefficient on the device
    size = engine.lib.msfem_tabulated_size(ctypes.byref(d), 3)
    tab = torch.from_numpy(engine.tabulate(prob, 3)).cuda()
    assert tab.numel() == size
    d.coef.kind = abi.COEF_TABULATED
    d.coef.ncomp = 3
    d.coef.qp_values = tab.data_ptr()
    d.memory = abi.MEM_DEVICE
    a = torch.from_numpy(got["basis"]).cuda()
    r = torch.from_numpy(ref["basis"]).cuda()
    err = torch.empty((2, 4), dtype=torch.float64, device="cuda")
    nrm = torch.empty((2, 4), dtype=torch.float64, device="cuda")
    rc = engine.lib.msfem_energy_error(engine.handle, ctypes.byref(d), a.data_ptr(), r.data_ptr(),
                                       err.data_ptr(), nrm.data_ptr())
    assert rc == abi.OK
    torch.cuda.synchronize()
    assert np.allclose(err.cpu().numpy(), err_h, rtol=1e-12, atol=0)
    assert np.allclose(nrm.cpu().numpy(), nrm_h, rtol=1e-14, atol=0)
