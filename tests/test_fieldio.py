"""The on-disk coefficient-field format: a round trip keeps the mesh, N and
every Gauss-point value bit for bit, the loaded field runs through the
oracle (CPU) and the CUDA path (GPU) to the same answers as the field it was
written from, and malformed files are rejected."""
import numpy as np
import pytest


def _field(pkg, oracle, uneven):
    W = pkg.workloads
    if uneven:
        corners = W.unit_cube_corners(2, 4)[[0, 3, 9, 14]]
        prob = W.problem(2, corners, np.array([4, 8, 2, 6], dtype=np.int32), {"kind": 2, "params": [0.9, 0.25]})
    else:
        prob = W.subset(W.fourier_square(K=64, N=32), [0, 77, 4095])
        prob = dict(prob)
        prob["n_fine"] = 8  # small N keeps the oracle fast
    return prob, oracle.tabulate(prob, 3)


@pytest.mark.parametrize("uneven", [False, True])
def test_round_trip_and_oracle(pkg, oracle, tmp_path, uneven):
    F = pkg.fieldio
    prob, tab = _field(pkg, oracle, uneven)
    path = tmp_path / "field.msfield"
    F.save_field(path, prob, tab, 3)
    got = F.load_field(path)
    assert np.array_equal(got["corners"], prob["corners"])
    assert np.array_equal(np.asarray(got["coef"]["qp_values"]), tab)
    if uneven:
        assert np.array_equal(got["n_fine_per_cell"], prob["n_fine_per_cell"])
    else:
        assert got["n_fine"] == prob["n_fine"]
    tprob = dict(prob)
    tprob["coef"] = {"kind": pkg._abi.COEF_TABULATED, "ncomp": 3, "qp_values": tab}
    a = oracle.run(tprob)
    b = oracle.run(got)
    assert np.array_equal(a["M"], b["M"]) and np.array_equal(a["F"], b["F"])


def test_malformed_files_are_rejected(pkg, oracle, tmp_path):
    F = pkg.fieldio
    prob, tab = _field(pkg, oracle, False)
    with pytest.raises(ValueError):
        F.save_field(tmp_path / "x", prob, tab[:-1], 3)
    bad = tmp_path / "bad.msfield"
    bad.write_bytes(b"NOTAFILE" + bytes(56))
    with pytest.raises(ValueError):
        F.load_field(bad)
    good = tmp_path / "good.msfield"
    F.save_field(good, prob, tab, 3)
    cut = tmp_path / "cut.msfield"
    cut.write_bytes(good.read_bytes()[:-8])
    with pytest.raises(ValueError):
        F.load_field(cut, mmap=False)


@pytest.mark.gpu
def test_loaded_field_on_the_gpu(pkg, oracle, engine, tmp_path):
    prob, tab = _field(pkg, oracle, True)
    path = tmp_path / "field.msfield"
    pkg.fieldio.save_field(path, prob, tab, 3)
    got = engine.run(pkg.fieldio.load_field(path), tol=1e-12)
    ref = oracle.run(pkg.fieldio.load_field(path))
    assert got["rc"] == 0
    assert np.abs(got["M"] - ref["M"]).max() < 1e-10 * np.abs(ref["M"]).max()


def test_round_trip_3d_scalar(pkg, oracle, tmp_path):
    """A 3D uneven-N scalar field (the sphere workload's layout, ncomp = 1)."""
    W, F = pkg.workloads, pkg.fieldio
    rng = np.random.default_rng(3)
    sp = np.column_stack([rng.uniform(0, 1, (50, 3)), rng.uniform(0.05, 0.1, 50)])
    prob = W.problem(3, W.unit_cube_corners(3, 2)[:3], np.array([2, 4, 3], dtype=np.int32),
                     {"kind": 4, "params": [1e4], "spheres": sp})
    tab = oracle.tabulate(prob, 1)
    path = tmp_path / "f3.msfield"
    F.save_field(path, prob, tab, 1)
    got = F.load_field(path, mmap=False)
    assert got["dim"] == 3 and got["coef"]["ncomp"] == 1
    assert np.array_equal(got["coef"]["qp_values"], tab)
    assert np.array_equal(got["n_fine_per_cell"], prob["n_fine_per_cell"])
    a = oracle.run(dict(prob, coef={"kind": pkg._abi.COEF_TABULATED, "ncomp": 1, "qp_values": tab}))
    b = oracle.run(got)
    assert np.array_equal(a["M"], b["M"])
