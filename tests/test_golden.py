"""Committed golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py from the FP64 oracle's direct solves).

CPU: the input generators still produce the fingerprinted inputs, the oracle
reproduces the fixtures (1e-12 relative: the fixtures may come from another
host's compiler), and the fixtures satisfy the structural invariants.
GPU: the CUDA path through the C-ABI reproduces them at the parity bars
(M, F 1e-10 relative; basis values 1e-9 absolute; coarse solution 1e-10)."""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
with open(os.path.join(HERE, "index.json")) as _f:
    INDEX = json.load(_f)
NAMES = sorted(INDEX)


def load_case(name):
    return dict(np.load(os.path.join(HERE, f"{name}.npz")))


def problem_of(pkg, name):
    W = pkg.workloads
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.cases(W)[name], mg


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


@pytest.mark.parametrize("name", NAMES)
def test_inputs_are_reproduced(pkg, name):
    (prob, _), _ = problem_of(pkg, name)
    meta = INDEX[name]
    assert sha(prob["corners"]) == meta["corners_sha256"]
    if "modes_sha256" in meta:
        assert sha(prob["coef"]["modes"]) == meta["modes_sha256"]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(pkg, oracle, name):
    (prob, coarse), mg = problem_of(pkg, name)
    g = load_case(name)
    ref = oracle.run(prob, want_basis=True)
    assert rel(ref["M"], g["M"]) < 1e-12
    assert rel(ref["F"], g["F"]) < 1e-12
    bp = mg.basis_prefix(prob, ref["basis"], INDEX[name]["basis_cells"])
    assert np.abs(bp - g["basis_prefix"]).max() < 1e-12
    if coarse is not None:
        dim, K, bc = coarse
        u = oracle.coarse_solve(dim, K, g["M"], g["F"], bc)
        assert rel(u, g["u"]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_golden_invariants(name):
    g = load_case(name)
    M = g["M"]
    scale = np.abs(M).max(axis=(1, 2))
    assert np.all(np.abs(M - np.transpose(M, (0, 2, 1))).max(axis=(1, 2)) <= 1e-13 * scale)
    # partition of unity: constants are in the kernel of every element matrix
    assert np.all(np.abs(M.sum(axis=2)).max(axis=1) <= 1e-11 * scale)
    assert np.all(np.linalg.eigvalsh(M)[:, 0] >= -1e-11 * scale)
    assert np.all(g["F"] > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(pkg, oracle, engine, name, precision):
    (prob, coarse), mg = problem_of(pkg, name)
    g = load_case(name)
    got = engine.run(prob, precision=precision, tol=1e-13, want_basis=True)
    assert got["rc"] == 0 and np.all(got["status"] == 0)
    assert rel(got["M"], g["M"]) < 1e-10
    assert rel(got["F"], g["F"]) < 1e-10
    bp = mg.basis_prefix(prob, got["basis"], INDEX[name]["basis_cells"])
    assert np.abs(bp - g["basis_prefix"]).max() < 1e-9
    if coarse is not None:
        dim, K, bc = coarse
        u = oracle.coarse_solve(dim, K, got["M"], got["F"], bc)
        assert rel(u, g["u"]) < 1e-10
