"""ctypes wrapper of the CPU FP64 oracle (oracle/msfem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline / reference arm.  The product
library never uses it.  Parity status: unpinned against reference outputs
(the reference cannot be built here and ships no golden vectors); pinned
against analytic known answers, see msfem_oracle.h.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmsfem_oracle.so")
SRC = os.path.join(_HERE, "msfem_oracle.c")

SOLVER_DIRECT = 0
SOLVER_SSOR_CG = 1
SOLVER_JACOBI_CG = 2
ORDER_LEX = 0
ORDER_DEALII = 1
COEF_TABULATED = 5  # OC_COEF_TABULATED (msfem_oracle.h), = MSFEM_COEF_TABULATED


class OcCoef(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("ncomp", ctypes.c_int32),
        ("params", ctypes.c_double * 8),
        ("qp_values", ctypes.c_void_p),
        ("qp_offset", ctypes.c_void_p),
        ("modes", ctypes.c_void_p),
        ("n_modes", ctypes.c_int32),
        ("n_spheres", ctypes.c_int32),
        ("spheres", ctypes.c_void_p),
    ]


class OcBatch(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("n_cells", ctypes.c_int32),
        ("n_fine", ctypes.c_int32),
        ("solver", ctypes.c_int32),
        ("corners", ctypes.c_void_p),
        ("n_fine_per_cell", ctypes.c_void_p),
        ("coef", OcCoef),
        ("f_value", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("tol_absolute", ctypes.c_int32),
        ("maxit", ctypes.c_int32),
        ("omega", ctypes.c_double),
        ("ordering", ctypes.c_int32),
        ("nthreads", ctypes.c_int32),
        ("raw_monomials", ctypes.c_int32),
        ("f_qp_values", ctypes.c_void_p),
        ("f_qp_offset", ctypes.c_void_p),
    ]


def build(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    stale = force or not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(f) > os.path.getmtime(LIB_PATH)
        for f in (SRC, os.path.join(_HERE, "msfem_oracle.h")))
    if stale:
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", LIB_PATH + ".tmp",
               SRC, "-lm"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + res.stderr)
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        lib.oc_run_batch.argtypes = [ctypes.POINTER(OcBatch), vp, vp, vp, vp, vp]
        lib.oc_run_batch.restype = ctypes.c_int
        lib.oc_assemble_cell.argtypes = [ctypes.POINTER(OcBatch), ctypes.c_int32, vp, vp]
        lib.oc_assemble_cell.restype = ctypes.c_int
        lib.oc_basis_q1.argtypes = [ctypes.POINTER(OcBatch), ctypes.c_int32, vp, vp]
        lib.oc_basis_q1.restype = None
        lib.oc_coef_eval.argtypes = [ctypes.POINTER(OcBatch), ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_int32, vp, vp]
        lib.oc_coef_eval.restype = None
        lib.oc_tabulate.argtypes = [ctypes.POINTER(OcBatch), ctypes.c_int32, vp]
        lib.oc_tabulate.restype = ctypes.c_int
        lib.oc_coarse_solve.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int32, vp]
        lib.oc_coarse_solve.restype = ctypes.c_int
        lib.oc_unit_cube_corners.argtypes = [ctypes.c_int32, ctypes.c_int32, vp]
        lib.oc_unit_cube_corners.restype = None
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def make_batch(problem, solver=SOLVER_DIRECT, tol=1e-12, tol_absolute=False, maxit=1000,
               omega=1.6, ordering=ORDER_LEX, nthreads=1, raw_monomials=False, keep=None):
    keep = [] if keep is None else keep
    b = OcBatch()
    b.dim = problem["dim"]
    corners = np.ascontiguousarray(problem["corners"], dtype=np.float64)
    keep.append(corners)
    b.n_cells = corners.shape[0]
    b.n_fine = int(problem.get("n_fine", 1))
    b.solver = solver
    b.corners = _p(corners)
    if "n_fine_per_cell" in problem:
        nf = np.ascontiguousarray(problem["n_fine_per_cell"], dtype=np.int32)
        keep.append(nf)
        b.n_fine_per_cell = _p(nf)
    c = problem["coef"]
    if (int(c["kind"]) == COEF_TABULATED and c.get("qp_offset") is None and "n_fine_per_cell" in problem):
        # uneven N without offsets: packed cell blocks of ncomp 2^d N_c^d
        # values in cell order (the layout the library reads and writes)
        nfc = np.asarray(problem["n_fine_per_cell"], dtype=np.int64) ** b.dim
        blocks = int(c.get("ncomp", 1)) * (1 << b.dim) * nfc
        c = dict(c)
        c["qp_offset"] = np.concatenate([[0], np.cumsum(blocks)[:-1]]).astype(np.int64)
    b.coef.kind = int(c["kind"])
    b.coef.ncomp = int(c.get("ncomp", 0))
    for i, v in enumerate(c.get("params", [])):
        b.coef.params[i] = float(v)
    for key, field in (("qp_values", "qp_values"), ("qp_offset", "qp_offset"),
                       ("modes", "modes"), ("spheres", "spheres")):
        if c.get(key) is not None:
            arr = np.ascontiguousarray(c[key], dtype=np.int64 if key == "qp_offset" else np.float64)
            keep.append(arr)
            setattr(b.coef, field, _p(arr))
            if key == "modes":
                b.coef.n_modes = arr.shape[-2]
            if key == "spheres":
                b.coef.n_spheres = arr.shape[0]
    b.f_value = float(problem.get("f_value", 1.0))
    fprob = problem
    if problem.get("f_qp_values") is not None and problem.get("f_qp_offset") is None:
        # packed cell blocks of 2^d N_c^d values: explicit offsets
        nfc = (np.asarray(problem["n_fine_per_cell"], dtype=np.int64) if "n_fine_per_cell" in problem
               else np.full(b.n_cells, b.n_fine, dtype=np.int64)) ** b.dim
        fprob = dict(problem)
        fprob["f_qp_offset"] = np.concatenate([[0], np.cumsum((1 << b.dim) * nfc)[:-1]]).astype(np.int64)
    for key in ("f_qp_values", "f_qp_offset"):
        if fprob.get(key) is not None:
            arr = np.ascontiguousarray(fprob[key], dtype=np.int64 if key == "f_qp_offset" else np.float64)
            keep.append(arr)
            setattr(b, key, _p(arr))
    b.tol = float(tol)
    b.tol_absolute = int(bool(tol_absolute))
    b.maxit = int(maxit)
    b.omega = float(omega)
    b.ordering = int(ordering)
    b.nthreads = int(nthreads)
    b.raw_monomials = int(bool(raw_monomials))
    return b


def basis_size(problem):
    dim = problem["dim"]
    nv = 1 << dim
    if "n_fine_per_cell" in problem:
        return int(np.sum(nv * (problem["n_fine_per_cell"].astype(np.int64) + 1) ** dim))
    return problem["corners"].shape[0] * nv * (problem["n_fine"] + 1) ** dim


def run(problem, solver=SOLVER_DIRECT, want_basis=False, **kw):
    """Whole batch on the CPU.  Returns dict(M, F, basis, iters, rel_res, nfail)."""
    keep = []
    b = make_batch(problem, solver=solver, keep=keep, **kw)
    nc, nv = b.n_cells, 1 << b.dim
    M = np.zeros((nc, nv, nv))
    F = np.zeros((nc, nv))
    iters = np.zeros((nc, nv), dtype=np.int32)
    rel = np.zeros((nc, nv))
    basis = np.zeros(basis_size(problem)) if want_basis else None
    nfail = load().oc_run_batch(ctypes.byref(b), _p(M), _p(F), _p(basis), _p(iters), _p(rel))
    return {"M": M, "F": F, "basis": basis, "iters": iters, "rel_res": rel, "nfail": nfail}


def assemble_cell(problem, cell=0):
    keep = []
    b = make_batch(problem, keep=keep)
    N = int(problem["n_fine_per_cell"][cell]) if "n_fine_per_cell" in problem else b.n_fine
    nn, ns = (N + 1) ** b.dim, 3 ** b.dim
    st = np.zeros((nn, ns))
    bl = np.zeros(nn)
    load().oc_assemble_cell(ctypes.byref(b), cell, _p(st), _p(bl))
    return st, bl


def energy_norms(problem, basis, basis_ref):
    """Per cell and basis function ||phi_i - ref_i||_A and ||ref_i||_A with A
    the oracle's own assembled fine stiffness over all nodes (the
    unconstrained diffusion_matrix, diffusion_problem_basis.tpp:159-242);
    bases in the basis-output layout.  Returns (err, ref_norm) [n][2^d]."""
    dim = problem["dim"]
    nv = 1 << dim
    nc = problem["corners"].shape[0]
    err = np.zeros((nc, nv))
    nrm = np.zeros((nc, nv))
    off = 0
    for c in range(nc):
        N = int(problem["n_fine_per_cell"][c]) if "n_fine_per_cell" in problem else int(problem["n_fine"])
        n = N + 1
        nn = n ** dim
        st, _ = assemble_cell(problem, c)
        shape = (n,) * dim  # [z][y][x] (x fastest)
        for i in range(nv):
            a = np.asarray(basis[off + i * nn: off + (i + 1) * nn])
            r = np.asarray(basis_ref[off + i * nn: off + (i + 1) * nn])
            for vec, out in ((a - r, err), (r, nrm)):
                v = vec.reshape(shape)
                vp = np.pad(v, 1)
                y = np.zeros(nn)
                for s_ in range(3 ** dim):
                    o = [(s_ // 3 ** k) % 3 - 1 for k in range(dim)]  # (ox, oy, oz)
                    sl = tuple(slice(1 + o[dim - 1 - ax], 1 + o[dim - 1 - ax] + n) for ax in range(dim))
                    y += st[:, s_] * vp[sl].ravel()
                out[c, i] = np.sqrt(max(float(vec @ y), 0.0))
        off += nv * nn
    return err, nrm


def basis_q1(problem, cell, x, raw_monomials=False):
    keep = []
    b = make_batch(problem, keep=keep, raw_monomials=raw_monomials)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(1 << b.dim)
    load().oc_basis_q1(ctypes.byref(b), cell, _p(xx), _p(out))
    return out


def tabulate(problem, ncomp):
    keep = []
    b = make_batch(problem, keep=keep)
    dim = problem["dim"]
    nq = 1 << dim
    if "n_fine_per_cell" in problem:
        size = int(np.sum(ncomp * nq * problem["n_fine_per_cell"].astype(np.int64) ** dim))
    else:
        size = b.n_cells * ncomp * nq * b.n_fine ** dim
    out = np.zeros(size)
    load().oc_tabulate(ctypes.byref(b), ncomp, _p(out))
    return out


def coarse_solve(dim, K, M, F, bc):
    u = np.zeros((K + 1) ** dim)
    Mc = np.ascontiguousarray(M, dtype=np.float64)
    Fc = np.ascontiguousarray(F, dtype=np.float64)
    rc = load().oc_coarse_solve(dim, K, _p(Mc), _p(Fc), bc, _p(u))
    if rc != 0:
        raise RuntimeError(f"coarse solve failed ({rc})")
    return u
