"""Python front-end of libmsfem_gpu.so: fills msfem_batch_desc from a problem
dict (see workloads.py) and calls the C-ABI.  The numerical work happens only
in the CUDA library; this module never computes a basis itself."""
import ctypes

import numpy as np

from . import _abi

PRECISION = {"fp64": _abi.PREC_FP64, "mixed": _abi.PREC_MIXED}


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Engine:
    """One handle = one GPU (reference: one MPI rank's DiffusionProblemBasis objects)."""

    def __init__(self, device=0, lib=None):
        self.lib = lib or _abi.load()
        h = ctypes.c_void_p()
        rc = self.lib.msfem_create(ctypes.byref(h), device)
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.msfem_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        """Launch on the caller's CUDA stream (0 / None: the handle's own
        non-blocking stream)."""
        rc = self.lib.msfem_set_stream(self.handle, ctypes.c_void_p(stream_handle or 0))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        self.stream_handle = stream_handle or 0

    def graph_info(self):
        """(captures, replays) of the handle's CUDA graph (msfem_graph_info)."""
        c, r = ctypes.c_int64(0), ctypes.c_int64(0)
        rc = self.lib.msfem_graph_info(self.handle, ctypes.byref(c), ctypes.byref(r))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return c.value, r.value

    # -- descriptor -------------------------------------------------------
    @staticmethod
    def make_desc(problem, precision="fp64", tol=1e-10, maxit=1000, check_interval=0,
                  warm_basis=None, memory=_abi.MEM_HOST, keep=None, tol_absolute=False):
        """msfem_batch_desc for host numpy data (memory=HOST).  `keep`
        collects the arrays whose buffers the descriptor points to.  The
        problem's optional "f_qp_values" / "f_qp_offset" tabulate f at the
        Gauss points; tol_absolute selects the reference's absolute stop."""
        keep = [] if keep is None else keep
        d = _abi.BatchDesc()
        d.dim = problem["dim"]
        corners = np.ascontiguousarray(problem["corners"], dtype=np.float64)
        keep.append(corners)
        d.n_cells = corners.shape[0]
        d.n_fine = int(problem.get("n_fine", 1))
        d.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        d.corners = _ptr(corners)
        if "n_fine_per_cell" in problem:
            nf = np.ascontiguousarray(problem["n_fine_per_cell"], dtype=np.int32)
            keep.append(nf)
            d.n_fine_per_cell = _ptr(nf)
        c = problem["coef"]
        d.coef.kind = int(c["kind"])
        d.coef.ncomp = int(c.get("ncomp", 0))
        for i, v in enumerate(c.get("params", [])):
            d.coef.params[i] = float(v)
        if c.get("qp_values") is not None:
            qv = np.ascontiguousarray(c["qp_values"], dtype=np.float64)
            keep.append(qv)
            d.coef.qp_values = _ptr(qv)
        if c.get("qp_offset") is not None:
            qo = np.ascontiguousarray(c["qp_offset"], dtype=np.int64)
            keep.append(qo)
            d.coef.qp_offset = _ptr(qo)
        if c.get("modes") is not None:
            md = np.ascontiguousarray(c["modes"], dtype=np.float64)
            keep.append(md)
            d.coef.modes = _ptr(md)
            d.coef.n_modes = md.shape[-2]
        if c.get("spheres") is not None:
            sp = np.ascontiguousarray(c["spheres"], dtype=np.float64)
            keep.append(sp)
            d.coef.spheres = _ptr(sp)
            d.coef.n_spheres = sp.shape[0]
        d.f_value = float(problem.get("f_value", 1.0))
        for key in ("f_qp_values", "f_qp_offset"):
            if problem.get(key) is not None:
                arr = np.ascontiguousarray(problem[key], dtype=np.int64 if key == "f_qp_offset" else np.float64)
                keep.append(arr)
                setattr(d, key, _ptr(arr))
        d.tol = float(tol)
        d.tol_absolute = int(bool(tol_absolute))
        d.maxit = int(maxit)
        d.memory = memory
        d.check_interval = int(check_interval)
        if warm_basis is not None:
            wb = np.ascontiguousarray(warm_basis, dtype=np.float64)
            keep.append(wb)
            d.warm_start = _abi.WARM_USER
            d.warm_basis = _ptr(wb)
        return d

    @staticmethod
    def basis_size(problem):
        dim = problem["dim"]
        nv = 1 << dim
        if "n_fine_per_cell" in problem:
            return int(np.sum(nv * (problem["n_fine_per_cell"].astype(np.int64) + 1) ** dim))
        return problem["corners"].shape[0] * nv * (problem["n_fine"] + 1) ** dim

    # -- calls --------------------------------------------------------------
    def run(self, problem, precision="fp64", tol=1e-10, maxit=1000, want_basis=False,
            warm_basis=None, check_interval=0, raise_on_failure=False, tol_absolute=False):
        keep = []
        d = self.make_desc(problem, precision, tol, maxit, check_interval, warm_basis, keep=keep,
                           tol_absolute=tol_absolute)
        nc, nv = d.n_cells, 1 << d.dim
        M = np.zeros((nc, nv, nv))
        F = np.zeros((nc, nv))
        status = np.zeros(nc, dtype=np.int32)
        iters = np.zeros((nc, nv), dtype=np.int32)
        basis = np.zeros(self.basis_size(problem)) if want_basis else None
        st = _abi.Stats()
        rc = self.lib.msfem_run_batch(self.handle, ctypes.byref(d), _ptr(M), _ptr(F), _ptr(basis),
                                      _ptr(status), _ptr(iters), ctypes.byref(st))
        if rc not in (_abi.OK, _abi.ERR_NOT_CONVERGED) or (raise_on_failure and rc != _abi.OK):
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return {"M": M, "F": F, "status": status, "iters": iters, "basis": basis,
                "stats": st.as_dict(), "rc": rc}

    def run_desc(self, desc, M, F, basis=None, status=None, iters=None, stats=True):
        """Raw call with caller-owned pointers (ints or None), e.g. device buffers."""
        st = _abi.Stats() if stats else None
        rc = self.lib.msfem_run_batch(self.handle, ctypes.byref(desc), M, F, basis, status, iters,
                                      ctypes.byref(st) if st is not None else None)
        if rc not in (_abi.OK, _abi.ERR_NOT_CONVERGED):
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return rc, (st.as_dict() if st is not None else None)

    def energy_error(self, problem, basis, basis_ref):
        """Per basis function ||phi_i - ref_i||_A and ||ref_i||_A (host arrays
        in the basis-output layout); returns (err, ref_norm) [n_cells][2^d]."""
        keep = []
        d = self.make_desc(problem, keep=keep)
        nc, nv = d.n_cells, 1 << d.dim
        a = np.ascontiguousarray(basis, dtype=np.float64)
        r = np.ascontiguousarray(basis_ref, dtype=np.float64)
        if a.size != self.basis_size(problem) or r.size != a.size:
            raise ValueError("basis arrays do not match the problem's basis layout")
        err = np.zeros((nc, nv))
        nrm = np.zeros((nc, nv))
        rc = self.lib.msfem_energy_error(self.handle, ctypes.byref(d), _ptr(a), _ptr(r), _ptr(err), _ptr(nrm))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return err, nrm

    def reconstruct(self, problem, basis, weights):
        """Fine solution u = sum_i w_i phi_i in every cell (msfem_reconstruct);
        basis in msfem_run_batch's layout, weights [n_cells][2^d]."""
        keep = []
        d = self.make_desc(problem, keep=keep)
        nv = 1 << d.dim
        b = np.ascontiguousarray(basis, dtype=np.float64).ravel()
        w = np.ascontiguousarray(weights, dtype=np.float64).ravel()
        assert b.size == self.basis_size(problem) and w.size == d.n_cells * nv
        u = np.zeros(b.size // nv)
        rc = self.lib.msfem_reconstruct(self.handle, ctypes.byref(d), _ptr(b), _ptr(w), _ptr(u))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return u

    def autotune(self, problem, precision="fp64", tol=1e-10, maxit=1000, sample_cells=1024):
        """Pick the fastest compiled launch shape / parameters for this
        problem's (dim, N class, precision); kept in the handle."""
        keep = []
        d = self.make_desc(problem, precision, tol, maxit, keep=keep)
        t = _abi.Tuning()
        rc = self.lib.msfem_autotune(self.handle, ctypes.byref(d), sample_cells, ctypes.byref(t))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return t.as_dict()

    def set_tuning(self, tuning):
        t = _abi.Tuning()
        for k, v in tuning.items():
            setattr(t, k, v)
        rc = self.lib.msfem_set_tuning(self.handle, ctypes.byref(t))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))

    def describe_tuning(self, tuning):
        """The compiled launch shape behind a tuning key and variant: its
        threads, strip height, occupancy, polynomial degree, cluster size and
        coarse spacing, and the number of shapes for the key."""
        t = _abi.Tuning()
        for k, v in tuning.items():
            setattr(t, k, v)
        rc = self.lib.msfem_describe_tuning(ctypes.byref(t))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return t.as_dict()

    def tabulate(self, problem, ncomp):
        keep = []
        d = self.make_desc(problem, keep=keep)
        size = self.lib.msfem_tabulated_size(ctypes.byref(d), ncomp)
        if size < 0:
            raise _abi.MsfemError(_abi.ERR_INVALID_ARG, "cannot size the tabulation")
        out = np.zeros(size)
        rc = self.lib.msfem_tabulate_coefficient(self.handle, ctypes.byref(d), ncomp, _ptr(out))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        return out
