"""Problem descriptions: coarse meshes, coefficient fields and the benchmark
workloads, as plain numpy data.

A problem is a dict:
  dim, corners [n_cells, 2^d, d] float64, n_fine (int) or n_fine_per_cell
  [n_cells] int32, coef (dict: kind, params, ncomp, qp_values, modes,
  spheres), f_value.

The coarse mesh of the reference's driver is GridGenerator::hyper_cube(0, 1)
refined n_refine times (include/base/diffusion_problem_ms.tpp:97-99); its
active cells are listed here lexicographically (x fastest), each with its
2^d corners in deal.II vertex order.  Random fields use a portable SplitMix64
generator so every machine draws the same coefficients.
"""
import math

import numpy as np

from . import _abi

MASK64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014) with Box-Muller normals."""

    def __init__(self, seed):
        self.state = seed & MASK64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def normal(self):
        u1 = max(self.uniform(), 1e-300)
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def unit_cube_corners(dim, K):
    """Corners [K^d, 2^d, d] of the K^d cells of [0,1]^d, cells lexicographic."""
    nv = 1 << dim
    idx = np.indices((K,) * dim).reshape(dim, -1)[::-1].T  # (cx, cy[, cz]), x fastest
    verts = np.array([[(v >> a) & 1 for a in range(dim)] for v in range(nv)], dtype=np.float64)
    return ((idx[:, None, :] + verts[None, :, :]) / K).astype(np.float64)


def fourier_modes(seed, n_modes=64, kmax=128 * math.pi, variance=1.0 / 64, dim=2):
    """Modes (kx, ky, kz, amp, phase): wavevector uniform in the disc/ball
    |k| <= kmax, amplitude N(0, variance), phase U[0, 2 pi)."""
    rng = SplitMix64(seed)
    out = np.zeros((n_modes, 5))
    sd = math.sqrt(variance)
    for m in range(n_modes):
        if dim == 2:
            r = kmax * math.sqrt(rng.uniform())
            ph = 2 * math.pi * rng.uniform()
            k = (r * math.cos(ph), r * math.sin(ph), 0.0)
        else:
            while True:
                k = tuple(kmax * (2 * rng.uniform() - 1) for _ in range(3))
                if k[0] ** 2 + k[1] ** 2 + k[2] ** 2 <= kmax * kmax:
                    break
        out[m, :3] = k
        out[m, 3] = sd * rng.normal()
        out[m, 4] = 2 * math.pi * rng.uniform()
    return out


def fourier_coef(seeds, dim=2, n_modes=64, kmax=128 * math.pi, variance=1.0 / 64):
    """Random SPD tensor A = R(theta) diag(e^g1, e^g2) R(theta)^T (2D, seeds for
    g1, g2, theta) or log-normal scalar e^g1 (3D, one seed)."""
    tables = [fourier_modes(s, n_modes, kmax, variance, dim) for s in seeds]
    return {"kind": _abi.COEF_FOURIER, "modes": np.ascontiguousarray(np.stack(tables)),
            "n_modes": n_modes}


_fields_lib = None


def _fields():
    """libmsfem_fields.so (built by build.build_fields)."""
    global _fields_lib
    if _fields_lib is None:
        import ctypes
        import os

        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libmsfem_fields.so")
        if not os.path.exists(path):
            raise OSError(f"libmsfem_fields.so not found at {path}: run build() first")
        lib = ctypes.CDLL(path)
        lib.msfem_spheres_rsa.argtypes = [ctypes.c_uint64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.POINTER(ctypes.c_int64)]
        lib.msfem_spheres_rsa.restype = ctypes.c_int
        _fields_lib = lib
    return _fields_lib


def spheres_rsa(seed, rmin=0.004, rmax=0.012, fraction=0.2, dim=3, max_tries=10_000_000):
    """Random sequential addition of non-overlapping spheres (discs in 2D) with
    radius U[rmin, rmax], centres U[0,1]^d, until the summed volume reaches
    `fraction` of the unit cube (msfem_spheres_rsa of libmsfem_fields.so).
    Returns [n, 4] (cx, cy, cz, r)."""
    import ctypes

    lib = _fields()
    n = ctypes.c_int64(0)
    cap = 1 << 16
    while True:
        out = np.zeros((cap, 4))
        rc = lib.msfem_spheres_rsa(seed, rmin, rmax, fraction, dim, max_tries, out.ctypes.data, cap,
                                   ctypes.byref(n))
        if rc == 0:
            return np.ascontiguousarray(out[:n.value])
        if rc != 1:
            raise ValueError("msfem_spheres_rsa: bad arguments")
        cap = int(n.value)


def problem(dim, corners, n_fine, coef, f_value=1.0):
    p = {"dim": dim, "corners": np.ascontiguousarray(corners, dtype=np.float64),
         "coef": dict(coef), "f_value": float(f_value)}
    if np.isscalar(n_fine):
        p["n_fine"] = int(n_fine)
    else:
        p["n_fine_per_cell"] = np.ascontiguousarray(n_fine, dtype=np.int32)
        p["n_fine"] = int(np.max(n_fine)) if len(n_fine) else 1
    return p


def reference_problem(dim=2, n_refine=3, n_refine_local=4):
    """The reference's own hard-coded problem: MatrixCoeff (with its PI_D),
    f = 2 (right_hand_side.tpp:22), coarse hyper_cube refined n_refine times,
    N = 2^n_refine_local fine cells per direction (source/main.cxx:23)."""
    K = 1 << n_refine
    return problem(dim, unit_cube_corners(dim, K), 1 << n_refine_local,
                   {"kind": _abi.COEF_REFERENCE}, f_value=2.0)


def sinsin_square(K=8, N=16):
    """2D unit square, K x K coarse cells, N = 16, a = 1 + 0.9 sin(2 pi x/eps)
    sin(2 pi y/eps), eps = 1/64, f = 1 (homogeneous Dirichlet on the global
    boundary)."""
    return problem(2, unit_cube_corners(2, K), N,
                   {"kind": _abi.COEF_SINSIN, "params": [0.9, 1.0 / 64]}, f_value=1.0)


# seeds (g1, g2, theta) of the random-Fourier tensor fields: the 64 x 64
# throughput field, and the 256 x 256 evaluation field of the mixed form and
# the warm start (never used for training)
FOURIER_SEEDS = (2, 20, 200)
EVAL_SEEDS = (3, 30, 300)


def fourier_square(K=64, N=32, seeds=FOURIER_SEEDS):
    """2D unit square, K x K coarse cells, N fine cells per direction, the
    random-Fourier SPD tensor a = R(theta) diag(e^g1, e^g2) R(theta)^T, f = 1."""
    return problem(2, unit_cube_corners(2, K), N, fourier_coef(seeds), f_value=1.0)


def spheres_cube(K=16, seed=4, sphere_seed=44, sizes=(8, 16, 24), contrast=1e4, spheres=None):
    """3D unit cube, K^3 coarse cells, N per cell drawn uniformly from `sizes`,
    background 1 plus non-overlapping spheres (r in [0.004, 0.012], volume
    fraction 0.2) of value `contrast`, f = 1."""
    rng = SplitMix64(seed)
    n_cells = K ** 3
    nf = np.array([sizes[int(rng.uniform() * len(sizes)) % len(sizes)] for _ in range(n_cells)],
                  dtype=np.int32)
    sp = spheres if spheres is not None else spheres_rsa(sphere_seed)
    coef = {"kind": _abi.COEF_SPHERES, "params": [contrast], "spheres": sp}
    return problem(3, unit_cube_corners(3, K), nf, coef, f_value=1.0)


def gauss_points(prob):
    """Physical QGauss(2) points of every fine cell, per coarse cell an array
    [2^d, N_c^d, d] in the TABULATED order (q x fastest over the reference
    directions, fine cells lexicographic), through the cell's multilinear map."""
    dim = prob["dim"]
    nv = 1 << dim
    g = np.array([0.5 - 0.5 / math.sqrt(3.0), 0.5 + 0.5 / math.sqrt(3.0)])
    out = []
    for c in range(prob["corners"].shape[0]):
        N = int(prob["n_fine_per_cell"][c]) if "n_fine_per_cell" in prob else int(prob["n_fine"])
        cidx = np.indices((N,) * dim).reshape(dim, -1)[::-1].T  # fine cells, x fastest
        pts = np.zeros((nv, cidx.shape[0], dim))
        for q in range(nv):
            t = (cidx + np.array([g[(q >> a) & 1] for a in range(dim)])) / N
            for v in range(nv):
                w = np.ones(t.shape[0])
                for a in range(dim):
                    w = w * (t[:, a] if (v >> a) & 1 else 1.0 - t[:, a])
                pts[q] += w[:, None] * prob["corners"][c, v][None, :]
        out.append(pts)
    return out


def with_rhs(prob, f):
    """The problem with a right-hand side f(x) (x [..., d] -> [...]) tabulated
    at the Gauss points: packed cell blocks [q][fine cell] in "f_qp_values"
    (RightHandSide::value_list at the QGauss(2) points)."""
    q = dict(prob)
    q["f_qp_values"] = np.ascontiguousarray(np.concatenate([f(p).ravel() for p in gauss_points(prob)]))
    return q


def subset(prob, cells):
    """Problem restricted to the given coarse cells (same coefficient)."""
    cells = np.asarray(cells)
    q = dict(prob)
    q["corners"] = np.ascontiguousarray(prob["corners"][cells])
    if "n_fine_per_cell" in prob:
        q["n_fine_per_cell"] = np.ascontiguousarray(prob["n_fine_per_cell"][cells])
    q["coef"] = dict(prob["coef"])
    if prob["coef"].get("kind") == _abi.COEF_TABULATED or prob.get("f_qp_values") is not None:
        raise ValueError("subset of a tabulated problem: tabulate after subsetting")
    return q
