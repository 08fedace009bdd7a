"""The native sphere generator (libmsfem_fields.so) against a plain-Python
restatement of random sequential addition with the same SplitMix64 stream:
the same spheres bit for bit, non-overlapping, at the requested fraction."""
import math

import numpy as np
import pytest


def rsa_python(W, seed, rmin, rmax, fraction, dim, max_tries=10_000_000):
    rng = W.SplitMix64(seed)
    h = 2 * rmax
    G = int(math.ceil(1.0 / h))
    grid, out, vol, tries = {}, [], 0.0, 0
    unit = (4.0 / 3.0) * math.pi if dim == 3 else math.pi
    while vol < fraction and tries < max_tries:
        tries += 1
        r = rmin + (rmax - rmin) * rng.uniform()
        c = [rng.uniform() for _ in range(dim)]
        gi = [min(G - 1, int(c[a] / h)) for a in range(dim)]
        rr = range(-1, 2)
        neigh = ([(gi[0] + i, gi[1] + j, gi[2] + k) for i in rr for j in rr for k in rr] if dim == 3
                 else [(gi[0] + i, gi[1] + j) for i in rr for j in rr])
        ok = True
        for key in neigh:
            for s in grid.get(key, ()):
                d2 = 0.0
                for a in range(dim):
                    d2 += (c[a] - s[a]) * (c[a] - s[a])
                if d2 < (r + s[3]) * (r + s[3]):
                    ok = False
                    break
            if not ok:
                break
        if not ok:
            continue
        sph = (c[0], c[1], c[2] if dim == 3 else 0.0, r)
        grid.setdefault(tuple(gi), []).append(sph)
        out.append(sph)
        vol += unit * math.pow(r, dim)
    return np.array(out, dtype=np.float64).reshape(-1, 4)


@pytest.mark.parametrize("dim,fraction,seed", [(3, 0.02, 44), (2, 0.3, 7), (3, 0.2, 5)])
def test_native_rsa_equals_python(built, dim, fraction, seed):
    W = built.workloads
    rmin, rmax = (0.004, 0.012) if dim == 3 else (0.01, 0.03)
    if dim == 3 and fraction > 0.1:
        rmin, rmax = 0.02, 0.05  # fewer, larger spheres: the full fraction in seconds of Python
    got = W.spheres_rsa(seed, rmin, rmax, fraction, dim)
    ref = rsa_python(W, seed, rmin, rmax, fraction, dim)
    assert got.shape == ref.shape and got.shape[0] > 10
    assert np.array_equal(got, ref)
    vol = np.sum((4.0 / 3.0) * np.pi * got[:, 3] ** 3 if dim == 3 else np.pi * got[:, 3] ** 2)
    assert fraction <= vol < fraction + ((4.0 / 3.0) * np.pi * rmax ** 3 if dim == 3 else np.pi * rmax ** 2)


def test_native_rsa_no_overlap_on_the_benchmark_field(built):
    """The 3D benchmark field (volume fraction 0.2): no two spheres overlap."""
    W = built.workloads
    sp = W.spheres_rsa(44)
    assert sp.shape[0] > 50_000
    h = 2 * 0.012
    G = int(math.ceil(1.0 / h))
    cell = np.minimum(G - 1, (sp[:, :3] / h).astype(int))
    key = (cell[:, 0] * G + cell[:, 1]) * G + cell[:, 2]
    order = np.argsort(key, kind="stable")
    buckets = {}
    for i in order:
        buckets.setdefault(int(key[i]), []).append(int(i))
    worst = np.inf
    for k, ids in buckets.items():
        cx, cy, cz = k // (G * G), (k // G) % G, k % G
        near = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    near += buckets.get(((cx + dx) * G + cy + dy) * G + cz + dz, [])
        a, b = np.array(ids), np.array(near)
        d = np.linalg.norm(sp[a, None, :3] - sp[None, b, :3], axis=-1) - sp[a, None, 3] - sp[None, b, 3]
        d[a[:, None] == b[None, :]] = np.inf
        worst = min(worst, float(d.min()))
    assert worst >= 0.0


def test_rsa_rejects_bad_arguments(built):
    W = built.workloads
    with pytest.raises(ValueError):
        W.spheres_rsa(1, 0.01, 0.005, 0.1, 3)
