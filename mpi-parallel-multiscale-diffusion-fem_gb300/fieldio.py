"""On-disk format of a tabulated coefficient field (a coarse mesh plus the
coefficient at every fine Gauss point, the TABULATED layout the kernels
read), so that fields generated once -- by msfem_tabulate_coefficient or by
any TensorFunction's value_list on the host -- are shared by the training-set
generator and the benchmarks without regenerating them.

File layout (little-endian, every section 8-byte aligned):

  offset  size            content
  0       8               magic b"MSFEMFLD"
  8       4 x u32         version (1), dim, ncomp, flags (bit 0: uneven N)
  24      u64             n_cells
  32      i32, u32        n_fine (uniform N, or the largest N), reserved (0)
  40      f64             f_value (the constant right-hand side)
  48      16              reserved (zeros)
  64      f64 [n_cells][2^d][d]              corners (deal.II vertex order)
  ...     i32 [n_cells], padded to 8 bytes   N per cell (uneven N only)
  ...     f64 [sum_c ncomp 2^d N_c^d]        the field: per cell
                                             [component][Gauss point][fine cell]

The payload is read with numpy.memmap, so a multi-GB field (256 x 256 cells,
N = 32, 3 components: 6.4 GB) is not copied on load; pinned or device staging
is the caller's choice.
"""
import numpy as np

from . import _abi

MAGIC = b"MSFEMFLD"
VERSION = 1
HEADER_BYTES = 64


def _payload_len(dim, ncomp, n_cells, n_fine, nf):
    nq = 1 << dim
    if nf is None:
        return n_cells * ncomp * nq * n_fine ** dim
    return int(np.sum(ncomp * nq * nf.astype(np.int64) ** dim))


def save_field(path, problem, table, ncomp):
    """Write problem's mesh and its tabulated coefficient `table` (the
    TABULATED layout, ncomp components) to `path`."""
    dim = int(problem["dim"])
    corners = np.ascontiguousarray(problem["corners"], dtype="<f8")
    n_cells = corners.shape[0]
    assert corners.shape == (n_cells, 1 << dim, dim)
    nf = problem.get("n_fine_per_cell")
    nf = None if nf is None else np.ascontiguousarray(nf, dtype="<i4")
    n_fine = int(nf.max()) if nf is not None else int(problem["n_fine"])
    table = np.ascontiguousarray(table, dtype="<f8").ravel()
    if table.size != _payload_len(dim, ncomp, n_cells, n_fine, nf):
        raise ValueError("table length does not match the mesh and ncomp")
    head = np.zeros(HEADER_BYTES, dtype=np.uint8)
    head[:8] = np.frombuffer(MAGIC, dtype=np.uint8)
    head[8:24] = np.frombuffer(np.array([VERSION, dim, ncomp, 1 if nf is not None else 0], dtype="<u4").tobytes(),
                               dtype=np.uint8)
    head[24:32] = np.frombuffer(np.array([n_cells], dtype="<u8").tobytes(), dtype=np.uint8)
    head[32:40] = np.frombuffer(np.array([n_fine, 0], dtype="<i4").tobytes(), dtype=np.uint8)
    head[40:48] = np.frombuffer(np.array([float(problem.get("f_value", 1.0))], dtype="<f8").tobytes(),
                                dtype=np.uint8)
    with open(path, "wb") as f:
        f.write(head.tobytes())
        f.write(corners.tobytes())
        if nf is not None:
            f.write(nf.tobytes())
            if nf.nbytes % 8:
                f.write(b"\0" * (8 - nf.nbytes % 8))
        f.write(table.tobytes())


def load_field(path, mmap=True):
    """Read a field file into a problem dict with a TABULATED coefficient
    (qp_values a read-only memmap unless mmap=False)."""
    with open(path, "rb") as f:
        head = f.read(HEADER_BYTES)
    if len(head) != HEADER_BYTES or head[:8] != MAGIC:
        raise ValueError(f"{path}: not a coefficient field file")
    version, dim, ncomp, flags = np.frombuffer(head[8:24], dtype="<u4")
    if version != VERSION:
        raise ValueError(f"{path}: unsupported version {version}")
    if dim not in (2, 3) or ncomp not in (1, dim * (dim + 1) // 2):
        raise ValueError(f"{path}: bad dim/ncomp")
    n_cells = int(np.frombuffer(head[24:32], dtype="<u8")[0])
    n_fine = int(np.frombuffer(head[32:36], dtype="<i4")[0])
    f_value = float(np.frombuffer(head[40:48], dtype="<f8")[0])
    nv = 1 << int(dim)
    off = HEADER_BYTES
    corners = np.fromfile(path, dtype="<f8", count=n_cells * nv * dim, offset=off).reshape(n_cells, nv, dim)
    off += corners.nbytes
    nf = None
    if flags & 1:
        nf = np.fromfile(path, dtype="<i4", count=n_cells, offset=off)
        off += (nf.nbytes + 7) // 8 * 8
    count = _payload_len(int(dim), int(ncomp), n_cells, n_fine, nf)
    if mmap:
        table = np.memmap(path, dtype="<f8", mode="r", offset=off, shape=(count,))
    else:
        table = np.fromfile(path, dtype="<f8", count=count, offset=off)
    if table.size != count:
        raise ValueError(f"{path}: truncated field")
    prob = {"dim": int(dim), "corners": corners, "f_value": f_value,
            "coef": {"kind": _abi.COEF_TABULATED, "ncomp": int(ncomp), "qp_values": table}}
    if nf is not None:
        prob["n_fine_per_cell"] = nf
        prob["n_fine"] = n_fine
    else:
        prob["n_fine"] = n_fine
    return prob
