"""Host-memory calls whose large inputs sit in pinned (page-locked,
device-mapped) host memory: the kernels read them in place over the CPU-GPU
link instead of copying them first.  Results equal the pageable-copy path bit
for bit (each cell's arithmetic is the same; only where the table is read
from differs)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pinned_table_is_read_in_place(pkg, engine, precision):
    torch = pytest.importorskip("torch")
    abi, W = pkg._abi, pkg.workloads
    n = 64
    prob = W.subset(W.fourier_square(K=64, N=32), np.arange(n))
    tab = np.ascontiguousarray(engine.tabulate(prob, 3))
    assert tab.nbytes >= 1 << 20
    tprob = dict(prob)
    tprob["coef"] = {"kind": abi.COEF_TABULATED, "ncomp": 3, "qp_values": tab}
    ref = engine.run(tprob, precision=precision, tol=1e-10)
    assert ref["rc"] == 0

    pinned = torch.from_numpy(tab).pin_memory()
    keep = []
    d = engine.make_desc(tprob, precision, 1e-10, keep=keep)
    d.coef.qp_values = pinned.data_ptr()
    M = np.zeros((n, 4, 4))
    F = np.zeros((n, 4))
    status = np.zeros(n, dtype=np.int32)
    st = abi.Stats()
    rc = engine.lib.msfem_run_batch(engine.handle, ctypes.byref(d), M.ctypes.data, F.ctypes.data, None,
                                    status.ctypes.data, None, ctypes.byref(st))
    assert rc == abi.OK, abi.last_error(engine.lib)
    assert np.all(status == 0)
    assert np.array_equal(M, ref["M"]) and np.array_equal(F, ref["F"])
    # the table's bytes still cross the link (read by the kernel): counted as H2D
    assert st.h2d_bytes >= tab.nbytes
