"""CPU tests of the C-ABI surface: the library loads, exports every symbol
include/msfem_gpu.h declares, rejects malformed input before touching a GPU,
and the ctypes mirror of the structs matches the C layout."""
import ctypes
import os
import re
import subprocess

import numpy as np

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "msfem_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\s*\*?\s*(msfem_\w+)\s*\(", src, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for want in ("msfem_create", "msfem_destroy", "msfem_run_batch", "msfem_last_error",
                 "msfem_set_stream", "msfem_tabulate_coefficient", "msfem_version"):
        assert want in names


def test_library_exports_every_declared_symbol(built):
    lib = built._abi.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) == set(built._abi.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", built._abi.LIB_PATH],
                         capture_output=True, text=True).stdout
    for name in declared_functions():
        assert re.search(rf"\bT {name}\b", out), name
    assert lib.msfem_version().startswith(b"msfem_gpu")


def test_struct_layout_matches_c(built, tmp_path):
    """Compile a probe against the header and compare sizeof/offsetof."""
    abi = built._abi
    probe = tmp_path / "probe.c"
    fields = {"msfem_batch_desc": (abi.BatchDesc, ["coef", "f_value", "tol", "maxit", "warm_basis",
                                                   "tol_absolute", "f_qp_values", "f_qp_offset"]),
              "msfem_coef_desc": (abi.CoefDesc, ["params", "qp_values", "n_modes", "spheres"]),
              "msfem_stats": (abi.Stats, ["max_rel_residual", "kernel_launches", "d2h_bytes"])}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "msfem_gpu.h"', "int main(void){"]
    for cname, (_, fl) in fields.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in fl:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    probe.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(probe), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True,
                                                         text=True).stdout.split("\n") if l)
    for cname, (cls, fl) in fields.items():
        assert int(out[cname]) == ctypes.sizeof(cls), cname
        for f in fl:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, (cname, f)


def test_invalid_descriptors_are_rejected_without_a_gpu(built):
    """Argument validation runs before any CUDA call: no handle needed for the
    descriptor checks, and a NULL handle is an argument error."""
    abi = built._abi
    lib = abi.load()
    d = abi.BatchDesc()
    d.dim = 4
    rc = lib.msfem_run_batch(None, ctypes.byref(d), None, None, None, None, None, None)
    assert rc == abi.ERR_INVALID_ARG
    rc = lib.msfem_run_batch(None, None, None, None, None, None, None, None)
    assert rc == abi.ERR_INVALID_ARG
    assert lib.msfem_tabulated_size(None, 1) == -1
    rc = lib.msfem_energy_error(None, ctypes.byref(d), None, None, None, None)
    assert rc == abi.ERR_INVALID_ARG
    rc = lib.msfem_reconstruct(None, ctypes.byref(d), None, None, None)
    assert rc == abi.ERR_INVALID_ARG
    corners = np.zeros((3, 4, 2))
    d.dim = 2
    d.n_cells = 3
    d.n_fine = 16
    d.corners = corners.ctypes.data
    d.coef.kind = abi.COEF_TABULATED
    d.coef.ncomp = 3
    assert lib.msfem_tabulated_size(ctypes.byref(d), 3) == 3 * 3 * 4 * 256
    buf = ctypes.create_string_buffer(256)
    assert lib.msfem_last_error(buf, 256) == 0


def test_describe_tuning_lists_the_compiled_shapes(built):
    """msfem_describe_tuning reports a compiled shape without a GPU: the
    N <= 32 mixed class holds the polynomial shapes and the two-level one
    (degree-2 smoothing, coarse spacing 4); bad keys are argument errors."""
    abi = built._abi
    lib = abi.load()

    def describe(**kw):
        t = abi.Tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        rc = lib.msfem_describe_tuning(ctypes.byref(t))
        return rc, t.as_dict()

    rc, first = describe(dim=2, n_max=32, precision=abi.PREC_MIXED, variant=0)
    assert rc == 0 and first["n_variants"] >= 2
    shapes = [describe(dim=2, n_max=32, precision=abi.PREC_MIXED, variant=v)[1] for v in range(first["n_variants"])]
    two_level = [t for t in shapes if t["coarse_spacing"] > 0]
    assert [(t["coarse_spacing"], t["poly_degree"], t["threads"], t["rows_per_thread"]) for t in two_level] == [(4, 2, 256, 4)]
    assert any(t["poly_degree"] == 5 and t["coarse_spacing"] == 0 for t in shapes)
    rc, fp64 = describe(dim=2, n_max=32, precision=abi.PREC_FP64, variant=0)
    assert rc == 0 and fp64["coarse_spacing"] == 0 and fp64["poly_degree"] == 0
    rc, c3 = describe(dim=3, n_max=24, precision=abi.PREC_MIXED, variant=0)
    assert rc == 0 and c3["n_variants"] >= 1
    assert max(describe(dim=3, n_max=24, precision=abi.PREC_MIXED, variant=v)[1]["cluster_ctas"]
               for v in range(c3["n_variants"])) == 8
    assert describe(dim=2, n_max=32, precision=abi.PREC_MIXED, variant=first["n_variants"])[0] == abi.ERR_INVALID_ARG
    assert describe(dim=4, n_max=32, precision=abi.PREC_MIXED, variant=0)[0] == abi.ERR_INVALID_ARG
    assert lib.msfem_describe_tuning(None) == abi.ERR_INVALID_ARG


def test_create_without_device_fails_cleanly(built):
    """On a machine without a GB300 msfem_create must fail with NO_DEVICE (or
    succeed on an sm_103 box) -- never fall back to the CPU."""
    import torch

    abi = built._abi
    lib = abi.load()
    h = ctypes.c_void_p()
    rc = lib.msfem_create(ctypes.byref(h), 0)
    if not torch.cuda.is_available():
        assert rc == abi.ERR_NO_DEVICE
        assert "device" in abi.last_error(lib).lower() or "cuda" in abi.last_error(lib).lower()
    else:
        if rc == abi.OK:
            lib.msfem_destroy(h)
        else:
            assert rc == abi.ERR_NO_DEVICE
