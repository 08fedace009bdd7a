"""GB300 (sm_103a) engine for the per-coarse-cell multiscale basis problems of
konsim83/MPI-Parallel-Multiscale-Diffusion-FEM (DiffusionProblemBasis<dim>::run,
include/base/diffusion_problem_basis.tpp:438-474).

The product is the CUDA library lib/libmsfem_gpu.so behind the C-ABI
include/msfem_gpu.h; this package builds it (build.py), binds it (_abi.py,
engine.py), describes workloads (workloads.py) and stores tabulated
coefficient fields on disk (fieldio.py).  It is imported under the
name ``msfem_gb300`` (the folder name is not an identifier).
"""
from . import _abi, build, engine, fieldio, sharding, surrogate, workloads  # noqa: F401
from .engine import Engine  # noqa: F401
