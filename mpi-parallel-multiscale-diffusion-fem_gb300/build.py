"""Build of the package's native libraries (in-tree, no cmake).

  lib/libmsfem_gpu.so   CUDA kernels + C-ABI, nvcc for sm_103a only
  lib/libmsfem_host.so  C++ host layer mirroring the reference's
                        DiffusionProblemBasis / coefficient interfaces,
                        linked against libmsfem_gpu.so
  lib/libmsfem_fields.so  host generators of the synthetic coefficient
                        fields (no CUDA)
"""
import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
INCLUDE = os.path.join(_REPO, "include")
CSRC = os.path.join(_HERE, "csrc")
HOST = os.path.join(_HERE, "host")
LIB_DIR = os.path.join(_HERE, "lib")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
              "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd, quiet):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    if not quiet and res.stderr.strip():
        print(res.stderr)
    return res


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _sources(folder, exts):
    out = []
    for root, _, files in os.walk(folder):
        for f in files:
            if f.endswith(exts):
                out.append(os.path.join(root, f))
    return sorted(out)


# translation units of libmsfem_gpu.so, compiled in parallel then linked
GPU_UNITS = ["msfem_gpu.cu", "k2d.cu", "k3d_fp64.cu", "k3d_mixed.cu", "cnn_tc.cu"]


def build_gpu(force=False, quiet=True, extra=()):
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    target = os.path.join(LIB_DIR, "libmsfem_gpu.so")
    headers = [f for f in _sources(CSRC, (".cuh", ".h"))] + [os.path.join(INCLUDE, "msfem_gpu.h")]
    procs, objs = [], []
    for unit in GPU_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(obj_dir, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [_nvcc(), *ARCH, *[f for f in NVCC_FLAGS if f != "-shared"], *extra, "-I", INCLUDE,
                   "-I", CSRC, "-c", "-o", obj + ".tmp", src]
            procs.append((cmd, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                                     text=True)))
    errors = []
    for cmd, obj, pr in procs:
        out, err = pr.communicate()
        if pr.returncode != 0:
            errors.append(" ".join(cmd) + "\n" + out + err)
        else:
            os.replace(obj + ".tmp", obj)
            if not quiet and err.strip():
                print(err)
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))
    if force or procs or _stale(target, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", target + ".tmp", *objs]
        _run(cmd, quiet)
        os.replace(target + ".tmp", target)
    return target


def build_probe(force=False, quiet=True):
    """FMA-rate probe used by bench.py for the roofline denominator."""
    os.makedirs(LIB_DIR, exist_ok=True)
    target = os.path.join(LIB_DIR, "libmsfem_probe.so")
    src = os.path.join(CSRC, "probe.cu")
    if force or _stale(target, [src]):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-o", target + ".tmp", src]
        _run(cmd, quiet)
        os.replace(target + ".tmp", target)
    return target


def build_host(force=False, quiet=True):
    """C++ mirror of the reference interfaces (no CUDA code; links the GPU lib)."""
    src = os.path.join(HOST, "msfem_host.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(LIB_DIR, exist_ok=True)
    target = os.path.join(LIB_DIR, "libmsfem_host.so")
    deps = _sources(HOST, (".cpp", ".hpp", ".h")) + [os.path.join(INCLUDE, "msfem_gpu.h"),
                                                      os.path.join(LIB_DIR, "libmsfem_gpu.so")]
    if force or _stale(target, deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", INCLUDE, "-I", HOST,
               "-o", target + ".tmp", src, "-L", LIB_DIR, "-lmsfem_gpu",
               "-Wl,-rpath,$ORIGIN"]
        _run(cmd, quiet)
        os.replace(target + ".tmp", target)
    return target


def build_fields(force=False, quiet=True):
    """Field generators; no fused multiply-adds, so the results are the same
    bits on every host (and as the Python restatement in the tests)."""
    src = os.path.join(HOST, "fields.cpp")
    os.makedirs(LIB_DIR, exist_ok=True)
    target = os.path.join(LIB_DIR, "libmsfem_fields.so")
    if force or _stale(target, [src, os.path.join(INCLUDE, "msfem_fields.h")]):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", INCLUDE,
               "-o", target + ".tmp", src]
        _run(cmd, quiet)
        os.replace(target + ".tmp", target)
    return target


def build_all(force=False, quiet=True):
    return [build_gpu(force, quiet), build_probe(force, quiet), build_host(force, quiet),
            build_fields(force, quiet)]
