"""The bench's side of the measurement contract that runs without a GPU:
the algorithmic work per CG iteration (the roofline numerator) against the
published per-iteration figures of the local problems, and the reference
arm (the reference algorithm on the host cores) printing one JSON line with
the contract's keys."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_work_per_iteration(bench):
    # W_it = 2 nnz(A_II) + 11 n_I with nnz(A_II) = (3N - 5)^d
    assert bench.flops_per_solve_iter(16) == 6173
    assert bench.flops_per_solve_iter(32) == 27133
    assert [bench.flops_per_solve_iter_3d(n) for n in (8, 16, 24)] == [17491, 196139, 735363]
    # no polynomial: the plain inner CG iteration costs what the FP64 one does
    assert bench.inner_flops_per_iter(32, 0) == bench.flops_per_solve_iter(32)
    # two-level V-cycle, smoothing degree 2 (M = 3), coarse spacing 4 at N = 32:
    # 7 stencils, 52 vector operations per node, 7 x 7 coarse nodes
    assert bench.inner_flops_per_iter(32, 2, 4) == 7 * 2 * 91 ** 2 + 52 * 31 ** 2 + 2 * 49 ** 2 + 28 * 49
    # a coarse grid without interior nodes leaves the smoother's count
    assert bench.inner_flops_per_iter(6, 2, 4) == bench.inner_flops_per_iter(6, 2)


def test_reference_arm_json_line(built, tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in line["config"]
