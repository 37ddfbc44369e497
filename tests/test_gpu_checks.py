"""The checked build (-DGLASS_GPU_CHECKS, lib/libglass_gb300_checks.so), the
stand-in for compute-sanitizer: the kernels of the ΔlogL path, its
double-float re-evaluation and the no-allocation entry point check their
indexed accesses against the buffers' extents and record any failure
(glass_gpu_check_status).  A child process runs batches on 64-, 256-, 1024-
and 4096-bin segments (N = 32 .. 4096, FP64 and mixed with the re-evaluation)
on the checked library: no check may fail, and the results must agree with the
oracle.  The product library reports itself unchecked."""
import json
import os
import subprocess
import sys

import pytest

import glass_gb300 as gg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_product_library_is_not_the_checked_build():
    from glass_gb300 import build

    build.build()
    assert gg.load_library().glass_gpu_checked_build() == 0


@pytest.mark.gpu
def test_checked_build_runs_every_fd_kernel_without_a_failed_check():
    from glass_gb300 import build

    lib = build.build(checks=True)
    env = dict(os.environ, GLASS_GB300_LIB=lib)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_build_run.py")], env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    for c in out["cases"]:
        assert c["check_fp64"] == 0 and c["check_mixed"] == 0, c
        assert c["fp64_rel_err"] < 1e-10, c
        assert c["mixed_abs_err"] < 1e-3, c
    assert any(c["reevaluated"] > 0 for c in out["cases"])  # the re-evaluation kernels ran
    assert out["noalloc_rc"] == 0 and out["noalloc_check"] == 0 and out["noalloc_rel_err"] < 1e-10, out
