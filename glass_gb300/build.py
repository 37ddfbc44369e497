"""Build recipe for the engine's shared library.

    python -m glass_gb300.build

compiles every translation unit in glass_gb300/csrc for sm_103a with nvcc (in
parallel) and links glass_gb300/lib/libglass_gb300.so, a plain C-ABI library
(include/glass_gb300.h) that depends only on the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libglass_gb300.so")
OBJ_DIR_CHECKS = os.path.join(HERE, "_build_checks")
LIB_CHECKS = os.path.join(OUT_DIR, "libglass_gb300_checks.so")
# the benchmark's FMA-throughput probe: a separate library, not the engine
PROBE_SRC = os.path.join(HERE, "probe", "fma_probe.cu")
PROBE_LIB = os.path.join(OUT_DIR, "libglass_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-I" + os.path.join(ROOT, "include")]
# The FP64 likelihood evaluates the delay and the carrier phase the way the
# reference does (ucb/src/glass_ucb_waveform.c:858-877, arguments of ~1e6 rad,
# where a fused multiply-add would round differently by up to ~1e-10 rad) with
# explicit round-to-nearest operations, so its translation units contract
# freely.  The no-allocation entry point, the F-statistic, the wavelet-domain
# waveform and the noise and sampler units keep contraction off: their
# results follow the reference's operation order throughout.  So do the host
# sums of the struct-based drop-ins (dropin_model.cu), which are bit-identical
# to the reference's x86 build only without contraction (gcc on aarch64
# contracts a * b + c by default).
PER_FILE_FLAGS = {"ucb_fd_noalloc.cu": ["-fmad=false"],
                  "wdm.cu": ["-Xcompiler", "-ffp-contract=off"],
                  "ucb_wavelet.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
                  "ucb_fstat.cu": ["-fmad=false"], "noise.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
                  "capi.cu": ["-Xcompiler", "-ffp-contract=off"], "sampler.cu": ["-fmad=false"],
                  "dropin_model.cu": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(lib: str, deps) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checks: bool = False) -> str:
    """Compile the engine (lib/libglass_gb300.so); with checks=True the
    checked build instead (lib/libglass_gb300_checks.so, -DGLASS_GPU_CHECKS:
    the kernels check their indexed accesses, see glass_gpu_check_status)."""
    lib = LIB_CHECKS if checks else LIB
    obj_dir = OBJ_DIR_CHECKS if checks else OBJ_DIR
    extra = ["-DGLASS_GPU_CHECKS"] if checks else []
    deps = (_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)])
    if not force and not _stale(lib, deps):
        if not checks:
            build_probe()
        return lib
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = ([cc] + ARCH + NVCC_FLAGS + extra + PER_FILE_FLAGS.get(os.path.basename(src), [])
               + ["-c", src, "-o", obj])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(" ".join(cmd))
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(_sources()))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = lib + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if not checks:
        build_probe(force)
    return lib


def build_probe(force: bool = False) -> str:
    if not force and not _stale(PROBE_LIB, [PROBE_SRC, os.path.abspath(__file__)]):
        return PROBE_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-shared", PROBE_SRC, "-o", PROBE_LIB, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {PROBE_SRC}:\n{r.stdout}\n{r.stderr}")
    return PROBE_LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, checks="--checks" in sys.argv))
