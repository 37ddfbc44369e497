"""Run by tests/test_gpu_checks.py in a child process whose engine library is
the checked build (GLASS_GB300_LIB=glass_gb300/lib/libglass_gb300_checks.so):
batches through every kernel of the ΔlogL path and its re-evaluation, after
each of which no bounds check may have failed, and the results must agree
with the oracle.  Prints one JSON line."""
import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import glass_gb300 as gg  # noqa: E402
from glass_gb300 import workloads as wl  # noqa: E402
from oracle.oracle import Port  # noqa: E402
from test_fd_gpu import _loud_batch, _random_bank  # noqa: E402

T = wl.T_YEAR


def main():
    lib = gg.load_library()
    assert lib.glass_gpu_checked_build() == 1, "not the checked build"
    port = Port()
    eng = gg.Engine(0)
    out = {"cases": []}
    word = ctypes.c_uint()

    def status():
        gg._check(lib.glass_gpu_check_status(eng._ctx, ctypes.byref(word)))
        return int(word.value)

    rng = np.random.default_rng(71)
    # N = 32 and 64 on 64-bin segments; N = 32 .. 1024 on 1024-bin segments;
    # loud sources (re-evaluated) on 1024 and 4096 bins (N up to 4096)
    for name, nseg, NFFT, amp, loud in (("nfft64", 8, 64, (1e-23, 1e-21), False),
                                        ("nfft1024", 16, 1024, (1e-23, 1e-21), False),
                                        ("loud1024", 8, 1024, (1e-22, 1e-21), True),
                                        ("loud4096", 4, 4096, (1e-22, 1e-21), True)):
        bank, inj = _random_bank(rng, nseg, NFFT, port, amp=amp)
        eng.upload(bank)
        if loud:
            seg, params, _ = _loud_batch(rng, inj, nseg)
        else:
            seg = np.repeat(np.arange(nseg, dtype=np.int32), 12)
            params = np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 12) for s in range(nseg)])
        tx = rng.normal(0, 5, len(seg))
        d64, t64, h64, s64 = eng.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_FP64)
        w64 = status()
        eng.set_mixed_tolerance(1e-3)
        n0 = eng.mixed_reevaluated()
        dmx, tmx, hmx, smx = eng.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_MIXED)
        wmx = status()
        reev = eng.mixed_reevaluated() - n0
        rA, rE = bank.interleaved()
        ref = port.dlogl_batch(T, NFFT, bank.qmin, np.ascontiguousarray(rA), np.ascontiguousarray(rE),
                               np.ascontiguousarray(bank.invCA), np.ascontiguousarray(bank.invCE), seg, params, tx)[0]
        ok = (s64 == 0) & np.isfinite(ref)
        out["cases"].append({
            "name": name, "n": int(len(seg)), "check_fp64": w64, "check_mixed": wmx, "reevaluated": int(reev),
            "ok": int(ok.sum()),
            "fp64_rel_err": float((np.abs(d64[ok] - ref[ok]) / np.maximum(1.0, np.abs(ref[ok]))).max()),
            "mixed_abs_err": float(np.abs(dmx[ok] - ref[ok]).max()),
        })
    # the no-allocation entry point (its own plan, slow and spectral launches)
    import torch

    dev = torch.device("cuda", 0)
    bank, inj = _random_bank(rng, 4, 256, port)
    eng.upload(bank)
    seg = np.repeat(np.arange(4, dtype=np.int32), 8)
    params = np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 8) for s in range(4)])
    ref = eng.dlogl_host(seg, params, precision=gg.PREC_FP64)[0]
    rA, rE = bank.interleaved()
    t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev)
         for x in (bank.qmin.astype(np.int32), rA, rE, bank.invCA, bank.invCE, seg, params)]
    d_dl = torch.empty(len(seg), dtype=torch.float64, device=dev)
    ptr = [ctypes.c_void_p(x.data_ptr()) for x in t]
    rc = lib.glass_gpu_dlogl_fp64_noalloc(ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream),
                                          gg.FORMATS["sangria"], T, 0.0, 256, 4, *ptr[:5], len(seg), ptr[5], ptr[6],
                                          None, ctypes.c_void_p(d_dl.data_ptr()), None, None, None)
    torch.cuda.synchronize(dev)
    out["noalloc_rc"] = int(rc)
    out["noalloc_check"] = status()
    out["noalloc_rel_err"] = float((np.abs(d_dl.cpu().numpy() - ref) / np.maximum(1.0, np.abs(ref))).max())
    eng.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
