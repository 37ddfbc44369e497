"""The batch entry point that allocates nothing (glass_gpu_dlogl_fp64_noalloc).

It exists for callers that cannot allocate GPU memory once they are running:
everything it needs besides the caller's own inputs and outputs sits in
fixed arrays inside the library.  Called through the C ABI with device
buffers, it must give what glass_gpu_dlogl_batch gives in FP64 (1e-10
relative, the FP64 tolerance of the other tests), and keep doing so on a
second call that finds the first call's leftovers in those arrays.  This file
is collected last so that a run stopping at its first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR
REL = 1e-10


def _bank(rng, port, nseg, NFFT):
    qmin, dA, dE, iA, iE, inj = [], [], [], [], [], []

    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        h = port.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    for _ in range(nseg):
        p = wl.draw_source(rng, 10 ** rng.uniform(np.log10(0.5e-3), np.log10(15e-3)), 10 ** rng.uniform(-23, -21))
        q, a, e, ia, ie = wl.make_segment(rng, [p], wf, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
    return wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                          invCA=np.array(iA), invCE=np.array(iE)), np.array(inj)


def test_noalloc_batch_matches_the_allocating_entry_point(port):
    torch = pytest.importorskip("torch")
    from glass_gb300 import build

    build.build()
    lib = gg.load_library()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(99)
    NFFT, nseg = 512, 6
    bank, inj = _bank(rng, port, nseg, NFFT)
    eng = gg.Engine(0)
    eng.upload(bank)
    rA, rE = bank.interleaved()
    d_q = torch.from_numpy(bank.qmin.astype(np.int32)).to(dev)
    d_rA = torch.from_numpy(np.ascontiguousarray(rA)).to(dev)
    d_rE = torch.from_numpy(np.ascontiguousarray(rE)).to(dev)
    d_iA = torch.from_numpy(np.ascontiguousarray(bank.invCA)).to(dev)
    d_iE = torch.from_numpy(np.ascontiguousarray(bank.invCE)).to(dev)
    stream = torch.cuda.current_stream(dev)

    def ptr(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    for call in range(2):  # the second call finds the first call's data in the fixed arrays
        n = 300 if call == 0 else 170
        seg = rng.integers(0, nseg, n).astype(np.int32)
        params = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 1)[0] for s in seg])
        params[::37, 0] += 3000.0  # a few templates outside their segment
        tx = rng.normal(0.0, 3.0, n)
        dl_ref, ty_ref, hh_ref, st_ref = eng.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_FP64)
        d_seg = torch.from_numpy(seg).to(dev)
        d_p = torch.from_numpy(params).to(dev)
        d_tx = torch.from_numpy(tx).to(dev)
        d_dl = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
        d_ty = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
        d_hh = torch.full((n,), -1.0, dtype=torch.float64, device=dev)
        d_st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        rc = lib.glass_gpu_dlogl_fp64_noalloc(ctypes.c_void_p(stream.cuda_stream), gg.FORMATS["sangria"], T, 0.0,
                                              NFFT, nseg, ptr(d_q), ptr(d_rA), ptr(d_rE), ptr(d_iA), ptr(d_iE), n,
                                              ptr(d_seg), ptr(d_p), ptr(d_tx), ptr(d_dl), ptr(d_ty), ptr(d_hh),
                                              ptr(d_st))
        assert rc == 0, lib.glass_gpu_last_error()
        torch.cuda.synchronize(dev)
        np.testing.assert_array_equal(d_st.cpu().numpy(), st_ref)
        for got, ref in ((d_dl, dl_ref), (d_ty, ty_ref), (d_hh, hh_ref)):
            got = got.cpu().numpy()
            err = np.abs(got - ref) / np.maximum(1.0, np.abs(ref))
            assert err.max() < REL, (call, err.max())
    # sizes beyond the fixed arrays are refused, not truncated
    big = lib.glass_gpu_dlogl_fp64_noalloc(ctypes.c_void_p(stream.cuda_stream), 0, T, 0.0, NFFT, nseg, ptr(d_q),
                                           ptr(d_rA), ptr(d_rE), ptr(d_iA), ptr(d_iE), gg.lib_constants()["GLASS_NOALLOC_MAX_ITEMS"] + 1,
                                           ptr(d_seg), ptr(d_p), None, ptr(d_dl), None, None, None)
    assert big == -2
    assert b"GLASS_NOALLOC_MAX_ITEMS" in lib.glass_gpu_last_error()  # the refusal says why
    eng.close()
