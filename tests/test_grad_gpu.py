"""Gradient of delta logL and Fisher matrix from the tangent kernels, checked
against central finite differences of the FP64 path and against the
reference's own finite-difference Fisher matrix (ucb_fisher,
ucb/src/glass_ucb_waveform.c:364-522, golden vectors in tests/golden/fisher.npz).
"""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def _bank(rng, port, nseg=8, NFFT=1024, f=(1e-3, 5e-3), amp=(-22.5, -21.3)):
    qmin, dA, dE, iA, iE, inj = [], [], [], [], [], []

    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        h = port.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    for s in range(nseg):
        p = wl.draw_source(rng, rng.uniform(*f), 10 ** rng.uniform(*amp), 1e-17)
        p[1] = np.clip(p[1], -0.9, 0.9)
        p[4] = np.clip(p[4], -0.9, 0.9)
        q, a, e, ia, ie = wl.make_segment(rng, [p], wf, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
    return wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                          invCA=np.array(iA), invCE=np.array(iE)), np.array(inj)


def test_gradient_matches_central_differences(engine, port):
    rng = np.random.default_rng(31)
    bank, inj = _bank(rng, port)
    engine.upload(bank)
    seg = np.arange(len(inj), dtype=np.int32)
    props = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 30.0), 1)[0] for s in seg])
    ty, g, F, st = engine.grad_fisher_host(seg, props)
    assert (st == 0).all(), st
    # the term agrees with the FP64 path (same size from the bandwidth rule)
    _, t64, _, _ = engine.dlogl_host(seg, props, precision=gg.PREC_FP64)
    assert np.abs(ty - t64).max() < 1e-3
    # central differences of the FP64 term, step 1e-6 in params-array units
    # (the step ucb_fisher uses)
    eps = 1e-6
    fd = np.zeros_like(g)
    for k in range(8):
        pp, pm = props.copy(), props.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        _, tp, _, _ = engine.dlogl_host(seg, pp, precision=gg.PREC_FP64)
        _, tm, _, _ = engine.dlogl_host(seg, pm, precision=gg.PREC_FP64)
        fd[:, k] = (tp - tm) / (2 * eps)
    sig = np.sqrt(np.maximum(np.einsum("nkk->nk", F), 1e-30))
    err = np.abs(g - fd) / (sig + np.abs(fd))
    assert err.max() < 2e-3, err.max(axis=0)


def test_fisher_matches_reference_ucb_fisher(engine, golden):
    g = golden("fisher.npz")
    n = len(g["params"])
    for k in range(n):
        invC = g["invC"][k]
        zero = np.zeros((1, 1024), complex)
        bank = wl.SegmentBank(T=T, NFFT=1024, qmin=np.array([g["qmin"][k]], np.int32), dA=zero, dE=zero,
                              invCA=invC[None], invCE=invC[None])
        engine.upload(bank)
        ty, grad, F, st = engine.grad_fisher_host(np.zeros(1, np.int32), g["params"][k:k + 1], fisher_mode=1)
        assert st[0] == 0
        ref = g["F"][k]
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        err = np.abs(F[0] - ref) / scale
        assert err.max() < 1e-3, (k, err.max(), np.unravel_index(err.argmax(), err.shape))
        # zero residual: d/dp of -(h|h)/2 is -(h | dh/dp) = -F[:, lnA] with the
        # Fisher matrix weighted like the gradient (noise at the template's bins)
        _, grad0, F0, _ = engine.grad_fisher_host(np.zeros(1, np.int32), g["params"][k:k + 1], fisher_mode=0)
        np.testing.assert_allclose(grad0[0], -F0[0][:, 3], rtol=1e-3, atol=1e-3 * np.sqrt(np.diag(F0[0])).max())


def test_fisher_big_templates_match_reference_ucb_fisher(engine, golden):
    """Templates of 2048 and 4096 samples on 8192-bin segments (the cluster
    kernels) against the reference's ucb_fisher."""
    g = golden("fisher_big.npz")
    NFFT = g["invC"].shape[1]
    for k in range(len(g["params"])):
        invC = g["invC"][k]
        zero = np.zeros((1, NFFT), complex)
        bank = wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array([g["qmin"][k]], np.int32), dA=zero, dE=zero,
                              invCA=invC[None], invCE=invC[None])
        engine.upload(bank)
        ty, grad, F, st = engine.grad_fisher_host(np.zeros(1, np.int32), g["params"][k:k + 1], fisher_mode=1)
        assert st[0] == 0
        ref = g["F"][k]
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        err = np.abs(F[0] - ref) / scale
        assert err.max() < 1e-3, (int(g["N"][k]), err.max(), np.unravel_index(err.argmax(), err.shape))
        _, grad0, F0, _ = engine.grad_fisher_host(np.zeros(1, np.int32), g["params"][k:k + 1], fisher_mode=0)
        np.testing.assert_allclose(grad0[0], -F0[0][:, 3], rtol=1e-3, atol=1e-3 * np.sqrt(np.diag(F0[0])).max())


def test_gradient_big_templates_match_central_differences(engine, port):
    """Proposals of 2048 and 4096 samples on an 8192-bin bank, mixed with
    small ones in the same batch: every size's gradient against central
    differences of the FP64 path."""
    rng = np.random.default_rng(33)
    bank, inj = _bank(rng, port, nseg=6, NFFT=8192, f=(5e-3, 2e-2), amp=(-21.0, -20.0))
    engine.upload(bank)
    seg = np.repeat(np.arange(len(inj), dtype=np.int32), 2)
    props = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 300.0), 1)[0] for s in seg])
    small = inj[:2].copy()
    small[:, 3] -= 4.0  # quieter copies: small templates on the same segments
    seg = np.concatenate([seg, np.arange(2, dtype=np.int32)])
    props = np.vstack([props, small])
    Ns = np.array([int(port.alignment(T, 8192, int(bank.qmin[s]), p)[0]) for s, p in zip(seg, props)])
    keep = Ns <= 4096  # the bandwidth rule can ask for the whole 8192-bin segment
    seg, props = seg[keep], props[keep]
    assert {2048, 4096} <= set(Ns[keep].tolist()), Ns
    ty, g, F, st = engine.grad_fisher_host(seg, props)
    assert (st == 0).all(), st
    _, t64, _, _ = engine.dlogl_host(seg, props, precision=gg.PREC_FP64)
    assert (np.abs(ty - t64) / np.maximum(1.0, np.abs(t64))).max() < 1e-6
    eps = 1e-6
    fd = np.zeros_like(g)
    for k in range(8):
        pp, pm = props.copy(), props.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        _, tp, _, _ = engine.dlogl_host(seg, pp, precision=gg.PREC_FP64)
        _, tm, _, _ = engine.dlogl_host(seg, pm, precision=gg.PREC_FP64)
        fd[:, k] = (tp - tm) / (2 * eps)
    sig = np.sqrt(np.maximum(np.einsum("nkk->nk", F), 1e-30))
    err = np.abs(g - fd) / (sig + np.abs(fd))
    assert err.max() < 2e-3, err.max(axis=0)


def test_fisher_aligned_matches_finite_differences(engine, port):
    """fisher_mode 0 (noise at the template's own bins) against forward
    differences of the oracle's waveform with aligned noise weights."""
    rng = np.random.default_rng(32)
    bank, inj = _bank(rng, port, nseg=2)
    engine.upload(bank)
    for s in range(2):
        p = inj[s]
        ty, grad, F, st = engine.grad_fisher_host(np.array([s], np.int32), p[None], fisher_mode=0)
        al = port.alignment(T, 1024, int(bank.qmin[s]), p)
        N, imin = int(al[0]), int(al[3])
        h0 = port.waveform(p, N, T)
        eps = 1e-6
        D = []
        for k in range(8):
            pp = p.copy()
            pp[k] += eps
            pm = p.copy()
            pm[k] -= eps
            hp, hm = port.waveform(pp, N, T), port.waveform(pm, N, T)
            D.append((hp[3:5] - hm[3:5]) / (2 * eps))
        j = imin + np.arange(N)
        ok = (j >= 0) & (j < 1024)
        w = np.zeros(N)
        w[ok] = bank.invCA[s][j[ok]]
        Fref = np.zeros((8, 8))
        for a in range(8):
            for b in range(8):
                for c in range(2):
                    ra = D[a][c][0::2] * D[b][c][0::2] + D[a][c][1::2] * D[b][c][1::2]
                    Fref[a, b] += 2 * np.sum(ra * w)
        scale = np.sqrt(np.outer(np.diag(Fref), np.diag(Fref)))
        assert (np.abs(F[0] - Fref) / scale).max() < 1e-3
