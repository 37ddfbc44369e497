"""Parity of the CUDA F-statistic (glass_gpu_fstat_batch, glass_gpu_fstat_proposal_host)
with the reference's get_Fstat_logL and build_fstatistic_proposal (golden
vectors made by the reference itself) and with the oracle's restatement of
them, through the C ABI.

Tolerances (FP64 path): logL_AE and the amplitude to 1e-9 relative (relative
to max(|value|, 1e-6 of the case's largest)), the inclination, polarisation
and phase to 1e-8 rad; the proposal density to 1e-9 relative.  The GPU
computes the same sums from whitened templates and data, in another order.
"""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR
REL = 1e-9
ANG = 1e-8


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def _bank(qmin, dA, dE, invCA, NFFT, invCE=None):
    """SegmentBank from interleaved (nseg, 2 NFFT) data."""
    dA = np.atleast_2d(dA)
    dE = np.atleast_2d(dE)
    invCA = np.atleast_2d(invCA)
    invCE = invCA if invCE is None else np.atleast_2d(invCE)
    return wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.atleast_1d(np.asarray(qmin, np.int32)),
                          dA=dA[:, 0::2] + 1j * dA[:, 1::2], dE=dE[:, 0::2] + 1j * dE[:, 1::2],
                          invCA=invCA.copy(), invCE=invCE.copy())


def assert_fstat_close(got, ref, rel=REL, ang=ANG):
    """rows of (logL_AE, A, iota, psi, phase)."""
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    for k in (0, 1):
        m = ok[:, k]
        if not m.any():
            continue
        scale = np.maximum(np.abs(ref[m, k]), np.abs(ref[m, k]).max() * 1e-6)
        scale = np.where(scale > 0, scale, 1.0)
        err = np.abs(got[m, k] - ref[m, k]) / scale
        assert err.max() < rel, (k, err.max(), np.argmax(err))
    for k in (2, 3, 4):
        m = ok[:, k]
        d = np.abs(got[m, k] - ref[m, k])
        if k == 4:
            d = np.minimum(d, 2 * np.pi - d)
        assert d.max(initial=0) < ang, (k, d.max(), np.argmax(d))


def test_fstat_matches_reference(engine, golden):
    g = golden("fstat.npz")
    for c in range(int(g["ncase"])):
        fmt = str(g[f"c{c}_fmt"])
        qmin = int(g[f"c{c}_qmin"])
        engine.upload(_bank(qmin, g[f"c{c}_dA"], g[f"c{c}_dE"], g[f"c{c}_invCA"], 1024), fmt=fmt)
        cells = g[f"c{c}_cells"]
        ll, fp, st = engine.fstat_host(np.zeros(len(cells), np.int32), cells)
        ref = g[f"c{c}_out"][:, 1:]
        assert_fstat_close(np.column_stack([ll, fp]), ref)
        outside = np.isnan(ref[:, 2]) & (ref[:, 0] == 0)
        np.testing.assert_array_equal(st[outside], gg.ITEM_OUTSIDE)
        assert (st[~outside] == 0).all()


def test_fstat_proposal_matches_reference(engine, golden):
    g = golden("fstat.npz")
    engine.upload(_bank(int(g["p_qmin"]), g["p_dA"], g["p_dE"], g["p_invCA"], 64))
    tensor, norm, maxp, nscan = engine.fstat_proposal_host(0, int(g["p_n_theta"]), int(g["p_n_phi"]))
    assert tensor.shape == g["p_tensor"].shape
    np.testing.assert_allclose(tensor, g["p_tensor"], rtol=REL)
    assert abs(norm - float(g["p_norm"])) < REL * abs(float(g["p_norm"]))
    assert abs(maxp - float(g["p_maxp"])) < REL * abs(float(g["p_maxp"]))
    assert nscan > 0


def _segments(port, rng, NFFT, specs):
    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        h = port.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    qs, A, E, iA, iE = [], [], [], [], []
    for f0, amp, fdot in specs:
        inj = wl.draw_source(rng, f0, amp, fdot)
        q, dA, dE, a, e = wl.make_segment(rng, [inj], wf, NFFT=NFFT, T=T)
        qs.append(q)
        A.append(dA)
        E.append(dE)
        iA.append(a)
        iE.append(e * rng.uniform(0.8, 1.25, NFFT))  # unequal A and E noise
    bank = wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qs, np.int32), dA=np.array(A), dE=np.array(E),
                          invCA=np.array(iA), invCE=np.array(iE))
    return bank


def test_fstat_every_size_on_a_multi_segment_bank(engine, port):
    """Filters of 16 to 4096 samples on two 8192-bin segments with unequal A
    and E noise (the reference weights both channels with the A noise),
    against the oracle."""
    rng = np.random.default_rng(11)
    NFFT = 8192
    bank = _segments(port, rng, NFFT, [(2.0e-3, 3e-22, 1e-17), (9.0e-3, 2e-22, 1e-15)])
    engine.upload(bank)
    rA, rE = bank.interleaved()
    cells, segs = [], []
    for s in range(2):
        q = int(bank.qmin[s])
        for fdot in (0.0, 1e-16, 1e-14, 5e-14, 1e-13, 2e-13, 3e-13, 1e-12, 3e-12, 1e-11):
            for _ in range(3):
                cells.append([(q + rng.uniform(0, NFFT)) / T, fdot, np.arccos(rng.uniform(-1, 1)),
                              rng.uniform(0, 2 * np.pi)])
                segs.append(s)
    cells = np.array(cells)
    segs = np.array(segs, np.int32)
    ll, fp, st = engine.fstat_host(segs, cells)
    ref = port.fstat_batch(T, NFFT, bank.qmin, rA, rE, bank.invCA, segs, cells)
    assert_fstat_close(np.column_stack([ll, fp]), ref)
    sizes = {port.bandwidth(c[0], c[1], np.cos(c[2]), 1e-22, T, NFFT) for c in cells}
    assert {16, 32, 64, 128, 256, 512, 1024, 2048, 4096} <= sizes, sizes
    assert (st == 0).all()


def test_fstat_statuses_and_edges(engine, port):
    rng = np.random.default_rng(12)
    bank = _segments(port, rng, 1024, [(3.0e-3, 2e-22, 1e-17)])
    engine.upload(bank)
    q = int(bank.qmin[0])
    th, ph = 1.0, 2.0
    cells = np.array([
        [(q + 0.5) / T, 0, th, ph],      # first bin: half the filter outside, bin 0 left out
        [(q + 1023.5) / T, 0, th, ph],   # last bin
        [(q - 30.5) / T, 0, th, ph],     # entirely below the segment
        [(q + 1100.5) / T, 0, th, ph],   # entirely above
        [np.nan, 0, th, ph],
        [-1e-3, 0, th, ph],
        [(q + 10.5) / T, 0, th, ph],     # bad segment (below)
    ])
    segs = np.array([0, 0, 0, 0, 0, 0, 5], np.int32)
    ll, fp, st = engine.fstat_host(segs, cells)
    assert list(st) == [0, 0, gg.ITEM_OUTSIDE, gg.ITEM_OUTSIDE, gg.ITEM_NONFINITE, gg.ITEM_NONFINITE,
                        gg.ITEM_BAD_SEGMENT]
    rA, rE = bank.interleaved()
    ref = port.fstat_batch(T, 1024, bank.qmin, rA, rE, bank.invCA, np.zeros(4, np.int32), cells[:4])
    assert_fstat_close(np.column_stack([ll[:4], fp[:4]]), ref)
    assert ll[2] == 0 and ll[3] == 0
    assert np.isnan(ll[4:]).all()


def test_fstat_device_entry_point_matches_host(engine, port):
    import torch

    rng = np.random.default_rng(13)
    bank = _segments(port, rng, 1024, [(5.0e-3, 2e-22, 1e-16)])
    engine.upload(bank)
    q = int(bank.qmin[0])
    n = 3000  # more than one warp of sizes, several CTAs per size
    cells = np.stack([(q + rng.uniform(0, 1024, n)) / T, np.where(rng.random(n) < 0.5, 0, 10 ** rng.uniform(-17, -13, n)),
                      np.arccos(rng.uniform(-1, 1, n)), rng.uniform(0, 2 * np.pi, n)], 1)
    segs = np.zeros(n, np.int32)
    ll, fp, st = engine.fstat_host(segs, cells)
    dc = torch.tensor(cells, device="cuda")
    ds = torch.tensor(segs, device="cuda")
    dl = torch.empty(n, dtype=torch.float64, device="cuda")
    dfp = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    dst = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    engine.fstat_device(ds, dc, dl, dfp, dst)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dl.cpu().numpy(), ll)
    np.testing.assert_array_equal(dfp.cpu().numpy(), fp)
    np.testing.assert_array_equal(dst.cpu().numpy(), st)
    rA, rE = bank.interleaved()
    sub = rng.choice(n, 200, replace=False)
    ref = port.fstat_batch(T, 1024, bank.qmin, rA, rE, bank.invCA, segs[sub], cells[sub])
    assert_fstat_close(np.column_stack([ll[sub], fp[sub]]), ref)
