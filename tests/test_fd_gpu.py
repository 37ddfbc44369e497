"""Parity of the CUDA Fourier-domain path with the reference (golden vectors)
and with the oracle, through the C ABI.

Tolerances: the plain FP64 path must match to 1e-10 relative (waveforms:
relative to the channel's largest value; delta logL: relative to
max(1, |logL|)).  The mixed-precision path, at its default tolerance, must
stay within |delta logL error| < 1e-3 of the FP64 path for every proposal
(the proposals its error bound cannot clear are evaluated again in
double-float, from FP32 or from FP64 series, inside the same launch
sequence).
"""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR
REL = 1e-10
MIXED_ABS = 1e-3


def assert_mixed_close(d_mixed, d_fp64, scale=None):
    err = np.abs(d_mixed - d_fp64)
    if scale is not None:
        err = err / scale
    assert (err < MIXED_ABS).all(), err.max()


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def test_drop_in_waveform_matches_reference(golden):
    g = golden("waveforms.npz")
    for i in range(len(g["N"])):
        fmt, N, NI, t0 = str(g["fmt"][i]), int(g["N"][i]), int(g["NI"][i]), float(g["t0"][i])
        ref = g[f"h{i}"]
        got = gg.ucb_waveform(g["params"][i], N, T, t0=t0, fmt=fmt, NI=NI)
        chans = range(5) if (fmt == "sangria" or NI > 1) else range(1)
        for c in chans:
            scale = np.abs(ref[c]).max()
            err = np.abs(got[c] - ref[c]).max() / scale
            assert err < REL, (fmt, N, NI, t0, c, err)
        if not (fmt == "sangria" or NI > 1):
            assert not got[1:].any()  # Y, Z, A, E untouched for NI == 1


def test_drop_in_waveform_with_given_orbit(port):
    """Positions supplied by the caller (the reference's orbit_function) are used as-is."""
    rng = np.random.default_rng(3)
    p = wl.draw_source(rng, 4e-3, 1e-22)
    N = 256
    pos = np.array([port.orbit(T * n / N) for n in range(N)])
    a = gg.ucb_waveform(p, N, T, orbit_xyz=pos)
    b = port.waveform(p, N, T)
    for c in range(5):
        assert np.abs(a[c] - b[c]).max() / np.abs(b[c]).max() < REL


def _case(g, k):
    return {key[len(f"c{k}_"):]: g[key] for key in g.files if key.startswith(f"c{k}_")}


def _residual(port, case):
    rA, rE = case["dA"].copy(), case["dE"].copy()
    for p in case["extra"]:
        al = port.alignment(T, 1024, int(case["qmin"]), p)
        N, imin = int(al[0]), int(al[3])
        h = port.waveform(p, N, T)
        for i in range(N):
            j = i + imin
            if 0 <= j < 1024:
                rA[2 * j:2 * j + 2] -= h[3][2 * i:2 * i + 2]
                rE[2 * j:2 * j + 2] -= h[4][2 * i:2 * i + 2]
    return rA, rE


def _bank_from_interleaved(qmin, rA, rE, iA, iE, NFFT=1024, t0=0.0):
    rA = np.atleast_2d(rA)
    rE = np.atleast_2d(rE)
    return wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.atleast_1d(np.asarray(qmin, np.int32)),
                          dA=rA[:, 0::2] + 1j * rA[:, 1::2], dE=rE[:, 0::2] + 1j * rE[:, 1::2],
                          invCA=np.atleast_2d(iA), invCE=np.atleast_2d(iE), t0=t0)


def test_fp64_delta_logl_matches_reference(engine, port, golden):
    g = golden("likelihood.npz")
    for k in range(int(g["ncase"])):
        case = _case(g, k)
        rA, rE = _residual(port, case)
        engine.upload(_bank_from_interleaved(int(case["qmin"]), rA, rE, case["invCA"], case["invCE"]))
        props = case["props"]
        dl, ty, hh, st = engine.dlogl_host(np.zeros(len(props), np.int32), props, precision=gg.PREC_FP64)
        assert (st == 0).all()
        logL = case["logL"]
        for j in range(1, len(props)):
            d_ref = logL[j] - logL[0]
            assert abs((ty[j] - ty[0]) - d_ref) < REL * max(1.0, abs(logL[j])), (k, j, ty[j] - ty[0], d_ref)
        if len(case["extra"]) == 0:
            for j in range(len(props)):
                assert abs(ty[j] - (logL[j] - case["logL_empty"])) < REL * max(1.0, abs(logL[j]))


def _random_bank(rng, nseg, NFFT, port, t0=0.0, log_f=(0.5e-3, 15e-3), amp=(1e-23, 1e-21)):
    qmin, dA, dE, iA, iE, inj = [], [], [], [], [], []

    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        h = port.waveform(p, int(al[0]), T, t0=t0)
        return int(al[0]), h[3], h[4]

    for s in range(nseg):
        f0 = 10 ** rng.uniform(np.log10(log_f[0]), np.log10(log_f[1]))
        a0 = 10 ** rng.uniform(np.log10(amp[0]), np.log10(amp[1]))
        p = wl.draw_source(rng, f0, a0, 1e-17)
        q, a, e, ia, ie = wl.make_segment(rng, [p], wf, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
    bank = wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                          invCA=np.array(iA), invCE=np.array(iE), t0=t0)
    return bank, np.array(inj)


def _oracle_terms(port, bank, seg, params, fmt="sangria"):
    rA, rE = bank.interleaved()
    out = []
    for s, p in zip(seg, params):
        t, h, N = port.dlogl_term(p, T, bank.NFFT, int(bank.qmin[s]), rA[s], rE[s], bank.invCA[s], bank.invCE[s],
                                  t0=bank.t0, fmt=fmt)
        out.append((t, h, N))
    return np.array(out)


@pytest.mark.parametrize("fmt", ["sangria", "phase", "frequency"])
def test_fp64_batch_matches_oracle_all_sizes(engine, port, fmt):
    """Config-1-like bank: f0 log-uniform over 0.5-15 mHz so N spans 32..1024."""
    rng = np.random.default_rng({"sangria": 11, "phase": 12, "frequency": 13}[fmt])
    bank, inj = _random_bank(rng, 16, 1024, port)
    engine.upload(bank, fmt=fmt)
    seg = rng.integers(0, 16, 96).astype(np.int32)
    params = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 1)[0] for s in seg])
    dl, ty, hh, st = engine.dlogl_host(seg, params, precision=gg.PREC_FP64)
    ref = _oracle_terms(port, bank, seg, params, fmt)
    assert (st == 0).all()
    Ns = set(ref[:, 2].astype(int))
    assert len(Ns) >= 3, Ns
    err = np.abs(ty - ref[:, 0]) / np.maximum(1.0, np.abs(ref[:, 0]))
    assert err.max() < REL, err.max()
    np.testing.assert_allclose(hh, ref[:, 1], rtol=1e-9, atol=1e-12)


def test_mixed_precision_error_budget(engine, port):
    rng = np.random.default_rng(21)
    bank, inj = _random_bank(rng, 32, 1024, port)
    engine.upload(bank)
    seg = np.repeat(np.arange(32, dtype=np.int32), 16)
    params = np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 16) for s in range(32)])
    tx = rng.normal(0, 5, len(seg))
    d64, t64, h64, s64 = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_FP64)
    d32, t32, h32, s32 = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_MIXED)
    assert (s64 == 0).all() and (s32 == 0).all()
    assert_mixed_close(d32, d64)
    np.testing.assert_allclose(d64, t64 - tx, rtol=0, atol=1e-9)
    np.testing.assert_allclose(h32, h64, rtol=1e-4)


def _loud_batch(rng, inj, nseg):
    """Proposals around each segment's source: jumps at 12 temperatures
    (1.5^k), and louder copies far from the data (amplitude x3 .. x30, f0
    moved by 0 .. 40 bins), where the FP32 error bound is largest."""
    seg, params, temps = [], [], []
    for s in range(nseg):
        for k in range(12):
            T_k = 1.5 ** k
            params.append(wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0) * np.sqrt(T_k), 1)[0])
            seg.append(s)
            temps.append(T_k)
        for fa in (3.0, 10.0, 30.0):
            for df in (0.0, 2.0, 40.0):
                p = inj[s].copy()
                p[3] += np.log(fa)
                p[0] += df
                params.append(p)
                seg.append(s)
                temps.append(1.5 ** 11)
    return np.array(seg, np.int32), np.array(params), np.array(temps)


def test_mixed_tolerance_tiers(engine, port):
    """Default tolerance: every proposal within 1e-3 of FP64, with the
    double-float re-evaluation used on loud templates; per-proposal scale
    (the temperature): |error| / T within 1e-3 with fewer re-evaluations;
    zero tolerance: no re-evaluation.  A CUDA-graph replay (conditional node
    around the re-evaluation) reproduces the direct launch exactly."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    bank, inj = _random_bank(rng, 16, 1024, port, amp=(1e-22, 1e-21))
    engine.upload(bank)
    seg, params, temps = _loud_batch(rng, inj, 16)
    tx = rng.normal(0, 5, len(seg))
    d64 = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_FP64)[0]
    try:
        engine.set_mixed_tolerance(1e-3)
        n0 = engine.mixed_reevaluated()
        dm = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_MIXED)[0]
        n1 = engine.mixed_reevaluated()
        assert_mixed_close(dm, d64)
        assert n1 > n0
        # per-proposal scale
        engine.set_mixed_tolerance_scale(temps)
        dt = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_MIXED)[0]
        n2 = engine.mixed_reevaluated()
        assert_mixed_close(dt, d64, scale=temps)
        assert 0 < n2 - n1 < n1 - n0
        engine.set_mixed_tolerance_scale(None)
        # raw mixed
        engine.set_mixed_tolerance(0.0)
        dr = engine.dlogl_host(seg, params, term_x=tx, precision=gg.PREC_MIXED)[0]
        assert engine.mixed_reevaluated() == n2
        assert np.abs(dr - d64).max() > np.abs(dm - d64).max()
        # graph replay of the default tolerance
        engine.set_mixed_tolerance(1e-3)
        dev = torch.device("cuda", 0)
        stream = torch.cuda.Stream(dev)
        engine.set_stream(stream.cuda_stream)
        d_seg = torch.from_numpy(seg).to(dev)
        d_p = torch.from_numpy(params).to(dev)
        d_tx = torch.from_numpy(tx).to(dev)
        out = torch.empty(len(seg), dtype=torch.float64, device=dev)
        with torch.cuda.stream(stream):
            engine.dlogl_device(d_seg, d_p, out, term_x=d_tx, precision=gg.PREC_MIXED)
        stream.synchronize()
        eager = out.cpu().numpy()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            engine.dlogl_device(d_seg, d_p, out, term_x=d_tx, precision=gg.PREC_MIXED)
        out.zero_()
        with torch.cuda.stream(stream):
            g.replay()
            g.replay()
        stream.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), eager)
        assert_mixed_close(eager, d64)
    finally:
        engine.set_stream(None)
        engine.set_mixed_tolerance(1e-3)
        engine.set_mixed_tolerance_scale(None)


def test_segment_edges_and_status(engine, port):
    """Templates that straddle either segment edge are clipped like
    add_ucb_model (ucb/src/glass_ucb_model.c:180-232); templates outside the
    segment leave logL unchanged; bad inputs are flagged per item."""
    rng = np.random.default_rng(5)
    bank, inj = _random_bank(rng, 2, 256, port, log_f=(3e-3, 3.2e-3))
    engine.upload(bank)
    p0 = inj[0].copy()
    cases = []
    for shift in (-150.0, -120.0, -100.0, 100.0, 120.0, 140.0, 2000.0, -2000.0):
        p = p0.copy()
        p[0] += shift
        cases.append(p)
    params = np.array(cases)
    seg = np.zeros(len(params), np.int32)
    dl, ty, hh, st = engine.dlogl_host(seg, params, precision=gg.PREC_FP64)
    ref = _oracle_terms(port, bank, seg, params)
    err = np.abs(ty - ref[:, 0]) / np.maximum(1.0, np.abs(ref[:, 0]))
    assert err.max() < REL
    assert st[-1] == gg.ITEM_OUTSIDE and st[-2] == gg.ITEM_OUTSIDE
    assert ty[-1] == 0.0 and ty[-2] == 0.0
    # mixed precision clips identically
    dm, tm, hm, sm = engine.dlogl_host(seg, params, precision=gg.PREC_MIXED)
    assert_mixed_close(tm, ty)
    # invalid inputs
    bad = np.array([p0, p0, p0, p0])
    bad[0, 3] = np.nan
    bad[1, 1] = 1.5
    segb = np.array([0, 0, 7, -1], np.int32)
    dl, ty, hh, st = engine.dlogl_host(segb, bad, precision=gg.PREC_FP64)
    assert st[0] & gg.ITEM_NONFINITE and st[1] & gg.ITEM_NONFINITE
    assert st[2] & gg.ITEM_BAD_SEGMENT and st[3] & gg.ITEM_BAD_SEGMENT
    assert np.isnan(dl).all()
    # empty batch is a no-op
    engine.dlogl_host(np.zeros(0, np.int32), np.zeros((0, 8)))


def test_t0_and_residual_update(engine, port):
    rng = np.random.default_rng(8)
    bank, inj = _random_bank(rng, 4, 512, port, t0=2.5e6)
    engine.upload(bank)
    seg = np.arange(4, dtype=np.int32)
    dl, ty, hh, st = engine.dlogl_host(seg, inj, precision=gg.PREC_FP64)
    ref = _oracle_terms(port, bank, seg, inj)
    assert (np.abs(ty - ref[:, 0]) / np.maximum(1, np.abs(ref[:, 0]))).max() < REL
    dm, tm, _, _ = engine.dlogl_host(seg, inj, precision=gg.PREC_MIXED)
    assert_mixed_close(tm, ty)
    # replace the residual of segment 2 with data minus the injection
    rA, rE = bank.interleaved()
    al = port.alignment(T, 512, int(bank.qmin[2]), inj[2])
    hw = port.waveform(inj[2], int(al[0]), T, t0=bank.t0)
    rA2, rE2 = rA[2].copy(), rE[2].copy()
    for i in range(int(al[0])):
        j = i + int(al[3])
        if 0 <= j < 512:
            rA2[2 * j:2 * j + 2] -= hw[3][2 * i:2 * i + 2]
            rE2[2 * j:2 * j + 2] -= hw[4][2 * i:2 * i + 2]
    engine.set_residual(2, rA2, rE2)
    dl2, ty2, hh2, st2 = engine.dlogl_host(np.array([2], np.int32), inj[2:3], precision=gg.PREC_FP64)
    t_ref, _, _ = port.dlogl_term(inj[2], T, 512, int(bank.qmin[2]), rA2, rE2, bank.invCA[2], bank.invCE[2],
                                  t0=bank.t0)
    assert abs(ty2[0] - t_ref) < REL * max(1, abs(t_ref))


def test_phase_timing(engine, port):
    """Per-phase durations of a step: refused before any timed step, four
    durations after one (plan, slow part and spectral positive; the
    re-evaluation non-negative), and the results unchanged by the events."""
    rng = np.random.default_rng(31)
    bank, inj = _random_bank(rng, 8, 1024, port)
    engine.upload(bank)
    seg = np.repeat(np.arange(8, dtype=np.int32), 32)
    params = np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 32) for s in range(8)])
    ref = engine.dlogl_host(seg, params, precision=gg.PREC_MIXED)
    with pytest.raises(gg.GlassError):
        engine.last_phase_ms()
    engine.set_phase_timing(True)
    try:
        got = engine.dlogl_host(seg, params, precision=gg.PREC_MIXED)
        ms = engine.last_phase_ms()
    finally:
        engine.set_phase_timing(False)
    assert len(ms) == 4 and all(v > 0 for v in ms[:3]) and ms[3] >= 0
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def test_host_entry_point_replays_follow_inputs_and_bank(engine, port):
    """The host-pointer entry point records its copy-in/kernels/copy-out
    sequence as a CUDA graph per batch shape and replays it: a replay must see
    the new inputs, and a new bank or template size must not reuse a graph that
    holds the old one.  Reference: the device-pointer entry point."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(41)
    bank, inj = _random_bank(rng, 8, 1024, port)
    engine.upload(bank)
    seg = np.repeat(np.arange(8, dtype=np.int32), 24)
    draws = [np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 24) for s in range(8)])
             for _ in range(3)]
    txs = [rng.normal(0, 5, len(seg)) for _ in range(3)]

    def device(params, tx, prec):
        d = torch.empty(len(seg), dtype=torch.float64, device="cuda")
        ty, hh = torch.empty_like(d), torch.empty_like(d)
        st = torch.empty(len(seg), dtype=torch.int32, device="cuda")
        dseg = torch.from_numpy(seg).cuda()
        engine.dlogl_device(dseg, torch.from_numpy(params).cuda(), d, ty, hh, st,
                            term_x=None if tx is None else torch.from_numpy(tx).cuda(), precision=prec)
        torch.cuda.synchronize()
        return d.cpu().numpy(), ty.cpu().numpy(), hh.cpu().numpy(), st.cpu().numpy()

    for prec in (gg.PREC_MIXED, gg.PREC_FP64):
        for k in (0, 1, 2, 1, 0):  # first call records, the others replay
            got = engine.dlogl_host(seg, draws[k], term_x=txs[k], precision=prec)
            for a, b in zip(got, device(draws[k], txs[k], prec)):
                np.testing.assert_array_equal(a, b)
        got = engine.dlogl_host(seg, draws[2], precision=prec)  # no term_x: another shape
        np.testing.assert_array_equal(got[0], device(draws[2], None, prec)[0])
    # a new bank (new device buffers) and a fixed template size
    bank2, inj2 = _random_bank(rng, 8, 1024, port)
    engine.upload(bank2)
    got = engine.dlogl_host(seg, draws[0], term_x=txs[0], precision=gg.PREC_MIXED)
    np.testing.assert_array_equal(got[0], device(draws[0], txs[0], gg.PREC_MIXED)[0])
    engine.set_template_size(256)
    try:
        got = engine.dlogl_host(seg, draws[0], term_x=txs[0], precision=gg.PREC_MIXED)
        np.testing.assert_array_equal(got[0], device(draws[0], txs[0], gg.PREC_MIXED)[0])
    finally:
        engine.set_template_size(0)


def test_large_templates_on_8192_bin_segments(engine, port):
    """Config-4 sizes: segments of 8192 bins, so that the bandwidth rule reaches
    N = 2048 and 4096 for loud sources (the SNR spread sets N).  Those sizes run
    in the per-size spectral kernels on forked streams beside the persistent
    kernel; FP64 against the oracle to 1e-10.  Mixed precision against FP64:
    within 1e-3 at the default tolerance (these templates, SNR in the
    thousands, are all re-evaluated in double-float), and without the
    re-evaluation within the FP32 template error (relative ~1e-6) times
    (h|h)."""
    rng = np.random.default_rng(77)
    NFFT, nseg = 8192, 3
    qmin, dA, dE, iA, iE, inj = [], [], [], [], [], []

    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        return int(al[0]), *port.waveform(p, int(al[0]), T)[3:5]

    for s in range(nseg):
        p = wl.draw_source(rng, 3e-3 + 1e-3 * s, 1e-20, 1e-17)
        q, a, e, ia, ie = wl.make_segment(rng, [p], wf, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
    bank = wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                          invCA=np.array(iA), invCE=np.array(iE))
    engine.upload(bank)
    # loud proposals near the injections, kept where the rule gives N <= 4096
    # (the engine's largest template; louder ones get N = 8192 on these segments)
    seg = np.repeat(np.arange(nseg, dtype=np.int32), 16)
    params = np.vstack([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 200.0), 16) for s in range(nseg)])
    params[:, 3] = np.log(10 ** rng.uniform(-21.0, -20.0, len(seg)))
    keep = np.array([port.alignment(T, NFFT, 0, p)[0] <= 4096 for p in params])
    seg, params = seg[keep], params[keep]
    ref = _oracle_terms(port, bank, seg, params)
    Ns = set(ref[:, 2].astype(int))
    assert {2048, 4096} <= Ns, Ns
    dl, ty, hh, st = engine.dlogl_host(seg, params, precision=gg.PREC_FP64)
    assert (st == 0).all()
    err = np.abs(ty - ref[:, 0]) / np.maximum(1.0, np.abs(ref[:, 0]))
    assert err.max() < REL, err.max()
    np.testing.assert_allclose(hh, ref[:, 1], rtol=1e-9)
    n0 = engine.mixed_reevaluated()
    d32, t32, h32, s32 = engine.dlogl_host(seg, params, precision=gg.PREC_MIXED)
    assert (s32 == 0).all()
    assert engine.mixed_reevaluated() > n0
    assert_mixed_close(t32, ty)
    np.testing.assert_allclose(h32, hh, rtol=1e-4)
    try:
        engine.set_mixed_tolerance(0.0)
        d32, t32, h32, s32 = engine.dlogl_host(seg, params, precision=gg.PREC_MIXED)
    finally:
        engine.set_mixed_tolerance(1e-3)
    assert (np.abs(t32 - ty) <= 1e-5 * np.maximum(1.0, hh)).all(), (np.abs(t32 - ty) / np.maximum(1.0, hh)).max()


def test_drop_in_waveform_from_concurrent_threads():
    """The reference calls ucb_waveform from OpenMP threads, one chain per
    thread (apps/src/ucb_mcmc.c:230): concurrent calls must each give the
    result of a sequential call.  Eight host threads, different sources and
    sizes, compared bit for bit."""
    import threading

    rng = np.random.default_rng(12)
    jobs = [(wl.draw_source(rng, 10 ** rng.uniform(-3.3, -2.0), 1e-22), int(32 << (k % 6))) for k in range(48)]
    want = [gg.ucb_waveform(p, N, T) for p, N in jobs]
    got = [None] * len(jobs)
    errors = []

    def worker(w):
        try:
            for rep in range(3):
                for k in range(w, len(jobs), 8):
                    got[k] = gg.ucb_waveform(jobs[k][0], jobs[k][1], T)
        except Exception as e:  # reported below; a thread's exception is not a test failure by itself
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(w,)) for w in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(len(jobs)):
        np.testing.assert_array_equal(got[k], want[k])


def test_host_access_paths_agree(engine, port):
    """glass_gpu_dlogl_batch_host gives the same bits through pinned staging
    and, where the device reads pageable host memory in place, through the
    gather/scatter kernels; graph replays pick up new host arrays of the same
    shape; NULL optional outputs are left out."""
    rng = np.random.default_rng(31)
    bank, inj = _random_bank(rng, 8, 1024, port)
    engine.upload(bank)
    n = 700
    seg = rng.integers(0, 8, n).astype(np.int32)
    draws = [np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 1)[0] for s in seg])
             for _ in range(3)]
    tx = rng.normal(0, 5, n)
    supported, direct = engine.host_access()
    assert direct == supported  # the default picks the in-place path where it exists
    modes = [0] + ([1] if supported else [])
    if not supported:
        with pytest.raises(gg.GlassError):
            engine.set_host_access(1)
    with pytest.raises(gg.GlassError):
        engine.set_host_access(2)
    res = {}
    try:
        for m in modes:
            engine.set_host_access(m)
            assert engine.host_access()[1] == (m == 1)
            for prec in (gg.PREC_FP64, gg.PREC_MIXED):
                for t in (None, tx):
                    for k, p in enumerate(draws):  # first call records, later calls replay
                        res[(m, prec, t is None, k)] = engine.dlogl_host(seg, p.copy(), term_x=t, precision=prec)
            # optional outputs left NULL
            dl = np.full(n, np.nan)
            p = draws[0].copy()
            gg._check(engine.lib.glass_gpu_dlogl_batch_host(engine._ctx, gg.PREC_MIXED, n, gg._pi(seg), gg._pd(p),
                                                            None, gg._pd(dl), None, None, None))
            np.testing.assert_array_equal(dl, res[(m, gg.PREC_MIXED, True, 0)][0])
    finally:
        engine.set_host_access(-1)
    for (m, prec, notx, k), r in res.items():
        ref = res[(0, prec, notx, k)]
        for a, b in zip(r, ref):
            np.testing.assert_array_equal(a, b)
        assert (r[3] == 0).all()
    # the draws differ, so a replay that kept old inputs would show
    for m in modes:
        assert not np.array_equal(res[(m, gg.PREC_FP64, True, 0)][1], res[(m, gg.PREC_FP64, True, 1)][1])
    # and the device entry point agrees
    import torch

    p = draws[2]
    d_out = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    d_st = torch.empty(n, dtype=torch.int32, device="cuda")
    d_seg, d_p, d_tx = (torch.tensor(a, device="cuda") for a in (seg, p, tx))
    torch.cuda.synchronize()
    engine.dlogl_device(d_seg, d_p, d_out[0], d_out[1], d_out[2], d_st, term_x=d_tx, precision=gg.PREC_MIXED)
    torch.cuda.synchronize()
    for a, b in zip(d_out, res[(modes[-1], gg.PREC_MIXED, False, 2)][:3]):
        np.testing.assert_array_equal(a.cpu().numpy(), b)
