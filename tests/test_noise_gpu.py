"""Parity of the CUDA noise-model likelihood (glass_gpu_noise_logl_batch) with
the reference's noise module (golden vectors made by the reference itself) and
with the oracle's restatement, through the C ABI.

Tolerance (FP64 path): 1e-10 relative on logL and 1e-10 |logL| absolute on
logL differences between models (the sampler's Hastings ratio uses those).
The GPU forms the inverse as cofactor / det; the reference takes
exp(log|cofactor| - log det), whose exponent carries ~|log det| eps ~ 2e-14 of
rounding.  Below ~1 mHz the three XYZ channels are nearly degenerate (the
T combination is suppressed, d3/d1 ~ 3e-7 at 0.1 mHz), the inverse's entries
are ~1/d3 and cancel in the quadratic form, and that 2e-14 becomes ~3e-6 of
logL (3e5) over 1024 bins: the two forms differ by that much on the CPU with
identical inputs.  Above ~2 mHz they agree to 1e-9 or exactly.
"""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR
REL = 1e-10


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def test_noise_logl_matches_reference(engine, golden):
    g = golden("noise.npz")
    for c in range(int(g["ncase"])):
        q = int(g[f"c{c}_qmin"])
        engine.noise_setup(T, q, g[f"c{c}_X"], g[f"c{c}_Y"], g[f"c{c}_Z"])
        inst, sgal = g[f"c{c}_inst"], g[f"c{c}_sgal"]
        for got, ref in ((engine.noise_logl_host(inst), g[f"c{c}_logl_inst"]),
                         (engine.noise_logl_host(inst, sgal), g[f"c{c}_logl_gal"])):
            np.testing.assert_allclose(got, ref, rtol=REL)
            np.testing.assert_allclose(got - got[0], ref - ref[0], atol=REL * abs(ref[0]))


def _data(port, rng, NF, q):
    inst0, sgal0 = wl.default_noise_params(T)
    X, Y, Z = wl.xyz_from_covariance(rng, port.noise_covariance(T, q / T, NF, inst0, sgal0))
    return X, Y, Z, inst0, sgal0


def test_noise_logl_15360_bins_against_oracle(engine, port):
    """The reference benchmark's grid size (apps/src/noise_likelihood_benchmarks.c:25),
    from 0.1 mHz across the 10 mHz acceleration cutoff, 48 models."""
    rng = np.random.default_rng(21)
    NF, q = 15360, int(1e-4 * T)
    X, Y, Z, inst0, sgal0 = _data(port, rng, NF, q)
    engine.noise_setup(T, q, X, Y, Z)
    inst = inst0 * np.exp(rng.uniform(-0.5, 0.5, (48, 12)))
    sgal = sgal0 + rng.uniform(-0.3, 0.3, (48, 5))
    for sg in (None, sgal):
        got = engine.noise_logl_host(inst, sg)
        ref = port.noise_logl(T, q / T, X, Y, Z, inst, sg)
        np.testing.assert_allclose(got, ref, rtol=REL)
        np.testing.assert_allclose(got - got[0], ref - ref[0], atol=REL * abs(ref[0]))


def test_noise_logl_device_entry_and_large_batches(engine, port):
    """More models than one grid row holds (65535), device pointers."""
    import torch

    rng = np.random.default_rng(22)
    NF, q = 1024, int(3e-3 * T)
    X, Y, Z, inst0, sgal0 = _data(port, rng, NF, q)
    engine.noise_setup(T, q, X, Y, Z)
    n = 70000
    inst = inst0 * np.exp(rng.uniform(-0.5, 0.5, (n, 12)))
    sgal = sgal0 + rng.uniform(-0.3, 0.3, (n, 5))
    host = engine.noise_logl_host(inst, sgal)
    di, ds = torch.tensor(inst, device="cuda"), torch.tensor(sgal, device="cuda")
    dl = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    engine.noise_logl_device(di, dl, ds)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dl.cpu().numpy(), host)
    sub = np.r_[0:8, 65530:65545, n - 8:n]
    ref = port.noise_logl(T, q / T, X, Y, Z, inst[sub], sgal[sub])
    np.testing.assert_allclose(host[sub], ref, rtol=REL)


def test_noise_errors(engine):
    with pytest.raises(gg.GlassError):
        engine.noise_setup(T, 0, np.zeros(8), np.zeros(8), np.zeros(8))


# ------------------------------------------------------------ wavelet domain
def test_noise_wavelet_logl_matches_reference(engine, golden):
    """my_noise_log_likelihood_wavelet_coarse with the instrument, stationary and
    modulated foreground covariances, Q = 1 and 8, two bands."""
    g = golden("noise_wavelet.npz")
    NF, NT, df = int(g["NF"]), int(g["NT"]), float(g["df"])
    for c in range(int(g["ncase"])):
        Q, lmin, b = int(g[f"c{c}_Q"]), int(g[f"c{c}_lmin"]), int(g[f"c{c}_band"])
        engine.noise_wavelet_setup(NF, NT, df, lmin, Q, g[f"b{b}_X"], g[f"b{b}_Y"], g[f"b{b}_Z"], g[f"c{c}_mod"])
        for mode in (0, 1, 2):
            got = engine.noise_wavelet_logl_host(g[f"c{c}_inst"], g[f"c{c}_sgal"], mode)
            ref = g[f"c{c}_logl{mode}"]
            np.testing.assert_allclose(got, ref, rtol=REL)
            np.testing.assert_allclose(got - got[0], ref - ref[0], atol=REL * abs(ref[0]))


def test_noise_wavelet_full_grid_against_oracle(engine, port):
    """460 layers of the 1024 x 2048 grid (0.33 .. 15.3 mHz), Q = 16, all modes,
    40 models, and device pointers."""
    import torch

    rng = np.random.default_rng(23)
    NF, NT, lmin, Nl, Q = 1024, 2048, 10, 460, 16
    df = 1.0 / (2 * 15.0 * NF)
    inst0, sgal0 = wl.default_noise_params(T)
    C6 = np.array([port.noise_covariance(T, (lmin + j) * df, 1, inst0, sgal0)[0] for j in range(Nl)]) / (NF * NT)
    X, Y, Z = wl.wavelet_noise_data(rng, C6, NT)
    mod = wl.galaxy_modulation_like(NT // Q)
    engine.noise_wavelet_setup(NF, NT, df, lmin, Q, X, Y, Z, mod)
    P = port.noise_coarse_stats(NT, Q, X, Y, Z)
    inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (40, 12)))
    sgal = sgal0 + rng.uniform(-0.2, 0.2, (40, 5))
    for mode in (0, 1, 2):
        got = engine.noise_wavelet_logl_host(inst, sgal, mode)
        ref = port.noise_wavelet_logl(NF, NT, df, lmin, P, Q, inst, sgal, mode, mod if mode == 2 else None)
        np.testing.assert_allclose(got, ref, rtol=REL)
        np.testing.assert_allclose(got - got[0], ref - ref[0], atol=REL * abs(ref[0]))
        di, dg = torch.tensor(inst, device="cuda"), torch.tensor(sgal, device="cuda")
        dl = torch.empty(40, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        engine.noise_wavelet_logl_device(di, dl, dg, mode)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dl.cpu().numpy(), got)


def test_noise_wavelet_errors(engine):
    with pytest.raises(gg.GlassError):
        engine.noise_wavelet_setup(1024, 256, 1e-5, 10, 512, np.zeros(256), np.zeros(256), np.zeros(256))
    engine.noise_wavelet_setup(1024, 256, 1e-5, 10, 8, np.ones(256), np.ones(256), np.ones(256))
    with pytest.raises(gg.GlassError):  # the modulated foreground needs the modulation
        engine.noise_wavelet_logl_host(np.ones((1, 12)), np.ones((1, 5)), mode=2)


# ------------------------------------------------- the UCB sampler's noise step
def _eta_bank(g, c):
    dA, dE = g[f"c{c}_dA"], g[f"c{c}_dE"]
    return wl.SegmentBank(T=T, NFFT=1024, qmin=np.array([int(g[f"c{c}_qmin"])], np.int32),
                          dA=(dA[0::2] + 1j * dA[1::2])[None], dE=(dE[0::2] + 1j * dE[1::2])[None],
                          invCA=g[f"c{c}_invCA"][None].copy(), invCE=g[f"c{c}_invCE"][None].copy())


def test_noise_step_matches_reference(engine, golden):
    """glass_gpu_noise_eta_batch against noise_model_mcmc's own likelihood change:
    FP64 to 1e-8, mixed precision (FP32 templates) to 2e-3."""
    g = golden("noise_eta.npz")
    for c in range(int(g["ncase"])):
        engine.upload(_eta_bank(g, c))
        p, e, ref = g[f"c{c}_params"], g[f"c{c}_eta"], g[f"c{c}_delta"]
        seg = np.zeros(len(p), np.int32)
        for prec, tol in ((gg.PREC_FP64, 1e-8), (gg.PREC_MIXED, 2e-3)):
            got, st = engine.noise_eta_host(seg, p, e[:, :2], e[:, 2:], precision=prec)
            assert (st == 0).all()
            np.testing.assert_allclose(got, ref, atol=tol)


def test_dlogl_channels_split_term_y(engine, golden, port):
    """term_ch sums to term_y, and each channel matches the oracle's per-channel
    sums over the template's bins."""
    import torch

    g = golden("noise_eta.npz")
    engine.upload(_eta_bank(g, 0))
    p = g["c0_params"]
    q = int(g["c0_qmin"])
    n = len(p)
    for prec, tol in ((gg.PREC_FP64, 1e-9), (gg.PREC_MIXED, 1e-3)):
        dseg = torch.zeros(n, dtype=torch.int32, device="cuda")
        dp = torch.tensor(p, device="cuda")
        dl, ty = torch.empty(n, dtype=torch.float64, device="cuda"), torch.empty(n, dtype=torch.float64, device="cuda")
        tch = torch.empty((n, 2), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        engine.dlogl_channels_device(dseg, dp, dl, tch, term_y=ty, precision=prec)
        torch.cuda.synchronize()
        tch, ty = tch.cpu().numpy(), ty.cpu().numpy()
        np.testing.assert_allclose(tch.sum(1), ty, rtol=1e-12, atol=1e-9)
        for i in range(n):
            dA, dE = g["c0_dA"], g["c0_dE"]
            al = port.alignment(T, 1024, q, p[i])
            N, i0 = int(al[0]), int(al[3])
            h = port.waveform(p[i], N, T)
            ref = [0.0, 0.0]
            for ch, (d, hc, ic) in enumerate(((dA, h[3], g["c0_invCA"]), (dE, h[4], g["c0_invCE"]))):
                for k in range(N):
                    j = i0 + k
                    if 0 <= j < 1024:
                        r = d[2 * j:2 * j + 2]
                        hh = hc[2 * k:2 * k + 2]
                        ref[ch] -= (((r - hh) ** 2).sum() - (r ** 2).sum()) * ic[j]
            np.testing.assert_allclose(tch[i], ref, atol=tol)
