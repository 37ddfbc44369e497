"""The oracle (oracle/glass_oracle.c) against the reference's own outputs.

The golden vectors were produced by the reference code itself
(tests/golden/make_golden.py); these tests pin the CPU restatement before it
is trusted as the checker for the CUDA path.
"""
import numpy as np
import pytest

from glass_gb300 import workloads as wl

T = wl.T_YEAR
REL = 1e-10


def test_waveforms_match_reference(port, golden):
    g = golden("waveforms.npz")
    for i in range(len(g["N"])):
        fmt, N, NI, t0 = str(g["fmt"][i]), int(g["N"][i]), int(g["NI"][i]), float(g["t0"][i])
        ref = g[f"h{i}"]
        got = port.waveform(g["params"][i], N, T, t0=t0, fmt=fmt, NI=NI)
        chans = range(5) if (fmt == "sangria" or NI > 1) else range(1)
        for c in chans:
            scale = np.abs(ref[c]).max()
            assert scale > 0
            err = np.abs(got[c] - ref[c]).max() / scale
            assert err < REL, (fmt, N, NI, t0, c, err)


def test_bandwidth_rule_is_exact(port, golden):
    g = golden("bandwidth.npz")
    got = np.array([port.bandwidth(g["f"][i], g["fdot"][i], g["costh"][i], g["amp"][i], T, int(g["nfft"][i]))
                    for i in range(len(g["f"]))])
    np.testing.assert_array_equal(got, g["bw"])
    al = np.array([port.alignment(T, 1024, int(g["align_qmin"][i]), g["align_params"][i])
                   for i in range(len(g["align_qmin"]))])
    np.testing.assert_array_equal(al, g["align"])


def test_noise_psd(port, golden):
    g = golden("bandwidth.npz")
    np.testing.assert_allclose(port.aenoise_ff(g["noise_f"]), g["noise_S"], rtol=1e-14)
    # the numpy restatement used to build synthetic segments agrees as well
    np.testing.assert_allclose(wl.aenoise_ff(g["noise_f"]), g["noise_S"], rtol=1e-13)


def _residual(port, case):
    """data minus the extra (non-proposed) sources of the case."""
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


def test_delta_loglikelihood_matches_reference(port, golden):
    g = golden("likelihood.npz")
    for k in range(int(g["ncase"])):
        case = {key[len(f"c{k}_"):]: g[key] for key in g.files if key.startswith(f"c{k}_")}
        rA, rE = _residual(port, case)
        terms = [port.dlogl_term(p, T, 1024, int(case["qmin"]), rA, rE, case["invCA"], case["invCE"])
                 for p in case["props"]]
        logL = case["logL"]
        for j in range(1, len(logL)):
            d_ref = logL[j] - logL[0]
            d_got = terms[j][0] - terms[0][0]
            tol = REL * max(1.0, abs(logL[j]))
            assert abs(d_got - d_ref) < tol, (k, j, d_got, d_ref)
        if len(case["extra"]) == 0:
            # term is logL(with source) - logL(empty model)
            for j in range(len(logL)):
                assert abs(terms[j][0] - (logL[j] - case["logL_empty"])) < REL * max(1.0, abs(logL[j]))


def test_fisher_matches_reference(port, golden):
    g = golden("fisher.npz")
    for k in range(len(g["params"])):
        F = port.fisher(g["params"][k], T, 1024, int(g["qmin"][k]), g["invC"][k], g["invC"][k])
        ref = g["F"][k]
        scale = np.abs(np.diag(ref))
        err = np.abs(F - ref) / np.sqrt(np.outer(scale, scale))
        assert err.max() < 1e-5, err.max()


def test_fft_convention(port):
    """kiss_fft forward convention: X[k] = sum x[n] exp(-2 pi i k n / N); an
    impulse transforms to all ones (apps/src/fft_wdm_unit_tests.c:473-490)."""
    rng = np.random.default_rng(1)
    for N in (32, 256, 4096):
        z = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        np.testing.assert_allclose(port.fft(z), np.fft.fft(z), rtol=1e-12, atol=1e-12 * np.abs(z).sum())
        imp = np.zeros(N, complex)
        imp[0] = 1
        np.testing.assert_allclose(port.fft(imp), np.ones(N), atol=1e-14)


def test_wdm_matches_reference(port, golden):
    """WDM window, forward (utils/src/glass_wavelet.c:293-303, 410-460) and
    inverse (:351-405 plus the inverse real FFT) on the reference's outputs."""
    g = golden("wdm.npz")
    for NF, NT in g["grids"]:
        key = f"{NF}x{NT}"
        win = port.wdm_window(int(NF), int(NT))
        np.testing.assert_allclose(win, g[f"win_{key}"], rtol=1e-13, atol=1e-15 * np.abs(win).max())
        np.testing.assert_allclose(port.wdm_window(int(NF), int(NT), forward=False), g[f"winv_{key}"], rtol=1e-13)
        fwd = port.wdm_forward(int(NF), int(NT), win, g[f"x_{key}"])
        ref = g[f"fwd_{key}"]
        assert np.abs(fwd - ref).max() < 1e-10 * np.abs(ref).max()
        inv = port.wdm_inverse(int(NF), int(NT), win, g[f"w_{key}"])
        ref = g[f"inv_{key}"]
        assert np.abs(inv - ref).max() < 1e-10 * np.abs(ref).max()
    win = port.wdm_window(64, 32)
    out = port.wdm_by_layers(64, 32, 10, 3, win, g["layers_in"])
    assert np.abs(out - g["layers_out"]).max() < 1e-10 * np.abs(g["layers_out"]).max()


@pytest.mark.parametrize("NF,NT", [(32, 64), (48, 64), (1536, 8)])
def test_wdm_impulse_known_answers(port, NF, NT):
    """The reference's own WDM convention checks (apps/src/fft_wdm_unit_tests.c:547-586):
    WDM(impulse) taken back to the frequency domain is the impulse's FFT (all
    ones), and the inverse transform recovers the impulse."""
    ND = NF * NT
    win = port.wdm_window(NF, NT)
    imp = np.zeros(ND)
    imp[0] = 1.0
    w = port.wdm_forward(NF, NT, win, imp)
    f = port.wdm_to_freq(NF, NT, win, w)
    ref = np.zeros(ND + 2)
    ref[0::2] = 1.0
    np.testing.assert_allclose(f, ref, rtol=1e-5, atol=1e-10)
    np.testing.assert_allclose(port.wdm_inverse(NF, NT, win, w), imp, atol=1e-10)


WAVELET_GRIDS = {"nf1024": (1024, 2048, 15.0 * 1024, 2.0**21 * 15.0), "nf1536": (1536, 4096, 7680.0, 4096 * 7680.0)}


def test_interpolated_orbit_grid(port, golden):
    g = golden("wavelet_waveform.npz")
    t, pos = port.orbit_grid(WAVELET_GRIDS["nf1024"][3], 0.0)
    np.testing.assert_array_equal(t, g["orbit_t"])
    np.testing.assert_array_equal(pos, g["orbit_pos"])


def test_wavelet_waveform_matches_reference(port, golden):
    """ucb_waveform_wavelet: same pixel list; values to the FFT's rounding."""
    g = golden("wavelet_waveform.npz")
    for i in range(len(g["grid"])):
        NF, NT, wdt, Tobs = WAVELET_GRIDS[str(g["grid"][i])]
        lst, xyz, _, _ = port.wavelet_waveform(g["params"][i], Tobs, float(g["t0"][i]), NF, NT, wdt, 1 / (2 * wdt),
                                               int(g["kmin"][i]), int(g["kmax"][i]))
        np.testing.assert_array_equal(lst, g[f"list{i}"])
        ref = g[f"xyz{i}"]
        assert np.abs(xyz[:, lst] - ref).max() / np.abs(ref).max() < 1e-12, i


def test_wavelet_likelihoods_match_reference(port, golden):
    """delta_log_likelihood, gaussian_log_likelhood_wavelet and snr_wavelet."""
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = WAVELET_GRIDS[str(g["grid"])]
    edge = int(g["edge"])
    for c in range(int(g["ncase"])):
        kmin, kmax = int(g[f"c{c}_kmin"]), int(g[f"c{c}_kmax"])
        d = g[f"c{c}_d"]
        invC = wl.wavelet_invC(kmax - kmin, NT, kmin, float(g[f"c{c}_scale"]))
        lx, hx, _, _ = port.wavelet_waveform(g[f"c{c}_inj"], Tobs, 0.0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)
        for q, p in enumerate(g[f"c{c}_props"]):
            ly, hy, _, _ = port.wavelet_waveform(p, Tobs, 0.0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)
            dl = port.wavelet_delta_logl(d, invC, hx, lx, hy, ly)
            ref = g[f"c{c}_dlogl"][q]
            assert abs(dl - ref) < 1e-10 * max(1.0, abs(ref)), (c, q, dl, ref)
            full = port.wavelet_logl_full(NT, kmin, edge, NT - edge, d, hy, ly, invC)
            ref = g[f"c{c}_logl_full"][q]
            assert abs(full - ref) < 1e-10 * max(1.0, abs(ref)), (c, q)
            snr = port.wavelet_snr(hy, ly, invC)
            assert abs(snr - g[f"c{c}_snr"][q]) < 1e-10 * g[f"c{c}_snr"][q]


# ------------------------------------------------------------- F-statistic
def _fstat_case(g, c):
    return (str(g[f"c{c}_fmt"]), int(g[f"c{c}_qmin"]), g[f"c{c}_dA"], g[f"c{c}_dE"], g[f"c{c}_invCA"],
            g[f"c{c}_cells"], g[f"c{c}_out"])


def assert_fstat_close(got, ref, rel=1e-11, ang=1e-10):
    """got, ref: rows of (logL_AE, A, iota, psi, phase).  logL and A to a
    relative tolerance, the angles to an absolute one; NaN where the
    reference has NaN (no filter bin inside the segment)."""
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    for k in (0, 1):
        m = ok[:, k]
        scale = np.maximum(np.abs(ref[m, k]), np.abs(ref[m, k]).max() * 1e-6 if m.any() else 0)
        scale = np.where(scale > 0, scale, 1.0)
        err = np.abs(got[m, k] - ref[m, k]) / scale
        assert err.max(initial=0) < rel, (k, err.max())
    for k in (2, 3, 4):
        m = ok[:, k]
        d = np.abs(got[m, k] - ref[m, k])
        if k == 4:  # phase is defined mod 2 pi
            d = np.minimum(d, 2 * np.pi - d)
        assert d.max(initial=0) < ang, (k, d.max())


def test_fstat_matches_reference(port, golden):
    """get_Fstat_logL (ucb/src/glass_ucb_fstatistic.c:646): logL_AE and the
    maximum-likelihood A, iota, psi, phase, in all three TDI formats, with
    template sizes from 16 to 512 and cells beyond both segment edges."""
    g = golden("fstat.npz")
    sizes = set()
    for c in range(int(g["ncase"])):
        fmt, qmin, dA, dE, iA, cells, ref = _fstat_case(g, c)
        got = port.fstat_batch(T, 1024, [qmin], dA, dE, iA, np.zeros(len(cells), np.int32), cells, fmt=fmt)
        assert_fstat_close(got, ref[:, 1:])
        sizes |= {port.bandwidth(x[0], x[1], np.cos(x[2]), 1e-22, T, 1024) for x in cells}
    assert {16, 32, 64, 128, 256, 512} <= sizes


def test_fstat_proposal_matches_reference(port, golden):
    """build_fstatistic_proposal (ucb/src/glass_ucb_proposal.c:1085): the
    normalised density over a 63 x 4 x 5 grid, its norm and maximum."""
    g = golden("fstat.npz")
    tensor, norm, maxp = port.fstat_proposal(T, 64, int(g["p_qmin"]), g["p_dA"], g["p_dE"], g["p_invCA"],
                                             int(g["p_n_theta"]), int(g["p_n_phi"]))
    assert tensor.shape == g["p_tensor"].shape
    np.testing.assert_allclose(tensor, g["p_tensor"], rtol=1e-11)
    assert abs(norm - float(g["p_norm"])) < 1e-11 * abs(float(g["p_norm"]))
    assert abs(maxp - float(g["p_maxp"])) < 1e-11 * abs(float(g["p_maxp"]))


def test_invert4_against_numpy(port):
    rng = np.random.default_rng(4)
    for _ in range(50):
        a = rng.standard_normal((4, 4))
        m = a @ a.T + 0.1 * np.eye(4)
        np.testing.assert_allclose(port.invert4(m), np.linalg.inv(m), rtol=1e-9, atol=1e-12)


# ---------------------------------------------------------- noise likelihood
def test_noise_likelihood_matches_reference(port, golden):
    """The noise module's XYZ likelihood (noise/src/glass_noise_model.c:389,
    :612, :1243; utils/src/glass_math.c:240): instrument only and with the
    galactic foreground, in four frequency bands."""
    g = golden("noise.npz")
    for c in range(int(g["ncase"])):
        fmin = int(g[f"c{c}_qmin"]) / T
        X, Y, Z = g[f"c{c}_X"], g[f"c{c}_Y"], g[f"c{c}_Z"]
        got = port.noise_logl(T, fmin, X, Y, Z, g[f"c{c}_inst"])
        np.testing.assert_allclose(got, g[f"c{c}_logl_inst"], rtol=1e-13)
        got = port.noise_logl(T, fmin, X, Y, Z, g[f"c{c}_inst"], g[f"c{c}_sgal"])
        np.testing.assert_allclose(got, g[f"c{c}_logl_gal"], rtol=1e-13)


def test_noise_wavelet_likelihood_matches_reference(port, golden):
    """my_noise_log_likelihood_wavelet_coarse (noise/src/glass_noise_model.c:1211)
    after the wavelet-domain instrument/foreground models and the stationary or
    modulated coarse covariance, at Q = 1 and 8, in two bands; and the cell
    statistics of coarse_grain_wavelet_data (:1057)."""
    g = golden("noise_wavelet.npz")
    NF, NT, df = int(g["NF"]), int(g["NT"]), float(g["df"])
    for c in range(int(g["ncase"])):
        Q, lmin, b = int(g[f"c{c}_Q"]), int(g[f"c{c}_lmin"]), int(g[f"c{c}_band"])
        P = port.noise_coarse_stats(NT, Q, g[f"b{b}_X"], g[f"b{b}_Y"], g[f"b{b}_Z"])
        for mode in (0, 1, 2):
            got = port.noise_wavelet_logl(NF, NT, df, lmin, P, Q, g[f"c{c}_inst"], g[f"c{c}_sgal"], mode,
                                          g[f"c{c}_mod"] if mode == 2 else None)
            np.testing.assert_allclose(got, g[f"c{c}_logl{mode}"], rtol=1e-13)


def _residual_minus_template(port, q, dA, dE, p, NFFT=1024):
    al = port.alignment(T, NFFT, q, p)
    N, i0 = int(al[0]), int(al[3])
    h = port.waveform(p, N, T)
    rA, rE = dA.copy(), dE.copy()
    for k in range(N):
        j = i0 + k
        if 0 <= j < NFFT:
            rA[2 * j:2 * j + 2] -= h[3][2 * k:2 * k + 2]
            rE[2 * j:2 * j + 2] -= h[4][2 * k:2 * k + 2]
    return rA, rE


def test_noise_step_matches_reference(port, golden):
    """noise_model_mcmc's likelihood change (ucb/src/glass_ucb_sampler.c:29-73)."""
    g = golden("noise_eta.npz")
    for c in range(int(g["ncase"])):
        q = int(g[f"c{c}_qmin"])
        for p, e, ref in zip(g[f"c{c}_params"], g[f"c{c}_eta"], g[f"c{c}_delta"]):
            rA, rE = _residual_minus_template(port, q, g[f"c{c}_dA"], g[f"c{c}_dE"], p)
            got = port.noise_eta_delta(rA, rE, g[f"c{c}_invCA"], g[f"c{c}_invCE"], e[:2], e[2:])
            assert abs(got - ref) < 1e-9, (c, got, ref)


# ------------------------------------------------------------------ sampler
def _ptmcmc_run(port, g, sweeps):
    NC = int(g["NC"])
    nens = len(g["seed0"])
    index = np.tile(np.arange(NC, dtype=np.int32), (nens, 1))
    seed = g["seed0"].astype(np.uint32).copy()
    acc = np.zeros((nens, NC))
    for _ in range(sweeps):
        port.ptmcmc(g["temperature"], g["logL"], index, seed, acc, g["logLnorm"])
    return index, seed, acc


def test_ptmcmc_matches_reference(port, golden):
    """ptmcmc (utils/src/glass_sampler.c:19-63): permutation, acceptance and the
    chains' seeds after one and after 40 sweeps, exactly."""
    g = golden("sampler.npz")
    for sweeps, tag in ((1, "1"), (int(g["sweeps"]), "N")):
        index, seed, acc = _ptmcmc_run(port, g, sweeps)
        np.testing.assert_array_equal(index, g["index" + tag])
        np.testing.assert_array_equal(seed, g["seed" + tag])
        np.testing.assert_array_equal(acc, g["acc" + tag])


def test_fisher_draw_matches_reference(port, golden):
    """draw_from_fisher (ucb/src/glass_ucb_proposal.c:348-391): four successive
    draws per chain, including reflections at cos = +-1, zero and negative
    eigenvalues and a NaN parameter: seeds and return values exactly, the
    drawn parameters to the last bits of the C library's log."""
    g = golden("fisher_draw.npz")
    seed = g["seed0"].copy()
    for k in range(4):
        y, logQ = port.fisher_draw(g["x"], g["evec"], g["evalue"], seed)
        np.testing.assert_array_equal(seed, g["seeds"][k])
        np.testing.assert_array_equal(logQ, g["logQ"][k])
        np.testing.assert_allclose(y, g["y"][k], rtol=1e-14, atol=0)
