"""The stochastic-background (SGWB) part of the noise-model likelihood:
the reference's own generate_sgwb_model / generate_sgwb_model_wavelet with
the three spectral templates, combined with the instrument and foreground as
its samplers do (tests/golden/sgwb.npz, made from the reference's sources
with a synthetic response table).  The oracle against the goldens runs on the
CPU; the GPU kernels against the goldens and the oracle are marked gpu."""
import numpy as np
import pytest

from glass_gb300 import workloads as wl

T = wl.T_YEAR
REL = 1e-10


def _close(got, ref, rel=REL):
    got, ref = np.asarray(got), np.asarray(ref)
    return np.abs(got - ref).max() <= rel * np.abs(ref).max()


def test_oracle_sgwb_covariance_matches_reference(golden, port):
    g = golden("sgwb.npz")
    f = g["fgrid"]
    R = port.sgwb_response(g["resp"], f)
    for t in range(3):
        for k in range(4):
            S = np.array([port.sgwb_psd(t, fi, g[f"t{t}_params"][k]) for fi in f])
            C = (R * S).T
            ref = g[f"t{t}_C"][k]
            # NaN where the reference's spectrum is NaN (a phase transition
            # with b + 4 < m at low frequency), equal to 1e-12 elsewhere
            np.testing.assert_array_equal(np.isnan(C), np.isnan(ref))
            fin = np.isfinite(ref)
            assert np.abs(C[fin] - ref[fin]).max() <= 1e-12 * np.abs(ref[fin]).max(), (t, k)


def test_oracle_sgwb_likelihood_matches_reference(golden, port):
    g = golden("sgwb.npz")
    resp = g["resp"]
    for c in range(2):
        fmin = int(g[f"c{c}_qmin"]) / T
        X, Y, Z = g[f"c{c}_X"], g[f"c{c}_Y"], g[f"c{c}_Z"]
        for t in range(3):
            sg = g[f"c{c}_t{t}_sgwb"]
            got = port.noise_logl_sgwb(T, fmin, X, Y, Z, g[f"c{c}_inst"], g[f"c{c}_sgal"], t, sg, resp)
            assert _close(got, g[f"c{c}_t{t}_logl"]), (c, t)
            got = port.noise_logl_sgwb(T, fmin, X, Y, Z, g[f"c{c}_inst"], None, t, sg, resp)
            assert _close(got, g[f"c{c}_t{t}_logl_inst"]), (c, t)
    NF, NT, df, lmin = int(g["NF"]), int(g["NT"]), float(g["df"]), int(g["lmin"])
    for Q in (1, 8):
        P = port.noise_coarse_stats(NT, Q, g["w_X"], g["w_Y"], g["w_Z"])
        for t in range(3):
            for mode in (0, 1, 2):
                got = port.noise_wavelet_logl_sgwb(NF, NT, df, lmin, P, Q, g["w_inst"], g["w_sgal"], mode,
                                                   g[f"w_Q{Q}_mod"] if mode == 2 else None, t,
                                                   g[f"w_Q{Q}_t{t}_sgwb"], g["resp"])
                assert _close(got, g[f"w_Q{Q}_t{t}_logl{mode}"]), (Q, t, mode)


def test_background_changes_the_likelihood(golden, port):
    """The fixtures discriminate: the background moves logL by far more than
    the test tolerance (so a kernel that dropped it would fail)."""
    g = golden("sgwb.npz")
    c = 1
    fmin = int(g[f"c{c}_qmin"]) / T
    X, Y, Z = g[f"c{c}_X"], g[f"c{c}_Y"], g[f"c{c}_Z"]
    base = port.noise_logl(T, fmin, X, Y, Z, g[f"c{c}_inst"], g[f"c{c}_sgal"])
    for t in range(3):
        ref = g[f"c{c}_t{t}_logl"]
        assert np.abs(ref - base).min() > 1e3 * REL * np.abs(ref).max(), t


@pytest.fixture(scope="module")
def engine():
    import glass_gb300 as gg
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


@pytest.mark.gpu
def test_gpu_sgwb_likelihood_matches_reference(engine, golden):
    g = golden("sgwb.npz")
    for c in range(2):
        q = int(g[f"c{c}_qmin"])
        engine.noise_setup(T, q, g[f"c{c}_X"], g[f"c{c}_Y"], g[f"c{c}_Z"])
        for t in range(3):
            engine.noise_sgwb_setup(t, g["resp"])
            sg = g[f"c{c}_t{t}_sgwb"]
            got = engine.noise_logl_host(g[f"c{c}_inst"], g[f"c{c}_sgal"], sgwb=sg)
            assert _close(got, g[f"c{c}_t{t}_logl"]), (c, t, np.abs(got - g[f"c{c}_t{t}_logl"]).max())
            got = engine.noise_logl_host(g[f"c{c}_inst"], None, sgwb=sg)
            assert _close(got, g[f"c{c}_t{t}_logl_inst"]), (c, t)
        # no background: the plain likelihood, unchanged by the template being set
        engine.noise_sgwb_setup(-1)
        got = engine.noise_logl_host(g[f"c{c}_inst"], g[f"c{c}_sgal"])
        assert np.isfinite(got).all()


@pytest.mark.gpu
def test_gpu_sgwb_wavelet_likelihood_matches_reference(engine, golden):
    g = golden("sgwb.npz")
    NF, NT, df, lmin = int(g["NF"]), int(g["NT"]), float(g["df"]), int(g["lmin"])
    for Q in (1, 8):
        engine.noise_wavelet_setup(NF, NT, df, lmin, Q, g["w_X"], g["w_Y"], g["w_Z"], mod=g[f"w_Q{Q}_mod"])
        for t in range(3):
            engine.noise_sgwb_setup(t, g["resp"])
            for mode in (0, 1, 2):
                got = engine.noise_wavelet_logl_host(g["w_inst"], g["w_sgal"], mode=mode, sgwb=g[f"w_Q{Q}_t{t}_sgwb"])
                ref = g[f"w_Q{Q}_t{t}_logl{mode}"]
                assert _close(got, ref), (Q, t, mode, np.abs(got - ref).max())
    engine.noise_sgwb_setup(-1)


@pytest.mark.gpu
def test_gpu_sgwb_batch_matches_oracle(engine, port):
    """A larger batch (256 models over 4096 bins from 1 mHz, every template)
    against the oracle, device pointers through the asynchronous entry point."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    inst0, sgal0 = wl.default_noise_params(T)
    q = int(1e-3 * T)
    X, Y, Z = wl.xyz_from_covariance(rng, port.noise_covariance(T, q / T, 4096, inst0, sgal0))
    engine.noise_setup(T, q, X, Y, Z)
    resp = wl.sgwb_response_table()
    dev = torch.device("cuda", 0)
    inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (256, 12)))
    sgal = sgal0 + rng.uniform(-0.2, 0.2, (256, 5))
    for t in range(3):
        sg = wl.sgwb_params_draw(rng, t, 256)
        engine.noise_sgwb_setup(t, resp)
        out = torch.empty(256, dtype=torch.float64, device=dev)
        engine.noise_logl_device(torch.from_numpy(inst).to(dev), out, sgal=torch.from_numpy(sgal).to(dev),
                                 sgwb=torch.from_numpy(sg).to(dev))
        torch.cuda.synchronize()
        ref = port.noise_logl_sgwb(T, q / T, X, Y, Z, inst, sgal, t, sg, resp)
        assert _close(out.cpu().numpy(), ref), t
    engine.noise_sgwb_setup(-1)
