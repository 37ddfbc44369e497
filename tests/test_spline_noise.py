"""The noise module's one- and two-channel spline noise model
(generate_spline_noise_model + noise_log_likelihood, the likelihood of
noise_spline_model_mcmc / _rjmcmc): tests/golden/spline_noise.npz was made
from the reference's own sources.  The oracle against the goldens runs on the
CPU; the GPU kernel against the goldens and the oracle is marked gpu."""
import numpy as np
import pytest

from glass_gb300 import workloads as wl

T = wl.T_YEAR
REL = 1e-12  # of |logL|: the kernel sums per thread, the reference in bin order
CASES = ("one", "two", "max")


def _case(g, name):
    return (int(g[f"{name}_qmin"]), g[f"{name}_transfer"], g[f"{name}_d"], g[f"{name}_nknots"],
            g[f"{name}_knot_f"], g[f"{name}_knot_C"], g[f"{name}_logl"])


def test_oracle_spline_noise_matches_reference(golden, port):
    g = golden("spline_noise.npz")
    for name in CASES:
        q, tr, d, nk, kf, kC, ref = _case(g, name)
        got = port.spline_noise_logl(T, q / T, d, tr, nk, kf, kC)
        np.testing.assert_array_equal(got, ref, err_msg=name)


def test_spline_changes_the_likelihood(golden, port):
    """The fixtures discriminate: moving one control point by 10% moves logL
    by far more than the tolerance; dropping the spline (transfer alone) by
    far more again."""
    g = golden("spline_noise.npz")
    for name in ("one", "two"):
        q, tr, d, nk, kf, kC, ref = _case(g, name)
        kC2 = kC.copy()
        kC2[:, :, 1] *= 1.1
        got = port.spline_noise_logl(T, q / T, d, tr, nk, kf, kC2)
        assert np.abs(got - ref).min() > 1e4 * REL * np.abs(ref).max(), name
        got = port.spline_noise_logl(T, q / T, d, tr, nk, kf, np.zeros_like(kC))
        assert np.abs(got - ref).min() > 1e5 * REL * np.abs(ref).max(), name


@pytest.fixture(scope="module")
def engine():
    import glass_gb300 as gg
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def _close(got, ref, rel=REL):
    return np.abs(np.asarray(got) - ref).max() <= rel * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_spline_noise_matches_reference(engine, golden):
    g = golden("spline_noise.npz")
    for name in CASES:
        q, tr, d, nk, kf, kC, ref = _case(g, name)
        engine.spline_noise_setup(T, q, tr, d[0], d[1] if len(d) == 2 else None)
        got = engine.spline_noise_logl_host(nk, kf, kC)
        assert _close(got, ref), (name, np.abs(got - ref).max())


@pytest.mark.gpu
def test_gpu_spline_noise_batch_matches_oracle(engine, port):
    """2000 models (2 .. 64 knots) on 8192 bins from 1 mHz, two channels,
    device pointers through the asynchronous entry point; one channel on a
    ragged 777-bin grid through the host entry point."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(41)
    dev = torch.device("cuda", 0)
    q, NFFT = int(1e-3 * T), 8192
    tr, d, ex = wl.spline_noise_data(rng, T, q, NFFT, 2, excess=3.0)
    nk, kf, kC = wl.spline_noise_models(rng, T, q, NFFT, ex, 2000, 64)
    engine.spline_noise_setup(T, q, tr, d[0], d[1])
    out = torch.full((2000,), np.nan, dtype=torch.float64, device=dev)
    engine.spline_noise_logl_device(*(torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (nk, kf, kC)), out)
    torch.cuda.synchronize()
    ref = port.spline_noise_logl(T, q / T, d, tr, nk, kf, kC)
    assert np.isfinite(ref).all()
    assert _close(out.cpu().numpy(), ref)
    q, NFFT = int(5e-3 * T), 777
    tr, d, ex = wl.spline_noise_data(rng, T, q, NFFT, 1)
    nk, kf, kC = wl.spline_noise_models(rng, T, q, NFFT, ex, 50, 30)
    engine.spline_noise_setup(T, q, tr, d[0])
    assert _close(engine.spline_noise_logl_host(nk, kf, kC), port.spline_noise_logl(T, q / T, d, tr, nk, kf, kC))


@pytest.mark.gpu
def test_gpu_spline_noise_argument_errors(engine):
    import glass_gb300 as gg

    rng = np.random.default_rng(43)
    q, NFFT = int(2e-3 * T), 256
    tr, d, ex = wl.spline_noise_data(rng, T, q, NFFT, 1)
    engine.spline_noise_setup(T, q, tr, d[0])
    nk, kf, kC = wl.spline_noise_models(rng, T, q, NFFT, ex, 4, 8)
    assert np.isfinite(engine.spline_noise_logl_host(nk, kf, kC)).all()
    assert len(engine.spline_noise_logl_host(nk[:0], kf[:0], kC[:0])) == 0
    bad = nk.copy()
    bad[2] = 1  # fewer than two knots
    with pytest.raises(gg.GlassError):
        engine.spline_noise_logl_host(bad, kf, kC)
    bad[2] = 9  # more than kmax
    with pytest.raises(gg.GlassError):
        engine.spline_noise_logl_host(bad, kf, kC)
    kf2 = kf.copy()
    kf2[3, 1] = kf2[3, 0]  # repeated knot frequency
    with pytest.raises(gg.GlassError):
        engine.spline_noise_logl_host(nk, kf2, kC)
    big = np.zeros((1, 513))
    big[0, :2] = kf[0, 0], kf[0, 1]
    with pytest.raises(gg.GlassError, match="kmax"):  # kmax above 512
        engine.spline_noise_logl_host(np.array([2], np.int32), big, big[:, None, :])
    with pytest.raises(gg.GlassError):  # two channels without the second
        gg._check(engine.lib.glass_gpu_spline_noise_setup(engine._ctx, 2, T, q, NFFT, gg._pd(tr), gg._pd(d[0]), None))
    # the context keeps its one-channel data
    assert np.isfinite(engine.spline_noise_logl_host(nk, kf, kC)).all()
