"""The noise module's one- and two-channel instrument (+ foreground) models:
Michelson X (generate_instrument_noise_model's case 1) and A/E (case 2) with
noise_log_likelihood (tests/golden/noise_channels.npz, made from the
reference's own sources).  The oracle against the goldens runs on the CPU;
the GPU kernel against the goldens and the oracle is marked gpu."""
import numpy as np
import pytest

from glass_gb300 import workloads as wl

T = wl.T_YEAR
REL = 1e-10  # of |logL|, as the three-channel noise likelihood


def _close(got, ref, rel=REL):
    got, ref = np.asarray(got), np.asarray(ref)
    return np.abs(got - ref).max() <= rel * np.abs(ref).max()


def _cases(g):
    for c in range(3):
        for nch in (1, 2):
            k = f"c{c}_n{nch}"
            yield k, int(g[f"{k}_qmin"]), g[f"{k}_d"], g[f"{k}_inst"], g[f"{k}_sgal"], g[f"{k}_logl"], \
                g[f"{k}_logl_inst"]


def test_oracle_noise_channels_match_reference(golden, port):
    g = golden("noise_channels.npz")
    for k, q, d, inst, sgal, ref, ref_inst in _cases(g):
        np.testing.assert_array_equal(port.noise_logl_channels(T, q / T, d, inst, sgal), ref, err_msg=k)
        np.testing.assert_array_equal(port.noise_logl_channels(T, q / T, d, inst, None), ref_inst, err_msg=k)


def test_noise_channels_discriminate(golden, port):
    """The link levels move the instrument-only logL by far more than the
    tolerance; the foreground moves it too where it is on (below 10 f1)."""
    g = golden("noise_channels.npz")
    for k, q, d, inst, sgal, ref, ref_inst in _cases(g):
        inst2 = inst.copy()
        inst2[:, [0, 6]] *= 1.01  # sacc12, soms12
        got = port.noise_logl_channels(T, q / T, d, inst2, None)
        assert np.abs(got - ref_inst).min() > 1e3 * REL * np.abs(ref_inst).max(), k
        if not k.startswith("c2"):
            assert np.abs(ref - ref_inst).min() > 1e3 * REL * np.abs(ref).max(), k


@pytest.fixture(scope="module")
def engine():
    import glass_gb300 as gg
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


@pytest.mark.gpu
def test_gpu_noise_channels_match_reference(engine, golden):
    g = golden("noise_channels.npz")
    for k, q, d, inst, sgal, ref, ref_inst in _cases(g):
        engine.noise_setup_channels(T, q, *d)
        got = engine.noise_logl_host(inst, sgal)
        assert _close(got, ref), (k, np.abs(got - ref).max())
        got = engine.noise_logl_host(inst, None)
        assert _close(got, ref_inst), (k, np.abs(got - ref_inst).max())


@pytest.mark.gpu
def test_gpu_noise_channels_batch_and_errors(engine, port):
    """A 512-model batch on 4096 two-channel bins from 1 mHz through device
    pointers; SGWB and qmin = 0 refused; three channels again afterwards."""
    import glass_gb300 as gg

    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(53)
    inst0, sgal0 = wl.default_noise_params(T)
    q, N = int(1e-3 * T), 4096
    d = rng.standard_normal((2, 2 * N)) * 3e-21
    engine.noise_setup_channels(T, q, d[0], d[1])
    inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (512, 12)))
    sgal = sgal0 + rng.uniform(-0.2, 0.2, (512, 5))
    dev = torch.device("cuda", 0)
    out = torch.full((512,), np.nan, dtype=torch.float64, device=dev)
    engine.noise_logl_device(torch.from_numpy(inst).to(dev), out, sgal=torch.from_numpy(sgal).to(dev))
    torch.cuda.synchronize()
    assert _close(out.cpu().numpy(), port.noise_logl_channels(T, q / T, d, inst, sgal))
    engine.noise_sgwb_setup(0, wl.sgwb_response_table())
    with pytest.raises(gg.GlassError, match="three channels"):
        engine.noise_logl_host(inst[:4], sgal[:4], sgwb=wl.sgwb_params_draw(rng, 0, 4))
    engine.noise_sgwb_setup(-1)
    with pytest.raises(gg.GlassError):
        engine.noise_setup_channels(T, 0, d[0, :64], d[1, :64])
    X, Y, Z = wl.xyz_from_covariance(rng, port.noise_covariance(T, q / T, 256, inst0, sgal0))
    engine.noise_setup_channels(T, q, X, Y, Z)
    assert _close(engine.noise_logl_host(inst[:8], sgal[:8]), port.noise_logl(T, q / T, X, Y, Z, inst[:8], sgal[:8]))
