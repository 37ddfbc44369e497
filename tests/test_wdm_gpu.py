"""Parity of the CUDA WDM transforms with the reference (golden vectors) and
with the oracle, through the C ABI.

FP64: the largest coefficient error is below 1e-10 of the largest coefficient
(the FFT orderings differ from kissfft's, so agreement is to rounding, about
1e-14).  FP32 (GLASS_PREC_MIXED): below 2e-5 of the largest coefficient.
The round trip forward -> inverse reconstructs the series (the WDM basis is
orthonormal): to 1e-12 in FP64.
"""
import numpy as np
import pytest

import glass_gb300 as gg

pytestmark = pytest.mark.gpu
REL64 = 1e-10
REL32 = 2e-5
GOLDEN_GRIDS = [(32, 64), (48, 64), (16, 256), (1536, 8)]


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def rel_err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("grid", GOLDEN_GRIDS)
def test_forward_matches_reference(engine, golden, grid):
    NF, NT = grid
    g = golden("wdm.npz")
    key = f"{NF}x{NT}"
    got = engine.wdm_forward_host(NF, NT, g[f"x_{key}"])
    assert rel_err(got, g[f"fwd_{key}"]) < REL64
    got32 = engine.wdm_forward_host(NF, NT, g[f"x_{key}"], precision=gg.PREC_MIXED)
    assert rel_err(got32, g[f"fwd_{key}"]) < REL32


@pytest.mark.parametrize("grid", GOLDEN_GRIDS)
def test_inverse_matches_reference(engine, golden, grid):
    NF, NT = grid
    g = golden("wdm.npz")
    key = f"{NF}x{NT}"
    got = engine.wdm_inverse_host(NF, NT, g[f"w_{key}"])
    assert rel_err(got, g[f"inv_{key}"]) < REL64
    got32 = engine.wdm_inverse_host(NF, NT, g[f"w_{key}"], precision=gg.PREC_MIXED)
    assert rel_err(got32, g[f"inv_{key}"]) < REL32


@pytest.mark.parametrize("grid,A,nx", [((64, 96), 0.0, 6.0), ((24, 128), 0.0, 4.0), ((32, 64), 0.01, 4.0),
                                       ((1536, 24), 0.0, 6.0)])
def test_other_grids_and_windows_match_oracle(engine, port, grid, A, nx):
    """Radix-3 grids (NT = 96, NF = 24, 1536) and non-default windows."""
    NF, NT = grid
    A = A * np.pi / NF  # fraction of the layer half-width
    rng = np.random.default_rng(NF * NT)
    x = rng.standard_normal(NF * NT)
    win = port.wdm_window(NF, NT, A, nx)
    np.testing.assert_allclose(gg.wdm_window(NF, NT, A, nx), win, rtol=0, atol=1e-15 * np.abs(win).max())
    ref = port.wdm_forward(NF, NT, win, x)
    assert rel_err(engine.wdm_forward_host(NF, NT, x, A=A, nx=nx), ref) < REL64
    w = rng.standard_normal(NF * NT)
    ref_inv = port.wdm_inverse(NF, NT, win, w)
    assert rel_err(engine.wdm_inverse_host(NF, NT, w, A=A, nx=nx), ref_inv) < REL64


def test_full_grid_forward_matches_oracle_and_round_trips(engine, port):
    """The 2^21-sample grid of 1024 layers x 2048 pixels with nx = 4."""
    NF, NT, nx = 1024, 2048, 4.0
    rng = np.random.default_rng(7)
    x = rng.standard_normal(NF * NT)
    win = port.wdm_window(NF, NT, 0.0, nx)
    ref = port.wdm_forward(NF, NT, win, x)
    got = engine.wdm_forward_host(NF, NT, x, nx=nx)
    assert rel_err(got, ref) < REL64
    back = engine.wdm_inverse_host(NF, NT, got, nx=nx)
    assert np.abs(back - x).max() < 1e-12 * np.abs(x).max()
    # orthonormal basis: energy is kept
    assert abs(np.sum(got**2) / np.sum(x**2) - 1) < 1e-12
    got32 = engine.wdm_forward_host(NF, NT, x, nx=nx, precision=gg.PREC_MIXED)
    assert rel_err(got32, ref) < REL32
    back32 = engine.wdm_inverse_host(NF, NT, got32, nx=nx, precision=gg.PREC_MIXED)
    assert np.abs(back32 - x).max() < REL32 * np.abs(x).max()


def test_reference_default_grid_round_trip(engine):
    """The reference's own grid for a year at 5 s cadence: 1536 layers x 4096
    pixels (M = 3 * 2^20 packed samples)."""
    NF, NT = 1536, 4096
    rng = np.random.default_rng(11)
    x = rng.standard_normal(NF * NT)
    w = engine.wdm_forward_host(NF, NT, x)
    back = engine.wdm_inverse_host(NF, NT, w)
    assert np.abs(back - x).max() < 1e-12 * np.abs(x).max()


def test_impulse_and_pixel_known_answers(engine, port):
    """A unit impulse in time spreads over the layers like the oracle's; a
    single wavelet pixel inverts to the oracle's basis function, and
    transforms back to the same single pixel."""
    NF, NT = 64, 128
    win = port.wdm_window(NF, NT)
    for k in (0, 1, 777, NF * NT - 1):
        x = np.zeros(NF * NT)
        x[k] = 1.0
        assert rel_err(engine.wdm_forward_host(NF, NT, x), port.wdm_forward(NF, NT, win, x)) < REL64
    for n, m in ((0, 0), (1, 0), (5, 3), (64, 31), (127, 63)):
        w = np.zeros(NF * NT)
        w[n + NT * m] = 1.0
        basis = engine.wdm_inverse_host(NF, NT, w)
        assert rel_err(basis, port.wdm_inverse(NF, NT, win, w)) < REL64
        again = engine.wdm_forward_host(NF, NT, basis)
        assert np.abs(again - w).max() < 1e-12


def test_device_pointers_in_place_and_unaligned(engine):
    torch = pytest.importorskip("torch")
    NF, NT = 128, 256
    rng = np.random.default_rng(5)
    x = rng.standard_normal(NF * NT)
    ref = engine.wdm_forward_host(NF, NT, x)
    dev = torch.from_numpy(x).cuda()
    out = torch.empty_like(dev)
    engine.wdm_forward_device(NF, NT, dev, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # in place, as the reference's wavelet_transform_timefreq works
    buf = dev.clone()
    engine.wdm_forward_device(NF, NT, buf, buf)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(buf.cpu().numpy(), ref)
    # 8-byte aligned but not 16-byte aligned input and output
    big = torch.zeros(NF * NT + 1, dtype=torch.float64, device="cuda")
    big[1:] = dev
    out2 = torch.zeros(NF * NT + 1, dtype=torch.float64, device="cuda")
    engine.wdm_forward_device(NF, NT, big[1:], out2[1:])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out2[1:].cpu().numpy(), ref)
    back = torch.zeros(NF * NT + 1, dtype=torch.float64, device="cuda")
    engine.wdm_inverse_device(NF, NT, out2[1:], back[1:])
    torch.cuda.synchronize()
    assert np.abs(back[1:].cpu().numpy() - x).max() < 1e-12 * np.abs(x).max()


def test_unsupported_grids_are_refused(engine):
    c = gg.lib_constants()
    for NF, NT in ((5, 64), (32, 10), (32, 8192), (1, 64)):
        with pytest.raises(gg.GlassError) as e:
            engine.wdm_forward_host(NF, NT, np.zeros(NF * NT))
        assert f"error {c['GLASS_ERR_SIZE']}" in str(e.value)
    with pytest.raises(gg.GlassError) as e:
        engine.wdm_forward_host(32, 64, np.zeros(32 * 64), nx=-1.0)
    assert f"error {c['GLASS_ERR_ARG']}" in str(e.value)
