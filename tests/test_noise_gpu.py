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
