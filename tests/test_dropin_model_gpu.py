"""Drop-ins for the reference's model, likelihood and Fisher entry points
(include/glass_gb300.h, "drop-ins for the model and likelihood headers"),
called with structs laid out as the reference's struct Data, Source, Model,
Noise and TDI, against the reference's own results (golden vectors made from
its sources) and the oracle: generate_ucb_model + gaussian_log_likelihood and
snr at 1e-10 (tests/golden/likelihood.npz), update_ucb_model against a fresh
generate, ucb_fisher against the reference's finite-difference Fisher matrix
(fisher.npz, fisher_big.npz) with its eigen-decomposition, and
wavelet_transform_timefreq_by_layers against the reference (wdm.npz) and the
oracle."""
import ctypes

import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
T = wl.T_YEAR
REL = 1e-10
from glass_gb300.refstructs import (Keep, Orbit, _D, bind_dropins, make_data, make_model, make_noise,
                                    make_source)

@pytest.fixture(scope="module")
def lib():
    from glass_gb300 import build

    build.build()
    L = bind_dropins(gg.load_library())
    return L


@pytest.fixture(scope="module")
def orbit(lib):
    o = Orbit()
    lib.initialize_analytic_orbit(ctypes.byref(o))
    return o


def test_generate_model_likelihood_and_snr_match_reference(lib, orbit, golden):
    g = golden("likelihood.npz")
    for k in range(int(g["ncase"])):
        c = {key[len(f"c{k}_"):]: g[key] for key in g.files if key.startswith(f"c{k}_")}
        keep = Keep()
        noise = make_noise(keep, c["invCA"], c["invCE"])
        data = make_data(keep, 1024, int(c["qmin"]), c["dA"], c["dE"], noise)
        for j, p in enumerate(c["props"]):
            model, srcs = make_model(keep, [p] + list(c["extra"]), 1024, noise)
            lib.generate_ucb_model(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(model), -1)
            ll = lib.gaussian_log_likelihood(ctypes.byref(data), ctypes.byref(model))
            assert abs(ll - c["logL"][j]) < REL * max(1.0, abs(c["logL"][j])), (k, j, ll, c["logL"][j])
            s = lib.snr(ctypes.byref(srcs[0]), ctypes.byref(noise))
            assert abs(s - c["snr"][j]) < REL * max(1.0, c["snr"][j]), (k, j, s, c["snr"][j])
            # the alignment the reference's own rule gives
            assert srcs[0].BW == 2 * gg.ucb_bandwidth(orbit.L, orbit.fstar, p[0] / T, p[7] / T / T, p[1],
                                                      np.exp(p[3]), T, 1024)
            assert srcs[0].imin == srcs[0].qmin - int(c["qmin"])


def test_update_model_matches_fresh_generate(lib, orbit, golden):
    """update_ucb_model (remove the current source's template from the
    proposed model, add the proposed one) gives the model and likelihood that
    generate_ucb_model gives for the proposed parameters."""
    g = golden("likelihood.npz")
    c = {key[3:]: g[key] for key in g.files if key.startswith("c1_")}
    keep = Keep()
    noise = make_noise(keep, c["invCA"], c["invCE"])
    data = make_data(keep, 1024, int(c["qmin"]), c["dA"], c["dE"], noise)
    extra = list(c["extra"])
    for j in range(1, 4):
        p = c["props"][j]
        mx, _ = make_model(keep, [c["props"][0]] + extra, 1024, noise)
        my, _ = make_model(keep, [c["props"][0]] + extra, 1024, noise)
        for m in (mx, my):
            lib.generate_ucb_model(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(m), -1)
        sy = my.source[0].contents
        for q in range(8):
            sy.params[q] = p[q]
        lib.update_ucb_model(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(mx), ctypes.byref(my), 0)
        ll = lib.gaussian_log_likelihood(ctypes.byref(data), ctypes.byref(my))
        assert abs(ll - c["logL"][j]) < REL * max(1.0, abs(c["logL"][j]))
        mf, _ = make_model(keep, [p] + extra, 1024, noise)
        lib.generate_ucb_model(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(mf), -1)
        A = np.ctypeslib.as_array(my.tdi.contents.A, (2048,))
        Af = np.ctypeslib.as_array(mf.tdi.contents.A, (2048,))
        assert np.abs(A - Af).max() < 1e-12 * np.abs(Af).max()


def test_fourier_nwip_is_the_reference_sum(lib):
    rng = np.random.default_rng(5)
    a, b, w = rng.standard_normal(64), rng.standard_normal(64), rng.uniform(0.5, 2, 32)
    ref = 0.0
    for n in range(32):
        ref += (a[2 * n] * b[2 * n] + a[2 * n + 1] * b[2 * n + 1]) * w[n]
    got = lib.fourier_nwip(a.ctypes.data_as(_D), b.ctypes.data_as(_D), w.ctypes.data_as(_D), 32)
    assert got == 2.0 * ref


@pytest.mark.parametrize("name", ["fisher.npz", "fisher_big.npz"])
def test_ucb_fisher_dropin_matches_reference(lib, orbit, golden, name):
    g = golden(name)
    NFFT = g["invC"].shape[1]
    for k in range(len(g["params"])):
        keep = Keep()
        invC = g["invC"][k]
        noise = make_noise(keep, invC, invC)
        data = make_data(keep, NFFT, int(g["qmin"][k]), np.zeros(2 * NFFT), np.zeros(2 * NFFT), noise)
        src = make_source(keep, g["params"][k], 2 * NFFT)
        lib.ucb_fisher(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(src), ctypes.byref(noise))
        F = np.array([[src.fisher_matrix[i][j] for j in range(8)] for i in range(8)])
        ref = g["F"][k]
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        assert (np.abs(F - ref) / scale).max() < 1e-3, (name, k)
        # eigen-decomposition: sorted, unit vectors, reconstructs F
        ev = np.array([src.fisher_evalue[i] for i in range(8)])
        V = np.array([[src.fisher_evectr[i][j] for j in range(8)] for i in range(8)])
        assert (np.diff(ev) <= 0).all()
        np.testing.assert_allclose(np.linalg.norm(V, axis=0), 1.0, rtol=1e-12)
        np.testing.assert_allclose(V @ np.diag(ev) @ V.T, F, rtol=0, atol=1e-10 * np.abs(F).max())
        np.testing.assert_allclose(ev, np.sort(np.linalg.eigvalsh(F))[::-1], rtol=1e-9,
                                   atol=1e-12 * np.abs(ev).max())


def test_matrix_eigenstuff_small_eigenvalues(lib):
    """Graded spectrum over 14 decades: every eigenvalue to full relative
    accuracy (Jacobi rotations keep it; the Fisher matrices of loud sources
    span that range)."""
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.standard_normal((8, 8)))
    lam = 10.0 ** np.linspace(10, -4, 8)
    D = np.diag(np.sqrt(lam))
    M = D @ (Q @ np.diag(rng.uniform(0.5, 2, 8)) @ Q.T) @ D
    keep = Keep()
    m = keep.ptrs(M)
    V = keep.ptrs(np.zeros((8, 8)))
    ev = np.zeros(8)
    lib.matrix_eigenstuff(m, V, ev.ctypes.data_as(_D), 8)
    ref = np.sort(np.linalg.eigvalsh(M))[::-1]
    np.testing.assert_allclose(ev, ref, rtol=1e-8)


def test_by_layers_dropin_matches_reference_and_oracle(lib, golden, port):
    g = golden("wdm.npz")
    win = gg.wdm_window(64, 32)
    x = np.array(g["layers_in"])
    w = (ctypes.c_int * 64)(64, 32)  # struct Wavelets begins with NF, NT
    lib.wavelet_transform_timefreq_by_layers(ctypes.cast(w, ctypes.c_void_p), 10, 3, win.ctypes.data_as(_D),
                                             x.ctypes.data_as(_D))
    ref = g["layers_out"]
    assert np.abs(x - ref).max() < 1e-10 * np.abs(ref).max()
    # a config-3 sized grid with a radix-3 length (2 layers: 3 NT samples)
    rng = np.random.default_rng(4)
    for NF, NT, jmin, NL in ((1024, 2048, 100, 2), (1024, 2048, 1, 1)):
        win = gg.wdm_window(NF, NT)
        x = rng.standard_normal(NT * (NL + 1))
        ref = port.wdm_by_layers(NF, NT, jmin, NL, win, x.copy())
        w = (ctypes.c_int * 64)(NF, NT)
        lib.wavelet_transform_timefreq_by_layers(ctypes.cast(w, ctypes.c_void_p), jmin, NL,
                                                 win.ctypes.data_as(_D), x.ctypes.data_as(_D))
        assert np.abs(x - ref).max() < 1e-10 * np.abs(ref).max(), (NF, NT, NL)
