"""Drop-ins for the wavelet-domain likelihood and Fisher entry points
(include/glass_gb300.h, "drop-ins for the model and likelihood headers"),
called with structs laid out as the reference's struct Data, Model, Source,
Noise, Orbit and Wavelets:

* wavelet_nwip, snr_wavelet and delta_log_likelihood are host sums in the
  reference's order: checked without a GPU on the oracle's waveforms against
  the reference's own results (tests/golden/wavelet_likelihood.npz);
* ucb_fisher_wavelet runs the batched GPU Fisher kernels: checked against the
  reference's own ucb_fisher_wavelet (tests/golden/fisher_wavelet.npz) with its
  eigen-decomposition."""
import ctypes

import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl
from glass_gb300.refstructs import (Data, Keep, _D, bind_dropins, make_noise_xyz, make_orbit_nodes, make_source,
                                    make_wavelet_model, make_wavelet_tdi, make_wavelets)

REL = 1e-10
WAVELET_GRIDS = {"nf1024": (1024, 2048, 15.0 * 1024, 2.0**21 * 15.0)}


@pytest.fixture(scope="module")
def lib():
    from glass_gb300 import build

    build.build()
    return bind_dropins(gg.load_library())


def test_sparse_likelihood_and_snr_drop_ins_match_reference(lib, golden, port):
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = WAVELET_GRIDS[str(g["grid"])]
    for c in range(int(g["ncase"])):
        kmin, kmax = int(g[f"c{c}_kmin"]), int(g[f"c{c}_kmax"])
        N = kmax - kmin
        keep = Keep()
        invC = wl.wavelet_invC(N, NT, kmin, float(g[f"c{c}_scale"]))
        noise = make_noise_xyz(keep, invC)
        data = Data()
        data.N, data.Nchannel, data.T = N, 3, Tobs
        data.tdi = ctypes.pointer(make_wavelet_tdi(keep, np.ascontiguousarray(g[f"c{c}_d"])))
        lx, hx, _, _ = port.wavelet_waveform(g[f"c{c}_inj"], Tobs, 0.0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)
        mx = make_wavelet_model(keep, hx, lx, noise)
        for q, p in enumerate(g[f"c{c}_props"]):
            ly, hy, _, _ = port.wavelet_waveform(p, Tobs, 0.0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)
            my = make_wavelet_model(keep, hy, ly, noise)
            dl = lib.delta_log_likelihood(ctypes.byref(data), ctypes.byref(mx), ctypes.byref(my))
            ref = g[f"c{c}_dlogl"][q]
            assert abs(dl - ref) < REL * max(1.0, abs(ref)), (c, q, dl, ref)
            src = make_source(keep, p, N, nch=3)
            src.tdi = my.tdi
            src.list, src.Nlist = my.list, my.Nlist
            s = lib.snr_wavelet(ctypes.byref(src), ctypes.byref(noise))
            assert abs(s - g[f"c{c}_snr"][q]) < REL * g[f"c{c}_snr"][q], (c, q)


def test_wavelet_nwip_is_the_reference_sum(lib):
    rng = np.random.default_rng(6)
    a, b, w = rng.standard_normal(100), rng.standard_normal(100), rng.uniform(0.5, 2, 100)
    lst = np.ascontiguousarray(rng.choice(100, 37, replace=False), np.int32)
    ref = 0.0
    for k in lst:
        ref += a[k] * b[k] * w[k]
    got = lib.wavelet_nwip(a.ctypes.data_as(_D), b.ctypes.data_as(_D), w.ctypes.data_as(_D),
                           lst.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(lst))
    assert got == ref


@pytest.mark.gpu
def test_ucb_fisher_wavelet_drop_in_matches_reference(lib, golden, port):
    g = golden("fisher_wavelet.npz")
    NF, NT, wdt, Tobs = (float(x) for x in g["grid"])
    NF, NT = int(NF), int(NT)
    kmin, kmax, imin, imax = int(g["kmin"]), int(g["kmax"]), int(g["imin"]), int(g["imax"])
    N = kmax - kmin
    keep = Keep()
    t, pos = port.orbit_grid(Tobs, 0.0)
    orbit = make_orbit_nodes(keep, t, pos)
    w = make_wavelets(keep, NF, NT, wdt, kmin, kmax, imin, imax)
    noise = make_noise_xyz(keep, wl.wavelet_invC(N, NT, kmin, 1e-22))
    data = Data()
    data.N, data.Nchannel, data.T, data.t0 = N, 3, Tobs, 0.0
    data.wdm = ctypes.cast(ctypes.pointer(w), ctypes.c_void_p)
    for s in range(len(g["params"])):
        src = make_source(keep, g["params"][s], N, nch=3)
        lib.ucb_fisher_wavelet(ctypes.byref(orbit), ctypes.byref(data), ctypes.byref(src), ctypes.byref(noise))
        F = np.array([[src.fisher_matrix[i][j] for j in range(8)] for i in range(8)])
        ref = g["F"][s]
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        assert (np.abs(F - ref) / scale).max() < 1e-6, s
        ev = np.array([src.fisher_evalue[i] for i in range(8)])
        V = np.array([[src.fisher_evectr[i][j] for j in range(8)] for i in range(8)])
        assert (ev > 0).all() and (np.diff(ev) <= 0).all()
        np.testing.assert_allclose(V @ np.diag(ev) @ V.T, F, rtol=0, atol=1e-10 * np.abs(F).max())
