"""The drop-in entry points with the reference's own signatures
(include/glass_gb300.h, "drop-ins for the wavelet headers"), called with
structs laid out as the reference's struct Orbit and struct Wavelets."""
import ctypes

import numpy as np
import pytest

import glass_gb300 as gg

pytestmark = pytest.mark.gpu
_D = ctypes.POINTER(ctypes.c_double)
_DD = ctypes.POINTER(_D)
REL = 1e-10


class Orbit(ctypes.Structure):
    """utils/src/glass_lisa.h:60-109"""
    _fields_ = [("OrbitFileName", ctypes.c_char * 1024), ("Norb", ctypes.c_int), ("L", ctypes.c_double),
                ("fstar", ctypes.c_double), ("ecc", ctypes.c_double), ("R", ctypes.c_double),
                ("lambda_0", ctypes.c_double), ("kappa_0", ctypes.c_double), ("t", _D), ("x", _DD), ("y", _DD),
                ("z", _DD), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p), ("dz", ctypes.c_void_p),
                ("orbit_function", ctypes.c_void_p)]


class Wavelets(ctypes.Structure):
    """utils/src/glass_wavelet.h:25-75"""
    _fields_ = [("NF", ctypes.c_int), ("NT", ctypes.c_int), ("cadence", ctypes.c_double), ("dt", ctypes.c_double),
                ("df", ctypes.c_double), ("frequency_steps", ctypes.c_int), ("fdot_steps", ctypes.c_int),
                ("d_fdot", ctypes.c_double), ("oversample", ctypes.c_int), ("Omega", ctypes.c_double),
                ("dOmega", ctypes.c_double), ("domega", ctypes.c_double), ("inv_root_dOmega", ctypes.c_double),
                ("B", ctypes.c_double), ("A", ctypes.c_double), ("BW", ctypes.c_double), ("deltaf", ctypes.c_double),
                ("fdot", _D), ("window", _D), ("window_freq_forward", _D), ("norm", ctypes.c_double),
                ("N", ctypes.c_int), ("T", ctypes.c_double), ("kmin", ctypes.c_int), ("kmax", ctypes.c_int),
                ("imin", ctypes.c_int), ("imax", ctypes.c_int), ("n_table", ctypes.c_void_p),
                ("table", ctypes.c_void_p)]


def _p(a):
    return a.ctypes.data_as(_D)


@pytest.fixture(scope="module")
def lib():
    from glass_gb300 import build

    build.build()
    L = gg.load_library()
    L.ucb_waveform_wavelet.argtypes = [ctypes.POINTER(Orbit), ctypes.POINTER(Wavelets), ctypes.c_double,
                                       ctypes.c_double, _D, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int), _D, _D, _D]
    L.wavelet_transform_timefreq.argtypes = [ctypes.POINTER(Wavelets), _D]
    L.wavelet_transform_freq.argtypes = [ctypes.POINTER(Wavelets), _D, _D]
    L.wavelet_transform_inverse_freq.argtypes = [ctypes.POINTER(Wavelets), _D, _D]
    return L


def make_orbit(t, pos):
    o = Orbit()
    o.Norb = len(t)
    keep = [np.ascontiguousarray(t)]
    o.t = _p(keep[0])
    for name, d in (("x", 0), ("y", 1), ("z", 2)):
        rows = [np.ascontiguousarray(pos[s, d]) for s in range(3)]
        keep += rows
        arr = (_D * 3)(*[_p(r) for r in rows])
        keep.append(arr)
        setattr(o, name, ctypes.cast(arr, _DD))
    return o, keep


def make_wavelets(NF, NT, wdt, kmin=0, kmax=0):
    w = Wavelets()
    w.NF, w.NT, w.dt, w.df, w.A, w.kmin, w.kmax = NF, NT, wdt, 1 / (2 * wdt), 0.0, kmin, kmax
    return w


def test_ucb_waveform_wavelet_drop_in(lib, golden, port):
    g = golden("wavelet_waveform.npz")
    grids = {"nf1024": (1024, 2048, 15.0 * 1024, 2.0**21 * 15.0), "nf1536": (1536, 4096, 7680.0, 4096 * 7680.0)}
    for i in (0, 1, 2, 3):
        NF, NT, wdt, Tobs = grids[str(g["grid"][i])]
        t0 = float(g["t0"][i])
        kmin, kmax = int(g["kmin"][i]), int(g["kmax"][i])
        t, pos = port.orbit_grid(Tobs, t0)
        orbit, keep = make_orbit(t, pos)
        w = make_wavelets(NF, NT, wdt, kmin, kmax)
        N = kmax - kmin
        X, Y, Z = np.zeros(N), np.zeros(N), np.zeros(N)
        lst = np.zeros(4 * NT, np.int32)
        nlist = ctypes.c_int()
        p = np.ascontiguousarray(g["params"][i])
        lib.ucb_waveform_wavelet(ctypes.byref(orbit), ctypes.byref(w), Tobs, t0, _p(p),
                                 lst.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.byref(nlist), _p(X), _p(Y),
                                 _p(Z))
        lst = lst[: nlist.value]
        np.testing.assert_array_equal(lst, g[f"list{i}"])
        ref = g[f"xyz{i}"]
        for c, h in enumerate((X, Y, Z)):
            assert np.abs(h[lst] - ref[c]).max() < REL * np.abs(ref[c]).max()


def test_wdm_drop_ins(lib, golden, port):
    g = golden("wdm.npz")
    for NF, NT in ((32, 64), (1536, 8)):
        key = f"{NF}x{NT}"
        w = make_wavelets(NF, NT, 1.0)
        x = np.ascontiguousarray(g[f"x_{key}"]).copy()
        lib.wavelet_transform_timefreq(ctypes.byref(w), _p(x))
        ref = g[f"fwd_{key}"]
        assert np.abs(x - ref).max() < REL * np.abs(ref).max()
        win = port.wdm_window(NF, NT)
        wd = np.ascontiguousarray(g[f"w_{key}"])
        freq = np.zeros(NF * NT + 2)
        lib.wavelet_transform_inverse_freq(ctypes.byref(w), _p(wd), _p(freq))
        ref = port.wdm_to_freq(NF, NT, win, wd)
        assert np.abs(freq - ref).max() < REL * np.abs(ref).max()
        back = np.zeros(NF * NT)
        lib.wavelet_transform_freq(ctypes.byref(w), _p(ref), _p(back))
        ref2 = port.wdm_from_freq(NF, NT, win, ref)
        assert np.abs(back - ref2).max() < REL * np.abs(ref2).max()
