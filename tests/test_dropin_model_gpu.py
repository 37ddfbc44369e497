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
c_int, c_double = ctypes.c_int, ctypes.c_double
_D = ctypes.POINTER(c_double)
_DD = ctypes.POINTER(_D)
_DDD = ctypes.POINTER(_DD)


class TDI(ctypes.Structure):
    """utils/src/glass_lisa.h:116-140"""
    _fields_ = [("X", _D), ("Y", _D), ("Z", _D), ("A", _D), ("E", _D), ("T", _D), ("Nchannel", c_int), ("N", c_int),
                ("delta", c_double)]


class Noise(ctypes.Structure):
    """utils/src/glass_data.h:337-360"""
    _fields_ = [("N", c_int), ("kmin", c_int), ("Nchannel", c_int), ("Nlayer", c_int), ("eta", _D), ("f", _D),
                ("C", _DDD), ("invC", _DDD), ("logdetC", _D), ("transfer", _D)]


class Data(ctypes.Structure):
    """utils/src/glass_data.h:50-97 (through the format string)"""
    _fields_ = [("N", c_int), ("NFFT", c_int), ("Nchannel", c_int), ("Nlayer", c_int), ("logN", c_double),
                ("cseed", ctypes.c_uint), ("nseed", ctypes.c_uint), ("iseed", ctypes.c_uint), ("T", c_double),
                ("sqT", c_double), ("t0", c_double), ("wdm", ctypes.c_void_p), ("qmin", c_int), ("qmax", c_int),
                ("qpad", c_int), ("lmin", c_int), ("lmax", c_int), ("fmin", c_double), ("fmax", c_double),
                ("sine_f_on_fstar", c_double), ("tdi", ctypes.POINTER(TDI)), ("raw", ctypes.POINTER(TDI)),
                ("dft", ctypes.POINTER(TDI)), ("dwt", ctypes.POINTER(TDI)), ("noise", ctypes.POINTER(Noise)),
                ("format", ctypes.c_char * 16)]


class Source(ctypes.Structure):
    """utils/src/glass_model.h:81-121"""
    _fields_ = ([("NP", c_int), ("params", _D), ("tdi", ctypes.POINTER(TDI))]
                + [(k, c_double) for k in ("f0", "dfdt", "d2fdt2", "amp", "psi", "cosi", "phiref", "phi", "costheta",
                                           "dL", "tref", "m1", "m2", "Mchirp", "Mtotal", "chi1", "chi2")]
                + [(k, c_int) for k in ("BW", "qmin", "qmax", "imin", "imax")]
                + [("fisher_matrix", _DD), ("fisher_evectr", _DD), ("fisher_evalue", _D),
                   ("fisher_update_flag", c_int), ("list", ctypes.POINTER(c_int)), ("Nlist", c_int)])


class Model(ctypes.Structure):
    """utils/src/glass_model.h:25-60"""
    _fields_ = [("NP", c_int), ("Nmax", c_int), ("Neff", c_int), ("Nlive", c_int),
                ("source", ctypes.POINTER(ctypes.POINTER(Source))), ("noise", ctypes.POINTER(Noise)),
                ("calibration", ctypes.c_void_p), ("tdi", ctypes.POINTER(TDI)), ("residual", ctypes.POINTER(TDI)),
                ("t0", c_double), ("prior", _DD), ("logPriorVolume", _D), ("logL", c_double),
                ("logLnorm", c_double), ("list", ctypes.POINTER(c_int)), ("Nlist", c_int),
                ("log_likelihood", ctypes.c_void_p), ("generate_signal_model", ctypes.c_void_p)]


class Orbit(ctypes.Structure):
    """utils/src/glass_lisa.h:60-109"""
    _fields_ = [("OrbitFileName", ctypes.c_char * 1024), ("Norb", c_int), ("L", c_double), ("fstar", c_double),
                ("ecc", c_double), ("R", c_double), ("lambda_0", c_double), ("kappa_0", c_double), ("t", _D),
                ("x", _DD), ("y", _DD), ("z", _DD), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("dz", ctypes.c_void_p), ("orbit_function", ctypes.c_void_p)]


class Keep:
    """Holds the numpy arrays behind a struct's pointers."""

    def __init__(self):
        self.refs = []

    def arr(self, a):
        a = np.ascontiguousarray(a, np.float64)
        self.refs.append(a)
        return a.ctypes.data_as(_D)

    def ptrs(self, rows):
        p = (_D * len(rows))(*[self.arr(r) for r in rows])
        self.refs.append(p)
        return ctypes.cast(p, _DD)


def make_tdi(keep, N, nch, A=None, E=None):
    t = TDI()
    t.X, t.Y, t.Z, t.T = (keep.arr(np.zeros(N)) for _ in range(4))
    t.A = keep.arr(np.zeros(N) if A is None else A)
    t.E = keep.arr(np.zeros(N) if E is None else E)
    t.Nchannel, t.N = nch, N
    keep.refs.append(t)
    return t


def make_noise(keep, invCA, invCE):
    n = Noise()
    n.N, n.Nchannel = len(invCA), 2
    rows = [[invCA, np.zeros_like(invCA)], [np.zeros_like(invCA), invCE]]
    outer = (_DD * 2)(*[keep.ptrs(r) for r in rows])
    keep.refs.append(outer)
    n.invC = ctypes.cast(outer, _DDD)
    n.C = n.invC
    keep.refs.append(n)
    return n


def make_data(keep, NFFT, qmin, dA, dE, noise, fmt=b"sangria"):
    d = Data()
    d.N, d.NFFT, d.Nchannel, d.Nlayer = 2 * NFFT, NFFT, 2, 1
    d.T, d.sqT, d.t0 = T, np.sqrt(T), 0.0
    d.qmin, d.qmax = qmin, qmin + NFFT
    d.tdi = ctypes.pointer(make_tdi(keep, 2 * NFFT, 2, dA, dE))
    d.noise = ctypes.pointer(noise)
    d.format = fmt
    keep.refs.append(d)
    return d


def make_source(keep, params, N, nch=2):
    s = Source()
    s.NP = 8
    s.params = keep.arr(np.array(params, np.float64))
    s.tdi = ctypes.pointer(make_tdi(keep, N, nch))
    s.fisher_matrix = keep.ptrs(np.zeros((8, 8)))
    s.fisher_evectr = keep.ptrs(np.zeros((8, 8)))
    s.fisher_evalue = keep.arr(np.zeros(8))
    keep.refs.append(s)
    return s


def make_model(keep, params_list, NFFT, noise):
    m = Model()
    srcs = [make_source(keep, p, 2 * NFFT) for p in params_list]
    arr = (ctypes.POINTER(Source) * max(1, len(srcs)))(*[ctypes.pointer(s) for s in srcs])
    keep.refs.append(arr)
    m.NP, m.Nmax, m.Nlive = 8, len(srcs), len(srcs)
    m.source = ctypes.cast(arr, ctypes.POINTER(ctypes.POINTER(Source)))
    m.noise = ctypes.pointer(noise)
    m.tdi = ctypes.pointer(make_tdi(keep, 2 * NFFT, 2))
    m.residual = ctypes.pointer(make_tdi(keep, 2 * NFFT, 2))
    keep.refs.append(m)
    return m, srcs


@pytest.fixture(scope="module")
def lib():
    from glass_gb300 import build

    build.build()
    L = gg.load_library()
    P = ctypes.POINTER
    L.initialize_analytic_orbit.argtypes = [P(Orbit)]
    L.generate_ucb_model.argtypes = [P(Orbit), P(Data), P(Model), c_int]
    L.update_ucb_model.argtypes = [P(Orbit), P(Data), P(Model), P(Model), c_int]
    L.gaussian_log_likelihood.argtypes = [P(Data), P(Model)]
    L.gaussian_log_likelihood.restype = c_double
    L.snr.argtypes = [P(Source), P(Noise)]
    L.snr.restype = c_double
    L.fourier_nwip.argtypes = [_D, _D, _D, c_int]
    L.fourier_nwip.restype = c_double
    L.ucb_alignment.argtypes = [P(Orbit), P(Data), P(Source)]
    L.ucb_fisher.argtypes = [P(Orbit), P(Data), P(Source), P(Noise)]
    L.matrix_eigenstuff.argtypes = [_DD, _DD, _D, c_int]
    L.wavelet_transform_timefreq_by_layers.argtypes = [ctypes.c_void_p, c_int, c_int, _D, _D]
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
