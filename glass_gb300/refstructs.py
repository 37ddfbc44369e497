"""ctypes layouts of the reference's structures (struct Orbit, Data, Source,
Model, Noise, TDI) and builders that fill them from numpy arrays, for calling
the drop-in entry points of include/glass_gb300.h from Python (the benchmark's
sequential leg and the tests).  The field order and types follow the
reference's headers, cited per class."""
from __future__ import annotations

import ctypes

import numpy as np

from .workloads import T_YEAR as T

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


class Wavelets(ctypes.Structure):
    """utils/src/glass_wavelet.h:25-75"""
    _fields_ = [("NF", c_int), ("NT", c_int), ("cadence", c_double), ("dt", c_double), ("df", c_double),
                ("frequency_steps", c_int), ("fdot_steps", c_int), ("d_fdot", c_double), ("oversample", c_int),
                ("Omega", c_double), ("dOmega", c_double), ("domega", c_double), ("inv_root_dOmega", c_double),
                ("B", c_double), ("A", c_double), ("BW", c_double), ("deltaf", c_double), ("fdot", _D),
                ("window", _D), ("window_freq_forward", _D), ("norm", c_double), ("N", c_int), ("T", c_double),
                ("kmin", c_int), ("kmax", c_int), ("imin", c_int), ("imax", c_int), ("n_table", ctypes.c_void_p),
                ("table", ctypes.c_void_p)]


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


def make_data(keep, NFFT, qmin, dA, dE, noise, fmt=b"sangria", T=T):
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




def make_orbit_nodes(keep, t, pos):
    """struct Orbit holding node times t and positions pos[sc, dim, node]."""
    o = Orbit()
    o.Norb = len(t)
    o.t = keep.arr(t)
    for name, d in (("x", 0), ("y", 1), ("z", 2)):
        setattr(o, name, keep.ptrs([pos[sc, d] for sc in range(3)]))
    keep.refs.append(o)
    return o


def make_wavelets(keep, NF, NT, wdt, kmin, kmax, imin=0, imax=0):
    w = Wavelets()
    w.NF, w.NT, w.dt, w.df, w.A = NF, NT, wdt, 1 / (2 * wdt), 0.0
    w.kmin, w.kmax, w.imin, w.imax = kmin, kmax, imin, imax
    keep.refs.append(w)
    return w


def make_noise_xyz(keep, invC):
    """struct Noise with the 3 x 3 inverse covariance invC[i, j, k] per pixel."""
    n = Noise()
    n.N, n.Nchannel = invC.shape[2], 3
    outer = (_DD * 3)(*[keep.ptrs([invC[i, j] for j in range(3)]) for i in range(3)])
    keep.refs.append(outer)
    n.invC = ctypes.cast(outer, _DDD)
    n.C = n.invC
    keep.refs.append(n)
    return n


def make_wavelet_tdi(keep, xyz):
    """struct TDI of the X, Y, Z pixel arrays xyz[3, N]."""
    t = TDI()
    N = xyz.shape[1]
    t.X, t.Y, t.Z = (keep.arr(xyz[c]) for c in range(3))
    t.A, t.E, t.T = (keep.arr(np.zeros(N)) for _ in range(3))
    t.Nchannel, t.N = 3, N
    keep.refs.append(t)
    return t


def make_wavelet_model(keep, xyz, pixels, noise):
    """struct Model of one wavelet-domain template: its pixel arrays, its
    pixel list and the noise it is weighted with."""
    m = Model()
    m.tdi = ctypes.pointer(make_wavelet_tdi(keep, xyz))
    lst = np.ascontiguousarray(pixels, np.int32)
    keep.refs.append(lst)
    m.list = lst.ctypes.data_as(ctypes.POINTER(c_int))
    m.Nlist = len(lst)
    m.noise = ctypes.pointer(noise)
    keep.refs.append(m)
    return m


def bind_dropins(L):
    """argtypes/restypes of the struct-based drop-ins on a loaded library."""
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
    L.wavelet_nwip.argtypes = [_D, _D, _D, P(c_int), c_int]
    L.wavelet_nwip.restype = c_double
    L.snr_wavelet.argtypes = [P(Source), P(Noise)]
    L.snr_wavelet.restype = c_double
    L.delta_log_likelihood.argtypes = [P(Data), P(Model), P(Model)]
    L.delta_log_likelihood.restype = c_double
    L.ucb_fisher_wavelet.argtypes = [P(Orbit), P(Data), P(Source), P(Noise)]
    return L
