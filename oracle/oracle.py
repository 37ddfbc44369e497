"""ctypes front end for the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the glass_gb300 package.

* ``Port``  wraps oracle/_build/liboracle.so, the CPU restatement of the GLASS
  UCB path in glass_oracle.c, glass_oracle_wdm.c and glass_oracle_wavelet.c
  (builds anywhere).
* ``Ref``   wraps oracle/_ref/libglassref.so, the reference's own sources
  compiled with stand-in headers (only where the reference tree exists).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libglassref.so")
# the reference source tree (development machine only): $GLASS_REFERENCE_SRC
REF_SRC = os.environ.get("GLASS_REFERENCE_SRC", "/root/reference")

FORMATS = {"sangria": 0, "phase": 1, "frequency": 2}
NOISE_MODELS = {"scirdv1": 0, "sangria": 1, "radler": 2}

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def _p(a):
    return a.ctypes.data_as(_D)


def _pi(a):
    return a.ctypes.data_as(_I)


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return PORT_SO


def build_ref() -> str | None:
    if not os.path.isdir(REF_SRC):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "-f", "Makefile.ref", f"REF={REF_SRC}"], check=True)
    return REF_SO


class Port:
    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build_port()
        self.lib = lib = ctypes.CDLL(path)
        for name in ("orc_fstar", "orc_aenoise_ff", "orc_aenoise", "orc_fourier_nwip"):
            getattr(lib, name).restype = ctypes.c_double
        lib.orc_aenoise_ff.argtypes = [ctypes.c_int, ctypes.c_double]
        lib.orc_aenoise.argtypes = [ctypes.c_double]
        lib.orc_ucb_bandwidth.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int]
        lib.orc_ucb_waveform.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, ctypes.c_int] + [_D] * 5 + [
            ctypes.c_int, ctypes.c_int]
        lib.orc_ucb_alignment.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _I]
        lib.orc_dlogl_term.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _D, _D, _D, _D, _D, _D, _D]
        lib.orc_dlogl_batch.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _I, _D, _D, _D,
                                        _D, ctypes.c_int, _I, _D, _D, _D, _D, _D, ctypes.c_int]
        lib.orc_ucb_fisher.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _D, _D, _D, _D]
        lib.orc_orbit_positions.argtypes = [ctypes.c_double, _D]
        lib.orc_forward_complex_fft.argtypes = [_D, ctypes.c_int]
        self._wdm_bind()
        self._wavelet_bind()
        self._fstat_bind()

    # --- Fourier-domain UCB path -------------------------------------------------
    def fstar(self) -> float:
        return self.lib.orc_fstar()

    def aenoise_ff(self, f, model="scirdv1"):
        m = NOISE_MODELS[model]
        return np.array([self.lib.orc_aenoise_ff(m, float(x)) for x in np.atleast_1d(f)])

    def bandwidth(self, f, fdot, costheta, amp, T, NFFT) -> int:
        return self.lib.orc_ucb_bandwidth(f, fdot, costheta, amp, T, NFFT)

    def alignment(self, T, NFFT, qmin, params):
        out = np.zeros(5, np.int32)
        self.lib.orc_ucb_alignment(T, NFFT, qmin, _p(np.ascontiguousarray(params, np.float64)), _pi(out))
        return out

    def waveform(self, params, N, T, t0=0.0, fmt="sangria", NI=2, NP=8):
        params = np.ascontiguousarray(params, np.float64)
        out = np.zeros((5, 2 * N))
        rc = self.lib.orc_ucb_waveform(FORMATS[fmt], T, t0, _p(params), NP, *[_p(out[i]) for i in range(5)], N, NI)
        if rc != 0:
            raise ValueError("N must be a power of two")
        return out  # X, Y, Z, A, E

    def dlogl_term(self, params, T, NFFT, qmin, rA, rE, invCA, invCE, t0=0.0, fmt="sangria"):
        term = np.zeros(1)
        hh = np.zeros(1)
        N = self.lib.orc_dlogl_term(FORMATS[fmt], T, t0, NFFT, qmin, _p(rA), _p(rE), _p(invCA), _p(invCE),
                                    _p(np.ascontiguousarray(params, np.float64)), _p(term), _p(hh))
        return term[0], hh[0], N

    def dlogl_batch(self, T, NFFT, seg_qmin, rA, rE, invCA, invCE, item_seg, params, term_x=None, t0=0.0,
                    fmt="sangria", nthreads=0):
        n = len(item_seg)
        dl, ty, hh = np.zeros(n), np.zeros(n), np.zeros(n)
        tx = None if term_x is None else np.ascontiguousarray(term_x, np.float64)
        self.lib.orc_dlogl_batch(FORMATS[fmt], T, t0, NFFT, _pi(np.ascontiguousarray(seg_qmin, np.int32)),
                                 _p(rA), _p(rE), _p(invCA), _p(invCE), n,
                                 _pi(np.ascontiguousarray(item_seg, np.int32)),
                                 _p(np.ascontiguousarray(params, np.float64)),
                                 _p(tx) if tx is not None else None, _p(dl), _p(ty), _p(hh), nthreads)
        return dl, ty, hh

    def max_threads(self) -> int:
        return self.lib.orc_max_threads()

    def fisher(self, params, T, NFFT, qmin, invCA, invCE, t0=0.0, fmt="sangria"):
        F = np.zeros(64)
        self.lib.orc_ucb_fisher(FORMATS[fmt], T, t0, NFFT, qmin, _p(invCA), _p(invCE),
                                _p(np.ascontiguousarray(params, np.float64)), _p(F))
        return F.reshape(8, 8)

    # --- F-statistic (ucb/src/glass_ucb_fstatistic.c, ucb/src/glass_ucb_proposal.c) ---
    def _fstat_bind(self):
        lib = self.lib
        lib.orc_fstat_logl.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _D, _D, _D] + [ctypes.c_double] * 4 + [_D]
        lib.orc_fstat_batch.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _I, _D, _D, _D,
                                        ctypes.c_int, _I, _D, _D, ctypes.c_int]
        lib.orc_fstat_proposal.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, _D, _D, _D, ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_int]
        lib.orc_ucb_fdot.restype = ctypes.c_double
        lib.orc_ucb_fdot.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.orc_segment_fmin.restype = ctypes.c_double
        lib.orc_segment_fmin.argtypes = [ctypes.c_int, ctypes.c_double]
        lib.orc_invert4.argtypes = [_D]
        lib.orc_fstat_params.argtypes = [_D, _D]

    def fstat_logl(self, T, NFFT, qmin, dA, dE, invCA, f0, fdot, theta, phi, t0=0.0, fmt="sangria"):
        """(logL_AE, A, iota, psi, phase), BW of get_Fstat_logL's A/E half."""
        out = np.zeros(5)
        bw = self.lib.orc_fstat_logl(FORMATS[fmt], T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), f0, fdot, theta,
                                     phi, _p(out))
        return out, bw

    def fstat_batch(self, T, NFFT, seg_qmin, dA, dE, invCA, cell_seg, cells, t0=0.0, fmt="sangria", nthreads=0):
        cells = np.ascontiguousarray(cells, np.float64).reshape(-1, 4)
        out = np.zeros((len(cells), 5))
        self.lib.orc_fstat_batch(FORMATS[fmt], T, t0, NFFT, _pi(np.ascontiguousarray(seg_qmin, np.int32)),
                                 _p(np.ascontiguousarray(dA, np.float64)), _p(np.ascontiguousarray(dE, np.float64)),
                                 _p(np.ascontiguousarray(invCA, np.float64)), len(cells),
                                 _pi(np.ascontiguousarray(cell_seg, np.int32)), _p(cells), _p(out), nthreads)
        return out

    def fstat_proposal(self, T, NFFT, qmin, dA, dE, invCA, n_theta, n_phi, t0=0.0, fmt="sangria", nthreads=0):
        """build_fstatistic_proposal on one segment: (tensor[n_f, n_theta, n_phi], norm, maxp)."""
        fmin = self.segment_fmin(qmin, T)
        n_f = int((fmin + NFFT / T - fmin) * T)
        tensor = np.zeros((n_f, n_theta, n_phi))
        info = np.zeros(3)
        self.lib.orc_fstat_proposal(FORMATS[fmt], T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), n_theta, n_phi,
                                    _p(tensor), _p(info), nthreads)
        return tensor, info[1], info[2]

    def ucb_fdot(self, Mc, f0):
        return self.lib.orc_ucb_fdot(Mc, f0)

    def segment_fmin(self, qmin, T):
        return self.lib.orc_segment_fmin(qmin, T)

    def invert4(self, M):
        m = np.ascontiguousarray(M, np.float64).reshape(16).copy()
        if self.lib.orc_invert4(_p(m)) != 0:
            raise np.linalg.LinAlgError("singular")
        return m.reshape(4, 4)

    def fstat_params(self, a):
        out = np.zeros(4)
        self.lib.orc_fstat_params(_p(np.ascontiguousarray(a, np.float64)), _p(out))
        return out

    # --- noise-model likelihood (noise/src/glass_noise_model.c) -------------------
    def noise_logl(self, T, fmin, X, Y, Z, inst, sgal=None, nthreads=0):
        """my_noise_log_likelihood of each noise model: inst [n, 12] (sacc[6],
        soms[6]), sgal [n, 5] or None; X, Y, Z interleaved (2 NFFT)."""
        lib = self.lib
        lib.orc_noise_logl_batch.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D, _D,
                                             ctypes.c_int, _D, _D, _D, ctypes.c_int]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        out = np.zeros(len(inst))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.orc_noise_logl_batch(T, fmin, len(X) // 2, _p(X), _p(Y), _p(Z), len(inst), _p(inst),
                                 _p(sg) if sg is not None else None, _p(out), nthreads)
        return out

    def noise_covariance(self, T, fmin, N, inst, sgal=None):
        """[N, 6] covariance entries xx, yy, zz, xy, xz, yz of one noise model."""
        lib = self.lib
        lib.orc_noise_covariance.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D, _D, _D]
        inst = np.ascontiguousarray(inst, np.float64).reshape(12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(5)
        out = np.zeros((N, 6))
        lib.orc_noise_covariance(T, fmin, N, _p(inst[:6].copy()), _p(inst[6:].copy()),
                                 _p(sg) if sg is not None else None, _p(out))
        return out

    def noise_wavelet_logl(self, NF, NT, df, lmin, P, Q, inst, sgal=None, mode=0, mod=None, nthreads=0):
        """my_noise_log_likelihood_wavelet_coarse of each noise model: P [6, Nlayer, NT/Q]
        cell statistics, mode 0 instrument / 1 stationary foreground / 2 modulated
        (mod [6, NT/Q])."""
        lib = self.lib
        lib.orc_noise_wavelet_logl_batch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _D, ctypes.c_int,
                                                     _D, _D, _D, ctypes.c_int]
        P = np.ascontiguousarray(P, np.float64)
        Nlayer = P.shape[1]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        md = None if mod is None else np.ascontiguousarray(mod, np.float64)
        out = np.zeros(len(inst))
        lib.orc_noise_wavelet_logl_batch(NF, NT, df, lmin, Nlayer, Q, _p(P), mode, _p(md) if md is not None else None,
                                         len(inst), _p(inst), _p(sg) if sg is not None else None, _p(out), nthreads)
        return out

    def sgwb_psd(self, sgwb_type, f, params):
        """The background's strain PSD of template sgwb_type at f > 0."""
        lib = self.lib
        lib.orc_sgwb_psd.argtypes = [ctypes.c_int, ctypes.c_double, _D]
        lib.orc_sgwb_psd.restype = ctypes.c_double
        p = np.zeros(4)
        p[:len(params)] = params
        return lib.orc_sgwb_psd(int(sgwb_type), float(f), _p(p))

    def sgwb_response(self, resp, f):
        """[6, len(f)] response xx, yy, zz, xy, xz, yz at f from the table rows resp [n, 7]."""
        lib = self.lib
        lib.orc_sgwb_response.argtypes = [ctypes.c_int, _D, ctypes.c_int, _D, _D]
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        f = np.ascontiguousarray(f, np.float64)
        out = np.zeros((6, len(f)))
        lib.orc_sgwb_response(len(r), _p(r), len(f), _p(f), _p(out))
        return out

    def noise_logl_sgwb(self, T, fmin, X, Y, Z, inst, sgal, sgwb_type, sgwb, resp, nthreads=0):
        """noise_logl with the background of template sgwb_type (sgwb [n, 4]) added last."""
        lib = self.lib
        lib.orc_noise_logl_sgwb_batch.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D, _D,
                                                  ctypes.c_int, _D, _D, ctypes.c_int, _D, ctypes.c_int, _D, _D,
                                                  ctypes.c_int]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        b = np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        out = np.zeros(len(inst))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.orc_noise_logl_sgwb_batch(T, fmin, len(X) // 2, _p(X), _p(Y), _p(Z), len(inst), _p(inst),
                                      _p(sg) if sg is not None else None, int(sgwb_type), _p(b), len(r), _p(r),
                                      _p(out), nthreads)
        return out

    def noise_wavelet_logl_sgwb(self, NF, NT, df, lmin, P, Q, inst, sgal, mode, mod, sgwb_type, sgwb, resp,
                                nthreads=0):
        """noise_wavelet_logl with the background added last to every cell."""
        lib = self.lib
        lib.orc_noise_wavelet_logl_sgwb_batch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                          ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _D,
                                                          ctypes.c_int, _D, _D, ctypes.c_int, _D, ctypes.c_int, _D,
                                                          _D, ctypes.c_int]
        P = np.ascontiguousarray(P, np.float64)
        Nlayer = P.shape[1]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        md = None if mod is None else np.ascontiguousarray(mod, np.float64)
        b = np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        out = np.zeros(len(inst))
        lib.orc_noise_wavelet_logl_sgwb_batch(NF, NT, df, lmin, Nlayer, Q, _p(P), mode,
                                              _p(md) if md is not None else None, len(inst), _p(inst),
                                              _p(sg) if sg is not None else None, int(sgwb_type), _p(b), len(r),
                                              _p(r), _p(out), nthreads)
        return out

    def rj_propose(self, Nlive, Neff, src, prior, logPV, rjw, grid, seed):
        """The birth/death proposal of ucb_rjmcmc per chain (orc_rj_propose):
        Nlive [n], Neff [n], src [n, maxsrc, 8], prior [8, 2], logPV [8],
        rjw [9], grid = (tensor [nf, nt, np], df, dt, dp, maxp, qmin, T) or
        None, seed [n] (advanced in place).  Returns move, slot, kind,
        params_y, logQxy, logQyx, logPy."""
        lib = self.lib
        _U = ctypes.POINTER(ctypes.c_uint)
        lib.orc_rj_propose.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _D, _D, _D, _D, _D, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_double, _U, _I, _I, _I, _D, _D, _D, _D]
        n, maxsrc = src.shape[0], src.shape[1]
        Nl = np.ascontiguousarray(Nlive, np.int32)
        Ne = np.ascontiguousarray(Neff, np.int32)
        sr = np.ascontiguousarray(src, np.float64)
        pr = np.ascontiguousarray(prior, np.float64).reshape(16)
        lv = np.ascontiguousarray(logPV, np.float64)
        w = np.ascontiguousarray(rjw, np.float64)
        if grid is None:
            ten, df, dt, dp, maxp, qmin, T = np.ones((1, 1, 1)), 1.0, 1.0, 1.0, 1.0, 0, 1.0
        else:
            ten, df, dt, dp, maxp, qmin, T = grid
        ten = np.ascontiguousarray(ten, np.float64)
        move, slot, kind = (np.zeros(n, np.int32) for _ in range(3))
        y = np.zeros((n, 8))
        qxy, qyx, lpy = np.zeros(n), np.zeros(n), np.zeros(n)
        lib.orc_rj_propose(n, maxsrc, _pi(Nl), _pi(Ne), _p(sr), _p(pr), _p(lv), _p(w), _p(ten), ten.shape[0],
                           ten.shape[1], ten.shape[2], df, dt, dp, maxp, int(qmin), T, seed.ctypes.data_as(_U),
                           _pi(move), _pi(slot), _pi(kind), _p(y), _p(qxy), _p(qyx), _p(lpy))
        return move, slot, kind, y, qxy, qyx, lpy

    def rj_accept(self, Nlive, src, move, slot, params_y, logQxy, logQyx, logPy, T, dlogl, hh, prior, logPV, seed,
                  logL_x, prior_only=False):
        """The acceptance half of ucb_rjmcmc (orc_rj_accept); Nlive, src,
        params_y, seed and logL_x are updated in place.  Returns accepted."""
        lib = self.lib
        _U = ctypes.POINTER(ctypes.c_uint)
        lib.orc_rj_accept.argtypes = [ctypes.c_int, ctypes.c_int, _I, _D, _I, _I, _D, _D, _D, _D, _D, _D, _D,
                                      ctypes.c_int, _D, _D, _U, _D, _I]
        n, maxsrc = src.shape[0], src.shape[1]
        acc = np.zeros(n, np.int32)
        pr = np.ascontiguousarray(prior, np.float64).reshape(16)
        lib.orc_rj_accept(n, maxsrc, _pi(Nlive), _p(src), _pi(np.ascontiguousarray(move, np.int32)),
                          _pi(np.ascontiguousarray(slot, np.int32)), _p(params_y), _p(np.ascontiguousarray(logQxy)),
                          _p(np.ascontiguousarray(logQyx)), _p(np.ascontiguousarray(logPy)),
                          _p(np.ascontiguousarray(T, np.float64)), _p(np.ascontiguousarray(dlogl, np.float64)),
                          _p(np.ascontiguousarray(hh, np.float64)) if hh is not None else None, int(prior_only),
                          _p(pr), _p(np.ascontiguousarray(logPV, np.float64)), seed.ctypes.data_as(_U), _p(logL_x),
                          _pi(acc))
        return acc

    def noise_logl_channels(self, T, fmin, d, inst, sgal=None):
        """noise_log_likelihood of the one-channel (d [1, 2 NFFT] = X) or
        two-channel (d [2, 2 NFFT] = A, E) instrument (+ foreground) model for
        each row of inst [n, 12] (sacc[0], soms[0] used), sgal [n, 5] or None."""
        lib = self.lib
        lib.orc_noise_logl_ch_batch.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D,
                                                ctypes.c_int, _D, _D, _D]
        d = np.ascontiguousarray(d, np.float64)
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        out = np.zeros(len(inst))
        lib.orc_noise_logl_ch_batch(d.shape[0], T, fmin, d.shape[1] // 2, _p(d[0]), _p(d[-1]), len(inst), _p(inst),
                                    _p(sg) if sg is not None else None, _p(out))
        return out

    def spline_noise_logl(self, T, fmin, d, transfer, nknots, knot_f, knot_C):
        """The spline noise model's noise_log_likelihood for each model: d [nch, 2 NFFT]
        (X; or A, E), knot_f [n, kmax], knot_C [n, nch, kmax], nknots [n]."""
        lib = self.lib
        lib.orc_spline_noise_logl_batch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    _D, _D, _D, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D]
        d = np.ascontiguousarray(d, np.float64)
        nch, NFFT = d.shape[0], d.shape[1] // 2
        kf = np.ascontiguousarray(knot_f, np.float64)
        kC = np.ascontiguousarray(knot_C, np.float64)
        nk = np.ascontiguousarray(nknots, np.int32)
        out = np.zeros(len(nk))
        lib.orc_spline_noise_logl_batch(nch, NFFT, T, fmin, _p(d[0]), _p(d[nch - 1]),
                                        _p(np.ascontiguousarray(transfer, np.float64)), len(nk), kf.shape[1], _pi(nk),
                                        _p(kf), _p(kC), _p(out))
        return out

    def noise_coarse_stats(self, NT, Q, X, Y, Z):
        """[6, Nlayer, NT/Q] cell statistics of wavelet data [Nlayer NT] (coarse_grain_wavelet_data)."""
        lib = self.lib
        lib.orc_noise_coarse_stats.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]
        Nlayer = len(X) // NT
        P = np.zeros((6, Nlayer, NT // Q))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.orc_noise_coarse_stats(NT, Nlayer, Q, _p(X), _p(Y), _p(Z), _p(P))
        return P

    def noise_eta_delta(self, rA, rE, invCA, invCE, eta_x, eta_y):
        """noise_model_mcmc's (logL + logLnorm)(eta_y) - (.)(eta_x) for one residual."""
        lib = self.lib
        lib.orc_noise_eta_delta.restype = ctypes.c_double
        lib.orc_noise_eta_delta.argtypes = [ctypes.c_int, _D, _D, _D, _D, _D, _D]
        rA, rE, invCA, invCE = (np.ascontiguousarray(a, np.float64) for a in (rA, rE, invCA, invCE))
        ex = np.ascontiguousarray(eta_x, np.float64)
        ey = np.ascontiguousarray(eta_y, np.float64)
        return lib.orc_noise_eta_delta(len(invCA), _p(rA), _p(rE), _p(invCA), _p(invCE), _p(ex), _p(ey))

    # --- sampler (utils/src/glass_sampler.c, ucb/src/glass_ucb_sampler.c) ---------
    def rand_r_seq(self, seeds, count):
        """[n, count] successive rand_r values from each seed; returns (values, new seeds)."""
        lib = self.lib
        lib.orc_rand_r_seq.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_int, _I]
        seeds = np.array(seeds, dtype=np.uint32).copy()
        out = np.zeros((len(seeds), count), np.int32)
        for i in range(len(seeds)):
            s = ctypes.c_uint(int(seeds[i]))
            lib.orc_rand_r_seq(ctypes.byref(s), count, out[i].ctypes.data_as(_I))
            seeds[i] = s.value
        return out, seeds

    def ptmcmc(self, temperature, logL, index, seed, acceptance, logLnorm=None):
        """In place on index [nens, NC] (int32), seed (uint32), acceptance (float64)."""
        lib = self.lib
        lib.orc_ptmcmc.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _D, _I, ctypes.POINTER(ctypes.c_uint), _D]
        nens, NC = index.shape
        lib.orc_ptmcmc(nens, NC, _p(np.ascontiguousarray(temperature, np.float64)),
                       _p(np.ascontiguousarray(logL, np.float64)),
                       _p(np.ascontiguousarray(logLnorm, np.float64)) if logLnorm is not None else None,
                       index.ctypes.data_as(_I), seed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), _p(acceptance))

    def mh_accept(self, T, logL_x, dlogl, logPx, logPy, logQxy, logQyx, seed, params_x, params_y, snr=None):
        """In place on logL_x, seed (uint32), params_x [n, 8]; returns accepted [n]."""
        lib = self.lib
        lib.orc_mh_accept.argtypes = [ctypes.c_int] + [_D] * 8 + [ctypes.POINTER(ctypes.c_uint), _D, _D, _I]
        n = len(dlogl)
        acc = np.zeros(n, np.int32)
        c = lambda a: _p(np.ascontiguousarray(a, np.float64))
        lib.orc_mh_accept(n, c(T), _p(logL_x), c(dlogl), c(logPx), c(logPy), c(logQxy), c(logQyx),
                          c(snr) if snr is not None else None, seed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                          _p(params_x), c(params_y), acc.ctypes.data_as(_I))
        return acc

    def fisher_draw(self, params_x, evec, evalue, seed):
        """draw_from_fisher for n chains: params_x [n, 8], evec [n, 8, 8]
        (evec[i, j, k] = fisher_evectr[j][k]), evalue [n, 8]; seed (uint32 [n])
        advanced in place; returns (params_y [n, 8], logQ [n])."""
        lib = self.lib
        lib.orc_fisher_draw.argtypes = [ctypes.c_int, _D, _D, _D, ctypes.POINTER(ctypes.c_uint), _D, _D]
        x = np.ascontiguousarray(params_x, np.float64).reshape(-1, 8)
        n = len(x)
        y = np.zeros((n, 8))
        logQ = np.zeros(n)
        lib.orc_fisher_draw(n, _p(x), _p(np.ascontiguousarray(evec, np.float64)),
                            _p(np.ascontiguousarray(evalue, np.float64)),
                            seed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), _p(y), _p(logQ))
        return y, logQ

    def orbit(self, t):
        out = np.zeros(9)
        self.lib.orc_orbit_positions(float(t), _p(out))
        return out.reshape(3, 3)

    def fft(self, z):
        z = np.ascontiguousarray(z, np.complex128).copy()
        self.lib.orc_forward_complex_fft(z.ctypes.data_as(_D), len(z))
        return z

    # --- WDM ------------------------------------------------------------------------
    def _wdm_bind(self):
        lib = self.lib
        lib.orc_incomplete_beta.restype = ctypes.c_double
        lib.orc_incomplete_beta.argtypes = [ctypes.c_double] * 3
        lib.orc_wdm_window.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D]
        for name in ("orc_wdm_forward", "orc_wdm_inverse", "orc_wdm_from_freq", "orc_wdm_to_freq"):
            getattr(lib, name).argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _D]
        lib.orc_rfft.argtypes = [_D, _D, ctypes.c_int]
        lib.orc_irfft.argtypes = [_D, _D, ctypes.c_int]
        lib.orc_complex_fft.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int]
        lib.orc_wdm_by_layers.argtypes = [ctypes.c_int] * 4 + [_D, _D]

    def wdm_window(self, NF, NT, A=0.0, nx=6.0, forward=True):
        out = np.zeros(NT // 2 + 1)
        self.lib.orc_wdm_window(NF, NT, A, nx, int(forward), _p(out))
        return out

    def wdm_forward(self, NF, NT, window, time):
        out = np.zeros(NF * NT)
        self.lib.orc_wdm_forward(NF, NT, _p(np.ascontiguousarray(window)), _p(np.ascontiguousarray(time)), _p(out))
        return out

    def wdm_inverse(self, NF, NT, window, wdm):
        out = np.zeros(NF * NT)
        self.lib.orc_wdm_inverse(NF, NT, _p(np.ascontiguousarray(window)), _p(np.ascontiguousarray(wdm)), _p(out))
        return out

    def wdm_to_freq(self, NF, NT, window, wdm):
        out = np.zeros(NF * NT + 2)
        self.lib.orc_wdm_to_freq(NF, NT, _p(np.ascontiguousarray(window)), _p(np.ascontiguousarray(wdm)), _p(out))
        return out

    def wdm_from_freq(self, NF, NT, window, freq):
        out = np.zeros(NF * NT)
        self.lib.orc_wdm_from_freq(NF, NT, _p(np.ascontiguousarray(window)), _p(np.ascontiguousarray(freq)), _p(out))
        return out

    def rfft(self, x):
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(len(x) + 2)
        self.lib.orc_rfft(_p(x), _p(out), len(x))
        return out

    def irfft(self, f, N):
        f = np.ascontiguousarray(f, np.float64)
        out = np.zeros(N)
        self.lib.orc_irfft(_p(f), _p(out), N)
        return out

    def wdm_by_layers(self, NF, NT, jmin, Nlayers, window, timedata):
        t = np.ascontiguousarray(timedata, np.float64).copy()
        self.lib.orc_wdm_by_layers(NF, NT, jmin, Nlayers, _p(np.ascontiguousarray(window)), _p(t))
        return t

    # --- wavelet-domain UCB path ---------------------------------------------------
    def _wavelet_bind(self):
        lib = self.lib
        lib.orc_orbit_nodes.argtypes = [ctypes.c_double]
        lib.orc_orbit_grid.argtypes = [ctypes.c_double, ctypes.c_double, _D, _D]
        lib.orc_wavelet_layers.argtypes = [ctypes.c_double, _D, ctypes.c_double, ctypes.c_double, _I, _I]
        lib.orc_ucb_waveform_wavelet.argtypes = [ctypes.c_double, ctypes.c_double, _D, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                 ctypes.c_int, ctypes.c_int, _I, _I, _D, _D, _D, _I]
        lib.orc_wavelet_dh_hh.argtypes = [ctypes.c_int, _D, _D, _D, _I, ctypes.c_int, _D, _D]
        lib.orc_wavelet_delta_logl.argtypes = [ctypes.c_int, _D, _D, _I, ctypes.c_int, _D, _I, ctypes.c_int, _D]
        lib.orc_wavelet_delta_logl.restype = ctypes.c_double
        lib.orc_wavelet_logl_full.argtypes = [ctypes.c_int] * 5 + [_D, _D, _I, ctypes.c_int, _D]
        lib.orc_wavelet_logl_full.restype = ctypes.c_double
        lib.orc_wavelet_snr.argtypes = [ctypes.c_int, _D, _I, ctypes.c_int, _D]
        lib.orc_wavelet_snr.restype = ctypes.c_double

    def orbit_grid(self, Tobs, t0=0.0):
        n = self.lib.orc_orbit_nodes(Tobs)
        t, pos = np.zeros(n), np.zeros((3, 3, n))
        self.lib.orc_orbit_grid(Tobs, t0, _p(t), _p(pos))
        return t, pos

    def wavelet_layers(self, Tobs, params, df, A=0.0):
        j, n = ctypes.c_int(), ctypes.c_int()
        self.lib.orc_wavelet_layers(Tobs, _p(np.ascontiguousarray(params, np.float64)), df, A, ctypes.byref(j),
                                    ctypes.byref(n))
        return j.value, n.value

    def wavelet_waveform(self, params, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax, A=0.0, nx=6.0):
        """(list, xyz [3, kmax-kmin], first layer, layer count)."""
        N = kmax - kmin
        xyz = np.zeros((3, N))
        lst = np.zeros(4 * NT, np.int32)
        n, nl = ctypes.c_int(), ctypes.c_int()
        j = self.lib.orc_ucb_waveform_wavelet(Tobs, t0, _p(np.ascontiguousarray(params, np.float64)), NF, NT, wdt,
                                              wdf, A, nx, kmin, kmax, _pi(lst), ctypes.byref(n), _p(xyz[0]),
                                              _p(xyz[1]), _p(xyz[2]), ctypes.byref(nl))
        return lst[:n.value].copy(), xyz, j, nl.value

    def wavelet_dh_hh(self, d, h, invC, lst):
        d = np.ascontiguousarray(d, np.float64)
        h = np.ascontiguousarray(h, np.float64)
        ic = np.ascontiguousarray(invC, np.float64)
        lst = np.ascontiguousarray(lst, np.int32)
        dh, hh = ctypes.c_double(), ctypes.c_double()
        self.lib.orc_wavelet_dh_hh(d.shape[-1], _p(d), _p(h), _p(ic), _pi(lst), len(lst), ctypes.byref(dh),
                                   ctypes.byref(hh))
        return dh.value, hh.value

    def draw_uniform_prior(self, prior16, logPV8, seed):
        """draw_from_uniform_prior: (params, logQ, seed after)."""
        lib = self.lib
        lib.ref_draw_uniform_prior.argtypes = [_D, _D, ctypes.POINTER(ctypes.c_uint), _D]
        lib.ref_draw_uniform_prior.restype = ctypes.c_double
        s = ctypes.c_uint(int(seed))
        p = np.zeros(8)
        q = lib.ref_draw_uniform_prior(_p(np.ascontiguousarray(prior16, np.float64)),
                                       _p(np.ascontiguousarray(logPV8, np.float64)), ctypes.byref(s), _p(p))
        return p, q, s.value

    def ucb_prior(self, params, prior16, logPV8, skyhist=None, dcostheta=0.0, dphi=0.0, nphi=0):
        """evaluate_ucb_prior (no catalogue prior): (logP, params after wrapping)."""
        lib = self.lib
        lib.ref_ucb_prior.argtypes = [_D, _D, _D, ctypes.c_int, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        lib.ref_ucb_prior.restype = ctypes.c_double
        p = np.ascontiguousarray(params, np.float64).copy()
        sh = None if skyhist is None else np.ascontiguousarray(skyhist, np.float64)
        lp = lib.ref_ucb_prior(_p(p), _p(np.ascontiguousarray(prior16, np.float64)),
                               _p(np.ascontiguousarray(logPV8, np.float64)), int(sh is not None),
                               _p(sh) if sh is not None else None, dcostheta, dphi, nphi)
        return lp, p

    def fisher_wavelet(self, params, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax, imin, imax, invC):
        """ucb_fisher_wavelet on one source: (F 8x8, regularised flag)."""
        lib = self.lib
        lib.ref_ucb_fisher_wavelet.argtypes = [ctypes.c_double, ctypes.c_double, _D, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_double] + [ctypes.c_int] * 4 + [_D, _D]
        lib.ref_ucb_fisher_wavelet.restype = ctypes.c_int
        F = np.zeros(64)
        reg = lib.ref_ucb_fisher_wavelet(Tobs, t0, _p(np.ascontiguousarray(params, np.float64).copy()), NF, NT,
                                         wdt, wdf, kmin, kmax, imin, imax,
                                         _p(np.ascontiguousarray(invC, np.float64).reshape(-1)), _p(F))
        return F.reshape(8, 8), bool(reg)

    def wavelet_delta_logl(self, d, invC, hx, lx, hy, ly):
        d, ic = np.ascontiguousarray(d, np.float64), np.ascontiguousarray(invC, np.float64)
        hx, hy = np.ascontiguousarray(hx, np.float64), np.ascontiguousarray(hy, np.float64)
        lx, ly = np.ascontiguousarray(lx, np.int32), np.ascontiguousarray(ly, np.int32)
        return self.lib.orc_wavelet_delta_logl(d.shape[-1], _p(d), _p(hx), _pi(lx), len(lx), _p(hy), _pi(ly),
                                               len(ly), _p(ic))

    def wavelet_logl_full(self, NT, kmin, imin, imax, d, h, lst, invC):
        d, h = np.ascontiguousarray(d, np.float64), np.ascontiguousarray(h, np.float64)
        lst, ic = np.ascontiguousarray(lst, np.int32), np.ascontiguousarray(invC, np.float64)
        return self.lib.orc_wavelet_logl_full(d.shape[-1], NT, kmin, imin, imax, _p(d), _p(h), _pi(lst), len(lst),
                                              _p(ic))

    def wavelet_snr(self, h, lst, invC):
        h, lst, ic = (np.ascontiguousarray(h, np.float64), np.ascontiguousarray(lst, np.int32),
                      np.ascontiguousarray(invC, np.float64))
        return self.lib.orc_wavelet_snr(h.shape[-1], _p(h), _pi(lst), len(lst), _p(ic))


class Ref:
    """The reference's own functions (oracle/_ref/libglassref.so)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            if build_ref() is None:
                raise FileNotFoundError("reference sources are not present on this machine")
        self.lib = lib = ctypes.CDLL(path)
        for name in ("ref_fstar", "ref_aenoise_ff", "ref_aenoise", "ref_fourier_nwip", "ref_log_likelihood"):
            getattr(lib, name).restype = ctypes.c_double
        lib.ref_aenoise_ff.argtypes = [ctypes.c_char_p, ctypes.c_double]
        lib.ref_aenoise.argtypes = [ctypes.c_double]
        lib.ref_ucb_bandwidth.argtypes = [ctypes.c_double] * 5 + [ctypes.c_int]
        lib.ref_ucb_waveform.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, _D, ctypes.c_int] + [
            _D] * 5 + [ctypes.c_int, ctypes.c_int]
        lib.ref_ucb_alignment.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _I]
        lib.ref_log_likelihood.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, _D, _D, _D, _D, ctypes.c_int, _D, _D]
        lib.ref_ucb_fisher.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _D, _D, _D, _D, _D, _D]

    def fstar(self):
        return self.lib.ref_fstar()

    def _wdm(self):
        lib = self.lib
        lib.ref_wdm_window.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _D]
        lib.ref_wdm_forward.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D]
        lib.ref_wdm_inverse.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D]
        lib.ref_wdm_by_layers.argtypes = [ctypes.c_int] * 4 + [_D]

    def wdm_window(self, NF, NT, A=0.0, forward=True):
        self._wdm()
        out = np.zeros(NT // 2 + 1)
        self.lib.ref_wdm_window(NF, NT, A, int(forward), _p(out))
        return out

    def wdm_forward(self, NF, NT, time):
        """wavelet_transform_timefreq (in place in the reference) on a copy."""
        self._wdm()
        t = np.ascontiguousarray(time, np.float64).copy()
        out = np.zeros(NF * NT)
        self.lib.ref_wdm_forward(NF, NT, _p(t), _p(out))
        return out

    def wdm_inverse(self, NF, NT, wdm):
        self._wdm()
        w = np.ascontiguousarray(wdm, np.float64).copy()
        out = np.zeros(NF * NT)
        self.lib.ref_wdm_inverse(NF, NT, _p(w), _p(out))
        return out

    def wdm_by_layers(self, NF, NT, jmin, Nlayers, timedata):
        self._wdm()
        t = np.ascontiguousarray(timedata, np.float64).copy()
        self.lib.ref_wdm_by_layers(NF, NT, jmin, Nlayers, _p(t))
        return t

    # --- wavelet-domain UCB path ---------------------------------------------------
    def _wavelet(self):
        lib = self.lib
        lib.ref_ucb_waveform_wavelet.argtypes = [ctypes.c_double, ctypes.c_double, _D, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _I,
                                                 _D, _D, _D]
        lib.ref_orbit_grid.argtypes = [ctypes.c_double, ctypes.c_double, _D, _D]
        lib.ref_wavelet_delta_logl.argtypes = [ctypes.c_int, _D, _D, _D, _I, ctypes.c_int, _D, _I, ctypes.c_int]
        lib.ref_wavelet_delta_logl.restype = ctypes.c_double
        lib.ref_wavelet_logl_full.argtypes = [ctypes.c_int] * 5 + [_D, _D, _I, ctypes.c_int, _D]
        lib.ref_wavelet_logl_full.restype = ctypes.c_double
        lib.ref_wavelet_snr.argtypes = [ctypes.c_int, _D, _I, ctypes.c_int, _D]
        lib.ref_wavelet_snr.restype = ctypes.c_double

    def orbit_grid(self, Tobs, t0=0.0):
        self._wavelet()
        n = self.lib.ref_orbit_grid(Tobs, t0, None, None)
        t, pos = np.zeros(n), np.zeros((3, 3, n))
        self.lib.ref_orbit_grid(Tobs, t0, _p(t), _p(pos))
        return t, pos

    def wavelet_waveform(self, params, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax):
        """ucb_waveform_wavelet (A = 0, window exponent 6): (list, xyz [3, kmax-kmin])."""
        self._wavelet()
        N = kmax - kmin
        xyz = np.zeros((3, N))
        lst = np.zeros(4 * NT, np.int32)
        n = self.lib.ref_ucb_waveform_wavelet(Tobs, t0, _p(np.ascontiguousarray(params, np.float64).copy()), NF, NT,
                                              wdt, wdf, kmin, kmax, _pi(lst), _p(xyz[0]), _p(xyz[1]), _p(xyz[2]))
        return lst[:n].copy(), xyz

    def draw_uniform_prior(self, prior16, logPV8, seed):
        """draw_from_uniform_prior: (params, logQ, seed after)."""
        lib = self.lib
        lib.ref_draw_uniform_prior.argtypes = [_D, _D, ctypes.POINTER(ctypes.c_uint), _D]
        lib.ref_draw_uniform_prior.restype = ctypes.c_double
        s = ctypes.c_uint(int(seed))
        p = np.zeros(8)
        q = lib.ref_draw_uniform_prior(_p(np.ascontiguousarray(prior16, np.float64)),
                                       _p(np.ascontiguousarray(logPV8, np.float64)), ctypes.byref(s), _p(p))
        return p, q, s.value

    def ucb_prior(self, params, prior16, logPV8, skyhist=None, dcostheta=0.0, dphi=0.0, nphi=0):
        """evaluate_ucb_prior (no catalogue prior): (logP, params after wrapping)."""
        lib = self.lib
        lib.ref_ucb_prior.argtypes = [_D, _D, _D, ctypes.c_int, _D, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        lib.ref_ucb_prior.restype = ctypes.c_double
        p = np.ascontiguousarray(params, np.float64).copy()
        sh = None if skyhist is None else np.ascontiguousarray(skyhist, np.float64)
        lp = lib.ref_ucb_prior(_p(p), _p(np.ascontiguousarray(prior16, np.float64)),
                               _p(np.ascontiguousarray(logPV8, np.float64)), int(sh is not None),
                               _p(sh) if sh is not None else None, dcostheta, dphi, nphi)
        return lp, p

    def fisher_wavelet(self, params, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax, imin, imax, invC):
        """ucb_fisher_wavelet on one source: (F 8x8, regularised flag)."""
        lib = self.lib
        lib.ref_ucb_fisher_wavelet.argtypes = [ctypes.c_double, ctypes.c_double, _D, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_double] + [ctypes.c_int] * 4 + [_D, _D]
        lib.ref_ucb_fisher_wavelet.restype = ctypes.c_int
        F = np.zeros(64)
        reg = lib.ref_ucb_fisher_wavelet(Tobs, t0, _p(np.ascontiguousarray(params, np.float64).copy()), NF, NT,
                                         wdt, wdf, kmin, kmax, imin, imax,
                                         _p(np.ascontiguousarray(invC, np.float64).reshape(-1)), _p(F))
        return F.reshape(8, 8), bool(reg)

    def wavelet_delta_logl(self, d, invC, hx, lx, hy, ly):
        self._wavelet()
        d, ic = np.ascontiguousarray(d, np.float64).copy(), np.ascontiguousarray(invC, np.float64).copy()
        hx, hy = np.ascontiguousarray(hx, np.float64).copy(), np.ascontiguousarray(hy, np.float64).copy()
        lx, ly = np.ascontiguousarray(lx, np.int32).copy(), np.ascontiguousarray(ly, np.int32).copy()
        return self.lib.ref_wavelet_delta_logl(d.shape[-1], _p(d), _p(ic), _p(hx), _pi(lx), len(lx), _p(hy),
                                               _pi(ly), len(ly))

    def wavelet_logl_full(self, NT, kmin, imin, imax, d, h, lst, invC):
        self._wavelet()
        d, h = np.ascontiguousarray(d, np.float64).copy(), np.ascontiguousarray(h, np.float64).copy()
        lst, ic = np.ascontiguousarray(lst, np.int32).copy(), np.ascontiguousarray(invC, np.float64).copy()
        return self.lib.ref_wavelet_logl_full(d.shape[-1], NT, kmin, imin, imax, _p(d), _p(h), _pi(lst), len(lst),
                                              _p(ic))

    def wavelet_snr(self, h, lst, invC):
        self._wavelet()
        h, lst, ic = (np.ascontiguousarray(h, np.float64).copy(), np.ascontiguousarray(lst, np.int32).copy(),
                      np.ascontiguousarray(invC, np.float64).copy())
        return self.lib.ref_wavelet_snr(h.shape[-1], _p(h), _pi(lst), len(lst), _p(ic))

    def aenoise_ff(self, f, model="scirdv1"):
        return np.array([self.lib.ref_aenoise_ff(model.encode(), float(x)) for x in np.atleast_1d(f)])

    def bandwidth(self, f, fdot, costheta, amp, T, NFFT):
        return self.lib.ref_ucb_bandwidth(f, fdot, costheta, amp, T, NFFT)

    def alignment(self, T, NFFT, qmin, params):
        out = np.zeros(5, np.int32)
        self.lib.ref_ucb_alignment(T, NFFT, qmin, _p(np.ascontiguousarray(params, np.float64).copy()), _pi(out))
        return out

    def waveform(self, params, N, T, t0=0.0, fmt="sangria", NI=2, NP=8):
        params = np.ascontiguousarray(params, np.float64).copy()
        out = np.zeros((5, 2 * N))
        self.lib.ref_ucb_waveform(fmt.encode(), T, t0, _p(params), NP, *[_p(out[i]) for i in range(5)], N, NI)
        return out

    def log_likelihood(self, T, NFFT, qmin, dA, dE, invCA, invCE, params, t0=0.0, fmt="sangria"):
        params = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        snr = np.zeros(len(params))
        ll = self.lib.ref_log_likelihood(fmt.encode(), T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), _p(invCE),
                                         len(params), _p(params), _p(snr))
        return ll, snr

    def fisher(self, params, T, NFFT, qmin, invCA, invCE, t0=0.0, fmt="sangria"):
        F, ev, evec = np.zeros(64), np.zeros(8), np.zeros(64)
        self.lib.ref_ucb_fisher(fmt.encode(), T, t0, NFFT, qmin, _p(invCA), _p(invCE),
                                _p(np.ascontiguousarray(params, np.float64).copy()), _p(F), _p(ev), _p(evec))
        return F.reshape(8, 8), ev, evec.reshape(8, 8)

    def fstat_logl(self, T, NFFT, qmin, dA, dE, invCA, cells, t0=0.0, fmt="sangria"):
        """get_Fstat_logL per cell (f0, fdot, theta, phi): rows of logL_X, logL_AE, A, iota, psi, phase."""
        lib = self.lib
        lib.ref_fstat_logl.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                       _D, _D, _D, ctypes.c_int, _D, _D]
        cells = np.ascontiguousarray(cells, np.float64).reshape(-1, 4)
        out = np.zeros((len(cells), 6))
        lib.ref_fstat_logl(fmt.encode(), T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), len(cells), _p(cells), _p(out))
        return out

    def fstat_proposal(self, T, NFFT, qmin, dA, dE, invCA, n_theta, n_phi, t0=0.0, fmt="sangria"):
        """build_fstatistic_proposal: (tensor[n_f, n_theta, n_phi], norm, maxp)."""
        lib = self.lib
        lib.ref_fstat_proposal.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, _D, _D, _D, ctypes.c_int, ctypes.c_int, _D, _D]
        tensor = np.zeros(NFFT * n_theta * n_phi + 64 * n_theta * n_phi)
        info = np.zeros(3)
        lib.ref_fstat_proposal(fmt.encode(), T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), n_theta, n_phi,
                               _p(tensor), _p(info))
        n_f = int(info[0])
        return tensor[:n_f * n_theta * n_phi].reshape(n_f, n_theta, n_phi), info[1], info[2]

    def noise_logl(self, T, fmin, X, Y, Z, inst, sgal=None):
        """The reference's instrument (+ foreground) covariance, inverse and
        my_noise_log_likelihood for each noise model."""
        lib = self.lib
        lib.ref_noise_logl.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D, _D, ctypes.c_int,
                                       _D, _D, _D]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        out = np.zeros(len(inst))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.ref_noise_logl(T, fmin, len(X) // 2, _p(X), _p(Y), _p(Z), len(inst), _p(inst),
                           _p(sg) if sg is not None else None, _p(out))
        return out

    def noise_wavelet_logl(self, NF, NT, dt, df, lmin, Q, X, Y, Z, inst, sgal=None, mode=0, mod=None):
        """The reference's coarse-grained wavelet noise likelihood for each model,
        and the cell statistics it used: (logl [n], P [6, Nlayer, NT/Q])."""
        lib = self.lib
        lib.ref_noise_wavelet_logl.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_int, _D,
                                               ctypes.c_int, _D, _D, _D, _D]
        Nlayer = len(X) // NT
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        md = None if mod is None else np.ascontiguousarray(mod, np.float64)
        out = np.zeros(len(inst))
        P = np.zeros((6, Nlayer, NT // Q))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.ref_noise_wavelet_logl(NF, NT, dt, df, lmin, Nlayer, Q, _p(X), _p(Y), _p(Z), mode,
                                   _p(md) if md is not None else None, len(inst), _p(inst),
                                   _p(sg) if sg is not None else None, _p(out), _p(P))
        return out, P

    def sgwb_model(self, sgwb_type, params, resp, f):
        """The reference's generate_sgwb_model on frequencies f: [len(f), 6]
        covariance xx, yy, zz, xy, xz, yz (response from the table rows resp)."""
        lib = self.lib
        lib.ref_sgwb_model.argtypes = [ctypes.c_int, _D, ctypes.c_int, _D, ctypes.c_int, _D, _D]
        p = np.zeros(4)
        p[:len(params)] = params
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        f = np.ascontiguousarray(f, np.float64)
        out = np.zeros((len(f), 6))
        lib.ref_sgwb_model(int(sgwb_type), _p(p), len(r), _p(r), len(f), _p(f), _p(out))
        return out

    def noise_logl_sgwb(self, T, fmin, X, Y, Z, inst, sgal, sgwb_type, sgwb, resp):
        """The reference's likelihood with the background added last."""
        lib = self.lib
        lib.ref_noise_logl_sgwb.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D, _D, ctypes.c_int,
                                            _D, _D, ctypes.c_int, _D, ctypes.c_int, _D, _D]
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        b = np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        out = np.zeros(len(inst))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.ref_noise_logl_sgwb(T, fmin, len(X) // 2, _p(X), _p(Y), _p(Z), len(inst), _p(inst),
                                _p(sg) if sg is not None else None, int(sgwb_type), _p(b), len(r), _p(r), _p(out))
        return out

    def noise_wavelet_logl_sgwb(self, NF, NT, dt, df, lmin, Q, X, Y, Z, inst, sgal, mode, mod, sgwb_type, sgwb,
                                resp):
        """The reference's coarse wavelet likelihood with the background."""
        lib = self.lib
        lib.ref_noise_wavelet_logl_sgwb.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, _D,
                                                    ctypes.c_int, _D, ctypes.c_int, _D, _D, ctypes.c_int, _D,
                                                    ctypes.c_int, _D, _D]
        Nlayer = len(X) // NT
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        md = None if mod is None else np.ascontiguousarray(mod, np.float64)
        b = np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        r = np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        out = np.zeros(len(inst))
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        lib.ref_noise_wavelet_logl_sgwb(NF, NT, dt, df, lmin, Nlayer, Q, _p(X), _p(Y), _p(Z), mode,
                                        _p(md) if md is not None else None, len(inst), _p(inst),
                                        _p(sg) if sg is not None else None, int(sgwb_type), _p(b), len(r), _p(r),
                                        _p(out))
        return out

    def rj_steps(self, T, NFFT, qmin, dA, dE, invCA, invCE, Neff, Nlive, src, prior, logPV, rjw, grid, temperature,
                 seed, nsteps, t0=0.0, fmt="sangria"):
        """The reference's ucb_rjmcmc, nsteps calls per chain (ref_rj_steps).
        Nlive, src [n, maxsrc, 8] and seed are updated in place.  Returns a
        dict of the per-call records [nsteps, n, ...] and logL0 [n]."""
        lib = self.lib
        _U = ctypes.POINTER(ctypes.c_uint)
        lib.ref_rj_steps.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                     _D, _D, _D, _D, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D, _D, _D, _D,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, _D, _U, ctypes.c_int, _D, _I, _D, _D, _D, _D,
                                     _I, _U]
        n, maxsrc = src.shape[0], src.shape[1]
        ten, df, dt, dp, maxp = grid
        ten = np.ascontiguousarray(ten, np.float64)
        K = nsteps
        out = {"logL0": np.zeros(n), "rec_gen": np.zeros((K, n), np.int32), "rec_params": np.zeros((K, n, 8)),
               "rec_snr": np.zeros((K, n)), "rec_logLy": np.zeros((K, n)), "logL": np.zeros((K, n)),
               "Nlive": np.zeros((K, n), np.int32), "seed": np.zeros((K, n), np.uint32)}
        lib.ref_rj_steps(fmt.encode(), T, t0, NFFT, qmin, _p(np.ascontiguousarray(dA)), _p(np.ascontiguousarray(dE)),
                         _p(np.ascontiguousarray(invCA)), _p(np.ascontiguousarray(invCE)), n, maxsrc,
                         np.ascontiguousarray(Neff, np.int32).ctypes.data_as(_I), Nlive.ctypes.data_as(_I), _p(src),
                         _p(np.ascontiguousarray(prior, np.float64).reshape(16)),
                         _p(np.ascontiguousarray(logPV, np.float64)), _p(np.ascontiguousarray(rjw, np.float64)),
                         _p(ten), ten.shape[0], ten.shape[1], ten.shape[2], df, dt, dp, maxp,
                         _p(np.ascontiguousarray(temperature, np.float64)), seed.ctypes.data_as(_U), K,
                         _p(out["logL0"]), out["rec_gen"].ctypes.data_as(_I), _p(out["rec_params"]),
                         _p(out["rec_snr"]), _p(out["rec_logLy"]), _p(out["logL"]), out["Nlive"].ctypes.data_as(_I),
                         out["seed"].ctypes.data_as(_U))
        return out

    def noise_logl_channels(self, T, fmin, d, inst, sgal=None):
        """The reference's one- or two-channel instrument (+ foreground)
        covariance, inverse and noise_log_likelihood for each noise model."""
        lib = self.lib
        lib.ref_noise_logl_channels.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D, _D,
                                                ctypes.c_int, _D, _D, _D]
        d = np.ascontiguousarray(d, np.float64)
        inst = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        sg = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        out = np.zeros(len(inst))
        lib.ref_noise_logl_channels(d.shape[0], T, fmin, d.shape[1] // 2, _p(d[0]), _p(d[-1]), len(inst), _p(inst),
                                    _p(sg) if sg is not None else None, _p(out))
        return out

    def spline_noise_logl(self, T, fmin, d, transfer, nknots, knot_f, knot_C):
        """The reference's generate_spline_noise_model + noise_log_likelihood."""
        lib = self.lib
        lib.ref_spline_noise_logl.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, _D,
                                              _D, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D]
        d = np.ascontiguousarray(d, np.float64)
        nch, NFFT = d.shape[0], d.shape[1] // 2
        kf = np.ascontiguousarray(knot_f, np.float64)
        kC = np.ascontiguousarray(knot_C, np.float64)
        nk = np.ascontiguousarray(nknots, np.int32)
        out = np.zeros(len(nk))
        lib.ref_spline_noise_logl(nch, NFFT, T, fmin, _p(d[0]), _p(d[nch - 1]),
                                  _p(np.ascontiguousarray(transfer, np.float64)), len(nk), kf.shape[1],
                                  nk.ctypes.data_as(_I), _p(kf), _p(kC), _p(out))
        return out

    def noise_eta(self, T, NFFT, qmin, dA, dE, invCA, invCE, params, eta, t0=0.0, fmt="sangria"):
        """noise_model_mcmc's likelihood change per chain: eta [n, 4] = xA, xE, yA, yE."""
        lib = self.lib
        lib.ref_noise_eta.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      _D, _D, _D, _D, ctypes.c_int, _D, _D, _D]
        params = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        eta = np.ascontiguousarray(eta, np.float64).reshape(-1, 4)
        out = np.zeros(len(params))
        lib.ref_noise_eta(fmt.encode(), T, t0, NFFT, qmin, _p(dA), _p(dE), _p(invCA), _p(invCE), len(params),
                          _p(params), _p(eta), _p(out))
        return out

    def fisher_draw(self, params_x, evec, evalue, seed):
        """The reference's draw_from_fisher chain by chain (same layout as the
        port's); seed advanced in place; returns (params_y, logQ)."""
        lib = self.lib
        lib.ref_fisher_draw.restype = ctypes.c_double
        lib.ref_fisher_draw.argtypes = [_D, _D, _D, ctypes.POINTER(ctypes.c_uint), _D]
        x = np.ascontiguousarray(params_x, np.float64).reshape(-1, 8)
        ev = np.ascontiguousarray(evec, np.float64).reshape(-1, 64)
        el = np.ascontiguousarray(evalue, np.float64).reshape(-1, 8)
        y = np.zeros_like(x)
        logQ = np.zeros(len(x))
        for i in range(len(x)):
            s = ctypes.c_uint(int(seed[i]))
            logQ[i] = lib.ref_fisher_draw(_p(x[i]), _p(ev[i]), _p(el[i]), ctypes.byref(s), _p(y[i]))
            seed[i] = s.value
        return y, logQ

    def ptmcmc(self, temperature, logL, index, seed, acceptance, logLnorm=None):
        """The reference's ptmcmc on one ladder, in place."""
        lib = self.lib
        lib.ref_ptmcmc.argtypes = [ctypes.c_int, _D, _D, _D, _I, ctypes.POINTER(ctypes.c_uint), _D]
        NC = len(index)
        lib.ref_ptmcmc(NC, _p(np.ascontiguousarray(temperature, np.float64)), _p(np.ascontiguousarray(logL, np.float64)),
                       _p(np.ascontiguousarray(logLnorm, np.float64)) if logLnorm is not None else None,
                       index.ctypes.data_as(_I), seed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), _p(acceptance))
