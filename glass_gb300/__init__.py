"""GB300 UCB likelihood engine: Python front end of libglass_gb300.so.

The library is a plain C ABI (include/glass_gb300.h).  This module binds it
with ctypes and mirrors the reference's call pattern for the UCB likelihood
path: upload the analysis segments once, then evaluate batches of proposals.
There is no CPU fallback: if the compiled library is missing, importing the
engine raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The engine library; GLASS_GB300_LIB selects another build of it (the test
# suite's checked build, lib/libglass_gb300_checks.so).
LIB_PATH = os.environ.get("GLASS_GB300_LIB") or os.path.join(HERE, "lib", "libglass_gb300.so")

PREC_FP64 = 0
PREC_MIXED = 1
FORMATS = {"sangria": 0, "phase": 1, "frequency": 2}

ITEM_NONFINITE = 1
ITEM_BAD_SEGMENT = 2
ITEM_OUTSIDE = 4
# glass_gpu_fisher_draw status codes
DRAW_OK, DRAW_NAN, DRAW_RNG_LIMIT = 0, 1, 2

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p

# Every symbol include/glass_gb300.h declares.
EXPORTS = (
    "ucb_waveform", "glass_ucb_waveform", "ucb_bandwidth",
    "glass_gpu_create", "glass_gpu_destroy", "glass_gpu_set_stream", "glass_gpu_last_error",
    "glass_gpu_bank_upload", "glass_gpu_bank_set_residual", "glass_gpu_dlogl_batch",
    "glass_gpu_dlogl_batch_host", "glass_gpu_last_launch_count", "glass_gpu_set_phase_timing",
    "glass_gpu_set_host_access", "glass_gpu_get_host_access",
    "glass_gpu_last_phase_ms",
    "glass_gpu_grad_fisher_batch", "glass_gpu_grad_fisher_batch_host", "glass_gpu_set_template_size",
    "glass_gpu_dlogl_fp64_noalloc", "glass_wdm_window", "glass_gpu_wdm_forward", "glass_gpu_wdm_inverse",
    "glass_gpu_wdm_forward_host", "glass_gpu_wdm_inverse_host",
    "glass_gpu_wavelet_setup", "glass_gpu_wavelet_set_data", "glass_gpu_wavelet_dlogl_batch",
    "glass_gpu_wavelet_dlogl_batch_host", "glass_gpu_wavelet_waveform_batch", "glass_gpu_wavelet_waveform_batch_host",
    "glass_gpu_wdm_to_freq", "glass_gpu_wdm_from_freq", "build_wdm_filter_freq", "wavelet_transform_timefreq",
    "wavelet_transform_freq", "wavelet_transform_inverse_freq", "ucb_waveform_wavelet", "ucb_waveform_wavelet_tab",
    "ucb_waveform_wavelet_slow", "glass_ucb_waveform_wavelet_tab", "glass_ucb_waveform_wavelet_slow",
    "glass_gpu_wavelet_fisher_batch", "glass_gpu_wavelet_fisher_batch_host",
    "glass_gpu_fstat_batch", "glass_gpu_fstat_batch_host", "glass_gpu_fstat_proposal_host",
    "glass_gpu_noise_setup", "glass_gpu_noise_logl_batch", "glass_gpu_noise_logl_batch_host",
    "glass_gpu_noise_wavelet_setup", "glass_gpu_noise_wavelet_logl_batch", "glass_gpu_noise_wavelet_logl_batch_host",
    "glass_gpu_dlogl_batch_channels", "glass_gpu_noise_eta_batch", "glass_gpu_noise_eta_batch_host",
    "glass_gpu_rand_r_fill", "glass_gpu_mh_accept", "glass_gpu_fisher_draw", "glass_gpu_ptmcmc",
    "glass_gpu_set_mixed_tolerance", "glass_gpu_set_mixed_tolerance_scale", "glass_gpu_mixed_reevaluated",
    "glass_gpu_wdm_by_layers_host", "wavelet_transform_timefreq_by_layers", "glass_gpu_set_tuning",
    "glass_gpu_get_tuning", "glass_gpu_sym_eigen8", "glass_gpu_prior_draw", "glass_gpu_ucb_prior",
    "analytic_orbits", "initialize_analytic_orbit", "map_array_to_ucb_params", "ucb_alignment", "add_ucb_model",
    "remove_ucb_model", "generate_ucb_model", "update_ucb_model", "fourier_nwip", "snr", "gaussian_log_likelihood",
    "matrix_eigenstuff", "ucb_fisher", "wavelet_nwip", "snr_wavelet", "delta_log_likelihood", "ucb_fisher_wavelet",
    "glass_gpu_noise_sgwb_setup", "glass_gpu_noise_logl_batch_sgwb", "glass_gpu_noise_logl_batch_sgwb_host",
    "glass_gpu_noise_wavelet_logl_batch_sgwb", "glass_gpu_noise_wavelet_logl_batch_sgwb_host",
    "glass_gpu_checked_build", "glass_gpu_check_status",
    "glass_gpu_spline_noise_setup", "glass_gpu_spline_noise_logl_batch", "glass_gpu_spline_noise_logl_batch_host",
    "glass_gpu_noise_setup_channels", "glass_gpu_rj_propose", "glass_gpu_rj_accept", "glass_gpu_wavelet_reevaluated",
)

_lib = None


class GlassError(RuntimeError):
    pass


class FstatGrid(ctypes.Structure):
    """glass_gpu_fstat_grid: the F-statistic proposal's density grid (device
    tensor) for the trans-dimensional step's F-statistic draw."""
    _fields_ = [("tensor", ctypes.c_void_p), ("n_f", ctypes.c_int), ("n_theta", ctypes.c_int),
                ("n_phi", ctypes.c_int), ("d_f", ctypes.c_double), ("d_theta", ctypes.c_double),
                ("d_phi", ctypes.c_double), ("maxp", ctypes.c_double), ("qmin", ctypes.c_int),
                ("T", ctypes.c_double)]


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the compiled engine; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GlassError(f"{path} is missing: build it with `python -m glass_gb300.build`")
    lib = ctypes.CDLL(path)
    lib.glass_gpu_last_error.restype = ctypes.c_char_p
    lib.glass_gpu_create.argtypes = [ctypes.c_int, ctypes.POINTER(_V)]
    lib.glass_gpu_destroy.argtypes = [_V]
    lib.glass_gpu_set_stream.argtypes = [_V, _V]
    lib.glass_gpu_last_launch_count.argtypes = [_V]
    lib.glass_gpu_set_phase_timing.argtypes = [_V, ctypes.c_int]
    lib.glass_gpu_fisher_draw.argtypes = [_V, ctypes.c_int] + [_V] * 7
    lib.glass_gpu_set_host_access.argtypes = [_V, ctypes.c_int]
    lib.glass_gpu_get_host_access.argtypes = [_V, _I, _I]
    lib.glass_gpu_last_phase_ms.argtypes = [_V, ctypes.POINTER(ctypes.c_float)]
    lib.glass_gpu_set_mixed_tolerance.argtypes = [_V, ctypes.c_double]
    lib.glass_gpu_set_mixed_tolerance_scale.argtypes = [_V, ctypes.c_int, _D]
    lib.glass_gpu_mixed_reevaluated.argtypes = [_V, _V]
    lib.glass_gpu_wavelet_reevaluated.argtypes = [_V, _V]
    lib.glass_gpu_set_tuning.argtypes = [_V, ctypes.c_char_p, ctypes.c_int]
    lib.glass_gpu_sym_eigen8.argtypes = [_V, ctypes.c_int, _V, _V, _V]
    lib.glass_gpu_prior_draw.argtypes = [_V, ctypes.c_int, _V, ctypes.c_int, _V, _V, _V, _V]
    lib.glass_gpu_ucb_prior.argtypes = [_V, ctypes.c_int, _V, _V, ctypes.c_int, _V, _V, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, _V]
    lib.glass_gpu_get_tuning.argtypes = [_V, ctypes.c_char_p, _V]
    lib.glass_gpu_bank_upload.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, _I, _D, _D, _D, _D]
    lib.glass_gpu_bank_set_residual.argtypes = [_V, ctypes.c_int, _D, _D]
    lib.glass_gpu_dlogl_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V, _V, _V, _V]
    lib.glass_gpu_dlogl_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D, _D, _D, _I]
    lib.glass_ucb_waveform.argtypes = [_D, ctypes.c_char_p, ctypes.c_double, ctypes.c_double, _D, ctypes.c_int,
                                       _D, _D, _D, _D, _D, ctypes.c_int, ctypes.c_int]
    lib.ucb_bandwidth.argtypes = [ctypes.c_double] * 7 + [ctypes.c_int]
    lib.ucb_bandwidth.restype = ctypes.c_int
    lib.glass_gpu_grad_fisher_batch.argtypes = [_V, ctypes.c_int, _V, _V, ctypes.c_int, _V, _V, _V, _V]
    lib.glass_gpu_grad_fisher_batch_host.argtypes = [_V, ctypes.c_int, _I, _D, ctypes.c_int, _D, _D, _D, _I]
    lib.glass_gpu_set_template_size.argtypes = [_V, ctypes.c_int]
    lib.glass_gpu_dlogl_fp64_noalloc.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_int] + [_V] * 5 + [ctypes.c_int] + [_V] * 7
    lib.glass_wdm_window.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _D]
    wdm_args = [_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
    lib.glass_gpu_wdm_forward.argtypes = wdm_args + [_V, _V]
    lib.glass_gpu_wdm_inverse.argtypes = wdm_args + [_V, _V]
    lib.glass_gpu_wdm_forward_host.argtypes = wdm_args + [_D, _D]
    lib.glass_gpu_wdm_inverse_host.argtypes = wdm_args + [_D, _D]
    lib.glass_gpu_wdm_to_freq.argtypes = wdm_args + [_V, _V]
    lib.glass_gpu_wdm_from_freq.argtypes = wdm_args + [_V, _V]
    lib.glass_ucb_waveform_wavelet_tab.argtypes = []
    lib.glass_ucb_waveform_wavelet_slow.argtypes = []
    lib.glass_gpu_wavelet_setup.argtypes = [_V, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
    lib.glass_gpu_wavelet_set_data.argtypes = [_V, _D, _D, _D, _D]
    lib.glass_gpu_wavelet_dlogl_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 6
    lib.glass_gpu_wavelet_dlogl_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D, _D, _I]
    lib.glass_gpu_wavelet_waveform_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 4
    lib.glass_gpu_wavelet_waveform_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _D, _I, _D, _I]
    lib.glass_gpu_wavelet_fisher_batch.argtypes = [_V, ctypes.c_int, _V, ctypes.c_int, ctypes.c_int, _V, _V]
    lib.glass_gpu_wavelet_fisher_batch_host.argtypes = [_V, ctypes.c_int, _D, ctypes.c_int, ctypes.c_int, _D, _I]
    lib.glass_gpu_fstat_batch.argtypes = [_V, ctypes.c_int, _V, _V, _V, _V, _V]
    lib.glass_gpu_fstat_batch_host.argtypes = [_V, ctypes.c_int, _I, _D, _D, _D, _I]
    lib.glass_gpu_fstat_proposal_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
    lib.glass_gpu_noise_setup.argtypes = [_V, ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _D, _D]
    lib.glass_gpu_noise_logl_batch.argtypes = [_V, ctypes.c_int, _V, _V, _V]
    lib.glass_gpu_noise_logl_batch_host.argtypes = [_V, ctypes.c_int, _D, _D, _D]
    lib.glass_gpu_noise_wavelet_setup.argtypes = [_V, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]
    lib.glass_gpu_noise_wavelet_logl_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V, _V]
    lib.glass_gpu_noise_wavelet_logl_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _D, _D, _D]
    lib.glass_gpu_noise_sgwb_setup.argtypes = [_V, ctypes.c_int, ctypes.c_int, _D]
    lib.glass_gpu_check_status.argtypes = [_V, ctypes.POINTER(ctypes.c_uint)]
    lib.glass_gpu_rj_propose.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V, ctypes.c_int, _V, _D,
                                         ctypes.POINTER(FstatGrid)] + [_V] * 9
    lib.glass_gpu_rj_accept.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 11 + [
        ctypes.c_int, ctypes.c_int, _V, ctypes.c_int, _V, _V, ctypes.c_double, ctypes.c_double, ctypes.c_int, _V, _V,
        _V]
    lib.glass_gpu_noise_setup_channels.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _D,
                                                   _D, _D]
    lib.glass_gpu_spline_noise_setup.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _D,
                                                 _D, _D]
    lib.glass_gpu_spline_noise_logl_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V]
    lib.glass_gpu_spline_noise_logl_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D]
    lib.glass_gpu_noise_logl_batch_sgwb.argtypes = [_V, ctypes.c_int, _V, _V, _V, _V]
    lib.glass_gpu_noise_logl_batch_sgwb_host.argtypes = [_V, ctypes.c_int, _D, _D, _D, _D]
    lib.glass_gpu_noise_wavelet_logl_batch_sgwb.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V, _V, _V]
    lib.glass_gpu_noise_wavelet_logl_batch_sgwb_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]
    lib.glass_gpu_dlogl_batch_channels.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 8
    lib.glass_gpu_noise_eta_batch.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 6
    lib.glass_gpu_noise_eta_batch_host.argtypes = [_V, ctypes.c_int, ctypes.c_int, _I, _D, _D, _D, _D, _I]
    lib.glass_gpu_rand_r_fill.argtypes = [_V, ctypes.c_int, ctypes.c_int, _V, _V]
    lib.glass_gpu_mh_accept.argtypes = [_V, ctypes.c_int] + [_V] * 12
    lib.glass_gpu_ptmcmc.argtypes = [_V, ctypes.c_int, ctypes.c_int] + [_V] * 6
    _lib = lib
    return lib


def _check(rc: int):
    if rc != 0:
        raise GlassError(f"glass_gb300 error {rc}: {_lib.glass_gpu_last_error().decode()}")


def _pd(a):
    return a.ctypes.data_as(_D)


def _pi(a):
    return a.ctypes.data_as(_I)


def _ptr(x):
    """Device address of a tensor-like object (anything with data_ptr()), or None."""
    if x is None:
        return None
    return ctypes.c_void_p(int(x.data_ptr()))


def lib_constants() -> dict:
    """Integer #defines of include/glass_gb300.h."""
    import re

    path = os.path.join(os.path.dirname(HERE), "include", "glass_gb300.h")
    out = {}
    for m in re.finditer(r"^#define\s+(GLASS_\w+)\s+(-?\d+)\s*(?:/\*.*)?$", open(path).read(), flags=re.M):
        out[m.group(1)] = int(m.group(2))
    return out


def ucb_bandwidth(L, fstar, f, fdot, costheta, amp, T, NFFT) -> int:
    return load_library().ucb_bandwidth(L, fstar, f, fdot, costheta, amp, T, NFFT)


def ucb_waveform(params, N, T, t0=0.0, fmt="sangria", NI=2, NP=8, orbit_xyz=None):
    """Single template through the drop-in ucb_waveform path.

    Returns a (5, 2N) array X, Y, Z, A, E in the reference layout.  With
    orbit_xyz (N x 3 x 3 positions in metres) the given orbit is used; otherwise
    the analytic orbit.
    """
    lib = load_library()
    p = np.ascontiguousarray(params, np.float64)
    out = np.zeros((5, 2 * N))
    ox = None if orbit_xyz is None else np.ascontiguousarray(orbit_xyz, np.float64)
    rc = lib.glass_ucb_waveform(_pd(ox) if ox is not None else None, fmt.encode(), T, t0, _pd(p), NP,
                                *[_pd(out[i]) for i in range(5)], N, NI)
    _check(rc)
    return out


PROBE_PATH = os.path.join(HERE, "lib", "libglass_probe.so")


def probe_fma_tflops(device: int = 0, fp64: bool = False) -> float:
    """Measured FMA throughput of the FP32 or FP64 pipe (TFLOP/s), from the
    benchmark's probe library (lib/libglass_probe.so, not part of the
    engine)."""
    if not os.path.exists(PROBE_PATH):
        raise GlassError(f"{PROBE_PATH} is not built (python -m glass_gb300.build)")
    lib = ctypes.CDLL(PROBE_PATH)
    lib.glass_gpu_probe_fma_tflops.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = ctypes.c_double()
    rc = lib.glass_gpu_probe_fma_tflops(device, int(fp64), ctypes.byref(out))
    if rc != 0:
        raise GlassError(f"FMA probe failed ({rc})")
    return out.value


WDM_NX = 6.0  # the reference's window exponent (WAVELET_FILTER_CONSTANT)


def wdm_window(NF: int, NT: int, A: float = 0.0, nx: float = WDM_NX, forward: bool = True) -> np.ndarray:
    """Meyer window phif[0..NT/2] of the WDM transform (host computation)."""
    out = np.empty(NT // 2 + 1)
    _check(load_library().glass_wdm_window(NF, NT, A, nx, int(forward), _pd(out)))
    return out


class Engine:
    """A context on one GPU holding a bank of A/E segments."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self._ctx = _V()
        _check(self.lib.glass_gpu_create(device, ctypes.byref(self._ctx)))
        self.nseg = 0
        self.NFFT = 0

    def close(self):
        if self._ctx:
            self.lib.glass_gpu_destroy(self._ctx)
            self._ctx = _V()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        _check(self.lib.glass_gpu_set_stream(self._ctx, _V(stream_handle) if stream_handle else None))

    def upload(self, bank, fmt: str = "sangria"):
        """bank: glass_gb300.workloads.SegmentBank (complex data, real invC)."""
        rA, rE = bank.interleaved()
        rA = np.ascontiguousarray(rA, np.float64)
        rE = np.ascontiguousarray(rE, np.float64)
        iA = np.ascontiguousarray(bank.invCA, np.float64)
        iE = np.ascontiguousarray(bank.invCE, np.float64)
        q = np.ascontiguousarray(bank.qmin, np.int32)
        _check(self.lib.glass_gpu_bank_upload(self._ctx, FORMATS[fmt], bank.T, bank.t0, bank.NFFT, len(q), _pi(q),
                                              _pd(rA), _pd(rE), _pd(iA), _pd(iE)))
        self.nseg, self.NFFT = len(q), bank.NFFT

    def set_residual(self, seg: int, rA, rE):
        rA = np.ascontiguousarray(rA, np.float64)
        rE = np.ascontiguousarray(rE, np.float64)
        _check(self.lib.glass_gpu_bank_set_residual(self._ctx, seg, _pd(rA), _pd(rE)))

    def dlogl_host(self, item_seg, params, term_x=None, precision=PREC_FP64):
        """Host arrays in, host arrays out: (dlogl, term_y, hh, status)."""
        seg = np.ascontiguousarray(item_seg, np.int32)
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        n = len(seg)
        assert p.shape[0] == n
        tx = None if term_x is None else np.ascontiguousarray(term_x, np.float64)
        dl, ty, hh = np.empty(n), np.empty(n), np.empty(n)
        st = np.empty(n, np.int32)
        _check(self.lib.glass_gpu_dlogl_batch_host(self._ctx, precision, n, _pi(seg), _pd(p),
                                                   _pd(tx) if tx is not None else None, _pd(dl), _pd(ty), _pd(hh),
                                                   _pi(st)))
        return dl, ty, hh, st

    def host_batch(self, n: int, with_term_x: bool = True) -> "HostBatch":
        """Host arrays for batches of n proposals, kept between calls (see HostBatch)."""
        return HostBatch(self, n, with_term_x)

    def dlogl_device(self, item_seg, params, dlogl, term_y=None, hh=None, status=None, term_x=None,
                     precision=PREC_MIXED):
        """Device tensors (int32 item_seg, float64 params [n,8], float64 outputs);
        asynchronous on the context's stream."""
        n = int(item_seg.numel())
        _check(self.lib.glass_gpu_dlogl_batch(self._ctx, precision, n, _ptr(item_seg), _ptr(params), _ptr(term_x),
                                              _ptr(dlogl), _ptr(term_y), _ptr(hh), _ptr(status)))

    def set_template_size(self, n: int = 0):
        """0: the reference's bandwidth rule; otherwise every proposal uses N = n."""
        _check(self.lib.glass_gpu_set_template_size(self._ctx, n))

    def grad_fisher_host(self, item_seg, params, fisher_mode=0, fisher=True):
        """Host arrays: (term_y [n], grad [n, 8], fisher [n, 8, 8] or None, status [n])."""
        seg = np.ascontiguousarray(item_seg, np.int32)
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        n = len(seg)
        ty, g = np.empty(n), np.empty((n, 8))
        F = np.empty((n, 8, 8)) if fisher else None
        st = np.empty(n, np.int32)
        _check(self.lib.glass_gpu_grad_fisher_batch_host(self._ctx, n, _pi(seg), _pd(p), fisher_mode,
                                                         _pd(ty), _pd(g), _pd(F) if F is not None else None,
                                                         _pi(st)))
        return ty, g, F, st

    def grad_fisher_device(self, item_seg, params, term_y, grad, fisher=None, status=None, fisher_mode=0):
        n = int(item_seg.numel())
        _check(self.lib.glass_gpu_grad_fisher_batch(self._ctx, n, _ptr(item_seg), _ptr(params), fisher_mode,
                                                    _ptr(term_y), _ptr(grad), _ptr(fisher), _ptr(status)))

    def wdm_forward_host(self, NF, NT, time, precision=PREC_FP64, A=0.0, nx=WDM_NX):
        """Time series (NF*NT) -> WDM coefficients (NF*NT, layout n + NT*m)."""
        x = np.ascontiguousarray(time, np.float64).reshape(-1)
        assert x.size == NF * NT
        out = np.empty(NF * NT)
        _check(self.lib.glass_gpu_wdm_forward_host(self._ctx, precision, NF, NT, A, nx, _pd(x), _pd(out)))
        return out

    def wdm_inverse_host(self, NF, NT, wdm, precision=PREC_FP64, A=0.0, nx=WDM_NX):
        w = np.ascontiguousarray(wdm, np.float64).reshape(-1)
        assert w.size == NF * NT
        out = np.empty(NF * NT)
        _check(self.lib.glass_gpu_wdm_inverse_host(self._ctx, precision, NF, NT, A, nx, _pd(w), _pd(out)))
        return out

    def wdm_forward_device(self, NF, NT, time, wdm, precision=PREC_FP64, A=0.0, nx=WDM_NX):
        """Device tensors of NF*NT float64; asynchronous on the context's stream."""
        _check(self.lib.glass_gpu_wdm_forward(self._ctx, precision, NF, NT, A, nx, _ptr(time), _ptr(wdm)))

    def wdm_inverse_device(self, NF, NT, wdm, time, precision=PREC_FP64, A=0.0, nx=WDM_NX):
        _check(self.lib.glass_gpu_wdm_inverse(self._ctx, precision, NF, NT, A, nx, _ptr(wdm), _ptr(time)))

    # --- wavelet-domain UCB path ---------------------------------------------------
    WV_MAX_LAYERS = 3

    def wavelet_setup(self, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax, A=0.0, nx=WDM_NX, orbit=None):
        """Segment of pixels [kmin, kmax) of an NF x NT grid (pixel duration wdt,
        bandwidth wdf).  orbit: (t [n], positions [3, 3, n] metres) or None for
        the interpolated analytic orbit."""
        if orbit is None:
            ot = op = None
            n = 0
        else:
            ot = np.ascontiguousarray(orbit[0], np.float64)
            op = np.ascontiguousarray(orbit[1], np.float64)
            n = len(ot)
        _check(self.lib.glass_gpu_wavelet_setup(self._ctx, Tobs, t0, NF, NT, wdt, wdf, A, nx, kmin, kmax, n,
                                                _pd(ot) if ot is not None else None,
                                                _pd(op) if op is not None else None))
        self.wv = dict(NT=NT, kmin=kmin, kmax=kmax, N=kmax - kmin)

    def wavelet_set_data(self, res, invC):
        """res: [3, N] residual X, Y, Z; invC: [3, 3, N] inverse covariance."""
        r = np.ascontiguousarray(res, np.float64)
        ic = np.ascontiguousarray(invC, np.float64)
        _check(self.lib.glass_gpu_wavelet_set_data(self._ctx, _pd(r[0]), _pd(r[1]), _pd(r[2]), _pd(ic)))

    def wavelet_waveform_host(self, params, values=True, precision=PREC_FP64):
        """(info [n, 4] = first layer, layers, first kept layer, kept layers
        (-1 when the parameters are invalid), xyz [n, 3, 3 NT] or None when
        values is False, status [n])."""
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        n = len(p)
        NT = self.wv["NT"]
        info = np.zeros((n, 4), np.int32)
        xyz = np.zeros((n, 3, self.WV_MAX_LAYERS * NT)) if values else None
        st = np.zeros(n, np.int32)
        _check(self.lib.glass_gpu_wavelet_waveform_batch_host(self._ctx, precision, n, _pd(p), _pi(info),
                                                              _pd(xyz) if values else None, _pi(st)))
        return info, xyz, st

    def wavelet_list(self, info_row):
        """Pixel list (k - kmin) of one item, in the order of its values."""
        _, _, jlo, c = (int(v) for v in info_row)
        NT, kmin = self.wv["NT"], self.wv["kmin"]
        if c <= 0:
            return np.zeros(0, np.int32)
        i = np.repeat(np.arange(NT), c)
        j = jlo + np.tile(np.arange(c), NT)
        return (i + j * NT - kmin).astype(np.int32)

    def wavelet_dlogl_host(self, params, term_x=None, precision=PREC_FP64):
        """(dlogl, term_y, hh, status) with term = (h|h) - 2 (d|h) over the
        item's pixels and dlogl = -(term_y - term_x)/2."""
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        n = len(p)
        tx = None if term_x is None else np.ascontiguousarray(term_x, np.float64)
        dl, ty, hh = np.empty(n), np.empty(n), np.empty(n)
        st = np.empty(n, np.int32)
        _check(self.lib.glass_gpu_wavelet_dlogl_batch_host(self._ctx, precision, n, _pd(p),
                                                           _pd(tx) if tx is not None else None,
                                                           _pd(dl), _pd(ty), _pd(hh), _pi(st)))
        return dl, ty, hh, st

    def wavelet_fisher_host(self, params, imin, imax):
        """(fisher [n, 8, 8], status [n]): ucb_fisher_wavelet for each source,
        over time pixels imin < t < imax."""
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        n = len(p)
        F = np.zeros((n, 8, 8))
        st = np.zeros(n, np.int32)
        _check(self.lib.glass_gpu_wavelet_fisher_batch_host(self._ctx, n, _pd(p), int(imin), int(imax), _pd(F),
                                                            _pi(st)))
        return F, st

    def fstat_host(self, cell_seg, cells):
        """F-statistic of cells (f0, fdot, theta, phi) on the bank's segments:
        (logL_AE [n], fparams [n, 4] = A, iota, psi, phase, status [n])."""
        seg = np.ascontiguousarray(cell_seg, np.int32)
        c = np.ascontiguousarray(cells, np.float64).reshape(-1, 4)
        n = len(seg)
        assert c.shape[0] == n
        ll, fp, st = np.empty(n), np.empty((n, 4)), np.empty(n, np.int32)
        _check(self.lib.glass_gpu_fstat_batch_host(self._ctx, n, _pi(seg), _pd(c), _pd(ll), _pd(fp), _pi(st)))
        return ll, fp, st

    def fstat_device(self, cell_seg, cells, logl, fparams=None, status=None):
        """Device tensors (int32 cell_seg, float64 cells [n, 4], float64 outputs);
        asynchronous on the context's stream."""
        n = int(cell_seg.numel())
        _check(self.lib.glass_gpu_fstat_batch(self._ctx, n, _ptr(cell_seg), _ptr(cells), _ptr(logl), _ptr(fparams),
                                              _ptr(status)))

    def fstat_proposal_host(self, seg, n_theta=20, n_phi=20):
        """build_fstatistic_proposal on one segment: (tensor [n_f, n_theta, n_phi],
        norm, maxp, number of cells that ran the chirp-mass scan)."""
        tensor = np.empty(self.NFFT * n_theta * n_phi)
        info = np.zeros(4)
        _check(self.lib.glass_gpu_fstat_proposal_host(self._ctx, int(seg), int(n_theta), int(n_phi), _pd(tensor),
                                                      _pd(info)))
        n_f = int(info[0])
        return tensor[:n_f * n_theta * n_phi].reshape(n_f, n_theta, n_phi), info[1], info[2], int(info[3])

    def noise_setup(self, T, qmin, X, Y, Z):
        """XYZ data (interleaved, 2 NFFT each) on the bins qmin/T + n/T."""
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        _check(self.lib.glass_gpu_noise_setup(self._ctx, float(T), int(qmin), len(X) // 2, _pd(X), _pd(Y), _pd(Z)))

    def noise_setup_channels(self, T, qmin, d0, d1=None, d2=None):
        """One channel (d0 = X), two (d0, d1 = A, E) or three (X, Y, Z),
        interleaved (2 NFFT each), on the bins qmin/T + n/T."""
        ds = [np.ascontiguousarray(a, np.float64) for a in (d0, d1, d2) if a is not None]
        ptr = [_pd(a) for a in ds] + [None] * (3 - len(ds))
        _check(self.lib.glass_gpu_noise_setup_channels(self._ctx, len(ds), float(T), int(qmin), len(ds[0]) // 2, *ptr))

    def noise_sgwb_setup(self, sgwb_type, resp=None):
        """The SGWB template (0 power law, 1 lognormal, 2 phase transition; -1
        none) and the response table rows [n, 7] = f, XX, YY, ZZ, XY, XZ, YZ."""
        r = None if resp is None else np.ascontiguousarray(resp, np.float64).reshape(-1, 7)
        _check(self.lib.glass_gpu_noise_sgwb_setup(self._ctx, int(sgwb_type), 0 if r is None else len(r),
                                                   _pd(r) if r is not None else None))

    def noise_logl_host(self, inst, sgal=None, sgwb=None):
        """my_noise_log_likelihood of each noise model: inst [n, 12], sgal [n, 5]
        or None, sgwb [n, 4] (the template's parameters first) or None."""
        i = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        g = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        b = None if sgwb is None else np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        out = np.empty(len(i))
        _check(self.lib.glass_gpu_noise_logl_batch_sgwb_host(self._ctx, len(i), _pd(i),
                                                             _pd(g) if g is not None else None,
                                                             _pd(b) if b is not None else None, _pd(out)))
        return out

    def noise_logl_device(self, inst, logl, sgal=None, sgwb=None):
        """Device tensors: inst [n, 12], sgal [n, 5] or None, sgwb [n, 4] or
        None, logl [n]; asynchronous."""
        n = int(inst.shape[0])
        _check(self.lib.glass_gpu_noise_logl_batch_sgwb(self._ctx, n, _ptr(inst), _ptr(sgal), _ptr(sgwb), _ptr(logl)))

    def spline_noise_setup(self, T, qmin, transfer, d0, d1=None):
        """The spline noise model's data: transfer [NFFT] and one (d0) or two
        (d0, d1) channels, interleaved (2 NFFT each), on the bins qmin/T + n/T."""
        tr = np.ascontiguousarray(transfer, np.float64)
        a = np.ascontiguousarray(d0, np.float64)
        b = None if d1 is None else np.ascontiguousarray(d1, np.float64)
        _check(self.lib.glass_gpu_spline_noise_setup(self._ctx, 1 if b is None else 2, float(T), int(qmin), len(tr),
                                                     _pd(tr), _pd(a), _pd(b) if b is not None else None))

    def spline_noise_logl_host(self, nknots, knot_f, knot_C):
        """noise_log_likelihood per model: nknots [n], knot_f [n, kmax],
        knot_C [n, nchannel, kmax]."""
        k = np.ascontiguousarray(nknots, np.int32)
        f = np.ascontiguousarray(knot_f, np.float64)
        c = np.ascontiguousarray(knot_C, np.float64)
        out = np.empty(len(k))
        _check(self.lib.glass_gpu_spline_noise_logl_batch_host(self._ctx, len(k), f.shape[1], _pi(k), _pd(f), _pd(c),
                                                               _pd(out)))
        return out

    def spline_noise_logl_device(self, nknots, knot_f, knot_C, logl):
        """Device tensors as spline_noise_logl_host's arrays; asynchronous."""
        n = int(nknots.numel())
        _check(self.lib.glass_gpu_spline_noise_logl_batch(self._ctx, n, int(knot_f.shape[1]), _ptr(nknots),
                                                          _ptr(knot_f), _ptr(knot_C), _ptr(logl)))

    def noise_wavelet_setup(self, NF, NT, df, lmin, Q, X, Y, Z, mod=None):
        """Wavelet data (pixel i of layer j at i + j NT) on layers lmin.., cells of Q
        pixels, and the foreground modulation [6, NT/Q] (or None)."""
        X, Y, Z = (np.ascontiguousarray(a, np.float64) for a in (X, Y, Z))
        md = None if mod is None else np.ascontiguousarray(mod, np.float64)
        _check(self.lib.glass_gpu_noise_wavelet_setup(self._ctx, int(NF), int(NT), float(df), int(lmin),
                                                      len(X) // int(NT), int(Q), _pd(X), _pd(Y), _pd(Z),
                                                      _pd(md) if md is not None else None))

    def noise_wavelet_logl_host(self, inst, sgal=None, mode=0, sgwb=None):
        i = np.ascontiguousarray(inst, np.float64).reshape(-1, 12)
        g = None if sgal is None else np.ascontiguousarray(sgal, np.float64).reshape(-1, 5)
        b = None if sgwb is None else np.ascontiguousarray(sgwb, np.float64).reshape(-1, 4)
        out = np.empty(len(i))
        _check(self.lib.glass_gpu_noise_wavelet_logl_batch_sgwb_host(self._ctx, int(mode), len(i), _pd(i),
                                                                     _pd(g) if g is not None else None,
                                                                     _pd(b) if b is not None else None, _pd(out)))
        return out

    def noise_wavelet_logl_device(self, inst, logl, sgal=None, mode=0, sgwb=None):
        n = int(inst.shape[0])
        _check(self.lib.glass_gpu_noise_wavelet_logl_batch_sgwb(self._ctx, int(mode), n, _ptr(inst), _ptr(sgal),
                                                                _ptr(sgwb), _ptr(logl)))

    def dlogl_channels_device(self, item_seg, params, dlogl, term_ch, term_y=None, hh=None, status=None, term_x=None,
                              precision=PREC_MIXED):
        """glass_gpu_dlogl_batch with per-channel terms term_ch [n, 2] (device tensors)."""
        n = int(item_seg.numel())
        _check(self.lib.glass_gpu_dlogl_batch_channels(self._ctx, precision, n, _ptr(item_seg), _ptr(params),
                                                       _ptr(term_x), _ptr(dlogl), _ptr(term_y), _ptr(hh),
                                                       _ptr(status), _ptr(term_ch)))

    def noise_eta_host(self, item_seg, params, eta_x, eta_y, precision=PREC_MIXED):
        """(logL + logLnorm)(eta_y) - (logL + logLnorm)(eta_x) per chain, and status."""
        seg = np.ascontiguousarray(item_seg, np.int32)
        p = np.ascontiguousarray(params, np.float64).reshape(-1, 8)
        ex = np.ascontiguousarray(eta_x, np.float64).reshape(-1, 2)
        ey = np.ascontiguousarray(eta_y, np.float64).reshape(-1, 2)
        n = len(seg)
        out, st = np.empty(n), np.empty(n, np.int32)
        _check(self.lib.glass_gpu_noise_eta_batch_host(self._ctx, precision, n, _pi(seg), _pd(p), _pd(ex), _pd(ey),
                                                       _pd(out), _pi(st)))
        return out, st

    def rand_r_fill_device(self, seed, out):
        """seed: int32 tensor [n] (unsigned bit pattern), out: int32 [n, count]."""
        n, count = int(out.shape[0]), int(out.shape[1])
        _check(self.lib.glass_gpu_rand_r_fill(self._ctx, n, count, _ptr(seed), _ptr(out)))

    def mh_accept_device(self, temperature, dlogl, logPx, logPy, logQxy, logQyx, seed, logL_x, params_x, params_y,
                         accepted=None, snr=None):
        n = int(dlogl.numel())
        _check(self.lib.glass_gpu_mh_accept(self._ctx, n, _ptr(temperature), _ptr(dlogl), _ptr(logPx), _ptr(logPy),
                                            _ptr(logQxy), _ptr(logQyx), _ptr(snr), _ptr(seed), _ptr(logL_x),
                                            _ptr(params_x), _ptr(params_y), _ptr(accepted)))

    def ptmcmc_device(self, temperature, logL, index, seed, acceptance, logLnorm=None):
        nens, NC = int(index.shape[0]), int(index.shape[1])
        _check(self.lib.glass_gpu_ptmcmc(self._ctx, nens, NC, _ptr(temperature), _ptr(logL), _ptr(logLnorm),
                                         _ptr(index), _ptr(seed), _ptr(acceptance)))

    def sym_eigen8_device(self, matrix, evec, evalue):
        """Eigen-decomposition of n symmetric 8x8 matrices (glass_gpu_sym_eigen8)."""
        n = int(matrix.numel() // 64)
        _check(self.lib.glass_gpu_sym_eigen8(self._ctx, n, _ptr(matrix), _ptr(evec), _ptr(evalue)))

    def prior_draw_device(self, prior, logPV, seed, params, logQ, per_chain=False):
        """draw_from_uniform_prior for n chains (glass_gpu_prior_draw)."""
        n = int(seed.numel())
        _check(self.lib.glass_gpu_prior_draw(self._ctx, n, _ptr(prior), int(per_chain), _ptr(logPV), _ptr(seed),
                                             _ptr(params), _ptr(logQ)))

    def ucb_prior_device(self, params, prior, logPV, logP, per_chain=False, skyhist=None, dcostheta=0.0, dphi=0.0,
                         nphi=0):
        """evaluate_ucb_prior for n chains (glass_gpu_ucb_prior); params wrapped in place."""
        n = int(params.numel() // 8)
        _check(self.lib.glass_gpu_ucb_prior(self._ctx, n, _ptr(params), _ptr(prior), int(per_chain), _ptr(logPV),
                                            _ptr(skyhist), float(dcostheta), float(dphi), int(nphi), _ptr(logP)))

    @staticmethod
    def fstat_grid(tensor, d_f, d_theta, d_phi, maxp, qmin, T):
        """The F-statistic draw's grid: tensor a device array [n_f, n_theta, n_phi]."""
        g = FstatGrid(ctypes.c_void_p(tensor.data_ptr()), int(tensor.shape[0]), int(tensor.shape[1]),
                      int(tensor.shape[2]), float(d_f), float(d_theta), float(d_phi), float(maxp), int(qmin), float(T))
        g._keep = tensor
        return g

    def rj_propose_device(self, Nlive, Neff, src, prior, logPV, rjweight, grid, seed, per_chain=False):
        """The birth/death proposal of ucb_rjmcmc (glass_gpu_rj_propose) for n
        chains: device tensors Nlive, Neff (int32 [n]), src [n, maxsrc, 8],
        seed [n] (advanced); rjweight 9 host floats; grid from fstat_grid (or
        None).  Returns device tensors (move, slot, kind, params_y, logQxy,
        logQyx, logPy, status)."""
        import torch

        n, maxsrc = int(src.shape[0]), int(src.shape[1])
        dev = src.device
        move, slot, kind, status = (torch.empty(n, dtype=torch.int32, device=dev) for _ in range(4))
        y = torch.empty((n, 8), dtype=torch.float64, device=dev)
        qxy, qyx, lpy = (torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3))
        w = np.ascontiguousarray(rjweight, np.float64)
        _check(self.lib.glass_gpu_rj_propose(self._ctx, n, maxsrc, _ptr(Nlive), _ptr(Neff), _ptr(src), _ptr(prior),
                                             int(per_chain), _ptr(logPV), _pd(w),
                                             ctypes.byref(grid) if grid is not None else None, _ptr(seed), _ptr(move),
                                             _ptr(slot), _ptr(kind), _ptr(y), _ptr(qxy), _ptr(qyx), _ptr(lpy),
                                             _ptr(status)))
        return move, slot, kind, y, qxy, qyx, lpy, status

    def rj_accept_device(self, Nlive, src, proposal, temperature, dlogl, hh, prior, logPV, seed, logL_x,
                         dlogl_is_term=False, prior_only=False, per_chain=False, skyhist=None, dcostheta=0.0,
                         dphi=0.0, nphi=0, accepted=None):
        """The acceptance half of ucb_rjmcmc (glass_gpu_rj_accept) on the
        proposal rj_propose_device returned; Nlive, src, seed and logL_x are
        updated in place."""
        move, slot, _, y, qxy, qyx, lpy = proposal[:7]
        n, maxsrc = int(src.shape[0]), int(src.shape[1])
        _check(self.lib.glass_gpu_rj_accept(self._ctx, n, maxsrc, _ptr(Nlive), _ptr(src), _ptr(move), _ptr(slot),
                                            _ptr(y), _ptr(qxy), _ptr(qyx), _ptr(lpy), _ptr(temperature), _ptr(dlogl),
                                            _ptr(hh), int(dlogl_is_term), int(prior_only), _ptr(prior),
                                            int(per_chain), _ptr(logPV), _ptr(skyhist), float(dcostheta), float(dphi),
                                            int(nphi), _ptr(seed), _ptr(logL_x), _ptr(accepted)))

    def fisher_draw_device(self, params_x, evec, evalue, seed, params_y, logQ=None, status=None):
        """draw_from_fisher for n chains (device tensors: params_x/params_y [n, 8],
        evec [n, 8, 8] with evec[i, j, k] = fisher_evectr[j][k], evalue [n, 8],
        seed uint32/int32 [n] advanced in place)."""
        n = int(params_x.shape[0])
        _check(self.lib.glass_gpu_fisher_draw(self._ctx, n, _ptr(params_x), _ptr(evec), _ptr(evalue), _ptr(seed),
                                              _ptr(params_y), _ptr(logQ), _ptr(status)))

    def wavelet_dlogl_device(self, params, dlogl, term_y=None, hh=None, status=None, term_x=None,
                             precision=PREC_FP64):
        n = int(params.shape[0])
        _check(self.lib.glass_gpu_wavelet_dlogl_batch(self._ctx, precision, n, _ptr(params), _ptr(term_x), _ptr(dlogl),
                                                      _ptr(term_y), _ptr(hh), _ptr(status)))

    def last_launch_count(self) -> int:
        return self.lib.glass_gpu_last_launch_count(self._ctx)

    def set_host_access(self, mode: int = -1):
        """How dlogl_host moves data: 1 in place (the device reads and writes
        the host arrays), 0 pinned staging copies, -1 in place where supported."""
        _check(self.lib.glass_gpu_set_host_access(self._ctx, int(mode)))

    def host_access(self):
        """(supported, direct): in-place host access possible / in use."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        _check(self.lib.glass_gpu_get_host_access(self._ctx, ctypes.byref(a), ctypes.byref(b)))
        return bool(a.value), bool(b.value)

    def set_phase_timing(self, enable: bool):
        _check(self.lib.glass_gpu_set_phase_timing(self._ctx, int(bool(enable))))

    def last_phase_ms(self):
        """(plan, slow part, spectral, re-evaluation) milliseconds of the last
        dlogl batch launched with phase timing on."""
        ms = (ctypes.c_float * 4)()
        _check(self.lib.glass_gpu_last_phase_ms(self._ctx, ms))
        return tuple(float(v) for v in ms)

    def set_mixed_tolerance(self, tol: float = 1e-3):
        """Mixed precision: proposals whose estimated delta-logL error exceeds
        tol are evaluated again in higher precision within the same batch
        (tol <= 0: off)."""
        _check(self.lib.glass_gpu_set_mixed_tolerance(self._ctx, float(tol)))

    def set_mixed_tolerance_scale(self, scale=None):
        """Per-proposal tolerance tol * scale[i] (e.g. the chains'
        temperatures); None: tol for all."""
        if scale is None:
            _check(self.lib.glass_gpu_set_mixed_tolerance_scale(self._ctx, 0, None))
        else:
            sc = np.ascontiguousarray(scale, np.float64)
            _check(self.lib.glass_gpu_set_mixed_tolerance_scale(self._ctx, int(sc.size), _pd(sc)))

    def set_tuning(self, key: str, value: int):
        """One launch-shape parameter of the mixed path (glass_gpu_set_tuning)."""
        _check(self.lib.glass_gpu_set_tuning(self._ctx, key.encode(), int(value)))

    def get_tuning(self, key: str) -> int:
        v = ctypes.c_int(0)
        _check(self.lib.glass_gpu_get_tuning(self._ctx, key.encode(), ctypes.byref(v)))
        return v.value

    def apply_tuning(self, path: str | None = None) -> dict:
        """Applies the autotuner's table (glass_gb300/tuning.json by default)
        for this GPU model, if it has an entry; returns what was applied."""
        from . import tune

        return tune.apply(self, path)

    def mixed_reevaluated(self) -> int:
        """Number of proposals re-evaluated in double-float so far
        (synchronises the stream)."""
        n = ctypes.c_ulonglong(0)
        _check(self.lib.glass_gpu_mixed_reevaluated(self._ctx, ctypes.byref(n)))
        return int(n.value)

    def wavelet_reevaluated(self) -> int:
        """Number of wavelet-domain sources the mixed likelihood evaluated
        again in FP64 so far (synchronises the stream)."""
        n = ctypes.c_ulonglong(0)
        _check(self.lib.glass_gpu_wavelet_reevaluated(self._ctx, ctypes.byref(n)))
        return int(n.value)


class HostBatch:
    """The host arrays of one batch of n proposals for
    glass_gpu_dlogl_batch_host, with their C pointers resolved once: the way a
    C caller keeps its proposal and result buffers from one sampler step to the
    next.  Fill item_seg, params (n x 8) and term_x, call run(), read dlogl,
    term_y, hh and status."""

    def __init__(self, engine: Engine, n: int, with_term_x: bool = True):
        self.engine = engine
        self.n = int(n)
        self.item_seg = np.zeros(self.n, np.int32)
        self.params = np.zeros((self.n, 8))
        self.term_x = np.zeros(self.n) if with_term_x else None
        self.dlogl, self.term_y, self.hh = np.empty(self.n), np.empty(self.n), np.empty(self.n)
        self.status = np.empty(self.n, np.int32)
        self._fn = engine.lib.glass_gpu_dlogl_batch_host
        self._args = (_pi(self.item_seg), _pd(self.params), _pd(self.term_x) if with_term_x else None,
                      _pd(self.dlogl), _pd(self.term_y), _pd(self.hh), _pi(self.status))

    def run(self, precision: int = PREC_MIXED):
        """Evaluate the batch (synchronous); results in dlogl, term_y, hh, status."""
        _check(self._fn(self.engine._ctx, precision, self.n, *self._args))
