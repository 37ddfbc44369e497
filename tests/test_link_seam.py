"""The drop-in link seam with the reference itself: when the reference's
library is a shared object (here oracle/_ref/libglassref.so, compiled from the
reference's sources by oracle/Makefile.ref) and this library is loaded ahead
of it, the reference's own calls to the drop-in symbols (its samplers calling
ucb_fisher, generate_ucb_model, gaussian_log_likelihood; ucb_fisher calling
ucb_alignment, ucb_waveform, matrix_eigenstuff; ucb_waveform_wavelet calling
wavelet_transform_timefreq_by_layers, ...) bind to this library.  Checked
through the dynamic linker's binding log with every symbol bound at load, so no
GPU is needed.  (Against the reference's default static archive the archive's
definitions win; the integration notes say so.)"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "libglassref.so")
OURS = os.path.join(ROOT, "glass_gb300", "lib", "libglass_gb300.so")


@pytest.mark.skipif(not (os.path.exists(REF) and os.path.exists(OURS)),
                    reason="needs the reference built as a shared object and this library built")
def test_reference_calls_bind_to_the_drop_ins():
    code = ("import ctypes; ctypes.CDLL(%r, mode=ctypes.RTLD_GLOBAL); ctypes.CDLL(%r)" % (OURS, REF))
    env = dict(os.environ, LD_BIND_NOW="1", LD_DEBUG="bindings")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    log = out.stderr
    # every drop-in the reference's own code calls (update_ucb_model has no
    # caller inside the reference library: the apps call it)
    for sym in ("ucb_waveform", "ucb_bandwidth", "analytic_orbits", "initialize_analytic_orbit",
                "map_array_to_ucb_params", "ucb_alignment", "add_ucb_model", "remove_ucb_model", "generate_ucb_model",
                "fourier_nwip", "snr", "gaussian_log_likelihood", "matrix_eigenstuff", "ucb_fisher",
                "wavelet_transform_timefreq_by_layers", "wavelet_transform_timefreq", "build_wdm_filter_freq",
                "wavelet_transform_freq", "wavelet_transform_inverse_freq", "ucb_waveform_wavelet", "wavelet_nwip",
                "snr_wavelet", "delta_log_likelihood", "ucb_fisher_wavelet"):
        lines = [ln for ln in log.splitlines() if "libglassref.so" in ln.split(" to ")[0] and f"`{sym}'" in ln]
        assert lines, sym
        assert all("libglass_gb300.so" in ln.split(" to ")[1] for ln in lines), lines
