"""The C-ABI library loads and exports every symbol include/glass_gb300.h
declares; host-only entry points agree with the reference (no GPU needed)."""
import os
import re

import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from glass_gb300 import build

    build.build()
    return gg.load_library()


def _declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w \*]*?)\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_what_the_module_binds():
    declared = _declared_functions()
    assert set(declared) == set(gg.EXPORTS), (declared, gg.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in _declared_functions():
        assert hasattr(lib, name), name


def test_bound_argument_counts_match_the_header(lib):
    """Every glass_gpu_* binding with argtypes has as many as the header's
    declaration has parameters (ctypes would pass a short list silently
    shifted or refuse it at call time)."""
    text = ""
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text += open(os.path.join(ROOT, "include", h)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    checked = 0
    for m in re.finditer(r"\b(glass_gpu_\w+)\s*\(([^;{]*)\)\s*;", text):
        name, params = m.group(1), m.group(2).strip()
        n = 0 if params in ("", "void") else len(params.split(","))
        at = getattr(lib, name).argtypes
        if at is None:
            continue
        assert len(at) == n, (name, len(at), n)
        checked += 1
    assert checked > 50


def test_ucb_bandwidth_matches_reference(lib, golden):
    g = golden("bandwidth.npz")
    L, fstar = 2.5e9, wl.FSTAR
    got = np.array([gg.ucb_bandwidth(L, fstar, g["f"][i], g["fdot"][i], g["costh"][i], g["amp"][i], wl.T_YEAR,
                                     int(g["nfft"][i])) for i in range(len(g["f"]))])
    np.testing.assert_array_equal(got, g["bw"])


def test_errors_are_reported_without_a_gpu(lib):
    """Argument checks run before any device call."""
    p = np.zeros(8)
    out = np.zeros((5, 2 * 48))
    rc = lib.glass_ucb_waveform(None, b"sangria", 1.0, 0.0, p.ctypes.data_as(gg._D), 8,
                                *[out[i].ctypes.data_as(gg._D) for i in range(5)], 48, 2)
    assert rc == -2  # GLASS_ERR_SIZE: 48 is not a power of two
    rc = lib.glass_ucb_waveform(None, b"nonsense", 1.0, 0.0, p.ctypes.data_as(gg._D), 8,
                                *[out[i].ctypes.data_as(gg._D) for i in range(5)], 32, 2)
    assert rc == -4  # GLASS_ERR_FORMAT
    assert b"Unsupported" in lib.glass_gpu_last_error()


def test_wdm_window_matches_reference(lib, golden):
    """glass_wdm_window (host) against build_wdm_filter_freq's own output."""
    g = golden("wdm.npz")
    for NF, NT in g["grids"]:
        key = f"{NF}x{NT}"
        np.testing.assert_array_equal(gg.wdm_window(int(NF), int(NT)), g[f"win_{key}"])
        np.testing.assert_array_equal(gg.wdm_window(int(NF), int(NT), forward=False), g[f"winv_{key}"])
    with pytest.raises(gg.GlassError):
        gg.wdm_window(32, 63)


def test_unbuilt_wavelet_variants_report_a_status(lib):
    """ucb_waveform_wavelet_tab / _slow are API-only here; their status forms
    say so without touching a GPU."""
    c = gg.lib_constants()
    assert lib.glass_ucb_waveform_wavelet_tab() == c["GLASS_ERR_STATE"]
    assert b"not implemented" in lib.glass_gpu_last_error()
    assert lib.glass_ucb_waveform_wavelet_slow() == c["GLASS_ERR_STATE"]
    assert b"not built" in lib.glass_gpu_last_error()


def test_wavelet_setup_argument_checks(lib):
    """Grid checks of glass_gpu_wavelet_setup run before any device call."""
    import ctypes

    c = gg.lib_constants()
    f = lib.glass_gpu_wavelet_setup
    V = ctypes.c_void_p(1)  # never dereferenced: the checks fail first
    assert f(V, 1e6, 0.0, 64, 250, 1.0, 0.5, 0.0, 6.0, 0, 250, 0, None, None) == c["GLASS_ERR_SIZE"]
    assert f(V, 1e6, 0.0, 64, 256, 1.0, 0.5, 0.0, 6.0, 100, 512, 0, None, None) == c["GLASS_ERR_ARG"]
    assert f(V, -1.0, 0.0, 64, 256, 1.0, 0.5, 0.0, 6.0, 0, 512, 0, None, None) == c["GLASS_ERR_ARG"]


def test_tuning_table_applies_the_entry_of_this_gpu(tmp_path, monkeypatch):
    """glass_gb300.tune.apply sets the recorded knobs of the GPU model it runs
    on, and nothing for a model the table does not know."""
    import json

    from glass_gb300 import tune

    table = {"GB300 test": {"knobs": {"slow_block": 128, "spec_ctas_per_sm": 2}}}
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps(table))

    class FakeEngine:
        def __init__(self):
            self.set = {}

        def set_tuning(self, k, v):
            self.set[k] = v

    monkeypatch.setattr(tune, "gpu_name", lambda device=0: "GB300 test")
    eng = FakeEngine()
    assert tune.apply(eng, str(path)) == {"slow_block": 128, "spec_ctas_per_sm": 2}
    assert eng.set == {"slow_block": 128, "spec_ctas_per_sm": 2}
    monkeypatch.setattr(tune, "gpu_name", lambda device=0: "other")
    eng = FakeEngine()
    assert tune.apply(eng, str(path)) == {} and eng.set == {}
