"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""

import ctypes
import os
import re

from jaxabm_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "jaxabm_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"ABM_API\s+[\w\s\*]+?\b(abm_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "abm_rng_split" in syms and "abm_randomwalk_run" in syms
    assert len(syms) >= 15


def test_every_declared_symbol_is_exported(lib):
    raw = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(raw, s)]
    assert not missing, missing


def test_every_declared_symbol_is_bound(lib):
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_status_strings(lib):
    assert lib.abm_status_string(0) == b"ok"
    assert lib.abm_status_string(_lib.ABM_ERR_WORKSPACE) == b"workspace too small"
    assert lib.abm_version() >= 100


def test_bad_arguments_rejected_without_gpu(lib):
    # argument validation happens before any CUDA call
    assert lib.abm_rng_split(None, 1, 2, None, 1, None) == _lib.ABM_ERR_BADARG
    assert lib.abm_randomwalk_run(None, None, 10, None, 5, 0.01, None, None, 0, None) == \
        _lib.ABM_ERR_BADARG
    assert lib.abm_randomwalk_workspace_bytes(10_000, 100) > 0


def test_sir_resident_entry_points_without_gpu(lib):
    """Host-side sizing and argument checks of the resident SIR path need no device: the
    scratch is a 256-byte queue header plus three 4-byte lists of max_agents (rounded to 16)
    entries per CTA; without a device no instance fits (0); bad arguments are rejected
    before any CUDA call."""
    assert lib.abm_sir_resident_scratch_bytes(1000, 2) == 256 + 2 * 1008 * 12
    assert lib.abm_sir_resident_scratch_bytes(0, 2) == 0
    assert lib.abm_sir_resident_scratch_bytes(1000, 0) == 0
    assert lib.abm_sir_resident_max_agents() >= 0
    assert lib.abm_sir_steps_resident(None, 1, None, 1000, 5, 2, None, None, None, 0, None,
                                      None) == _lib.ABM_ERR_BADARG


def test_normal_build_is_not_range_checked(lib):
    """The normal library reports itself as unchecked and has no bounds detail; the
    range-checked one is a separate file (built on request)."""
    assert lib.abm_checked_build() == 0
    assert lib.abm_bounds_detail() == b""
    assert _lib.CHECKED_LIB_PATH != _lib.LIB_PATH


def test_checked_library_is_chosen_by_the_environment(monkeypatch):
    monkeypatch.setenv("JAXABM_CHECKED", "1")
    assert _lib.default_path() == _lib.CHECKED_LIB_PATH
    monkeypatch.setenv("JAXABM_CHECKED", "0")
    assert _lib.default_path() == _lib.LIB_PATH
