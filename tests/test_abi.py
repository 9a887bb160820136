"""The C-ABI library builds for sm_103a, loads, and exports every entry point of include/ptgpu.h.
(No compute calls: this runs on machines without a GPU.)"""
import ctypes

import pytest

from projectracer_gb300 import build as pt_build
from projectracer_gb300.config import PtConfig
from projectracer_gb300.engine import HEADER, header_symbols


@pytest.fixture(scope="module")
def lib():
    path = pt_build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = header_symbols()
    for name in ("pt_init", "pt_finalize", "pt_upload_state", "pt_download_state", "pt_solve_psi", "pt_step",
                 "pt_stats", "pt_tracers_to_corners", "pt_set_guess_mode", "pt_last_error"):
        assert name in syms, name


def test_library_exports_all_declared_symbols(lib):
    for name in header_symbols():
        assert hasattr(lib, name), f"{name} declared in {HEADER} but not exported"


def test_config_struct_layout_matches_header():
    # pt_config: 16 int32, one int64, 24 doubles, 9 int32, 4 bytes of padding, 2 doubles, 4 int32, 2 doubles,
    # one uint64 (LP64)
    tail = 16 * 4 + 8 + 24 * 8 + 9 * 4 + 4 + 2 * 8  # krylov
    assert PtConfig.krylov.offset == tail
    assert PtConfig.dist_factor.offset == tail + 4 * 4
    assert PtConfig.eq_seed.offset == tail + 4 * 4 + 2 * 8
    assert ctypes.sizeof(PtConfig) == tail + 4 * 4 + 3 * 8
    assert PtConfig.damping.offset == 16 * 4 + 8 + 24 * 8 + 9 * 4 + 4
    assert PtConfig.discrete_types.offset == 16 * 4 + 8 + 24 * 8 + 4 * 4
    assert PtConfig.reference_rounding.offset == 16 * 4 + 8 + 24 * 8 + 5 * 4


def test_last_error_without_context(lib):
    lib.pt_last_error.restype = ctypes.c_char_p
    lib.pt_solve_psi.argtypes = [ctypes.c_void_p]
    rc = lib.pt_solve_psi(None)
    assert rc == -7  # PT_ERR_STATE: no context yet
    assert b"pt_init" in lib.pt_last_error()
