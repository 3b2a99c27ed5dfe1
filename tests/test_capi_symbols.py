"""The C ABI library loads and exports every symbol include/tpl_gb300.h declares.
Host-only calls (no kernel launch) are exercised without a GPU."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def capi(built):
    from torchproteinlibrary_gb300 import capi
    return capi


def test_exports_every_declared_symbol(capi):
    lib = capi.lib()
    names = capi.declared_symbols()
    assert "tpl_a2b_forward_f32" in names and "tpl_a2b_backward_f32" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(capi):
    lib = capi.lib()
    assert lib.tpl_status_string(0) == b"ok"
    for code in range(-8, 0):
        assert lib.tpl_status_string(code) != b"unknown status"
    assert lib.tpl_version() >= 100


def test_workspace_sizes(capi):
    lib = capi.lib()
    small = lib.tpl_a2b_workspace_bytes(4, 100, None)
    big = lib.tpl_a2b_workspace_bytes(4096, 1000, None)
    assert 64 < small < big
    assert lib.tpl_a2b_workspace_bytes(-1, 10, None) == 0
    # far below the reference's A ([B, 48L] floats) + dr_dangle ([B, 3, 27 L^2] floats)
    assert big < 4096 * 48 * 1000 * 4 / 10


def test_argument_errors_without_launch(capi):
    lib = capi.lib()
    # negative sizes and null buffers are rejected before anything is enqueued
    assert lib.tpl_a2b_forward_f32(None, None, None, None, 0, -1, 10, None, None) == -1
    assert lib.tpl_a2b_forward_f32(None, None, None, None, 0, 4, 10, None, None) == -1
    dummy = ctypes.c_void_p(16)
    assert lib.tpl_a2b_forward_f32(dummy, dummy, dummy, None, 0, 4, 10, None, None) == -2  # no workspace
    bad = capi.options(residues_per_thread=3)
    assert lib.tpl_a2b_forward_f32(dummy, dummy, dummy, dummy, 1 << 20, 4, 10, ctypes.byref(bad), None) == -1
    # empty batches are a no-op
    assert lib.tpl_a2b_forward_f32(None, None, None, None, 0, 0, 10, None, None) == 0
