"""CPU checks of the C ABI library: it loads, exports every declared symbol,
and its host-side argument checks work without touching a GPU."""
import ctypes
import os
import re

import pytest

from aloha_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(aloha_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = abi.lib()
    declared = _declared()
    assert declared, "no declarations found in include/*.h"
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert declared == set(abi.EXPORTS)


def test_abi_version_and_status_strings():
    L = abi.lib()
    assert L.aloha_abi_version() == 1
    assert L.aloha_status_string(0) == b"ok"
    assert L.aloha_status_string(8) == b"missing brick"
    assert L.aloha_status_string(12345) == b"unknown status"


def test_default_params_match_the_configured_workloads():
    p = abi.RenderParams()
    assert abi.lib().aloha_default_render_params(ctypes.byref(p)) == 0
    assert p.dt == 0.5 and abs(p.et_alpha - 0.99) < 1e-7 and p.spp == 1
    assert p.num_islands == 1 and p.composite_mode == abi.COMPOSITE_FP32


def test_null_arguments_are_rejected_without_a_gpu():
    L = abi.lib()
    assert L.aloha_create(0, None) == abi.ERR_NULL_POINTER
    assert L.aloha_destroy(None) == abi.ERR_NULL_POINTER
    assert L.aloha_default_render_params(None) == abi.ERR_NULL_POINTER
    assert L.aloha_render(None, 0, None, None) == abi.ERR_NULL_POINTER
    assert L.aloha_composite_over(None, None, 1, 1, 1, 0, None, None) == abi.ERR_NULL_POINTER


def test_create_reports_an_error_instead_of_crashing_when_no_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = abi.lib().aloha_create(0, ctypes.byref(h))
    assert rc in (abi.ERR_CUDA, abi.ERR_OUT_OF_RANGE)
    assert not h.value


def test_brick_desc_is_the_vol_header_layout():
    assert ctypes.sizeof(abi.BrickDesc) == 80
    assert ctypes.sizeof(abi.RenderParams) == 14 * 4
