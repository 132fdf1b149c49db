"""CPU-side checks of the C ABI: the library builds, loads and exports every
entry point that include/puffgpu.h declares; parameter validation works
without a device."""
import ctypes
import os
import re

import pytest

import puffin_gb300 as P
from puffin_gb300 import lib as L

HDR = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "puffgpu.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pf_[a-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(L.SYMBOLS)


def test_library_exports_every_symbol():
    lib = L.load(build_if_missing=True)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_params_struct_matches_header():
    src = open(HDR).read()
    body = src[src.index("typedef struct pf_params"):src.index("} pf_params;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for m in re.finditer(r"\b(double|int32_t)\s+([^;]+);", body):
        for f in m.group(2).split(","):
            fields.append((m.group(1), f.strip()))
    got = [(("double" if t is ctypes.c_double else "int32_t"), n) for n, t in L.Params._fields_]
    assert got == fields


def test_defaults_follow_reference():
    p = P.default_params()
    assert (p.nbx, p.nby, p.nbz2) == (16, 16, 37)
    assert p.sfilt_frac == float(__import__("numpy").float32(0.3))
    assert p.redist_every == 60 and p.qfilter == 1 and p.sbeta == 1.0


def test_create_rejects_bad_params_without_touching_a_device():
    lib = L.load()
    p = P.default_params(eta=0.0)
    h = ctypes.c_void_p()
    assert lib.pf_create(ctypes.byref(p), ctypes.byref(h)) == L.PF_BAD_ARG
    assert b"invalid" in lib.pf_last_error(None)
    p = P.default_params(eta=1e-4, nx=3, ny=3, one_d=1)
    assert lib.pf_create(ctypes.byref(p), ctypes.byref(h)) == L.PF_BAD_ARG


def test_no_device_is_reported_not_faked():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(P.PuffinError) as e:
        P.Puffin(P.default_params(eta=1e-4))
    assert e.value.code == L.PF_NO_DEVICE
