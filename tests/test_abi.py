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


def test_python_defaults_equal_the_library_defaults():
    """lib.DEFAULTS (used to describe workloads without loading the CUDA
    library) holds exactly what pf_default_params writes."""
    lib = L.load()
    got = L.Params()
    lib.pf_default_params(ctypes.byref(got))
    want = P.default_params()
    for name, _ in L.Params._fields_:
        assert getattr(got, name) == getattr(want, name), name


def test_describing_a_workload_does_not_load_the_cuda_library():
    import subprocess
    import sys
    code = ("import sys; from puffin_gb300 import configs, lib; "
            "w = configs.config2(np_=4096, nz2=64); "
            "assert lib._lib is None; "
            "maps = open('/proc/self/maps').read(); "
            "sys.exit(1 if 'libpuffgpu' in maps else 0)")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


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
