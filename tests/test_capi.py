"""CPU tests of the C ABI: the library builds, loads and exports every symbol
declared in include/vfem.h; host-only helpers work without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT
from vulkanfem_gb300 import api, domains


def declared_symbols():
    out = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        out |= set(re.findall(r"\b(vfem_[a-z0-9_]+)\s*\(", text))
    return out


def test_library_exports_every_declared_symbol():
    lib = api.load_library()
    syms = declared_symbols()
    assert len(syms) >= 18
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert syms <= set(api.EXPORTED)


def test_host_helpers_without_gpu():
    lib = api.load_library()
    ke = api.hex8_stiffness(1.0, 0.3)
    assert np.abs(ke - domains.hex8_stiffness(1.0, 0.3)).max() < 1e-15
    o = api.make_options()
    assert o.rtol == 1e-6 and o.omega == 0.6 and o.replace_every == 0 and o.check_every == 8
    assert o.replace_delta == 0.05
    oc = api.Options()
    lib.vfem_options_default(ctypes.byref(oc))  # the C defaults are the Python ones
    for name, _ in api.Options._fields_:
        if name != "reserved":
            assert getattr(oc, name) == getattr(o, name) or name == "precision", name
    assert lib.vfem_status_string(0) == b"ok"
    assert lib.vfem_status_string(4) == b"not converged"
    bad = np.zeros(576)
    assert lib.vfem_hex8_stiffness(1.0, 0.5, bad) == 1  # nu = 0.5 is invalid


def test_cpp_shim_compiles_and_links(tmp_path):
    """include/vfem.hpp (reference names over the C ABI) builds a reference-style caller."""
    import subprocess
    from vulkanfem_gb300 import build as vbuild
    lib = api.load_library() and vbuild.LIB
    exe = tmp_path / "shim_example"
    cmd = ["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "shim_example.cpp"),
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()


def test_create_reports_errors_instead_of_aborting():
    """Invalid input returns a status code (the reference asserts or misbehaves)."""
    lib = api.load_library()
    vox = np.ones((2, 2, 2), np.uint8)
    ke = np.ascontiguousarray(domains.hex8_stiffness().reshape(-1))
    h = ctypes.c_void_p()
    fixed = np.array([0], np.int64)
    s = lib.vfem_problem_create(vox.reshape(-1), 2, 2, 2, ke, None, fixed, 1, 0, 0, ctypes.byref(h))
    assert s != 0 and not h.value


def test_create_rejects_an_empty_fixed_set():
    """Without fixed nodes the stiffness is singular (rigid-body modes): the
    set-up refuses with VFEM_ERR_INVALID_ARGUMENT before touching the device."""
    lib = api.load_library()
    vox = np.ones((2, 2, 2), np.uint8)
    ke = np.ascontiguousarray(domains.hex8_stiffness().reshape(-1))
    h = ctypes.c_void_p()
    fixed = np.zeros(1, np.int64)
    s = lib.vfem_problem_create(vox.reshape(-1), 2, 2, 2, ke, None, fixed, 0, 2, 0, ctypes.byref(h))
    assert s == 1 and not h.value
    assert b"fixed" in lib.vfem_last_error_message()
