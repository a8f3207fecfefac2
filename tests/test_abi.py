"""CPU checks of the C ABI: the library builds, loads and exports exactly the
entry points include/od_gb300.h declares (no compute calls without a GPU)."""
import os
import re
import subprocess

from opendeformer_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "od_gb300.h")


def declared():
    hdr = open(HEADER).read()
    return set(re.findall(r"^(?:od_status|const char\*|int)\s+(od_[a-z_0-9]+)\s*\(", hdr, re.M))


def test_header_declares_the_bound_surface():
    assert declared() == set(api.SIGNATURES)


def test_library_exports_every_declared_symbol():
    lib = api.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", api.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (od_[a-z_0-9]+)\b", out))
    assert declared() <= exported
    for name in declared():
        assert getattr(lib, name) is not None
    with open(HEADER) as f:
        version = int(re.search(r"#define OD_ABI_VERSION (\d+)", f.read()).group(1))
    assert lib.od_abi_version() == version
    assert lib.od_status_string(4) == b"OD_ERR_NAN"


def test_header_compiles_as_c():
    src = os.path.join(ROOT, "include", "od_gb300.h")
    r = subprocess.run(["gcc", "-x", "c", "-std=c99", "-fsyntax-only", "-Wall", "-Werror", src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
