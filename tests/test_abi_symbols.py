"""The C-ABI library loads on a machine without a GPU and exports every
function include/grasp_gpu.h declares, the angular-coefficient library
every function include/grasp_angular.h declares; the synthetic-input library
(inputs/) exports what inputs/grasp_synth.h declares. No compute calls here."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:gg|gs|ga)_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


@pytest.fixture(scope="module")
def libs():
    from grasp_gb300 import build
    from inputs import build as ibuild
    return build.build(), ibuild.build()


def test_gpu_header_symbols_exported(libs):
    names = declared("include/grasp_gpu.h")
    assert len(names) >= 30
    syms = exported(libs[0])
    missing = [n for n in names if n not in syms]
    assert not missing, missing


def test_synth_header_symbols_exported(libs):
    names = declared("inputs/grasp_synth.h")
    syms = exported(libs[1])
    assert not [n for n in names if n not in syms]


def test_angular_header_symbols_exported(libs):
    from grasp_gb300 import angular, build
    names = declared("include/grasp_angular.h")
    assert len(names) >= 6
    syms = exported(build.LIB_ANGULAR)
    assert not [n for n in names if n not in syms]
    assert set(names) <= set(angular.SYMBOLS)


def test_gpu_library_loads_and_reports_errors(libs):
    lib = ctypes.CDLL(libs[0])
    lib.gg_version.restype = ctypes.c_int
    assert lib.gg_version() == 1
    lib.gg_last_error.restype = ctypes.c_char_p
    # argument checks run before any device call
    h = ctypes.c_void_p()
    assert lib.gg_ctx_create(-1, ctypes.byref(h)) != 0
    assert lib.gg_last_error()


def test_python_bindings_cover_header(libs):
    from grasp_gb300 import _lib
    assert set(declared("include/grasp_gpu.h")) <= set(_lib.GPU_SYMBOLS)
    from inputs import synth
    assert set(declared("inputs/grasp_synth.h")) <= set(synth.SYNTH_SYMBOLS)


@pytest.mark.parametrize("header", ["include/grasp_gpu.h", "include/grasp_angular.h", "inputs/grasp_synth.h"])
@pytest.mark.parametrize("lang", [["gcc", "-x", "c", "-std=c99"], ["g++", "-x", "c++", "-std=c++17"]])
def test_header_compiles_alone(header, lang, tmp_path):
    """Each public header compiles on its own, as C and as C++, and its
    declarations are not hidden in a comment (the symbol list above is taken
    with comments removed, so an unclosed comment would hide names from it)."""
    src = tmp_path / "h.c"
    src.write_text('#include "%s"\nint main(void) { return 0; }\n' % os.path.join(ROOT, header))
    r = subprocess.run(lang + ["-Wall", "-Wextra", "-Werror", "-fsyntax-only", str(src)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    text = open(os.path.join(ROOT, header)).read()
    assert text.count("/*") == text.count("*/"), "unbalanced comment markers"
