"""include/tupan_gb300.h is the drop-in boundary for C, C++ and FFI
callers (cgo, ctypes, cffi): it must compile on its own as C99 and C++11,
and a C program that includes it must link against the library's exports."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tupan_gb300.h")


@pytest.mark.parametrize("cc,std,lang", [("gcc", "c99", "c"),
                                         ("g++", "c++11", "c++")])
def test_header_compiles_alone(cc, std, lang):
    if shutil.which(cc) is None:
        pytest.skip(cc + " not installed")
    subprocess.check_call([cc, "-std=" + std, "-Wall", "-Werror",
                           "-fsyntax-only", "-x", lang, HEADER])


def test_c_program_links_against_the_library(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not installed")
    from tupan_gb300 import lib
    so = lib.library_path("float64")
    if not os.path.exists(so):
        pytest.skip("library not built")
    src = tmp_path / "use.c"
    src.write_text(
        '#include "tupan_gb300.h"\n'
        "int main(void) {\n"
        "    /* referenced, not called: no GPU is needed to link */\n"
        "    void (*f[])(void) = {(void (*)(void))acc_kernel,\n"
        "                         (void (*)(void))acc_jerk_kernel,\n"
        "                         (void (*)(void))sakura_kernel,\n"
        "                         (void (*)(void))tupan_gb300_last_error};\n"
        "    return f[0] == 0;\n"
        "}\n")
    exe = tmp_path / "use"
    subprocess.check_call(["gcc", "-std=c99", "-I",
                           os.path.join(ROOT, "include"), str(src), "-o",
                           str(exe), so])
