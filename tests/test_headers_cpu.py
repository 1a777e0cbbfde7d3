"""Compile checks of the public C header and of the LAMMPS pair style (CPU).

* include/mlipg.h must compile on its own as C99 and as C++17 with every
  warning an error: it is what a C, C++ or FFI binding of the library
  includes.
* lammps/pair_mlip_gtinv_gpu.cpp is syntax-checked against minimal stand-ins
  for the LAMMPS declarations it uses (tests/lammps_stub; LAMMPS itself is not
  part of this repository), with the header's style-registration block too.
* the C example of the integration notes (tests/c_api_example.c) compiles,
  links against the library and runs: a GPU evaluation or MLIPG_ENOGPU.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")
HEADER = os.path.join(INCLUDE, "mlipg.h")
STYLE_DIR = os.path.join(REPO, "lammps-mlip-package_gb300", "lammps")
STUBS = os.path.join(REPO, "tests", "lammps_stub")
WARN = ["-Wall", "-Wextra", "-Werror"]


def run(cmd, stdin=None):
    p = subprocess.run(cmd, input=stdin, capture_output=True, text=True)
    assert p.returncode == 0, " ".join(cmd) + "\n" + p.stderr


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_compiles_as_c99():
    run(["gcc", "-std=c99", "-pedantic", "-fsyntax-only", *WARN, "-x", "c", HEADER])


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_header_compiles_as_cxx17():
    run(["g++", "-std=c++17", "-pedantic", "-fsyntax-only", *WARN, "-x", "c++", HEADER])


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_lammps_pair_style_compiles():
    run(["g++", "-std=c++17", "-fsyntax-only", *WARN, "-I", STUBS, "-I", INCLUDE,
         os.path.join(STYLE_DIR, "pair_mlip_gtinv_gpu.cpp")])
    # the registration block LAMMPS's style_pair.h includes
    # (both styles, mlip_gtinv/gpu and mlip_pair/gpu, map to the one class)
    src = ('#define PAIR_CLASS\n'
           '#define CAT2(a, b) a##b\n'
           '#define CAT(a, b) CAT2(a, b)\n'
           '#define PairStyle(key, Class) static const char *CAT(style_key, __LINE__) = #key;\n'
           '#include "pair_mlip_gtinv_gpu.h"\n')
    run(["g++", "-std=c++17", "-fsyntax-only", *WARN, "-I", STUBS, "-I", INCLUDE, "-I",
         STYLE_DIR, "-x", "c++", "-"], stdin=src)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_example_links_and_runs(potdir, tmp_path):
    import mlipg   # builds the library if needed
    lib = mlipg.lib()._name
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "c_api_example")
    run(["gcc", "-std=c99", *WARN, "-I", INCLUDE, os.path.join(REPO, "tests", "c_api_example.c"),
         "-o", exe, "-L", libdir, "-lmlipg", "-Wl,-rpath," + libdir])
    p = subprocess.run([exe, potdir["gtinv-820"]], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "elements 2" in p.stdout
