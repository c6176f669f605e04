"""The drop-in at the C level: the reference's own test program (run_tests.cc)
compiles and links, unchanged, against include/ftcrypto.h and libftcrypto.so.
Needs the reference sources (FT_REF_SRC, as oracle/build_ref.sh); skipped
where they are absent.  Running it needs a GPU and the reference sources
together, which no machine here has; its assertions are restated as GPU
tests (test_gpu_parity.py: test_run_tests_cases)."""
import os
import subprocess

import pytest

import libftcrypto_gb300 as lib
import oracle

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), os.pardir))
PROGRAM = os.path.join(oracle.ref_src(), "run_tests.cc")


@pytest.mark.skipif(not os.path.isfile(PROGRAM), reason="reference sources absent")
def test_reference_test_program_builds_against_this_library(tmp_path):
    lib.build()
    libdir = os.path.dirname(lib.LIB_PATH)
    exe = tmp_path / "run_tests"
    subprocess.run(["g++", "-std=c++17", "-o", str(exe), PROGRAM, "-I", os.path.join(ROOT, "include"),
                    "-L", libdir, "-lftcrypto", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True)
    assert exe.exists()
    # every ft_* symbol the program calls resolves in libftcrypto.so
    out = subprocess.run(["nm", "-u", str(exe)], check=True, capture_output=True, text=True).stdout
    used = {ln.split()[-1] for ln in out.splitlines() if ln.split() and ln.split()[-1].startswith("ft_")}
    assert used, "the program calls the library"
    defined = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], check=True, capture_output=True,
                             text=True).stdout
    exported = {ln.split()[-1] for ln in defined.splitlines() if " T " in ln}
    assert used <= exported, used - exported
