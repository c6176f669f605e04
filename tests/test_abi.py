"""The drop-in boundary without a GPU: libftcrypto.so builds for sm_103a,
loads, exports every function that include/*.h declares (and the 38 of the
reference's ftcrypto.h), and its host-only paths behave like the reference."""
import os
import re
import subprocess

import pytest

import libftcrypto_gb300 as lib
from libftcrypto_gb300 import _lib

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), os.pardir))

REFERENCE_API = """ft_error_str ft_crypto_init ft_crypto_device_memory ft_array_init_scalar
ft_array_init_point ft_array_get_subset ft_array_get_range ft_array_assign_to_subset
ft_array_assign_zero_to_subset ft_array_assign_to_range ft_array_delete_subset ft_array_delete_range
ft_array_to_bytes_folded ft_array_to_bytes_affine ft_array_to_bytes ft_array_from_bytes_folded
ft_array_from_bytes_affine ft_array_from_bytes ft_array_validate ft_array_from_scalars
ft_array_from_small_scalars ft_array_free ft_array_get_length ft_array_set_length ft_array_mux
ft_array_contains ft_add ft_reduce_isum ft_sub ft_scale ft_neg ft_mul ft_index ft_equal ft_not_equal
ft_array_prescan ft_array_scan ft_array_reduce""".split()


def header_functions():
    names = []
    for h in ("ftcrypto.h", "ftcrypto_gb300.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\b(ftx?_\w+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def so():
    lib.build()
    return lib.LIB_PATH


def exported(path):
    out = subprocess.check_output(["nm", "-D", "--defined-only", path]).decode()
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_reference_api_is_38_functions():
    assert len(REFERENCE_API) == 38


def test_exports_every_declared_function(so):
    syms = exported(so)
    declared = header_functions()
    assert set(REFERENCE_API) <= set(declared)
    missing = [n for n in declared if n not in syms]
    assert not missing, missing
    assert set(_lib.SIGNATURES) == set(declared)


def test_loads_and_binds(so):
    L = _lib.load(so)
    for name in _lib.SIGNATURES:
        assert hasattr(L, name)


def test_error_strings(so):
    assert lib.error_str(0) == "no error"
    assert lib.error_str(2) == "parameter sizes did not mmatch"  # the reference's spelling
    assert lib.error_str(10) == "device or driver does not support a required feature"
    assert lib.error_str(11) == lib.error_str(-1) == "bad error value"


def test_constants_match_reference_header():
    txt = open(os.path.join(ROOT, "include", "ftcrypto.h")).read()
    assert re.search(r"#define FT_EXTENDED_POINT_BYTES 160\b", txt)
    assert re.search(r"#define FT_FOLDED_POINT_BYTES 32\b", txt)
    assert re.search(r"#define FT_ED25519_SCALARBYTES 32\b", txt)


def test_init_without_gpu_reports_device_error(so):
    L = _lib.load(so)
    code = L.ft_crypto_init()
    if code == 0:
        pytest.skip("a GPU is present")
    assert code == 10
