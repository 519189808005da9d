"""CPU tests of the C ABI: the library loads, exports every symbol the headers
declare, and its host-side logic (status codes, argument checks, the type
switch) behaves; with no GPU, device calls fail loudly instead of falling
back."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import sdg
from helpers import ROOT, operators


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(sdg_\w+)\s*\(", text)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 30
    lib = ctypes.CDLL(sdg.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "sdg_advect.h"\nint main(void){return SDG_OK;}\n')
    r = os.system(f"gcc -std=c99 -Wall -Werror -fsyntax-only -I{ROOT}/include {src}")
    assert r == 0


def test_binding_struct_layouts_match_the_library():
    lib = ctypes.CDLL(sdg.LIB_PATH)
    lib.sdg_struct_size.argtypes = [ctypes.c_char_p]
    lib.sdg_struct_size.restype = ctypes.c_size_t
    for name, cls in (("sdg_server_config", sdg.ServerConfig), ("sdg_request", sdg.Request),
                      ("sdg_result", sdg.Result), ("sdg_server_stats", sdg.ServerStats)):
        assert lib.sdg_struct_size(name.encode()) == ctypes.sizeof(cls), name
    assert lib.sdg_struct_size(b"no_such_struct") == 0


def test_status_strings():
    assert sdg.status_string(sdg.OK) == "ok"
    for st in range(-9, 0):
        assert sdg.status_string(st) not in ("", "unknown status")
    assert sdg.status_string(-1234) == "unknown status"


def test_dg_optr_kernel_setup_accepts_reference_strings():
    sdg.dg_optr_kernel_setup("GENERAL")
    assert sdg.dg_optr_kernel_type() == sdg.OPT_GENERAL
    sdg.dg_optr_kernel_setup("OPT1    ")  # trailing blanks as character(len=8)
    assert sdg.dg_optr_kernel_type() == sdg.OPT_OPT1
    with pytest.raises(sdg.SdgError) as e:
        sdg.dg_optr_kernel_setup("OPT2")
    assert e.value.status == sdg.ERR_BAD_OPTTYPE
    assert sdg.dg_optr_kernel_type() == sdg.OPT_OPT1  # unchanged by the failure
    sdg.dg_optr_kernel_setup("EVENODD ")  # the even-odd extension
    assert sdg.dg_optr_kernel_type() == sdg.OPT_EVENODD
    sdg.dg_optr_kernel_setup("OPT1")


def test_operator_generate_rejects_bad_order():
    for p in (0, 16, -1):
        with pytest.raises(sdg.SdgError) as e:
            sdg.operator_generate(p)
        assert e.value.status == sdg.ERR_UNSUPPORTED_ORDER


def test_argument_checks_come_before_any_device_work():
    x, D, Dt, L = operators(2)
    Nq, Np, NfpTot, Ne, NeA = 3, 27, 54, 2, 2
    z = np.zeros(Np * NeA)
    vm = np.ones(NfpTot * Ne, dtype=np.int32)
    sdg.dg_optr_kernel_setup("OPT1")
    with pytest.raises(sdg.SdgError) as e:  # Np inconsistent with Nq
        sdg.advect3d_eq_cal_tend(z.copy(), z, z, z, z, D, Dt, L, vm, vm, np.zeros(3 * NfpTot * Ne),
                                 np.zeros(3 * Np * Ne), np.zeros(NfpTot * Ne), Nq, 26, NfpTot,
                                 Ne, NeA)
    assert e.value.status == sdg.ERR_INVALID_ARG
    with pytest.raises(sdg.SdgError) as e:  # order 16
        sdg.tensorprod_divlike_dirXYZ(D, Dt, z, z, z, 17)
    assert e.value.status == sdg.ERR_UNSUPPORTED_ORDER
    with pytest.raises(sdg.SdgError) as e:
        sdg.Solver(0, 2, 2, 2, D, L)
    assert e.value.status == sdg.ERR_INVALID_ARG
    with pytest.raises(sdg.SdgError) as e:
        sdg.Solver(2, 2, 2, 2, D, L, opt=7)
    assert e.value.status == sdg.ERR_BAD_OPTTYPE


@pytest.mark.skipif(sdg.device_count() > 0, reason="a GPU is present")
def test_without_a_gpu_the_compute_path_fails_loudly():
    x, D, Dt, L = operators(3)
    with pytest.raises(sdg.SdgError) as e:
        sdg.Solver(2, 2, 2, 3, D, L)
    assert e.value.status == sdg.ERR_NO_DEVICE
    with pytest.raises(sdg.SdgError) as e:
        sdg.tensorprod_Lift_hexahedral(L, np.zeros(6 * 16), 4)
    assert e.value.status == sdg.ERR_NO_DEVICE


def test_operator_variants_reject_bad_arguments():
    """Argument checks run before any device work, so they hold without a GPU."""
    x, D, Dt, L = operators(3)
    with pytest.raises(sdg.SdgError):
        sdg.tensorprod_gradlike_dirXYZ(D, Dt, np.zeros(64), 17)
    assert sdg.lib.sdg_tensorprod_divlike_dirXYZ_var5_dev(None, None, None, None, None, None,
                                                          None, None, 4, 1, None) != 0
    assert sdg.lib.sdg_tensorprod_divlike_dirXYZ_var5_dev(None, None, None, None, None, None,
                                                          None, None, 4, 0, None) == 0
    with pytest.raises(sdg.SdgError):
        sdg.element_matvec_dir(4, D, np.zeros(64), 4)
    assert sdg.lib.sdg_element_matvec_dir_dev(0, None, None, None, 4, 1, None) != 0
