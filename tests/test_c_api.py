"""The C ABI from a plain C caller (CPU only).

include/mcg.h is the drop-in boundary, so it must compile as C99 with every warning an error and
link against libmcgpu.so alone.  tests/c_api/host_calls.c makes the calls of the integration
notes: the MDBAS reader, the exclusion and 1-4 builder, null-argument rejection, and the device
calls, which without a GPU must fail with MCG_ECUDA and an error text.  The header must also
compile as C++11, the standard mc_cpp itself is built with.  The Fortran/C interface header
(include/charmmene_gpu.h) must compile as C and its seven symbols link from libcharmmene_gpu.so.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from mc_cpp_gb300 import build, mdbas, native, systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib_dir():
    build.build()
    return os.path.dirname(native.LIB_PATH)


def test_header_compiles_as_cxx11(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    src = tmp_path / "h.cpp"
    src.write_text('#include "mcg.h"\nint main() { mcg_system_desc d = {}; return d.natom; }\n')
    r = subprocess.run(["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + INC, str(src),
                        "-o", str(tmp_path / "h")], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_fortran_interface_header_compiles_as_c_and_links(lib_dir, tmp_path):
    """include/charmmene_gpu.h from C: the seven symbols resolve in libcharmmene_gpu.so."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    src = tmp_path / "f.c"
    src.write_text('#include "charmmene_gpu.h"\n'
                   'int main(void) {\n'
                   '    void (*fns[7])(void) = {(void (*)(void))set_pbc_, (void (*)(void))set_ens_,\n'
                   '        (void (*)(void))set_ff_and_cor_, (void (*)(void))get_energy_, (void (*)(void))set_coords_,\n'
                   '        (void (*)(void))get_mass_, (void (*)(void))clean_};\n'
                   '    return fns[0] == 0;\n}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I" + INC, str(src), "-o",
                        str(tmp_path / "f"), "-L" + lib_dir, "-lcharmmene_gpu", "-Wl,-rpath," + lib_dir],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_plain_c_caller(lib_dir, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "host_calls")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + INC,
                        os.path.join(ROOT, "tests", "c_api", "host_calls.c"), "-o", exe, "-L" + lib_dir, "-lmcgpu",
                        "-Wl,-rpath," + lib_dir], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    s = systems.peptide_in_water(40, 500, L=24.6, seed=4)
    cor, ff = str(tmp_path / "sys.cor"), str(tmp_path / "sys.ff")
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    r = subprocess.run([exe, cor, ff], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = dict(ln.split(None, 1) for ln in r.stdout.splitlines())
    L = native.lib()
    assert int(got["abi"]) == L.mcg_abi_version()
    assert int(got["mdbas_read"]) == native.MCG_OK and int(got["natom"]) == s.natom
    # the same exclusion and 1-4 counts as the library called from Python on the same files
    xml = str(tmp_path / "sys.xml")
    mdbas.write_xml(s, xml, "sys.cor", "sys.ff")
    s2 = mdbas.read_xml(xml)
    d, keep = native.make_desc(s2)
    counts = np.zeros(s2.natom, np.int32)
    total, n14 = C.c_int64(0), C.c_int(0)
    native.check(L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)))
    assert int(got["build_exclusions"]) == native.MCG_OK
    assert int(got["excl_total"]) == total.value and int(got["pairs14"]) == n14.value
    assert int(got["null_create"]) == native.MCG_EINVAL and got["null_create_error"] == "set"
    assert int(got["null_energy"]) == native.MCG_EINVAL
    if int(got["devices"]) == 0:
        assert int(got["create"]) == native.MCG_ECUDA and got["create_error"] == "set"
        assert int(got["batch_create"]) == native.MCG_ECUDA
    else:
        assert int(got["create"]) == native.MCG_OK and int(got["energy"]) == native.MCG_OK
    assert int(got["mdbas_free"]) == native.MCG_OK
