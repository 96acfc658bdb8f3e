"""CPU-side checks of the C ABI library and the host logic (no device compute)."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, mdbas, native, systems


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()
    return native.lib()


def test_exports_every_declared_symbol():
    out = subprocess.check_output(["nm", "-D", "--defined-only", native.LIB_PATH]).decode()
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    declared = native.declared_symbols()
    assert declared, "no declarations parsed from include/mcg.h"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing


def test_abi_version_and_errors_without_device():
    L = native.lib()
    assert L.mcg_abi_version() == 1
    if L.mcg_device_count() == 0:
        s = systems.argon_fcc(2)
        d, keep = native.make_desc(s)
        h = C.c_void_p()
        rc = L.mcg_create(C.byref(d), C.byref(h))
        assert rc == native.MCG_ECUDA
        assert b"no CUDA device" in L.mcg_last_error()


def test_host_exclusions_match_reference_rows():
    # the library's host-side List_nonBonded restatement, no device needed
    for name in ("diala_vac", "nma_solvated", "peptide"):
        s = goldens.system(name, "full")
        d, keep = native.make_desc(s)
        L = native.lib()
        counts = np.zeros(s.natom, np.int32)
        total = C.c_int64(0)
        n14 = C.c_int(0)
        native.check(L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)))
        ent = np.zeros(max(1, total.value), np.int32)
        p14 = np.zeros(max(2, 2 * n14.value), np.int32)
        native.check(L.mcg_build_exclusions(C.byref(d), native.pi(counts), native.pi(ent), total.value, C.byref(total),
                                            native.pi(p14), len(p14), C.byref(n14)))
        rows = np.split(ent[:total.value], np.cumsum(counts)[:-1])
        rec = goldens.record(name, "full")
        assert goldens.rows_digest(rows) == rec["excl_digest"]
        if rec["pairs14"] is not None:
            assert p14[:2 * n14.value].reshape(-1, 2).tolist() == rec["pairs14"]


def test_invalid_descriptions_rejected_on_host():
    L = native.lib()
    s = systems.argon_fcc(2)
    d, keep = native.make_desc(s)
    counts = np.zeros(s.natom, np.int32)
    total = C.c_int64(0)
    n14 = C.c_int(0)
    d.natom = 0
    assert L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)) == native.MCG_EINVAL
    d.natom = s.natom
    d.cut_mode = 7
    assert L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)) == native.MCG_EINVAL
    d.cut_mode = 1
    d.cutoff = 40.0   # beyond half the box: minimum image undefined
    assert L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)) == native.MCG_EINVAL
    assert b"half the box" in L.mcg_last_error()
    d.cutoff = 12.0
    bad = np.array(s.x)
    bad[3] = np.nan
    d.x = native.pd(bad)
    assert L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)) == native.MCG_EINVAL


def test_mdbas_roundtrip_and_reader():
    s = systems.peptide_in_water(nwat=50, L=20.0)
    with tempfile.TemporaryDirectory() as d:
        mdbas.write_cor(s, os.path.join(d, "a.cor"))
        mdbas.write_forfield(s, os.path.join(d, "a.ff"))
        mdbas.write_xml(s, os.path.join(d, "a.xml"), "a.cor", "a.ff")
        t = mdbas.read_xml(os.path.join(d, "a.xml"))
    for k in ("x", "y", "z", "q", "eps", "sig", "eps14", "sig14", "bond_k", "angle_theta0", "dihe_phi0", "impr_k"):
        assert np.array_equal(getattr(s, k), getattr(t, k)), k
    assert np.array_equal(s.bonds, t.bonds) and np.array_equal(s.dihedrals, t.dihedrals)
    assert t.moves == s.moves


@pytest.mark.parametrize("name", ["argon864", "water4096", "water512", "peptide"])
def test_synthetic_systems_regenerate_bitwise(name):
    goldens.system(name)  # asserts the coordinate digest recorded with the reference's goldens
