"""CPU-side checks of the C ABI library and the host logic (no device compute)."""
import ctypes as C
import os
import subprocess
import sys
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
    h = C.c_void_p()
    # an invalid description is rejected on the host, with or without a device
    d, keep = native.make_desc(systems.argon_fcc(2))          # 11.45 A box: cutoff beyond half the box
    assert L.mcg_create(C.byref(d), C.byref(h)) == native.MCG_EINVAL
    assert b"half the box" in L.mcg_last_error()
    if L.mcg_device_count() == 0:
        d, keep = native.make_desc(systems.argon_fcc(6))
        rc = L.mcg_create(C.byref(d), C.byref(h))
        assert rc == native.MCG_ECUDA
        assert b"no CUDA device" in L.mcg_last_error()


def test_null_handles_rejected_on_host():
    """Handle-taking entry points check their arguments before any device work."""
    L = native.lib()
    i64, f32 = C.c_int64(0), C.c_float(0)
    assert L.mcg_set_prune_buffer(None, 0.5) == native.MCG_EINVAL
    assert L.mcg_prune_stats(None, C.byref(i64), C.byref(i64), C.byref(f32)) == native.MCG_EINVAL
    assert L.mcg_set_pair_kernel(None, 0) == native.MCG_EINVAL
    assert L.mcg_time_nonbonded_flushed(None, 1, C.byref(f32)) == native.MCG_EINVAL
    assert L.mcg_kernel_launches(None, C.byref(i64)) == native.MCG_EINVAL
    assert L.mcg_cluster_stats(None, C.byref(i64), C.byref(i64), C.byref(i64)) == native.MCG_EINVAL
    assert L.mcg_group_stats(None, C.byref(i64), C.byref(i64), C.byref(i64)) == native.MCG_EINVAL
    d = C.c_double(0)
    x = (C.c_double * 4)()
    assert L.mcg_energy_host(None, x, x, x, C.byref(d)) == native.MCG_EINVAL
    assert L.mcg_batch_save(None, b"/tmp/x.ckpt") == native.MCG_EINVAL
    assert L.mcg_batch_load(None, b"/tmp/x.ckpt") == native.MCG_EINVAL
    assert L.mcg_batch_sweep_logged(None, None, 0) == native.MCG_EINVAL
    assert b"null" in L.mcg_last_error()


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


def _shim():
    path = os.path.join(native.HERE, "_lib", "libcharmmene_gpu.so")
    assert os.path.exists(path), path
    return path


def test_fortran_shim_exports_the_reference_symbols():
    out = subprocess.check_output(["nm", "-D", "--defined-only", _shim()]).decode()
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    hdr = open(os.path.join(os.path.dirname(native.HERE), "include", "charmmene_gpu.h")).read()
    import re
    declared = set(re.findall(r"\bvoid\s+([a-z_]+_)\s*\(", hdr))
    # the seven entry points of src/FORTRAN_interface.cpp:23-106
    assert declared == {"set_pbc_", "set_ens_", "set_ff_and_cor_", "get_energy_", "set_coords_", "get_mass_", "clean_"}
    assert declared <= exported, declared - exported


@pytest.mark.parametrize("name", ["peptide", "nma_solvated"])
def test_mdbas_reader_matches_python_reader(name, tmp_path):
    """mcg_mdbas_read (the library's IO_MDBAS restatement) against mdbas.read_cor/read_forfield."""
    s = goldens.system(name, "switch")
    cor, ff = str(tmp_path / "s.cor"), str(tmp_path / "s.dat")
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    c = mdbas.read_cor(cor)
    f = mdbas.read_forfield(ff, c["natom"])
    L = native.lib()
    h = C.c_void_p()
    native.check(L.mcg_mdbas_read(cor.encode(), ff.encode(), C.byref(h)))
    try:
        d = native.SystemDesc()
        native.check(L.mcg_mdbas_fill(h, C.byref(d)))
        n = d.natom
        assert n == c["natom"] == s.natom and d.param_units == 0

        def arr(p, m, dt=np.float64):
            return np.ctypeslib.as_array(p, shape=(m,)).astype(dt) if m else np.zeros(0, dt)
        for k in ("x", "y", "z"):
            assert np.array_equal(arr(getattr(d, k), n), c[k])
        for k in ("q", "eps", "sig", "eps14", "sig14", "mass"):
            assert np.array_equal(arr(getattr(d, k), n), f[k]), k
        assert np.array_equal(arr(d.resid, n, np.int32), c["resid"])
        assert np.array_equal(np.ctypeslib.as_array(d.frozen, shape=(n,)), f["frozen"])
        nb = d.nbond
        assert nb == len(f.get("bonds", []))
        if nb:
            assert np.array_equal(arr(d.bond_atoms, 2 * nb, np.int32).reshape(-1, 2), f["bonds"])
            assert np.array_equal(arr(d.bond_k, nb), f["bond_k"]) and np.array_equal(arr(d.bond_r0, nb), f["bond_r0"])
        na = d.nangle
        if na:
            assert np.array_equal(arr(d.angle_atoms, 3 * na, np.int32).reshape(-1, 3), f["angles"])
            assert np.array_equal(arr(d.angle_theta0, na), f["angle_theta0"])
        nd = d.ndihe
        if nd:
            assert np.array_equal(arr(d.dihe_atoms, 4 * nd, np.int32).reshape(-1, 4), f["dihedrals"])
            assert np.array_equal(arr(d.dihe_mult, nd), f["dihe_mult"])
        ni = d.nimpr
        if ni:
            assert np.array_equal(arr(d.impr_phi0, ni), f["impr_phi0"])
        # exclusions built from the file-read description equal those from the Python system
        d.pbc_type, d.cut_mode, d.cutoff, d.cuton, d.dcut, d.temp = 1, 1, s.cutoff, s.cuton, s.dcut, s.temp
        d.box[0] = d.box[1] = d.box[2] = s.box[0]
        counts = np.zeros(n, np.int32)
        total, n14 = C.c_int64(0), C.c_int(0)
        native.check(L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)))
        d2, keep = native.make_desc(s)
        counts2 = np.zeros(n, np.int32)
        native.check(L.mcg_build_exclusions(C.byref(d2), native.pi(counts2), None, 0, C.byref(total), None, 0, C.byref(n14)))
        assert np.array_equal(counts, counts2)
    finally:
        L.mcg_mdbas_free(h)


def test_mdbas_reader_rejects_bad_files(tmp_path):
    L = native.lib()
    h = C.c_void_p()
    assert L.mcg_mdbas_read(b"/nonexistent.cor", b"/nonexistent.dat", C.byref(h)) == native.MCG_EIO
    s = goldens.system("peptide", "switch")
    cor, ff = str(tmp_path / "s.cor"), str(tmp_path / "s.dat")
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    txt = open(ff).read().replace("vdw %d" % s.natom, "vdw %d" % (s.natom - 1))
    open(ff, "w").write(txt)
    assert L.mcg_mdbas_read(cor.encode(), ff.encode(), C.byref(h)) == native.MCG_EIO
    assert b"vdw count" in L.mcg_last_error()
    open(ff, "w").write("atoms 3\nbogus 2\n")
    assert L.mcg_mdbas_read(cor.encode(), ff.encode(), C.byref(h)) == native.MCG_EIO


def test_fortran_shim_exits_like_the_reference_without_a_device(tmp_path):
    """No GPU here: set_ff_and_cor_ must print the reason and exit with a negative status, the
    reference's error convention (FField_MDBAS.cpp:68-71), instead of returning garbage."""
    if native.lib().mcg_device_count() > 0:
        pytest.skip("a device is present")
    s = goldens.system("peptide", "switch")
    cor, ff = str(tmp_path / "s.cor"), str(tmp_path / "s.dat")
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    prog = ("import ctypes as C; L = C.CDLL(%r); d = C.c_double; "
            "L.set_pbc_(b'cubic', C.byref(d(%r)), C.byref(d(%r)), C.byref(d(%r)), C.byref(d(90)), C.byref(d(90)), C.byref(d(90))); "
            "L.set_ens_(C.byref(C.c_int(%d)), C.byref(d(300.0))); "
            "L.set_ff_and_cor_(b'switch', C.byref(d(12.0)), C.byref(d(10.0)), C.byref(d(2.0)), %r, %r)"
            % (_shim(), s.box[0], s.box[0], s.box[0], s.natom, ff.encode(), cor.encode()))
    r = subprocess.run([sys.executable, "-c", prog], capture_output=True, text=True)
    assert r.returncode != 0
    assert "no CUDA device" in r.stderr
