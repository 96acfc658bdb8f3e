"""The reference's Fortran/C energy interface (libcharmmene_gpu.so, src/FORTRAN_interface.cpp) on
the device, fed the reference's own inputs written as MDBAS files: get_energy_ (kcal/mol) equals
the reference's FField_MDBAS energies within 1e-10 relative, as the plain FP64 path must."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, mdbas, native

pytestmark = pytest.mark.gpu
KCAL = 418.4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _run(prog):
    # the shim holds one system per process (file-scope state, as the reference): one process per case
    r = subprocess.run([sys.executable, "-c", prog], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


PRELUDE = """
import ctypes as C, json, numpy as np
L = C.CDLL(%(lib)r)
d = C.c_double
L.set_pbc_(%(pbc)r, C.byref(d(%(a)r)), C.byref(d(%(b)r)), C.byref(d(%(c)r)), C.byref(d(90)), C.byref(d(90)), C.byref(d(90)))
L.set_ens_(C.byref(C.c_int(%(n)d)), C.byref(d(%(t)r)))
L.set_ff_and_cor_(%(mode)r, C.byref(d(%(rc)r)), C.byref(d(%(ron)r)), C.byref(d(%(skin)r)), %(ff)r, %(cor)r)
e = np.zeros(10)
L.get_energy_(e.ctypes.data_as(C.POINTER(C.c_double)))
"""


def _prelude(s, mode, tmp_path):
    cor, ff = str(tmp_path / "s.cor"), str(tmp_path / "s.dat")
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    a, b, c = s.box
    return PRELUDE % dict(lib=os.path.join(native.HERE, "_lib", "libcharmmene_gpu.so"),
                          pbc=s.pbc_type.encode(), a=a, b=b, c=c, n=s.natom, t=s.temp, mode=mode.encode(),
                          rc=s.cutoff, ron=s.cuton, skin=s.dcut, ff=ff.encode(), cor=cor.encode())


@pytest.mark.parametrize("name,mode", [(n, m) for n in goldens.REFERENCE_INPUTS for m in ("full", "switch")])
def test_get_energy_matches_reference(name, mode, tmp_path):
    s = goldens.system(name, mode)
    out = _run(_prelude(s, mode, tmp_path) + "print(json.dumps(e.tolist()))")
    e = np.array(__import__("json").loads(out.strip().splitlines()[-1])) * KCAL
    want = np.array(goldens.record(name, mode)["ener"])
    scale = max(1.0, float(np.max(np.abs(want))))
    assert np.all(np.abs(e - want) <= 1e-10 * scale), (e, want)


def test_set_coords_and_masses(tmp_path):
    s = goldens.system("nma_solvated", "switch")
    rng = np.random.default_rng(3)
    xyz = s.coords() + rng.uniform(-0.05, 0.05, (s.natom, 3))
    np.save(tmp_path / "xyz.npy", xyz)
    prog = _prelude(s, "switch", tmp_path) + (
        "xyz = np.load(%r)\n"
        "x, y, z = (np.ascontiguousarray(xyz[:, k]) for k in range(3))\n"
        "P = C.POINTER(C.c_double)\n"
        "L.set_coords_(x.ctypes.data_as(P), y.ctypes.data_as(P), z.ctypes.data_as(P))\n"
        "e2 = np.zeros(10); L.get_energy_(e2.ctypes.data_as(P))\n"
        "m = np.zeros(%d); L.get_mass_(m.ctypes.data_as(P)); L.clean_()\n"
        "print(json.dumps([e.tolist(), e2.tolist(), m.tolist()]))\n" % (str(tmp_path / "xyz.npy"), s.natom))
    e, e2, m = __import__("json").loads(_run(prog).strip().splitlines()[-1])
    assert np.array_equal(np.array(m), s.mass)
    # the Verlet list stays the one built by set_ff_and_cor_, as in the reference: the same
    # energy as the C ABI engine with the list built at the original coordinates
    from mc_cpp_gb300.engine import FFieldCUDA
    ff = FFieldCUDA(s, "fp64", moves=False)
    ff.setCoords(xyz)
    want = ff.getE10() / KCAL
    assert np.allclose(np.array(e2), want, rtol=1e-12, atol=1e-9), (e2, want)
    assert not np.allclose(e2, e)
