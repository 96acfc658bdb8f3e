"""The allocation-free energy entry point against the regular one, through the C ABI.

mcg_energy_switch_fp64_noalloc serves callers that cannot allocate device memory at the moment
they need an energy (a host code whose pool owns the whole GPU, or a loop that cannot afford
cudaMalloc's implicit synchronisation); its scratch is a fixed static device array.  Here the test
itself owns the device buffers (allocated with torch), calls the entry point twice in a row and
checks both results against mcg_energy on the same system: FP64, within 1e-12 relative (the two
paths sum the same pairs in a different order).  Systems without 1-4 pairs, so the main-list
energy is the whole nonbonded energy.  This file sorts last so a failure here leaves every other
test already run.
"""
import ctypes as C

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, native
from mc_cpp_gb300.engine import FFieldCUDA

pytestmark = pytest.mark.gpu
REL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


@pytest.mark.parametrize("name", ["water512", "argon864"])
def test_noalloc_energy_matches_regular_entry_point(name):
    torch = pytest.importorskip("torch")
    s = goldens.system(name, "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    want = ff.getE10()
    assert len(ff.pairs14()) == 0
    rows = ff.pairlist()
    n = s.natom
    cap = max(1, max(len(r) for r in rows))
    nbr = np.zeros((n, cap), np.int32)
    nup = np.zeros(n, np.int32)
    for i, r in enumerate(rows):
        nbr[i, :len(r)] = r
        nup[i] = len(r)
    pq = np.stack([s.x, s.y, s.z, s.q], 1)
    es = np.stack([np.sqrt(s.eps * 418.4), s.sig], 1)
    dev = torch.device("cuda:0")
    d_pq = torch.from_numpy(pq).to(dev).contiguous()
    d_es = torch.from_numpy(es).to(dev).contiguous()
    d_nbr = torch.from_numpy(nbr).to(dev).contiguous()
    d_nup = torch.from_numpy(nup).to(dev).contiguous()
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    box = (C.c_double * 3)(*[float(v) for v in s.box])
    L = native.lib()
    results = []
    for _ in range(2):
        out.zero_()
        rc = L.mcg_energy_switch_fp64_noalloc(n, d_pq.data_ptr(), d_es.data_ptr(), d_nbr.data_ptr(), d_nup.data_ptr(),
                                              cap, native.PBC[s.pbc_type], box, s.cutoff, s.cuton, out.data_ptr(), None)
        native.check(rc)
        torch.cuda.synchronize()
        results.append(out.cpu().numpy().copy())
    for got in results:
        assert abs(got[0] - want[3]) <= REL * abs(want[3]) + 1e-9, (got, want[3:5])
        assert abs(got[1] - want[4]) <= REL * abs(want[4]) + 1e-9, (got, want[3:5])
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_oversized_systems():
    L = native.lib()
    box = (C.c_double * 3)(30.0, 30.0, 30.0)
    rc = L.mcg_energy_switch_fp64_noalloc(300000, 256, 256, 256, 256, 8, 1, box, 12.0, 10.0, 256, None)
    assert rc == native.MCG_EINVAL
    assert b"natom must be in" in L.mcg_last_error()
