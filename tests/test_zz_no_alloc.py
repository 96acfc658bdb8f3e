"""The allocation-free energy entry point, through the C ABI.

mcg_energy_switch_fp64_noalloc serves callers that cannot allocate device memory at the moment
they need an energy (a host code whose pool owns the whole GPU, or a loop that cannot afford
cudaMalloc's implicit synchronisation); its scratch is a fixed static device array.  Here the test
itself owns the device buffers (allocated with torch) and calls the entry point twice in a row:

* on the cubic water and argon boxes, both results are checked against the reference's own
  (elec, vdw) recorded in the golden fixtures and against mcg_energy;
* on a vacuum (no periodic box) and an orthorhombic water box, against the CPU oracle;
* on a side stream (a torch stream's handle) instead of the default stream;
* with damaged rows (counts above the capacity, partners outside the system): those entries are
  skipped, and the energy equals that of the valid entries.

FP64 everywhere: 1e-12 relative against the library's own energy, 1e-10 against the reference and
the oracle (the paths sum the same pairs in different orders).  Systems without 1-4 pairs, so the
main-list energy is the whole nonbonded energy.  This file sorts last so a failure here leaves
every other test already run.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, native
from mc_cpp_gb300.engine import FFieldCUDA

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as orc  # noqa: E402

pytestmark = pytest.mark.gpu
REL_SELF = 1e-12
REL_REF = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _rows(ff, n):
    rows = ff.pairlist()
    cap = max(1, max(len(r) for r in rows))
    nbr = np.zeros((n, cap), np.int32)
    nup = np.zeros(n, np.int32)
    for i, r in enumerate(rows):
        nbr[i, :len(r)] = r
        nup[i] = len(r)
    return nbr, nup, cap


def _call(torch, s, nbr, nup, cap, stream=None, calls=2):
    dev = torch.device("cuda:0")
    pq = np.stack([s.x, s.y, s.z, s.q], 1)
    es = np.stack([np.sqrt(s.eps * 418.4), s.sig], 1)
    d_pq = torch.from_numpy(pq).to(dev).contiguous()
    d_es = torch.from_numpy(es).to(dev).contiguous()
    d_nbr = torch.from_numpy(nbr).to(dev).contiguous()
    d_nup = torch.from_numpy(nup).to(dev).contiguous()
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    box = (C.c_double * 3)(*[float(v) for v in s.box])
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    L = native.lib()
    results = []
    for _ in range(calls):
        out.fill_(np.nan)
        rc = L.mcg_energy_switch_fp64_noalloc(s.natom, d_pq.data_ptr(), d_es.data_ptr(), d_nbr.data_ptr(),
                                              d_nup.data_ptr(), cap, native.PBC[s.pbc_type], box, s.cutoff, s.cuton,
                                              out.data_ptr(), handle)
        native.check(rc)
        if stream is None:
            torch.cuda.synchronize()
        else:
            stream.synchronize()
        results.append(out.cpu().numpy().copy())
    return results


def _close(got, want, rel):
    return all(abs(g - w) <= rel * abs(w) + 1e-9 for g, w in zip(got, want))


@pytest.mark.parametrize("name", ["water512", "argon864"])
def test_noalloc_energy_matches_reference_goldens(name):
    torch = pytest.importorskip("torch")
    s = goldens.system(name, "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    assert len(ff.pairs14()) == 0
    mine = ff.getE10()[3:5]
    gold = goldens.record(name, "switch")["ener"][3:5]     # the reference's (elec, vdw), iu
    nbr, nup, cap = _rows(ff, s.natom)
    results = _call(torch, s, nbr, nup, cap)
    for got in results:
        assert _close(got, gold, REL_REF), (got, gold)
        assert _close(got, mine, REL_SELF), (got, mine)
    assert np.array_equal(results[0], results[1])


def test_noalloc_vacuum_and_orthorhombic_boxes_match_the_oracle():
    torch = pytest.importorskip("torch")
    base = goldens.system("water512", "switch")
    vac = base.copy()
    vac.pbc_type = "none"
    orb = base.copy()
    orb.pbc_type = "orbic"
    orb.box = (base.box[0], base.box[0] * 1.01, base.box[0] * 0.99)
    for s in (vac, orb):
        ff = FFieldCUDA(s, "fp64", moves=False)
        want = orc.Oracle(s, moves=False).energy()[3:5]
        nbr, nup, cap = _rows(ff, s.natom)
        results = _call(torch, s, nbr, nup, cap)
        for got in results:
            assert _close(got, want, REL_REF), (s.pbc_type, got, want)
        assert np.array_equal(results[0], results[1])
        ff.close()


def test_noalloc_on_a_side_stream():
    torch = pytest.importorskip("torch")
    s = goldens.system("water512", "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    want = ff.getE10()[3:5]
    nbr, nup, cap = _rows(ff, s.natom)
    side = torch.cuda.Stream()
    for got in _call(torch, s, nbr, nup, cap, stream=side):
        assert _close(got, want, REL_SELF), (got, want)


def test_noalloc_skips_damaged_row_entries():
    torch = pytest.importorskip("torch")
    s = goldens.system("water512", "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    nbr, nup, cap = _rows(ff, s.natom)
    clean = _call(torch, s, nbr, nup, cap, calls=1)[0]
    # widen the rows by two slots holding partners outside the system, and count them in
    bad = np.zeros((s.natom, cap + 2), np.int32)
    bad[:, :cap] = nbr
    badup = nup.copy()
    for i in range(0, s.natom, 7):
        bad[i, nup[i]] = s.natom + 5 + i            # past the last atom
        bad[i, nup[i] + 1] = -3                      # negative
        badup[i] = nup[i] + 2
    badup[1::11] = 10 ** 6                           # counts far above the capacity: clamped
    for i in range(1, s.natom, 11):
        bad[i, nup[i]:] = -1                         # the rest of such a row holds only invalid partners
    for got in _call(torch, s, bad, badup, cap + 2):
        assert _close(got, clean, REL_SELF), (got, clean)


def test_noalloc_rejects_oversized_systems():
    L = native.lib()
    box = (C.c_double * 3)(30.0, 30.0, 30.0)
    rc = L.mcg_energy_switch_fp64_noalloc(300000, 256, 256, 256, 256, 8, 1, box, 12.0, 10.0, 256, None)
    assert rc == native.MCG_EINVAL
    assert b"natom must be in" in L.mcg_last_error()
