"""Pins the CPU oracle (oracle/mc_oracle.cpp) to the reference's own outputs (tests/golden/).

Every comparison here is exact (==): the oracle restates FField_MDBAS, List_nonBonded and
MC_metropolis with the reference's operation order and no FMA contraction.
"""
import numpy as np
import pytest

import goldens
import oracle as orc

MODES = ("full", "switch")
CASES = [(n, m) for n in goldens.REFERENCE_INPUTS for m in MODES] + \
        [(n, m) for n in ("argon864", "water512", "peptide") for m in MODES] + [("water4096", "switch")]


@pytest.fixture(scope="module", autouse=True)
def _build():
    orc.build()


@pytest.mark.parametrize("name,mode", CASES)
def test_energy_components_bitwise(name, mode):
    s = goldens.system(name, mode)
    o = orc.Oracle(s, moves=False)
    e = o.energy()
    want = np.array(goldens.record(name, mode)["ener"])
    assert np.array_equal(e, want), (e, want)


@pytest.mark.parametrize("name,mode", CASES)
def test_exclusions_and_14(name, mode):
    s = goldens.system(name, mode)
    o = orc.Oracle(s, moves=False)
    rec = goldens.record(name, mode)
    rows = o.excl_rows()
    assert goldens.rows_digest(rows) == rec["excl_digest"]
    assert sum(len(r) for r in rows) == rec["excl_total"]
    p14 = o.pairs14()
    assert len(p14) == rec["n14"]
    if rec["pairs14"] is not None:
        assert p14.tolist() == rec["pairs14"]


@pytest.mark.parametrize("name", [n for n, m in CASES if m == "switch"])
def test_verlet_rows_equal_reference(name):
    s = goldens.system(name, "switch")
    o = orc.Oracle(s, moves=False)
    rec = goldens.record(name, "switch")
    assert o.verlet_total() == rec["verlet_total"] == rec["list_pairs"]
    assert goldens.rows_digest(o.verlet_rows()) == rec["verlet_digest"]


def test_native_xml_energies():
    for name in goldens.REFERENCE_INPUTS:
        rec = goldens.golden()["systems"][name]["native_xml"]
        assert rec["ener"] == goldens.record(name, rec["cut_mode"])["ener"]


# (golden trace, steps checked, system, seed)
MC = [("nma_switch", 200), ("argon864", 600), ("water512", 300), ("peptide", 8)]


@pytest.mark.parametrize("name,steps", MC)
def test_metropolis_trace_bitwise(name, steps):
    g = goldens.golden()["mc"][name]
    if name == "nma_switch":
        s = goldens.system("nma_solvated", "switch")
    else:
        s = goldens.system(name)
    o = orc.Oracle(s)
    tr, _, _ = o.mc_run(steps, g["seed"])
    want = goldens.trace(name)[:steps]
    assert np.array_equal(tr, want), np.argwhere(tr != want)[:5]


def test_reference_acceptance_counts_nma():
    # the reference's own run: NMA switch, 500 steps, seed 1234 -> TRN 245/75, ROT 255/100
    g = goldens.golden()["mc"]["nma_switch"]
    assert g["trials"] == [245, 255]
    assert g["accepted"] == [75, 100]


def test_delta_e_matches_energy_difference():
    s = goldens.system("water512")
    o = orc.Oracle(s, moves=False)
    rng = np.random.default_rng(0)
    e0 = o.energy()[0]
    xyz = s.coords()
    for _ in range(5):
        m = int(rng.integers(0, 512))
        idx = np.arange(3 * m, 3 * m + 3)
        new = xyz[idx] + rng.uniform(-0.2, 0.2, 3)
        de = o.delta_e(idx, new)
        moved = xyz.copy()
        moved[idx] = new
        o.set_coords(moved)
        e1 = o.energy()[0]
        o.set_coords(xyz)
        # nonbonded only: bonded terms of a rigidly translated water are unchanged up to rounding
        assert abs(de - (e1 - e0)) < 1e-6 * max(1.0, abs(e0)) * 1e-6 + 1e-6


# ---- the batched chain restatement (oracle/batch_oracle.cpp) --------------------------------
def test_philox_restatement_known_answers():
    """Philox4x32-10 against the known-answer vectors published with the algorithm (Random123)."""
    assert orc.philox4x32_10([0, 0, 0, 0], [0, 0]) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert orc.philox4x32_10([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert orc.philox4x32_10([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)


@pytest.mark.parametrize("name", ["water512", "argon864"])
def test_batch_restatement_energy_equals_pinned_oracle(name):
    """The batched restatement's all-pairs FP64 energy equals the pinned oracle's switched energy
    (every pair within the cutoff is in the Verlet list, so both sum the same pairs)."""
    s = goldens.system(name, "switch")
    want = orc.Oracle(s, moves=False).energy()
    b = orc.BatchChainOracle(s, chain=0, seed=1)
    assert abs(b.energy() - (want[3] + want[4])) <= 1e-10 * abs(want[3] + want[4])


def test_long_argon_fixture_extends_the_short_trace():
    """The 1e5-move argon fixture and the 2,000-step trace come from the same reference run
    (seed 1234): their common steps agree exactly."""
    import os
    g = goldens.golden()["mc"]["argon864_long"]
    ref = np.load(os.path.join(goldens.GOLD_DIR, "argon864_long.npz"))
    short = goldens.trace("argon864")
    k = len(short)
    assert g["nsteps"] == 100000 and g["seed"] == goldens.golden()["mc"]["argon864"]["seed"]
    assert np.array_equal(ref["imvatm"][:k], short[:, 2].astype(np.int32))
    assert np.array_equal(ref["de"][:k], short[:, 9])
    assert np.array_equal(ref["alpha"][:k], short[:, 10])
    assert np.array_equal(np.unpackbits(ref["accepted"])[:k], short[:, 11].astype(np.uint8))
    assert int(np.unpackbits(ref["accepted"])[:g["nsteps"]].sum()) == g["accepted"][0]
