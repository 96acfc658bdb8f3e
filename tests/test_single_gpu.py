"""Parity of the single-system device engine (FField_CUDA's path) with the reference, through the C ABI.

Tolerances (relative to the magnitude of the total; energies in internal units):
  FP64 plain:  every energy component within 1e-10 relative of the reference's value; Verlet rows,
               exclusion rows and 1-4 pairs bit-exact as sets.
  mixed:       total energy within 1e-6 relative; each dE within 1e-4 kcal/mol.
"""
import os
import numpy as np
import pytest

import goldens
import oracle as orc
from mc_cpp_gb300 import build, native, systems
from mc_cpp_gb300.engine import FFieldCUDA

pytestmark = pytest.mark.gpu
KCAL = 418.4
FP64_REL = 1e-10
MIX_REL = 1e-6
MIX_DE_KCAL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    orc.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _close(a, b, rel):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(1.0, float(np.max(np.abs(b))))
    return np.all(np.abs(a - b) <= rel * scale), np.max(np.abs(a - b)) / scale


CASES = [(n, m) for n in goldens.REFERENCE_INPUTS for m in ("full", "switch")] + \
        [(n, m) for n in ("argon864", "water512", "water4096", "peptide") for m in ("full", "switch")] + \
        [("water33334", "switch")]


@pytest.mark.parametrize("name,mode", CASES)
def test_energy_fp64_matches_reference(name, mode):
    s = goldens.system(name, mode)
    ff = FFieldCUDA(s, "fp64", moves=False)
    e = ff.getE10()
    want = np.array(goldens.record(name, mode)["ener"])
    ok, err = _close(e, want, FP64_REL)
    assert ok, (name, mode, err, e, want)


@pytest.mark.parametrize("name,mode", CASES)
def test_energy_mixed_within_tolerance(name, mode):
    s = goldens.system(name, mode)
    ff = FFieldCUDA(s, "mixed", moves=False)
    e = ff.getE10()
    want = np.array(goldens.record(name, mode)["ener"])
    rel = abs(e[0] - want[0]) / max(1.0, abs(want[0]))
    assert rel <= MIX_REL, (name, mode, rel)


@pytest.mark.parametrize("name", [n for n, m in CASES if m == "switch"])
def test_verlet_rows_bit_exact_sets(name):
    s = goldens.system(name, "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    rec = goldens.record(name, "switch")
    rows = ff.pairlist()
    assert sum(len(r) for r in rows) == rec["verlet_total"]
    assert goldens.rows_digest(rows) == rec["verlet_digest"]
    assert goldens.rows_digest(ff.exclusions()) == rec["excl_digest"]
    if rec["pairs14"] is not None:
        assert ff.pairs14().tolist() == rec["pairs14"]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name,mode", [("water512", "switch"), ("peptide", "switch"), ("diala_vac", "full"),
                                       ("nma_solvated", "full")])
def test_delta_e_against_oracle(name, mode, prec):
    s = goldens.system(name, mode)
    ff = FFieldCUDA(s, prec, moves=False)
    o = orc.Oracle(s, moves=False)
    rng = np.random.default_rng(11)
    xyz = s.coords()
    L = s.box[0]
    for trial in range(12):
        if name == "diala_vac":
            idx = np.array([int(rng.integers(0, s.natom))])
        else:
            r = int(rng.integers(0, s.resid.max())) + 1
            idx = np.nonzero(s.resid == r)[0]
            if len(idx) > 40 and trial % 2:
                idx = idx[:1]
        new = xyz[idx] + rng.uniform(-0.3, 0.3, 3)
        new -= L * np.round(new / L)
        de = ff.delta_e(idx, new)
        want_nb = o.delta_e(idx, new)
        # bonded part from the oracle's totals
        o.set_coords(xyz)
        e0 = o.energy()
        moved = xyz.copy()
        moved[idx] = new
        o.set_coords(moved)
        e1 = o.energy()
        o.set_coords(xyz)
        bonded = (e1[5:10] - e0[5:10]).sum()
        want = want_nb + bonded
        if prec == "fp64":
            assert abs(de - want) <= 1e-9 * KCAL + 1e-12 * abs(e0[0]), (trial, de, want)
        else:
            assert abs(de - want) / KCAL <= MIX_DE_KCAL, (trial, de, want)


def test_commit_then_energy_consistent():
    s = goldens.system("water512")
    ff = FFieldCUDA(s, "fp64", moves=False)
    e0 = ff.getE()
    xyz = s.coords()
    idx = np.array([30, 31, 32])
    new = xyz[idx] + np.array([0.1, -0.05, 0.07])
    de = ff.delta_e(idx, new)
    ff.commit()
    e1 = ff.getE()
    assert abs((e1 - e0) - de) <= 1e-8 * KCAL
    got = ff.coords()
    assert np.array_equal(got[idx], new)


@pytest.mark.parametrize("name,steps", [("argon864", 2000), ("water512", 300), ("nma_switch", 500), ("peptide", 30)])
def test_metropolis_replay_matches_reference_trace(name, steps):
    """Replays the reference's moves and random numbers: same move/instance/displacement/angle
    draws, dE within tolerance, and the accept decisions agree except logged ties."""
    g = goldens.golden()["mc"][name]
    s = goldens.system("nma_solvated", "switch") if name == "nma_switch" else goldens.system(name)
    want = goldens.trace(name)[:steps]
    ff = FFieldCUDA(s, "fp64")
    follow = np.stack([want[:, 1], want[:, 11]], 1).astype(np.int32)
    tr, etot, nacc, nties = ff.metropolis(steps, g["seed"], follow=follow)
    assert np.array_equal(tr[:, 1:7], want[:, 1:7])           # imvtyp, imvatm, r0..r2, rang: identical draws
    drawn = want[:, 10] >= 0
    assert np.array_equal(tr[:, 10] >= 0, drawn)              # alpha drawn on the same steps
    assert np.array_equal(tr[drawn, 10], want[drawn, 10])
    assert np.array_equal(tr[:, 11], want[:, 11])             # after following ties
    assert nties <= max(1, steps // 1000), nties
    de_err = np.abs(tr[:, 9] - want[:, 9]) / KCAL
    assert de_err.max() <= 1e-6, de_err.max()                 # kcal/mol
    if steps == g["nsteps"]:
        assert abs(etot - g["final_etot"]) <= 1e-9 * abs(g["final_etot"]) + 1e-6


def test_metropolis_free_run_agrees_without_following():
    g = goldens.golden()["mc"]["argon864"]
    s = goldens.system("argon864")
    ff = FFieldCUDA(s, "fp64")
    tr, etot, nacc, nties = ff.metropolis(2000, g["seed"])
    want = goldens.trace("argon864")
    assert nties == 0
    assert int(want[:, 11].sum()) == nacc
    assert np.array_equal(tr[:, 11], want[:, 11])


# ---- edge cases -------------------------------------------------------------------------
def _tiny(natom, L=20.0, seed=0, cut="switch"):
    s = systems.argon_random(natom, natom / L ** 3, seed)
    s.cut_mode = cut
    if natom > 1:
        s.q = np.where(np.arange(natom) % 2 == 0, 0.5, -0.5)
    return s


@pytest.mark.parametrize("natom", [1, 2, 3, 7])
@pytest.mark.parametrize("mode", ["full", "switch"])
def test_tiny_systems_match_oracle_bitwise_terms(natom, mode):
    s = _tiny(natom, L=26.0, seed=natom, cut=mode)
    ff = FFieldCUDA(s, "fp64", moves=False)
    o = orc.Oracle(s, moves=False)
    e, w = ff.getE10(), o.energy()
    assert np.allclose(e, w, rtol=1e-13, atol=1e-13), (e, w)
    if mode == "switch":
        assert goldens.rows_digest(ff.pairlist()) == goldens.rows_digest(o.verlet_rows())


def test_half_box_ties_and_cell_boundaries():
    # atoms exactly L/2 apart (MIC tie) and on cell boundaries; rint rounds half away from zero
    L = 30.0
    s = _tiny(6, L=L)
    xyz = np.array([[0.0, 0, 0], [15.0, 0, 0], [-7.5, 3.0, 0.0], [7.5, 7.5, 7.5], [-7.5, 0, 14.0], [3.0, -15.0, 4.0]])
    s.set_coords(xyz)
    s.cutoff, s.cuton, s.dcut = 14.0, 10.0, 1.0
    for mode in ("full", "switch"):
        s.cut_mode = mode
        ff = FFieldCUDA(s, "fp64", moves=False)
        o = orc.Oracle(s, moves=False)
        assert np.allclose(ff.getE10(), o.energy(), rtol=1e-13, atol=1e-12)
        if mode == "switch":
            assert goldens.rows_digest(ff.pairlist()) == goldens.rows_digest(o.verlet_rows())


def test_frozen_pairs_and_orthorhombic_and_no_pbc():
    s = goldens.system("water512", "switch")
    s.frozen = np.zeros(s.natom, np.uint8)
    s.frozen[:300] = 1
    s.pbc_type = "orbic"
    s.box = (s.box[0], s.box[0] * 1.01, s.box[0] * 0.99)
    ff = FFieldCUDA(s, "fp64", moves=False)
    o = orc.Oracle(s, moves=False)
    assert goldens.rows_digest(ff.pairlist()) == goldens.rows_digest(o.verlet_rows())
    ok, err = _close(ff.getE10(), o.energy(), FP64_REL)
    assert ok, err
    d = goldens.system("diala_vac", "switch")
    d.pbc_type = "none"
    ff = FFieldCUDA(d, "fp64", moves=False)
    o = orc.Oracle(d, moves=False)
    ok, err = _close(ff.getE10(), o.energy(), FP64_REL)
    assert ok, err


def test_list_capacity_grows_on_dense_clusters():
    s = goldens.system("water512", "switch")
    xyz = s.coords()
    xyz[:600] *= 0.35          # squeeze a third of the box: rows far above the density estimate
    s.set_coords(xyz)
    ff = FFieldCUDA(s, "fp64", moves=False)
    o = orc.Oracle(s, moves=False)
    assert goldens.rows_digest(ff.pairlist()) == goldens.rows_digest(o.verlet_rows())


def test_invalid_calls_return_status():
    s = goldens.system("water512")
    ff = FFieldCUDA(s, "fp64", moves=False)
    with pytest.raises(native.McgError) as ei:
        ff.delta_e([3, 3], np.zeros((2, 3)))
    assert ei.value.code == native.MCG_EINVAL
    with pytest.raises(native.McgError):
        ff.delta_e([s.natom], np.zeros((1, 3)))
    with pytest.raises(native.McgError):
        ff.delta_e(np.arange(2000), np.zeros((2000, 3)))
    with pytest.raises(native.McgError):
        ff.delta_e([0], np.array([[np.nan, 0, 0]]))
    with pytest.raises(native.McgError):
        ff.commit()
    # the handle stays usable after rejected calls
    assert np.isfinite(ff.getE())


def test_metropolis_1e5_moves_match_the_reference_run():
    """The small plain configuration at its stated length: 864 argon atoms, 1e5 single-atom moves
    of the reference's random stream (seed 1234), FP64, recorded from the compiled reference
    (tests/golden/argon864_long.npz).  Without following, every decision equals the reference's
    and every dE agrees within 1e-6 kcal/mol; the final running energy agrees within 1e-9."""
    g = goldens.golden()["mc"]["argon864_long"]
    ref = np.load(os.path.join(goldens.GOLD_DIR, "argon864_long.npz"))
    n = g["nsteps"]
    acc_ref = np.unpackbits(ref["accepted"])[:n].astype(bool)
    s = goldens.system("argon864")
    ff = FFieldCUDA(s, "fp64")
    tr, etot, nacc, nties = ff.metropolis(n, g["seed"])
    assert nties == 0
    assert np.array_equal(tr[:, 2].astype(np.int32), ref["imvatm"])        # same moved atoms
    assert np.array_equal(tr[:, 11] != 0, acc_ref)                         # same decisions, all 1e5
    assert nacc == g["accepted"][0]
    drawn = ref["alpha"] >= 0
    assert np.array_equal(tr[:, 10] >= 0, drawn)
    assert np.array_equal(tr[drawn, 10], ref["alpha"][drawn])               # the same alpha draws
    assert (np.abs(tr[:, 9] - ref["de"]) / KCAL).max() <= 1e-6
    assert abs(etot - g["final_etot"]) <= 1e-9 * abs(g["final_etot"])


def test_device_metropolis_run_matches_the_reference_run():
    """Without per-step output, the 864-atom argon run (translation moves, no bonded terms) runs on
    the device, a launch per list-update period, on the reference's random words: over the 1e5
    recorded moves it accepts exactly the reference's count and ends at its running energy."""
    g = goldens.golden()["mc"]["argon864_long"]
    s = goldens.system("argon864")
    ff = FFieldCUDA(s, "fp64")
    _, etot, nacc, nties = ff.metropolis(g["nsteps"], g["seed"], trace=False)
    assert nties == 0
    assert nacc == g["accepted"][0]
    assert abs(etot - g["final_etot"]) <= 1e-9 * abs(g["final_etot"])


def test_device_metropolis_run_equals_the_host_loop():
    """The device run and the host loop (taken when a trace is asked for) make the same decisions
    on the same seed and leave bitwise the same coordinates; their running energies differ only in
    the summation order of the dE terms."""
    s = goldens.system("argon864")
    dev = FFieldCUDA(s, "fp64")
    host = FFieldCUDA(s, "fp64")
    l_dev, l_host = dev.kernel_launches(), host.kernel_launches()
    _, e_dev, a_dev, _ = dev.metropolis(3000, 99, trace=False)
    _, e_host, a_host, _ = host.metropolis(3000, 99, trace=True)
    # the device run takes a launch per 50 steps (and the list builds between), the host loop at
    # least one per step: the run without a trace did run on the device
    l_dev, l_host = dev.kernel_launches() - l_dev, host.kernel_launches() - l_host
    assert l_dev < 3000 // 4 and l_host >= 3000, (l_dev, l_host)
    assert a_dev == a_host
    assert np.array_equal(dev.coords(), host.coords())
    assert abs(e_dev - e_host) <= 1e-10 * abs(e_host)
    # the engines stay usable: a fresh energy equals the running one
    assert abs(dev.getE() - e_dev) <= 1e-9 * abs(e_dev)
