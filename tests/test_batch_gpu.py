"""Batched chains (the persistent sweep kernel) against the FP64 oracle, through the C ABI.

Tolerances: the FP64 recompute of the device equals the oracle's energy of the same coordinates
within 1e-10 relative; the running energy (initial FP64 energy plus the accepted mixed-precision
dE) stays within 1e-6 relative of the FP64 recompute; rigid geometry is kept to 1e-5 A.  The
mixed-precision recompute is within 1e-6 of max(|E|, 10 kcal/mol per molecule): these seeded
boxes start unrelaxed, with totals that nearly cancel, so |E| alone is no scale for FP32 pair
terms of ~10^4 iu.
"""
import numpy as np
import pytest

import oracle as orc
from mc_cpp_gb300 import build, native, systems
from mc_cpp_gb300.engine import BatchChains

pytestmark = pytest.mark.gpu
KCAL = 418.4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    orc.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _waters(sizes=(512, 700, 1100, 2300), seed=21, temp=300.0):
    return [systems.water_box(n, seed=seed + k, temp=temp + 10 * k) for k, n in enumerate(sizes)]


def _scale(B, e):
    """max(|E|, 10 kcal/mol per molecule): the size of the energy of a relaxed box of these chains."""
    return np.maximum(np.abs(e), 10.0 * KCAL * B.sizes / 3)


def _oracle_nonbonded(s, xyz):
    t = s.copy()
    t.set_coords(xyz)
    o = orc.Oracle(t, moves=False)
    e = o.energy()
    return e[3] + e[4]


def test_initial_energies_match_oracle():
    ch = _waters()
    B = BatchChains(ch, seed=5)
    e = B.energy_fp64()
    for k, s in enumerate(ch):
        want = _oracle_nonbonded(s, s.coords())
        assert abs(e[k] - want) <= 1e-10 * abs(want), (k, e[k], want)
    _, _, etot = B.stats()
    assert np.allclose(etot, e, rtol=0, atol=0)
    em = B.energy_mixed()
    assert np.all(np.abs(em - e) <= 1e-6 * _scale(B, e)), (em, e)


def test_sweeps_keep_running_energy_and_geometry():
    ch = _waters()
    B = BatchChains(ch, seed=6)
    B.sweep(4)
    t, a, etot = B.stats()
    assert np.all(t == 4 * (B.sizes // 3))
    assert np.all(a > 0) and np.all(a < t)
    e = B.energy_fp64()
    rel = np.abs(etot - e) / np.abs(e)
    assert rel.max() <= 1e-6, rel
    assert (np.abs(B.energy_mixed() - e) / _scale(B, e)).max() <= 1e-6
    for k, s in enumerate(ch):
        xyz = B.coords(k)
        want = _oracle_nonbonded(s, xyz)
        assert abs(e[k] - want) <= 1e-10 * abs(want)
        L = s.box[0]
        o, h1, h2 = xyz[0::3], xyz[1::3], xyz[2::3]
        for h in (h1, h2):
            d = h - o
            d -= L * np.round(d / L)
            assert np.abs(np.linalg.norm(d, axis=1) - 0.9572).max() < 1e-5
        d = h1 - h2
        d -= L * np.round(d / L)
        hh = 2 * 0.9572 * np.sin(np.radians(104.52 / 2))
        assert np.abs(np.linalg.norm(d, axis=1) - hh).max() < 1e-5


def test_deterministic_for_a_seed():
    ch = _waters((512, 900))
    B1 = BatchChains(ch, seed=9)
    B2 = BatchChains(ch, seed=9)
    B1.sweep(2)
    B2.sweep(2)
    for k in range(2):
        assert np.array_equal(B1.coords(k), B2.coords(k))
    assert np.array_equal(B1.stats()[2], B2.stats()[2])
    B3 = BatchChains(ch, seed=10)
    B3.sweep(2)
    assert not np.array_equal(B1.coords(0), B3.coords(0))


def test_list_rebuilds_keep_energy_exact():
    ch = _waters((600, 1500))
    for s in ch:
        s.dcut = 0.4          # small skin: the half-skin trigger fires every few moves
    B = BatchChains(ch, seed=12)
    B.sweep(3)
    rb, _ = B.counters()
    assert rb >= 10           # list builds of both chains, most of them inside the sweeps
    _, _, etot = B.stats()
    e = B.energy_fp64()
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6
    # the lists in place after the sweeps still hold every pair inside the cutoff
    assert (np.abs(B.energy_mixed() - e) / _scale(B, e)).max() <= 1e-6


def _pairs_within(xyz, apr, L, rc):
    """Residue pairs (r < q) with an atom pair within rc (minimum image), by brute force."""
    n = len(xyz) // apr
    X = xyz.reshape(n, apr, 3)
    need = []
    for r in range(n - 1):
        d = X[r + 1:, None, :, :] - X[r, :, None, :][None]          # (q, k, b, 3)
        d -= L * np.round(d / L)
        close = (np.einsum("qkbi,qkbi->qkb", d, d) <= rc * rc).any(axis=(1, 2))
        need.extend((r, r + 1 + q) for q in np.nonzero(close)[0])
    return need


def test_lists_kept_between_sweeps_stay_complete():
    """Chains keep their lists across sweeps until their atoms have moved enough; the lists in
    place after every sweep must still hold every residue pair with an atom pair inside the cutoff
    (checked by brute force on the host), and energies over kept and fresh lists agree."""
    ch = _waters((900, 2600, 5000), seed=47)
    B = BatchChains(ch, seed=19)
    e0 = B.energy_fp64()
    rb0, _ = B.counters()
    for k in range(4):
        B.sweep(1)
        for c in (0, 1):
            rows = [set(r.tolist()) for r in B.lists(c)]
            miss = [(r, q) for r, q in _pairs_within(B.coords(c), 3, ch[c].box[0], 12.0)
                    if q not in rows[r] or r not in rows[q]]
            assert not miss, (k, c, miss[:5])
        kept = B.energy_mixed()           # over the lists in place
        rb, _ = B.counters()
        B.update_lists()
        fresh = B.energy_mixed()          # over lists built from the current coordinates
        # the same pairs inside the cutoff, summed in another order
        assert np.all(np.abs(kept - fresh) <= 1e-8 * _scale(B, fresh)), (k, kept, fresh)
    assert rb - rb0 < 3 * 4 + 5        # fewer builds than one per chain and sweep (plus the forced ones)
    assert not np.allclose(B.energy_fp64(), e0)


def test_orthorhombic_chain():
    """A chain in an orthorhombic box (different edge per axis): the fixed-point mirrors, the
    minimum image of every displacement, the cell grid and the lists follow each axis's edge."""
    cub = systems.water_box(700, seed=51)
    orb = systems.water_box(900, seed=52)
    L = orb.box[0]
    scale = np.array([1.0, 1.08, 0.93])
    orb.set_coords(orb.coords() * scale)
    orb.pbc_type = "orbic"
    orb.box = tuple(L * scale)
    B = BatchChains([cub, orb], seed=9)
    B.sweep(2)
    _, a, etot = B.stats()
    e = B.energy_fp64()
    assert np.all(a > 0)
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6
    assert abs(e[1] - _oracle_nonbonded(orb, B.coords(1))) <= 1e-10 * abs(e[1])
    rows = [set(r.tolist()) for r in B.lists(1)]
    miss = [(r, q) for r, q in _pairs_within(B.coords(1), 3, np.array(orb.box), 12.0)
            if q not in rows[r] or r not in rows[q]]
    assert not miss, miss[:5]


def test_argon_chains_and_mixed_residue_sizes():
    ar = [systems.argon_random(n, rho, seed, temp=t) for n, rho, seed, t in ((500, 0.02, 1, 100.0), (900, 0.018, 2, 130.0))]
    B = BatchChains(ar, seed=3)
    B.sweep(3)
    _, a, etot = B.stats()
    e = B.energy_fp64()
    assert np.all(a > 0)
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6
    for k, s in enumerate(ar):
        assert abs(e[k] - _oracle_nonbonded(s, B.coords(k))) <= 1e-10 * abs(e[k])
    # argon and water in one batch take the generic residue-size kernel
    mix = [ar[0], _waters((512,))[0]]
    M = BatchChains(mix, seed=4)
    M.sweep(2)
    _, _, etot = M.stats()
    e = M.energy_fp64()
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6


def test_host_buffer_run_roundtrip():
    ch = _waters((512, 800))
    B = BatchChains(ch, seed=14)
    n = B.natoms
    out = np.zeros((3, n))
    B.run_host(None, 0, out)
    xyz0 = np.concatenate([s.coords() for s in ch]).T
    assert np.abs(out - xyz0).max() < 1e-9
    a, e = B.run_host(out.copy(), 2, out)
    ef = B.energy_fp64()
    assert (np.abs(e - ef) / np.abs(ef)).max() <= 1e-6
    got = np.concatenate([B.coords(k) for k in range(2)]).T
    assert np.array_equal(got, out)


def test_host_import_of_exported_coordinates_changes_nothing():
    """Coordinates given back exactly as exported leave every chain as it was: a host-buffer run
    of one sweep is bitwise one plain sweep (coordinates, running energies, counters)."""
    ch = _waters((600, 900, 700), seed=35)
    A = BatchChains(ch, seed=16)
    B = BatchChains(ch, seed=16)
    out = np.zeros((3, B.natoms))
    for _ in range(2):
        B.run_host(None, 0, out)
        B.run_host(out.copy(), 1, out)
        A.sweep(1)
    for k in range(len(ch)):
        assert np.array_equal(A.coords(k), B.coords(k))
    for a, b in zip(A.stats(), B.stats()):
        assert np.array_equal(a, b)
    assert np.array_equal(np.concatenate([A.coords(k) for k in range(len(ch))]).T, out)


def test_host_import_rebuilds_only_chains_that_moved():
    """Importing coordinates rebuilds the lists of exactly the chains whose atoms moved beyond the
    rebuild threshold from their list-build positions, and recomputes the energies of the chains
    whose coordinates changed."""
    ch = _waters((600, 900), seed=33)
    B = BatchChains(ch, seed=15)
    out = np.zeros((3, B.natoms))
    B.run_host(None, 0, out)
    rb0, _ = B.counters()
    _, e = B.run_host(out.copy(), 0, out)          # unchanged coordinates: the lists stay valid
    rb1, _ = B.counters()
    assert rb1 == rb0
    ef = B.energy_fp64()
    assert np.all(np.abs(e - ef) <= 1e-6 * _scale(B, ef))
    xin = out.copy()
    idx = ch[0].natom + np.arange(300)             # 100 molecules of chain 1, 2.6 A (half skin: 1 A)
    xin[:, idx] += 1.5
    _, e = B.run_host(xin, 0, out)
    rb2, _ = B.counters()
    assert rb2 == rb1 + 1
    rows = [set(r.tolist()) for r in B.lists(1)]
    miss = [(r, q) for r, q in _pairs_within(B.coords(1), 3, ch[1].box[0], 12.0) if q not in rows[r] or r not in rows[q]]
    assert not miss, miss[:5]
    ef = B.energy_fp64()
    assert np.all(np.abs(e - ef) <= 1e-6 * _scale(B, ef))


def test_invalid_batches_rejected():
    w = systems.water_box(512, seed=3)
    flexible = w.copy()
    # without bonds and angles no intra-residue pair is excluded: not a rigid residue
    for k in ("angles", "angle_type", "angle_k", "angle_theta0", "bonds", "bond_type", "bond_k", "bond_r0", "bond_beta"):
        setattr(flexible, k, getattr(flexible, k)[:0])
    with pytest.raises(native.McgError) as ei:
        BatchChains([w, flexible])
    assert ei.value.code == native.MCG_ENOTSUP
    small = systems.water_box(100, seed=1)    # box < 2 * cutoff
    with pytest.raises(native.McgError) as ei:
        BatchChains([small])
    assert ei.value.code == native.MCG_EINVAL


@pytest.mark.parametrize("speculation,clusters", [(4, -1), (4, 0), (8, 0), (2, 0), (16, -1), (16, 0), (32, 0)])
def test_speculative_sweep_reproduces_sequential_chain(speculation, clusters):
    """Moves evaluated together (up to 16 on one CTA, 32 on a two-CTA cluster) must give the
    sequential chain: same random numbers, same decisions, same coordinates.  dE sums differ only
    in float summation order, so a decision could flip only at an exact tie (~1e-7 per move)."""
    ch = _waters((4000, 2600, 1500), seed=31)
    seq = BatchChains(ch, seed=17, speculation=1, clusters=-1)
    spec = BatchChains(ch, seed=17, speculation=speculation, clusters=clusters)
    if clusters == 0:
        assert spec.tuning()["clusters"] == 1
    seq.sweep(2)
    spec.sweep(2)
    t1, a1, e1 = seq.stats()
    t2, a2, e2 = spec.stats()
    assert np.array_equal(t1, t2)
    assert np.abs(a1 - a2).max() <= 1
    same = [np.array_equal(seq.coords(k), spec.coords(k)) for k in range(len(ch))]
    assert sum(same) >= len(ch) - 1, same
    ef = spec.energy_fp64()
    assert (np.abs(e2 - ef) / np.abs(ef)).max() <= 1e-6


def test_dmax_adjustment_follows_the_reference_rule():
    """MC::adjust_dmax (MC.cpp:165-173) after every dmax_each-th move of a chain, per move type.
    With a 100% target no window exceeds it, so every adjustment multiplies dmax by 0.9: after n
    moves, dmax = dmax0 * 0.9^floor(n / each), across sweep boundaries.  With a 0% target a window
    that accepted a move of the type grows dmax by 1.1, never past the cap."""
    ch = _waters((600, 900), seed=41)
    B = BatchChains(ch, seed=5, dmax_each=(10, 14), dmax_target=(100.0, 100.0))
    B.sweep(2)
    t, r = B.dmax()
    n = np.array([600, 900]) * 2
    assert np.allclose(t, 0.15 * 0.9 ** (n // 10), rtol=1e-12, atol=0), t
    assert np.allclose(r, 15.0 * 0.9 ** (n // 14), rtol=1e-12, atol=0), r
    _, _, etot = B.stats()
    e = B.energy_fp64()
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6
    G = BatchChains(ch, seed=5, dmax_each=(10, 10), dmax_target=(0.0, 0.0), dmax_max=(0.2, 20.0))
    G.sweep(1)
    t, r = G.dmax()
    assert np.all(t <= 0.2) and np.all(r <= 20.0)
    assert np.all(t > 0.15) and np.all(r > 15.0)
    with pytest.raises(native.McgError):
        BatchChains(ch, dmax_each=(10, 0), dmax_max=(0.1, 0.0))      # cap below the initial dmax


@pytest.mark.parametrize("speculation", [4, 8, 16])
def test_speculative_sweep_with_dmax_adjustment_is_sequential(speculation):
    """Iterations end at the move after which dmax is adjusted, so moves evaluated together share
    one dmax and the chain equals the sequential one, dmax included."""
    ch = _waters((2600, 1500), seed=43)
    kw = dict(seed=23, clusters=-1, dmax_each=(7, 11), dmax_target=(25.0, 15.0))
    seq = BatchChains(ch, speculation=1, **kw)
    spec = BatchChains(ch, speculation=speculation, **kw)
    seq.sweep(2)
    spec.sweep(2)
    t1, a1, _ = seq.stats()
    t2, a2, _ = spec.stats()
    assert np.array_equal(t1, t2)
    same = [np.array_equal(seq.coords(k), spec.coords(k)) for k in range(len(ch))]
    assert sum(same) >= len(ch) - 1, same
    d1, d2 = seq.dmax(), spec.dmax()
    for k in range(len(ch)):
        if same[k]:
            assert d1[0][k] == d2[0][k] and d1[1][k] == d2[1][k]
    assert not np.allclose(d1[0], 0.15)          # adjusted


def test_autotune_picks_a_shape_and_keeps_the_chain_exact(tmp_path, monkeypatch):
    monkeypatch.setenv("MCG_TUNE_CACHE", str(tmp_path / "tune.txt"))
    ch = _waters((512, 1500, 3000), seed=41)
    B = BatchChains(ch, seed=8)
    t = B.autotune(trial_sweeps=1, use_cache=False)
    assert (t["threads_per_chain"], t["ctas_per_sm"]) in ((512, 1), (512, 2), (256, 2), (128, 4), (128, 8)) and t["clusters"] in (0, 1)
    assert t["speculation"] in (0, 1, 2, 4, 8) and t["ms_per_sweep"] > 0 and not t["from_cache"]
    assert {k: t[k] for k in ("threads_per_chain", "ctas_per_sm", "speculation", "clusters")} == B.tuning()
    tr, a, etot = B.stats()
    sweeps = tr // (B.sizes // 3)                      # every shape: 1 warm-up + 1 timed sweep
    assert np.all(tr == sweeps * (B.sizes // 3)) and np.all(sweeps == sweeps[0]) and sweeps[0] >= 8
    B.sweep(2)
    _, _, etot = B.stats()
    e = B.energy_fp64()
    assert (np.abs(etot - e) / np.abs(e)).max() <= 1e-6
    # a second batch of the same workload takes the cached shape without trial sweeps
    B2 = BatchChains(ch, seed=8)
    t2 = B2.autotune(trial_sweeps=1, use_cache=True)
    assert t2["from_cache"]
    assert [t2[k] for k in ("threads_per_chain", "ctas_per_sm", "speculation", "clusters")] == \
           [t[k] for k in ("threads_per_chain", "ctas_per_sm", "speculation", "clusters")]
    assert np.all(B2.stats()[0] == 0)
    assert (tmp_path / "tune.txt").read_text().count("\n") == 1


def test_phase_timing_adds_up():
    ch = _waters((800, 2000), seed=43)
    B = BatchChains(ch, seed=2)
    B.sweep(1)
    tot, lists, sweep = B.time_phases(3)
    assert lists > 0 and sweep > 0
    assert lists + sweep <= tot * 1.01 + 0.05
    assert np.all(B.stats()[0] == 4 * (B.sizes // 3))


def _snapshot(B):
    t, a, e = B.stats()
    dt, dr = B.dmax()
    return t, a, e, dt, dr, [B.coords(k) for k in range(B.nchains)], B.pairs()


@pytest.mark.parametrize("shape", ["same", "other"])
def test_checkpoint_resume_is_bit_exact(tmp_path, shape):
    """Sweeping 4, saving, loading into a fresh batch of the same chains and sweeping 4 more gives
    bitwise the chains of 8 sweeps without the save: coordinates, running energies, counters,
    pair counts and adjusted dmax.  With shape 'other' the fresh batch starts with another launch
    shape, and the load re-applies the saved one."""
    chains = _waters((600, 1500, 900))
    kw = dict(dmax_trn=0.15, dmax_rot=15.0, seed=9, dmax_each=(30, 30), dmax_target=(40.0, 40.0),
              threads_per_chain=256, speculation=4, clusters=-1)
    A = BatchChains(chains, **kw)
    A.sweep(4)
    ck = str(tmp_path / "batch.ckpt")
    A.save(ck)
    A.sweep(4)
    want = _snapshot(A)
    kw2 = dict(kw) if shape == "same" else dict(kw, threads_per_chain=512, speculation=0, clusters=0)
    B = BatchChains(chains, **kw2)
    B.sweep(1)                                  # state to be overwritten by the load
    B.load(ck)
    assert B.tuning()["threads_per_chain"] == 256
    B.sweep(4)
    got = _snapshot(B)
    for w, g in zip(want[:5], got[:5]):
        assert np.array_equal(w, g), (w, g)
    for w, g in zip(want[5], got[5]):
        assert np.array_equal(w, g)
    # a checkpoint restores the pair counters too (statistics of the chain, not of the batch)
    assert np.array_equal(want[6], got[6])
    A.close()
    B.close()


def test_checkpoint_rejects_other_batches_and_damaged_files(tmp_path):
    chains = _waters((600, 900))
    A = BatchChains(chains, seed=9)
    A.sweep(1)
    ck = tmp_path / "a.ckpt"
    A.save(str(ck))
    other = BatchChains(chains, seed=10)                       # another Philox key
    with pytest.raises(native.McgError) as ei:
        other.load(str(ck))
    assert ei.value.code == native.MCG_EINVAL
    fewer = BatchChains(chains[:1], seed=9)
    with pytest.raises(native.McgError) as ei:
        fewer.load(str(ck))
    assert ei.value.code == native.MCG_EINVAL
    raw = ck.read_bytes()
    (tmp_path / "short.ckpt").write_bytes(raw[:-100])
    bad = bytearray(raw)
    bad[len(raw) // 2] ^= 0x40
    (tmp_path / "flip.ckpt").write_bytes(bytes(bad))
    for name in ("short.ckpt", "flip.ckpt", "missing.ckpt"):
        with pytest.raises(native.McgError) as ei:
            A.load(str(tmp_path / name))
        assert ei.value.code == native.MCG_EIO
    # the batch is unchanged by the failed loads and still sweeps
    t0 = A.stats()[0]
    A.sweep(1)
    assert (A.stats()[0] > t0).all()


def test_host_buffer_run_from_pinned_memory_equals_pageable():
    """With page-locked host buffers the import and export kernels read and write them directly
    (no staging copy); the result is bitwise the staged run from ordinary (pageable) buffers:
    exported coordinates, running energies and accepted counts, step after step."""
    torch = pytest.importorskip("torch")
    ch = _waters((600, 900, 700), seed=41)
    P = BatchChains(ch, seed=18)
    Q = BatchChains(ch, seed=18)
    n = P.natoms
    pin_in = torch.empty((3, n), dtype=torch.float64, pin_memory=True).numpy()
    pin_out = torch.empty((3, n), dtype=torch.float64, pin_memory=True).numpy()
    out = np.zeros((3, n))
    P.run_host(None, 0, pin_out)
    Q.run_host(None, 0, out)
    assert np.array_equal(pin_out, out)
    for _ in range(3):
        pin_in[...] = pin_out
        ap, ep = P.run_host(pin_in, 1, pin_out)
        aq, eq = Q.run_host(out.copy(), 1, out)
        assert np.array_equal(pin_out, out)
        assert np.array_equal(ap, aq) and np.array_equal(ep, eq)
