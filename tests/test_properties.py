"""Invariance properties of the energies, on the oracle (CPU) and on the device engine (GPU).

  - Translation: every atom shifted by one vector, coordinates wrapped back into the box the way
    the reference wraps them (x - L * rint(x / L), round half away from zero), leaves the total
    energy unchanged.  The same pairs are summed; only the last bits of each distance change.
  - Permutation: the residues of a water or argon box renumbered in a random order (each
    residue's atoms kept together, bonds and angles renumbered with them) leave it unchanged.
    The same pairs are summed in another order.  Residues stay contiguous, so the reference's
    half-index exclusion storage (pairs with 0 < j - i < N/2) excludes the same pairs.
  - Reversal: a move followed by the move back gives dE(move) + dE(back) = 0.

Tolerances: FP64 (the oracle and the plain engine) 1e-9 relative on totals (each side is within
1e-10 of the reference's arithmetic) and 1e-8 kcal/mol on dE; mixed 3e-6 relative on totals and
2e-4 kcal/mol on dE (each side is within the per-result mixed tolerances of FP64, 1e-6 relative
and 1e-4 kcal/mol, so their difference is within twice those; 3e-6 leaves room for the division
by the mixed total instead of the FP64 one).
"""
import numpy as np
import pytest

import goldens
import oracle as orc

KCAL = 418.4
FP64_REL = 1e-9
MIX_REL = 3e-6
FP64_DE = 1e-8 * KCAL
MIX_DE = 2e-4 * KCAL
SHIFT = np.array([3.1, -7.3, 11.9])


def wrapped(xyz, box):
    """The reference's periodic wrap (Tools::rint: round half away from zero)."""
    L = np.asarray(box, np.float64)
    t = xyz / L
    r = np.where(t >= 0.0, np.floor(t + 0.5), np.ceil(t - 0.5))
    return xyz - L * r


def translated(s, shift=SHIFT):
    t = s.copy()
    t.set_coords(wrapped(s.coords() + shift, s.box))
    return t


def permuted(s, seed):
    """The residues of s (contiguous blocks of equal resid) in a random order, renumbered."""
    rng = np.random.default_rng(seed)
    resid = np.asarray(s.resid)
    starts = np.flatnonzero(np.r_[True, resid[1:] != resid[:-1]])
    ends = np.r_[starts[1:], s.natom]
    order = rng.permutation(len(starts))
    new_of_old = np.empty(s.natom, np.int64)
    old_of_new = np.concatenate([np.arange(starts[r], ends[r]) for r in order])
    new_of_old[old_of_new] = np.arange(s.natom)
    p = s.copy()
    for name in ("x", "y", "z", "q", "eps", "sig", "eps14", "sig14", "mass", "frozen"):
        setattr(p, name, np.ascontiguousarray(np.asarray(getattr(s, name))[old_of_new]))
    if s.resid_seg is not None:
        p.resid_seg = np.asarray(s.resid_seg)[old_of_new].copy()
    if s.atom_type is not None:
        p.atom_type = np.asarray(s.atom_type)[old_of_new].copy()
    for name in ("resname", "atname", "segname"):
        v = getattr(s, name)
        if len(v) == s.natom:
            setattr(p, name, [v[a] for a in old_of_new])
    sizes = (ends - starts)[order]
    p.resid = np.repeat(np.arange(1, len(order) + 1), sizes).astype(np.asarray(s.resid).dtype)
    for name in ("bonds", "ub", "angles", "dihedrals", "impropers"):
        a = np.asarray(getattr(s, name))
        if a.size:
            setattr(p, name, new_of_old[a].astype(a.dtype))
    return p


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


# ---------------------------------------------------------------------------------- oracle (CPU)

@pytest.fixture(scope="module")
def _oracle_built():
    orc.build()


@pytest.mark.parametrize("name,mode", [("argon864", "switch"), ("water512", "switch"), ("water512", "full"),
                                       ("water4096", "switch")])
def test_oracle_energy_invariant_under_translation_and_permutation(_oracle_built, name, mode):
    s = goldens.system(name, mode)
    e = orc.Oracle(s, moves=False).energy()[0]
    et = orc.Oracle(translated(s), moves=False).energy()[0]
    ep = orc.Oracle(permuted(s, 7), moves=False).energy()[0]
    assert _rel(et, e) <= FP64_REL, (et, e)
    assert _rel(ep, e) <= FP64_REL, (ep, e)


def test_oracle_move_then_move_back_cancels(_oracle_built):
    s = goldens.system("water512", "switch")
    o = orc.Oracle(s, moves=False)
    rng = np.random.default_rng(4)
    xyz = s.coords()
    for _ in range(6):
        m = int(rng.integers(0, 512))
        idx = np.arange(3 * m, 3 * m + 3)
        new = xyz[idx] + rng.uniform(-0.2, 0.2, 3)
        d1 = o.delta_e(idx, new)
        moved = xyz.copy()
        moved[idx] = new
        o.set_coords(moved)
        d2 = o.delta_e(idx, xyz[idx])
        o.set_coords(xyz)
        assert abs(d1 + d2) <= FP64_DE, (d1, d2)


# ---------------------------------------------------------------------------- device engine (GPU)

@pytest.fixture(scope="module")
def _engine():
    from mc_cpp_gb300 import build, native
    from mc_cpp_gb300.engine import FFieldCUDA
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")
    return FFieldCUDA


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name,mode", [("argon864", "switch"), ("water512", "switch"), ("water4096", "switch"),
                                       ("water512", "full")])
def test_engine_energy_invariant_under_translation_and_permutation(_engine, prec, name, mode):
    s = goldens.system(name, mode)
    tol = FP64_REL if prec == "fp64" else MIX_REL
    e = _engine(s, prec, moves=False).getE10()[0]
    et = _engine(translated(s), prec, moves=False).getE10()[0]
    ep = _engine(permuted(s, 7), prec, moves=False).getE10()[0]
    assert _rel(et, e) <= tol, (prec, et, e)
    assert _rel(ep, e) <= tol, (prec, ep, e)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_engine_move_then_move_back_cancels(_engine, prec):
    s = goldens.system("water4096", "switch")
    ff = _engine(s, prec, moves=False)
    tol = FP64_DE if prec == "fp64" else MIX_DE
    rng = np.random.default_rng(4)
    xyz = s.coords()
    for _ in range(6):
        m = int(rng.integers(0, 4096))
        idx = np.arange(3 * m, 3 * m + 3)
        new = xyz[idx] + rng.uniform(-0.2, 0.2, 3)
        d1 = ff.delta_e(idx, new)
        ff.commit()
        d2 = ff.delta_e(idx, xyz[idx])
        ff.commit()
        assert abs(d1 + d2) <= tol, (prec, d1, d2)


def test_pruning_criterion_keeps_every_pair_within_cutoff(_oracle_built):
    """The mixed pair kernel's row pruning rule, checked on the oracle's Verlet list in FP64.

    Rows pruned at positions P0 to the pairs within rc + b keep every list pair that is within rc
    at P1, as long as no atom moved more than b/2 between P0 and P1 (triangle inequality through
    the minimum image).  Moves of up to b/2 - 1e-3 A (the engine's re-prune limit) are tried in
    the directions that close pairs fastest, each atom towards the centre of the box."""
    s = goldens.system("water4096", "switch")
    o = orc.Oracle(s, moves=False)
    L = np.asarray(s.box, np.float64)
    rc, b = s.cutoff, 0.5
    xyz0 = s.coords()
    rows = o.verlet_rows()
    i = np.repeat(np.arange(s.natom), [len(r) for r in rows])
    j = np.concatenate(rows)

    def dist(xyz):
        d = xyz[j] - xyz[i]
        d -= L * np.round(d / L)
        return np.sqrt((d * d).sum(1))

    kept = dist(xyz0) <= rc + b
    assert kept.sum() < len(j)                         # pruning removes entries
    rng = np.random.default_rng(11)
    lim = 0.5 * b - 1e-3
    for trial in range(3):
        if trial == 0:                                 # every atom towards the box centre
            v = -xyz0 / np.linalg.norm(xyz0, axis=1, keepdims=True)
        else:                                          # random directions
            v = rng.normal(size=xyz0.shape)
            v /= np.linalg.norm(v, axis=1, keepdims=True)
        xyz1 = xyz0 + lim * v
        inside = dist(xyz1) <= rc
        assert not np.any(inside & ~kept), int(np.sum(inside & ~kept))
    # and the limit is needed: two atoms of a pruned-out pair, each moved 0.35 A (more than b/2)
    # towards the other, come within rc, so rows this old must be pruned again
    d0 = dist(xyz0)
    k = int(np.flatnonzero((~kept) & (d0 <= rc + b + 0.2))[0])
    dv = xyz0[j[k]] - xyz0[i[k]]
    dv -= L * np.round(dv / L)
    u = dv / np.linalg.norm(dv)
    xyz1 = xyz0.copy()
    xyz1[i[k]] += 0.35 * u
    xyz1[j[k]] -= 0.35 * u
    assert dist(xyz1)[k] <= rc and not kept[k]
