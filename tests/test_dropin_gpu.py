"""The drop-in call sequence: MC_metropolis::run's getE() calls on coordinates the caller moves in
place, through the C ABI entry FField_CUDA::getE() uses (mcg_energy_host).

MC_metropolis::run (MC_metropolis.cpp:62-165) calls getE() once before the loop, then per trial
move getE() (eold), moves the atoms in the AtomList, getE() (enew), restores the atoms of a
rejected move, and calls askListUpdate() every 50 steps.  FField_CUDA::askListUpdate first passes
the AtomList's coordinates to mcg_energy_host (so an accepted move is on the device), then calls
mcg_update_lists.  These tests run exactly that sequence on plain arrays (the AtomList's
coordinate vectors), without the reference's objects, which are absent where the GPU is:

* argon, 864 atoms: the reference's own 2,000 recorded moves (tests/golden/trace_argon864.npy)
  applied as Move.hpp does; every eold and enew equals the reference's getE() within 1e-10
  relative, and the criterion on enew - eold reproduces its decisions;
* water, 512 molecules, residue translations and rotations drawn here: every getE() equals a full
  upload and recompute on a second handle (FP64 within 1e-10 relative; mixed precision within
  1e-6), including after list updates and rejected moves;
* invalid coordinates are rejected with MCG_EINVAL and the handle recovers; a change of more than
  1,024 atoms falls back to one full recompute.
"""
import math
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
KCAL = 418.4
REL64 = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _wrap(v, L):
    # Move.hpp re-wraps each moved atom with PerConditions::applyPBC (Tools::rint: half away from zero)
    t = (1.0 / L) * v
    return v - L * float(int(t + 0.5) if t >= 0 else int(t - 0.5))


def test_dropin_sequence_reproduces_the_reference_argon_run():
    g = goldens.golden()["mc"]["argon864"]
    want = goldens.trace("argon864")
    s = goldens.system("argon864")
    L = s.box[0]
    inst = orc.Oracle(s).move_instances(0)
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    ff = FFieldCUDA(s, "fp64", moves=False)
    beta = 1.0 / (0.83144621 / KCAL * s.temp)          # the reference's units (MC_metropolis.cpp:188)
    etot = ff.getE_host(x, y, z)
    ties = 0
    for st, row in enumerate(want, 1):
        atoms = [a for lo, hi in inst[int(row[2])][0] for a in range(lo, hi + 1)]
        eold = ff.getE_host(x, y, z)
        assert abs(eold - row[7]) <= REL64 * abs(row[7]), (st, eold, row[7])
        back = [(x[a], y[a], z[a]) for a in atoms]
        for a in atoms:
            x[a] = _wrap(x[a] + row[3], L)
            y[a] = _wrap(y[a] + row[4], L)
            z[a] = _wrap(z[a] + row[5], L)
        enew = ff.getE_host(x, y, z)
        assert abs(enew - row[8]) <= REL64 * abs(row[8]), (st, enew, row[8])
        de = enew - eold
        mine = de <= np.finfo(float).eps or (row[10] >= 0 and row[10] < math.exp(-beta * de))
        accepted = row[11] != 0
        if mine != accepted:
            ties += 1
            assert abs(row[10] - math.exp(-beta * de)) < 1e-9, (st, row[10], de)
        if accepted:
            etot += de
        else:
            for a, (bx, by, bz) in zip(atoms, back):
                x[a], y[a], z[a] = bx, by, bz
        if st % 50 == 0:
            ff.getE_host(x, y, z)
            ff.askListUpdate(st)
    assert ties == 0
    assert abs(etot - g["final_etot"]) <= 1e-9 * abs(g["final_etot"])


def _rot(v, axis, ang):
    axis = axis / np.linalg.norm(axis)
    c, s = math.cos(ang), math.sin(ang)
    return v * c + np.cross(axis, v) * s + axis * np.dot(axis, v) * (1 - c)


@pytest.mark.parametrize("precision,tol", [("fp64", REL64), ("mixed", 1e-6)])
def test_dropin_sequence_matches_full_recomputes_on_water(precision, tol):
    s = goldens.system("water512", "switch")
    L = s.box[0]
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    ff = FFieldCUDA(s, precision, moves=False)
    full = FFieldCUDA(s, precision, moves=False)
    rng = np.random.default_rng(3)
    beta = 1.0 / (0.0019872 * s.temp * KCAL)          # physical units: dE in iu -> kcal/mol

    def check(e):
        full.setCoords(np.stack([x, y, z], 1))
        want = full.getE()
        assert abs(e - want) <= tol * abs(want), (e, want)
    e = ff.getE_host(x, y, z)
    check(e)
    nacc = 0
    for st in range(1, 301):
        r = int(rng.integers(0, s.natom // 3))
        atoms = np.arange(3 * r, 3 * r + 3)
        eold = ff.getE_host(x, y, z)
        if st % 7 == 0:
            check(eold)
        back = np.stack([x[atoms], y[atoms], z[atoms]], 1)
        if rng.random() < 0.5:
            d = rng.uniform(-0.15, 0.15, 3)
            new = back + d
        else:
            piv = back[0]
            off = back - piv
            off -= L * np.round(off / L)
            ang = math.radians(rng.uniform(-15, 15))
            new = piv + np.array([_rot(o, rng.normal(size=3), ang) for o in off])
        new -= L * np.round(new / L)
        x[atoms], y[atoms], z[atoms] = new[:, 0], new[:, 1], new[:, 2]
        enew = ff.getE_host(x, y, z)
        if st % 7 == 0:
            check(enew)
        de = enew - eold
        if de <= 0 or rng.random() < math.exp(-beta * de):
            nacc += 1
        else:
            x[atoms], y[atoms], z[atoms] = back[:, 0], back[:, 1], back[:, 2]
        if st % 50 == 0:
            ff.getE_host(x, y, z)
            ff.askListUpdate(st)
            check(ff.getE_host(x, y, z))
    assert 0 < nacc < 300
    check(ff.getE_host(x, y, z))


def test_dropin_entry_rejects_bad_coordinates_and_recovers():
    s = goldens.system("water512", "switch")
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    ff = FFieldCUDA(s, "fp64", moves=False)
    e0 = ff.getE_host(x, y, z)
    x[5] = np.nan
    with pytest.raises(native.McgError) as ei:
        ff.getE_host(x, y, z)
    assert ei.value.code == native.MCG_EINVAL
    x[5] = s.x[5]
    assert ff.getE_host(x, y, z) == e0
    # more than 1024 atoms changed: one full recompute
    x[:2000] += 0.01
    full = FFieldCUDA(s, "fp64", moves=False)
    full.setCoords(np.stack([x, y, z], 1))
    assert abs(ff.getE_host(x, y, z) - full.getE()) <= REL64 * abs(full.getE())
