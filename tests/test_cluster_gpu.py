"""Cluster-pair form of the Verlet list and the cluster-pair mixed energy kernels, through the C ABI.

The cluster list must encode the half Verlet list exactly (every pair once, in one 64-bit mask),
and every kernel variant must give the FP64 energy within the mixed tolerance: total within 1e-6
relative of the FP64 engine (the reference's arithmetic), electrostatic and LJ parts within 1e-6
of the larger of the two.  Inputs with argon contacts at 1.65 A (the reference's argon_box
example) are checked at 2e-6: there (sigma/r)^12 multiplies the FP32 rounding of sigma/r twelvefold
and a few such pairs carry the whole energy.
"""
import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, native, systems
from mc_cpp_gb300.engine import FFieldCUDA

pytestmark = pytest.mark.gpu
KCAL = 418.4
MIX_REL = 1e-6
N_LIST_VARIANTS = 4
N_CLUSTER_END = 6          # variants 4 and 5 are the cluster-pair kernels


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _check_variants(s, ff, want, tol=MIX_REL):
    """Every variant against the FP64 energy; returns the energies by variant."""
    _, nv = ff.pair_kernel()
    assert nv > N_LIST_VARIANTS
    scale = max(1.0, abs(want[3]), abs(want[4]))
    got = {}
    for v in range(nv):
        try:
            ff.set_pair_kernel(v)
        except native.McgError as err:
            # the group-pair variants (tests/test_group_kernel_gpu.py) need the class table
            if v >= N_CLUSTER_END and err.code == native.MCG_ENOTSUP:
                continue
            raise
        e = ff.getE10()
        rel = abs(e[0] - want[0]) / max(1.0, abs(want[0]))
        assert rel <= tol, (v, rel, e[0], want[0])
        assert abs(e[3] - want[3]) <= tol * scale, (v, e[3], want[3])
        assert abs(e[4] - want[4]) <= tol * scale, (v, e[4], want[4])
        got[v] = e
    return got


@pytest.mark.parametrize("name", ["argon864", "water512", "water4096", "peptide", "water33334", "nma_solvated",
                                  "trhbn_solvated", "argon_box"])
def test_cluster_list_encodes_verlet_list_and_energies_agree(name):
    s = goldens.system(name, "switch")
    if s.pbc_type == "none":
        pytest.skip("cluster kernels cover periodic boxes")
    ff = FFieldCUDA(s, "mixed", moves=False)
    ncl, npairs, nbits = ff.cluster_stats()
    lp, _ = ff.pair_count()
    assert ncl >= (s.natom + 7) // 8 and npairs > 0
    assert nbits == lp, (nbits, lp)          # every Verlet pair in exactly one mask bit
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    _check_variants(s, ff, want, 2 * MIX_REL if name == "argon_box" else MIX_REL)


def test_cluster_energy_is_deterministic_and_tuner_picks_a_variant():
    s = goldens.system("water4096", "switch")
    ff = FFieldCUDA(s, "mixed", moves=False)
    e1 = ff.getE10()
    v, nv = ff.pair_kernel()
    assert 0 <= v < nv
    for var in range(N_LIST_VARIANTS, nv):
        ff.set_pair_kernel(var)
        a, b = ff.getE10(), ff.getE10()
        assert np.array_equal(a, b)          # fixed-order sums: bitwise repeatable
    assert np.isfinite(e1).all()


def test_cluster_kernels_follow_stale_lists_and_commits():
    """Moves committed without a list update: both kernels sum the stale Verlet list (pairs that
    came within rc but are not in it stay out), and agree with the FP64 engine on the same list."""
    s = goldens.system("water512", "switch")
    mix = FFieldCUDA(s, "mixed", moves=False)
    f64 = FFieldCUDA(s, "fp64", moves=False)
    rng = np.random.default_rng(5)
    xyz = s.coords()
    for t in range(40):
        res = int(rng.integers(0, s.natom // 3))
        idx = np.array([3 * res, 3 * res + 1, 3 * res + 2])
        new = xyz[idx] + rng.uniform(-0.6, 0.6, 3)
        for ff in (mix, f64):
            ff.delta_e(idx, new)
            ff.commit()
        xyz[idx] = new
    want = f64.getE10()
    _check_variants(s, mix, want)
    for ff in (mix, f64):
        ff.askListUpdate()
    ncl, npairs, nbits = mix.cluster_stats()
    assert nbits == mix.pair_count()[0]
    _check_variants(s, mix, f64.getE10())


@pytest.mark.parametrize("natom", [2, 3, 7, 9, 17])
def test_cluster_kernels_on_tiny_and_padded_systems(natom):
    s = systems.argon_random(natom, natom / 26.0 ** 3, natom)
    s.cut_mode = "switch"
    s.q = np.where(np.arange(natom) % 2 == 0, 0.5, -0.5)
    ff = FFieldCUDA(s, "mixed", moves=False)
    ncl, npairs, nbits = ff.cluster_stats()
    assert ncl >= 1 and nbits == ff.pair_count()[0]
    _check_variants(s, ff, FFieldCUDA(s, "fp64", moves=False).getE10())


def test_cluster_kernels_on_dense_region_and_orthorhombic_box():
    s = goldens.system("water512", "switch")
    xyz = s.coords()
    xyz[:600] *= 0.6           # a dense third of the box: long columns and long cluster rows
    s.set_coords(xyz)
    s.pbc_type = "orbic"
    s.box = (s.box[0], s.box[0] * 1.01, s.box[0] * 0.99)
    ff = FFieldCUDA(s, "mixed", moves=False)
    assert ff.cluster_stats()[2] == ff.pair_count()[0]
    _check_variants(s, ff, FFieldCUDA(s, "fp64", moves=False).getE10())


def test_cluster_kernels_follow_frozen_pairs():
    """Pairs of two frozen atoms are not in the Verlet list (List_nonBonded.cpp:867), so they are not
    in the masks either."""
    s = goldens.system("water512", "switch")
    s.frozen = np.zeros(s.natom, np.uint8)
    s.frozen[:600] = 1
    ff = FFieldCUDA(s, "mixed", moves=False)
    lp, _ = ff.pair_count()
    assert ff.cluster_stats()[2] == lp
    assert lp < FFieldCUDA(goldens.system("water512", "switch"), "mixed", moves=False).pair_count()[0]
    _check_variants(s, ff, FFieldCUDA(s, "fp64", moves=False).getE10())


def test_pair_kernel_selection_errors():
    s = goldens.system("water512", "switch")
    ff = FFieldCUDA(s, "fp64", moves=False)
    with pytest.raises(native.McgError):
        ff.set_pair_kernel(N_LIST_VARIANTS)      # FP64 systems have no cluster list
    assert ff.cluster_stats() == (0, 0, 0)
    mix = FFieldCUDA(s, "mixed", moves=False)
    with pytest.raises(native.McgError):
        mix.set_pair_kernel(99)
    mix.set_pair_kernel(-1)
