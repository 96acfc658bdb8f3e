"""Group-pair form of the pair kernel's rows and the group-pair energy kernels, through the C ABI.

Groups are runs of at most 4 consecutive atoms of one residue; every atom pair of the rows the
per-atom list kernels read (the pruned Verlet rows, or the whole rows with pruning off) is one bit
of one group pair's mask.  Checked:
  - the masks encode exactly the rows' pairs (their count equals the pruned entries, or the
    half-list size without pruning);
  - every group variant gives the per-atom list kernel's energy to the FP32 summation order
    (2e-7 of max(|E_elec|, |E_vdw|)) and the FP64 energy within the mixed tolerance (1e-6 of the
    total), on cubic, orthorhombic and argon (one-atom groups) boxes;
  - the group rows follow new pruned rows after displacements, commits and list updates;
  - repeated energies are bitwise equal (fixed-order sums);
  - a system without the parameter-class table has no group variants (MCG_ENOTSUP);
  - the packed variants (8, 9: partner atoms placed relative to the row group's first atom) agree
    on a box where half the box less rc lies between the water's smallest and largest hydrogen
    offsets, so some rows take the relative placement and the others the per-pair displacement.
"""
import copy

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, native, systems
from mc_cpp_gb300.engine import FFieldCUDA

pytestmark = pytest.mark.gpu
MIX_REL = 1e-6
ORDER_REL = 2e-7
GROUP_VARIANTS = (6, 7, 8, 9)
PACKED_VARIANTS = (8, 9)


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _agree(a, b, want, tag):
    scale = max(1.0, abs(b[3]), abs(b[4]))
    assert abs(a[3] - b[3]) <= ORDER_REL * scale, (tag, a[3], b[3])
    assert abs(a[4] - b[4]) <= ORDER_REL * scale, (tag, a[4], b[4])
    assert abs(a[0] - want[0]) <= MIX_REL * max(1.0, abs(want[0])), (tag, a[0], want[0])


def _orbic(s):
    t = copy.deepcopy(s)
    t.pbc_type = "orbic"
    t.box = (s.box[0], s.box[0] * 1.01, s.box[0] * 0.99)
    return t


@pytest.mark.parametrize("name", ["argon864", "water512", "water4096", "peptide", "water33334", "water4096_orbic"])
@pytest.mark.parametrize("prune", [True, False])
def test_group_rows_encode_the_rows_and_energies_agree(name, prune):
    s = goldens.system(name.replace("_orbic", ""), "switch")
    if name.endswith("_orbic"):
        s = _orbic(s)
    ff = FFieldCUDA(s, "mixed", moves=False)
    ref = FFieldCUDA(s, "mixed", moves=False)
    if not prune:
        ff.set_prune_buffer(0.0)
        ref.set_prune_buffer(0.0)
    ref.set_pair_kernel(0)
    base = ref.getE10()
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    ng, nent, nbits = ff.group_stats()
    rows = ref.prune_stats()[0] if prune else ref.pair_count()[0]
    assert nbits == rows, (nbits, rows)      # every row pair in exactly one mask bit
    assert ng >= s.natom // 4 and 0 < nent <= nbits
    for v in GROUP_VARIANTS:
        ff.set_pair_kernel(v)
        e = ff.getE10()
        _agree(e, base, want, (name, prune, v))
        assert np.array_equal(e, ff.getE10())


def test_group_rows_follow_moves_commits_and_list_updates():
    s = goldens.system("water4096", "switch")
    gr = FFieldCUDA(s, "mixed", moves=False)
    ref = FFieldCUDA(s, "mixed", moves=False)
    f64 = FFieldCUDA(s, "fp64", moves=False)
    gr.set_pair_kernel(GROUP_VARIANTS[0])
    ref.set_pair_kernel(0)
    _agree(gr.getE10(), ref.getE10(), f64.getE10(), "start")
    rng = np.random.default_rng(11)
    xyz = s.coords()
    d = rng.normal(size=xyz.shape)
    d *= 0.3 / np.linalg.norm(d, axis=1, keepdims=True)       # beyond half the prune buffer
    for ff in (gr, ref, f64):
        ff.setCoords(xyz + d)
    _agree(gr.getE10(), ref.getE10(), f64.getE10(), "after displacements")
    assert gr.group_stats()[2] == ref.prune_stats()[0]
    idx = np.array([300, 301, 302])
    new = (xyz + d)[idx] + np.array([0.0, 0.35, 0.0])
    for ff in (gr, ref, f64):
        ff.delta_e(idx, new)
        ff.commit()
    _agree(gr.getE10(), ref.getE10(), f64.getE10(), "after a commit")
    for ff in (gr, ref, f64):
        ff.askListUpdate()
    _agree(gr.getE10(), ref.getE10(), f64.getE10(), "after a list update")
    assert gr.group_stats()[2] == ref.prune_stats()[0]


def test_no_group_variants_without_the_class_table():
    s = copy.deepcopy(goldens.system("water4096", "switch"))
    rng = np.random.default_rng(3)
    s.q = np.asarray(s.q, np.float64) * (1.0 + 1e-3 * rng.uniform(-1.0, 1.0, s.natom))   # 12,288 classes
    ff = FFieldCUDA(s, "mixed", moves=False)
    with pytest.raises(native.McgError) as ei:
        ff.set_pair_kernel(GROUP_VARIANTS[0])
    assert ei.value.code == native.MCG_ENOTSUP
    assert ff.group_stats() == (0, 0, 0)
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    e = ff.getE10()                                    # the tuner skips the group variants
    assert abs(e[0] - want[0]) <= MIX_REL * abs(want[0])


def test_packed_variants_with_rows_on_both_placements():
    # L = 25.7 A: half the box less rc is 0.85 A, and the molecules' largest hydrogen offset
    # component from the oxygen lies between 0.6 and 0.96 A: 43% of the rows take the relative
    # placement, the others the per-pair displacement
    s = systems.water_box(550, seed=21, L=25.7)
    ref = FFieldCUDA(s, "mixed", moves=False)
    ref.set_pair_kernel(0)
    base = ref.getE10()
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    for prune in (True, False):
        ff = FFieldCUDA(s, "mixed", moves=False)
        if not prune:
            ff.set_prune_buffer(0.0)
        for v in PACKED_VARIANTS:
            ff.set_pair_kernel(v)
            e = ff.getE10()
            _agree(e, base, want, ("water550", prune, v))
            assert np.array_equal(e, ff.getE10())
