"""The mixed periodic switch pair kernel's row pruning and parameter classes, through the C ABI.

Pruning only shortens the rows the pair kernel walks; the pairs it sums must stay the Verlet
list's pairs within the cutoff.  So, for every per-atom list variant:
  - energies with pruning on (the default 0.5 A buffer) and off agree to the FP32 per-lane
    summation order: within 2e-7 of max(|E_elec|, |E_vdw|);
  - both agree with the FP64 engine (the reference's arithmetic) within the mixed tolerance,
    1e-6 relative on the total.
The pruned rows hold at least the pairs within the cutoff and fewer entries than the list.
Displacements below half the buffer keep the rows (no new prune); a displacement beyond it, by
set_coords or by a committed move, prunes again before the next energy.

Atom parameters reach the kernel from a shared-memory table of the system's distinct
(q, eps, sig) classes when there are at most 1024 of them, else by a per-atom gather; a system
with a distinct charge on every atom takes the second path and must meet the same tolerance.
"""
import copy

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, native
from mc_cpp_gb300.engine import FFieldCUDA

pytestmark = pytest.mark.gpu
MIX_REL = 1e-6
ORDER_REL = 2e-7
N_LIST_VARIANTS = 4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _agree(a, b, want, tag):
    scale = max(1.0, abs(b[3]), abs(b[4]))
    assert abs(a[3] - b[3]) <= ORDER_REL * scale, (tag, a[3], b[3])
    assert abs(a[4] - b[4]) <= ORDER_REL * scale, (tag, a[4], b[4])
    for e in (a, b):
        assert abs(e[0] - want[0]) <= MIX_REL * max(1.0, abs(want[0])), (tag, e[0], want[0])


@pytest.mark.parametrize("name", ["argon864", "water512", "water4096", "peptide", "water33334"])
def test_pruned_rows_keep_every_pair_within_cutoff(name):
    s = goldens.system(name, "switch")
    pr = FFieldCUDA(s, "mixed", moves=False)
    whole = FFieldCUDA(s, "mixed", moves=False)
    whole.set_prune_buffer(0.0)
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    for v in range(N_LIST_VARIANTS):
        pr.set_pair_kernel(v)
        whole.set_pair_kernel(v)
        _agree(pr.getE10(), whole.getE10(), want, (name, v))
    entries, prunes, ms = pr.prune_stats()
    list_pairs, in_cut = pr.pair_count()
    assert prunes == 1 and ms > 0.0
    assert in_cut <= entries < list_pairs, (in_cut, entries, list_pairs)
    assert whole.prune_stats() == (0, 0, 0.0)


def test_pruned_rows_follow_displacements_and_commits():
    s = goldens.system("water4096", "switch")
    pr = FFieldCUDA(s, "mixed", moves=False)
    whole = FFieldCUDA(s, "mixed", moves=False)
    whole.set_prune_buffer(0.0)
    f64 = FFieldCUDA(s, "fp64", moves=False)
    for ff in (pr, whole):
        ff.set_pair_kernel(0)
    _agree(pr.getE10(), whole.getE10(), f64.getE10(), "start")
    assert pr.prune_stats()[1] == 1

    # every atom 0.24 A in a random direction (below half the buffer): same rows, same pairs
    rng = np.random.default_rng(5)
    xyz = s.coords()
    d = rng.normal(size=xyz.shape)
    d *= 0.24 / np.linalg.norm(d, axis=1, keepdims=True)
    moved = xyz + d
    for ff in (pr, whole, f64):
        ff.setCoords(moved)
    _agree(pr.getE10(), whole.getE10(), f64.getE10(), "below half the buffer")
    assert pr.prune_stats()[1] == 1

    # one atom 0.3 A from its position at the prune: pruned again
    moved2 = moved.copy()
    moved2[7] = xyz[7] + np.array([0.3, 0.0, 0.0])
    for ff in (pr, whole, f64):
        ff.setCoords(moved2)
    _agree(pr.getE10(), whole.getE10(), f64.getE10(), "beyond half the buffer")
    assert pr.prune_stats()[1] == 2

    # a committed residue move of 0.3 A: pruned again before the next energy
    idx = np.array([30, 31, 32])
    new = moved2[idx] + np.array([0.0, 0.3, 0.0])
    des = []
    for ff in (pr, whole, f64):
        des.append(ff.delta_e(idx, new))
        ff.commit()
    _agree(pr.getE10(), whole.getE10(), f64.getE10(), "after a commit")
    assert pr.prune_stats()[1] == 3
    assert abs(des[0] - des[2]) <= 1e-4 * 418.4

    # a list update prunes again as well
    for ff in (pr, whole, f64):
        ff.askListUpdate()
    _agree(pr.getE10(), whole.getE10(), f64.getE10(), "after a list update")
    assert pr.prune_stats()[1] == 4


def test_prune_buffer_arguments():
    s = goldens.system("water512", "switch")
    ff = FFieldCUDA(s, "mixed", moves=False)
    L = native.lib()
    assert L.mcg_set_prune_buffer(ff.h, -1.0) == native.MCG_EINVAL
    assert L.mcg_set_prune_buffer(ff.h, float("nan")) == native.MCG_EINVAL
    f64 = FFieldCUDA(s, "fp64", moves=False)
    assert L.mcg_set_prune_buffer(f64.h, 0.5) == native.MCG_ENOTSUP
    assert L.mcg_set_prune_buffer(f64.h, 0.0) == native.MCG_OK


def test_per_atom_parameters_beyond_the_class_table():
    s = copy.deepcopy(goldens.system("water4096", "switch"))
    rng = np.random.default_rng(3)
    s.q = np.asarray(s.q, np.float64) * (1.0 + 1e-3 * rng.uniform(-1.0, 1.0, s.natom))   # 12,288 classes
    want = FFieldCUDA(s, "fp64", moves=False).getE10()
    ff = FFieldCUDA(s, "mixed", moves=False)
    whole = FFieldCUDA(s, "mixed", moves=False)
    whole.set_prune_buffer(0.0)
    for v in range(N_LIST_VARIANTS):
        ff.set_pair_kernel(v)
        whole.set_pair_kernel(v)
        _agree(ff.getE10(), whole.getE10(), want, ("per-atom", v))
