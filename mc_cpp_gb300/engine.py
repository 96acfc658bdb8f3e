"""Python mirror of the reference's FField interface, backed by libmcgpu.so.

``FFieldCUDA`` has the reference's method names (include/FField.hpp:52-153): ``getE()`` returns
the total energy in internal units, ``getE10()`` the ten components of ``getE(double ener[10])``,
``askListUpdate(step)`` rebuilds the Verlet list.  Like the reference's MC driver, callers may
change coordinates between calls; ``setCoords`` pushes them to the device.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import native
from .mdbas import System

KCALTOIU = 418.4


def selection(s: System, mv) -> np.ndarray:
    """Selection::select_main (src/Selection.cpp:73-160) for one MoveSpec."""
    n = s.natom
    if mv.sel_mode == "all":
        return np.ones(n, np.int32)
    if mv.sel_mode == "none":
        return np.zeros(n, np.int32)
    if mv.sel_mode == "residue_name":
        return np.array([1 if r == mv.sele else 0 for r in s.resname], np.int32)
    if mv.sel_mode == "residue_id":
        return (np.asarray(s.resid) == int(mv.sele)).astype(np.int32)
    if mv.sel_mode == "atom_idx":
        return (np.arange(1, n + 1) == int(mv.sele)).astype(np.int32)
    raise ValueError("unknown sel_mode %r" % mv.sel_mode)


class FFieldCUDA:
    """One system on the device (FField_MDBAS + List_nonBonded semantics)."""

    def __init__(self, system: System, precision: str = "fp64", moves: bool = True):
        L = native.lib()
        self.s = system
        self.n = system.natom
        self.precision = precision
        desc, keep = native.make_desc(system, precision)
        h = C.c_void_p()
        native.check(L.mcg_create(C.byref(desc), C.byref(h)))
        self.h = h
        self.nmoves = 0
        if moves:
            for mv in system.moves:
                self.add_move(mv)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            native.lib().mcg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- FField interface
    def getE(self) -> float:
        return float(self.getE10()[0])

    def getE10(self) -> np.ndarray:
        e = np.zeros(10)
        native.check(native.lib().mcg_energy(self.h, native.pd(e)))
        return e

    def getE_host(self, x, y, z) -> float:
        """FField::getE() on caller-owned coordinate arrays (float64, natom each) that the caller
        moves in place between calls, as MC_metropolis does; only what changed is sent to the device
        (mcg_energy_host)."""
        e = C.c_double(0)
        native.check(native.lib().mcg_energy_host(self.h, native.pd(x), native.pd(y), native.pd(z), C.byref(e)))
        return e.value

    def askListUpdate(self, step: int = 0) -> None:
        native.check(native.lib().mcg_update_lists(self.h))

    # ---- coordinates and moves
    def setCoords(self, xyz) -> None:
        xyz = np.asarray(xyz, np.float64)
        x, y, z = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
        native.check(native.lib().mcg_set_coords(self.h, native.pd(x), native.pd(y), native.pd(z)))

    def coords(self) -> np.ndarray:
        x, y, z = (np.zeros(self.n) for _ in range(3))
        native.check(native.lib().mcg_get_coords(self.h, native.pd(x), native.pd(y), native.pd(z)))
        return np.stack([x, y, z], 1)

    def delta_e(self, atoms, new_xyz) -> float:
        atoms = np.ascontiguousarray(atoms, np.int32)
        new_xyz = np.asarray(new_xyz, np.float64)
        x, y, z = (np.ascontiguousarray(new_xyz[:, k]) for k in range(3))
        de = np.zeros(1)
        native.check(native.lib().mcg_delta_e(self.h, len(atoms), native.pi(atoms), native.pd(x), native.pd(y),
                                              native.pd(z), native.pd(de)))
        return float(de[0])

    def time_nonbonded(self, reps: int) -> float:
        """Device ms of reps launches of the switched pair kernel alone."""
        ms = C.c_float(0)
        native.check(native.lib().mcg_time_nonbonded(self.h, reps, C.byref(ms)))
        return ms.value

    def kernel_launches(self) -> int:
        """Kernel launches issued by this handle so far."""
        v = C.c_int64(0)
        native.check(native.lib().mcg_kernel_launches(self.h, C.byref(v)))
        return v.value

    def time_nonbonded_flushed(self, reps: int) -> float:
        """Device ms of reps launches of the switched pair kernel, the L2 cache flushed before each."""
        ms = C.c_float(0)
        native.check(native.lib().mcg_time_nonbonded_flushed(self.h, reps, C.byref(ms)))
        return ms.value

    def set_pair_kernel(self, variant: int) -> None:
        """Pins the mixed periodic switch-energy kernel (-1: fastest by timing at the first use;
        0..3 per-atom list kernels; 4, 5 cluster-pair kernels; 6..9 group-pair kernels)."""
        native.check(native.lib().mcg_set_pair_kernel(self.h, variant))

    def pair_kernel(self):
        """(variant in use or -1, number of variants)."""
        v, n = C.c_int(0), C.c_int(0)
        native.check(native.lib().mcg_get_pair_kernel(self.h, C.byref(v), C.byref(n)))
        return v.value, n.value

    def cluster_stats(self):
        """(clusters, cluster pairs, Verlet pairs in the masks) of the cluster form of the list."""
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        native.check(native.lib().mcg_cluster_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def group_stats(self):
        """(groups, group pairs, atom pairs in their masks) of the group form of the rows."""
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        native.check(native.lib().mcg_group_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_prune_buffer(self, buffer: float) -> None:
        """Prune buffer (A) of the rows the mixed periodic switch energy reads; 0 = whole list."""
        native.check(native.lib().mcg_set_prune_buffer(self.h, float(buffer)))

    def prune_stats(self):
        """(entries of the pruned rows, prunes so far, last prune's device time in ms)."""
        a, b, t = C.c_int64(0), C.c_int64(0), C.c_float(0)
        native.check(native.lib().mcg_prune_stats(self.h, C.byref(a), C.byref(b), C.byref(t)))
        return a.value, b.value, t.value

    def pair_count(self):
        """(list pairs, pairs within the cutoff at the current coordinates)."""
        a, b = C.c_int64(0), C.c_int64(0)
        native.check(native.lib().mcg_pair_count(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def commit(self) -> None:
        native.check(native.lib().mcg_commit(self.h))

    def pairlist(self):
        """Half Verlet rows (j > i, sorted), as a list of arrays."""
        counts = np.zeros(self.n, np.int32)
        total = C.c_int64(0)
        native.check(native.lib().mcg_get_pairlist(self.h, native.pi(counts), None, 0, C.byref(total)))
        ent = np.zeros(max(1, total.value), np.int32)
        native.check(native.lib().mcg_get_pairlist(self.h, native.pi(counts), native.pi(ent), total.value, C.byref(total)))
        return np.split(ent[:total.value], np.cumsum(counts)[:-1])

    def exclusions(self):
        counts = np.zeros(self.n, np.int32)
        total = C.c_int64(0)
        native.check(native.lib().mcg_get_exclusions(self.h, native.pi(counts), None, 0, C.byref(total)))
        ent = np.zeros(max(1, total.value), np.int32)
        native.check(native.lib().mcg_get_exclusions(self.h, native.pi(counts), native.pi(ent), total.value, C.byref(total)))
        return np.split(ent[:total.value], np.cumsum(counts)[:-1])

    def pairs14(self) -> np.ndarray:
        n = C.c_int(0)
        native.check(native.lib().mcg_get_pairs14(self.h, None, 0, C.byref(n)))
        buf = np.zeros(max(2, 2 * n.value), np.int32)
        native.check(native.lib().mcg_get_pairs14(self.h, native.pi(buf), len(buf), C.byref(n)))
        return buf[:2 * n.value].reshape(-1, 2)

    def add_move(self, mv) -> int:
        sel = selection(self.s, mv)
        r = native.check(native.lib().mcg_add_move(self.h, native.MVTYPE[mv.move_type], native.MVMODE[mv.move_mode],
                                                   native.pi(sel), mv.dmax_value, mv.dmax_target, mv.dmax_each))
        self.nmoves += 1
        return r

    def metropolis(self, nsteps: int, seed: int, acceptance: str = "reference", trace: bool = True, follow=None):
        """MC_metropolis::run on this engine; returns (trace[nsteps,12], final_etot, n_accepted, n_ties)."""
        tr = np.zeros((max(1, nsteps), 12))
        fe = C.c_double(0)
        na = C.c_int64(0)
        nt = C.c_int64(0)
        fol = None
        if follow is not None:
            fol = np.ascontiguousarray(follow, np.int32).reshape(-1)
        native.check(native.lib().mcg_metropolis_run(self.h, nsteps, seed, native.ACCEPT[acceptance],
                                                     native.pd(tr) if trace else None,
                                                     native.pi(fol) if fol is not None else None,
                                                     C.byref(fe), C.byref(na), C.byref(nt)))
        return tr[:nsteps], fe.value, na.value, nt.value


    def metropolis_saving(self, nsteps: int, seed: int, save_each: int, acceptance: str = "reference"):
        """MC_metropolis::run with its outputs: (frames[nsave, natom, 3], energies[nsave] (iu),
        final_etot, n_accepted), one frame and energy after every save_each-th step."""
        nsave = nsteps // save_each if save_each > 0 else 0
        frames = np.zeros((max(1, nsave), self.n, 3))
        energies = np.zeros(max(1, nsave))
        fe = C.c_double(0)
        na = C.c_int64(0)
        native.check(native.lib().mcg_metropolis_run_saving(self.h, nsteps, seed, native.ACCEPT[acceptance], save_each,
                                                            native.pd(frames), native.pd(energies), C.byref(fe),
                                                            C.byref(na)))
        return frames[:nsave], energies[:nsave], fe.value, na.value


class BatchChains:
    """Hundreds of independent NVT chains advanced by one persistent kernel per sweep."""

    def __init__(self, chains, dmax_trn: float = 0.15, dmax_rot: float = 15.0, acceptance: str = "physical",
                 seed: int = 1, threads_per_chain: int = 0, list_capacity: int = 0, ctas_per_sm: int = 0,
                 speculation: int = 0, clusters: int = 0, dmax_each=(0, 0), dmax_target=(50.0, 50.0),
                 dmax_max=(0.0, 0.0)):
        L = native.lib()
        self.nchains = len(chains)
        arr = (native.SystemDesc * self.nchains)()
        self._keep = []
        for k, s in enumerate(chains):
            d, keep = native.make_desc(s, "mixed")
            arr[k] = d
            self._keep.append(keep)
        opts = native.BatchOpts(dmax_trn, dmax_rot, native.ACCEPT[acceptance], threads_per_chain, list_capacity, seed,
                                ctas_per_sm, speculation, clusters, (C.c_int * 2)(*dmax_each),
                                (C.c_double * 2)(*dmax_target), (C.c_double * 2)(*dmax_max))
        h = C.c_void_p()
        native.check(L.mcg_batch_create(arr, self.nchains, C.byref(opts), C.byref(h)))
        self.h = h
        self.natoms = int(L.mcg_batch_natoms(h))
        self.sizes = np.array([L.mcg_batch_chain_natoms(h, k) for k in range(self.nchains)])
        # atoms per residue of each chain (rigid residues of one size per chain)
        self._apr_of = [int(np.count_nonzero(s.resid == s.resid[0])) for s in chains]

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            native.lib().mcg_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sweep(self, n: int = 1) -> None:
        native.check(native.lib().mcg_batch_sweep(self.h, n))

    def sweep_logged(self):
        """One sweep with per-move records: a list with, for each chain, its moves of this sweep in
        order (structured array of native.MOVE_DTYPE)."""
        nres = [int(n) // a for n, a in zip(self.sizes, self._apr_of)]
        rec = np.zeros(sum(nres), native.MOVE_DTYPE)
        native.check(native.lib().mcg_batch_sweep_logged(self.h, rec.ctypes.data, len(rec)))
        return np.split(rec, np.cumsum(nres)[:-1])

    def save(self, path: str) -> None:
        """Exact checkpoint of every chain (mcg_batch_save)."""
        native.check(native.lib().mcg_batch_save(self.h, os.fsencode(path)))

    def load(self, path: str) -> None:
        """Restores a checkpoint of a batch made from the same chains and options (mcg_batch_load)."""
        native.check(native.lib().mcg_batch_load(self.h, os.fsencode(path)))

    def time_sweeps(self, n: int) -> float:
        ms = C.c_float(0)
        native.check(native.lib().mcg_batch_time_sweeps(self.h, n, C.byref(ms)))
        return ms.value

    def time_phases(self, n: int):
        """Device ms of n sweeps: (total, list rebuilds, sweep kernel alone)."""
        a, b, c = C.c_float(0), C.c_float(0), C.c_float(0)
        native.check(native.lib().mcg_batch_time_phases(self.h, n, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, trial_sweeps: int = 2, use_cache: bool = True) -> dict:
        """Times every candidate launch shape on trial_sweeps real sweeps and keeps the fastest."""
        t = native.BatchTuning()
        native.check(native.lib().mcg_batch_autotune(self.h, trial_sweeps, int(use_cache), C.byref(t)))
        return {"threads_per_chain": t.threads_per_chain, "ctas_per_sm": t.ctas_per_sm, "speculation": t.speculation,
                "clusters": t.clusters, "ms_per_sweep": t.ms_per_sweep, "from_cache": bool(t.from_cache)}

    def tuning(self) -> dict:
        t = native.BatchTuning()
        native.check(native.lib().mcg_batch_get_tuning(self.h, C.byref(t)))
        return {"threads_per_chain": t.threads_per_chain, "ctas_per_sm": t.ctas_per_sm, "speculation": t.speculation,
                "clusters": t.clusters}

    def stats(self):
        t = np.zeros(self.nchains, np.int64)
        a = np.zeros(self.nchains, np.int64)
        e = np.zeros(self.nchains)
        native.check(native.lib().mcg_batch_stats(self.h, t.ctypes.data_as(native._i64), a.ctypes.data_as(native._i64),
                                                  native.pd(e)))
        return t, a, e

    def pairs(self) -> np.ndarray:
        p = np.zeros(self.nchains, np.int64)
        native.check(native.lib().mcg_batch_pairs(self.h, p.ctypes.data_as(native._i64)))
        return p

    def lists(self, chain: int):
        """The chain's residue neighbour lists as they are now (one array per residue)."""
        nres = int(self.sizes[chain]) // self._apr(chain)
        counts = np.zeros(nres, np.int32)
        total = C.c_int64(0)
        L = native.lib()
        native.check(L.mcg_batch_get_lists(self.h, chain, native.pi(counts), None, 0, C.byref(total)))
        ent = np.zeros(max(1, total.value), np.int32)
        native.check(L.mcg_batch_get_lists(self.h, chain, native.pi(counts), native.pi(ent), total.value, C.byref(total)))
        return np.split(ent[:total.value], np.cumsum(counts)[:-1])

    def _apr(self, chain: int) -> int:
        return self._apr_of[chain]

    def update_lists(self) -> None:
        native.check(native.lib().mcg_batch_update_lists(self.h))

    def energy_fp64(self) -> np.ndarray:
        e = np.zeros(self.nchains)
        native.check(native.lib().mcg_batch_energy_fp64(self.h, native.pd(e)))
        return e

    def energy_mixed(self) -> np.ndarray:
        e = np.zeros(self.nchains)
        native.check(native.lib().mcg_batch_energy_mixed(self.h, native.pd(e)))
        return e

    def coords(self, chain: int) -> np.ndarray:
        n = int(self.sizes[chain])
        x, y, z = (np.zeros(n) for _ in range(3))
        native.check(native.lib().mcg_batch_get_coords(self.h, chain, native.pd(x), native.pd(y), native.pd(z)))
        return np.stack([x, y, z], 1)

    def set_coords(self, chain: int, xyz) -> None:
        xyz = np.asarray(xyz, np.float64)
        x, y, z = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
        native.check(native.lib().mcg_batch_set_coords(self.h, chain, native.pd(x), native.pd(y), native.pd(z)))

    def run_host(self, xyz_in, nsweeps: int, xyz_out):
        """Host-buffer run: xyz_in/xyz_out are (3, natoms) float64 arrays (pinned for speed) or None."""
        a = np.zeros(self.nchains, np.int64)
        e = np.zeros(self.nchains)
        native.check(native.lib().mcg_batch_run_host(self.h, native.pd(xyz_in) if xyz_in is not None else None, nsweeps,
                                                     native.pd(xyz_out) if xyz_out is not None else None,
                                                     a.ctypes.data_as(native._i64), native.pd(e)))
        return a, e

    def dmax(self):
        """Current (translation A, rotation degrees) dmax of every chain."""
        t = np.zeros(self.nchains)
        r = np.zeros(self.nchains)
        native.check(native.lib().mcg_batch_get_dmax(self.h, native.pd(t), native.pd(r)))
        return t, r

    def counters(self):
        rb = C.c_int64(0)
        nl = C.c_int64(0)
        native.check(native.lib().mcg_batch_counters(self.h, C.byref(rb), C.byref(nl)))
        return rb.value, nl.value
