"""ctypes binding of the CPU restatement in oracle/mc_oracle.cpp.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
legs, never by the mc_cpp_gb300 package.  ``Oracle(system)`` mirrors the reference's object graph
(AtomList + FField_MDBAS + List_nonBonded + List_Moves) for one system.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmc_oracle.so")
_lib = None

PBC = {"none": 0, "cubic": 1, "orbic": 2}
CUT = {"full": 0, "switch": 1}
MVTYPE = {"trn": 1, "rot": 2}
MVMODE = {"residue": 0, "all": 1, "atom": 2}

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)


def build() -> str:
    subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                 C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_atoms.argtypes = [C.c_void_p] + [_d] * 9 + [C.POINTER(C.c_ubyte), _i]
        L.orc_set_coords.argtypes = [C.c_void_p, _d, _d, _d]
        L.orc_get_coords.argtypes = [C.c_void_p, _d, _d, _d]
        L.orc_set_bonds.argtypes = [C.c_void_p, C.c_int, _i, _i, _d, _d, _d]
        L.orc_set_ub.argtypes = [C.c_void_p, C.c_int, _i, _d, _d]
        L.orc_set_angles.argtypes = [C.c_void_p, C.c_int, _i, _i, _d, _d]
        L.orc_set_dihedrals.argtypes = [C.c_void_p, C.c_int, _i, _i, _i, _d, _d, _d]
        L.orc_set_impropers.argtypes = [C.c_void_p, C.c_int, _i, _i, _i, _d, _d, _d]
        L.orc_build_lists.argtypes = [C.c_void_p]
        L.orc_update_verlet.argtypes = [C.c_void_p]
        L.orc_energy.restype = C.c_double
        L.orc_energy.argtypes = [C.c_void_p, _d]
        for f in (L.orc_excl_row, L.orc_verlet_row):
            f.restype = C.c_int
            f.argtypes = [C.c_void_p, C.c_int, _i, C.c_int]
        L.orc_pairs14.restype = C.c_int
        L.orc_pairs14.argtypes = [C.c_void_p, _i, C.c_int]
        L.orc_verlet_total.restype = C.c_longlong
        L.orc_verlet_total.argtypes = [C.c_void_p]
        L.orc_pairs_in_cutoff.restype = C.c_longlong
        L.orc_pairs_in_cutoff.argtypes = [C.c_void_p]
        L.orc_add_move.restype = C.c_int
        L.orc_add_move.argtypes = [C.c_void_p, C.c_int, C.c_int, _i, C.c_double, C.c_double, C.c_int]
        L.orc_move_instances.restype = C.c_int
        L.orc_move_instances.argtypes = [C.c_void_p, C.c_int]
        L.orc_move_instance.restype = C.c_int
        L.orc_move_instance.argtypes = [C.c_void_p, C.c_int, C.c_int, _i, C.c_int, _i]
        L.orc_mc_run.restype = C.c_int
        L.orc_mc_run.argtypes = [C.c_void_p, C.c_int, C.c_ulonglong, _d, _d, C.POINTER(C.c_longlong)]
        L.orc_set_acceptance_units.argtypes = [C.c_void_p, C.c_int]
        L.orc_delta_e.restype = C.c_double
        L.orc_delta_e.argtypes = [C.c_void_p, C.c_int, _i, _d, _d, _d]
        # batched chain restatement (batch_oracle.cpp)
        L.orcb_create.restype = C.c_void_p
        L.orcb_create.argtypes = [C.c_int, C.c_int, _d, _d, _d, _d, C.c_double, C.c_double, C.c_double, C.c_int,
                                  C.c_uint64, C.c_int, _d, _i, _d, _d]
        L.orcb_destroy.argtypes = [C.c_void_p]
        L.orcb_set_coords.argtypes = [C.c_void_p, _d, _d, _d]
        L.orcb_get_coords.argtypes = [C.c_void_p, _d, _d, _d]
        L.orcb_set_moves.argtypes = [C.c_void_p, C.c_uint64]
        L.orcb_get_dmax.argtypes = [C.c_void_p, _d]
        L.orcb_energy.restype = C.c_double
        L.orcb_energy.argtypes = [C.c_void_p]
        L.orcb_follow.argtypes = [C.c_void_p, C.c_int, C.c_void_p, _d]
        L.orcb_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _pd(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_d)


def _pi(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(_i)


def selection(system, mv) -> np.ndarray:
    """Selection::select_main (src/Selection.cpp:73-160) for one MoveSpec."""
    n = system.natom
    s = np.zeros(n, np.int32)
    if mv.sel_mode == "all":
        s[:] = 1
    elif mv.sel_mode == "residue_name":
        s[:] = [1 if r == mv.sele else 0 for r in system.resname]
    elif mv.sel_mode == "residue_id":
        s[:] = (system.resid == int(mv.sele)).astype(np.int32)
    elif mv.sel_mode == "atom_idx":
        s[:] = (np.arange(1, n + 1) == int(mv.sele)).astype(np.int32)
    return s


class Oracle:
    """One system on the CPU restatement."""

    def __init__(self, s, build_lists: bool = True, moves: bool = True):
        L = lib()
        self.s = s
        self.n = s.natom
        a, b, c = s.box
        self.h = L.orc_create(s.natom, PBC[s.pbc_type], a, b, c, CUT[s.cut_mode], s.cutoff, s.cuton, s.dcut, s.temp)
        self._keep = []
        L.orc_set_atoms(self.h, _pd(s.x), _pd(s.y), _pd(s.z), _pd(s.q), _pd(s.eps), _pd(s.sig), _pd(s.eps14),
                        _pd(s.sig14), _pd(s.mass), np.ascontiguousarray(s.frozen, np.uint8).ctypes.data_as(C.POINTER(C.c_ubyte)),
                        _pi(s.resid))
        if len(s.bonds):
            L.orc_set_bonds(self.h, len(s.bonds), _pi(s.bonds), _pi(s.bond_type), _pd(s.bond_k), _pd(s.bond_r0), _pd(s.bond_beta))
        if len(s.ub):
            L.orc_set_ub(self.h, len(s.ub), _pi(s.ub), _pd(s.ub_k), _pd(s.ub_r0))
        if len(s.angles):
            L.orc_set_angles(self.h, len(s.angles), _pi(s.angles), _pi(s.angle_type), _pd(s.angle_k), _pd(s.angle_theta0))
        if len(s.dihedrals):
            L.orc_set_dihedrals(self.h, len(s.dihedrals), _pi(s.dihedrals), _pi(s.dihe_type), _pi(s.dihe_order),
                                _pd(s.dihe_k), _pd(s.dihe_phi0), _pd(s.dihe_mult))
        if len(s.impropers):
            L.orc_set_impropers(self.h, len(s.impropers), _pi(s.impropers), _pi(s.impr_type), _pi(s.impr_order),
                                _pd(s.impr_k), _pd(s.impr_phi0), _pd(s.impr_mult))
        if build_lists:
            L.orc_build_lists(self.h)
        if moves:
            for mv in s.moves:
                sel = selection(s, mv)
                L.orc_add_move(self.h, MVTYPE[mv.move_type], MVMODE[mv.move_mode], _pi(sel), mv.dmax_value,
                               mv.dmax_target, mv.dmax_each)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def energy(self) -> np.ndarray:
        e = np.zeros(10)
        lib().orc_energy(self.h, e.ctypes.data_as(_d))
        return e

    def set_coords(self, xyz):
        xyz = np.asarray(xyz, np.float64)
        lib().orc_set_coords(self.h, _pd(xyz[:, 0]), _pd(xyz[:, 1]), _pd(xyz[:, 2]))

    def coords(self) -> np.ndarray:
        x, y, z = (np.zeros(self.n) for _ in range(3))
        lib().orc_get_coords(self.h, x.ctypes.data_as(_d), y.ctypes.data_as(_d), z.ctypes.data_as(_d))
        return np.stack([x, y, z], 1)

    def update_verlet(self):
        lib().orc_update_verlet(self.h)

    def excl_rows(self):
        buf = np.zeros(4096, np.int32)
        rows = []
        for i in range(self.n):
            c = lib().orc_excl_row(self.h, i, buf.ctypes.data_as(_i), len(buf))
            rows.append(buf[:c].copy())
        return rows

    def pairs14(self) -> np.ndarray:
        n = lib().orc_pairs14(self.h, None, 0)
        buf = np.zeros(max(1, 2 * n), np.int32)
        lib().orc_pairs14(self.h, buf.ctypes.data_as(_i), len(buf))
        return buf[:2 * n].reshape(-1, 2)

    def verlet_rows(self):
        buf = np.zeros(1 << 16, np.int32)
        rows = []
        for i in range(self.n):
            c = lib().orc_verlet_row(self.h, i, buf.ctypes.data_as(_i), len(buf))
            rows.append(buf[:c].copy())
        return rows

    def verlet_total(self) -> int:
        return int(lib().orc_verlet_total(self.h))

    def pairs_in_cutoff(self) -> int:
        return int(lib().orc_pairs_in_cutoff(self.h))

    def move_instances(self, t):
        out = []
        buf = np.zeros(4096, np.int32)
        piv = C.c_int(0)
        for k in range(lib().orc_move_instances(self.h, t)):
            nr = lib().orc_move_instance(self.h, t, k, buf.ctypes.data_as(_i), len(buf), C.byref(piv))
            out.append((buf[:2 * nr].reshape(-1, 2).copy(), piv.value))
        return out

    def set_acceptance_units(self, units: str):
        lib().orc_set_acceptance_units(self.h, {"reference": 0, "physical": 1}[units])

    def mc_run(self, nsteps: int, seed: int, trace: bool = True):
        tr = np.zeros((nsteps, 12)) if trace else None
        fe = C.c_double(0)
        na = C.c_longlong(0)
        rc = lib().orc_mc_run(self.h, nsteps, seed, tr.ctypes.data_as(_d) if trace else None, C.byref(fe), C.byref(na))
        if rc != 0:
            raise RuntimeError("orc_mc_run failed: %d" % rc)
        return tr, fe.value, na.value

    def delta_e(self, idx, new_xyz) -> float:
        idx = np.ascontiguousarray(idx, np.int32)
        new_xyz = np.asarray(new_xyz, np.float64)
        return lib().orc_delta_e(self.h, len(idx), _pi(idx), _pd(new_xyz[:, 0]), _pd(new_xyz[:, 1]), _pd(new_xyz[:, 2]))


def philox4x32_10(ctr, key) -> tuple:
    """One block of the batched engine's random stream, from the restatement."""
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orcb_philox(c.ctypes.data, k.ctypes.data, o.ctypes.data)
    return tuple(int(v) for v in o)


class BatchChainOracle:
    """One batched chain (rigid residues of apr atoms, periodic box) on the FP64 restatement of
    the batched sweep's moves (batch_oracle.cpp), with the batch's Philox key (seed, chain)."""

    FIELDS = ("match", "pos_err", "de64", "acc64", "acc_rule", "alpha", "thr64", "alpha_match")

    def __init__(self, s, chain: int, seed: int, dmax=(0.15, 15.0), each=(0, 0), target=(50.0, 50.0), cap=None,
                 acceptance: str = "physical"):
        apr = int(np.count_nonzero(s.resid == s.resid[0]))
        box = np.array(s.box if s.pbc_type == "orbic" else (s.box[0],) * 3, np.float64)
        if cap is None:
            cap = tuple(2.0 * d if e > 0 else d for d, e in zip(dmax, each))
        self._arrays = [box, np.asarray(dmax, np.float64), np.asarray(each, np.int32), np.asarray(target, np.float64),
                        np.asarray(cap, np.float64)]
        self.n = s.natom
        self.h = lib().orcb_create(s.natom, apr, _pd(box), _pd(s.q), _pd(s.eps), _pd(s.sig), s.cutoff, s.cuton, s.temp,
                                   {"reference": 0, "physical": 1}[acceptance], seed, chain,
                                   _pd(self._arrays[1]), _pi(self._arrays[2]), _pd(self._arrays[3]),
                                   _pd(self._arrays[4]))
        if not self.h:
            raise ValueError("invalid batched chain")
        self.set_coords(s.coords())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orcb_destroy(self.h)
            self.h = None

    def set_coords(self, xyz):
        xyz = np.asarray(xyz, np.float64)
        lib().orcb_set_coords(self.h, _pd(xyz[:, 0]), _pd(xyz[:, 1]), _pd(xyz[:, 2]))

    def coords(self) -> np.ndarray:
        x, y, z = (np.zeros(self.n) for _ in range(3))
        lib().orcb_get_coords(self.h, x.ctypes.data_as(_d), y.ctypes.data_as(_d), z.ctypes.data_as(_d))
        return np.stack([x, y, z], 1)

    def set_moves(self, moves: int):
        lib().orcb_set_moves(self.h, int(moves))

    def dmax(self):
        d = np.zeros(2)
        lib().orcb_get_dmax(self.h, d.ctypes.data_as(_d))
        return d

    def energy(self) -> float:
        return float(lib().orcb_energy(self.h))

    def follow(self, records) -> dict:
        """Checks and follows a chain's records of one logged sweep (structured array of
        struct mcg_batch_move); returns per-move arrays named by FIELDS."""
        rec = np.ascontiguousarray(records)
        assert rec.dtype.itemsize == 216
        out = np.zeros((len(rec), 8))
        lib().orcb_follow(self.h, len(rec), rec.ctypes.data, out.ctypes.data_as(_d))
        return {k: out[:, i] for i, k in enumerate(self.FIELDS)}
