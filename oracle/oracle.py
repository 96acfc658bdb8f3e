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
