"""ctypes binding of libmcgpu.so (the C ABI declared in include/mcg.h).

The library is built in-tree by mc_cpp_gb300.build.  Loading fails loudly when it is missing or
when a declared symbol is absent: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmcgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "mcg.h")

MCG_OK, MCG_EINVAL, MCG_ECUDA, MCG_ECAPACITY, MCG_ETIMEOUT, MCG_ENOTSUP, MCG_EIO = 0, -1, -2, -3, -4, -5, -6
STATUS_NAMES = {0: "MCG_OK", -1: "MCG_EINVAL", -2: "MCG_ECUDA", -3: "MCG_ECAPACITY", -4: "MCG_ETIMEOUT",
                -5: "MCG_ENOTSUP", -6: "MCG_EIO"}
PBC = {"none": 0, "cubic": 1, "orbic": 2}
CUT = {"full": 0, "switch": 1}
PREC = {"fp64": 0, "mixed": 1}
MVTYPE = {"trn": 1, "rot": 2}
MVMODE = {"residue": 0, "all": 1, "atom": 2}
ACCEPT = {"reference": 0, "physical": 1}

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)
_i64 = C.POINTER(C.c_int64)


class McgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(code, "?"), code, msg))
        self.code = code


class SystemDesc(C.Structure):
    _fields_ = [
        ("natom", C.c_int),
        ("x", _d), ("y", _d), ("z", _d), ("q", _d),
        ("eps", _d), ("sig", _d), ("eps14", _d), ("sig14", _d),
        ("mass", _d), ("frozen", C.POINTER(C.c_ubyte)), ("resid", _i),
        ("pbc_type", C.c_int), ("box", C.c_double * 3),
        ("cut_mode", C.c_int), ("cutoff", C.c_double), ("cuton", C.c_double), ("dcut", C.c_double),
        ("temp", C.c_double), ("precision", C.c_int),
        ("nbond", C.c_int), ("bond_atoms", _i), ("bond_type", _i), ("bond_k", _d), ("bond_r0", _d), ("bond_beta", _d),
        ("nub", C.c_int), ("ub_atoms", _i), ("ub_k", _d), ("ub_r0", _d),
        ("nangle", C.c_int), ("angle_atoms", _i), ("angle_type", _i), ("angle_k", _d), ("angle_theta0", _d),
        ("ndihe", C.c_int), ("dihe_atoms", _i), ("dihe_type", _i), ("dihe_order", _i), ("dihe_k", _d),
        ("dihe_phi0", _d), ("dihe_mult", _d),
        ("nimpr", C.c_int), ("impr_atoms", _i), ("impr_type", _i), ("impr_order", _i), ("impr_k", _d),
        ("impr_phi0", _d), ("impr_mult", _d),
        ("param_units", C.c_int),
    ]


class BatchOpts(C.Structure):
    _fields_ = [("dmax_trn", C.c_double), ("dmax_rot", C.c_double), ("acceptance_units", C.c_int),
                ("threads_per_chain", C.c_int), ("list_capacity", C.c_int), ("seed", C.c_uint64),
                ("ctas_per_sm", C.c_int), ("speculation", C.c_int), ("clusters", C.c_int),
                ("dmax_each", C.c_int * 2), ("dmax_target", C.c_double * 2), ("dmax_max", C.c_double * 2)]


class BatchTuning(C.Structure):
    _fields_ = [("threads_per_chain", C.c_int), ("ctas_per_sm", C.c_int), ("speculation", C.c_int),
                ("ms_per_sweep", C.c_float), ("from_cache", C.c_int), ("clusters", C.c_int)]


# one record of a logged sweep (struct mcg_batch_move)
MOVE_DTYPE = np.dtype([("de", np.float64), ("residue", np.int32), ("flags", np.int32), ("alpha_hi", np.uint32),
                       ("alpha_lo", np.uint32), ("xyz", np.float64, (8, 3))], align=True)
assert MOVE_DTYPE.itemsize == 216

_lib = None


def declared_symbols():
    """Function names declared in include/mcg.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mcg_[a-z0-9_]+)\s*\(", txt)))


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libmcgpu.so is not built (%s): run mc_cpp_gb300.build.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    if missing:
        raise RuntimeError("libmcgpu.so lacks declared symbols: %s" % missing)
    P = C.c_void_p
    sig = {
        "mcg_abi_version": (C.c_int, []),
        "mcg_last_error": (C.c_char_p, []),
        "mcg_device_count": (C.c_int, []),
        "mcg_create": (C.c_int, [C.POINTER(SystemDesc), C.POINTER(P)]),
        "mcg_destroy": (C.c_int, [P]),
        "mcg_set_coords": (C.c_int, [P, _d, _d, _d]),
        "mcg_get_coords": (C.c_int, [P, _d, _d, _d]),
        "mcg_energy": (C.c_int, [P, _d]),
        "mcg_energy_host": (C.c_int, [P, _d, _d, _d, _d]),
        "mcg_update_lists": (C.c_int, [P]),
        "mcg_delta_e": (C.c_int, [P, C.c_int, _i, _d, _d, _d, _d]),
        "mcg_commit": (C.c_int, [P]),
        "mcg_get_pairlist": (C.c_int, [P, _i, _i, C.c_int64, _i64]),
        "mcg_get_exclusions": (C.c_int, [P, _i, _i, C.c_int64, _i64]),
        "mcg_get_pairs14": (C.c_int, [P, _i, C.c_int, _i]),
        "mcg_build_exclusions": (C.c_int, [C.POINTER(SystemDesc), _i, _i, C.c_int64, _i64, _i, C.c_int, _i]),
        "mcg_add_move": (C.c_int, [P, C.c_int, C.c_int, _i, C.c_double, C.c_double, C.c_int]),
        "mcg_metropolis_run": (C.c_int, [P, C.c_int, C.c_uint64, C.c_int, _d, _i, _d, _i64, _i64]),
        "mcg_metropolis_run_saving": (C.c_int, [P, C.c_int, C.c_uint64, C.c_int, C.c_int, _d, _d, _d, _i64]),
        "mcg_batch_create": (C.c_int, [C.POINTER(SystemDesc), C.c_int, C.POINTER(BatchOpts), C.POINTER(P)]),
        "mcg_batch_destroy": (C.c_int, [P]),
        "mcg_batch_sweep": (C.c_int, [P, C.c_int]),
        "mcg_batch_sweep_logged": (C.c_int, [P, C.c_void_p, C.c_int64]),
        "mcg_batch_save": (C.c_int, [P, C.c_char_p]),
        "mcg_batch_load": (C.c_int, [P, C.c_char_p]),
        "mcg_batch_stats": (C.c_int, [P, _i64, _i64, _d]),
        "mcg_batch_energy_fp64": (C.c_int, [P, _d]),
        "mcg_batch_get_coords": (C.c_int, [P, C.c_int, _d, _d, _d]),
        "mcg_batch_set_coords": (C.c_int, [P, C.c_int, _d, _d, _d]),
        "mcg_batch_natoms": (C.c_int64, [P]),
        "mcg_batch_chain_natoms": (C.c_int, [P, C.c_int]),
        "mcg_batch_counters": (C.c_int, [P, _i64, _i64]),
        "mcg_batch_time_sweeps": (C.c_int, [P, C.c_int, C.POINTER(C.c_float)]),
        "mcg_batch_time_phases": (C.c_int, [P, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "mcg_batch_autotune": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(BatchTuning)]),
        "mcg_batch_get_tuning": (C.c_int, [P, C.POINTER(BatchTuning)]),
        "mcg_batch_run_host": (C.c_int, [P, _d, C.c_int, _d, _i64, _d]),
        "mcg_batch_energy_mixed": (C.c_int, [P, _d]),
        "mcg_batch_pairs": (C.c_int, [P, _i64]),
        "mcg_batch_update_lists": (C.c_int, [P]),
        "mcg_batch_get_dmax": (C.c_int, [P, _d, _d]),
        "mcg_batch_get_lists": (C.c_int, [P, C.c_int, _i, _i, C.c_int64, _i64]),
        "mcg_pair_count": (C.c_int, [P, _i64, _i64]),
        "mcg_time_nonbonded": (C.c_int, [P, C.c_int, C.POINTER(C.c_float)]),
        "mcg_time_nonbonded_flushed": (C.c_int, [P, C.c_int, C.POINTER(C.c_float)]),
        "mcg_kernel_launches": (C.c_int, [P, _i64]),
        "mcg_set_pair_kernel": (C.c_int, [P, C.c_int]),
        "mcg_get_pair_kernel": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "mcg_cluster_stats": (C.c_int, [P, _i64, _i64, _i64]),
        "mcg_group_stats": (C.c_int, [P, _i64, _i64, _i64]),
        "mcg_set_prune_buffer": (C.c_int, [P, C.c_double]),
        "mcg_prune_stats": (C.c_int, [P, _i64, _i64, C.POINTER(C.c_float)]),
        "mcg_mdbas_read": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(P)]),
        "mcg_mdbas_natom": (C.c_int, [P]),
        "mcg_mdbas_fill": (C.c_int, [P, C.POINTER(SystemDesc)]),
        "mcg_mdbas_free": (C.c_int, [P]),
        "mcg_probe_fp32_tflops": (C.c_int, [_d]),
        "mcg_energy_switch_fp64_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                                     C.c_int, _d, C.c_double, C.c_double, C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc < 0:
        raise McgError(rc, lib().mcg_last_error().decode(errors="replace"))
    return rc


def pd(a):
    return a.ctypes.data_as(_d)


def pi(a):
    return a.ctypes.data_as(_i)


def make_desc(s, precision: str = "fp64"):
    """SystemDesc for an mc_cpp_gb300.mdbas.System; returns (desc, keepalive)."""
    keep = []

    def dbl(a):
        a = np.ascontiguousarray(a, np.float64)
        keep.append(a)
        return pd(a)

    def it(a):
        a = np.ascontiguousarray(a, np.int32)
        keep.append(a)
        return pi(a)

    d = SystemDesc()
    d.natom = s.natom
    d.x, d.y, d.z, d.q = dbl(s.x), dbl(s.y), dbl(s.z), dbl(s.q)
    d.eps, d.sig, d.eps14, d.sig14 = dbl(s.eps), dbl(s.sig), dbl(s.eps14), dbl(s.sig14)
    d.mass = dbl(s.mass)
    fr = np.ascontiguousarray(s.frozen, np.uint8)
    keep.append(fr)
    d.frozen = fr.ctypes.data_as(C.POINTER(C.c_ubyte))
    d.resid = it(s.resid)
    d.pbc_type = PBC[s.pbc_type]
    d.box = (C.c_double * 3)(*[float(v) for v in s.box])
    d.cut_mode = CUT[s.cut_mode]
    d.cutoff, d.cuton, d.dcut, d.temp = s.cutoff, s.cuton, s.dcut, s.temp
    d.precision = PREC[precision]
    d.nbond = len(s.bonds)
    if d.nbond:
        d.bond_atoms, d.bond_type, d.bond_k, d.bond_r0, d.bond_beta = (it(s.bonds), it(s.bond_type), dbl(s.bond_k),
                                                                        dbl(s.bond_r0), dbl(s.bond_beta))
    d.nub = len(s.ub)
    if d.nub:
        d.ub_atoms, d.ub_k, d.ub_r0 = it(s.ub), dbl(s.ub_k), dbl(s.ub_r0)
    d.nangle = len(s.angles)
    if d.nangle:
        d.angle_atoms, d.angle_type, d.angle_k, d.angle_theta0 = (it(s.angles), it(s.angle_type), dbl(s.angle_k),
                                                                  dbl(s.angle_theta0))
    d.ndihe = len(s.dihedrals)
    if d.ndihe:
        d.dihe_atoms, d.dihe_type, d.dihe_order = it(s.dihedrals), it(s.dihe_type), it(s.dihe_order)
        d.dihe_k, d.dihe_phi0, d.dihe_mult = dbl(s.dihe_k), dbl(s.dihe_phi0), dbl(s.dihe_mult)
    d.nimpr = len(s.impropers)
    if d.nimpr:
        d.impr_atoms, d.impr_type, d.impr_order = it(s.impropers), it(s.impr_type), it(s.impr_order)
        d.impr_k, d.impr_phi0, d.impr_mult = dbl(s.impr_k), dbl(s.impr_phi0), dbl(s.impr_mult)
    return d, keep
