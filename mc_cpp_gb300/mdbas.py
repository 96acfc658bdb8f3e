"""MDBAS coordinate (.cor) and forcefield (forfield.dat) files, and the reference's XML input.

The formats follow the reference reader: ``IO_MDBAS::read_coord`` (src/IO_MDBAS.cpp:77-128:
``*`` title lines, an atom count, then 10 whitespace-separated fields per atom) and
``IO_MDBAS::read_ff`` (src/IO_MDBAS.cpp:130-505: ``atoms``, ``bonds``, ``urey-bradley``,
``angles``, ``dihedrals``, ``impropers``, ``vdw`` and ``end`` sections, ``#`` comments, keywords
case-insensitive).  Values are kept in file units (kcal/mol, degrees, the MDBAS half-sigma); the
engine applies the reference's unit conversions itself (epsilon -> sqrt(eps * 418.4), k * 418.4,
degrees -> radians).

``write_*`` produce files the reference itself reads, with whitespace-separated ids so systems
above 99,999 atoms parse (the fixed-width CHARMM layout merges fields there).
"""
from __future__ import annotations

import dataclasses
import os
import xml.etree.ElementTree as ET
from typing import List, Optional

import numpy as np

__all__ = ["System", "MoveSpec", "read_cor", "read_forfield", "read_xml", "write_cor",
           "write_forfield", "write_xml", "quantize"]


@dataclasses.dataclass
class MoveSpec:
    """One ``<move>`` of the reference's ``<movelist>`` (src/Parser.cpp:220-245)."""
    move_type: str = "trn"         # "trn" | "rot"
    move_mode: str = "residue"     # "residue" | "all" | "atom"
    sel_mode: str = "all"          # "all" | "none" | "residue_id" | "residue_name" | "atom_idx"
    sele: str = ""
    dmax_value: float = 0.5
    dmax_target: float = 50.0
    dmax_each: int = 0


@dataclasses.dataclass
class System:
    """A molecular system in the reference's data model (AtomList + topology + run settings)."""
    natom: int
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    q: np.ndarray
    eps: np.ndarray            # forcefield-file epsilon, kcal/mol (positive)
    sig: np.ndarray            # MDBAS half-sigma, Angstrom
    eps14: np.ndarray
    sig14: np.ndarray
    mass: np.ndarray
    frozen: np.ndarray         # uint8
    resid: np.ndarray          # global residue id, 1-based, consecutive (cor column 2)
    resname: List[str]
    atname: List[str]
    segname: List[str] = dataclasses.field(default_factory=list)
    resid_seg: Optional[np.ndarray] = None
    atom_type: Optional[np.ndarray] = None
    bonds: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2), np.int32))
    bond_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    bond_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    bond_r0: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    bond_beta: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    ub: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2), np.int32))
    ub_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    ub_r0: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    angles: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.int32))
    angle_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    angle_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    angle_theta0: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    dihedrals: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.int32))
    dihe_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    dihe_order: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    dihe_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    dihe_phi0: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    dihe_mult: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    impropers: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.int32))
    impr_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    impr_order: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    impr_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    impr_phi0: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    impr_mult: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    # run settings (the XML's pbc / ensemble / forcefield / movelist / mc nodes)
    pbc_type: str = "cubic"    # "none" | "cubic" | "orbic"
    box: tuple = (0.0, 0.0, 0.0)
    cut_mode: str = "switch"   # "full" | "switch"
    cutoff: float = 12.0
    cuton: float = 10.0
    dcut: float = 2.0
    temp: float = 300.0
    moves: List[MoveSpec] = dataclasses.field(default_factory=list)
    nsteps: int = 0
    seed: int = 0
    save_each: int = 0         # <mc save_each>: steps between tr.xyz frames / ener.dat lines (0: none)

    def coords(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1)

    def set_coords(self, xyz: np.ndarray) -> None:
        self.x = np.ascontiguousarray(xyz[:, 0], dtype=np.float64)
        self.y = np.ascontiguousarray(xyz[:, 1], dtype=np.float64)
        self.z = np.ascontiguousarray(xyz[:, 2], dtype=np.float64)

    def copy(self) -> "System":
        return dataclasses.replace(self, **{f.name: (getattr(self, f.name).copy()
                                                    if isinstance(getattr(self, f.name), np.ndarray)
                                                    else getattr(self, f.name))
                                            for f in dataclasses.fields(self)})


def quantize(a, decimals: int = 6) -> np.ndarray:
    """Round through decimal text so the array equals what a text reader parses back."""
    fmt = "%.{}f".format(decimals)
    return np.array([float(fmt % v) for v in np.asarray(a, dtype=np.float64).ravel()]).reshape(np.shape(a))


# ---------------------------------------------------------------- readers
def read_cor(path: str) -> dict:
    """IO_MDBAS::read_coord (src/IO_MDBAS.cpp:77-128)."""
    with open(path) as f:
        lines = f.read().split("\n")
    k = 0
    while k < len(lines) and lines[k].startswith("*"):
        k += 1
    natom = int(lines[k].split()[0])
    toks = " ".join(lines[k + 1:]).split()
    if len(toks) < 10 * natom:
        raise ValueError("truncated .cor file: %s" % path)
    rec = [toks[10 * i:10 * i + 10] for i in range(natom)]
    return dict(
        natom=natom,
        atom_id=np.array([int(r[0]) for r in rec], np.int32),
        resid=np.array([int(r[1]) for r in rec], np.int32),
        resname=[r[2] for r in rec],
        atname=[r[3] for r in rec],
        x=np.array([float(r[4]) for r in rec]),
        y=np.array([float(r[5]) for r in rec]),
        z=np.array([float(r[6]) for r in rec]),
        segname=[r[7] for r in rec],
        resid_seg=np.array([int(r[8]) for r in rec], np.int32),
    )


def read_forfield(path: str, natom: int) -> dict:
    """IO_MDBAS::read_ff (src/IO_MDBAS.cpp:130-505).  Values stay in file units."""
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n")]
    out = dict(atom_type=np.zeros(natom, np.int32), q=np.zeros(natom), mass=np.zeros(natom),
               frozen=np.zeros(natom, np.uint8), eps=np.zeros(natom), sig=np.zeros(natom),
               eps14=np.zeros(natom), sig14=np.zeros(natom))
    i = 0

    def records(n):
        nonlocal i
        got = []
        while len(got) < n:
            if i >= len(lines):
                raise ValueError("truncated forcefield file")
            ln = lines[i]
            i += 1
            if ln.startswith("#"):
                continue
            got.append(ln.split())
        return got

    while i < len(lines):
        ln = lines[i].lower()
        i += 1
        if ln.startswith("#") or not ln.split():
            continue
        t = ln.split()
        key = t[0]
        cnt = int(t[1]) if len(t) > 1 else 0
        if key == "atoms":
            if cnt != natom:
                raise ValueError("atom count differs between .cor and forcefield")
            for r in records(cnt):
                a = int(r[0]) - 1
                out["atom_type"][a] = int(r[2])
                out["q"][a] = float(r[3])
                out["mass"][a] = float(r[4])
                out["frozen"][a] = 1 if int(r[5]) else 0
        elif key == "bonds":
            rs = records(cnt)
            out["bonds"] = np.array([[int(r[0]) - 1, int(r[1]) - 1] for r in rs], np.int32).reshape(-1, 2)
            out["bond_type"] = np.array([int(r[2]) for r in rs], np.int32)
            out["bond_k"] = np.array([float(r[3]) for r in rs])
            out["bond_r0"] = np.array([float(r[4]) for r in rs])
            out["bond_beta"] = np.array([float(r[5]) for r in rs])
        elif key == "constraints":
            if cnt:
                raise ValueError("constraints sections are not supported (the reference loops forever on them)")
        elif key == "urey-bradley":
            rs = records(cnt)
            out["ub"] = np.array([[int(r[0]) - 1, int(r[1]) - 1] for r in rs], np.int32).reshape(-1, 2)
            out["ub_k"] = np.array([float(r[2]) for r in rs])
            out["ub_r0"] = np.array([float(r[3]) for r in rs])
        elif key == "angles":
            rs = records(cnt)
            out["angles"] = np.array([[int(r[j]) - 1 for j in range(3)] for r in rs], np.int32).reshape(-1, 3)
            out["angle_type"] = np.array([int(r[3]) for r in rs], np.int32)
            out["angle_k"] = np.array([float(r[4]) for r in rs])
            out["angle_theta0"] = np.array([float(r[5]) for r in rs])
        elif key in ("dihedrals", "impropers"):
            rs = records(cnt)
            p = "dihe" if key == "dihedrals" else "impr"
            out[key] = np.array([[int(r[j]) - 1 for j in range(4)] for r in rs], np.int32).reshape(-1, 4)
            out[p + "_type"] = np.array([int(r[4]) for r in rs], np.int32)
            out[p + "_order"] = np.array([int(r[5]) for r in rs], np.int32)
            out[p + "_k"] = np.array([float(r[6]) for r in rs])
            out[p + "_phi0"] = np.array([float(r[7]) for r in rs])
            out[p + "_mult"] = np.array([float(r[8]) for r in rs])
        elif key == "vdw":
            if cnt != natom:
                raise ValueError("vdw count differs from the atom count")
            for k, r in enumerate(records(cnt)):
                a = int(r[0]) - 1
                if a != k:
                    raise ValueError("vdw parameters missing for atom %d" % k)
                out["eps"][a] = float(r[2])
                out["sig"][a] = float(r[3])
                out["eps14"][a] = float(r[5])
                out["sig14"][a] = float(r[6])
        elif key == "end":
            break
        else:
            raise ValueError("unknown forcefield keyword %r" % key)
    return out


def read_xml(path: str) -> System:
    """Parser_XML (src/Parser.cpp:29-279) for the nodes this engine uses."""
    root = ET.parse(path).getroot()
    base = os.path.dirname(os.path.abspath(path))
    kw = dict(pbc_type="none", box=(0.0, 0.0, 0.0), cut_mode="full", cutoff=12.0, cuton=10.0, dcut=2.0,
              temp=0.0, moves=[], nsteps=10000, seed=0, save_each=0)
    natom = 0
    ffile = cor = None
    for node in root:
        a = node.attrib
        if node.tag == "pbc":
            kw["pbc_type"] = a.get("pbc_type", "none").strip().lower()
            if kw["pbc_type"] != "none":
                kw["box"] = (float(a.get("a", 0)), float(a.get("b", 0)), float(a.get("c", 0)))
        elif node.tag == "ensemble":
            natom = int(a.get("N", 0))
            kw["temp"] = float(a.get("T", 0))
        elif node.tag == "forcefield":
            ffile = a.get("ff_file", "").strip()
            kw["cut_mode"] = a.get("cut_type", "full").strip().lower()
            if kw["cut_mode"] == "switch":
                kw["cutoff"] = float(a.get("cutoff", 12.0))
                kw["cuton"] = float(a.get("cuton", 10.0))
                kw["dcut"] = float(a.get("delta_cut", 2.0))
        elif node.tag == "atomlist":
            cor = a.get("cor_path", "").strip()
        elif node.tag == "movelist":
            for mv in node.findall("move"):
                m = mv.attrib
                kw["moves"].append(MoveSpec(m.get("move_type", "trn").strip().lower(),
                                            m.get("move_mode", "all").strip().lower(),
                                            m.get("sel_mode", "all").strip().lower(), m.get("sele", ""),
                                            float(m.get("dmax_value", 0.5)), float(m.get("dmax_target", 50.0)),
                                            int(m.get("dmax_each", 100))))
        elif node.tag == "mc":
            kw["nsteps"] = int(node.attrib.get("nsteps", 10000))
            kw["seed"] = int(node.attrib.get("seed", 0))
            kw["save_each"] = int(node.attrib.get("save_each", 0))
    c = read_cor(os.path.join(base, cor))
    if c["natom"] != natom:
        raise ValueError("atom count of the .cor differs from the XML")
    f = read_forfield(os.path.join(base, ffile), natom)
    fields = {k: v for k, v in f.items()}
    return System(natom=natom, x=c["x"], y=c["y"], z=c["z"], resid=c["resid"], resname=c["resname"],
                  atname=c["atname"], segname=c["segname"], resid_seg=c["resid_seg"], **fields, **kw)


# ---------------------------------------------------------------- writers
def _g(v: float) -> str:
    return repr(float(v))


def write_cor(s: System, path: str) -> None:
    seg = s.segname or ["SYS"] * s.natom
    rseg = s.resid_seg if s.resid_seg is not None else s.resid
    with open(path, "w") as f:
        f.write("* generated by mc_cpp_gb300\n*\n")
        f.write("%d\n" % s.natom)
        for i in range(s.natom):
            f.write("%d %d %s %s %s %s %s %s %d 0.0\n" % (i + 1, s.resid[i], s.resname[i], s.atname[i],
                                                          _g(s.x[i]), _g(s.y[i]), _g(s.z[i]), seg[i], rseg[i]))


def write_forfield(s: System, path: str) -> None:
    at = s.atom_type if s.atom_type is not None else np.ones(s.natom, np.int32)
    with open(path, "w") as f:
        f.write("# generated by mc_cpp_gb300\n")
        f.write("atoms %d\n" % s.natom)
        for i in range(s.natom):
            f.write("%d %s %d %s %s %d\n" % (i + 1, s.atname[i], at[i], _g(s.q[i]), _g(s.mass[i]), int(s.frozen[i])))
        f.write("bonds %d\n" % len(s.bonds))
        for k in range(len(s.bonds)):
            f.write("%d %d %d %s %s %s\n" % (s.bonds[k, 0] + 1, s.bonds[k, 1] + 1, s.bond_type[k], _g(s.bond_k[k]),
                                             _g(s.bond_r0[k]), _g(s.bond_beta[k])))
        f.write("urey-bradley %d\n" % len(s.ub))
        for k in range(len(s.ub)):
            f.write("%d %d %s %s\n" % (s.ub[k, 0] + 1, s.ub[k, 1] + 1, _g(s.ub_k[k]), _g(s.ub_r0[k])))
        f.write("angles %d\n" % len(s.angles))
        for k in range(len(s.angles)):
            a = s.angles[k] + 1
            f.write("%d %d %d %d %s %s\n" % (a[0], a[1], a[2], s.angle_type[k], _g(s.angle_k[k]), _g(s.angle_theta0[k])))
        for key, p in (("dihedrals", "dihe"), ("impropers", "impr")):
            arr = getattr(s, key)
            f.write("%s %d\n" % (key, len(arr)))
            for k in range(len(arr)):
                a = arr[k] + 1
                f.write("%d %d %d %d %d %d %s %s %s\n" % (a[0], a[1], a[2], a[3], getattr(s, p + "_type")[k],
                                                          getattr(s, p + "_order")[k], _g(getattr(s, p + "_k")[k]),
                                                          _g(getattr(s, p + "_phi0")[k]), _g(getattr(s, p + "_mult")[k])))
        f.write("vdw %d\n" % s.natom)
        for i in range(s.natom):
            f.write("%d 0 %s %s 0.0 %s %s 0.0\n" % (i + 1, _g(s.eps[i]), _g(s.sig[i]), _g(s.eps14[i]), _g(s.sig14[i])))
        f.write("end\n")


def write_xml(s: System, path: str, cor_name: str, ff_name: str, nsteps: int = 0, seed: int = 1,
              save_each: int = 0) -> None:
    """An input the reference's Parser_XML reads (save_each = 0: no trajectory files)."""
    a, b, c = s.box
    mv = "".join('    <move move_type="%s" move_mode="%s" sel_mode="%s" sele="%s" dmax_value="%r" '
                 'dmax_each="%d" dmax_target="%r" />\n' % (m.move_type, m.move_mode, m.sel_mode, m.sele,
                                                          float(m.dmax_value), m.dmax_each, float(m.dmax_target))
                 for m in s.moves)
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<inputFile title="generated">\n')
        f.write('  <pbc pbc_type="%s" a="%r" b="%r" c="%r" alpha="90.0" beta="90.0" gamma="90.0"/>\n'
                % (s.pbc_type, float(a), float(b), float(c)))
        f.write('  <ensemble ens_type="nvt" N="%d" T="%r" />\n' % (s.natom, float(s.temp)))
        if s.cut_mode == "switch":
            f.write('  <forcefield ff_type="mdbas" ff_file="%s" cut_type="switch" cutoff="%r" cuton="%r" '
                    'delta_cut="%r" />\n' % (ff_name, float(s.cutoff), float(s.cuton), float(s.dcut)))
        else:
            f.write('  <forcefield ff_type="mdbas" ff_file="%s" cut_type="full" />\n' % ff_name)
        f.write('  <atomlist list_mode="file" file_type="cor" cor_path="%s" />\n' % cor_name)
        f.write("  <movelist>\n%s  </movelist>\n" % mv)
        f.write('  <mc nsteps="%d" save_each="%d" seed="%d"/>\n</inputFile>\n' % (nsteps, save_each, seed))


# ---------------------------------------------------------------- compact fixtures
_ARRAYS = ("x", "y", "z", "q", "eps", "sig", "eps14", "sig14", "mass", "frozen", "resid", "resid_seg", "atom_type",
           "bonds", "bond_type", "bond_k", "bond_r0", "bond_beta", "ub", "ub_k", "ub_r0", "angles", "angle_type",
           "angle_k", "angle_theta0", "dihedrals", "dihe_type", "dihe_order", "dihe_k", "dihe_phi0", "dihe_mult",
           "impropers", "impr_type", "impr_order", "impr_k", "impr_phi0", "impr_mult")


def save_npz(s: System, path: str) -> None:
    """Store a System losslessly as a compressed .npz (used for test fixtures)."""
    arr = {k: getattr(s, k) for k in _ARRAYS if getattr(s, k) is not None}
    meta = dict(natom=s.natom, pbc_type=s.pbc_type, box=list(s.box), cut_mode=s.cut_mode, cutoff=s.cutoff,
                cuton=s.cuton, dcut=s.dcut, temp=s.temp, nsteps=s.nsteps, seed=s.seed,
                moves=[dataclasses.asdict(m) for m in s.moves])
    import json
    np.savez_compressed(path, __meta__=np.frombuffer(json.dumps(meta).encode(), np.uint8),
                        __names__=np.frombuffer("\n".join(["|".join(s.resname), "|".join(s.atname),
                                                           "|".join(s.segname)]).encode(), np.uint8), **arr)


def load_npz(path: str) -> System:
    import json
    z = np.load(path)
    meta = json.loads(bytes(z["__meta__"]).decode())
    names = bytes(z["__names__"]).decode().split("\n")
    kw = {k: z[k] for k in _ARRAYS if k in z.files}
    moves = [MoveSpec(**m) for m in meta.pop("moves")]
    box = tuple(meta.pop("box"))
    return System(resname=names[0].split("|"), atname=names[1].split("|"),
                  segname=names[2].split("|") if names[2] else [], moves=moves, box=box, **meta, **kw)
