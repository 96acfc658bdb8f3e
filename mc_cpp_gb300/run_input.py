"""Runs one of mc_cpp's XML inputs on this engine and writes mc_cpp's output files.

    python -m mc_cpp_gb300.run_input input.xml [--precision fp64|mixed] [--outdir DIR]

The program flow of mc_cpp's main for an MC input (src/mc_cpp.cpp, Parser_XML src/Parser.cpp:29-279):
read the XML and the MDBAS .cor / forcefield files it names, build the force field and the move
list, then run MC_metropolis::run for <mc nsteps> steps from <mc seed>.  With <mc save_each> > 0 the
run writes, as MC does (src/MC.cpp:60-70, 93-108; src/MC_metropolis.cpp:156-162):

  tr.xyz    one XYZ frame after every save_each-th step: the atom count, "#At step <st>", then one
            line per atom "<symbol>\\t%10.5lf\\t%10.5lf\\t%10.5lf" (the symbol is the .cor atom name);
  ener.dat  one line per saved step, "<st>\\t%lf" with the running total energy in internal units.

Differences from mc_cpp: a seed of 0 draws from the operating system's entropy source here as
std::random_device does there, so such runs are not reproducible in either program; the energies
come from this library's FP64 engine (or its mixed-precision engine with --precision mixed).
"""
from __future__ import annotations

import argparse
import os
import secrets
import sys
import time

from . import mdbas
from .engine import FFieldCUDA


def write_xyz_frame(f, st: int, symbols, xyz) -> None:
    """One frame of MC::write_traj (src/MC.cpp:93-108)."""
    f.write("%d\n" % len(symbols))
    f.write("#At step %d\n" % st)
    for sym, (x, y, z) in zip(symbols, xyz):
        f.write("%s\t%10.5f\t%10.5f\t%10.5f\n" % (sym, x, y, z))


def write_ener_line(f, st: int, etot: float) -> None:
    """One line of ener.dat (src/MC_metropolis.cpp:161)."""
    f.write("%d\t%f\n" % (st, etot))


def run(xml_path: str, precision: str = "fp64", outdir: str = ".", acceptance: str = "reference", log=None):
    """Runs the input; returns a summary dict (steps, accepted, final total energy in iu)."""
    s = mdbas.read_xml(xml_path)
    if not s.moves:
        raise ValueError("the input has no <movelist> moves (MC::initial_checks_before_running)")
    seed = s.seed if s.seed != 0 else secrets.randbits(32)
    ff = FFieldCUDA(s, precision)
    e0 = ff.getE()
    t0 = time.perf_counter()
    frames, energies, etot, nacc = ff.metropolis_saving(s.nsteps, seed, s.save_each, acceptance)
    secs = time.perf_counter() - t0
    if s.save_each > 0:
        os.makedirs(outdir, exist_ok=True)
        symbols = [str(a) for a in s.atname]
        with open(os.path.join(outdir, "tr.xyz"), "w") as fx, open(os.path.join(outdir, "ener.dat"), "w") as fe:
            for k in range(len(energies)):
                st = (k + 1) * s.save_each
                write_xyz_frame(fx, st, symbols, frames[k])
                write_ener_line(fe, st, energies[k])
    ff.close()
    out = {"input": xml_path, "natom": s.natom, "steps": s.nsteps, "seed": seed, "accepted": nacc,
           "initial_etot_iu": e0, "final_etot_iu": etot, "seconds": secs, "saved": len(energies)}
    if log is not None:
        log.write("%(input)s: %(natom)d atoms, %(steps)d steps (seed %(seed)d), %(accepted)d accepted, "
                  "E %(initial_etot_iu).6f -> %(final_etot_iu).6f iu in %(seconds).2f s\n" % out)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("xml")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--outdir", default=".")
    ap.add_argument("--acceptance", choices=["reference", "physical"], default="reference",
                    help="reference: beta in mol/kcal applied to dE in internal units, as MC_metropolis")
    a = ap.parse_args(argv)
    run(a.xml, a.precision, a.outdir, a.acceptance, log=sys.stdout)
    return 0


if __name__ == "__main__":
    sys.exit(main())
