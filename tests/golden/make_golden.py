"""Regenerates the golden fixtures in tests/golden/ from the compiled reference.

Run from the repository root in a container that has the reference sources:

    python tests/golden/make_golden.py --ref <path of the mc_cpp sources>
    python tests/golden/make_golden.py --ref <path> --only-argon-long   # the 1e5-move trace alone

It builds the reference and the probe (oracle/ref.mk), converts the reference's own example
inputs (test/*.xml) into compact .npz fixtures, and records what the reference computes on them
and on the seeded synthetic systems of mc_cpp_gb300.systems:

* golden.json   energies (10 components, internal units, 17 significant digits), Verlet and
                exclusion row digests and sizes, 1-4 pair lists, coordinate digests of the
                synthetic systems, MC summaries;
* trace_*.npy   per-step Metropolis traces (12 doubles per step, see oracle/ref_probe.cpp);
* argon864_long.npz  the 1e5-move argon run (seed 1234) in compact form: per step the moved atom,
                the reference's dE (iu), its alpha draw (-1 when none was drawn) and the decision.

Nothing at test time reads the reference: tests load only these files.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from mc_cpp_gb300 import mdbas, systems  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests"))
from goldens import coords_digest, rows_digest  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden")
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe")


def read_lists(path, n):
    buf = np.fromfile(path, np.int32)
    p = 0
    def take():
        nonlocal p
        c = int(buf[p]); p += 1
        r = buf[p:p + c].copy(); p += c
        return r
    excl = [take() for _ in range(n)]
    p14 = take().reshape(-1, 2)
    verlet = [take() for _ in range(n)]
    return excl, p14, verlet


def probe(*args, cwd=None):
    out = subprocess.check_output([PROBE] + list(args), cwd=cwd, stderr=subprocess.DEVNULL).decode()
    return json.loads(out.strip().splitlines()[-1])


def write_inputs(s, d, name, cut_mode=None):
    s = s.copy()
    if cut_mode:
        s.cut_mode = cut_mode
    cor, ff, xml = (os.path.join(d, name + ext) for ext in (".cor", ".ff", ".xml"))
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    mdbas.write_xml(s, xml, os.path.basename(cor), os.path.basename(ff))
    return xml


def record_system(s, name, tmp, modes, lists=True):
    rec = {}
    for mode in modes:
        xml = write_inputs(s, tmp, "%s_%s" % (name, mode), mode)
        e = probe("energy", xml, cwd=tmp)
        r = dict(ener=e["ener"], list_pairs=e["list_pairs"])
        if lists:
            lp = os.path.join(tmp, "lists.bin")
            subprocess.check_call([PROBE, "lists", xml, lp], cwd=tmp, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            excl, p14, verlet = read_lists(lp, s.natom)
            r["excl_digest"] = rows_digest(excl)
            r["excl_total"] = int(sum(len(x) for x in excl))
            r["pairs14"] = p14.tolist() if len(p14) <= 2000 else None
            r["n14"] = int(len(p14))
            if mode == "switch":
                r["verlet_digest"] = rows_digest(verlet)
                r["verlet_total"] = int(sum(len(x) for x in verlet))
        rec[mode] = r
        print(name, mode, r["ener"][0], flush=True)
    return rec


def record_mc(s, name, tmp, nsteps, seed):
    xml = write_inputs(s, tmp, name + "_mc", None)
    tr = os.path.join(tmp, "trace.bin")
    res = probe("mc", xml, str(nsteps), str(seed), tr, cwd=tmp)
    t = np.fromfile(tr, np.float64).reshape(-1, 12)
    np.save(os.path.join(GOLD, "trace_%s.npy" % name), t)
    acc = [int(t[t[:, 1] == k, 11].sum()) for k in range(len(s.moves))]
    tri = [int((t[:, 1] == k).sum()) for k in range(len(s.moves))]
    print(name, "mc", res, tri, acc, flush=True)
    return dict(nsteps=nsteps, seed=seed, final_etot=res["final_etot"], trials=tri, accepted=acc,
                seconds=res["seconds"])


def record_mc_long(s, name, tmp, nsteps, seed):
    """A long single-move-type run kept compact: moved atom, dE, alpha and decision per step."""
    xml = write_inputs(s, tmp, name + "_mc", None)
    tr = os.path.join(tmp, "trace_long.bin")
    res = probe("mc", xml, str(nsteps), str(seed), tr, cwd=tmp)
    t = np.fromfile(tr, np.float64).reshape(-1, 12)
    assert len(t) == nsteps and (t[:, 1] == 0).all()
    np.savez_compressed(os.path.join(GOLD, "%s.npz" % name), imvatm=t[:, 2].astype(np.int32), de=t[:, 9],
                        alpha=t[:, 10], accepted=np.packbits(t[:, 11].astype(np.uint8)),
                        eold=t[::1000, 7], enew=t[::1000, 8])
    print(name, "mc", res, int(t[:, 11].sum()), flush=True)
    return dict(nsteps=nsteps, seed=seed, final_etot=res["final_etot"], trials=[nsteps],
                accepted=[int(t[:, 11].sum())], seconds=res["seconds"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="directory of the FHedin/mc_cpp sources")
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--only-argon-long", action="store_true",
                    help="record only the 1e5-move argon trace and merge it into golden.json")
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-f", "oracle/ref.mk", "REF=" + a.ref, "-j8"], cwd=ROOT)
    if a.only_argon_long:
        with open(os.path.join(GOLD, "golden.json")) as f:
            gold = json.load(f)
        with tempfile.TemporaryDirectory() as tmp:
            gold["mc"]["argon864_long"] = record_mc_long(systems.argon_fcc(), "argon864_long", tmp, 100000, 1234)
        with open(os.path.join(GOLD, "golden.json"), "w") as f:
            json.dump(gold, f, indent=1)
        return
    gold = {"units": "internal (1 kcal/mol = 418.4 iu)", "systems": {}, "mc": {}, "synthetic": {}}
    with tempfile.TemporaryDirectory() as tmp:
        # the reference's own example inputs
        for name in ("argon_box", "diala_vac", "nma_solvated", "trhbn_solvated"):
            s = mdbas.read_xml(os.path.join(a.ref, "test", name + ".xml"))
            mdbas.save_npz(s, os.path.join(GOLD, name + ".npz"))
            e_native = probe("energy", os.path.join(a.ref, "test", name + ".xml"), cwd=os.path.join(a.ref, "test"))
            rec = record_system(s, name, tmp, ("full", "switch"))
            rec["native_xml"] = dict(cut_mode=s.cut_mode, ener=e_native["ener"])
            gold["systems"][name] = rec
        nma = mdbas.read_xml(os.path.join(a.ref, "test", "nma_solvated.xml"))
        nma.cut_mode = "switch"
        gold["mc"]["nma_switch"] = record_mc(nma, "nma_switch", tmp, 500, 1234)
        # seeded synthetic systems (regenerated from their seeds at test time)
        syn = {
            "argon864": systems.argon_fcc(),
            "water4096": systems.water_box(),
            "water512": systems.water_box(512, seed=7),
            "peptide": systems.peptide_in_water(),
        }
        if not a.skip_large:
            syn["water33334"] = systems.water_box(33334, seed=6)
        for name, s in syn.items():
            modes = ("switch", "full") if s.natom <= 20000 else ("switch",)
            rec = record_system(s, name, tmp, modes)
            rec["coords_digest"] = coords_digest(s)
            rec["natom"] = s.natom
            gold["synthetic"][name] = rec
        gold["mc"]["argon864"] = record_mc(syn["argon864"], "argon864", tmp, 2000, 1234)
        gold["mc"]["water512"] = record_mc(syn["water512"], "water512", tmp, 300, 99)
        gold["mc"]["peptide"] = record_mc(syn["peptide"], "peptide", tmp, 30, 5)
        gold["mc"]["argon864_long"] = record_mc_long(syn["argon864"], "argon864_long", tmp, 100000, 1234)
    with open(os.path.join(GOLD, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)


if __name__ == "__main__":
    main()
