"""Access to the golden fixtures in tests/golden/ (made by tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np

from mc_cpp_gb300 import mdbas, systems

GOLD_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KCAL = 418.4

SYNTHETIC = {
    "argon864": lambda: systems.argon_fcc(),
    "water4096": lambda: systems.water_box(),
    "water512": lambda: systems.water_box(512, seed=7),
    "peptide": lambda: systems.peptide_in_water(),
    "water33334": lambda: systems.water_box(33334, seed=6),
}
REFERENCE_INPUTS = ("argon_box", "diala_vac", "nma_solvated", "trhbn_solvated")

_gold = None


def golden():
    global _gold
    if _gold is None:
        with open(os.path.join(GOLD_DIR, "golden.json")) as f:
            _gold = json.load(f)
    return _gold


def rows_digest(rows) -> str:
    """sha256 over (i, len, sorted row) for every row: equality of row sets, order-free."""
    h = hashlib.sha256()
    for i, r in enumerate(rows):
        r = np.sort(np.asarray(r, np.int32))
        h.update(np.array([i, len(r)], np.int32).tobytes())
        h.update(r.tobytes())
    return h.hexdigest()


def coords_digest(s) -> str:
    h = hashlib.sha256()
    for a in (s.x, s.y, s.z):
        h.update(np.ascontiguousarray(a, np.float64).tobytes())
    return h.hexdigest()


def system(name: str, cut_mode: str = None):
    """A golden system: a reference example input (.npz) or a regenerated synthetic one."""
    if name in REFERENCE_INPUTS:
        s = mdbas.load_npz(os.path.join(GOLD_DIR, name + ".npz"))
    else:
        s = SYNTHETIC[name]()
        want = golden()["synthetic"][name]["coords_digest"]
        assert coords_digest(s) == want, "synthetic system %s did not regenerate bitwise" % name
    if cut_mode:
        s.cut_mode = cut_mode
    return s


def record(name: str, mode: str):
    g = golden()
    return (g["systems"] if name in REFERENCE_INPUTS else g["synthetic"])[name][mode]


def trace(name: str) -> np.ndarray:
    return np.load(os.path.join(GOLD_DIR, "trace_%s.npy" % name))
