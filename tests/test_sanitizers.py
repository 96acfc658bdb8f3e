"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer (CPU only).

The reference's own Verlet builder overflows its neighbour rows on long runs (a heap overflow
that ASan finds), so the host code here is checked the same way.  tests/sanitize/host_check.cpp
is linked with the library's host-only sources (MDBAS readers, host system with exclusion and
1-4 lists, move instances: mc_cpp_gb300/csrc/mdbas_io.cpp, topology.cpp) and with the oracle
(oracle/mc_oracle.cpp), all built with -fsanitize=address,undefined.  It runs on a solvated
flexible chain (bonds, angles, Urey-Bradley, dihedrals, impropers, 1-4 pairs; 1,540 atoms)
written as MDBAS files, and on truncated and corrupted copies of those files.  Any sanitizer
report ends the run with an error (halt_on_error), and every figure it prints must equal the
unsanitized library's and oracle's exactly.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as orc
from mc_cpp_gb300 import build, mdbas, native, systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mc_cpp_gb300", "csrc")
SOURCES = [os.path.join(ROOT, "tests", "sanitize", "host_check.cpp"), os.path.join(CSRC, "mdbas_io.cpp"),
           os.path.join(CSRC, "topology.cpp"), os.path.join(ROOT, "oracle", "mc_oracle.cpp")]
MVTYPE = {"trn": 1, "rot": 2}
MVMODE = {"residue": 0, "all": 1, "atom": 2}
PBC = {"none": 0, "cubic": 1, "orbic": 2}
CUT = {"full": 0, "switch": 1}


def _sanitizers_available(tmp):
    src = os.path.join(tmp, "probe.cpp")
    with open(src, "w") as f:
        f.write("int main() { return 0; }\n")
    r = subprocess.run(["g++", "-fsanitize=address,undefined", src, "-o", os.path.join(tmp, "probe")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    return r.returncode == 0


@pytest.fixture(scope="module")
def host_check(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    tmp = str(tmp_path_factory.mktemp("sanitize"))
    if not _sanitizers_available(tmp):
        pytest.skip("g++ has no address/undefined sanitizer runtime here")
    exe = os.path.join(tmp, "host_check")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off", "-fopenmp",
           "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-I" + os.path.join(ROOT, "include"),
           "-I" + CSRC] + SOURCES + ["-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return exe


def _system_files(tmp):
    s = systems.peptide_in_water(40, 500, L=24.6, seed=4)
    cor, ff, xml = (os.path.join(tmp, n) for n in ("sys.cor", "sys.ff", "sys.xml"))
    mdbas.write_cor(s, cor)
    mdbas.write_forfield(s, ff)
    mdbas.write_xml(s, xml, "sys.cor", "sys.ff")
    s2 = mdbas.read_xml(xml)             # exactly what the files hold
    a, b, c = s2.box
    settings = os.path.join(tmp, "settings.txt")
    with open(settings, "w") as f:
        f.write("%d %r %r %r %d %r %r %r %r\n" % (PBC[s2.pbc_type], a, b, c, CUT[s2.cut_mode], s2.cutoff, s2.cuton,
                                                  s2.dcut, s2.temp))
    moves = os.path.join(tmp, "moves.txt")
    with open(moves, "w") as f:
        for m in s2.moves:
            sel = orc.selection(s2, m).astype(bool)
            r = np.asarray(s2.resid)[sel]
            lo, hi = int(r.min()), int(r.max())
            assert np.array_equal(sel, (np.asarray(s2.resid) >= lo) & (np.asarray(s2.resid) <= hi))
            f.write("%d %d %d %d %r %r %d\n" % (MVTYPE[m.move_type], MVMODE[m.move_mode], lo, hi,
                                                float(m.dmax_value), float(m.dmax_target), m.dmax_each))
    # malformed copies: truncated coordinates, a non-numeric parameter, an empty pair, a missing file
    lines = open(cor).read().splitlines(True)
    bad = []
    p = os.path.join(tmp, "trunc.cor")
    with open(p, "w") as f:
        f.writelines(lines[:len(lines) // 2])
    bad.append((p, ff))
    text = open(ff).read().split("\n")
    for i, ln in enumerate(text):
        toks = ln.split()
        if len(toks) >= 4 and toks[0].isdigit():
            toks[-1] = "x1.5"
            text[i] = " ".join(toks)
            break
    p = os.path.join(tmp, "corrupt.ff")
    with open(p, "w") as f:
        f.write("\n".join(text))
    bad.append((cor, p))
    e1, e2 = os.path.join(tmp, "empty.cor"), os.path.join(tmp, "empty.ff")
    open(e1, "w").close()
    open(e2, "w").close()
    bad.append((e1, e2))
    bad.append((os.path.join(tmp, "missing.cor"), ff))
    return s2, cor, ff, settings, moves, bad


def test_host_code_and_oracle_clean_under_sanitizers(host_check, tmp_path):
    s, cor, ff, settings, moves, bad = _system_files(str(tmp_path))
    env = dict(os.environ, ASAN_OPTIONS="halt_on_error=1:detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", OMP_NUM_THREADS="2")
    args = [host_check, cor, ff, settings, moves] + [x for pair in bad for x in pair]
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "runtime error" not in r.stderr and "Sanitizer" not in r.stderr, r.stderr[-4000:]
    got = dict(ln.split() for ln in r.stdout.splitlines())

    # the unsanitized library on the same files
    build.build()
    orc.build()
    L = native.lib()
    d, keep = native.make_desc(s)
    counts = np.zeros(s.natom, np.int32)
    total, n14 = C.c_int64(0), C.c_int(0)
    native.check(L.mcg_build_exclusions(C.byref(d), native.pi(counts), None, 0, C.byref(total), None, 0, C.byref(n14)))
    assert int(got["natom"]) == s.natom
    assert int(got["excl_total"]) == total.value
    assert int(got["pairs14"]) == n14.value > 0
    # the unsanitized oracle
    o = orc.Oracle(s)
    for t in range(len(s.moves)):
        assert int(got["instances_%d" % t]) == len(o.move_instances(t))
    assert float(got["energy"]) == o.energy()[0]
    assert int(got["verlet_total"]) == o.verlet_total()
    idx = np.flatnonzero(np.asarray(s.resid) == 2)
    new = s.coords()[idx] + np.array([0.1, -0.05, 0.07])
    assert float(got["delta_e"]) == o.delta_e(idx, new)
    _, fe, nacc = o.mc_run(120, 1234, trace=False)
    assert float(got["mc_final"]) == fe
    assert int(got["mc_accepted"]) == nacc
    for k in range(len(bad)):
        assert int(got["bad_%d" % k]) != native.MCG_OK, k
