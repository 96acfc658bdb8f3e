"""mc_cpp's XML inputs run end to end on this engine, with mc_cpp's output files (tr.xyz, ener.dat).

The GPU case runs the seeded argon input whose reference run is recorded in tests/golden (2,000
steps, seed 1234): the last ener.dat line must hold the reference's final running energy (within
1e-9 relative, the replay tolerance, plus the %lf rounding) and the accepted count must match.
"""
import io

import numpy as np
import pytest

import goldens
from mc_cpp_gb300 import build, mdbas, native, run_input


def test_output_lines_follow_mc_write_traj_and_ener_dat():
    f = io.StringIO()
    run_input.write_xyz_frame(f, 50, ["OH2", "H1"], np.array([[1.234567, -22.5, 0.0], [100.123456789, 3.0, -4e-6]]))
    assert f.getvalue() == ("2\n#At step 50\nOH2\t   1.23457\t -22.50000\t   0.00000\n"
                            "H1\t 100.12346\t   3.00000\t  -0.00000\n")
    g = io.StringIO()
    run_input.write_ener_line(g, 100, -598952.3088748201)
    assert g.getvalue() == "100\t-598952.308875\n"


def _write_input(tmp_path, name, nsteps, seed, save_each):
    s = goldens.system(name)
    mdbas.write_cor(s, str(tmp_path / "in.cor"))
    mdbas.write_forfield(s, str(tmp_path / "in.ff"))
    mdbas.write_xml(s, str(tmp_path / "in.xml"), "in.cor", "in.ff", nsteps=nsteps, seed=seed, save_each=save_each)
    return s, str(tmp_path / "in.xml")


def test_xml_keeps_the_run_settings(tmp_path):
    s, xml = _write_input(tmp_path, "argon864", 2000, 1234, 500)
    t = mdbas.read_xml(xml)
    assert (t.nsteps, t.seed, t.save_each, len(t.moves)) == (2000, 1234, 500, 1)
    assert t.natom == s.natom and np.array_equal(t.x, s.x)


@pytest.mark.gpu
def test_reference_input_runs_end_to_end(tmp_path):
    build.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")
    g = goldens.golden()["mc"]["argon864"]
    s, xml = _write_input(tmp_path, "argon864", g["nsteps"], g["seed"], 500)
    out = run_input.run(xml, outdir=str(tmp_path / "run"))
    assert out["accepted"] == g["accepted"][0]
    lines = open(tmp_path / "run" / "ener.dat").read().splitlines()
    assert [int(ln.split("\t")[0]) for ln in lines] == [500, 1000, 1500, 2000]
    last = float(lines[-1].split("\t")[1])
    assert abs(last - g["final_etot"]) <= 1e-9 * abs(g["final_etot"]) + 1e-6, (last, g["final_etot"])
    xyz = open(tmp_path / "run" / "tr.xyz").read().splitlines()
    assert len(xyz) == 4 * (2 + s.natom)
    assert xyz[0] == str(s.natom) and xyz[1] == "#At step 500"
    assert xyz[-s.natom - 1] == "#At step 2000"
    last_frame = np.array([[float(v) for v in ln.split("\t")[1:]] for ln in xyz[-s.natom:]])
    assert all(ln.split("\t")[0] == "AR" for ln in xyz[-s.natom:])
    half = np.array(s.box) / 2 + 1e-4
    assert np.all(np.abs(last_frame) <= half)        # moved atoms are re-wrapped into the box
    assert np.abs(last_frame - s.coords()).max() > 0.01
