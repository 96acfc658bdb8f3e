"""The FField_CUDA adapter (mc_cpp_gb300/adapter/) built inside the reference: it must compile
against mc_cpp's own headers with the reference's flags, link with the reference objects and
libmcgpu.so, and follow the reference's error convention.  Runs where the reference sources are
present (the recipe oracle/ref.mk knows where); skipped elsewhere."""
import os
import subprocess

import pytest

import goldens
from mc_cpp_gb300 import build, mdbas, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _make(*targets):
    return subprocess.run(["make", "-s", "-f", "oracle/ref.mk", "-j8"] + list(targets), cwd=ROOT,
                          capture_output=True, text=True)


@pytest.fixture(scope="module")
def adapter_check():
    if _make("ref-present").returncode != 0:
        pytest.skip("reference sources not present")
    build.build()
    r = _make("oracle/_ref/adapter_check")
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(ROOT, "oracle", "_ref", "adapter_check")


def test_adapter_builds_and_maps_errors_to_the_reference_convention(adapter_check, tmp_path):
    s = goldens.system("diala_vac", "switch")
    mdbas.write_cor(s, str(tmp_path / "s.cor"))
    mdbas.write_forfield(s, str(tmp_path / "s.dat"))
    mdbas.write_xml(s, str(tmp_path / "s.xml"), "s.cor", "s.dat")
    r = subprocess.run([adapter_check, str(tmp_path / "s.xml"), repr(s.cuton)], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=600)
    if native.lib().mcg_device_count() == 0:
        # no device: the reference's convention, message on stderr and a negative exit status
        assert r.returncode == (native.MCG_ECUDA & 0xff), (r.returncode, r.stderr)
        assert "FField_CUDA create failed" in r.stderr and "no CUDA device" in r.stderr
    else:
        import json
        assert r.returncode == 0, r.stderr
        e = json.loads(r.stdout.strip().splitlines()[-1])
        for a, b in zip(e["cuda"], e["mdbas"]):
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), e
