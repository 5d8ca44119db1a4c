"""The C++ host (conf in, conf out) driving the GPU engine reproduces the
reference's regression goldens text-identically (GPU), the way the
reference's own ctest compares them (src/Apps/run.cpp:38-92)."""
import os
import subprocess

import pytest

from conftest import CONF, ROOT

pytestmark = pytest.mark.gpu

CLI = os.path.join(ROOT, "rockable_gb300", "_lib", "rockable-gb300")


@pytest.mark.parametrize("case,out", [("512_particles", "conf101"), ("518_poly", "conf3001")])
def test_cli_reproduces_golden(case, out, golden_dir, gpu_lib, tmp_path):
    d = golden_dir / case
    r = subprocess.run([CLI, str(d / CONF[case]), "-o", str(tmp_path), "-n", str(tmp_path / out), "-r",
                        str(d / "golden.conf")], cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "regression: identical" in r.stdout
