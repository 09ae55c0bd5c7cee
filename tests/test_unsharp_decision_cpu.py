"""The decision rule of the GPU's exact UnsharpMaskFilter point-wise step
(itk-rs_gb300/csrc/unsharp.cuh), restated on the host in
tests/cpp/unsharp_decision.c, never disagrees with the reference's f64
sequence on the voxels it decides: random and adversarial f32 pairs, and every
u8 pair for a set of amounts and thresholds."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_unsharp_decision_rule(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "unsharp_decision")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-frounding-math", os.path.join(HERE, "cpp", "unsharp_decision.c"),
                    "-o", exe, "-lm"], check=True)
    r = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout.splitlines()[0] and " 0 mismatches" in r.stdout.splitlines()[1]
