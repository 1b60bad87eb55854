"""The BVH8 structural rules (check_node8), applied by the host validator to
host-built trees and by the GPU builder's k_check_* kernels to device-built
ones: host-built trees pass at every node width and size, and each defect
planted in a copy of a valid tree (child index, slot/rank, internal mask,
leaf counts, leaf ranges, leaf order) is refused.  Host code only."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "optix-path-tracer_gb300", "csrc")


def test_bvh_structural_rules(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "bvh_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "bvh_check_driver.cpp"),
                    os.path.join(CSRC, "bvh_host.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    lines = out.stdout.strip().splitlines()
    failed = [l for l in lines if l.startswith("FAIL")]
    assert not failed, failed
    assert out.returncode == 0 and lines[-1] == "ALL PASS"
    # 7 widths x 7 sizes of valid trees, 10 planted defects
    assert sum(l.startswith("PASS ") for l in lines) == 59
