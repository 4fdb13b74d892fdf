"""The La Budde lane schedules (host_common.h) cover every product exactly once and their owner
lists name exactly the pieces of each coefficient: a host-only C++ check, compiled with nvcc."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_lb_schedules_cover_every_product_once(tmp_path):
    from thewalrus_gb300 import _native as nat
    nvcc = nat._nvcc()
    if not (os.path.exists(nvcc) or shutil.which(nvcc)):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "lb_schedule_check")
    build = subprocess.run([nvcc, "-std=c++17", "-O1", "-o", exe, os.path.join(HERE, "lb_schedule_check.cu")],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, timeout=300)
    assert build.returncode == 0, build.stdout.decode()
    run = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, timeout=120)
    assert run.returncode == 0 and run.stdout.decode().strip() == "ok", run.stdout.decode()
