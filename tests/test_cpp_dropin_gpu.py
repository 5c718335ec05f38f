"""The reference's QR test sequence (tests/test_qr_tall.cpp, tests/test_qr_fat.cpp)
compiled against the drop-in header <rnp_gpu/QR.hpp> and the C ABI library,
run on the GPU; every residual it prints must be at most 10 (m n eps units)."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_reference_test_sequence_through_cpp_header(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rnp2_gb300 import _build

    _build.build()
    exe = tmp_path / "test_qr_tall_fat_gpu"
    src = os.path.join(ROOT, "tests", "cpp", "test_qr_tall_fat_gpu.cpp")
    cmd = [_build._nvcc(), "-std=c++17", "-O2", "-x", "cu", "-arch=sm_103a", src, "-o", str(exe),
           "-L" + _build.LIBDIR, "-lqr_gb300", "-Xlinker", "-rpath=" + _build.LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert r.stdout.strip().endswith("OK")
