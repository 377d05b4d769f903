"""The reference's own GPU test programs (tests/cosine_comparison_test.cpp,
tests/encoding_comparison_test.cpp, tests/GPU_encode_test.cpp) compile and
link unchanged against the GPU.cuh drop-in, with the reference's CPU sources
(src/HV.cpp, src/encoder.cpp) beside it in place of src/encode.cu and
src/cosine.cu.  Build only (no GPU needed); skipped without the reference."""
import os
import subprocess
import tempfile

import pytest

from oracle.build import REF_ROOT as REF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bacterial-classification_gb300")


@pytest.mark.parametrize("prog", ["cosine_comparison_test.cpp", "encoding_comparison_test.cpp",
                                  "GPU_encode_test.cpp"])
def test_reference_tests_link_against_dropin(hdc, prog):
    if not os.path.exists(os.path.join(REF, "tests", prog)):
        pytest.skip("reference checkout not present")
    import build as pkg_build
    pkg_build.build()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "a.out")
        cmd = ["g++", "-std=c++20", "-O1", "-DNORM_COSINE", "-w",
               "-I" + os.path.join(PKG, "dropin"), "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REF, "src"),
               os.path.join(REF, "tests", prog), os.path.join(REF, "src", "HV.cpp"),
               os.path.join(REF, "src", "encoder.cpp"), os.path.join(PKG, "dropin", "gpu_dropin.cpp"),
               "-L" + pkg_build.OUT, "-lhdc_gb300", "-Wl,-rpath," + pkg_build.OUT, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        assert os.path.getsize(exe) > 0


# the reference's own applications and tests written against src/encoder.h, built against the
# GPU-backed encoder.h drop-in (HVCache on the GPU) with the reference's HV.cpp beside it
@pytest.mark.parametrize("prog", ["targets/identify.cpp", "targets/propogate-children.cpp", "tests/query-test.cpp",
                                  "tests/sim-test.cpp"])
def test_reference_programs_link_against_encoder_dropin(hdc, prog):
    if not os.path.exists(os.path.join(REF, prog)):
        pytest.skip("reference checkout not present")
    import build as pkg_build
    pkg_build.build()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "a.out")
        cmd = ["g++", "-std=c++20", "-O1", "-DNORM_COSINE", "-w",
               "-I" + os.path.join(PKG, "dropin", "hvcache"), "-I" + os.path.join(PKG, "dropin"),
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REF, "src"),
               os.path.join(REF, prog), os.path.join(REF, "src", "HV.cpp"),
               os.path.join(PKG, "dropin", "hvcache", "encoder_gpu.cpp"), os.path.join(PKG, "dropin", "hierarchy.cpp"),
               "-L" + pkg_build.OUT, "-lhdc_gb300", "-Wl,-rpath," + pkg_build.OUT, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
        assert "HVCache::similarity" in syms or "HVCache::get" in syms
        assert "HVCache::compute" not in syms  # the CPU encoder of src/encoder.cpp is not linked
