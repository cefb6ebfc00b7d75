"""The host-side UVF reader and writer, the .1dt / .2dt parsers, the LZ4
codec and the frame image writer, built from the library's own sources with
AddressSanitizer, UndefinedBehaviorSanitizer and LeakSanitizer and run on
valid, truncated, bit-flipped and overwritten inputs
(tests/sanitize_host.cpp).  A malformed file must come back as a status,
never as a crash, an out-of-bounds access or undefined behaviour.  No GPU."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

CSRC = os.path.join(ROOT, "imagevis3d_gb300", "csrc")


@pytest.fixture(scope="module")
def sanitized(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("san") / "sanitize_host")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-fno-omit-frame-pointer", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
           os.path.join(ROOT, "tests", "sanitize_host.cpp"), os.path.join(CSRC, "uvf.cpp"),
           os.path.join(CSRC, "uvf_api.cpp"), os.path.join(CSRC, "lz4.cpp"), os.path.join(CSRC, "image_io.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in r.stderr.lower() or "ubsan" in r.stderr.lower()):
        pytest.skip("sanitizer runtime not available: " + r.stderr.strip().splitlines()[-1])
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_host_parsers_and_codec_under_sanitizers(sanitized, tmp_path, seed):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([sanitized, str(tmp_path), str(seed)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "ok: 0 failed checks" in r.stdout, (r.stdout + r.stderr)[-4000:]
