"""Race detection for the CPU oracle's threaded code (the counterpart of the reference's
`go test -race`): tests/tsan_oracle.cpp runs every threaded oracle path with 4 workers under
ThreadSanitizer and must finish without a report; a program with a planted race, built the same
way, must be reported, which shows the sanitizer is active."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLAGS = ["-O1", "-g", "-std=c++17", "-fsanitize=thread", "-pthread"]
ENV = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66")

RACY = r"""
#include <cstdio>
#include <thread>
int main() {
    long x = 0;
    std::thread a([&] { for (int i = 0; i < 100000; ++i) ++x; });
    std::thread b([&] { for (int i = 0; i < 100000; ++i) ++x; });
    a.join();
    b.join();
    std::printf("%ld\n", x);
    return 0;
}
"""


def build(tmp_path, name, sources):
    exe = os.path.join(tmp_path, name)
    r = subprocess.run(["g++", *FLAGS, "-I", os.path.join(ROOT, "oracle"), *sources, "-o", exe],
                       capture_output=True, text=True)
    if r.returncode != 0:
        if "tsan" in r.stderr.lower() or "sanitize" in r.stderr.lower():
            pytest.skip("ThreadSanitizer is not available: " + r.stderr.strip()[-200:])
        raise AssertionError(r.stderr[-2000:])
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_oracle_threaded_paths_have_no_data_race(tmp_path):
    racy_src = os.path.join(tmp_path, "racy.cpp")
    with open(racy_src, "w") as f:
        f.write(RACY)
    racy = build(str(tmp_path), "racy", [racy_src])
    r = subprocess.run([racy], capture_output=True, text=True, env=ENV, timeout=120)
    assert r.returncode != 0 and "ThreadSanitizer" in r.stderr, "the sanitizer missed a planted race"
    exe = build(str(tmp_path), "tsan_oracle",
                [os.path.join(ROOT, "oracle", "bh_oracle.cpp"), os.path.join(ROOT, "tests", "tsan_oracle.cpp")])
    r = subprocess.run([exe], capture_output=True, text=True, env=ENV, timeout=600)
    assert r.returncode == 0 and "ThreadSanitizer" not in r.stderr, r.stderr[-3000:]
    assert r.stdout.startswith("ok")
