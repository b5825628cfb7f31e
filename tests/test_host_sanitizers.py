"""The host C++ (pass planner, FP64 fusion, greedy scheduler, C-ABI argument
checks) under AddressSanitizer + UndefinedBehaviorSanitizer: the CPU tests of
those parts run in a child process against a sanitizer build of libhqs.so
and must finish without a report."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
import hiqsimulator_gb300.capi as capi
capi.LIB_PATH = {lib!r}
import pytest
rc = pytest.main([{tests!r} + "/test_planner.py", {tests!r} + "/test_fusion_host.py",
                  {tests!r} + "/test_boundary.py", "-q", "-x", "-p", "no:cacheprovider", "-k", "not stub"])
assert capi.load()._name == {lib!r}
sys.exit(int(rc))
"""


def _runtime(name):
    p = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_host_code_clean_under_asan_and_ubsan(hqs):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not (asan and ubsan):
        pytest.skip("gcc sanitizer runtimes not installed")
    from hiqsimulator_gb300._build import build_sanitized
    lib = build_sanitized()
    env = dict(os.environ, LD_PRELOAD=asan + " " + ubsan,
               ASAN_OPTIONS="detect_leaks=0:protect_shadow_gap=0:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    code = CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), lib=lib)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env,
                       cwd=ROOT)
    report = r.stdout[-3000:] + r.stderr[-3000:]
    assert r.returncode == 0, report
    assert "ERROR: AddressSanitizer" not in report and "runtime error:" not in report, report
