"""The reference-side adapter (wnd-charm_gb300/adapter): a
FeatureComputationPlanExecutor subclass and signatures::compute_plan's GB300
body, compiled against the reference's own headers and linked with the
reference library built from its sources (oracle/build_ref.sh) and with
libwndcharm_gb300.so.  Where the reference checkout is present the adapter
must build, and its demo must run the reference's CPU executor and the GB300
executor on the same ImageMatrix: without a GPU every GB300 call fails with
the library's message (no crash, nothing else); with one the rows agree."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("WNDCHARM_REFERENCE", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")) or not shutil.which("g++"),
                    reason="needs the reference checkout and g++")
def test_adapter_builds_against_the_reference_and_runs():
    lib = os.path.join(REPO, "wnd-charm_gb300", "build", "libwndcharm_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("libwndcharm_gb300.so not built")
    b = subprocess.run([os.path.join(REPO, "wnd-charm_gb300", "adapter", "build_adapter.sh"), REF],
                       capture_output=True, text=True, timeout=900)
    assert b.returncode == 0, b.stderr[-2000:]
    r = subprocess.run([os.path.join(REPO, "wnd-charm_gb300", "adapter", "_build", "adapter_demo")],
                       capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "adapter OK" in r.stdout
    assert r.stdout.count("plan ") == 2
