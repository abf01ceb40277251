"""bench.py on the host: the reference arm's JSON line (the oracle port timed on
the CPU cores) and the roofline work model, without a GPU."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def test_reference_arm_line():
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=900, cwd=REPO)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "images/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_stage_work_model():
    B = 128
    # the Chebyshev transforms: 3 per image (the image and its Fourier plane at 512^2,
    # its wavelet plane at 520^2), two n^3 products each, a multiply and an add per term
    assert bench.stage_work("Chebyshev", B) == ("fp64", B * 2 * 2 * (2 * 512 ** 3 + 520 ** 3))
    assert bench.stage_work("Chebyshev", B, "fp64") == bench.stage_work("Chebyshev", B, "mixed")
    # f14 is FP64 work unless the mixed form runs its pairs-of-floats chain; Zernike only in the FP64 form
    assert bench.stage_work("Haralick Textures", B, "mixed", "pairs") is None
    assert bench.stage_work("Haralick Textures", B, "mixed", "exact")[0] == "fp64"
    assert bench.stage_work("Haralick Textures", B, "fp64")[0] == "fp64"
    assert bench.stage_work("Zernike Coefficients", B, "mixed") is None
    assert bench.stage_work("Tamura Textures", B)[0] == "fp64"
    assert bench.stage_work("no such stage", B) is None
