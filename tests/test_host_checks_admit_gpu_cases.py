"""(CPU) The host-side checks (configuration validation, launch-size bounds,
host buffer checks) refuse nothing the GPU tests use: on a machine without
a GPU, every GPU-marked test must get as far as the CUDA runtime and fail
there with the missing-device error, not earlier with a refusal."""
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
DEVICE_ERRORS = ("cudaGetDeviceCount", "Found no NVIDIA driver", "cudaErrorNoDevice", "cudaErrorInsufficientDriver")


def test_gpu_tests_reach_the_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the GPU tests run for real")
    env = dict(os.environ, COLUMNS="400")
    r = subprocess.run([sys.executable, "-m", "pytest", str(ROOT / "tests"), "-q", "-m", "gpu", "-p",
                        "no:cacheprovider", "-rfE", "--tb=short"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    failures = [ln for ln in r.stdout.splitlines() if re.match(r"^(FAILED|ERROR) ", ln)]
    assert failures, r.stdout[-2000:]
    other = []
    for ln in failures:
        if any(e in ln for e in DEVICE_ERRORS):
            continue
        # the C++ demo prints its device error instead of results
        if "test_cpp_api_forward_backward_match_python" in ln and "KeyError" in ln:
            continue
        other.append(ln)
    assert not other, "\n".join(other)
