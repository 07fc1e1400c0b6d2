import glob
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def reference_dir():
    """The reference checkout: $H264R_REFERENCE_DIR, else where the oracle
    recipe (oracle/Makefile, print-ref) expects it."""
    env = os.environ.get("H264R_REFERENCE_DIR")
    if env:
        return env
    import subprocess
    try:
        out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""
    return out.splitlines()[-1] if out else ""


def fixture_names():
    return sorted(os.path.basename(p)[:-len(".h264r.gz")] for p in glob.glob(os.path.join(HERE, "golden", "*.h264r.gz")))


def load_fixture(name):
    from h264r_dump import read_dump
    pics = read_dump(os.path.join(HERE, "golden", name + ".h264r.gz"))
    with open(os.path.join(HERE, "golden", name + ".json")) as f:
        meta = json.load(f)
    assert len(meta["pictures"]) == len(pics)
    return pics, meta


@pytest.fixture(scope="session")
def engine_lib():
    """libh264r.so built in-tree (builds it when missing)."""
    from h264_video_decoder_demo_gb300 import build
    if not os.path.exists(build.LIB):
        build.build_engine()
    from h264_video_decoder_demo_gb300 import engine
    return engine.lib()


@pytest.fixture(scope="session")
def gpu_ctx(engine_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a host without CUDA")
    from h264_video_decoder_demo_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
