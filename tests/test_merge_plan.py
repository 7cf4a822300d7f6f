"""The streamed merge plan (csrc/emv_plan.cpp) on the CPU: for every k the
pair lists cover every unordered pair {Y, X\\Y} of every subset exactly once
with both halves staged, phases stage rows of one size class, and shared
memory fits.  The checks live in tests/merge_plan_check.cpp, built here with
g++."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "steiner_edge_linear_gb300", "csrc")
STREAM_SMEM_BYTES = 224 * 1024  # emv_device.cu


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("plan") / "merge_plan_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "merge_plan_check.cpp"),
                    os.path.join(CSRC, "emv_plan.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("k", list(range(2, 16)))
def test_merge_plan_covers_every_pair_once(checker, k):
    out = subprocess.run([checker, str(k), str(STREAM_SMEM_BYTES)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith(f"ok k={k} streamed_levels={k - 1} "), out.stdout


def test_relaxation_chunk_rule(checker):
    """Chunk rows per level: within the kernels' record widths, never more
    launches than 512-byte records take, and the worked n = 1e5 / 2^20 cases."""
    out = subprocess.run([checker, "chunks"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok chunks"), out.stdout + out.stderr


def test_value_width_rules(checker):
    """16-bit merge / relaxation rules at their thresholds, with unknown level
    maxima and without 32-bit wrap-around."""
    out = subprocess.run([checker, "widths"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.startswith("ok widths"), out.stdout + out.stderr


def test_smaller_budget_still_covers(checker):
    """A quarter of the shared memory forces more groups and row tiles."""
    out = subprocess.run([checker, "12", str(STREAM_SMEM_BYTES // 4)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
