"""Build libadseismic_gb300.so in-tree (nvcc, sm_103a only)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_PATH = os.path.join(HERE, "lib", "libadseismic_gb300.so")


def build_library(jobs: int = 8, verbose: bool = False) -> str:
    """Compile every CUDA translation unit in parallel and link the C-ABI library."""
    cmd = ["make", "-C", CSRC, f"-j{jobs}"]
    if not verbose:
        cmd.insert(1, "-s")
    subprocess.run(cmd, check=True)
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"build did not produce {LIB_PATH}")
    return LIB_PATH
