"""Writes the GPU per-stage arrays of one golden case to an .npz file, for
offline comparison with the reference fixtures:

    python tests/save_gpu_arrays.py box12_shock out.npz
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import gpu_dump  # noqa: E402
from conftest import SMALL_CASES  # noqa: E402

if __name__ == "__main__":
    case, path = sys.argv[1], sys.argv[2]
    np.savez_compressed(path, **gpu_dump.run(*SMALL_CASES[case]))
