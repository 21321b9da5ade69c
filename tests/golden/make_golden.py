"""Regenerate the oracle fixtures: python tests/golden/make_golden.py"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import cases  # noqa: E402
from golden_io import run_fixture_case  # noqa: E402

if __name__ == "__main__":
    for name in ("reg1d", "reg3d", "jonswap1d", "slosh"):
        out = run_fixture_case(cases.ALL[name])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, {k: v.shape for k, v in list(out.items())[:3]})
