"""Fixtures from the reference's own result files.

python tests/golden/make_ref_benchmarks.py [REFERENCE_ROOT]

Reads Benchmark/Sloshing/Ref_data/probes.dat and
Benchmark/Regular_3D/Ref_data/probes.dat (probe records written by the
reference HOS-NWT, 61d13.5 format) with their prob.inp probe positions, and
stores the numbers in ref_sloshing.npz and ref_regular3d.npz beside this
script, together with the run configuration that each file's input echo
states. The reference tree is only needed to regenerate the fixtures.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_probes(path):
    rows = []
    with open(path) as f:
        for ln in f:
            if ln.startswith(("#", "TITLE", "VARIABLES")) or not ln.strip():
                continue
            rows.append([float(x.replace("D", "E")) for x in ln.split()])
    return np.array(rows)


def read_xy(path):
    with open(path) as f:
        vals = [ln.split() for ln in f if ln.strip()]
    return np.array([[float(v[0]), float(v[1]) if len(v) > 1 else 0.0] for v in vals])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    bench = os.path.join(root, "Benchmark")
    # Sloshing: 4th natural mode, 0.2 m, linear (M = 1), 129 modes, 20 Hz output
    # (configuration from the Ref_data input echo)
    s = read_probes(os.path.join(bench, "Sloshing", "Ref_data", "probes.dat"))
    np.savez_compressed(os.path.join(HERE, "ref_sloshing.npz"), records=s,
                        probes=read_xy(os.path.join(bench, "Sloshing", "prob.inp")),
                        numerics=np.array([129, 1, 33, 1, 1, 1]))
    # Regular_3D: 30 deg Dalrymple wave, M = 3, 256 x 32 modes, 10 Hz output
    r = read_probes(os.path.join(bench, "Regular_3D", "Ref_data", "probes.dat"))
    np.savez_compressed(os.path.join(HERE, "ref_regular3d.npz"), records=r,
                        probes=read_xy(os.path.join(bench, "Regular_3D", "prob.inp")),
                        numerics=np.array([256, 32, 16, 3, 3, 3]))
    print("sloshing", s.shape, "regular_3d", r.shape)
