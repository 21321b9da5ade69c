"""Fixtures from the reference's own result files.

python tests/golden/make_ref_benchmarks.py REFERENCE_ROOT

Reads the probe records that the reference HOS-NWT wrote in
Benchmark/Sloshing, Benchmark/Regular_3D, Benchmark/Irreg_2D and
Benchmark/Irreg_3D (Ref_data/*.dat, 61d13.5 format) with their prob.inp
probe positions (and the wave files of the irregular runs), and stores them
in ref_sloshing.npz, ref_regular3d.npz, ref_irreg2d.npz and ref_irreg3d.npz
beside this script, together with the run configuration that each file's
input echo states. The reference tree is only needed to regenerate the fixtures.
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
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_ref_benchmarks.py REFERENCE_ROOT "
                         "(the HOS-NWT source tree holding Benchmark/)")
    root = sys.argv[1]
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
    # Irreg_2D: the Hs4_Tp10 file wave, second-order wavemaker (i_wmk = 2),
    # M = 3, 512 modes, 30 Hz output over 50 s; the wave file's components
    # are stored too, since the run reads them
    d = os.path.join(bench, "Irreg_2D")
    g = read_probes(os.path.join(d, "Ref_data", "probes_Hs4_Tp10.dat"))
    with open(os.path.join(d, "Hs4_Tp10.cfg")) as f:
        cfg = [ln.strip() for ln in f if ln.strip()]
    comp = []
    with open(os.path.join(d, "Hs4_Tp10.dat")) as f:
        for ln in f:
            if ln.strip():
                comp.append([float(t) for t in ln.replace(",", " ").split()])
    np.savez_compressed(os.path.join(HERE, "ref_irreg2d.npz"), records=g,
                        probes=read_xy(os.path.join(d, "prob.inp")),
                        numerics=np.array([512, 1, 32, 3, 3, 1]), cfg=np.array(cfg),
                        components=np.array(comp))
    # Irreg_3D: an Edinburgh Designs .txt wave (OCEAN reader, icase 31),
    # i_wmk = 2, M = 3 on 256 x 32 modes, 10 Hz output over 256 s
    d = os.path.join(bench, "Irreg_3D")
    g3 = read_probes(os.path.join(d, "Ref_data", "probes.dat"))
    with open(os.path.join(d, "CAT1__22.txt"), encoding="latin-1") as f:
        txt = f.read().splitlines()
    np.savez_compressed(os.path.join(HERE, "ref_irreg3d.npz"), records=g3,
                        probes=read_xy(os.path.join(d, "prob.inp")),
                        numerics=np.array([256, 32, 16, 3, 3, 3]), txt=np.array(txt))
    print("sloshing", s.shape, "regular_3d", r.shape, "irreg_2d", g.shape, len(comp), "irreg_3d", g3.shape)
