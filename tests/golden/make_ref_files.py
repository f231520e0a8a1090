"""Generate tests/golden/ref_files.json from the reference's own file code.

Runs oracle/_ref/ref_files (the reference's src/init.cu particle-file reader
and src/diagnostic.cu writers, compiled from its sources with host-memory
copies, see oracle/ref_pin.py) on a small seeded case and stores its inputs
and the files it wrote.  Run from the repository root where the reference
sources are present:  python tests/golden/make_ref_files.py
"""
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import ref_pin  # noqa: E402

NCX, NCY, DS = 4, 8, 0.5
INPUT = ("#execution configuration\nn_ini = 0;\nn_prev = 0;\nn_save = 10;\nn_fin = 100;\n"
         "ne = 1.0e14;\nTe = 1.0e3;\nbeta = 1.0e-1;\ngamma = 1.0e3;\nphi_p = -5.0e0;\n"
         f"ncx = {NCX};\nncy = {NCY};\nds = 5.0e-1;\ndt = 1.0e-3;\n")
SPECIAL = [-0.0, 5e-324, 1.7976931348623157e308, -1e-300, 0.1, 1.0 / 3.0]


def particles(rng):
    """Row-sorted particles (the order the reference's snapshots have), rows
    2 and 5 empty, one y exactly on a row boundary, special velocities."""
    rows = [r for r in range(NCY) if r not in (2, 5)]
    out = []
    for r in rows:
        for _ in range(rng.integers(1, 9)):
            out.append([rng.uniform(0, NCX * DS), rng.uniform(r * DS, (r + 1) * DS),
                        rng.normal(), rng.normal()])
    a = np.array(out)
    a = a[np.argsort(np.floor(a[:, 1] / DS), kind="stable")]
    a[3, 1] = np.floor(a[3, 1] / DS) * DS
    for k, v in enumerate(SPECIAL):
        a[5 + 2 * k, 2 + k % 2] = v
    return a


def text(a, header):
    lines = [header] if header else []
    lines += [" %.17e %.17e %.17e %.17e " % tuple(r) for r in a]
    return "".join(x + "\n" for x in lines)


def main():
    rng = np.random.default_rng(12)
    p = particles(rng)
    mesh = rng.normal(size=(NCY + 1) * (NCX + 1)) * 10.0 ** rng.integers(-30, 30, size=(NCY + 1) * (NCX + 1))
    mesh[:len(SPECIAL)] = SPECIAL
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "input"))
        with open(os.path.join(d, "input", "input_data"), "w") as f:
            f.write(INPUT)
        with open(os.path.join(d, "input", "particles_in.dat"), "w") as f:
            f.write(text(p, "# x y vx vy"))
        with open(os.path.join(d, "input", "particles_noheader.dat"), "w") as f:
            f.write(text(p, None))
        mesh.astype("<f8").tofile(os.path.join(d, "input", "mesh.bin"))
        ref_pin.run_files(d)
        files = {}
        for name in sorted(os.listdir(os.path.join(d, "output"))):
            with open(os.path.join(d, "output", name)) as f:
                files[name] = f.read()
    res = {"input_data": INPUT, "ncx": NCX, "ncy": NCY, "ds": DS,
           "particles": [[float(v).hex() for v in r] for r in p],
           "mesh": [float(v).hex() for v in mesh], "header": "x y vx vy", "files": files}
    path = os.path.join(ROOT, "tests", "golden", "ref_files.json")
    with open(path, "w") as f:
        json.dump(res, f, indent=0)
    print(f"wrote {path}: {len(p)} particles, files {sorted(files)}")


if __name__ == "__main__":
    main()
