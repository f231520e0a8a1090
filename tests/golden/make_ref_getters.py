"""Generate tests/golden/ref_getters.json from the reference's own getters.

Runs oracle/ref_pin (the reference's src/init.cu getters compiled from its
sources, see oracle/ref_pin.py) on a set of input_data files and stores every
derived parameter as exact hex doubles.  Run from the repository root where
the reference sources are present:  python tests/golden/make_ref_getters.py
"""
import json
import os
import random
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import ref_pin  # noqa: E402

TEMPLATE = ("#execution configuration\nn_ini = {n_ini};\nn_prev = {n_prev};\nn_save = {n_save};\n"
            "n_fin = {n_fin};\nne = {ne};\nTe = {Te};\nbeta = {beta};\ngamma = {gamma};\n"
            "phi_p = {phi_p};\nncx = {ncx};\nncy = {ncy};\nds = {ds};\ndt = {dt};\n")


def cases():
    out = [
        # the input shipped with the reference (input/input_data)
        dict(n_ini=0, n_prev=0, n_save=100, n_fin=200000, ne="1.0e14", Te="1.0e3", beta="1.0e-1",
             gamma="1.0e3", phi_p="-5.0e0", ncx=127, ncy=1021, ds="1.0e-1", dt="1.0e-3"),
        # the 64x256 workload (n = 160, phi_p = -5 kTe/e)
        dict(n_ini=0, n_prev=0, n_save=100, n_fin=1000, ne="4.2246e15", Te="1.0e3", beta="1.0",
             gamma="100.0", phi_p="-0.43102", ncx=64, ncy=256, ds="0.5", dt="0.05"),
        # the 512x2048 workload (n = 800)
        dict(n_ini=0, n_prev=0, n_save=100, n_fin=500, ne="1.6898e14", Te="1.0e3", beta="0.1",
             gamma="1836.0", phi_p="-0.43102", ncx=512, ncy=2048, ds="0.5", dt="0.05"),
    ]
    rnd = random.Random(0)
    for _ in range(5):
        out.append(dict(n_ini=rnd.randint(0, 50), n_prev=rnd.randint(0, 5), n_save=rnd.randint(1, 500),
                        n_fin=rnd.randint(100, 10 ** 6), ne=f"{rnd.uniform(1e13, 1e17):.6e}",
                        Te=f"{rnd.uniform(300.0, 5e4):.4e}", beta=f"{rnd.uniform(0.01, 2.0):.5e}",
                        gamma=f"{rnd.uniform(20.0, 2000.0):.4e}", phi_p=f"{rnd.uniform(-20.0, 5.0):.5e}",
                        ncx=rnd.randint(8, 1024), ncy=rnd.randint(8, 4096),
                        ds=f"{rnd.uniform(0.05, 1.0):.4e}", dt=f"{rnd.uniform(1e-3, 0.1):.4e}"))
    return out


def main():
    res = []
    for c in cases():
        text = TEMPLATE.format(**c)
        res.append({"input_data": text, "reference": ref_pin.run(text)})
    path = os.path.join(ROOT, "tests", "golden", "ref_getters.json")
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print(f"wrote {len(res)} cases to {path}")


if __name__ == "__main__":
    main()
