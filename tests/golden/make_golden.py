"""Regenerate the golden fixtures of the CPU oracle (tests/golden/*.npz).

    python tests/golden/make_golden.py

Each fixture is one seeded scenario run through the oracle for a few whole steps,
in FP32 (the reference's real(kind=4), x**0.5 as gfortran's powf and FP32 sums) and
in FP64, keeping the interior u, v, w, p and the press diagnostics.  The fixtures pin
the oracle: a change to its arithmetic shows up as a mismatch in
tests/test_cpu_golden.py, and the GPU tests compare the solver with them directly.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "mpi-les_gb300"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

CASES = {  # name: (im, jm, km, seed, steps, nmaxp)
    "oracle_30x20x16_s8": (30, 20, 16, 8, 3, 50),
}


def run_case(im, jm, km, seed, steps, nmaxp, prec):
    import lesgpu
    from helpers import make_ref, scenario
    sc = scenario(im, jm, km, seed=seed)
    orc = make_ref(prec, sc, lesgpu.Params(nmaxp=nmaxp), sqrt_half=0, red64=0 if prec == 4 else 1)
    for n in range(1, steps + 1):
        orc.step(n, steps)
    lo, hi = (1, 1, 1), (im, jm, km)
    out = {nm: orc.get(fid, lo, hi) for nm, fid in (("u", lesgpu.U), ("v", lesgpu.V), ("w", lesgpu.W),
                                                     ("p", lesgpu.P))}
    dg = orc.diag()
    out["diag"] = np.array([dg["iters"], dg["sor"], dg["uout"], dg["rhsav"], dg["pav"]])
    return out


def main():
    from oracle import ref
    ref.build()
    for name, (im, jm, km, seed, steps, nmaxp) in CASES.items():
        arrays = {}
        for prec in (4, 8):
            res = run_case(im, jm, km, seed, steps, nmaxp, prec)
            for k, v in res.items():
                # fields as float32 (the FP64 results only back a 1e-4 comparison); diagnostics in FP64
                arrays[f"{k}{prec * 8}"] = v.astype(np.float64 if k == "diag" else np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
