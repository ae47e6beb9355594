"""The oracle against its committed golden fixtures (tests/golden, made by
tests/golden/make_golden.py): the FP32 restatement must reproduce them bit for bit,
the FP64 one to float32 rounding.  A change to the oracle's arithmetic shows here."""
import os

import numpy as np
import pytest

import lesgpu
from helpers import make_ref, scenario
from oracle import ref

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASE = ("oracle_30x20x16_s8", 30, 20, 16, 8, 3, 50)


@pytest.mark.parametrize("prec", [4, 8])
def test_oracle_reproduces_golden(prec):
    ref.build()
    name, im, jm, km, seed, steps, nmaxp = CASE
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    orc = make_ref(prec, scenario(im, jm, km, seed=seed), lesgpu.Params(nmaxp=nmaxp), sqrt_half=0,
                   red64=0 if prec == 4 else 1)
    for n in range(1, steps + 1):
        orc.step(n, steps)
    lo, hi = (1, 1, 1), (im, jm, km)
    for nm, fid in (("u", lesgpu.U), ("v", lesgpu.V), ("w", lesgpu.W), ("p", lesgpu.P)):
        x = orc.get(fid, lo, hi).astype(np.float32)
        assert np.array_equal(x.view(np.uint32), g[f"{nm}{prec * 8}"].view(np.uint32)), nm
    dg = orc.diag()
    assert int(dg["iters"]) == int(g[f"diag{prec * 8}"][0])
