"""The SOR tile-shape autotuner (les_gpu_tune_sor) and its size-class table.

The tuner only changes which CTA computes which cell, so a tuned domain's fields
must equal an untuned one's bit for bit; the table must steer new domains of the
class (alone, or as batch members) and nothing else.
"""
import numpy as np
import pytest

import lesgpu
from helpers import make_gpu, scenario

pytestmark = pytest.mark.gpu


@pytest.fixture
def clean_table():
    keys = []
    yield keys
    for im, jm, km, shared in keys:
        lesgpu.set_sor_tuned(im, jm, km, shared, None)


def _steps(d, n):
    for q in range(1, n + 1):
        d.step(q, n)
    d.sync()


def test_tune_alone_picks_a_timed_shape_and_keeps_fields(built_lib, clean_table):
    sc = scenario(150, 60, 20, seed=91)
    clean_table.append((150, 60, 20, False))
    params = lesgpu.Params(nmaxp=6)
    ref = make_gpu(sc, params)
    _steps(ref, 3)
    d = make_gpu(sc, params)
    shape, us, report = d.tune_sor(False)
    nx, ny, kc, depth = shape
    assert nx in (16, 32) and ny in (16, 20, 24, 28, 32) and 1 <= kc <= sc.km and depth in (1, 2)
    assert us > 0 and f"nx={nx} ny={ny} kchunk={kc} depth={depth}:" in report
    assert report.count("us\n") >= 8  # tile heights x k chunks were timed
    assert "depth=2" in report  # and two-iteration marches
    assert lesgpu.sor_tuned(150, 60, 20, False) == shape
    assert lesgpu.sor_tuned(150, 60, 20, True) is None
    assert d.sor_shape() == shape
    _steps(d, 3)
    for fid in lesgpu.STATE_FIELDS:
        x, y = ref.download(fid), d.download(fid)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), lesgpu.FIELD_NAMES[fid]
    # a new domain of the class starts with the tuned shape; a fixed shape still wins
    e = make_gpu(sc, params)
    assert e.sor_shape() == shape
    e.set_sor_shape(32, 16, 0, 1)
    assert e.sor_shape()[:2] == (32, 16) and e.sor_shape()[3] == 1


def test_tune_shared_steers_batch_members(built_lib, clean_table):
    sc = scenario(96, 64, 12, seed=92)
    clean_table.append((96, 64, 12, True))
    params = lesgpu.Params(nmaxp=4)
    a = make_gpu(sc, params)
    shape, us, report = a.tune_sor(True)
    assert shape[0] in (16, 32) and shape[2] == sc.km and us > 0
    assert "replicas=" in report and "nx=16" in report and "nx=32" in report
    b = make_gpu(scenario(96, 64, 12, seed=93), params)
    alone = b.sor_shape()
    batch = lesgpu.Batch()
    batch.add(b, 1, 2)
    assert b.sor_shape() == shape
    while batch.step() > 0:
        pass
    batch.sync()
    assert b.nonfinite() == 0
    batch.close()
    assert alone[0] == 32  # alone, untuned: the model's 32-column choice


def test_tune_without_fused_sweep_and_table_edits(built_lib, clean_table):
    d = make_gpu(scenario(40, 21, 8, seed=94), lesgpu.Params())  # odd jm: per-subroutine SOR
    assert d.tune_sor(False)[0] == (0, 0, 0, 0)
    clean_table.append((70, 50, 30, True))
    lesgpu.set_sor_tuned(70, 50, 30, True, (16, 20, 0))
    assert lesgpu.sor_tuned(70, 50, 30, True) == (16, 20, 30, 1)
    lesgpu.set_sor_tuned(70, 50, 30, True, (32, 32, 0, 2))
    assert lesgpu.sor_tuned(70, 50, 30, True) == (32, 32, 30, 2)
    lesgpu.set_sor_tuned(70, 50, 30, True, None)
    assert lesgpu.sor_tuned(70, 50, 30, True) is None
    for bad in ((24, 20, 0), (32, 32, 0, 1), (16, 24, 0, 2), (32, 28, 10, 2)):
        with pytest.raises(lesgpu.LesError):
            lesgpu.set_sor_tuned(70, 50, 30, True, bad)
