"""les_main, the main.f95 time loop on the library (mpi-les_gb300/host/les_main.cpp): a
C++ program driving the C-ABI, whose output files equal those of the same run driven
from Python, bit for bit; its per-subroutine mode and its restart."""
import os
import subprocess

import numpy as np
import pytest

import ftnio
import lesgpu
from helpers import scenario

pytestmark = pytest.mark.gpu

MAIN = os.path.join(os.path.dirname(lesgpu.LIB_PATH), "les_main")
IDS = {"u": lesgpu.U, "v": lesgpu.V, "w": lesgpu.W, "p": lesgpu.P, "usum": lesgpu.USUM, "vsum": lesgpu.VSUM,
       "wsum": lesgpu.WSUM, "fold": lesgpu.FOLD, "gold": lesgpu.GOLD, "hold": lesgpu.HOLD, "f": lesgpu.F,
       "g": lesgpu.G, "h": lesgpu.H, "aveu": lesgpu.AVEU, "avew": lesgpu.AVEW, "avev": lesgpu.AVEV,
       "aveuu": lesgpu.AVEUU, "aveww": lesgpu.AVEWW, "avevv": lesgpu.AVEVV, "uwfx": lesgpu.UWFX}
SHAPE = (40, 24, 12)


def _run(*args):
    r = subprocess.run([MAIN, "--dims", "x".join(map(str, SHAPE)), "--seed", "7", "--quiet", *args],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _same_file(path, names, want, header=None):
    got, n, t = ftnio.read_fields(path, names, SHAPE, header=header is not None)
    for nm in names:
        w = np.zeros(SHAPE, np.float32) if nm == "fghold" else want[nm]
        assert np.array_equal(got[nm].view(np.uint32), w.view(np.uint32)), (path, nm)
    if header is not None:
        assert (n, np.float32(t)) == (header[0], np.float32(header[1])), path


def _snapshot(d, names):
    return {nm: d.download(IDS[nm], (1, 1, 1), SHAPE) for nm in names if nm != "fghold"}


def test_files_equal_the_python_driven_run(built_lib, tmp_path):
    out = tmp_path / "data"
    _run("--nmax", "4", "--n1", "3", "--out", str(out))
    d = lesgpu.Domain(*SHAPE, lesgpu.Params(sor_fixed=0))
    d.setup_scenario(scenario(*SHAPE, seed=7))
    dt = np.float32(0.05)
    for n in range(1, 5):
        d.step(n, 4)
        if n == 2:  # n == n1 - 1: the restart pair
            _same_file(str(out / ftnio.data30_name(2)), ftnio.DATA30, _snapshot(d, ftnio.DATA30), (2, dt))
            _same_file(str(out / ftnio.data31_name(2)), ftnio.DATA31, _snapshot(d, ftnio.DATA31))
        d.aveflow(n, 3, 4)
    _same_file(str(out / ftnio.data30_name(4)), ftnio.DATA30, _snapshot(d, ftnio.DATA30), (4, np.float32(3) * dt))
    _same_file(str(out / ftnio.data31_name(4)), ftnio.DATA31, _snapshot(d, ftnio.DATA31))
    _same_file(str(out / "data20"), ftnio.DATA20, _snapshot(d, ftnio.DATA20))
    _same_file(str(out / "data21"), ftnio.DATA21, _snapshot(d, ftnio.DATA21))
    _same_file(str(out / "data10"), ftnio.DATA10, _snapshot(d, ftnio.DATA10))
    _same_file(str(out / "data11"), ftnio.DATA11, _snapshot(d, ftnio.DATA11))
    assert sorted(os.listdir(out)) == sorted(["data10", "data11", "data20", "data21", ftnio.data30_name(2),
                                             ftnio.data31_name(2), ftnio.data30_name(4), ftnio.data31_name(4)])


def test_per_stage_mode_and_restart(built_lib, tmp_path):
    a, b, c = tmp_path / "graph", tmp_path / "stages", tmp_path / "restarted"
    _run("--nmax", "4", "--n1", "3", "--out", str(a))
    text = _run("--nmax", "4", "--n1", "3", "--out", str(b), "--per-stage")
    for name in ("data20", "data21", "data10", "data11", ftnio.data30_name(4)):
        assert (a / name).read_bytes() == (b / name).read_bytes(), name
    assert "les_main: 4 steps" in text
    # restart from the n = 2 pair into a fresh set-up, steps 3..4 (ifdata.f95:252-480)
    _run("--n0", "3", "--nmax", "4", "--n1", "3", "--out", str(c), "--no-aveflow",
         "--restart", str(a / ftnio.data30_name(2)), str(a / ftnio.data31_name(2)))
    d = lesgpu.Domain(*SHAPE, lesgpu.Params(sor_fixed=0))
    d.setup_scenario(scenario(*SHAPE, seed=7))
    d.read_restart(str(a / ftnio.data30_name(2)), str(a / ftnio.data31_name(2)))
    for n in (3, 4):
        d.step(n, 4)
    _same_file(str(c / "data20"), ftnio.DATA20, _snapshot(d, ftnio.DATA20))
