"""CPU checks: the product's host set-up against the oracle, and the C-ABI surface.

No GPU needed: the set-up routines (grid.f95, init.f95:82-107, feedbfm.f95) and the
scenario generator are host code of the solver library.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import lesgpu
from helpers import make_ref, scenario
from oracle import ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions(header):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(les_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    names = _declared_functions(os.path.join(ROOT, "include", "les_gpu.h"))
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_field_ids_match_oracle(built_lib):
    sc = scenario(12, 8, 6)
    r = make_ref(4, sc)
    r.aveflow(1, 1, 1)  # the time-average fields exist from the first aveflow on
    for fid in list(lesgpu.FIELD_NAMES) + [lesgpu.BMASK1, lesgpu.CMASK1, lesgpu.DMASK1, lesgpu.CN1]:
        lb, ub = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
        assert r.extents(fid) == (lb, ub), fid
    for fid in (lesgpu.DX1, lesgpu.DY1, lesgpu.DZN, lesgpu.DZS, lesgpu.DXS, lesgpu.DYS, lesgpu.Z2, lesgpu.CN2L,
                lesgpu.CN2S, lesgpu.CN3L, lesgpu.CN3S, lesgpu.CN4L, lesgpu.CN4S, lesgpu.DELX1):
        lb, ub = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
        rl, ru = r.extents(fid)
        assert (rl[0], ru[0]) == (lb[0], ub[0]), fid


@pytest.mark.parametrize("dz_law,km", [(1, 20), (1, 90), (0, 64)])
def test_grid_matches_oracle(built_lib, dz_law, km):
    im, jm = 30, 20
    g = lesgpu.setup_grid(im, jm, km, dz_law=dz_law)
    sc = scenario(im, jm, km, dz_law=dz_law)
    r = make_ref(4, sc)
    for name, fid in (("dx1", lesgpu.DX1), ("dy1", lesgpu.DY1), ("dzn", lesgpu.DZN), ("dzs", lesgpu.DZS),
                      ("dxs", lesgpu.DXS), ("dys", lesgpu.DYS), ("z2", lesgpu.Z2)):
        o = r.get(fid).ravel(order="F").astype(np.float32)
        assert np.array_equal(g[name].view(np.uint32), o.view(np.uint32)), name


def test_poisson_and_masks_match_oracle(built_lib):
    im, jm, km = 26, 18, 22
    sc = scenario(im, jm, km, seed=4, coverage=0.4)
    g = lesgpu.setup_grid(im, jm, km)
    lib = lesgpu.load_library()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    cn = {n: np.zeros(s, np.float32) for n, s in (("cn2s", im), ("cn2l", im), ("cn3s", jm), ("cn3l", jm),
                                                  ("cn4s", km), ("cn4l", km))}
    cn1 = np.zeros((im, jm, km), np.float32, order="F")
    assert lib.les_setup_poisson(im, jm, km, fp(g["dxs"]), fp(g["dys"]), fp(g["dzs"]), fp(cn["cn2s"]),
                                 fp(cn["cn2l"]), fp(cn["cn3s"]), fp(cn["cn3l"]), fp(cn["cn4s"]), fp(cn["cn4l"]),
                                 fp(cn1)) == 0
    r = make_ref(4, sc)
    for name, fid in (("cn2s", lesgpu.CN2S), ("cn2l", lesgpu.CN2L), ("cn3s", lesgpu.CN3S), ("cn3l", lesgpu.CN3L),
                      ("cn4s", lesgpu.CN4S), ("cn4l", lesgpu.CN4L)):
        o = r.get(fid).ravel(order="F").astype(np.float32)
        assert np.array_equal(cn[name].view(np.uint32), o.view(np.uint32)), name
    assert np.array_equal(cn1.view(np.uint32), r.get(lesgpu.CN1).astype(np.float32).view(np.uint32))
    zbm, uin, vin, win = lesgpu.generate_scenario(sc)
    masks = {n: np.zeros(s, np.float32, order="F") for n, s in (
        ("a", (im + 2, jm + 2, km + 2)), ("b", (im + 3, jm + 2, km + 2)), ("c", (im + 2, jm + 3, km + 2)),
        ("d", (im + 2, jm + 2, km + 2)))}
    assert lib.les_setup_masks(im, jm, km, fp(zbm), fp(g["z2"]), fp(g["dzn"]), fp(masks["a"]), fp(masks["b"]),
                               fp(masks["c"]), fp(masks["d"])) == 0
    for n, fid in (("a", 19), ("b", lesgpu.BMASK1), ("c", lesgpu.CMASK1), ("d", lesgpu.DMASK1)):
        assert np.array_equal(masks[n], r.get(fid).astype(np.float32)), n
    assert 0.0 < masks["d"][1:-1, 1:-1, 1:-1].mean() < 1.0


def test_scenario_generator_is_deterministic_and_in_range(built_lib):
    sc = scenario(96, 64, 48, seed=17, coverage=0.3)
    a = lesgpu.generate_scenario(sc)
    b = lesgpu.generate_scenario(sc)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    zbm, uin, vin, win = a
    cov = (zbm > 0).mean()
    assert 0.3 <= cov <= 0.45, cov
    assert zbm.max() <= 60.0 and zbm[zbm > 0].min() >= 10.0
    assert np.all(zbm[: 96 // 8 - 1, :] == 0) and np.all(zbm[96 - 96 // 8:, :] == 0)
    # power law u = 5 (z/100)^0.2 with z = z2(k) + 0.5 dzn(k), noise within +-1e-3
    g = lesgpu.setup_grid(96, 64, 48)
    z = g["z2"][1:49].astype(np.float64) + 0.5 * g["dzn"][2:50].astype(np.float64)
    u = 5.0 * (z / 100.0) ** 0.2
    assert np.abs(uin - u[None, :]).max() <= 1.01e-3
    assert np.abs(vin).max() <= 1.01e-3 and np.abs(win).max() <= 1.01e-3
    c = lesgpu.generate_scenario(scenario(96, 64, 48, seed=18))
    assert not np.array_equal(c[0], zbm)


@pytest.mark.parametrize("kw", [
    dict(im=60, jm=40, km=20, seed=5),
    dict(im=150, jm=150, km=90, seed=1),
    dict(im=96, jm=64, km=64, seed=123456789012, coverage=0.41, direction_deg=217.5, u_ref=7.3),
    dict(im=64, jm=256, km=48, seed=77, inflow_law=0, coverage=0.15),
    dict(im=80, jm=40, km=60, seed=9, dz_law=0, direction_deg=-30.0),
    dict(im=32, jm=16, km=12, seed=3, coverage=0.0),
])
def test_oracle_scenario_is_the_products(built_lib, kw):
    """The oracle's restatement of the scenario generator gives the product's arrays bit
    for bit, so the CPU baseline and the checker build their inputs without the product."""
    sc = lesgpu.Scenario(**kw)
    a = lesgpu.generate_scenario(sc)
    b = ref.scenario(**{k: getattr(sc, k) for k in ("im", "jm", "km", "seed", "dz_law", "dz0", "dz_ratio",
                                                    "coverage", "fp_min", "fp_max", "h_min", "h_max",
                                                    "inflow_law", "u_ref", "z_ref", "pl_exp", "direction_deg",
                                                    "noise")})
    for x, y in zip(a, b):
        assert x.shape == y.shape
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_direction_rotates_inflow(built_lib):
    sc = scenario(40, 32, 20, seed=3, direction_deg=30.0, noise=0.0)
    _, uin, vin, _ = lesgpu.generate_scenario(sc)
    ang = np.degrees(np.arctan2(vin, uin))
    assert np.allclose(ang, 30.0, atol=1e-3)
    sc2 = scenario(40, 32, 20, seed=3, direction_deg=120.0, noise=0.0)
    _, u2, v2, _ = lesgpu.generate_scenario(sc2)
    assert np.allclose(np.degrees(np.arctan2(v2, u2)), 30.0, atol=1e-3)


def _area_sequential(im, jm, km, dx1, dy1, dzn):
    """press.f95:65-72 in FP64: k outer, i inner, each product rounded to FP32."""
    t = ((dx1[2:im + 2][:, None] * dy1[1:jm + 1][None, :]).astype(np.float32)[:, :, None]
         * dzn[2:km + 2][None, None, :]).astype(np.float32)
    s = 0.0
    for x in np.transpose(t, (2, 1, 0)).astype(np.float64).ravel().tolist():
        s += x
    return s


@pytest.mark.parametrize("case", ["uniform", "stretched", "steep", "three_dx", "random_dx"])
def test_setup_area_equals_the_sequential_sum(built_lib, case):
    im, jm, km = 60, 44, 24
    g = lesgpu.setup_grid(im, jm, km, dz_law=1, dz0=0.01 if case == "steep" else 2.0,
                          dz_ratio=1.9 if case == "steep" else (1.0 if case == "uniform" else 1.04))
    dx1, dy1, dzn = g["dx1"].copy(), g["dy1"].copy(), g["dzn"].copy()
    rng = np.random.default_rng(3)
    if case == "three_dx":
        dx1[:] = rng.choice(np.array([3.0, 4.0, 5.5], np.float32), dx1.size)
        dy1[:] = rng.choice(np.array([2.0, 3.3], np.float32), dy1.size)
    if case == "random_dx":
        dx1[:] = rng.uniform(1.0, 5.0, dx1.size).astype(np.float32)
    got = lesgpu.setup_area(im, jm, km, dx1, dy1, dzn)
    assert got == _area_sequential(im, jm, km, dx1, dy1, dzn), case


def test_les_main_builds_and_refuses_to_run_without_a_gpu(built_lib, tmp_path):
    """The C++ main program is built beside the library; with no GPU it stops with
    status 1 and says why (no CPU fallback)."""
    import subprocess
    main = os.path.join(os.path.dirname(built_lib), "les_main")
    r = subprocess.run([main, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "usage: les_main" in r.stdout
    r = subprocess.run([main, "--dims", "bad"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([main, "--dims", "24x16x8", "--nmax", "2", "--out", str(tmp_path / "d"), "--quiet"],
                       capture_output=True, text=True, timeout=300)
    if r.returncode != 0:  # no GPU here
        assert r.returncode == 1 and "les_gpu_create" in r.stderr, r.stderr
