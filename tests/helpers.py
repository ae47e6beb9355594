"""Shared test helpers: paired GPU domain + oracle on identical inputs."""
from __future__ import annotations

import numpy as np

import lesgpu
from oracle import ref

STATE = (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P, lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.FOLD, lesgpu.GOLD,
         lesgpu.HOLD, lesgpu.USUM, lesgpu.VSUM, lesgpu.WSUM, lesgpu.RHS, lesgpu.SM)


def scenario(im=40, jm=24, km=20, seed=7, **kw) -> lesgpu.Scenario:
    return lesgpu.Scenario(im=im, jm=jm, km=km, seed=seed, **kw)


def make_ref(prec: int, sc: lesgpu.Scenario, params: lesgpu.Params | None = None, *, sqrt_half=1, red64=1,
             fast=False) -> ref.Ref:
    params = params or lesgpu.Params()
    zbm, uin, vin, win = lesgpu.generate_scenario(sc)
    vn = params.vn if prec == 4 else 15.83e-6
    return ref.Ref(prec, sc.im, sc.jm, sc.km, zbm, uin, vin, win, dt=params.dt, ro=params.ro, vn=vn,
                   alpha=params.alpha, beta=params.beta, omega=params.omega, pjuge=params.pjuge, dx=sc.dx,
                   dy=sc.dy, dz_law=sc.dz_law, dz0=sc.dz0, dz_ratio=sc.dz_ratio, nmaxp=params.nmaxp,
                   sor_fixed=params.sor_fixed, red64=red64, sqrt_half=sqrt_half, fast=fast)


def make_gpu(sc: lesgpu.Scenario, params: lesgpu.Params | None = None) -> lesgpu.Domain:
    d = lesgpu.Domain(sc.im, sc.jm, sc.km, params or lesgpu.Params())
    d.setup_scenario(sc)
    return d


def random_state(sc: lesgpu.Scenario, seed: int = 11) -> dict[int, np.ndarray]:
    """Random values over the full declared extents of every state field (halos too)."""
    rng = np.random.default_rng(seed)
    out = {}
    for fid in STATE:
        lb, ub = lesgpu.declared_extents(fid, sc.im, sc.jm, sc.km)
        shape = tuple(ub[q] - lb[q] + 1 for q in range(3))
        if fid == lesgpu.U:
            a = rng.uniform(2.0, 6.0, shape)
        elif fid == lesgpu.SM:
            a = rng.uniform(0.0, 0.5, shape)
        else:
            a = rng.uniform(-1.0, 1.0, shape)
        out[fid] = np.asfortranarray(a.astype(np.float32))
    return out


def load_state(gpu: lesgpu.Domain, orc: ref.Ref, st: dict[int, np.ndarray]):
    for fid, a in st.items():
        gpu.upload(fid, a)
        orc.set(fid, a.astype(np.float64))


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max|a-b| / max|b| (the error measure of the parity contract)."""
    den = float(np.abs(b).max())
    return float(np.abs(a.astype(np.float64) - b).max()) / (den if den > 0 else 1.0)


def interior(fid, sc):
    lo = {lesgpu.W: (1, 1, 1)}.get(fid, (1, 1, 1))
    return lo, (sc.im, sc.jm, sc.km)
