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


def poisson_coeffs(orc: ref.Ref, im: int, jm: int, km: int) -> dict:
    """The SOR coefficients of init.f95:82-107 and the interior spacings, from an oracle."""
    g = lambda f: orc.get(f).ravel()
    return dict(c2l=g(lesgpu.CN2L)[:, None, None], c2s=g(lesgpu.CN2S)[:, None, None],
                c3l=g(lesgpu.CN3L)[None, :, None], c3s=g(lesgpu.CN3S)[None, :, None],
                c4l=g(lesgpu.CN4L)[None, None, :], c4s=g(lesgpu.CN4S)[None, None, :],
                cn1=orc.get(lesgpu.CN1), dx1=g(lesgpu.DX1)[2:2 + im], dy1=g(lesgpu.DY1)[1:1 + jm],
                dzn=g(lesgpu.DZN)[2:2 + km])


def poisson_apply(c: dict, p: np.ndarray) -> np.ndarray:
    """The operator whose fixed point press's SOR seeks (press.f95:93-96 with reltmp = 0):
    cn2l p(i+1) + cn2s p(i-1) + cn3l p(j+1) + cn3s p(j-1) + cn4l p(k+1) + cn4s p(k-1) - p/cn1,
    with the halos boundp1/boundp2 give p: Neumann in i and k, periodic in j."""
    pe = np.concatenate([p[1:], p[-1:]], 0)
    pw = np.concatenate([p[:1], p[:-1]], 0)
    pn, ps = np.roll(p, -1, 1), np.roll(p, 1, 1)
    pu = np.concatenate([p[:, :, 1:], p[:, :, -1:]], 2)
    pd = np.concatenate([p[:, :, :1], p[:, :, :-1]], 2)
    return (c["c2l"] * pe + c["c2s"] * pw + c["c3l"] * pn + c["c3s"] * ps + c["c4l"] * pu + c["c4s"] * pd
            - p / c["cn1"])


def manufactured_pressure(orc64: ref.Ref, im: int, jm: int, km: int, dt: float = 0.05, seed: int = 5):
    """A known pressure p* and the velocity u that makes press's rhs equal to A p*.

    p* mixes smooth modes in i, j, k with a little noise and is shifted along cos(pi z)
    so that A p* has zero volume-weighted mean (press subtracts that mean, rhsav, before
    its SOR; A p* must stay in A's range).  With f = g = h = v = w = 0, press forms rhs =
    ((u(i) - u(i-1))/dx1(i))/dt (press.f95:49-58), so u(i) = u(i-1) + dt dx1(i) rhs*(i).
    Returns (u over u's declared extents, the expected p after press = p* minus its
    volume-weighted mean, since press removes pav; the SOR started from p = 0)."""
    c = poisson_coeffs(orc64, im, jm, km)
    rng = np.random.default_rng(seed)
    x = (np.arange(1, im + 1) - 0.5) / im
    y = (np.arange(1, jm + 1) - 0.5) / jm
    z = (np.arange(1, km + 1) - 0.5) / km
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    q0 = (np.cos(np.pi * X) * np.sin(2 * np.pi * Y) + 0.5 * np.cos(2 * np.pi * X) * np.cos(np.pi * Z)
          + 0.3 * np.cos(3 * np.pi * Z) * np.cos(4 * np.pi * Y) + 0.1 * rng.uniform(-1, 1, X.shape))
    q1 = np.cos(np.pi * Z)
    w = c["dx1"][:, None, None] * c["dy1"][None, :, None] * c["dzn"][None, None, :]
    ps = q0 - (w * poisson_apply(c, q0)).sum() / (w * poisson_apply(c, q1)).sum() * q1
    rhs = poisson_apply(c, ps)
    u = np.zeros((im + 2, jm + 3, km + 2))  # (0:im+1, -1:jm+1, 0:km+1)
    col = np.zeros((jm, km))
    for i in range(1, im + 1):
        col = col + dt * c["dx1"][i - 1] * rhs[i - 1]
        u[i, 2:jm + 2, 1:km + 1] = col
    expect = ps - (w * ps).sum() / w.sum()
    return np.asfortranarray(u), expect
