"""Stage-by-stage parity of the GPU kernels against the FP32 oracle (bit for bit).

Each test loads the same random state (every field, halos included) into a GPU
domain and into the oracle, runs ONE reference subroutine on both, and compares
every field the subroutine may touch over its full declared extents.  The oracle
runs with x**0.5 evaluated as sqrt (the GPU's IEEE sqrt); all other FP32
operations are identical, so the comparison is exact.  press is exact except for
the FP64 reductions (rhsav, pav), whose summation order differs: its tolerance is
stated in the test.
"""
import numpy as np
import pytest

import lesgpu
from helpers import STATE, load_state, make_gpu, make_ref, random_state, scenario
from oracle import ref

pytestmark = pytest.mark.gpu

SHAPES = [(40, 24, 20), (37, 18, 11), (64, 32, 9)]
# x/y spacings: 4 m (powers of two: reciprocal-multiplication path) and 3 m x 5 m
SPACINGS = [(4.0, 4.0), (3.0, 5.0)]


def _pair(shape, seed=5, spacing=(4.0, 4.0), **pkw):
    sc = scenario(*shape, seed=seed, dx=spacing[0], dy=spacing[1])
    params = lesgpu.Params(**pkw)
    gpu = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    st = random_state(sc, seed=seed + 100)
    load_state(gpu, orc, st)
    return sc, gpu, orc


def _assert_same(gpu, orc, fids, what):
    for fid in fids:
        g = gpu.download(fid)
        o = orc.get(fid).astype(np.float32)
        bad = np.argwhere(g.view(np.uint32) != o.view(np.uint32))
        assert bad.size == 0, (
            f"{what}: field {lesgpu.FIELD_NAMES[fid]} differs at {len(bad)} entries, first (0-based) "
            f"{bad[0].tolist()} gpu={g[tuple(bad[0])]!r} oracle={o[tuple(bad[0])]!r}")


@pytest.mark.parametrize("shape", SHAPES)
def test_velnw(built_lib, shape):
    sc, gpu, orc = _pair(shape)
    gpu.velnw(); orc.stage(ref.VELNW)
    _assert_same(gpu, orc, STATE, "velnw")


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("n", [1, 7])
def test_bondv1(built_lib, shape, n):
    sc, gpu, orc = _pair(shape)
    gpu.bondv1(n); orc.stage(ref.BONDV1, n)
    _assert_same(gpu, orc, STATE, f"bondv1(n={n})")
    assert np.float32(gpu.diag()["uout"]) == np.float32(orc.diag()["uout"])


@pytest.mark.parametrize("spacing", SPACINGS)
@pytest.mark.parametrize("shape", SHAPES)
def test_velfg(built_lib, shape, spacing):
    sc, gpu, orc = _pair(shape, spacing=spacing)
    gpu.velfg(); orc.stage(ref.VELFG)
    _assert_same(gpu, orc, STATE, "velfg")


@pytest.mark.parametrize("kchunk", [1, 3, 7])
def test_velfg_march_chunks(built_lib, monkeypatch, kchunk):
    """The velfg k-march split into chunks of planes (each re-forming the faces of its
    first plane): bit for bit the oracle's, with tiles partial in i (70 = 2 x 31 + 8)
    and in j (20 = 2 x 8 + 4)."""
    monkeypatch.setenv("LES_VELFG_KCHUNK", str(kchunk))
    sc, gpu, orc = _pair((70, 20, 10), spacing=(3.0, 5.0))
    gpu.velfg(); orc.stage(ref.VELFG)
    _assert_same(gpu, orc, STATE, f"velfg kchunk={kchunk}")


@pytest.mark.parametrize("shape", SHAPES)
def test_feedbf(built_lib, shape):
    sc, gpu, orc = _pair(shape)
    gpu.feedbf(); orc.stage(ref.FEEDBF)
    _assert_same(gpu, orc, STATE, "feedbf")


@pytest.mark.parametrize("spacing", SPACINGS)
@pytest.mark.parametrize("shape", SHAPES)
def test_les(built_lib, shape, spacing):
    sc, gpu, orc = _pair(shape, spacing=spacing)
    # les reads the diu arrays that velfg leaves behind: run velfg first on both
    gpu.velfg(); orc.stage(ref.VELFG)
    gpu.les(); orc.stage(ref.LES)
    _assert_same(gpu, orc, STATE, "les")


@pytest.mark.parametrize("shape", [(3, 2, 3), (70, 9, 47)])
def test_les_small_and_chunked(built_lib, shape):
    """velfg then les at the smallest domain (one partial 32 x 8 tile, tensor-copy boxes
    mostly outside the arrays) and at a depth that splits the sm pass and the viscous
    march into several k chunks, with partial tiles in i and j: bitwise the oracle's."""
    sc, gpu, orc = _pair(shape)
    gpu.velfg(); orc.stage(ref.VELFG)
    gpu.les(); orc.stage(ref.LES)
    _assert_same(gpu, orc, STATE, f"les {shape}")


@pytest.mark.parametrize("shape", SHAPES)
def test_adam(built_lib, shape):
    sc, gpu, orc = _pair(shape)
    gpu.adam(); orc.stage(ref.ADAM)
    _assert_same(gpu, orc, STATE, "adam")


@pytest.mark.parametrize("shape", SHAPES)
def test_bondfg_boundp(built_lib, shape):
    sc, gpu, orc = _pair(shape)
    gpu.bondfg(); orc.stage(ref.BONDFG)
    gpu.boundp1(); orc.stage(ref.BOUNDP1)
    gpu.boundp2(); orc.stage(ref.BOUNDP2)
    _assert_same(gpu, orc, STATE, "bondfg+boundp1+boundp2")


@pytest.mark.parametrize("shape", SHAPES)
def test_press(built_lib, shape):
    sc, gpu, orc = _pair(shape, nmaxp=12)
    gpu.press(3, 10); orc.stage(ref.PRESS, 3, 10)
    dg, do = gpu.diag(), orc.diag()
    assert dg["iters"] == do["iters"] == 12
    # rhsav/pav are FP64 sums in a different order: equal after rounding to FP32, or 1 ulp apart
    for key in ("rhsav", "pav"):
        a, b = np.float32(dg[key]), np.float32(do[key])
        assert abs(int(a.view(np.int32)) - int(b.view(np.int32))) <= 1, (key, a, b)
    assert abs(dg["sor"] - do["sor"]) <= 1e-5 * abs(do["sor"]) + 1e-30
    for fid in (lesgpu.P, lesgpu.RHS):
        g = gpu.download(fid).astype(np.float64)
        o = orc.get(fid)
        err = np.abs(g - o).max() / np.abs(o).max()
        assert err <= 2e-6, (lesgpu.FIELD_NAMES[fid], err)
    _assert_same(gpu, orc, (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.F, lesgpu.G, lesgpu.H), "press (f,g,h,u,v,w)")


@pytest.mark.parametrize("stage", ["velnw", "velfg", "les", "press"])
def test_stages_piecewise_vertical_grid(built_lib, stage):
    """The reference's piecewise vertical spacing law (grid.f95:114-132, km >= 58): the
    vertical divisions (dzn, dzs, their sums) run through the reciprocal-corrected
    division, which must give the IEEE quotients bit for bit."""
    sc = scenario(24, 16, 60, seed=41, dz_law=0)
    params = lesgpu.Params(nmaxp=6)
    gpu = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    load_state(gpu, orc, random_state(sc, seed=141))
    if stage == "velnw":
        gpu.velnw(); orc.stage(ref.VELNW)
    elif stage == "velfg":
        gpu.velfg(); orc.stage(ref.VELFG)
    elif stage == "les":
        gpu.velfg(); orc.stage(ref.VELFG)
        gpu.les(); orc.stage(ref.LES)
    else:
        gpu.press(2, 5); orc.stage(ref.PRESS, 2, 5)
        for fid in (lesgpu.P, lesgpu.RHS):
            g = gpu.download(fid).astype(np.float64)
            o = orc.get(fid)
            assert np.abs(g - o).max() / np.abs(o).max() <= 2e-6, lesgpu.FIELD_NAMES[fid]
        return
    _assert_same(gpu, orc, STATE, stage)


def _assert_same_nan(gpu, orc, fids, what):
    """Bitwise equality, with any NaN equal to any NaN (payloads differ by platform)."""
    for fid in fids:
        g = gpu.download(fid)
        o = orc.get(fid).astype(np.float32)
        same = (g.view(np.uint32) == o.view(np.uint32)) | (np.isnan(g) & np.isnan(o))
        bad = np.argwhere(~same)
        assert bad.size == 0, (f"{what}: field {lesgpu.FIELD_NAMES[fid]} differs at {len(bad)} entries, first "
                               f"{bad[0].tolist()} gpu={g[tuple(bad[0])]!r} oracle={o[tuple(bad[0])]!r}")


@pytest.mark.parametrize("stage", ["velnw", "velfg", "les", "rhs"])
@pytest.mark.parametrize("spacing", SPACINGS)
def test_stages_extreme_dividends(built_lib, stage, spacing):
    """Dividends outside the reciprocal-corrected range (below 2^-100, above 2^100,
    zero, signed zero) planted in the state: those cells take the IEEE recomputation
    and must still match the oracle bit for bit."""
    sc = scenario(40, 24, 12, seed=51, dx=spacing[0], dy=spacing[1])
    params = lesgpu.Params(nmaxp=3)
    gpu = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    st = random_state(sc, seed=151)
    rng = np.random.default_rng(152)
    # 3x3x3 blocks of one value, so that differences and averages inside a block are
    # tiny, zero or huge too.  Huge values stay out of the rhs case: its FP64 sum would
    # then depend on the summation order.
    vals = (1e-33, -3e-36, -0.0, 0.0, 1e-39) + (() if stage == "rhs" else (2e31,))
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P, lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.SM):
        a = st[fid]
        for val in vals:
            for _ in range(3):
                lo = [int(rng.integers(0, n - 3)) for n in a.shape]
                a[lo[0]:lo[0] + 3, lo[1]:lo[1] + 3, lo[2]:lo[2] + 3] = np.float32(val)
    load_state(gpu, orc, st)
    if stage == "velnw":
        gpu.velnw(); orc.stage(ref.VELNW)
    elif stage == "velfg":
        gpu.velfg(); orc.stage(ref.VELFG)
    elif stage == "les":
        gpu.velfg(); orc.stage(ref.VELFG)
        gpu.les(); orc.stage(ref.LES)
    else:
        # press: bondfg, rhs (the divisions under test), rhs - rhsav, SOR.  With rhsav equal
        # in FP32 on both sides the stored rhs must agree bit for bit.
        gpu.press(2, 5); orc.stage(ref.PRESS, 2, 5)
        _assert_same_nan(gpu, orc, (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.F, lesgpu.G, lesgpu.H), "press")
        ra, rb = np.float32(gpu.diag()["rhsav"]), np.float32(orc.diag()["rhsav"])
        assert abs(int(ra.view(np.int32)) - int(rb.view(np.int32))) <= 1, (ra, rb)
        if ra == rb:
            _assert_same_nan(gpu, orc, (lesgpu.RHS,), "press rhs")
        return
    _assert_same_nan(gpu, orc, STATE, stage)


@pytest.mark.parametrize("stage", ["velnw", "velfg", "les", "rhs"])
def test_stages_all_blocks_deferred(built_lib, stage):
    """A state scaled to ~1e-31 puts most dividends below 2^-100: nearly every block is
    left to the fixup kernel (more blocks than its grid), and the result must still be
    the oracle's bit for bit."""
    sc = scenario(70, 20, 10, seed=53)
    params = lesgpu.Params(nmaxp=3)
    gpu = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    st = random_state(sc, seed=153)
    for fid in (lesgpu.U, lesgpu.V, lesgpu.W, lesgpu.P, lesgpu.F, lesgpu.G, lesgpu.H):
        st[fid] = np.asfortranarray((st[fid].astype(np.float64) * 1e-31).astype(np.float32))
    load_state(gpu, orc, st)
    if stage == "velnw":
        gpu.velnw(); orc.stage(ref.VELNW)
    elif stage == "velfg":
        gpu.velfg(); orc.stage(ref.VELFG)
    elif stage == "les":
        gpu.velfg(); orc.stage(ref.VELFG)
        gpu.les(); orc.stage(ref.LES)
    else:
        gpu.press(2, 5); orc.stage(ref.PRESS, 2, 5)
        ra, rb = np.float32(gpu.diag()["rhsav"]), np.float32(orc.diag()["rhsav"])
        assert abs(int(ra.view(np.int32)) - int(rb.view(np.int32))) <= 1, (ra, rb)
        if ra == rb:
            _assert_same_nan(gpu, orc, (lesgpu.RHS,), "press rhs")
        return
    _assert_same_nan(gpu, orc, STATE, stage)


@pytest.mark.parametrize("spacing", SPACINGS)
def test_wall_at_rest_gives_nan_like_the_reference(built_lib, spacing):
    """vel2.f95:138,173 divide by the wall speed uspd (vspd): where u = v = 0 on the
    first level the reference forms 0/0, a NaN that les and press then carry.  The GPU
    reproduces it where the reference does, through velfg, les and a whole step."""
    sc = scenario(32, 16, 8, seed=57, dx=spacing[0], dy=spacing[1])
    params = lesgpu.Params(nmaxp=3)
    gpu = make_gpu(sc, params)
    orc = make_ref(4, sc, params, sqrt_half=1, red64=1)
    st = random_state(sc, seed=157)
    for fid in (lesgpu.U, lesgpu.V):  # at rest on k = 1 over a patch (and its neighbours)
        st[fid][8:15, 5:11, 1] = 0.0
    load_state(gpu, orc, st)
    gpu.velfg(); orc.stage(ref.VELFG)
    f = gpu.download(lesgpu.F)
    assert np.isnan(f).any(), "the 0/0 of the wall function did not appear"
    _assert_same_nan(gpu, orc, (lesgpu.F, lesgpu.G, lesgpu.H), "velfg")
    gpu.les(); orc.stage(ref.LES)
    _assert_same_nan(gpu, orc, (lesgpu.F, lesgpu.G, lesgpu.H, lesgpu.SM), "les")
    assert gpu.nonfinite() == 0  # u, v, w, p are still finite before velnw/press use f
