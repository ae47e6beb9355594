"""The boundary passes that the step runs as one launch each, checked on the CPU.

boundsm (boundsm.f95:5-69), boundp1 + boundp2 at the end of press (boundp.f95) and
bondv1's periodic side flow + top and underground (bondv1.f95:210-268) are sequences of
passes, each reading what the one before wrote.  The kernels k_boundsm_all,
k_boundp_all and k_bondv1_sides (mpi-les_gb300/csrc/les_kernels.cu) write every halo
point in one pass from a single source point.  Here the pass sequences are restated
loop by loop on small random arrays whose halos hold stale values, and compared bit for
bit with the source-point rules those kernels implement (the same segments and index
arithmetic).  The GPU stage tests hold the kernels themselves against the oracle.
"""
import numpy as np
import pytest

SHAPES = [(5, 4, 3), (7, 2, 4), (3, 6, 2), (4, 1, 3), (9, 5, 6)]


class Arr:
    """A 3-D float32 array indexed by reference indices from (i0, j0, k0)."""

    def __init__(self, a, i0, j0, k0):
        self.a, self.o = a, (i0, j0, k0)

    def __getitem__(self, ijk):
        i, j, k = ijk
        return self.a[i - self.o[0], j - self.o[1], k - self.o[2]]

    def __setitem__(self, ijk, v):
        i, j, k = ijk
        self.a[i - self.o[0], j - self.o[1], k - self.o[2]] = v


def _same(x, y):
    return np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("shape", SHAPES)
def test_boundsm_one_pass(shape):
    im, jm, km = shape
    rng = np.random.default_rng(11 + im)
    base = rng.standard_normal((im + 3, jm + 3, km + 2)).astype(np.float32)  # i, j = -1.., k = 0..
    seq = Arr(base.copy(), -1, -1, 0)
    for k in range(0, km + 2):          # i halos, j = -1..jm+1
        for j in range(-1, jm + 2):
            seq[0, j, k] = seq[1, j, k]
            seq[im + 1, j, k] = seq[im, j, k]
    for k in range(0, km + 2):          # j halos, i = 0..im+1
        for i in range(0, im + 2):
            seq[i, jm + 1, k] = seq[i, jm, k]
            seq[i, 0, k] = seq[i, 1, k]
    for j in range(-1, jm + 2):         # k halos, i = 0..im+1, j = -1..jm+1
        for i in range(0, im + 2):
            seq[i, j, 0] = -seq[i, j, 1]
            seq[i, j, km + 1] = seq[i, j, km]
    src = Arr(base, -1, -1, 0)
    one = Arr(base.copy(), -1, -1, 0)
    nk, ni, nj = (im + 2) * (jm + 3), (jm + 3) * km, im * km
    for t in range(2 * nk + 2 * ni + 2 * nj):  # k_boundsm_all's segments
        if t < 2 * nk:
            r = t % nk
            k = 0 if t < nk else km + 1
            i, j = r % (im + 2), r // (im + 2) - 1
        elif t < 2 * nk + 2 * ni:
            u = t - 2 * nk
            r = u % ni
            i = 0 if u < ni else im + 1
            j, k = r % (jm + 3) - 1, r // (jm + 3) + 1
        else:
            u = t - 2 * nk - 2 * ni
            r = u % nj
            j = 0 if u < nj else jm + 1
            i, k = r % im + 1, r // im + 1
        is_ = min(max(i, 1), im)
        js = -1 if j == -1 else min(max(j, 1), jm)
        ks = min(max(k, 1), km)
        v = src[is_, js, ks]
        one[i, j, k] = -v if k == 0 else v
    assert _same(seq.a, one.a)


@pytest.mark.parametrize("shape", SHAPES)
def test_boundp_one_pass(shape):
    im, jm, km = shape
    rng = np.random.default_rng(23 + im)
    base = rng.standard_normal((im + 2, jm + 2, km + 2)).astype(np.float32)  # 0..im+1, 0..jm+1, 0..km+1
    seq = Arr(base.copy(), 0, 0, 0)
    for k in range(0, km + 2):          # boundp1: i halos (Neumann), j = 0..jm+1
        for j in range(0, jm + 2):
            seq[0, j, k] = seq[1, j, k]
            seq[im + 1, j, k] = seq[im, j, k]
    for k in range(0, km + 2):          # then periodic j halos, i = 0..im+1
        for i in range(0, im + 2):
            seq[i, 0, k] = seq[i, jm, k]
            seq[i, jm + 1, k] = seq[i, 1, k]
    for j in range(0, jm + 2):          # boundp2: k halos (Neumann)
        for i in range(0, im + 2):
            seq[i, j, 0] = seq[i, j, 1]
            seq[i, j, km + 1] = seq[i, j, km]
    src = Arr(base, 0, 0, 0)
    one = Arr(base.copy(), 0, 0, 0)
    nk, ni, nj = (im + 2) * (jm + 2), (jm + 2) * km, im * km
    for t in range(2 * nk + 2 * ni + 2 * nj):  # k_boundp_all's segments
        if t < 2 * nk:
            r = t % nk
            k = 0 if t < nk else km + 1
            i, j = r % (im + 2), r // (im + 2)
        elif t < 2 * nk + 2 * ni:
            u = t - 2 * nk
            r = u % ni
            i = 0 if u < ni else im + 1
            j, k = r % (jm + 2), r // (jm + 2) + 1
        else:
            u = t - 2 * nk - 2 * ni
            r = u % nj
            j = 0 if u < nj else jm + 1
            i, k = r % im + 1, r // im + 1
        is_ = min(max(i, 1), im)
        js = jm if j == 0 else (1 if j == jm + 1 else j)
        ks = min(max(k, 1), km)
        one[i, j, k] = src[is_, js, ks]
    assert _same(seq.a, one.a)


@pytest.mark.parametrize("shape", SHAPES)
def test_bondv1_sides_one_pass(shape):
    im, jm, km = shape
    rng = np.random.default_rng(37 + im)
    mk = lambda: rng.standard_normal((im + 2, jm + 3, km + 2)).astype(np.float32)  # 0.., j = -1.., 0..
    base = [mk(), mk(), mk()]
    u, v, w = (Arr(x.copy(), 0, -1, 0) for x in base)
    for k in range(0, km + 2):          # periodic side flow, i = 0..im+1 (w: k <= km)
        for i in range(0, im + 2):
            u[i, 0, k] = u[i, jm, k]; u[i, jm + 1, k] = u[i, 1, k]
            v[i, 0, k] = v[i, jm, k]; v[i, jm + 1, k] = v[i, 1, k]
            if k <= km:
                w[i, 0, k] = w[i, jm, k]; w[i, jm + 1, k] = w[i, 1, k]
    for j in range(-1, jm + 2):         # top and underground
        for i in range(0, im + 2):
            if j >= 0:
                u[i, j, 0] = -u[i, j, 1]; u[i, j, km + 1] = u[i, j, km]
                v[i, j, 0] = -v[i, j, 1]; v[i, j, km + 1] = v[i, j, km]
            w[i, j, 0] = 0.0
            w[i, j, km] = 0.0
    su, sv, sw = (Arr(x, 0, -1, 0) for x in base)
    ou, ov, ow = (Arr(x.copy(), 0, -1, 0) for x in base)
    ni = im + 2
    na, nb, nc = 2 * km * ni, 2 * (jm + 2) * ni, 2 * (jm + 3) * ni
    for t in range(na + nb + nc):  # k_bondv1_sides' segments
        if t < na:
            r = t % (km * ni)
            j = 0 if t < km * ni else jm + 1
            i, k = r % ni, r // ni + 1
            js = jm if j == 0 else 1
            ou[i, j, k] = su[i, js, k]
            ov[i, j, k] = sv[i, js, k]
            if k <= km - 1:
                ow[i, j, k] = sw[i, js, k]
        elif t < na + nb:
            q = t - na
            r = q % ((jm + 2) * ni)
            k = 0 if q < (jm + 2) * ni else km + 1
            i, j = r % ni, r // ni
            js = jm if j == 0 else (1 if j == jm + 1 else j)
            ks = 1 if k == 0 else km
            ou[i, j, k] = -su[i, js, ks] if k == 0 else su[i, js, ks]
            ov[i, j, k] = -sv[i, js, ks] if k == 0 else sv[i, js, ks]
        else:
            q = t - na - nb
            r = q % ((jm + 3) * ni)
            k = 0 if q < (jm + 3) * ni else km
            i, j = r % ni, r // ni - 1
            ow[i, j, k] = 0.0
    for a, b in ((u, ou), (v, ov), (w, ow)):
        assert _same(a.a, b.a)
