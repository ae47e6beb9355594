"""Python host binding of the GB300 MPI-LES solver (ctypes over include/les_gpu.h).

``Domain`` mirrors the reference's per-step interface: one method per Fortran
subroutine of the time loop (src/main.f95:260-296) with the same name and order --
``velnw``, ``bondv1(n)``, ``velfg``, ``feedbf``, ``les``, ``adam``, ``press(n, nmax)``
plus ``bondfg``, ``boundp1``, ``boundp2`` -- and ``step(n, nmax)`` for the whole
fused step (the counterpart of ``run_LES_kernel``).  Fields move in and out in the
reference's Fortran layout (column-major numpy arrays with the declared extents).

There is no CPU fallback: every method runs on the GPU through the compiled
library, and constructing a Domain fails loudly when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblesgpu.so")

# field ids (include/les_gpu.h)
U, V, W, P, F, G, H, FOLD, GOLD, HOLD, USUM, VSUM, WSUM, RHS, SM = range(1, 16)
BMASK1, CMASK1, DMASK1, CN1 = 16, 17, 18, 20
DX1, DY1, DZN, DZS, DXS, DYS, Z2, CN2L, CN2S, CN3L, CN3S, CN4L, CN4S, DELX1 = range(32, 46)
UIN, VIN, WIN = 53, 54, 55
# time averages of Domain.aveflow (aveflow.f95:7-22), download only
AVEU, AVEV, AVEW, AVEP, AVEL, AVEUU, AVEVV, AVEWW, AVESM, AVESMSM, UWFX = range(100, 111)
AVE_FIELDS = (AVEU, AVEV, AVEW, AVEP, AVEL, AVEUU, AVEVV, AVEWW, AVESM, AVESMSM, UWFX)

FIELD_NAMES = {
    U: "u", V: "v", W: "w", P: "p", F: "f", G: "g", H: "h", FOLD: "fold", GOLD: "gold",
    HOLD: "hold", USUM: "usum", VSUM: "vsum", WSUM: "wsum", RHS: "rhs", SM: "sm",
    AVEU: "aveu", AVEV: "avev", AVEW: "avew", AVEP: "avep", AVEL: "avel", AVEUU: "aveuu", AVEVV: "avevv",
    AVEWW: "aveww", AVESM: "avesm", AVESMSM: "avesmsm", UWFX: "uwfx",
}
STATE_FIELDS = (U, V, W, P, F, G, H, FOLD, GOLD, HOLD, USUM, VSUM, WSUM)

PROF_SOR, PROF_VELFG, PROF_LES, PROF_VELNW, PROF_STEP, PROF_SOR_SWEEP = range(6)

ERRORS = {0: "ok", -1: "bad argument", -2: "CUDA error", -3: "call out of order",
          -4: "out of device memory", -5: "non-finite values", -6: "busy", -7: "file error"}
IO_LITTLE_ENDIAN = 1


def declared_extents(fid: int, im: int, jm: int, km: int):
    """(lb, ub) of a field as declared in src/main.f95:63-159."""
    t = {
        U: ((0, -1, 0), (im + 1, jm + 1, km + 1)), V: ((0, -1, 0), (im + 1, jm + 1, km + 1)),
        W: ((0, -1, -1), (im + 1, jm + 1, km + 1)), P: ((0, 0, 0), (im + 2, jm + 2, km + 1)),
        RHS: ((0, 0, 0), (im + 1, jm + 1, km + 1)), SM: ((-1, -1, 0), (im + 1, jm + 1, km + 1)),
        FOLD: ((1, 1, 1), (im, jm, km)), GOLD: ((1, 1, 1), (im, jm, km)), HOLD: ((1, 1, 1), (im, jm, km)),
        BMASK1: ((-1, 0, 0), (im + 1, jm + 1, km + 1)), CMASK1: ((0, -1, 0), (im + 1, jm + 1, km + 1)),
        DMASK1: ((0, 0, 0), (im + 1, jm + 1, km + 1)), CN1: ((1, 1, 1), (im, jm, km)),
    }
    for fid2 in (F, G, H, USUM, VSUM, WSUM):
        t[fid2] = ((0, 0, 0), (im, jm, km))
    one = {DX1: (-1, im + 1), DY1: (0, jm + 1), DZN: (-1, km + 2), DZS: (-1, km + 2), DXS: (0, im),
           DYS: (0, jm), Z2: (0, km + 2), CN2L: (1, im), CN2S: (1, im), CN3L: (1, jm), CN3S: (1, jm),
           CN4L: (1, km), CN4S: (1, km), DELX1: (1, km)}
    if fid in t:
        return t[fid]
    if fid in one:
        lo, hi = one[fid]
        return (lo, 0, 0), (hi, 0, 0)
    if fid in (UIN, VIN, WIN):
        return (1, 1, 0), (jm, km, 0)
    if fid in (AVEU, AVEV):
        return (1, 1, 0), (im, jm, km)
    if fid == AVEW:
        return (1, 1, 0), (im + 1, jm, km + 2)
    if fid in AVE_FIELDS:
        return (1, 1, 1), (im, jm, km)
    raise KeyError(fid)


class LesDims(C.Structure):
    _fields_ = [("im", C.c_int), ("jm", C.c_int), ("km", C.c_int)]


class LesParams(C.Structure):
    _fields_ = [("dt", C.c_float), ("ro", C.c_float), ("vn", C.c_float), ("alpha", C.c_float),
                ("beta", C.c_float), ("omega", C.c_float), ("pjuge", C.c_float), ("nmaxp", C.c_int),
                ("sor_fixed", C.c_int), ("sor_ksplit", C.c_int)]


class LesScenario(C.Structure):
    _fields_ = [("im", C.c_int), ("jm", C.c_int), ("km", C.c_int), ("dx", C.c_float), ("dy", C.c_float),
                ("dz_law", C.c_int), ("dz0", C.c_float), ("dz_ratio", C.c_float), ("seed", C.c_ulonglong),
                ("coverage", C.c_float), ("fp_min", C.c_int), ("fp_max", C.c_int), ("h_min", C.c_float),
                ("h_max", C.c_float), ("inflow_law", C.c_int), ("u_ref", C.c_float), ("z_ref", C.c_float),
                ("pl_exp", C.c_float), ("direction_deg", C.c_float), ("noise", C.c_float)]


def vn_reference() -> float:
    """vn = 15.83*10.**(-6.) of set.f95:92, evaluated in FP32 as gfortran folds it."""
    return float(np.float32(15.83) * np.float32(1e-6))


@dataclasses.dataclass
class Params:
    """Physical constants (set.f95:89-95) and SOR controls (press.f95:43-45)."""
    dt: float = 0.05
    ro: float = 1.1763
    vn: float = dataclasses.field(default_factory=vn_reference)
    alpha: float = -10.0
    beta: float = -1.0
    omega: float = 1.0
    pjuge: float = 1e-4
    nmaxp: int = 50
    sor_fixed: int = 1
    sor_ksplit: int = 0  # 1: never split the SOR march in k (domains sharing the GPU)

    def to_c(self) -> LesParams:
        return LesParams(self.dt, self.ro, self.vn, self.alpha, self.beta, self.omega, self.pjuge,
                         self.nmaxp, self.sor_fixed, self.sor_ksplit)


@dataclasses.dataclass
class Scenario:
    """Seeded synthetic urban scenario (replaces the GIS inputs, feedbfm.f95:52-77)."""
    im: int = 150
    jm: int = 150
    km: int = 90
    dx: float = 4.0
    dy: float = 4.0
    dz_law: int = 1
    dz0: float = 2.0
    dz_ratio: float = 1.04
    seed: int = 1
    coverage: float = 0.30
    fp_min: int = 5
    fp_max: int = 20
    h_min: float = 10.0
    h_max: float = 60.0
    inflow_law: int = 1
    u_ref: float = 5.0
    z_ref: float = 100.0
    pl_exp: float = 0.2
    direction_deg: float = 0.0
    noise: float = 1e-3

    def to_c(self) -> LesScenario:
        return LesScenario(self.im, self.jm, self.km, self.dx, self.dy, self.dz_law, self.dz0, self.dz_ratio,
                           self.seed, self.coverage, self.fp_min, self.fp_max, self.h_min, self.h_max,
                           self.inflow_law, self.u_ref, self.z_ref, self.pl_exp, self.direction_deg, self.noise)


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load liblesgpu.so (build it with mpi-les_gb300/build.py); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"GB300 solver library not built: {path} (run mpi-les_gb300/build.py)")
    lib = C.CDLL(path)
    vp, ip_, fp_ = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float)
    sig = {
        "les_setup_grid": (C.c_int, [C.c_int] * 3 + [C.c_float, C.c_float, C.c_int, C.c_float, C.c_float] + [fp_] * 9),
        "les_setup_poisson": (C.c_int, [C.c_int] * 3 + [fp_] * 10),
        "les_setup_masks": (C.c_int, [C.c_int] * 3 + [fp_] * 7),
        "les_scenario_generate": (C.c_int, [C.POINTER(LesScenario)] + [fp_] * 4),
        "les_domain_bytes": (C.c_size_t, [C.c_int] * 3),
        "les_gpu_create": (C.c_int, [C.POINTER(LesDims), C.POINTER(LesParams), C.POINTER(vp)]),
        "les_gpu_destroy": (C.c_int, [vp]),
        "les_gpu_upload": (C.c_int, [vp, C.c_int, fp_, ip_, ip_]),
        "les_gpu_download": (C.c_int, [vp, C.c_int, fp_, ip_, ip_]),
        "les_gpu_download_async": (C.c_int, [vp, C.c_int, fp_, ip_, ip_, C.POINTER(C.c_longlong)]),
        "les_gpu_download_wait": (C.c_int, [vp, C.c_longlong]),
        "les_gpu_commit_setup": (C.c_int, [vp]),
        "les_gpu_feedbfm": (C.c_int, [vp, fp_]),
        "les_setup_area": (C.c_int, [C.c_int] * 3 + [fp_] * 3 + [C.POINTER(C.c_double)]),
        "les_gpu_setup_scenario": (C.c_int, [vp, C.POINTER(LesScenario)]),
        "les_gpu_velnw": (C.c_int, [vp]),
        "les_gpu_bondv1": (C.c_int, [vp, C.c_int]),
        "les_gpu_velfg": (C.c_int, [vp]),
        "les_gpu_feedbf": (C.c_int, [vp]),
        "les_gpu_les": (C.c_int, [vp]),
        "les_gpu_adam": (C.c_int, [vp]),
        "les_gpu_press": (C.c_int, [vp, C.c_int, C.c_int]),
        "les_gpu_bondfg": (C.c_int, [vp]),
        "les_gpu_boundp1": (C.c_int, [vp]),
        "les_gpu_boundp2": (C.c_int, [vp]),
        "les_gpu_step": (C.c_int, [vp, C.c_int, C.c_int]),
        "les_gpu_run": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
        "les_gpu_sync": (C.c_int, [vp]),
        "les_gpu_diag": (C.c_int, [vp, C.POINTER(C.c_double)]),
        "les_gpu_check_finite": (C.c_int, [vp, C.POINTER(C.c_longlong)]),
        "les_gpu_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "les_gpu_launch_count": (C.c_longlong, [vp]),
        "les_gpu_last_error": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
        "les_gpu_profile": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "les_gpu_set_sor_shape": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "les_gpu_aveflow": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
        "les_gpu_sor_shape": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "les_gpu_tune_sor": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_char_p,
                                       C.c_size_t]),
        "les_sor_tuned": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
        "les_sor_set_tuned": (C.c_int, [C.c_int] * 9),
        "les_gpu_write_data20": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "les_gpu_write_data21": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "les_gpu_write_data30": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_float, C.c_int]),
        "les_gpu_write_data31": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "les_gpu_write_data10": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "les_gpu_write_data11": (C.c_int, [vp, C.c_char_p, C.c_int]),
        "les_gpu_ifdata_out": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, ip_]),
        "les_gpu_read_restart": (C.c_int, [vp, C.c_char_p, C.c_char_p, ip_, fp_]),
        "les_batch_create": (C.c_int, [C.POINTER(vp)]),
        "les_batch_destroy": (C.c_int, [vp]),
        "les_batch_admit": (C.c_int, [C.POINTER(LesDims), C.c_size_t, ip_]),
        "les_batch_add": (C.c_int, [vp, vp, C.c_int, C.c_int, ip_]),
        "les_batch_remove": (C.c_int, [vp, C.c_int]),
        "les_batch_step": (C.c_int, [vp, ip_]),
        "les_batch_sync": (C.c_int, [vp]),
        "les_batch_slot": (C.c_int, [vp, C.c_int, ip_, ip_]),
        "les_batch_set_wait_limit": (C.c_int, [vp, C.c_longlong, C.c_int]),
        "les_batch_set_sor_launch": (C.c_int, [vp, C.c_int]),
        "les_batch_last_error": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _iarr(t):
    return (C.c_int * 3)(*t)


def setup_grid(im, jm, km, dx=4.0, dy=4.0, dz_law=1, dz0=2.0, dz_ratio=1.04):
    """grid.f95 arrays for runtime sizes, as a dict of float32 arrays (Fortran extents)."""
    lib = load_library()
    a = {n: np.zeros(s, np.float32) for n, s in (("dx1", im + 3), ("dxl", im + 1), ("dxs", im + 1), ("dy1", jm + 2),
                                                  ("dyl", jm + 1), ("dys", jm + 1), ("dzn", km + 4), ("dzs", km + 4),
                                                  ("z2", km + 3))}
    rc = lib.les_setup_grid(im, jm, km, dx, dy, dz_law, dz0, dz_ratio, *[_fptr(a[n]) for n in
                            ("dx1", "dxl", "dxs", "dy1", "dyl", "dys", "dzn", "dzs", "z2")])
    if rc:
        raise ValueError(f"les_setup_grid: {ERRORS.get(rc, rc)}")
    return a


def setup_area(im: int, jm: int, km: int, dx1, dy1, dzn) -> float:
    """The FP64 interior volume press divides by (press.f95:65-72), as summed
    sequentially over k, j, i (dx1(-1:im+1), dy1(0:jm+1), dzn(-1:km+2))."""
    lib = load_library()
    a = [np.ascontiguousarray(x, np.float32) for x in (dx1, dy1, dzn)]
    if (a[0].size, a[1].size, a[2].size) != (im + 3, jm + 2, km + 4):
        raise ValueError("setup_area: dx1, dy1, dzn must have extents -1:im+1, 0:jm+1, -1:km+2")
    out = C.c_double(0.0)
    rc = lib.les_setup_area(im, jm, km, *[_fptr(x) for x in a], C.byref(out))
    if rc:
        raise ValueError(f"les_setup_area: {ERRORS.get(rc, rc)}")
    return out.value


def generate_scenario(sc: Scenario):
    """(zbm[im,jm], uin[jm,km], vin, win) as Fortran-ordered float32 arrays."""
    lib = load_library()
    zbm = np.zeros((sc.im, sc.jm), np.float32, order="F")
    uin, vin, win = (np.zeros((sc.jm, sc.km), np.float32, order="F") for _ in range(3))
    c = sc.to_c()
    rc = lib.les_scenario_generate(C.byref(c), _fptr(zbm), _fptr(uin), _fptr(vin), _fptr(win))
    if rc:
        raise ValueError(f"les_scenario_generate: {ERRORS.get(rc, rc)}")
    return zbm, uin, vin, win


class LesError(RuntimeError):
    pass


def sor_tuned(im: int, jm: int, km: int, shared: bool, device: int = 0):
    """The tuned SOR shape (nx, ny, kchunk, depth) of a size class, or None if it was
    never tuned."""
    out = (C.c_int * 4)()
    rc = load_library().les_sor_tuned(im, jm, km, 1 if shared else 0, device, out)
    if rc < 0:
        raise LesError(f"les_sor_tuned: {ERRORS.get(rc, rc)}")
    return tuple(int(x) for x in out) if rc == 1 else None


def set_sor_tuned(im: int, jm: int, km: int, shared: bool, shape, device: int = 0) -> None:
    """Enter (or with shape None erase) a size class's SOR shape (nx, ny, kchunk[, depth])
    in the tuned table."""
    nx, ny, kc, depth = (tuple(shape) + (1,))[:4] if shape else (0, 0, 0, 0)
    rc = load_library().les_sor_set_tuned(im, jm, km, 1 if shared else 0, device, nx, ny, kc, depth)
    if rc:
        raise LesError(f"les_sor_set_tuned: {ERRORS.get(rc, rc)}")


def tune_classes(domains, shared: bool) -> dict:
    """Tune the SOR shape once per size class among `domains` (committed Domain
    objects) that has no tuned entry yet; returns {(im, jm, km): (shape, us)}."""
    done = {}
    for d in domains:
        key = (d.im, d.jm, d.km)
        if key in done or sor_tuned(*key, shared) is not None:
            continue
        shape, us, _ = d.tune_sor(shared)
        done[key] = (shape, us)
    return done


class Domain:
    """One urban domain resident on the GPU, advanced by the reference's subroutines."""

    def __init__(self, im: int, jm: int, km: int, params: Params | None = None):
        self.lib = load_library()
        self.im, self.jm, self.km = im, jm, km
        self.params = params or Params()
        self._h = C.c_void_p()
        dims = LesDims(im, jm, km)
        prm = self.params.to_c()
        rc = self.lib.les_gpu_create(C.byref(dims), C.byref(prm), C.byref(self._h))
        if rc:
            raise LesError(f"les_gpu_create failed: {ERRORS.get(rc, rc)}")

    # ---------------------------------------------------------------- lifecycle
    def close(self):
        if self._h:
            self.lib.les_gpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int, what: str):
        if rc:
            buf = C.create_string_buffer(512)
            self.lib.les_gpu_last_error(self._h, buf, 512)
            raise LesError(f"{what}: {ERRORS.get(rc, rc)}: {buf.value.decode(errors='replace')}")

    # ---------------------------------------------------------------- data movement
    def upload(self, fid: int, arr: np.ndarray, lb=None, ub=None):
        dlb, dub = declared_extents(fid, self.im, self.jm, self.km)
        lb = tuple(lb) if lb is not None else dlb
        ub = tuple(ub) if ub is not None else dub
        a = np.asfortranarray(arr, dtype=np.float32)
        n = [ub[q] - lb[q] + 1 for q in range(3)]
        if a.size != n[0] * n[1] * n[2]:
            raise ValueError(f"field {fid}: array of {a.size} values for extents {lb}..{ub}")
        self._check(self.lib.les_gpu_upload(self._h, fid, _fptr(a), _iarr(lb), _iarr(ub)), "upload")

    def download(self, fid: int, lb=None, ub=None) -> np.ndarray:
        dlb, dub = declared_extents(fid, self.im, self.jm, self.km)
        lb = tuple(lb) if lb is not None else dlb
        ub = tuple(ub) if ub is not None else dub
        shape = tuple(ub[q] - lb[q] + 1 for q in range(3))
        out = np.zeros(shape, np.float32, order="F")
        self._check(self.lib.les_gpu_download(self._h, fid, _fptr(out), _iarr(lb), _iarr(ub)), "download")
        return out

    def download_async(self, fid: int, out: np.ndarray, lb=None, ub=None) -> int:
        """Queue a download of a 3-D field's box into `out` (Fortran-ordered float32 of
        the box's shape, kept alive by the caller); returns the ticket for
        download_wait.  The box is snapshotted in stream order, so steps queued after
        this call do not change what arrives."""
        dlb, dub = declared_extents(fid, self.im, self.jm, self.km)
        lb = tuple(lb) if lb is not None else dlb
        ub = tuple(ub) if ub is not None else dub
        shape = tuple(ub[q] - lb[q] + 1 for q in range(3))
        if out.shape != shape or out.dtype != np.float32 or not out.flags.f_contiguous:
            raise ValueError(f"download_async: out must be Fortran-ordered float32 of shape {shape}")
        t = C.c_longlong(-1)
        self._check(self.lib.les_gpu_download_async(self._h, fid, _fptr(out), _iarr(lb), _iarr(ub), C.byref(t)),
                    "download_async")
        return t.value

    def download_wait(self, ticket: int) -> None:
        self._check(self.lib.les_gpu_download_wait(self._h, ticket), "download_wait")

    def commit(self):
        self._check(self.lib.les_gpu_commit_setup(self._h), "commit_setup")

    def feedbfm(self, zbm: np.ndarray):
        """feedbfm.f95:87-116 on the device: the b, c, d masks from zbm (im, jm)."""
        z = np.asfortranarray(zbm, dtype=np.float32)
        if z.shape != (self.im, self.jm):
            raise ValueError(f"feedbfm: zbm must have shape {(self.im, self.jm)}")
        self._check(self.lib.les_gpu_feedbfm(self._h, _fptr(z)), "feedbfm")

    def setup_scenario(self, sc: Scenario):
        c = sc.to_c()
        self._check(self.lib.les_gpu_setup_scenario(self._h, C.byref(c)), "setup_scenario")

    # ---------------------------------------------------------------- the reference's subroutines
    def velnw(self):
        self._check(self.lib.les_gpu_velnw(self._h), "velnw")

    def bondv1(self, n: int):
        self._check(self.lib.les_gpu_bondv1(self._h, n), "bondv1")

    def velfg(self):
        self._check(self.lib.les_gpu_velfg(self._h), "velfg")

    def feedbf(self):
        self._check(self.lib.les_gpu_feedbf(self._h), "feedbf")

    def les(self):
        self._check(self.lib.les_gpu_les(self._h), "les")

    def adam(self):
        self._check(self.lib.les_gpu_adam(self._h), "adam")

    def press(self, n: int, nmax: int):
        self._check(self.lib.les_gpu_press(self._h, n, nmax), "press")

    def bondfg(self):
        self._check(self.lib.les_gpu_bondfg(self._h), "bondfg")

    def boundp1(self):
        self._check(self.lib.les_gpu_boundp1(self._h), "boundp1")

    def boundp2(self):
        self._check(self.lib.les_gpu_boundp2(self._h), "boundp2")

    def step(self, n: int, nmax: int):
        self._check(self.lib.les_gpu_step(self._h, n, nmax), "step")

    def run(self, n0: int, nsteps: int, nmax: int):
        self._check(self.lib.les_gpu_run(self._h, n0, nsteps, nmax), "run")

    def sync(self):
        self._check(self.lib.les_gpu_sync(self._h), "sync")

    def diag(self) -> dict:
        out = (C.c_double * 5)()
        self._check(self.lib.les_gpu_diag(self._h, out), "diag")
        return {"iters": int(out[0]), "sor": out[1], "uout": out[2], "rhsav": out[3], "pav": out[4]}

    def nonfinite(self) -> int:
        bad = C.c_longlong(0)
        rc = self.lib.les_gpu_check_finite(self._h, C.byref(bad))
        if rc not in (0, -5):
            self._check(rc, "check_finite")
        return int(bad.value)

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.les_gpu_stream(self._h, C.byref(s)), "stream")
        return s.value or 0

    def aveflow(self, n: int, n1: int, nmax: int) -> None:
        """aveflow.f95 after step n: time averages from step n1, finalised at nmax
        (download AVEU..UWFX)."""
        self._check(self.lib.les_gpu_aveflow(self._h, n, n1, nmax), "aveflow")

    # ------------------------------------------------- result and restart files
    @staticmethod
    def _io_flags(big_endian: bool) -> int:
        return 0 if big_endian else IO_LITTLE_ENDIAN

    def write_data20(self, path: str, big_endian: bool = True) -> None:
        """data20 of press.f95:205-216 (u, v, w, p, usum, vsum, wsum)."""
        self._check(self.lib.les_gpu_write_data20(self._h, os.fsencode(path), self._io_flags(big_endian)),
                    "write_data20")

    def write_data21(self, path: str, big_endian: bool = True) -> None:
        """data21 of adam.f95:20-27 (fold, gold, hold, fghold = zeros)."""
        self._check(self.lib.les_gpu_write_data21(self._h, os.fsencode(path), self._io_flags(big_endian)),
                    "write_data21")

    def write_data30(self, path: str, n: int, time: float, big_endian: bool = True) -> None:
        """data30 of anime.f95:370-490: (n, time), u, v, w, p, usum, vsum, wsum."""
        self._check(self.lib.les_gpu_write_data30(self._h, os.fsencode(path), n, time,
                                                  self._io_flags(big_endian)), "write_data30")

    def write_data31(self, path: str, big_endian: bool = True) -> None:
        """data31 of anime.f95:492-595: f, g, h, fold, gold, hold."""
        self._check(self.lib.les_gpu_write_data31(self._h, os.fsencode(path), self._io_flags(big_endian)),
                    "write_data31")

    def write_data10(self, path: str, big_endian: bool = True) -> None:
        """data10 of aveflow.f95:209-263 (aveu, avew, avev), after aveflow at nmax."""
        self._check(self.lib.les_gpu_write_data10(self._h, os.fsencode(path), self._io_flags(big_endian)),
                    "write_data10")

    def write_data11(self, path: str, big_endian: bool = True) -> None:
        """data11 of aveflow.f95:273-344 (aveuu, aveww, avevv, uwfx), after aveflow at nmax."""
        self._check(self.lib.les_gpu_write_data11(self._h, os.fsencode(path), self._io_flags(big_endian)),
                    "write_data11")

    def ifdata_out(self, directory: str, n: int, n1: int, nmax: int, time: float,
                   big_endian: bool = True) -> bool:
        """ifdata_out of anime.f95:326 (after every step, main.f95:318): writes
        data30NNNNNN.dat and data31NNNNNN.dat into `directory` when n == n1-1 or
        n == nmax; returns whether it wrote."""
        w = C.c_int(0)
        self._check(self.lib.les_gpu_ifdata_out(self._h, os.fsencode(directory), n, n1, nmax, time,
                                                self._io_flags(big_endian), C.byref(w)), "ifdata_out")
        return bool(w.value)

    def read_restart(self, data30: str, data31: str) -> tuple[int, float]:
        """The restart read of ifdata.f95:252-480: loads the interiors of the 13 state
        fields from data30/data31 (either byte order); returns (n, time)."""
        n, t = C.c_int(0), C.c_float(0.0)
        self._check(self.lib.les_gpu_read_restart(self._h, os.fsencode(data30), os.fsencode(data31),
                                                  C.byref(n), C.byref(t)), "read_restart")
        return n.value, t.value

    def set_sor_shape(self, nx: int = 0, ny: int = 0, kchunk: int = 0, depth: int = 0) -> None:
        """Fix the SOR sweep's tile shape and fusion depth (0 = automatic); see
        les_gpu_set_sor_shape."""
        self._check(self.lib.les_gpu_set_sor_shape(self._h, nx, ny, kchunk, depth), "set_sor_shape")

    def sor_shape(self) -> tuple[int, int, int, int]:
        """(nx, ny, kchunk, depth) of the SOR sweep in use; zeros for the per-subroutine path."""
        out = (C.c_int * 4)()
        self._check(self.lib.les_gpu_sor_shape(self._h, out), "sor_shape")
        return tuple(int(x) for x in out)

    def tune_sor(self, shared: bool) -> tuple[tuple[int, int, int, int], float, str]:
        """Time the SOR tile shapes and fusion depths for this domain's size class (alone,
        or sharing the GPU with other domains), keep the fastest for the class; returns
        (shape, microseconds per iteration, report of every candidate)."""
        out = (C.c_int * 4)()
        us = C.c_double(0.0)
        rep = C.create_string_buffer(16384)
        self._check(self.lib.les_gpu_tune_sor(self._h, 1 if shared else 0, out, C.byref(us), rep, 16384),
                    "tune_sor")
        return tuple(int(x) for x in out), us.value, rep.value.decode()

    def profile(self, what: int, reps: int) -> float:
        """Average ms per repetition of one stage (it really runs and advances the state)."""
        ms = C.c_double(0.0)
        self._check(self.lib.les_gpu_profile(self._h, what, reps, C.byref(ms)), "profile")
        return ms.value

    def launch_count(self) -> int:
        return int(self.lib.les_gpu_launch_count(self._h))


class Batch:
    """Many resident domains stepped together (les_batch_*), members joining and leaving
    between steps: each member's whole-step graph on its own stream, or (persistent_sor)
    each member's step around one persistent SOR launch over all members' tiles."""

    def __init__(self, persistent_sor: bool = False):
        self.lib = load_library()
        self._b = C.c_void_p()
        rc = self.lib.les_batch_create(C.byref(self._b))
        if rc:
            raise RuntimeError(f"les_batch_create failed ({rc})")
        self.members: dict[int, Domain] = {}
        if persistent_sor:
            self.set_sor_launch(True)

    def _check(self, rc: int, what: str):
        if rc:
            buf = C.create_string_buffer(512)
            self.lib.les_batch_last_error(self._b, buf, 512)
            raise RuntimeError(f"les_batch_{what} failed ({rc}): {buf.value.decode(errors='replace')}")

    @staticmethod
    def admit(im: int, jm: int, km: int, reserve_bytes: int = 0) -> bool:
        """Whether the device's free memory holds one more domain of these dims."""
        lib = load_library()
        ok = C.c_int(0)
        rc = lib.les_batch_admit(C.byref(LesDims(im, jm, km)), reserve_bytes, C.byref(ok))
        if rc:
            raise RuntimeError(f"les_batch_admit failed ({rc})")
        return bool(ok.value)

    def add(self, dom: "Domain", n0: int, nmax: int) -> int:
        slot = C.c_int(-1)
        self._check(self.lib.les_batch_add(self._b, dom._h, n0, nmax, C.byref(slot)), "add")
        self.members[slot.value] = dom
        return slot.value

    def remove(self, slot: int) -> "Domain":
        self._check(self.lib.les_batch_remove(self._b, slot), "remove")
        return self.members.pop(slot)

    def step(self) -> int:
        """One step of every unfinished member; returns the members with steps left."""
        live = C.c_int(0)
        self._check(self.lib.les_batch_step(self._b, C.byref(live)), "step")
        return live.value

    def sync(self):
        self._check(self.lib.les_batch_sync(self._b), "sync")

    def set_sor_launch(self, persistent: bool) -> None:
        """True: SOR iterations 2..nmaxp of all members in one persistent launch over their
        tiles; False (default): each member's whole-step graph on its own stream."""
        self._check(self.lib.les_batch_set_sor_launch(self._b, 1 if persistent else 0), "set_sor_launch")

    def set_wait_limit(self, polls: int, hold_slot: int = -1) -> None:
        """Bound the batched SOR launch's dependency waits (polls of about 128 ns); a
        hold_slot >= 0 makes that member's wait impossible (the give-up path, for tests)."""
        self._check(self.lib.les_batch_set_wait_limit(self._b, polls, hold_slot), "set_wait_limit")

    def progress(self, slot: int) -> tuple[int, int]:
        """(next step index, nmax) of a member; finished once next > nmax."""
        n, nmax = C.c_int(0), C.c_int(0)
        self._check(self.lib.les_batch_slot(self._b, slot, C.byref(n), C.byref(nmax)), "slot")
        return n.value, nmax.value

    def close(self):
        if self._b:
            self.lib.les_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
