"""Python binding of the C ABI in include/gbmd.h (ctypes over libgbmd.so).

This is the Python face of the same boundary the C++ adapter classes in
``cabanamd_gb300/host`` use.  There is no CPU fallback: if libgbmd.so is
missing or no CUDA device is present, constructing a :class:`Context`
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libgbmd.so"

GBMD_OK = 0
ERR_NAMES = {1: "ARG", 2: "CUDA", 3: "CAPACITY", 4: "LOST_ATOM", 5: "TIMEOUT", 6: "IO",
             7: "NODEVICE", 8: "CANCELLED"}
PREC_FP64 = 0
PREC_MIXED = 1
FORCE_LJ = 0
FORCE_NNP = 1
KT = {"force": 0, "neigh": 1, "sort": 2, "integrate": 3, "thermo": 4, "nnp_sf": 5,
      "nnp_mlp": 6, "nnp_force": 7}


class GbmdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbmd error {code} ({ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


class MDParams(C.Structure):
    _fields_ = [("force_cut", C.c_double), ("skin", C.c_double), ("half", C.c_int),
                ("rebuild_every", C.c_int), ("thermo_every", C.c_int),
                ("max_neigh_guess", C.c_int)]


# Every symbol declared in include/gbmd.h (checked by tests/test_abi.py).
EXPORTS = [
    "gbmd_create", "gbmd_destroy", "gbmd_last_error", "gbmd_version", "gbmd_set_units",
    "gbmd_set_box", "gbmd_set_types", "gbmd_set_precision", "gbmd_upload_atoms",
    "gbmd_host_register", "gbmd_host_unregister",
    "gbmd_download_atoms", "gbmd_num_atoms", "gbmd_exchange", "gbmd_binning",
    "gbmd_neigh_build", "gbmd_set_list_images", "gbmd_check_bounded_wait", "gbmd_neigh_size",
    "gbmd_neigh_download", "gbmd_lj_coeff",
    "gbmd_set_force_type", "gbmd_zero_force", "gbmd_force_compute", "gbmd_force_energy",
    "gbmd_integrate_initial", "gbmd_integrate_final", "gbmd_scale_velocities",
    "gbmd_thermo", "gbmd_thermo_noalloc", "gbmd_md_init",
    "gbmd_md_run", "gbmd_md_step_count", "gbmd_md_last_run", "gbmd_set_graphs",
    "gbmd_graph_replays", "gbmd_set_tuning", "gbmd_set_shapes", "gbmd_get_shapes",
    "gbmd_nnp_load",
    "gbmd_nnp_download",
    "gbmd_set_profiling", "gbmd_kernel_time", "gbmd_synchronize",
    # include/gbmd_serve.h (wrapped by cabanamd_gb300.serve)
    "gbmd_engine_create", "gbmd_engine_destroy", "gbmd_engine_last_error", "gbmd_engine_now",
    "gbmd_job_submit", "gbmd_engine_step", "gbmd_job_poll", "gbmd_job_error",
    "gbmd_job_result", "gbmd_job_release", "gbmd_job_cancel", "gbmd_engine_get_stats",
]

_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libgbmd.so (built by cabanamd_gb300.build.build_lib)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    # GBMD_LIBRARY points at an alternative build of the same library
    # (e.g. one compiled with different tile constants).
    p = Path(path) if path else Path(os.environ.get("GBMD_LIBRARY", LIB_PATH))
    if not p.exists():
        raise FileNotFoundError(
            f"{p} not found: build the CUDA library first (python -c 'import __graft_entry__ as g;"
            " g.build()')")
    L = C.CDLL(str(p))
    vp = C.c_void_p
    D = C.POINTER(C.c_double)
    i64 = C.c_int64
    L.gbmd_create.argtypes = [C.POINTER(vp), C.c_int]
    L.gbmd_destroy.argtypes = [vp]
    L.gbmd_destroy.restype = None
    L.gbmd_last_error.argtypes = [vp]
    L.gbmd_last_error.restype = C.c_char_p
    L.gbmd_set_units.argtypes = [vp, C.c_double, C.c_double, C.c_double]
    L.gbmd_set_box.argtypes = [vp, D, D]
    L.gbmd_set_types.argtypes = [vp, C.c_int, D]
    L.gbmd_set_precision.argtypes = [vp, C.c_int]
    L.gbmd_upload_atoms.argtypes = [vp, i64, vp, vp, vp, vp]
    L.gbmd_download_atoms.argtypes = [vp, vp, vp, vp, vp, vp]
    L.gbmd_host_register.argtypes = [vp, C.c_size_t]
    L.gbmd_host_unregister.argtypes = [vp]
    L.gbmd_num_atoms.argtypes = [vp, C.POINTER(i64)]
    L.gbmd_exchange.argtypes = [vp]
    L.gbmd_binning.argtypes = [vp, C.c_double]
    L.gbmd_neigh_build.argtypes = [vp, C.c_double, C.c_int, C.c_int]
    L.gbmd_set_list_images.argtypes = [vp, C.c_int]
    L.gbmd_check_bounded_wait.argtypes = [vp, C.c_double]
    L.gbmd_neigh_size.argtypes = [vp, C.POINTER(i64), C.POINTER(C.c_int32)]
    L.gbmd_neigh_download.argtypes = [vp, vp, vp, vp]
    L.gbmd_lj_coeff.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
    L.gbmd_set_force_type.argtypes = [vp, C.c_int]
    L.gbmd_zero_force.argtypes = [vp]
    L.gbmd_force_compute.argtypes = [vp]
    L.gbmd_force_energy.argtypes = [vp, D]
    L.gbmd_integrate_initial.argtypes = [vp]
    L.gbmd_integrate_final.argtypes = [vp]
    L.gbmd_thermo.argtypes = [vp, D, D]
    L.gbmd_scale_velocities.argtypes = [vp, C.c_double]
    L.gbmd_thermo_noalloc.argtypes = [vp, vp, vp, i64, C.c_double, C.c_double, vp, vp]
    L.gbmd_md_init.argtypes = [vp, C.POINTER(MDParams), D]
    L.gbmd_md_run.argtypes = [vp, C.c_int, D, C.c_int, C.POINTER(C.c_int)]
    L.gbmd_md_step_count.argtypes = [vp, C.POINTER(i64)]
    L.gbmd_md_last_run.argtypes = [vp, D, C.POINTER(i64)]
    L.gbmd_set_graphs.argtypes = [vp, C.c_int]
    L.gbmd_graph_replays.argtypes = [vp, C.POINTER(i64)]
    L.gbmd_set_tuning.argtypes = [vp, C.c_int]
    L.gbmd_set_shapes.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.gbmd_get_shapes.argtypes = [vp, C.POINTER(C.c_int)]
    L.gbmd_nnp_load.argtypes = [vp, C.c_char_p, C.c_double, C.c_double]
    L.gbmd_nnp_download.argtypes = [vp, vp, vp, C.POINTER(C.c_int)]
    L.gbmd_set_profiling.argtypes = [vp, C.c_int]
    L.gbmd_kernel_time.argtypes = [vp, C.c_int, D, C.POINTER(i64)]
    L.gbmd_synchronize.argtypes = [vp]
    from . import serve as _serve  # serving-engine signatures
    _serve.declare(L)
    if path is None:
        _lib = L
    return L


def aligned_empty(shape, dtype, align: int = 65536) -> np.ndarray:
    """An uninitialised array whose data starts on an `align`-byte boundary
    (a whole number of host pages, so that pinning it with host_register
    locks only its own pages)."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    raw = np.empty(nbytes + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off:off + nbytes].view(dt).reshape(shape)


class PinnedHost:
    """Page-locks and maps numpy arrays for the lifetime of the object
    (gbmd_host_register), so that upload_atoms / download_atoms read and
    write them in place from the GPU, over the host link."""

    def __init__(self, *arrays):
        self.lib = load_library()
        self.ptrs = []
        for a in arrays:
            if not a.flags.c_contiguous:
                raise ValueError("PinnedHost: arrays must be C-contiguous")
            rc = self.lib.gbmd_host_register(a.ctypes.data, a.nbytes)
            if rc != GBMD_OK:
                self.close()
                raise GbmdError(rc, "gbmd_host_register failed")
            self.ptrs.append(a.ctypes.data)
        self.arrays = arrays

    def close(self):
        for p in self.ptrs:
            self.lib.gbmd_host_unregister(p)
        self.ptrs = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ptr(a):
    return None if a is None else a.ctypes.data


@dataclass
class Atoms:
    x: np.ndarray
    v: np.ndarray
    f: np.ndarray
    type: np.ndarray
    id: np.ndarray

    def by_id(self) -> "Atoms":
        o = np.argsort(self.id, kind="stable")
        return Atoms(self.x[o], self.v[o], self.f[o], self.type[o], self.id[o])


class Context:
    """One gbmd context: a System plus its modules on one GPU stream."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.gbmd_create(C.byref(h), device)
        if rc != GBMD_OK:
            raise GbmdError(rc, "gbmd_create failed (no CUDA device or bad device index)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbmd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc: int):
        if rc != GBMD_OK:
            raise GbmdError(rc, self.last_error())

    def last_error(self) -> str:
        return self.lib.gbmd_last_error(self.h).decode()

    # System
    def set_units(self, boltz, mvv2e, dt):
        self._chk(self.lib.gbmd_set_units(self.h, boltz, mvv2e, dt))

    def set_box(self, lo, hi):
        lo = np.ascontiguousarray(lo, np.float64)
        hi = np.ascontiguousarray(hi, np.float64)
        self._chk(self.lib.gbmd_set_box(self.h, _dp(lo), _dp(hi)))

    def set_types(self, mass):
        m = np.ascontiguousarray(mass, np.float64)
        self._chk(self.lib.gbmd_set_types(self.h, len(m), _dp(m)))

    def set_precision(self, prec: int):
        self._chk(self.lib.gbmd_set_precision(self.h, prec))

    def upload_atoms(self, x, v, type_, id_):
        x = np.ascontiguousarray(x, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        t = np.ascontiguousarray(type_, np.int32)
        i = np.ascontiguousarray(id_, np.int32)
        self._chk(self.lib.gbmd_upload_atoms(self.h, len(x), x.ctypes.data, _ptr(v),
                                             t.ctypes.data, i.ctypes.data))

    def num_atoms(self) -> int:
        n = C.c_int64()
        self._chk(self.lib.gbmd_num_atoms(self.h, C.byref(n)))
        return n.value

    def download_atoms(self, out: Atoms | None = None) -> Atoms:
        """The atoms in the current order; into `out`'s arrays when given
        (e.g. pinned host mirrors, see PinnedHost)."""
        n = self.num_atoms()
        if out is not None:
            if out.x.shape != (n, 3) or len(out.id) != n:
                raise ValueError("download_atoms: out has the wrong size")
            x, v, f, t, i = out.x, out.v, out.f, out.type, out.id
        else:
            x = np.zeros((n, 3))
            v = np.zeros((n, 3))
            f = np.zeros((n, 3))
            t = np.zeros(n, np.int32)
            i = np.zeros(n, np.int32)
        self._chk(self.lib.gbmd_download_atoms(self.h, x.ctypes.data, v.ctypes.data,
                                               f.ctypes.data, t.ctypes.data, i.ctypes.data))
        return Atoms(x, v, f, t, i)

    # Comm / Binning / Neighbor
    def exchange(self):
        self._chk(self.lib.gbmd_exchange(self.h))

    def binning(self, cut):
        self._chk(self.lib.gbmd_binning(self.h, cut))

    def neigh_build(self, cut, half, max_neigh_guess=50):
        self._chk(self.lib.gbmd_neigh_build(self.h, cut, int(half), int(max_neigh_guess)))

    def check_bounded_wait(self, seconds: float = 0.05) -> int:
        """Run a device wait that expires (nothing completes it); returns
        the status code (GBMD_ERR_TIMEOUT when the bound works)."""
        return int(self.lib.gbmd_check_bounded_wait(self.h, float(seconds)))

    def set_list_images(self, periodic: bool):
        """False: lists without periodic images (CabanaMD's tree lists)."""
        self._chk(self.lib.gbmd_set_list_images(self.h, int(bool(periodic))))

    def neigh_size(self):
        t = C.c_int64()
        m = C.c_int32()
        self._chk(self.lib.gbmd_neigh_size(self.h, C.byref(t), C.byref(m)))
        return t.value, m.value

    def neigh_download(self):
        n = self.num_atoms()
        tot, _ = self.neigh_size()
        cnt = np.zeros(n, np.int32)
        j = np.zeros(max(tot, 1), np.int32)
        img = np.zeros(max(tot, 1), np.int8)
        self._chk(self.lib.gbmd_neigh_download(self.h, cnt.ctypes.data, j.ctypes.data,
                                               img.ctypes.data))
        off = np.zeros(n + 1, np.int64)
        np.cumsum(cnt, out=off[1:])
        return off, j[:tot], img[:tot]

    # Force
    def lj_coeff(self, i, j, eps, sigma, cut):
        self._chk(self.lib.gbmd_lj_coeff(self.h, i, j, eps, sigma, cut))

    def set_force_type(self, ft):
        self._chk(self.lib.gbmd_set_force_type(self.h, ft))

    def zero_force(self):
        self._chk(self.lib.gbmd_zero_force(self.h))

    def force_compute(self):
        self._chk(self.lib.gbmd_force_compute(self.h))

    def force_energy(self) -> float:
        e = C.c_double()
        self._chk(self.lib.gbmd_force_energy(self.h, C.byref(e)))
        return e.value

    # Integrator / thermo
    def integrate_initial(self):
        self._chk(self.lib.gbmd_integrate_initial(self.h))

    def integrate_final(self):
        self._chk(self.lib.gbmd_integrate_final(self.h))

    def scale_velocities(self, factor):
        self._chk(self.lib.gbmd_scale_velocities(self.h, float(factor)))

    def thermo(self):
        T = C.c_double()
        KE = C.c_double()
        self._chk(self.lib.gbmd_thermo(self.h, C.byref(T), C.byref(KE)))
        return T.value, KE.value

    # Whole loop
    def md_init(self, force_cut, skin, half, rebuild_every=20, thermo_every=10,
                max_neigh_guess=50):
        p = MDParams(force_cut, skin, int(half), rebuild_every, thermo_every, max_neigh_guess)
        row = np.zeros(4)
        self._chk(self.lib.gbmd_md_init(self.h, C.byref(p), _dp(row)))
        return row

    def md_run(self, nsteps, max_rows=None):
        if max_rows is None:
            max_rows = nsteps + 1
        rows = np.zeros((max(max_rows, 1), 4))
        nr = C.c_int()
        self._chk(self.lib.gbmd_md_run(self.h, int(nsteps), _dp(rows), int(max_rows),
                                       C.byref(nr)))
        return rows[:nr.value]

    def last_run(self):
        """(device ms, kernel launches) of the last md_run."""
        ms = C.c_double()
        n = C.c_int64()
        self._chk(self.lib.gbmd_md_last_run(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_graphs(self, on: bool):
        """CUDA graphs of md_run's fused LJ steps (on by default)."""
        self._chk(self.lib.gbmd_set_graphs(self.h, int(on)))

    def graph_replays(self) -> int:
        r = C.c_int64()
        self._chk(self.lib.gbmd_graph_replays(self.h, C.byref(r)))
        return r.value

    def set_tuning(self, on: bool):
        """Autotune the tile shapes at md_init (on by default)."""
        self._chk(self.lib.gbmd_set_tuning(self.h, int(bool(on))))

    def set_shapes(self, lj_threads=128, lj_prefetch=16, nb_warps=12, nb_out=32):
        """Fix the tile shapes (switches tuning off)."""
        self._chk(self.lib.gbmd_set_shapes(self.h, lj_threads, lj_prefetch, nb_warps, nb_out))

    def shapes(self) -> dict:
        v = (C.c_int * 5)()
        self._chk(self.lib.gbmd_get_shapes(self.h, v))
        return {"lj_threads": v[0], "lj_prefetch": v[1], "nb_warps": v[2], "nb_out": v[3],
                "tuned": bool(v[4])}

    def step_count(self):
        s = C.c_int64()
        self._chk(self.lib.gbmd_md_step_count(self.h, C.byref(s)))
        return s.value

    # NNP
    def nnp_load(self, directory, cflength=1.0, cfenergy=1.0):
        self._chk(self.lib.gbmd_nnp_load(self.h, str(directory).encode(), cflength, cfenergy))

    def nnp_download(self):
        n = self.num_atoms()
        nsf = C.c_int()
        self._chk(self.lib.gbmd_nnp_download(self.h, None, None, C.byref(nsf)))
        G = np.zeros((n, nsf.value))
        E = np.zeros(n)
        self._chk(self.lib.gbmd_nnp_download(self.h, G.ctypes.data, E.ctypes.data,
                                             C.byref(nsf)))
        return G, E

    # Timing
    def set_profiling(self, on: bool):
        self._chk(self.lib.gbmd_set_profiling(self.h, int(on)))

    def kernel_time(self, which: str):
        ms = C.c_double()
        cnt = C.c_int64()
        self._chk(self.lib.gbmd_kernel_time(self.h, KT[which], C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    def synchronize(self):
        self._chk(self.lib.gbmd_synchronize(self.h))
