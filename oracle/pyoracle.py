"""ctypes binding of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import build_oracle

MAXT = 8
IMG_ZERO = 13


class Grid(C.Structure):
    _fields_ = [("nc", C.c_int * 3), ("h", C.c_double * 3), ("lo", C.c_double * 3),
                ("L", C.c_double * 3)]


class LJ(C.Structure):
    _fields_ = [("ntypes", C.c_int), ("lj1", C.c_double * (MAXT * MAXT)),
                ("lj2", C.c_double * (MAXT * MAXT)), ("cutsq", C.c_double * (MAXT * MAXT))]


class List(C.Structure):
    _fields_ = [("n", C.c_int64), ("off", C.POINTER(C.c_int64)), ("j", C.POINTER(C.c_int32)),
                ("img", C.POINTER(C.c_int8))]


class RunCfg(C.Structure):
    _fields_ = [("force_cut", C.c_double), ("skin", C.c_double), ("half", C.c_int),
                ("rebuild_every", C.c_int), ("thermo_every", C.c_int), ("nsteps", C.c_int),
                ("nthreads", C.c_int), ("boltz", C.c_double), ("mvv2e", C.c_double),
                ("dt", C.c_double), ("ntypes", C.c_int), ("mass", C.c_double * MAXT),
                ("time_from_step", C.c_int), ("loop_seconds", C.c_double)]


_lib = None

_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(str(path))
        P3 = C.c_double * 3
        L.orc_exchange_self.argtypes = [C.c_int64, _D, P3]
        L.orc_make_grid.argtypes = [P3, P3, C.c_double, C.POINTER(Grid)]
        L.orc_sort_atoms.argtypes = [C.c_int64, C.POINTER(Grid), _D, C.c_void_p, C.c_void_p,
                                     _I32, _I32, C.c_void_p]
        L.orc_halo.restype = C.c_int64
        L.orc_halo.argtypes = [C.c_int64, _D, P3, P3, C.c_double,
                               C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_int8))]
        L.orc_neigh_brute.argtypes = [C.c_int64, C.c_int64, _D, C.c_double, C.c_int,
                                      C.POINTER(List)]
        L.orc_image_positions.argtypes = [C.c_int64, _D, C.c_void_p, C.c_void_p, P3, _D]
        L.orc_neigh_cells.argtypes = [C.c_int64, _D, C.POINTER(Grid), P3, C.c_double, C.c_double,
                                      C.c_int, C.c_int, C.POINTER(List)]
        L.orc_list_free.argtypes = [C.POINTER(List)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_lj_init.argtypes = [C.POINTER(LJ), C.c_int]
        L.orc_lj_coeff.argtypes = [C.POINTER(LJ), C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_double]
        L.orc_lj_force.argtypes = [C.c_int64, _D, _I32, C.POINTER(LJ), C.POINTER(List), P3,
                                   C.c_int, C.c_int, _D]
        L.orc_lj_energy.restype = C.c_double
        L.orc_lj_energy.argtypes = [C.c_int64, _D, _I32, C.POINTER(LJ), C.POINTER(List), P3,
                                    C.c_int, C.c_int]
        L.orc_nve_initial.argtypes = [C.c_int64, _D, _D, _D, _I32, _D, C.c_double, C.c_double,
                                      C.c_int]
        L.orc_nve_final.argtypes = [C.c_int64, _D, _D, _I32, _D, C.c_double, C.c_double, C.c_int]
        L.orc_sum_mv2.restype = C.c_double
        L.orc_sum_mv2.argtypes = [C.c_int64, _D, _I32, _D, C.c_int]
        L.orc_run_lj.restype = C.c_int
        L.orc_run_lj.argtypes = [C.c_int64, _D, _D, _D, _I32, _I32, P3, P3, C.POINTER(LJ),
                                 C.POINTER(RunCfg), _D, C.c_int]
        _lib = L
    return _lib


def _p3(a):
    return (C.c_double * 3)(*[float(t) for t in a])


def make_grid(lo, hi, cut) -> Grid:
    g = Grid()
    lib().orc_make_grid(_p3(lo), _p3(hi), float(cut), C.byref(g))
    return g


def exchange_self(x: np.ndarray, L) -> None:
    lib().orc_exchange_self(len(x), x, _p3(L))


def sort_atoms(g: Grid, x, v, f, type_, id_):
    n = len(x)
    perm = np.zeros(n, np.int64)
    lib().orc_sort_atoms(n, C.byref(g), x,
                         v.ctypes.data if v is not None else None,
                         f.ctypes.data if f is not None else None,
                         type_, id_, perm.ctypes.data)
    return perm


def halo(x, lo, hi, depth):
    src = C.POINTER(C.c_int32)()
    img = C.POINTER(C.c_int8)()
    ng = lib().orc_halo(len(x), x, _p3(lo), _p3(hi), float(depth), C.byref(src), C.byref(img))
    s = np.ctypeslib.as_array(src, shape=(max(ng, 1),))[:ng].copy()
    m = np.ctypeslib.as_array(img, shape=(max(ng, 1),))[:ng].copy()
    lib().orc_free(C.cast(src, C.c_void_p))
    lib().orc_free(C.cast(img, C.c_void_p))
    return s, m


def _take_list(lst: List):
    n = lst.n
    off = np.ctypeslib.as_array(lst.off, shape=(n + 1,)).copy()
    tot = int(off[-1])
    if tot:
        j = np.ctypeslib.as_array(lst.j, shape=(tot,)).copy()
        img = np.ctypeslib.as_array(lst.img, shape=(tot,)).copy()
    else:
        j = np.zeros(0, np.int32)
        img = np.zeros(0, np.int8)
    lib().orc_list_free(C.byref(lst))
    return off, j, img


def neigh_brute(x_all, nlocal, cut, half):
    """Brute-force list of the first nlocal of the explicit particles x_all."""
    lst = List()
    x_all = np.ascontiguousarray(x_all, np.float64)
    lib().orc_neigh_brute(int(nlocal), len(x_all), x_all, float(cut), int(half), C.byref(lst))
    off, j, _ = _take_list(lst)
    return off, j


def image_positions(x, gsrc, gimg, L):
    gsrc = np.ascontiguousarray(gsrc, np.int32)
    gimg = np.ascontiguousarray(gimg, np.int8)
    xg = np.zeros((len(gsrc), 3))
    if len(gsrc):
        lib().orc_image_positions(len(gsrc), x, gsrc.ctypes.data, gimg.ctypes.data, _p3(L), xg)
    return xg


def periodic_brute(x, lo, hi, cut, half):
    """Brute force over locals + the single-rank halo ghosts, returned as
    per-atom sorted lists of (partner index, image code) pairs."""
    L = np.asarray(hi, float) - np.asarray(lo, float)
    gsrc, gimg = halo(x, lo, hi, cut)
    xg = image_positions(x, gsrc, gimg, L)
    off, j = neigh_brute(np.vstack([x, xg]) if len(xg) else x, len(x), cut, half)
    n = len(x)
    src = np.where(j < n, j, gsrc[np.clip(j - n, 0, max(len(gsrc) - 1, 0))] if len(gsrc) else j)
    img = np.where(j < n, IMG_ZERO, gimg[np.clip(j - n, 0, max(len(gimg) - 1, 0))]
                   if len(gimg) else IMG_ZERO)
    return off, src.astype(np.int32), img.astype(np.int8)


def neigh_cells(x, g: Grid, hi, depth, cut, half, nthreads=1):
    lst = List()
    rc = lib().orc_neigh_cells(len(x), x, C.byref(g), _p3(hi), float(depth), float(cut),
                               int(half), int(nthreads), C.byref(lst))
    if rc:
        raise RuntimeError("orc_neigh_cells: atoms are not in cell order")
    return _take_list(lst)


class ListHandle:
    """Keeps a CSR list alive in C memory for force/energy calls."""

    def __init__(self, off, j, img):
        self.off = np.ascontiguousarray(off, np.int64)
        self.j = np.ascontiguousarray(j, np.int32)
        self.img = np.ascontiguousarray(img, np.int8)
        self.s = List(len(self.off) - 1,
                      self.off.ctypes.data_as(C.POINTER(C.c_int64)),
                      self.j.ctypes.data_as(C.POINTER(C.c_int32)),
                      self.img.ctypes.data_as(C.POINTER(C.c_int8)))


def lj_params(coeffs, ntypes=1) -> LJ:
    p = LJ()
    lib().orc_lj_init(C.byref(p), ntypes)
    for (i, j, eps, sig, cut) in coeffs:
        lib().orc_lj_coeff(C.byref(p), i - 1, j - 1, eps, sig, cut)
    return p


def lj_force(x, type_, p: LJ, lh: ListHandle, L, half, nthreads=1):
    f = np.zeros_like(x)
    lib().orc_lj_force(len(x), x, type_, C.byref(p), C.byref(lh.s), _p3(L), int(half),
                       int(nthreads), f)
    return f


def lj_energy(x, type_, p: LJ, lh: ListHandle, L, half, nthreads=1):
    return lib().orc_lj_energy(len(x), x, type_, C.byref(p), C.byref(lh.s), _p3(L), int(half),
                               int(nthreads))


def nve_initial(x, v, f, type_, mass, dt, mvv2e, nthreads=1):
    lib().orc_nve_initial(len(x), x, v, f, type_, np.ascontiguousarray(mass, np.float64), dt,
                          mvv2e, nthreads)


def nve_final(v, f, type_, mass, dt, mvv2e, nthreads=1):
    lib().orc_nve_final(len(v), v, f, type_, np.ascontiguousarray(mass, np.float64), dt, mvv2e,
                        nthreads)


def sum_mv2(v, type_, mass, nthreads=1):
    return lib().orc_sum_mv2(len(v), v, type_, np.ascontiguousarray(mass, np.float64), nthreads)


def run_lj(x, v, type_, id_, lo, hi, coeffs, *, force_cut, skin, half, rebuild_every,
           thermo_every, nsteps, boltz, mvv2e, dt, mass, nthreads=1, time_from_step=0,
           timing=None):
    """CbnMD::init + run with the LJ force.  Arrays are modified in place
    (x, v end in the final cell order); returns (thermo rows, f).  When
    ``timing`` is a dict it receives the wall time of steps after
    ``time_from_step``."""
    mass = list(mass)
    cfg = RunCfg(float(force_cut), float(skin), int(half), int(rebuild_every), int(thermo_every),
                 int(nsteps), int(nthreads), float(boltz), float(mvv2e), float(dt), len(mass),
                 (C.c_double * MAXT)(*(mass + [1.0] * (MAXT - len(mass)))),
                 int(time_from_step), 0.0)
    p = lj_params(coeffs, len(mass))
    f = np.zeros_like(x)
    rows_max = (nsteps // thermo_every + 2) if thermo_every > 0 else 1
    th = np.zeros((rows_max, 4))
    nr = lib().orc_run_lj(len(x), x, v, f, type_, id_, _p3(lo), _p3(hi), C.byref(p),
                          C.byref(cfg), th, rows_max)
    if nr < 0:
        raise RuntimeError("orc_run_lj failed")
    if timing is not None:
        timing["loop_seconds"] = cfg.loop_seconds
    return th[:nr], f


# ---------------------------------------------------------------------------
# NNP (oracle/nnp.c)
NNP_MAXSF = 64
NNP_MAXLAYERS = 4


class NNP(C.Structure):
    _fields_ = [("nsf", C.c_int), ("type", C.c_int * NNP_MAXSF),
                ("e1", C.c_int * NNP_MAXSF), ("e2", C.c_int * NNP_MAXSF),
                ("eta", C.c_double * NNP_MAXSF), ("rs", C.c_double * NNP_MAXSF),
                ("lam", C.c_double * NNP_MAXSF), ("zeta", C.c_double * NNP_MAXSF),
                ("rc", C.c_double * NNP_MAXSF), ("gmin", C.c_double * NNP_MAXSF),
                ("gmax", C.c_double * NNP_MAXSF), ("smin", C.c_double), ("smax", C.c_double),
                ("nlayers", C.c_int), ("nodes", C.c_int * (NNP_MAXLAYERS + 1)),
                ("act", C.c_char * (NNP_MAXLAYERS + 1)),
                ("woff", C.c_int * (NNP_MAXLAYERS + 1)), ("boff", C.c_int * (NNP_MAXLAYERS + 1)),
                ("w", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)),
                ("e_offset", C.c_double), ("conv_energy", C.c_double),
                ("mean_energy", C.c_double)]


class NNPHandle:
    """An orc_nnp built from one element of a cabanamd_gb300.nnp_files.Potential,
    keeping the packed weight arrays alive.  Neighbour elements are indices
    into pot.elements (atomic-number order)."""

    def __init__(self, pot, elem=None):
        elem = elem or pot.elements[0]
        m = NNP()
        sfs = pot.symfns[elem]
        m.nsf = len(sfs)
        for k, s in enumerate(sfs):
            m.type[k] = s.type
            m.e1[k] = pot.elements.index(s.neighbors[0])
            m.e2[k] = pot.elements.index(s.neighbors[-1])
            m.eta[k] = s.eta
            m.rs[k] = s.rs
            m.lam[k] = s.lam
            m.zeta[k] = s.zeta
            m.rc[k] = s.rc
            m.gmin[k] = pot.gmin[elem][k]
            m.gmax[k] = pot.gmax[elem][k]
        m.smin, m.smax = pot.smin, pot.smax
        W, B = pot.W[elem], pot.b[elem]
        m.nlayers = len(W)
        m.nodes[0] = m.nsf
        acts = "l" + pot.activations
        wl, bl, wo, bo = [], [], 0, 0
        for l in range(1, m.nlayers + 1):
            m.nodes[l] = W[l - 1].shape[0]
            m.woff[l] = wo
            m.boff[l] = bo
            wl.append(np.ascontiguousarray(W[l - 1], np.float64).ravel())
            bl.append(np.ascontiguousarray(B[l - 1], np.float64).ravel())
            wo += W[l - 1].size
            bo += B[l - 1].size
        m.act = acts.encode()[: NNP_MAXLAYERS + 1]
        self.w = np.concatenate(wl)
        self.b = np.concatenate(bl)
        m.w = self.w.ctypes.data_as(C.POINTER(C.c_double))
        m.b = self.b.ctypes.data_as(C.POINTER(C.c_double))
        m.e_offset = pot.atom_energy.get(elem, 0.0)
        m.conv_energy = 1.0
        m.mean_energy = 0.0
        self.m = m


def _nnp_lib():
    L = lib()
    if not hasattr(L, "_nnp_ready"):
        L.orc_nnp_compute.restype = C.c_double
        L.orc_nnp_compute.argtypes = [C.c_int64, _D, C.POINTER(List), C.c_double * 3,
                                      C.POINTER(NNP), C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
        L.orc_nnp_compute_multi.restype = C.c_double
        L.orc_nnp_compute_multi.argtypes = [C.c_int64, _D, C.c_void_p, C.POINTER(List),
                                            C.c_double * 3, C.c_void_p, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_nnp_energy.restype = C.c_double
        L.orc_nnp_energy.argtypes = [C.c_int64, C.c_double, C.POINTER(NNP)]
        L.orc_nnp_compute_multi_mt.restype = C.c_double
        L.orc_nnp_compute_multi_mt.argtypes = [C.c_int64, _D, C.c_void_p, C.POINTER(List),
                                               C.c_double * 3, C.c_void_p, C.c_int, C.c_int,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_int]
        L.orc_run_nnp.restype = C.c_int
        L.orc_run_nnp.argtypes = [C.c_int64, _D, _D, _D, _I32, _I32, C.c_double * 3,
                                  C.c_double * 3, C.c_void_p, C.c_int, C.POINTER(RunCfg), _D,
                                  C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p]
        L._nnp_ready = True
    return L


def nnp_compute(x, lh: ListHandle, L, h: NNPHandle, forces=True):
    """Returns dict(G, E, dEdG, f, esum, energy)."""
    n = len(x)
    nsf = h.m.nsf
    G = np.zeros((n, nsf))
    E = np.zeros(n)
    dEdG = np.zeros((n, nsf))
    f = np.zeros((n, 3)) if forces else None
    esum = _nnp_lib().orc_nnp_compute(n, x, C.byref(lh.s), _p3(L), C.byref(h.m),
                                      G.ctypes.data, E.ctypes.data, dEdG.ctypes.data,
                                      f.ctypes.data if forces else None)
    energy = _nnp_lib().orc_nnp_energy(n, esum, C.byref(h.m))
    return dict(G=G, E=E, dEdG=dEdG, f=f, esum=esum, energy=energy)


def nnp_compute_mt(x, type_, lh: ListHandle, L, pot, nthreads, forces=True):
    """nnp_compute_multi on nthreads OpenMP threads (forces equal the serial
    ones up to the order of the threads' additions)."""
    hs = [NNPHandle(pot, e) for e in pot.elements]
    arr = (NNP * len(hs))(*[h.m for h in hs])
    n = len(x)
    gs = max(h.m.nsf for h in hs)
    t = np.ascontiguousarray(type_, np.int32)
    G = np.zeros((n, gs))
    E = np.zeros(n)
    f = np.zeros((n, 3)) if forces else None
    esum = _nnp_lib().orc_nnp_compute_multi_mt(n, x, t.ctypes.data, C.byref(lh.s), _p3(L),
                                               C.cast(arr, C.c_void_p), len(hs), gs,
                                               G.ctypes.data, E.ctypes.data, None,
                                               f.ctypes.data if forces else None, int(nthreads))
    return dict(G=G, E=E, f=f, esum=esum, energy=_nnp_lib().orc_nnp_energy(n, esum,
                                                                           C.byref(hs[0].m)))


def run_nnp(x, v, type_, id_, lo, hi, pot, *, force_cut, skin, rebuild_every, thermo_every,
            nsteps, boltz, mvv2e, dt, mass, nthreads=1, snap_step=-1, time_from_step=0,
            timing=None):
    """CbnMD::init + run with the NNP force (full list of cutoff force_cut +
    skin, atoms of type t use element pot.elements[t]).  Arrays are modified
    in place (x, v end in the final cell order).  Returns (thermo rows, f,
    snapshot) where snapshot is None or dict(x, v, f, id) of the state after
    step snap_step, in that step's order."""
    hs = [NNPHandle(pot, e) for e in pot.elements]
    arr = (NNP * len(hs))(*[h.m for h in hs])
    mass = list(mass)
    cfg = RunCfg(float(force_cut), float(skin), 0, int(rebuild_every), int(thermo_every),
                 int(nsteps), int(nthreads), float(boltz), float(mvv2e), float(dt), len(mass),
                 (C.c_double * MAXT)(*(mass + [1.0] * (MAXT - len(mass)))),
                 int(time_from_step), 0.0)
    n = len(x)
    f = np.zeros_like(x)
    rows_max = (nsteps // thermo_every + 2) if thermo_every > 0 else 1
    th = np.zeros((rows_max, 4))
    snap = None
    ptrs = [None] * 4
    if snap_step >= 0:
        snap = dict(x=np.zeros((n, 3)), v=np.zeros((n, 3)), f=np.zeros((n, 3)),
                    id=np.zeros(n, np.int32))
        ptrs = [snap[k].ctypes.data for k in ("x", "v", "f", "id")]
    nr = _nnp_lib().orc_run_nnp(n, x, v, f, type_, id_, _p3(lo), _p3(hi),
                                C.cast(arr, C.c_void_p), len(hs), C.byref(cfg), th, rows_max,
                                int(snap_step), *ptrs)
    if nr < 0:
        raise RuntimeError("orc_run_nnp failed")
    if timing is not None:
        timing["loop_seconds"] = cfg.loop_seconds
    return th[:nr], f, snap


def nnp_compute_multi(x, type_, lh: ListHandle, L, pot, forces=True):
    """Several elements: atom i uses element type_[i] of pot (atomic-number
    order).  G and dEdG rows are padded to the largest function count.
    Returns dict(G, E, dEdG, f, esum, energy, handles)."""
    hs = [NNPHandle(pot, e) for e in pot.elements]
    arr = (NNP * len(hs))(*[h.m for h in hs])
    n = len(x)
    gs = max(h.m.nsf for h in hs)
    t = np.ascontiguousarray(type_, np.int32)
    G = np.zeros((n, gs))
    E = np.zeros(n)
    dEdG = np.zeros((n, gs))
    f = np.zeros((n, 3)) if forces else None
    esum = _nnp_lib().orc_nnp_compute_multi(n, x, t.ctypes.data, C.byref(lh.s), _p3(L),
                                            C.cast(arr, C.c_void_p), len(hs), gs, G.ctypes.data,
                                            E.ctypes.data, dEdG.ctypes.data,
                                            f.ctypes.data if forces else None)
    energy = _nnp_lib().orc_nnp_energy(n, esum, C.byref(hs[0].m))
    return dict(G=G, E=E, dEdG=dEdG, f=f, esum=esum, energy=energy, handles=hs)

