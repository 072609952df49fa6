"""CPU FP64 oracle for GRASP's CI hot path (test infrastructure only).

This package is the checker for the CUDA path. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may
import it; the product library never does.

The C++ restatement lives in ``oracle.cpp`` (built by ``oracle/Makefile``
into ``oracle/_build/liboracle.so``). This module loads it with ctypes and
offers numpy-friendly wrappers whose names follow the reference subroutines
(QUAD, YZK, SLATER, RINTI, GENINTRK, RKINTC, SETHAM, SPICMV2, DSPEVX, GDVD,
INIEST2, MANEIG).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)
_int = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, a few seconds)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class OrList(C.Structure):
    _fields_ = [
        ("nlab", C.c_int64),
        ("lab", _i32),
        ("start", _i64),
        ("loc", _i32),
        ("coeff", _d),
    ]


class OrBlock(C.Structure):
    _fields_ = [("ncf", C.c_int), ("iendc", _i64), ("irow", _i32), ("iq", C.POINTER(C.c_uint8)),
                ("tlist", OrList), ("kmaxf", C.c_int), ("vlists", C.POINTER(OrList)), ("nev", C.c_int),
                ("evec", _d), ("wt", _d)]


class OrDvdParams(C.Structure):
    _fields_ = [
        ("lim", C.c_int), ("ilow", C.c_int), ("ihigh", C.c_int), ("niv", C.c_int),
        ("mblock", C.c_int), ("maxiter", C.c_int),
        ("crite", C.c_double), ("critc", C.c_double), ("critr", C.c_double), ("ortho", C.c_double),
        ("robust", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, _d]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_get_grid.argtypes = [C.c_void_p, _d, _d, _d]
        L.or_get_qic.argtypes = [C.c_void_p, _d, _d]
        L.or_set_orbitals.argtypes = [C.c_void_p, C.c_int, C.c_int, _int, _int, _d, _d]
        L.or_quad.restype = C.c_double
        L.or_quad.argtypes = [C.c_void_p, C.c_int, _d]
        L.or_yzk.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _d]
        L.or_ypot.argtypes = [C.c_void_p, C.c_int, _i32, _d, _d]
        L.or_xpot.argtypes = [C.c_void_p, C.c_int, _i32, _d, _d, _d]
        L.or_cofpot.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(OrCof), C.c_int, _i32, _d, C.c_double,
                                _d, _d, _d]
        L.or_setlag.argtypes = [C.c_void_p, C.c_int, _i32, _d, _int, C.POINTER(OrCof), _d]
        L.or_brintf.restype = C.c_double
        L.or_brintf.argtypes = [C.c_void_p] + [C.c_int] * 6 + [C.c_double, _d, C.c_double]
        L.or_genintbreit.restype = C.c_int64
        L.or_genintbreit.argtypes = [C.c_void_p, C.c_int, C.c_double, _d, C.c_double, _i32, _d, _i32, _int, C.c_int]
        L.or_slater.restype = C.c_double
        L.or_slater.argtypes = [C.c_void_p] + [C.c_int] * 5
        L.or_rinti.restype = C.c_double
        L.or_rinti.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _int]
        L.or_triangrk.argtypes = [C.c_int] * 3
        L.or_genintrk.restype = C.c_int64
        L.or_genintrk.argtypes = [C.c_void_p, C.c_int, _i32, _d, _i32, _int, C.c_int]
        L.or_rkintc.argtypes = [C.c_int, _i32, _d, _i32] + [C.c_int] * 5 + [_d]
        L.or_clrx.restype = C.c_double
        L.or_clrx.argtypes = [C.c_int] * 3
        L.or_setham.argtypes = [C.c_void_p, C.c_int, C.c_int64, _i64, C.POINTER(C.c_uint8),
                                C.POINTER(OrList), C.c_int, C.POINTER(OrList), _d]
        L.or_setcof.argtypes = [C.c_void_p, C.c_int, C.POINTER(OrBlock), C.c_int, C.c_int, C.c_double, C.c_int,
                                _int, _i32, _d, _int, _i32, _d, _int, _i32, _d]
        L.or_shift_eav.restype = C.c_double
        L.or_shift_eav.argtypes = [C.c_int, _i64, _d]
        L.or_spicmv2.argtypes = [C.c_int, C.c_int, _i64, _i32, _d, _d, _d]
        L.or_spodmv.argtypes = [C.c_int, C.c_int, _i64, _i32, _d, C.c_double, _d, _d]
        L.or_dnicmv.argtypes = [C.c_int, C.c_int, _d, _d, _d]
        L.or_dspevx.argtypes = [C.c_int, _d, C.c_int, C.c_int, _d, _d]
        L.or_iniest2.argtypes = [C.c_int, C.c_int, C.c_int, _d, _d, _i64, _i32]
        L.or_gdvd.argtypes = [C.c_int, _i64, _i32, _d, _d, C.POINTER(OrDvdParams), _d, C.c_int64,
                              _int, _int, _int, C.c_int]
        L.or_maneig.argtypes = [C.c_int, C.c_int, C.c_int, _i64, _i32, _d, _d, _d, _int, _int, _int, C.c_int,
                                C.c_int, C.c_int, _d]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


class OrCof(C.Structure):
    """One orbital's SETCOF lists (YPOT's NYA/YA, XPOT's NXA/XA, DACON's NDA/DA)."""
    _fields_ = [("ny", C.c_int), ("nya", _i32), ("ya", _d), ("nx", C.c_int), ("nxa", _i32), ("xa", _d),
                ("nd", C.c_int), ("nda", _i32), ("da", _d)]


def _cof(d, keep):
    arrs = [np.ascontiguousarray(d.get(k, []), t) for k, t in
            (("nya", np.int32), ("ya", np.float64), ("nxa", np.int32), ("xa", np.float64),
             ("nda", np.int32), ("da", np.float64))]
    keep.extend(arrs)
    nya, ya, nxa, xa, nda, da = arrs
    return OrCof(nya.size, _p(nya, _i32), _p(ya, _d), nxa.size, _p(nxa, _i32), _p(xa, _d),
                 nda.size, _p(nda, _i32), _p(da, _d))


class Oracle:
    """One radial grid + orbital set, like the reference's grid_C/wave_C globals."""

    def __init__(self, n=590, rnt=None, h=0.05, c=137.035999139, zz=None, z=None):
        if rnt is None:
            rnt = 2.0e-6 / z if z else 2.0e-6
        self.n, self.rnt, self.h, self.c = n, rnt, h, c
        if zz is None:
            zz = np.full(n, float(z) if z else 0.0)
        self.zz = np.ascontiguousarray(zz, dtype=np.float64)
        self._h = lib().or_create(n, rnt, h, c, _p(self.zz, _d))
        if not self._h:
            raise ValueError("or_create failed")
        self.nw = 0

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_destroy(self._h)
            self._h = None

    def grid(self):
        r = np.zeros(self.n + 10); rp = np.zeros(self.n + 10); rpor = np.zeros(self.n + 10)
        lib().or_get_grid(self._h, _p(r, _d), _p(rp, _d), _p(rpor, _d))
        return r, rp, rpor

    def qic(self):
        c = np.zeros(4); cnc = np.zeros(12)
        lib().or_get_qic(self._h, _p(c, _d), _p(cnc, _d))
        return c, cnc.reshape(3, 4)

    def set_orbitals(self, nak, mf, pf, qf):
        """pf, qf: arrays [nw, ld] (row = orbital); stored column-major like PF(NNNP, NW)."""
        self.nak = np.ascontiguousarray(nak, dtype=np.int32)
        self.mf = np.ascontiguousarray(mf, dtype=np.int32)
        self.pf = np.ascontiguousarray(pf, dtype=np.float64)
        self.qf = np.ascontiguousarray(qf, dtype=np.float64)
        nw, ld = self.pf.shape
        rc = lib().or_set_orbitals(self._h, nw, ld, _p(self.nak, _int), _p(self.mf, _int),
                                   _p(self.pf, _d), _p(self.qf, _d))
        if rc != 0:
            raise ValueError(f"or_set_orbitals failed: {rc}")
        self.nw = nw

    def quad(self, ta, mtp):
        ta = np.array(ta, dtype=np.float64)
        if ta.size < mtp + 3:
            ta = np.concatenate([ta, np.zeros(mtp + 3 - ta.size)])
        return lib().or_quad(self._h, mtp, _p(ta, _d))

    def yzk(self, k, i, j):
        yk = np.zeros(self.n)
        mtp = lib().or_yzk(self._h, k, i, j, _p(yk, _d))
        return yk, mtp

    def ypot(self, nya, ya):
        """YPOT (rmcdhf90/ypot.f90): the direct potential YP(1:N) of the
        coefficient list (NYA labels, YA coefficients)."""
        nya = np.ascontiguousarray(nya, np.int32); ya = np.ascontiguousarray(ya, np.float64)
        yp = np.zeros(self.n)
        if lib().or_ypot(self._h, nya.size, _p(nya, _i32), _p(ya, _d), _p(yp, _d)) != 0:
            raise ValueError("ypot: label outside the orbital set")
        return yp

    def xpot(self, nxa, xa):
        """XPOT (rmcdhf90/xpot.f90): the exchange potential XP(1:N), XQ(1:N)."""
        nxa = np.ascontiguousarray(nxa, np.int32); xa = np.ascontiguousarray(xa, np.float64)
        xp = np.zeros(self.n); xq = np.zeros(self.n)
        if lib().or_xpot(self._h, nxa.size, _p(nxa, _i32), _p(xa, _d), _p(xp, _d), _p(xq, _d)) != 0:
            raise ValueError("xpot: label outside the orbital set")
        return xp, xq

    def cofpot(self, j, ucfj, cof, iecc=(), ecv=(), accy=None):
        """COFPOT after SETCOF (rmcdhf90/cofpot.f90:30-33): YPOT, XPOT, LAGCON,
        DACON of orbital j from its lists (dict nya/ya/nxa/xa/nda/da);
        returns YP, XP, XQ."""
        keep = []
        c = _cof(cof, keep)
        iecc = np.ascontiguousarray(iecc, np.int32); ecv = np.ascontiguousarray(ecv, np.float64)
        accy = self.h ** 6 if accy is None else accy
        yp, xp, xq = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        if lib().or_cofpot(self._h, j, ucfj, C.byref(c), iecc.size, _p(iecc, _i32), _p(ecv, _d), accy,
                           _p(yp, _d), _p(xp, _d), _p(xq, _d)) != 0:
            raise ValueError("cofpot: label outside the orbital set")
        return yp, xp, xq

    def setlag(self, iecc, ucf, lfix, cofs):
        """SETLAG (rmcdhf90/setlag.f90:140-223): ECV of each pair iecc[k] =
        LI + 215 LJ; cofs[orbital - 1] = that orbital's lists."""
        keep = []
        arr = (OrCof * len(cofs))(*[_cof(c, keep) for c in cofs])
        iecc = np.ascontiguousarray(iecc, np.int32); ucf = np.ascontiguousarray(ucf, np.float64)
        lfix = np.ascontiguousarray(lfix, np.int32)
        ecv = np.zeros(iecc.size)
        if lib().or_setlag(self._h, iecc.size, _p(iecc, _i32), _p(ucf, _d), _p(lfix, _int), arr, _p(ecv, _d)) != 0:
            raise ValueError("setlag: bad list or pair")
        return ecv

    def slater(self, a, b, c, d, k):
        return lib().or_slater(self._h, a, b, c, d, k)

    def brintf(self, itype, a, b, c, d, k, wfact, e, accy=None):
        """BRINTF (rci90/brintf.f90): one Breit integral of type 1..6; e = the
        orbital energies, wfact = the frequency scale (bess_C WFACT)."""
        e = np.ascontiguousarray(e, np.float64)
        accy = self.h ** 6 if accy is None else accy
        return lib().or_brintf(self._h, itype, a, b, c, d, k, wfact, _p(e, _d), accy)

    def genintbreit(self, itype, wfact, e, accy=None, nthreads=1):
        """GENINTBREIT1/2 (rci90/genintbreit1.f90, genintbreit2.f90): INDTP,
        VALTP, KSTARTBREIT and J2MAX of the type-1 or type-2 table."""
        e = np.ascontiguousarray(e, np.float64)
        accy = self.h ** 6 if accy is None else accy
        j2 = C.c_int(0)
        kst = np.zeros(64, np.int32)
        nb = lib().or_genintbreit(self._h, itype, wfact, _p(e, _d), accy, None, None, _p(kst, _i32), C.byref(j2),
                                  nthreads)
        ind = np.zeros(nb, np.int32); val = np.zeros(nb)
        lib().or_genintbreit(self._h, itype, wfact, _p(e, _d), accy, _p(ind, _i32), _p(val, _d), _p(kst, _i32),
                             C.byref(j2), nthreads)
        return ind, val, kst[:j2.value + 2].copy(), j2.value

    def rinti(self, j, k, mode=0):
        err = C.c_int(0)
        v = lib().or_rinti(self._h, j, k, mode, C.byref(err))
        if err.value:
            raise ValueError("RINTI: orbitals have different kappa")
        return v

    def genintrk(self, kmax=-1, nthreads=1):
        j2 = C.c_int(0)
        n = lib().or_genintrk(self._h, kmax, None, None, None, C.byref(j2), 1)
        if n < 0:
            raise ValueError("GENINTRK: k beyond KLIMIT")
        kloop = j2.value if kmax < 0 else kmax
        ind = np.zeros(n, np.int32); val = np.zeros(n); ks = np.zeros(kloop + 2, np.int32)
        lib().or_genintrk(self._h, kmax, _p(ind, _i32), _p(val, _d), _p(ks, _i32), C.byref(j2), nthreads)
        return ind, val, ks, j2.value

    def rkintc(self, table, a, b, c, d, k):
        ind, val, ks = table[:3]
        out = C.c_double(0)
        rc = lib().or_rkintc(self.nw, _p(ind, _i32), _p(val, _d), _p(ks, _i32), a, b, c, d, k, C.byref(out))
        if rc != 0:
            raise KeyError("Rkintc Integral not found")
        return out.value

    def setcof(self, blocks, eol, j, ucfj):
        """SETCOF (rmcdhf90/setcof.f90) for orbital j. blocks: dicts with ncf,
        iendc, irow, iq ([ncf x nw] bytes), tlist, vlists (dicts of lab,
        start, loc, coeff), and the mixing data: evec ([ncf x nev]) and wt
        (nev level weights) when eol, else wt = the ncf CSF weights."""
        keep = []

        def mk(d):
            lab = np.ascontiguousarray(d["lab"], np.int32); st = np.ascontiguousarray(d["start"], np.int64)
            loc = np.ascontiguousarray(d["loc"], np.int32); co = np.ascontiguousarray(d["coeff"], np.float64)
            keep.extend([lab, st, loc, co])
            return OrList(lab.size, _p(lab, _i32), _p(st, _i64), _p(loc, _i32), _p(co, _d))

        obs = []
        for b in blocks:
            iendc = np.ascontiguousarray(b["iendc"], np.int64); irow = np.ascontiguousarray(b["irow"], np.int32)
            iq = np.ascontiguousarray(b["iq"], np.uint8); wt = np.ascontiguousarray(b["wt"], np.float64)
            vl = (OrList * max(1, len(b["vlists"])))(*[mk(v) for v in b["vlists"]])
            keep.extend([iendc, irow, iq, wt, vl])
            if eol:
                ev = np.asfortranarray(np.asarray(b["evec"], np.float64).reshape(b["ncf"], -1))
                keep.append(ev)
                evp, nev = _p(ev, _d), ev.shape[1]
            else:
                evp, nev = None, 0
            obs.append(OrBlock(b["ncf"], _p(iendc, _i64), _p(irow, _i32), iq.ctypes.data_as(C.POINTER(C.c_uint8)),
                               mk(b["tlist"]), len(b["vlists"]) - 1, vl, nev, evp, _p(wt, _d)))
        arr = (OrBlock * len(obs))(*obs)
        cap = 4096
        while True:
            ny, nx, nd = C.c_int(), C.c_int(), C.c_int()
            nya = np.zeros(cap, np.int32); ya = np.zeros(cap); nxa = np.zeros(cap, np.int32); xa = np.zeros(cap)
            nda = np.zeros(cap, np.int32); da = np.zeros(cap)
            rc = lib().or_setcof(self._h, len(obs), arr, int(bool(eol)), j, ucfj, cap, C.byref(ny), _p(nya, _i32),
                                 _p(ya, _d), C.byref(nx), _p(nxa, _i32), _p(xa, _d), C.byref(nd), _p(nda, _i32),
                                 _p(da, _d))
            if rc == -2:
                cap = max(ny.value, nx.value, nd.value)
                continue
            return dict(nya=nya[:ny.value].copy(), ya=ya[:ny.value].copy(), nxa=nxa[:nx.value].copy(),
                        xa=xa[:nx.value].copy(), nda=nda[:nd.value].copy(), da=da[:nd.value].copy())

    def setham(self, ncf, nelmnt, iendc, iq, tlist, vlists):
        """tlist / vlists: dicts with 'lab', 'start', 'loc', 'coeff' numpy arrays."""
        keep = []

        def mk(d):
            lab = np.ascontiguousarray(d["lab"], np.int32); st = np.ascontiguousarray(d["start"], np.int64)
            loc = np.ascontiguousarray(d["loc"], np.int32); co = np.ascontiguousarray(d["coeff"], np.float64)
            keep.extend([lab, st, loc, co])
            return OrList(lab.size, _p(lab, _i32), _p(st, _i64), _p(loc, _i32), _p(co, _d))

        tl = mk(tlist)
        vl = (OrList * len(vlists))(*[mk(v) for v in vlists])
        emt = np.zeros(nelmnt)
        iendc = np.ascontiguousarray(iendc, np.int64)
        iq = np.ascontiguousarray(iq, np.uint8)
        rc = lib().or_setham(self._h, ncf, nelmnt, _p(iendc, _i64), _p(iq, C.POINTER(C.c_uint8)),
                             C.byref(tl), len(vlists) - 1, vl, _p(emt, _d))
        if rc != 0:
            raise ValueError("SETHAM: LOC beyond NELMNT")
        return emt


def shift_eav(ncf, iendc, emt):
    iendc = np.ascontiguousarray(iendc, np.int64)
    return lib().or_shift_eav(ncf, _p(iendc, _i64), _p(emt, _d))


def spicmv2(n, iendc, irow, emt, b):
    b = np.asfortranarray(b.reshape(n, -1), dtype=np.float64)
    m = b.shape[1]
    c = np.zeros((n, m), order="F")
    iendc = np.ascontiguousarray(iendc, np.int64); irow = np.ascontiguousarray(irow, np.int32)
    emt = np.ascontiguousarray(emt, np.float64)
    lib().or_spicmv2(n, m, _p(iendc, _i64), _p(irow, _i32), _p(emt, _d), _p(b, _d), _p(c, _d))
    return c


def spodmv(n, iendc, irow, emt, eav, b):
    """SPODMV's C = (H - EAV) B from rows with the diagonal unshifted."""
    b = np.asfortranarray(b.reshape(n, -1), dtype=np.float64)
    m = b.shape[1]
    c = np.zeros((n, m), order="F")
    iendc = np.ascontiguousarray(iendc, np.int64); irow = np.ascontiguousarray(irow, np.int32)
    emt = np.ascontiguousarray(emt, np.float64)
    lib().or_spodmv(n, m, _p(iendc, _i64), _p(irow, _i32), _p(emt, _d), float(eav), _p(b, _d), _p(c, _d))
    return c


def dnicmv(n, ap, b):
    """DNICMV's C = A B, A's lower triangle packed by rows."""
    b = np.asfortranarray(b.reshape(n, -1), dtype=np.float64)
    m = b.shape[1]
    c = np.zeros((n, m), order="F")
    ap = np.ascontiguousarray(ap, np.float64)
    lib().or_dnicmv(n, m, _p(ap, _d), _p(b, _d), _p(c, _d))
    return c


def dspevx(ap, n, il, iu):
    ap = np.ascontiguousarray(ap, np.float64)
    m = iu - il + 1
    w = np.zeros(m); z = np.zeros((m, n))
    rc = lib().or_dspevx(n, _p(ap, _d), il, iu, _p(w, _d), _p(z, _d))
    if rc:
        raise ValueError("dspevx failed")
    return w, z.T


def maneig(flavour, ncf, nvec, iendc, irow, emt, nthreads=1, robust=False, maxiter=0):
    iendc = np.ascontiguousarray(iendc, np.int64); irow = np.ascontiguousarray(irow, np.int32)
    emt = np.ascontiguousarray(emt, np.float64)
    ev = np.zeros(nvec); vec = np.zeros((nvec, ncf))
    nl, nm, ie = C.c_int(0), C.c_int(0), C.c_int(0)
    secs = np.zeros(2)
    rc = lib().or_maneig(flavour, ncf, nvec, _p(iendc, _i64), _p(irow, _i32), _p(emt, _d), _p(ev, _d),
                         _p(vec, _d), C.byref(nl), C.byref(nm), C.byref(ie), nthreads, int(robust), int(maxiter),
                         _p(secs, _d))
    if rc < 0:
        raise RuntimeError(f"MANEIG failed rc={rc} ierr={ie.value}")
    return ev, vec.T, dict(nloops=nl.value, nmv=nm.value, ierr=ie.value, t_iniest2=secs[0], t_dvdson=secs[1])


def clrx(ka, k, kb):
    return lib().or_clrx(ka, k, kb)


def triangrk(la, k, lb):
    return bool(lib().or_triangrk(la, k, lb))
