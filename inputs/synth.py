"""Seeded synthetic inputs with the reference's formats (see inputs/grasp_synth.h).

Orbital sets, screened-hydrogenic Dirac spinors (DCBSRW at Z - sigma), and
CI blocks (CSF occupations, mcp.30 structure, T/V lists).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)
_int = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)


def ptr(a, t):
    return a.ctypes.data_as(t)


class GSBlockSpec(C.Structure):
    _fields_ = [
        ("nw", C.c_int), ("np", _int), ("nak", _int), ("frozen", _u8), ("nref", C.c_int), ("refs", _u8),
        ("max_rank", C.c_int), ("two_j", C.c_int), ("parity", C.c_int), ("kmaxf", C.c_int),
        ("max_ncf", C.c_int64), ("density", C.c_double), ("coeff_scale", C.c_double), ("seed", C.c_uint64),
    ]


# symbol name -> (restype, argtypes); every symbol grasp_synth.h declares
SYNTH_SYMBOLS = {
    "gs_dcbsrw": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, _d, C.c_int, C.c_double, _d, _d, _d, _d, _int]),
    "gs_screenpar": (C.c_int, [C.c_int, _int, C.c_int, _d]),
    "gs_block_generate": (C.c_int, [C.POINTER(GSBlockSpec), C.POINTER(C.c_void_p)]),
    "gs_block_free": (None, [C.c_void_p]),
    "gs_block_sizes": (C.c_int, [C.c_void_p, _int, _i64, _int, _int, _i64, _i64]),
    "gs_block_structure": (C.c_int, [C.c_void_p, _i64, _i32, _u8]),
    "gs_block_list": (C.c_int, [C.c_void_p, C.c_int, _i32, _i64, _i32, _i32, _d]),
    "gs_synthetic_h": (C.c_int, [C.c_int, C.c_double, C.c_uint64, _i64, _i32, _d]),
}

_synth = None


def lib():
    """libgraspsynth, built on first use."""
    global _synth
    if _synth is None:
        _build.build()
        _synth = C.CDLL(_build.LIB_SYNTH)
        for name, (res, args) in SYNTH_SYMBOLS.items():
            f = getattr(_synth, name)
            f.restype = res
            f.argtypes = args
    return _synth


def check(status):
    if status != 0:
        raise ValueError(f"synthetic-input generator rejected its arguments (status {status})")
    return status

CVAC = 137.035999139  # lib9290/setcon.f90:25 (ALFAI)
NNNP = 590            # parameter_def_M.f90:23


def lval(kappa):
    return kappa if kappa > 0 else -kappa - 1


def nkj(kappa):
    return 2 * abs(kappa) - 1


def orbital_set(nmax, lmax, kappa_max=None):
    """GRASP orbital order: n ascending, then l, kappa = -(l+1) before +l... as
    rcsfgenerate lists subshells (ns, np-, np, nd-, nd, ...)."""
    out = []
    for n in range(1, nmax + 1):
        for l in range(0, min(n - 1, lmax) + 1):
            kaps = [-1] if l == 0 else [l, -(l + 1)]
            for k in kaps:
                if kappa_max is not None and abs(k) > kappa_max:
                    continue
                out.append((n, k))
    return out


def grid(n=NNNP, z=1.0, h=0.05):
    """RADGRD exponential grid (HP = 0), RNT = 2e-6 / Z (rci90/getcid.f90:233-237).
    Returns r[n + 10] (R(1..N+10))."""
    rnt = 2.0e-6 / z
    i = np.arange(n + 10, dtype=np.float64)
    ett = np.ones(n + 10)
    eph = np.exp(h)
    e = 1.0
    r = np.zeros(n + 10)
    for k in range(1, n + 10):
        e = eph * e
        r[k] = rnt * (e - 1.0)
    del i, ett
    return rnt, r


def dcbsrw(n, kappa, z, r, ntp, c=CVAC, accy=None, h=0.05):
    if accy is None:
        accy = (h * h * h) ** 2
    r = np.ascontiguousarray(r, np.float64)
    p = np.zeros(ntp); q = np.zeros(ntp)
    e = C.c_double(); pz = C.c_double(); mtp = C.c_int()
    rc = lib().gs_dcbsrw(n, kappa, float(z), c, ptr(r, _d), ntp, accy, C.byref(e), C.byref(pz), ptr(p, _d),
                                ptr(q, _d), C.byref(mtp))
    if rc != 0:
        raise ValueError(f"DCBSRW: invalid (n={n}, kappa={kappa}, z={z})")
    return p, q, mtp.value, e.value, pz.value


@dataclass
class Orbitals:
    np_: np.ndarray
    nak: np.ndarray
    mf: np.ndarray
    pf: np.ndarray  # [nw, ld]
    qf: np.ndarray
    e: np.ndarray
    zeff: np.ndarray

    @property
    def nw(self):
        return len(self.nak)


def hydrogenic_orbitals(orbs, z, sigma, r, n=NNNP, c=CVAC, h=0.05, ld=None):
    """Screened hydrogenic orbitals, FRMHYD style: DCBSRW at Z_eff = Z - sigma."""
    ld = ld or n
    nw = len(orbs)
    pf = np.zeros((nw, ld)); qf = np.zeros((nw, ld))
    mf = np.zeros(nw, np.int32); e = np.zeros(nw)
    zeff = np.asarray([z - s for s in sigma], dtype=np.float64)
    for j, (nq, k) in enumerate(orbs):
        p, q, m, ee, _ = dcbsrw(nq, k, zeff[j], r[:n], n, c=c, h=h)
        pf[j, :n] = p; qf[j, :n] = q; mf[j] = m; e[j] = ee
    return Orbitals(np.array([o[0] for o in orbs], np.int32), np.array([o[1] for o in orbs], np.int32), mf, pf, qf,
                    e, zeff)


def screenpar(nak, ncore):
    nak = np.ascontiguousarray(nak, np.int32)
    s = np.zeros(len(nak))
    lib().gs_screenpar(len(nak), ptr(nak, _int), ncore, ptr(s, _d))
    return s


@dataclass
class CIBlock:
    """One J/parity block: mcp.30 structure, occupations and the T/V lists."""
    ncf: int
    nnz: int
    nconf: int
    kmaxf: int
    iendc: np.ndarray   # int64[ncf+1]
    irow: np.ndarray    # int32[nnz]
    iq: np.ndarray      # uint8[ncf, nw]
    tlist: dict
    vlists: list = field(default_factory=list)

    @property
    def density(self):
        return self.nnz / (self.ncf * (self.ncf + 1) / 2)

    @property
    def ncontr(self):
        return int(self.tlist["loc"].size + sum(v["loc"].size for v in self.vlists))


def ci_block(orbs, refs, frozen, two_j=0, parity=0, kmaxf=None, max_rank=2, max_ncf=0, density=0.0,
             coeff_scale=1.0, seed=1):
    """Generate a synthetic CI block (see inputs/grasp_synth.h)."""
    nw = len(orbs)
    npq = np.array([o[0] for o in orbs], np.int32)
    nak = np.array([o[1] for o in orbs], np.int32)
    if kmaxf is None:
        kmaxf = max(nkj(k) for k in nak)
    refs = np.ascontiguousarray(np.asarray(refs, np.uint8).reshape(-1, nw))
    frozen = np.ascontiguousarray(np.asarray(frozen, np.uint8))
    spec = GSBlockSpec(nw, ptr(npq, _int), ptr(nak, _int), ptr(frozen, _u8), refs.shape[0], ptr(refs, _u8),
                            max_rank, two_j, parity, kmaxf, max_ncf, density, coeff_scale, seed)
    h = C.c_void_p()
    L = lib()
    rc = L.gs_block_generate(C.byref(spec), C.byref(h))
    if rc != 0:
        raise ValueError(f"gs_block_generate failed ({rc})")
    try:
        ncf = C.c_int(); nnz = C.c_int64(); nconf = C.c_int(); km = C.c_int()
        nlab = np.zeros(kmaxf + 2, np.int64); ncon = np.zeros(kmaxf + 2, np.int64)
        L.gs_block_sizes(h, C.byref(ncf), C.byref(nnz), C.byref(nconf), C.byref(km), ptr(nlab, _i64), ptr(ncon, _i64))
        iendc = np.zeros(ncf.value + 1, np.int64); irow = np.zeros(nnz.value, np.int32)
        iq = np.zeros((ncf.value, nw), np.uint8)
        L.gs_block_structure(h, ptr(iendc, _i64), ptr(irow, _i32), ptr(iq, _u8))
        lists = []
        for li in range(kmaxf + 2):
            d = dict(lab=np.zeros(nlab[li], np.int32), start=np.zeros(nlab[li] + 1, np.int64),
                     iclmn=np.zeros(ncon[li], np.int32), loc=np.zeros(ncon[li], np.int32),
                     coeff=np.zeros(ncon[li], np.float64))
            L.gs_block_list(h, li, ptr(d["lab"], _i32), ptr(d["start"], _i64), ptr(d["iclmn"], _i32),
                            ptr(d["loc"], _i32), ptr(d["coeff"], _d))
            lists.append(d)
    finally:
        L.gs_block_free(h)
    return CIBlock(ncf.value, nnz.value, nconf.value, km.value, iendc, irow, iq, lists[0], lists[1:])


def occupation(orbs, spec):
    """Occupation vector from {(n, kappa): q}."""
    q = np.zeros(len(orbs), np.uint8)
    for j, o in enumerate(orbs):
        q[j] = spec.get(o, 0)
    return q
