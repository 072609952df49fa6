"""T/V angular-coefficient lists for a GRASP CSF list (libgraspangular,
include/grasp_angular.h): the input SETHAM takes, produced from the CSF
list's couplings by the determinant route described in that header.

    csl = formats.read_csl("rcsf.c")
    blk = angular.block_lists(csl, 0)      # first J/parity block
    H = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    H.setham(blk.iq, blk.tlist, blk.vlists)  # blk.iq is zero: the lists hold all of H

The lists hold the whole Dirac-Coulomb Hamiltonian, core included, so the
occupations handed to SETHAM are zero (no average-energy diagonal pieces).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)
_int = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)


class GABlockSpec(C.Structure):
    _fields_ = [("nw", C.c_int), ("nak", _int), ("ncsf", C.c_int), ("iq", _u8), ("jqs", _int), ("nu", _int),
                ("xj", _int), ("two_j", C.c_int), ("cutoff", C.c_double), ("nthreads", C.c_int),
                ("average_split", C.c_int)]


SYMBOLS = {
    "ga_block_generate": (C.c_int, [C.POINTER(GABlockSpec), C.POINTER(C.c_void_p)]),
    "ga_block_free": (None, [C.c_void_p]),
    "ga_block_sizes": (C.c_int, [C.c_void_p, _int, _i64, _int, _i64, _i64]),
    "ga_block_structure": (C.c_int, [C.c_void_p, _i64, _i32]),
    "ga_block_list": (C.c_int, [C.c_void_p, C.c_int, _i32, _i64, _i32, _i32, _d]),
    "ga_last_error": (C.c_char_p, []),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_ANGULAR):
            _build.build()
        L = C.CDLL(_build.LIB_ANGULAR)
        for name, (res, args) in SYMBOLS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


@dataclass
class AngularBlock:
    """One J/parity block: mcp.30 structure and the T/V lists (SETHAM's input)."""
    ncf: int
    nnz: int
    kmaxf: int
    two_j: int
    parity: int
    iendc: np.ndarray
    irow: np.ndarray
    iq: np.ndarray          # occupations for SETHAM: the CSFs' (average_split) or zeros (whole H in the lists)
    occupations: np.ndarray  # the CSFs' subshell occupations [ncf, nw]
    tlist: dict
    vlists: list = field(default_factory=list)

    @property
    def ncontr(self):
        return int(self.tlist["loc"].size + sum(v["loc"].size for v in self.vlists))


def block_lists(csl, block, cutoff=-1.0, nthreads=0, average_split=False) -> AngularBlock:
    """Structure and T/V lists of block `block` (0-based) of a CslFile.
    average_split: rangular's convention for rmcdhf (the occupation-driven
    diagonal pieces left to SETHAM; .iq then holds the occupations), else
    the whole H in the lists and .iq zero."""
    b = csl.blocks[block]
    nw = len(csl.subshells)
    nak = np.ascontiguousarray([k for _, k in csl.subshells], np.int32)
    iq = np.ascontiguousarray(b.iq, np.uint8)
    jqs = np.ascontiguousarray(b.jqs, np.int32)
    nu = np.ascontiguousarray(b.nu, np.int32)
    xj = np.ascontiguousarray(b.xj, np.int32)
    spec = GABlockSpec(nw, _p(nak, _int), b.ncsf, _p(iq, _u8), _p(jqs, _int), _p(nu, _int), _p(xj, _int), b.two_j,
                       cutoff, nthreads, int(bool(average_split)))
    h = C.c_void_p()
    L = lib()
    if L.ga_block_generate(C.byref(spec), C.byref(h)) != 0:
        raise ValueError("angular lists: " + L.ga_last_error().decode())
    try:
        ncf = C.c_int(); nnz = C.c_int64(); km = C.c_int()
        L.ga_block_sizes(h, C.byref(ncf), C.byref(nnz), C.byref(km), None, None)
        nlab = np.zeros(km.value + 2, np.int64); ncon = np.zeros(km.value + 2, np.int64)
        L.ga_block_sizes(h, None, None, None, _p(nlab, _i64), _p(ncon, _i64))
        iendc = np.zeros(ncf.value + 1, np.int64); irow = np.zeros(nnz.value, np.int32)
        L.ga_block_structure(h, _p(iendc, _i64), _p(irow, _i32))
        lists = []
        for li in range(km.value + 2):
            d = dict(lab=np.zeros(nlab[li], np.int32), start=np.zeros(nlab[li] + 1, np.int64),
                     iclmn=np.zeros(ncon[li], np.int32), loc=np.zeros(ncon[li], np.int32),
                     coeff=np.zeros(ncon[li], np.float64))
            L.ga_block_list(h, li, _p(d["lab"], _i32), _p(d["start"], _i64), _p(d["iclmn"], _i32),
                            _p(d["loc"], _i32), _p(d["coeff"], _d))
            lists.append(d)
    finally:
        L.ga_block_free(h)
    iq_setham = iq.copy() if average_split else np.zeros((ncf.value, nw), np.uint8)
    return AngularBlock(ncf.value, nnz.value, km.value, b.two_j, b.parity, iendc, irow, iq_setham, iq.copy(),
                        lists[0], lists[1:])


def mcp_set(csl, nelec, average_split=True, **kw):
    """All blocks of a CSF list as an McpSet (grasp_gb300.formats): what
    rangular writes to mcp.30/31/32+k for rmcdhf, with write_mcp then giving
    the files. average_split=True keeps SETHAM's occupation-driven diagonal
    pieces out of the lists (rangular's convention for rmcdhf)."""
    from . import formats as F
    blocks, idblk, kmaxf = [], [], 0
    for bi, b in enumerate(csl.blocks):
        ab = block_lists(csl, bi, average_split=average_split, **kw)
        kmaxf = max(kmaxf, ab.kmaxf)
        blocks.append(F.McpBlock(ab.ncf, ab.iendc, ab.irow, ab.tlist, list(ab.vlists)))
        j = f"{b.two_j}/2" if b.two_j % 2 else f"{b.two_j // 2}"
        idblk.append(f"{j:>4}{'+' if b.parity > 0 else '-'}   "[:8])
    empty = dict(lab=np.zeros(0, np.int32), start=np.zeros(1, np.int64), loc=np.zeros(0, np.int32),
                 coeff=np.zeros(0), iclmn=np.zeros(0, np.int32))
    for blk in blocks:
        while len(blk.vlists) < kmaxf + 1:
            blk.vlists.append(dict(empty))
    return F.McpSet(ncore=csl.ncore, nelec=nelec, ncf=sum(b.ncf for b in blocks), nw=len(csl.subshells),
                    kmaxf=kmaxf, idblk=idblk, blocks=blocks)
