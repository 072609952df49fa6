"""Python mirror of the reference's interface for the CI hot path, over the
C ABI of libgraspgpu (include/grasp_gpu.h).

Names follow the reference: :meth:`Context.genintrk` (rci90/genintrk.f90),
:meth:`Context.slater` (lib9290/slater.f90), :meth:`Context.rinti`
(lib9290/rinti.f90), :meth:`Context.rkintc` (rci90/rkintc.f90),
:meth:`HMatrix.setham` (rmcdhf90/setham.f90), :meth:`HMatrix.spicmv2`
(lib9290/spicmv2.f90), :meth:`HMatrix.maneig` (rci90/maneig.f90 /
rmcdhf90/maneig.f90). Errors the reference turns into STOP raise GGError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import GGCof, GGDvdParams, GGList, _d, _i32, _i64, _int, _u8, check, ptr

FP64 = 0
SPLIT = 1


class Context:
    """One GPU context: grid (grid_C), orbitals (wave_C), R^k and I(ab) tables."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(_lib.gpu().gg_ctx_create(device, C.byref(self._h)))
        self.nw = 0
        self.n = 0
        # handle boxes of the matrices made on this context: closing the
        # context destroys them first (finalisers of objects collected
        # together run in no particular order)
        self._children = []

    def close(self):
        if self._h:
            for box in self._children:
                if box[0]:
                    _lib.gpu().gg_hmat_destroy(box[0])
                    box[0] = C.c_void_p()
            self._children = []
            _lib.gpu().gg_ctx_destroy(self._h)
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

    # grid_C / npot_C
    def set_grid(self, n, rnt, h, c, zz, r=None, rp=None, rpor=None):
        zz = np.ascontiguousarray(zz, np.float64)
        args = [None, None, None]
        if r is not None:
            self._r = [np.ascontiguousarray(x, np.float64) for x in (r, rp, rpor)]
            args = [ptr(x, _d) for x in self._r]
        check(_lib.gpu().gg_set_grid(self._h, n, rnt, h, c, *args, ptr(zz, _d)))
        self.n = n

    def grid(self):
        r = np.zeros(self.n + 10); rp = np.zeros(self.n + 10); rpor = np.zeros(self.n + 10)
        check(_lib.gpu().gg_get_grid(self._h, ptr(r, _d), ptr(rp, _d), ptr(rpor, _d)))
        return r, rp, rpor

    # wave_C
    def set_orbitals(self, nak, mf, pf, qf):
        nak = np.ascontiguousarray(nak, np.int32); mf = np.ascontiguousarray(mf, np.int32)
        pf = np.ascontiguousarray(pf, np.float64); qf = np.ascontiguousarray(qf, np.float64)
        nw, ld = pf.shape
        check(_lib.gpu().gg_set_orbitals(self._h, nw, ld, ptr(nak, _int), ptr(mf, _int), ptr(pf, _d), ptr(qf, _d)))
        self.nw = nw

    def genintrk(self, kmax=-1, precision=FP64):
        n = C.c_int64(); j2 = C.c_int()
        check(_lib.gpu().gg_genintrk(self._h, kmax, precision, C.byref(n), C.byref(j2)))
        self.n_rk = n.value
        self.kloop = j2.value if kmax < 0 else kmax
        return n.value, j2.value

    def rk_table(self):
        ind = np.zeros(self.n_rk, np.int32); val = np.zeros(self.n_rk); ks = np.zeros(self.kloop + 2, np.int32)
        check(_lib.gpu().gg_get_rk_table(self._h, ptr(ind, _i32), ptr(val, _d), ptr(ks, _i32)))
        return ind, val, ks

    def rkintc(self, a, b, c, d, k):
        out = C.c_double()
        check(_lib.gpu().gg_rkintc(self._h, a, b, c, d, k, C.byref(out)))
        return out.value

    def slater(self, a, b, c, d, k):
        out = C.c_double()
        check(_lib.gpu().gg_slater(self._h, a, b, c, d, k, C.byref(out)))
        return out.value

    def ypot(self, nya, ya):
        """YPOT (rmcdhf90/ypot.f90): the direct potential YP(1:N) of a SETCOF
        list (NYA labels (IOY2*215 + IOY1)*215 + K, YA coefficients)."""
        nya = np.ascontiguousarray(nya, np.int32); ya = np.ascontiguousarray(ya, np.float64)
        yp = np.zeros(self.n)
        check(_lib.gpu().gg_ypot(self._h, nya.size, ptr(nya, _i32), ptr(ya, _d), ptr(yp, _d)))
        return yp

    def xpot(self, nxa, xa):
        """XPOT (rmcdhf90/xpot.f90): the exchange potential XP(1:N), XQ(1:N) of
        a SETCOF list (NXA labels ((IORB*215 + IOY2)*215 + IOY1)*215 + K)."""
        nxa = np.ascontiguousarray(nxa, np.int32); xa = np.ascontiguousarray(xa, np.float64)
        xp = np.zeros(self.n); xq = np.zeros(self.n)
        check(_lib.gpu().gg_xpot(self._h, nxa.size, ptr(nxa, _i32), ptr(xa, _d), ptr(xp, _d), ptr(xq, _d)))
        return xp, xq

    def cofpot(self, j, ucfj, cof, iecc=(), ecv=(), accy=0.0):
        """COFPOT after SETCOF (gg_cofpot): YPOT, XPOT, LAGCON, DACON of
        orbital j from its lists (dict nya/ya/nxa/xa/nda/da); (YP, XP, XQ)."""
        keep = []
        c = _mkcof(cof, keep)
        iecc = np.ascontiguousarray(iecc, np.int32); ecv = np.ascontiguousarray(ecv, np.float64)
        n = self.n
        yp, xp, xq = np.zeros(n), np.zeros(n), np.zeros(n)
        check(_lib.gpu().gg_cofpot(self._h, int(j), float(ucfj), C.byref(c), iecc.size, ptr(iecc, _i32),
                                   ptr(ecv, _d), float(accy), ptr(yp, _d), ptr(xp, _d), ptr(xq, _d)))
        return yp, xp, xq

    def setlag(self, iecc, ucf, lfix, cofs):
        """SETLAG's multipliers (gg_setlag) for the pairs iecc[k] = LI + 215 LJ;
        cofs[orbital - 1] = that orbital's lists (None for orbitals in no pair)."""
        keep = []
        empty = {}
        arr = (GGCof * len(cofs))(*[_mkcof(c if c is not None else empty, keep) for c in cofs])
        iecc = np.ascontiguousarray(iecc, np.int32); ucf = np.ascontiguousarray(ucf, np.float64)
        lfix = np.ascontiguousarray(lfix, np.int32)
        ecv = np.zeros(iecc.size)
        check(_lib.gpu().gg_setlag(self._h, iecc.size, ptr(iecc, _i32), ptr(ucf, _d), ptr(lfix, _int), arr,
                                   ptr(ecv, _d)))
        return ecv

    def setcof_prepare(self, hmats, wt, evec=None, eol=True):
        """SETCOF's sums for every orbital (gg_setcof_prepare): hmats in
        rmcdhf's block order (lists uploaded); eol: evec[b] (NCF_b x nev_b) and
        wt[b] (nev_b level weights); else wt[b] = the NCF_b CSF weights."""
        nb = len(hmats)
        keep = []
        hs = (C.c_void_p * nb)(*[h._h for h in hmats])
        wts = [np.ascontiguousarray(w, np.float64) for w in wt]
        keep += wts
        wp = (_d * nb)(*[ptr(w, _d) for w in wts])
        if eol:
            evs = [np.asfortranarray(np.asarray(v, np.float64).reshape(h.ncf, -1)) for v, h in zip(evec, hmats)]
            keep += evs
            ep = (_d * nb)(*[ptr(v, _d) for v in evs])
            nev = np.array([v.shape[1] for v in evs], np.int32)
        else:
            ep = (_d * nb)()
            nev = np.zeros(nb, np.int32)
        check(_lib.gpu().gg_setcof_prepare(self._h, nb, hs, ptr(nev, _int), ep, wp, int(bool(eol))))

    def setcof(self, j, ucfj):
        """SETCOF(EOL, J)'s lists (gg_setcof) from the prepared sums: a dict
        nya/ya, nxa/xa, nda/da (gg_cofpot's and cofpot's input)."""
        cap = 1024
        while True:
            ny, nx, nd = C.c_int(), C.c_int(), C.c_int()
            nya = np.zeros(cap, np.int32); ya = np.zeros(cap); nxa = np.zeros(cap, np.int32); xa = np.zeros(cap)
            nda = np.zeros(cap, np.int32); da = np.zeros(cap)
            st = _lib.gpu().gg_setcof(self._h, int(j), float(ucfj), cap, C.byref(ny), ptr(nya, _i32), ptr(ya, _d),
                                      C.byref(nx), ptr(nxa, _i32), ptr(xa, _d), C.byref(nd), ptr(nda, _i32),
                                      ptr(da, _d))
            if st == _lib_status("GG_ERR_RANGE"):
                cap = max(ny.value, nx.value, nd.value)
                continue
            check(st)
            return dict(nya=nya[:ny.value].copy(), ya=ya[:ny.value].copy(), nxa=nxa[:nx.value].copy(),
                        xa=xa[:nx.value].copy(), nda=nda[:nd.value].copy(), da=da[:nd.value].copy())

    def genintbreit(self, itype, wfact, e, accy=0.0):
        """GENINTBREIT1/2 on the device (gg_genintbreit): (INDTP, VALTP,
        KSTARTBREIT, J2MAX) of the type-1 or type-2 table."""
        e = np.ascontiguousarray(e, np.float64)
        nb = C.c_int64(); j2 = C.c_int()
        check(_lib.gpu().gg_genintbreit(self._h, int(itype), float(wfact), ptr(e, _d), float(accy), C.byref(nb),
                                        C.byref(j2)))
        ind = np.zeros(nb.value, np.int32); val = np.zeros(nb.value); kst = np.zeros(j2.value + 2, np.int32)
        check(_lib.gpu().gg_get_breit_table(self._h, int(itype), ptr(ind, _i32), ptr(val, _d), ptr(kst, _i32)))
        return ind, val, kst, j2.value

    def brint(self, itype, a, b, c, d, k):
        """BRINT1/BRINT2: a value of the context's table (gg_brint)."""
        v = C.c_double()
        check(_lib.gpu().gg_brint(self._h, int(itype), a, b, c, d, k, C.byref(v)))
        return v.value

    def brintf(self, items, wfact, e, accy=0.0):
        """BRINTF for rows (type, ia, ib, ic, id, k) of items (gg_brintf)."""
        it = np.ascontiguousarray(np.asarray(items, np.int32).reshape(-1, 6))
        e = np.ascontiguousarray(e, np.float64)
        out = np.zeros(it.shape[0])
        check(_lib.gpu().gg_brintf(self._h, it.shape[0], ptr(it, _i32), float(wfact), ptr(e, _d), float(accy),
                                   ptr(out, _d)))
        return out

    def rinti(self, j, k, mode=0):
        out = C.c_double()
        check(_lib.gpu().gg_rinti(self._h, j, k, mode, C.byref(out)))
        return out.value

    def iabint_table(self):
        t = np.zeros(self.nw * self.nw)
        check(_lib.gpu().gg_iabint_table(self._h, ptr(t, _d)))
        return t.reshape(self.nw, self.nw)

    def batched_tune(self):
        """The batched matvec variant of the last gg_maneig_batched on this
        context and the tuner's times: dict(chosen=name, ms={name: ms})."""
        ch = C.c_int(); nv = C.c_int()
        ms = np.zeros(6)
        check(_lib.gpu().gg_batched_tune_info(self._h, C.byref(ch), C.byref(nv), ptr(ms, _d)))
        name = lambda v: _lib.gpu().gg_tune_variant_name(2, v).decode()  # noqa: E731
        return dict(chosen=name(ch.value), ms={name(v): float(ms[v]) for v in range(nv.value)})

    def host_read_timing(self, nbytes, mode=0, iters=10):
        """ms per pass over a pinned host buffer (gg_host_read_timing): mode 0
        read by a kernel over the host link, 1 copied by cudaMemcpyAsync."""
        ms = C.c_double()
        check(_lib.gpu().gg_host_read_timing(self._h, int(nbytes), int(mode), int(iters), C.byref(ms)))
        return ms.value

    def stage_stat(self, which):
        return _lib.gpu().gg_stage_stat(self._h, which)

    def mark(self, slot):
        """Record a CUDA event (slot 0..7) on the context stream."""
        check(_lib.gpu().gg_event_record(self._h, slot))

    def elapsed(self, a, b):
        """Milliseconds between two marks (synchronises on b)."""
        ms = C.c_double()
        check(_lib.gpu().gg_event_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def synchronize(self):
        check(_lib.gpu().gg_ctx_synchronize(self._h))


def _mkcof(d, keep):
    arrs = [np.ascontiguousarray(d.get(k, []), t) for k, t in
            (("nya", np.int32), ("ya", np.float64), ("nxa", np.int32), ("xa", np.float64),
             ("nda", np.int32), ("da", np.float64))]
    keep.extend(arrs)
    nya, ya, nxa, xa, nda, da = arrs
    return GGCof(nya.size, ptr(nya, _i32), ptr(ya, _d), nxa.size, ptr(nxa, _i32), ptr(xa, _d),
                 nda.size, ptr(nda, _i32), ptr(da, _d))


def _mklist(d, keep):
    lab = np.ascontiguousarray(d["lab"], np.int32); st = np.ascontiguousarray(d["start"], np.int64)
    loc = np.ascontiguousarray(d["loc"], np.int32); co = np.ascontiguousarray(d["coeff"], np.float64)
    keep.extend([lab, st, loc, co])
    return GGList(lab.size, ptr(lab, _i32), ptr(st, _i64), ptr(loc, _i32), ptr(co, _d))


class HMatrix:
    """One Hamiltonian block on the device (hmat_C: EMT, IROW, IENDC)."""

    def __init__(self, ctx: Context, ncf, iendc, irow):
        self.ctx = ctx
        self.ncf = int(ncf)
        self.iendc = np.ascontiguousarray(iendc, np.int64)
        self.irow = np.ascontiguousarray(irow, np.int32)
        self.nnz = int(self.iendc[-1])
        self._box = [C.c_void_p()]
        check(_lib.gpu().gg_hmat_create(ctx._h, self.ncf, self.nnz, ptr(self.iendc, _i64), ptr(self.irow, _i32),
                                        C.byref(self._box[0])))
        ctx._children.append(self._box)
        self.eav = None

    @classmethod
    def host(cls, ctx: Context, ncf, iendc, irow, emt, eav=0.0, precision=FP64):
        """A block kept in pinned host memory and read over the host link by
        every product (gg_hmat_create_host, SPODMV's role): emt as rci writes
        it to rci.res, the diagonal shifted by eav. Products and solves use
        the given precision only."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.ncf = int(ncf)
        self.iendc = np.ascontiguousarray(iendc, np.int64)
        self.irow = np.ascontiguousarray(irow, np.int32)
        self.nnz = int(self.iendc[-1])
        emt = np.ascontiguousarray(emt, np.float64)
        if emt.size != self.nnz:
            raise ValueError("emt must hold IENDC(NCF) values")
        self._box = [C.c_void_p()]
        check(_lib.gpu().gg_hmat_create_host(ctx._h, self.ncf, self.nnz, ptr(self.iendc, _i64), ptr(self.irow, _i32),
                                             ptr(emt, _d), float(eav), int(precision), C.byref(self._box[0])))
        ctx._children.append(self._box)
        self.eav = float(eav)
        return self

    @classmethod
    def packed(cls, ctx: Context, ncf, ap):
        """A dense block from its lower triangle packed by rows (DNICMV's EMT,
        gg_hmat_create_packed)."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.ncf = int(ncf)
        ap = np.ascontiguousarray(ap, np.float64)
        if ap.size != self.ncf * (self.ncf + 1) // 2:
            raise ValueError("ap must hold NCF (NCF + 1) / 2 values")
        r = np.arange(self.ncf, dtype=np.int64)
        self.iendc = np.concatenate([[0], np.cumsum(r + 1)]).astype(np.int64)
        self.irow = np.concatenate([np.arange(1, i + 2, dtype=np.int32) for i in range(self.ncf)])
        self.nnz = int(self.iendc[-1])
        self._box = [C.c_void_p()]
        check(_lib.gpu().gg_hmat_create_packed(ctx._h, self.ncf, ptr(ap, _d), C.byref(self._box[0])))
        ctx._children.append(self._box)
        self.eav = None
        return self

    @property
    def host_precision(self):
        """The precision a host-resident matrix was built for; None on the device."""
        p = _lib.gpu().gg_hmat_host_precision(self._h)
        return None if p < 0 else p

    def spodmv(self, b):
        """SPODMV: C = (H - EAV) B for a host-resident matrix, in its precision."""
        b = np.asfortranarray(np.asarray(b, np.float64).reshape(self.ncf, -1))
        c = np.zeros_like(b, order="F")
        check(_lib.gpu().gg_spodmv(self.ctx._h, self._h, b.shape[1], ptr(b, _d), ptr(c, _d)))
        return c

    @classmethod
    def view(cls, src, ctx=None):
        """A matrix sharing src's structure, lists and assembly plan, with its
        own EMT (gg_hmat_create_view): the same block for another ion."""
        ctx = src.ctx if ctx is None else ctx
        self = cls.__new__(cls)
        self.ctx = ctx
        self.ncf, self.nnz, self.iendc, self.irow = src.ncf, src.nnz, src.iendc, src.irow
        self._box = [C.c_void_p()]
        check(_lib.gpu().gg_hmat_create_view(ctx._h, src._h, C.byref(self._box[0])))
        ctx._children.append(self._box)
        self._source = src
        self.eav = None
        return self

    @property
    def _h(self):
        return self._box[0]

    def close(self):
        if self._box[0] and self.ctx._h:
            _lib.gpu().gg_hmat_destroy(self._box[0])
            self._box[0] = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setham_upload(self, iq, tlist, vlists):
        keep = []
        iq = np.ascontiguousarray(iq, np.uint8)
        tl = _mklist(tlist, keep)
        vl = (GGList * max(1, len(vlists)))(*[_mklist(v, keep) for v in vlists])
        check(_lib.gpu().gg_setham_upload(self.ctx._h, self._h, ptr(iq, _u8), C.byref(tl), len(vlists) - 1, vl))

    def setham_assemble(self):
        eav = C.c_double()
        check(_lib.gpu().gg_setham_assemble(self.ctx._h, self._h, C.byref(eav)))
        self.eav = eav.value
        return self.eav

    def setham(self, iq, tlist, vlists):
        """SETHAM + the EAV shift of MATRIX; returns EAV. EMT stays on the device."""
        self.setham_upload(iq, tlist, vlists)
        return self.setham_assemble()

    def emt(self):
        out = np.zeros(self.nnz)
        check(_lib.gpu().gg_hmat_get_emt(self._h, ptr(out, _d)))
        return out

    def set_emt(self, emt):
        emt = np.ascontiguousarray(emt, np.float64)
        check(_lib.gpu().gg_hmat_set_emt(self._h, ptr(emt, _d)))

    def spicmv2(self, b, precision=FP64):
        b = np.asfortranarray(np.asarray(b, np.float64).reshape(self.ncf, -1))
        c = np.zeros_like(b, order="F")
        check(_lib.gpu().gg_spicmv2(self.ctx._h, self._h, b.shape[1], ptr(b, _d), ptr(c, _d), precision))
        return c

    def maneig(self, nvec, flavour=0, precision=FP64, lim=0, maxiter=0, critr=0.0, critc=0.0, crite=0.0,
               robust=False, raise_on_maxiter=True, mblock=0, start=None):
        """MANEIG; start: [ncf x k] orthonormal start vectors (rmcdhf's warm
        start from the previous eigenvectors) instead of INIEST2."""
        st0 = None
        if start is not None:
            st0 = np.asfortranarray(np.asarray(start, np.float64).reshape(self.ncf, -1))
        p = GGDvdParams(flavour, precision, lim, maxiter, critr, critc, crite, int(robust), int(mblock),
                        0 if st0 is None else st0.shape[1], None if st0 is None else ptr(st0, _d))
        ev = np.zeros(nvec); vec = np.zeros((nvec, self.ncf))
        nl, nm, ie = C.c_int(), C.c_int(), C.c_int()
        st = _lib.gpu().gg_maneig(self.ctx._h, self._h, nvec, C.byref(p), ptr(ev, _d), ptr(vec, _d), C.byref(nl),
                                  C.byref(nm), C.byref(ie))
        info = dict(nloops=nl.value, nmv=nm.value, ierr=ie.value, status=st)
        if st != 0 and (raise_on_maxiter or st != _lib_status("GG_ERR_CONVERGE")):
            check(st)
        return ev, vec.T.copy(), info


    def tune(self, kernel, m=1):
        """The SpMV autotuner's result for this matrix (include/grasp_gpu.h,
        gg_hmat_tune): dict(chosen=name, ms={name: ms per launch})."""
        ch = C.c_int(); nv = C.c_int()
        ms = np.zeros(16)
        check(_lib.gpu().gg_hmat_tune(self._h, kernel, m, C.byref(ch), C.byref(nv), ptr(ms, _d)))
        name = lambda v: _lib.gpu().gg_tune_variant_name(kernel, v).decode()  # noqa: E731
        return dict(chosen=name(ch.value), ms={name(v): float(ms[v]) for v in range(nv.value)})

    def tune_force(self, kernel, m, variant):
        check(_lib.gpu().gg_hmat_tune_force(self._h, kernel, m, variant))

    def matvec_timing(self, precision=FP64, iters=20):
        """(ms per y = H x launch, algorithmic bytes per launch)."""
        ms = C.c_double(); by = C.c_double()
        check(_lib.gpu().gg_matvec_timing(self.ctx._h, self._h, precision, iters, C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def spmm_timing(self, m, iters=20):
        """(ms per split Y = H X launch over m vectors, algorithmic bytes per launch)."""
        ms = C.c_double(); by = C.c_double()
        check(_lib.gpu().gg_spmm_timing(self.ctx._h, self._h, m, iters, C.byref(ms), C.byref(by)))
        return ms.value, by.value


def maneig_batched(ctx, hmats, nvec, precision=FP64, lim=0, maxiter=0, critr=0.0, raise_on_maxiter=True):
    """MANEIG for many blocks in one batched GPU Davidson (gg_maneig_batched).

    The reference calls MANEIG once per J/parity block from its block loop
    (rci90/matrix.f90:177-187). ``hmats`` are assembled HMatrix objects (any
    contexts of one device), ``nvec`` the roots per block (an int or one per
    block). Returns ``[(eval, evec), ...]`` per block (evec columns are the
    eigenvectors, dominant component positive) and the per-block
    ``nloops``, ``nmv`` and ``ierr`` arrays."""
    nb = len(hmats)
    nv = np.full(nb, nvec, np.int32) if np.isscalar(nvec) else np.ascontiguousarray(nvec, np.int32)
    ncf = np.array([h.ncf for h in hmats], np.int64)
    ev = np.zeros(int(nv.sum()))
    vec = np.zeros(int((ncf * nv).sum()))
    hs = (C.c_void_p * nb)(*[h._h.value for h in hmats])
    nl, nm, ie = (np.zeros(nb, np.int32) for _ in range(3))
    p = GGDvdParams(0, precision, lim, maxiter, critr, 0.0, 0.0, 0, 0)
    st = _lib.gpu().gg_maneig_batched(ctx._h, nb, hs, ptr(nv, _int), C.byref(p), ptr(ev, _d), ptr(vec, _d),
                                      ptr(nl, _int), ptr(nm, _int), ptr(ie, _int))
    if st != 0 and (raise_on_maxiter or st != _lib_status("GG_ERR_CONVERGE")):
        check(st)
    out, eo, vo = [], 0, 0
    for b in range(nb):
        r, n = int(nv[b]), int(ncf[b])
        out.append((ev[eo:eo + r].copy(), vec[vo:vo + n * r].reshape(r, n).T.copy()))
        eo += r
        vo += n * r
    return out, dict(nloops=nl, nmv=nm, ierr=ie, status=st)


def projected_eig(s, m, mvec=None):
    """DVDSON's projected eigenproblem (DSPEVX on S, libdvd90/dvdson.f90:724)
    on the host: the lowest ``m`` eigenvalues of the symmetric matrix ``s``
    (its upper triangle is read) and the eigenvectors of the lowest ``mvec``."""
    s = np.asarray(s, np.float64)
    n = s.shape[0]
    mvec = m if mvec is None else mvec
    ap = np.concatenate([s[: j + 1, j] for j in range(n)]).astype(np.float64)
    w = np.zeros(m)
    z = np.zeros((max(mvec, 1), n))
    check(_lib.gpu().gg_projected_eig(n, ptr(ap, _d), m, mvec, ptr(w, _d), ptr(z, _d)))
    return w, z[:mvec].T.copy()


def _lib_status(name):
    return {"GG_ERR_CONVERGE": -7, "GG_ERR_RANGE": -5}[name]


def launch_count():
    """Kernels libgraspgpu has launched in this process."""
    return int(_lib.gpu().gg_launch_count())


class pinned:
    """Context manager that page-locks numpy arrays for the duration."""

    def __init__(self, *arrays):
        self.arrays = [a for a in arrays if a is not None and a.nbytes > 0]

    def __enter__(self):
        for a in self.arrays:
            check(_lib.gpu().gg_host_register(C.c_void_p(a.ctypes.data), a.nbytes))
        return self

    def __exit__(self, *exc):
        for a in self.arrays:
            _lib.gpu().gg_host_unregister(C.c_void_p(a.ctypes.data))


def rci_select_ivec(eval_, evec, ivec):
    """rci's choice of states (rci90/maneig.f90:496-516): MANEIG solves for
    the lowest NVECMX = max(IVEC) eigenpairs, then brings eigenpair IVEC(i)
    to position i by the same sequence of swaps and keeps the first NVEC.
    eval_[nvecmx], evec[ncf, nvecmx]; ivec 1-based. Returns (eval, evec)
    with NVEC = len(ivec) columns."""
    ev = np.array(eval_, dtype=np.float64, copy=True)
    vec = np.array(evec, dtype=np.float64, copy=True)
    nvecmx = ev.size
    iwork = list(range(1, nvecmx + 1))
    for i in range(1, len(ivec) + 1):
        iofset = int(ivec[i - 1])
        loc = iwork[i - 1]
        if iofset == loc:
            continue
        ev[[iofset - 1, i - 1]] = ev[[i - 1, iofset - 1]]
        iwork[i - 1] = iwork[iofset - 1]
        iwork[iofset - 1] = loc
        vec[:, [iofset - 1, i - 1]] = vec[:, [i - 1, iofset - 1]]
    return ev[:len(ivec)].copy(), vec[:, :len(ivec)].copy()
