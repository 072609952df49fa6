"""Small, fixed command lines for the profiler (ncu) runs whose summaries sit
in profiles/. Each target builds the Fe XV workload once and runs only the
kernel family it is named for, a few times:

  python -m inputs.profile_targets spmv     # 3 full-size y = H x launches per precision
  python -m inputs.profile_targets spmm     # split Y = H X launches for 1 to 16 vectors
  python -m inputs.profile_targets solve    # one full MANEIG (split, MBLOCK = NVEC) (launch list)
  python -m inputs.profile_targets solve2   # a warm-up MANEIG, then the measured one; prints the launch
                                            # counts that separate them in a launch list
  python -m inputs.profile_targets rk       # the R^k table of the 40-orbital k <= 8 workload
  python -m inputs.profile_targets rk_split # the same on the tensor cores (fp16 Ozaki digits, tcgen05)
  python -m inputs.profile_targets batch    # two batched solves of the 310-block workload (split)
  python -m inputs.profile_targets batch8   # the same for 8 ions (80 blocks), for detailed captures
  python -m inputs.profile_targets breit    # the type-1 Breit table of the Ne VII orbital set (16 subshells)
  python -m inputs.profile_targets setcof   # SETCOF's device pass over the Fe XV block's lists
  python -m inputs.profile_targets potentials  # from those lists: COFPOT of orbital 5, SETLAG over the
                                            # 55 same-kappa pairs (twice each)
"""
from __future__ import annotations

import sys


def _fe15_context():
    from grasp_gb300 import Context, HMatrix
    from . import workloads
    w = workloads.fe15()
    b = w.block
    ctx = Context(0)
    ctx.set_grid(w.n, w.rnt, w.h, w.c, w.zz)
    ctx.set_orbitals(w.orb.nak, w.orb.mf, w.orb.pf, w.orb.qf)
    ctx.genintrk()
    ctx.iabint_table()
    H = HMatrix(ctx, b.ncf, b.iendc, b.irow)
    H.setham(b.iq, b.tlist, b.vlists)
    return w, ctx, H


def spmv():
    from grasp_gb300 import FP64, SPLIT
    w, ctx, H = _fe15_context()
    for prec in (FP64, SPLIT):
        ms, by = H.matvec_timing(prec, 3)
        print(f"precision {prec}: {ms * 1e3:.1f} us per launch, {by / 1e6:.1f} MB algorithmic")


def spmm():
    w, ctx, H = _fe15_context()
    for m in (1, 2, 5, 10, 16):
        ms, by = H.spmm_timing(m, 5)
        print(f"split Y = H X, {m} vectors: {ms * 1e3:.1f} us per launch, {by / 1e6:.1f} MB algorithmic, "
              f"{by / (ms * 1e-3) / 1e9:.0f} GB/s")


def solve():
    from grasp_gb300 import SPLIT
    w, ctx, H = _fe15_context()
    ev, vec, info = H.maneig(w.nroots, flavour=0, precision=SPLIT, mblock=w.nroots)
    print("loops", info["nloops"], "E0", ev[0])


def solve2():
    from grasp_gb300 import SPLIT
    from grasp_gb300.core import launch_count
    w, ctx, H = _fe15_context()
    H.maneig(w.nroots, flavour=0, precision=SPLIT, mblock=w.nroots)  # tunes, builds workspaces and graphs
    ctx.synchronize()
    l0 = launch_count()
    ev, vec, info = H.maneig(w.nroots, flavour=0, precision=SPLIT, mblock=w.nroots)
    ctx.synchronize()
    print("launches before the measured solve", l0, "in it", launch_count() - l0, "loops", info["nloops"])


def rk(precision=0):
    from grasp_gb300 import Context
    from . import workloads
    w = workloads.rk40()
    ctx = Context(0)
    ctx.set_grid(w.n, w.rnt, w.h, w.c, w.zz)
    ctx.set_orbitals(w.orb.nak, w.orb.mf, w.orb.pf, w.orb.qf)
    for _ in range(3):
        n, _ = ctx.genintrk(kmax=8, precision=precision)
    print("R^k integrals", n, "ms", ctx.stage_stat(0))


def rk_split():
    rk(precision=1)


def batch(zs=None):
    from grasp_gb300 import SPLIT, Context, maneig_batched
    from . import workloads
    w = workloads.batch() if zs is None else workloads.batch(zs=zs)
    ctx = Context(0)
    hs = workloads.assemble_batch(w, ctx)
    for _ in range(2):
        res, info = maneig_batched(ctx, hs, w.nroots, precision=SPLIT)
    print("blocks", len(hs), "iterations", ctx.stage_stat(21), "ms", ctx.stage_stat(3))


def breit():
    """The type-1 Breit table of the Ne VII orbital set (n <= 4, l <= 3:
    16 subshells), WFACT 1 with the orbitals' Dirac energies, twice."""
    from grasp_gb300 import Context
    from . import workloads
    w = workloads.ne7()
    ctx = Context(0)
    ctx.set_grid(w.n, w.rnt, w.h, w.c, w.zz)
    ctx.set_orbitals(w.orb.nak, w.orb.mf, w.orb.pf, w.orb.qf)
    for _ in range(2):
        ind, val, kst, j2 = ctx.genintbreit(1, 1.0, w.orb.e)
    print("integrals", ind.size, "ms", ctx.stage_stat(31), "kernels ms", ctx.stage_stat(33))


def setcof():
    """SETCOF's device pass over the Fe XV block's lists with its 10
    eigenvectors (EOL, equal weights), twice."""
    import numpy as np

    from grasp_gb300 import SPLIT
    w, ctx, H = _fe15_context()
    ev, vec, info = H.maneig(w.nroots, flavour=0, precision=SPLIT, mblock=w.nroots)
    wt = np.full(w.nroots, 1.0 / w.nroots)
    for _ in range(2):
        ctx.setcof_prepare([H], [wt], [vec], eol=True)
    print("lists of orbital 5:", {k: len(v) for k, v in ctx.setcof(5, 2.0).items()})


def potentials():
    """COFPOT of orbital 5 (136 / 6,587 / 4 YPOT / XPOT / DACON terms) and
    SETLAG over the Fe XV orbitals' 55 same-kappa pairs, from the device
    SETCOF lists of the block's 10 eigenvectors; twice each."""
    import numpy as np

    from grasp_gb300 import SPLIT
    w, ctx, H = _fe15_context()
    ev, vec, info = H.maneig(w.nroots, flavour=0, precision=SPLIT, mblock=w.nroots)
    nw = len(w.orb.nak)
    ctx.setcof_prepare([H], [np.full(w.nroots, 1.0 / w.nroots)], [vec], eol=True)
    lists = [ctx.setcof(j, 2.0) for j in range(1, nw + 1)]
    nak = np.asarray(w.orb.nak)
    pairs = np.array([i + 215 * j for j in range(2, nw + 1) for i in range(1, j) if nak[i - 1] == nak[j - 1]],
                     np.int32)
    ucf = 1.0 + 0.05 * np.arange(nw)
    for _ in range(2):
        ctx.cofpot(5, ucf[4], lists[4])
        ctx.setlag(pairs, ucf, np.zeros(nw, np.int32), lists)
    print("XPOT terms of orbital 5:", len(lists[4]["nxa"]), "pairs:", pairs.size)


if __name__ == "__main__":
    {"spmv": spmv, "spmm": spmm, "solve": solve, "solve2": solve2, "rk": rk, "rk_split": rk_split, "batch": batch,
     "batch8": lambda: batch(zs=tuple(range(10, 18))), "breit": breit, "setcof": setcof,
     "potentials": potentials}[sys.argv[1]]()
