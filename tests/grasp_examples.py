"""The GRASP-written example runs in tests/golden/grasp_examples, set up as
the reference's programs set them up (test infrastructure):

- the grid of the run (RADGRD, HP = 0) from RNT, H and N in its summary;
- the nuclear potential ZZ = -r V(r): point nucleus (ZZ = Z) or the Fermi
  distribution of NUCPOT (lib9290/nucpot.f90:43-83, with the series ES of
  lib9290/es.f90:23-60), its c and a taken from isodata in fm and converted
  with FMTOAU = 1e-13 / AINFCM (lib9290/setcon.f90:105, lodiso.f90:43-44);
  these runs used the 1986 constants (c = 137.0359895, printed in their
  summaries; AINFCM = 0.529177249e-8 reproduces the c and a they print);
- the orbitals as LODRWF leaves them (lib9290/lodrwf.f90:100-134): the run
  wrote them on the same grid, so INTRPQ (intrpq.f90) takes the stored
  values at the grid points, sets MF to the last stored point and makes the
  norm RINT(J,J,0) one; then ORTHSC (orthsc.f90:36-85) Schmidt-orthogonalises
  each orbital against the earlier ones of the same kappa;
- the orbital order of the CSF list (core subshells, then peel subshells);
- the Dirac-Coulomb level energies the rmcdhf run printed (.sum).
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

from grasp_gb300 import formats as F

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grasp_examples")
RUNS = {"He": "data_He/3Pn6", "Ge": "data_Ge/2Fn5"}
AINFCM_1986 = 0.529177249e-8


def _num(s):
    return float(s.replace("D", "E"))


def subshell_kappa(label):
    """'4p-' -> (4, 1), '4p' -> (4, -2), '4s' -> (4, -1): GRASP's subshell
    notation, j = l - 1/2 for a trailing '-'."""
    m = re.fullmatch(r"(\d+)([spdfghiklmn])(-?)", label.strip())
    n, l = int(m.group(1)), "spdfghiklmn".index(m.group(2))
    return n, (l if m.group(3) else -(l + 1))


def read_summary(path):
    text = open(path).read()
    out = {
        "z": _num(re.search(r"atomic number is\s+(\S+);", text).group(1)),
        "c": _num(re.search(r"Speed of light =\s+(\S+)", text).group(1)),
        "rnt": _num(re.search(r"RNT\s+=\s+(\S+)", text).group(1)),
        "h": _num(re.search(r"\bH\s+=\s+(\S+)", text).group(1)),
        "n": int(re.search(r"\bN\s+=\s+(\d+);", text).group(1)),
        "fermi": "Fermi nucleus" in text,
    }
    levels = []
    part = text.split("Eigenenergies:")[1].split("Weights")[0]
    for m in re.finditer(r"^\s+(\d+)\s+(\d+(?:/2)?)\s+([+-])\s+(\S+)", part, re.M):
        j = m.group(2)
        two_j = int(j[:-2]) if j.endswith("/2") else 2 * int(j)
        levels.append((int(m.group(1)), two_j, m.group(3), _num(m.group(4))))
    out["levels"] = levels
    return out


def read_isodata(path):
    vals = []
    for line in open(path):
        try:
            vals.append(float(line))
        except ValueError:
            pass
    return {"z": vals[0], "a_mass": vals[1], "a_fm": vals[2], "c_fm": vals[3], "mass_amu": vals[4]}


def radgrd(n, rnt, h):
    """R, RP, RPOR on N + 10 points (lib9290/radgrd.f90:48-60, HP = 0)."""
    r = np.zeros(n + 10); rp = np.zeros(n + 10); rpor = np.zeros(n + 10)
    eph = math.exp(h)
    e = 1.0
    rp[0] = rnt
    for i in range(1, n + 10):
        e = eph * e
        r[i] = rnt * (e - 1.0)
        rp[i] = rnt * e
        rpor[i] = rp[i] / r[i]
    return r, rp, rpor


def _es(f):
    """ES (lib9290/es.f90): S2 = sum (-1)^n e^(nf)/n^2, S3 = sum (-1)^n e^(nf)/n^3,
    summed until S2 stops changing."""
    s2 = s3 = 0.0
    fase = 1.0
    n = 0
    while True:
        n += 1
        obn = 1.0 / n
        fase = -fase
        t2 = fase * math.exp(n * f) * obn * obn
        last = s2
        s2 += t2
        s3 += t2 * obn
        if abs(s2) == abs(last):
            return s2, s3


def nucpot_fermi(z, c, a, r, n):
    """ZZ(1:N) of a Fermi nucleus (lib9290/nucpot.f90:43-83)."""
    pi = 4.0 * math.atan(1.0)
    abc = a / c
    tabc = 2.0 * abc
    abc2 = abc * abc
    thabc2 = 3.0 * abc2
    abc3 = abc2 * abc
    cba = c / a
    h3php = 1.5 + 0.5 * pi * pi * abc2
    _, s3mcba = _es(-cba)
    sabc3 = 6.0 * abc3
    dmsas = -sabc3 * s3mcba
    en = 1.0 + abc2 * pi * pi + dmsas
    zbn = z / en
    zz = np.zeros(n)
    for i in range(n):
        ri = r[i]
        rmcba = (ri - c) / a
        rbc = ri / c
        if rbc <= 1.0:
            s2, s3 = _es(rmcba)
            zz[i] = zbn * (dmsas + sabc3 * s3 + rbc * (h3php - thabc2 * s2 - 0.5 * rbc * rbc))
        else:
            s2, s3 = _es(-rmcba)
            zz[i] = z * (1.0 + thabc2 * (rbc * s2 + tabc * s3) / en)
    return zz


def read_csf_subshells(path):
    """Core and peel subshell labels of a .c CSF list, in its order."""
    lines = open(path).read().splitlines()
    core = lines[lines.index("Core subshells:") + 1].split()
    peel = lines[lines.index("Peel subshells:") + 1].split()
    return core + peel, len(core)


def _rint(o, rp, pf, qf, mf, i, j):
    """RINT(I, J, 0) (lib9290/rint.f90): QUAD of RP (P_i P_j + Q_i Q_j) up to min(MF)."""
    mtp = int(min(mf[i], mf[j]))
    ta = np.zeros(mtp + 3)
    ta[1:mtp] = (pf[i, 1:mtp] * pf[j, 1:mtp] + qf[i, 1:mtp] * qf[j, 1:mtp]) * rp[1:mtp]
    return o.quad(ta, mtp)


def load(run, oracle_mod):
    """dict(n, rnt, h, c, z, zz, nak, np, mf, pf [nw, n], qf, labels, ncore,
    levels, summary) of the named example run ('He' or 'Ge')."""
    base = os.path.join(ROOT, RUNS[run])
    sm = read_summary(base + ".sum")
    n, rnt, h, c, z = sm["n"], sm["rnt"], sm["h"], sm["c"], sm["z"]
    r, rp, _ = radgrd(n, rnt, h)
    if sm["fermi"]:
        iso = read_isodata(os.path.join(os.path.dirname(base), "isodata"))
        fmtoau = 1.0e-13 / AINFCM_1986
        zz = nucpot_fermi(z, iso["c_fm"] * fmtoau, iso["a_fm"] * fmtoau, r, n)
    else:
        zz = np.full(n, z)
    labels, ncore = read_csf_subshells(base + ".c")
    wanted = [subshell_kappa(s) for s in labels]
    stored = {(o.np, o.nak): o for o in F.read_rwfn(base + ".w")}
    nw = len(wanted)
    pf = np.zeros((nw, n)); qf = np.zeros((nw, n)); mf = np.zeros(nw, np.int32)
    o = oracle_mod.Oracle(n=n, rnt=rnt, h=h, c=c, zz=zz)
    # LODRWF + INTRPQ on the run's own grid
    for j, key in enumerate(wanted):
        w = stored[key]
        my = w.p.size
        mf[j] = min(my, n - 1)
        pf[j, 1:mf[j]] = w.p[1:mf[j]]
        qf[j, 1:mf[j]] = w.q[1:mf[j]]
        fac = 1.0 / math.sqrt(_rint(o, rp, pf, qf, mf, j, j))
        pf[j, :mf[j]] *= fac
        qf[j, :mf[j]] *= fac
    # ORTHSC
    nak = np.array([k for _, k in wanted], np.int32)
    eps = 0.01 * h ** 6
    for l in range(1, nw):
        changed = False
        mtp0 = int(mf[l])
        for k in range(l):
            if nak[k] != nak[l]:
                continue
            changed = True
            ov = _rint(o, rp, pf, qf, mf, l, k)
            mtp = int(max(mf[l], mf[k]))
            mtp0 = max(mtp0, int(mf[k]))
            pf[l, :mtp] -= ov * pf[k, :mtp]
            qf[l, :mtp] -= ov * qf[k, :mtp]
        if changed:
            mf[l] = mtp0
            fac = 1.0 / math.sqrt(_rint(o, rp, pf, qf, mf, l, l))
            pf[l, 1:mtp0] *= fac
            qf[l, 1:mtp0] *= fac
            m = mtp0
            while m >= 1 and abs(pf[l, m - 1]) < eps:
                pf[l, m - 1] = 0.0
                qf[l, m - 1] = 0.0
                m -= 1
            mf[l] = m
    return dict(n=n, rnt=rnt, h=h, c=c, z=z, zz=zz, nak=nak, np=np.array([p for p, _ in wanted], np.int32), mf=mf,
                pf=pf, qf=qf, labels=labels, ncore=ncore, levels=sm["levels"], summary=sm,
                e=np.array([stored[key].e for key in wanted]))
