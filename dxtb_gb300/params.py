"""
GFN1/GFN2-xTB parameter tables in the flat layout of ``include/dxtb_gb300.h``.

Reads the packaged parameter files (converted from dxtb's
``param/gfn{1,2}/*.toml``), expands every shell into its contracted
Gaussians (STO-nG of Stewart, JCP 52, 431 (1970); GFN1's second hydrogen
s shell orthonormalised against the first) and fills the float64/int32
tables the kernels read. Layout offsets are parsed from the C header so
that host and device can never disagree.

Reference: basis/slater.py:69-146, basis/ortho.py:74-110,
basis/bas.py:124-168, xtb/base.py:107-186, xtb/gfn1.py:66-165,
xtb/gfn2.py:67-156, param/module/utils.py:480-530.
"""

from __future__ import annotations

import json
import math
import re
from functools import lru_cache
from pathlib import Path

import numpy as np

from .data import radii

PKG = Path(__file__).resolve().parent
HEADER = PKG.parent / "include" / "dxtb_gb300.h"


@lru_cache(maxsize=1)
def layout() -> dict[str, int]:
    """Integer values of every ``#define DXTB_*`` in the header."""
    env: dict[str, int] = {}
    for line in HEADER.read_text().splitlines():
        m = re.match(r"#define\s+(DXTB_\w+)\s+(.+?)\s*(/\*.*)?$", line)
        if not m:
            continue
        expr = m.group(2)
        if not re.fullmatch(r"[\w\s\+\-\*\(\)/]+", expr):
            continue
        try:
            env[m.group(1)] = int(eval(expr, {"__builtins__": {}}, dict(env)))
        except Exception:
            pass
    return env


@lru_cache(maxsize=4)
def load_par(method: str) -> dict:
    with open(PKG / "data" / f"{method}.json") as fh:
        par = json.load(fh)
    par["element"] = {int(k): v for k, v in par["element"].items()}
    return par


@lru_cache(maxsize=1)
def _stong() -> dict:
    return dict(np.load(PKG / "data" / "stong.npz"))


_DFACT = (1.0, 1.0, 3.0, 15.0, 105.0, 945.0)


def sto_ng(ng: int, n: int, l: int, zeta: float) -> tuple[np.ndarray, np.ndarray]:
    """Normalised STO-nG contraction of a Slater shell (exponents, coefficients)."""
    itype = n + (0, 4, 7, 9, 10)[l] - 1
    if n == 6 and ng == 6:
        itype = 15 + l
    tab = _stong()[f"sto{ng}g"]
    alpha = tab[1, itype, :].astype(np.float64) * zeta * zeta
    coeff = tab[0, itype, :].astype(np.float64)
    coeff = coeff * (2.0 / math.pi * alpha) ** 0.75 * np.sqrt(4.0 * alpha) ** l / math.sqrt(_DFACT[l])
    return alpha, coeff / math.sqrt(_self_overlap(alpha, coeff, l))


def _self_overlap(alpha: np.ndarray, coeff: np.ndarray, l: int) -> float:
    p = alpha[:, None] + alpha[None, :]
    pref = (math.pi / p) ** 1.5 * _DFACT[l] / (2.0 * p) ** l
    return float((coeff[:, None] * coeff[None, :] * pref).sum())


def _s_overlap(ai, aj, ci, cj) -> float:
    p = ai[:, None] + aj[None, :]
    return float(((math.pi / p) ** 1.5 * ci[:, None] * cj[None, :]).sum())


def orthonormalise(a1, c1, a2, c2):
    """Second s shell orthonormalised to the first (Gram-Schmidt)."""
    ov = _s_overlap(a1, a2, c1, c2)
    a = np.concatenate([a2, a1])
    c = np.concatenate([c2, -ov * c1])
    return a, c / math.sqrt(_s_overlap(a, a, c, c))


class Tables:
    """Flat parameter tables of one method plus the per-element shell map."""

    def __init__(self, method: str):
        method = method.lower().replace("-", "").replace("_", "")
        method = {"gfn1xtb": "gfn1", "gfn2xtb": "gfn2"}.get(method, method)
        if method not in ("gfn1", "gfn2"):
            raise ValueError(f"Unknown method '{method}'")
        self.method = method
        L = layout()
        par = load_par(method)
        self.par = par
        maxz, maxsht, maxprim = L["DXTB_MAXZ"], L["DXTB_MAXSHT"], L["DXTB_MAXPRIM"]
        f = np.zeros(L["DXTB_P_SIZE"], dtype=np.float64)
        i = np.zeros(L["DXTB_I_SIZE"], dtype=np.int32)
        ev2au = radii.EV2AU
        self.el_shells: dict[int, list[int]] = {}
        self.el_angular: dict[int, list[int]] = {}
        t = 0
        for z in range(1, maxz):
            e = par["element"].get(z)
            if e is None:
                continue
            i[L["DXTB_I_EL_SH0"] + z] = t
            i[L["DXTB_I_EL_NSH"] + z] = len(e["angular"])
            self.el_angular[z] = list(e["angular"])
            types = []
            prev = None
            for k, l in enumerate(e["angular"]):
                a, c = sto_ng(e["ngauss"][k], e["pqn"][k], l, e["slater"][k])
                if method == "gfn1" and not e["valence"][k]:
                    a, c = orthonormalise(prev[0], prev[1], a, c)
                prev = (a, c)
                # unit self-overlap with the integral kernel's own formula
                c = c / math.sqrt(_self_overlap(a, c, l))
                if len(a) > maxprim:
                    raise ValueError("too many primitives")
                f[L["DXTB_P_ALPHA"] + t * maxprim : L["DXTB_P_ALPHA"] + t * maxprim + len(a)] = a
                f[L["DXTB_P_COEFF"] + t * maxprim : L["DXTB_P_COEFF"] + t * maxprim + len(c)] = c
                f[L["DXTB_P_LEVEL"] + t] = e["levels"][k] * ev2au
                f[L["DXTB_P_KCN"] + t] = e["kcn"][k] * ev2au
                f[L["DXTB_P_SHPOLY"] + t] = e["shpoly"][k]
                f[L["DXTB_P_REFOCC"] + t] = e["refocc"][k]
                f[L["DXTB_P_LGAM"] + t] = e["lgam"][k]
                f[L["DXTB_P_SLATER"] + t] = e["slater"][k]
                i[L["DXTB_I_L"] + t] = l
                i[L["DXTB_I_NPRIM"] + t] = len(a)
                i[L["DXTB_I_VALENCE"] + t] = 1 if e["valence"][k] else 0
                i[L["DXTB_I_ELEM"] + t] = z
                types.append(t)
                t += 1
            self.el_shells[z] = types
            for key, off in (
                ("en", "DXTB_P_EN"), ("gam", "DXTB_P_GAM"), ("gam3", "DXTB_P_GAM3"),
                ("zeff", "DXTB_P_ZEFF"), ("arep", "DXTB_P_AREP"), ("dkernel", "DXTB_P_DKERNEL"),
                ("qkernel", "DXTB_P_QKERNEL"), ("mprad", "DXTB_P_MPRAD"), ("mpvcn", "DXTB_P_MPVCN"),
            ):
                f[L[off] + z] = e[key]
        if t > maxsht:
            raise ValueError("too many shell types")
        self.nshelltypes = t
        for tab, off in ((radii.COV_D3, "DXTB_P_RCOV"), (radii.ATOMIC_RADII, "DXTB_P_RAD"),
                         (radii.VDW_D3, "DXTB_P_VDW")):
            v = np.nan_to_num(tab[:maxz], nan=0.0)
            f[L[off] : L[off] + len(v)] = v
        # element-pair scaling, default 1 (param/module/param.py get_pair_param)
        kp = np.ones((maxz, maxz))
        for za, zb, v in par["hamiltonian"]["xtb"].get("kpair", []):
            kp[za, zb] = kp[zb, za] = v
        f[L["DXTB_P_KPAIR"] : L["DXTB_P_KPAIR"] + maxz * maxz] = kp.ravel()
        # shell-pair scaling k_{ll'} (valence-valence) from the shell table
        xtb = par["hamiltonian"]["xtb"]
        shell = xtb["shell"]
        lab = "spdfg"
        kvv = np.ones((5, 5))
        for la in range(5):
            for lb in range(5):
                ka, kb = lab[la] * 2, lab[lb] * 2
                if method == "gfn1":
                    kaa, kbb = shell.get(ka, 1.0), shell.get(kb, 1.0)
                else:
                    kaa, kbb = shell.get(ka, 1.0), shell.get(kb, 1.0)
                kvv[la, lb] = shell.get(lab[la] + lab[lb], shell.get(lab[lb] + lab[la], 0.5 * (kaa + kbb)))
        f[L["DXTB_P_KSHELL"] : L["DXTB_P_KSHELL"] + 25] = kvv.ravel()
        to = par.get("thirdorder", {})
        es3_shell = isinstance(to.get("shell"), dict)
        if es3_shell:
            sc = [to["shell"].get(x, 0.0) for x in ("s", "p", "d", "f", "g")]
            f[L["DXTB_P_ES3SCALE"] : L["DXTB_P_ES3SCALE"] + 5] = sc
        S = L["DXTB_P_SCAL"]
        f[S + L["DXTB_S_KPOL"]] = xtb.get("kpol", 2.0)
        f[S + L["DXTB_S_WEXP"]] = xtb.get("wexp", 0.0)
        f[S + L["DXTB_S_ENSCALE"]] = xtb.get("enscale", 0.0)
        f[S + L["DXTB_S_GEXP"]] = par["charge"]["effective"]["gexp"]
        rep = par["repulsion"]["effective"]
        f[S + L["DXTB_S_REP_KEXP"]] = rep["kexp"]
        f[S + L["DXTB_S_REP_KLIGHT"]] = rep.get("klight", -1.0)
        mp = par.get("multipole", {}).get("damped")
        if mp:
            f[S + L["DXTB_S_DMP3"]] = mp["dmp3"]
            f[S + L["DXTB_S_DMP5"]] = mp["dmp5"]
            f[S + L["DXTB_S_MP_KEXP"]] = mp["kexp"]
            f[S + L["DXTB_S_MP_SHIFT"]] = mp["shift"]
            f[S + L["DXTB_S_MP_RMAX"]] = mp["rmax"]
        f[S + L["DXTB_S_CN_CUTOFF"]] = 25.0
        f[S + L["DXTB_S_REP_CUTOFF"]] = rep.get("cutoff", 25.0)
        IS = L["DXTB_I_SCAL"]
        i[IS + L["DXTB_IS_METHOD"]] = 1 if method == "gfn1" else 2
        i[IS + L["DXTB_IS_CN_KIND"]] = 0 if xtb.get("cn", "exp") == "exp" else 1
        i[IS + L["DXTB_IS_AVERAGE"]] = {"harmonic": 0, "arithmetic": 1, "geometric": 2}[
            par["charge"]["effective"]["average"]
        ]
        i[IS + L["DXTB_IS_ES3_SHELL"]] = 1 if es3_shell else 0
        i[IS + L["DXTB_IS_MULTIPOLE"]] = 1 if mp else 0
        self.f64 = f
        self.i32 = i
        self.multipole = bool(mp)
        self.es3_shell = es3_shell
        self.cn_kind = 0 if xtb.get("cn", "exp") == "exp" else 1
        # shells and spherical orbitals per element (0 for elements without parameters)
        self.el_nsh = np.zeros(maxz, dtype=np.int64)
        self.el_nao = np.zeros(maxz, dtype=np.int64)
        for z, ang in self.el_angular.items():
            self.el_nsh[z] = len(ang)
            self.el_nao[z] = sum(2 * l + 1 for l in ang)

    def check_elements(self, numbers) -> None:
        z = set(int(v) for v in np.asarray(numbers).ravel() if v > 0)
        missing = [v for v in z if v not in self.el_shells]
        if missing:
            raise ValueError(f"No {self.method} parameters for elements {missing}")
        for tab, name in ((radii.COV_D3, "covalent"), (radii.ATOMIC_RADII, "atomic")):
            radii.lookup(tab, sorted(z), name)
