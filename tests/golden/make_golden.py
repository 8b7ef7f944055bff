"""Generates the golden fixtures of tests/golden from the reference checkout.

Run where the reference tree is present, with its path in $EDYN_REFERENCE:

    EDYN_REFERENCE=<reference checkout> python tests/golden/make_golden.py

1. gri30_mech_golden.json -- GRI-Mech 3.0 as read by an independent,
   pure-Python CHEMKIN-II reader written here (not the library's C++
   parser): species molecular weights (from single-precision atomic
   weights, as the reference's interpreter declares them), NASA-7 ranges
   and coefficients, and per reaction the stoichiometry, Arrhenius
   parameters with E converted to K, third-body efficiencies and fall-off
   data. The library's parser output (mech.edyn) is checked against it.
2. equil_tp_ch4air_T1300_p1.json -- the Cantera TP-equilibrium composition
   of stoichiometric CH4/air at 1300 K, 1 atm that the reference ships
   (WORK/Examples/CH4_GRI3.0/MFR/equilTP_phi1.0_p1.0_T1300.0.txt), used to
   pin the oracle's Gibbs functions and equilibrium constants.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("EDYN_REFERENCE", ""))
MECH = REF / "WORK/Examples/CH4_GRI3.0/SOD/GRI3.0_CH4"
EQUIL = REF / "WORK/Examples/CH4_GRI3.0/MFR/equilTP_phi1.0_p1.0_T1300.0.txt"

ATOMIC = {"H": 1.00797, "HE": 4.00260, "C": 12.01115, "N": 14.00670, "O": 15.99940, "AR": 39.94800}


def f32(x: float) -> float:
    return float(np.float32(x))


def parse_therm(lines, species):
    data = {}
    i = 0
    while i < len(lines):
        l1 = lines[i]
        if len(l1) >= 80 and l1[79] == "1":
            name = l1[:18].split()[0]
            if name in species and name not in data:
                l2, l3, l4 = lines[i + 1], lines[i + 2], lines[i + 3]
                nums = [float(l2[15 * j:15 * j + 15]) for j in range(5)]
                nums += [float(l3[15 * j:15 * j + 15]) for j in range(5)]
                nums += [float(l4[15 * j:15 * j + 15]) for j in range(4)]
                comp = []
                for col in (24, 29, 34, 39, 73):
                    el, cnt = l1[col:col + 2].strip(), l1[col + 2:col + 5].strip()
                    if el and cnt and int(float(cnt)) != 0:
                        comp.append((el.upper(), int(float(cnt))))
                data[name] = dict(tlo=float(l1[45:55]), thi=float(l1[55:65]), tmid=float(l1[65:73]),
                                  high=nums[0:7], low=nums[7:14], comp=comp)
                i += 4
                continue
        i += 1
    return data


def split_species(side: str, species: set):
    out = {}
    tb = False
    for tok in re.split(r"(?<!^)\+(?![^(]*\))", side):
        if not tok:
            continue
        if tok.upper() == "M":
            tb = True
            continue
        coef, name = 1, tok
        if name not in species:
            m = re.match(r"^(\d+)(.*)$", tok)
            coef, name = int(m.group(1)), m.group(2)
        out[name] = out.get(name, 0) + coef
    return out, tb


def parse_chem(text: str):
    lines = [l.split("!")[0].rstrip() for l in text.splitlines()]
    species, reactions = [], []
    sec = None
    for l in lines:
        t = l.strip()
        if not t:
            continue
        u = t.upper()
        if sec != "REAC":
            if u.startswith("ELEM"):
                sec = "ELEM"
                continue
            if u.startswith("SPEC"):
                sec = "SPEC"
                continue
            if u.startswith("REAC"):
                sec = "REAC"
                continue
            if u.startswith("END"):
                sec = None
                continue
            if sec == "SPEC":
                species += [s for s in t.split() if s.upper() != "END"]
            continue
        if u.startswith("END"):
            break
        if "=" in t:
            tok = t.split()
            eq = "".join(tok[:-3])
            A, b, E = map(float, tok[-3:])
            rev = "<=>" in eq or ("=" in eq and "=>" not in eq)
            lhs, rhs = re.split(r"<=>|=>|=", eq)
            fall = None
            for side in ("lhs", "rhs"):
                s = lhs if side == "lhs" else rhs
                m = re.search(r"\(\+([^)]*)\)", s)
                if m:
                    fall = m.group(1)
                    s = s[:m.start()] + s[m.end():]
                if side == "lhs":
                    lhs = s
                else:
                    rhs = s
            re_, tbl = split_species(lhs, set(species))
            pr_, tbr = split_species(rhs, set(species))
            reactions.append(dict(eq=eq, rev=rev, reac=re_, prod=pr_, A=A, beta=b, E=E,
                                  tb=bool(tbl or tbr), falloff=fall, low=None, troe=None, eff={}, dup=False))
        else:
            r = reactions[-1]
            for key, val in re.findall(r"([A-Za-z0-9()\-*,]+)\s*(?:/([^/]*)/)?", t):
                K = key.upper()
                if K in ("DUP", "DUPLICATE"):
                    r["dup"] = True
                elif K == "LOW":
                    r["low"] = [float(v) for v in val.split()]
                elif K == "TROE":
                    r["troe"] = [float(v) for v in val.split()]
                elif key in species:
                    r["eff"][key] = float(val)
    return species, reactions


def main():
    if not os.environ.get("EDYN_REFERENCE") or not MECH.exists():
        sys.exit("set EDYN_REFERENCE to the reference checkout (its GRI-Mech 3.0 directory was not found)")
    species, reactions = parse_chem((MECH / "chem.inp").read_text())
    therm = parse_therm((MECH / "therm.dat").read_text().splitlines(), set(species))
    efac = f32(4.184) / 8.314510
    sp_out = []
    for s in species:
        d = therm[s]
        w = 0.0
        for el, n in d["comp"]:
            w = w + f32(ATOMIC[el]) * float(np.float32(n))
        sp_out.append(dict(name=s, W=w, tlo=d["tlo"], tmid=d["tmid"], thi=d["thi"], low=d["low"], high=d["high"],
                           comp=d["comp"]))
    rx_out = []
    for r in reactions:
        rx_out.append(dict(eq=r["eq"], rev=r["rev"], reac=r["reac"], prod=r["prod"], A=r["A"], beta=r["beta"],
                           E_R=r["E"] * efac, tb=r["tb"], falloff=r["falloff"],
                           low=None if r["low"] is None else [r["low"][0], r["low"][1], r["low"][2] * efac],
                           troe=r["troe"], eff=r["eff"], dup=r["dup"]))
    (HERE / "gri30_mech_golden.json").write_text(json.dumps(dict(species=sp_out, reactions=rx_out), indent=0))
    lines = EQUIL.read_text().split()
    n = int(lines[0])
    X = {lines[1 + 2 * i]: float(lines[2 + 2 * i]) for i in range(n)}
    (HERE / "equil_tp_ch4air_T1300_p1.json").write_text(json.dumps(
        dict(source="Cantera TP equilibrium, stoichiometric CH4/air, shipped with the reference",
             T=1300.0, p_atm=1.0, X=X), indent=0))
    print("wrote", HERE / "gri30_mech_golden.json", "and", HERE / "equil_tp_ch4air_T1300_p1.json")


if __name__ == "__main__":
    main()
