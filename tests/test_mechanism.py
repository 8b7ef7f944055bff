"""Mechanism front end: the library's CHEMKIN parser vs an independent reader.

The committed mech.edyn (written by the library's parser) must agree with
tests/golden/gri30_mech_golden.json (written by a separate pure-Python
reader of the same chem.inp/therm.dat, tests/golden/make_golden.py).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import reference_dir

ROOT = Path(__file__).resolve().parent.parent
GOLD = json.loads((ROOT / "tests/golden/gri30_mech_golden.json").read_text())
MECH_TXT = (ROOT / "fortrancfd_gb300/data/gri30/mech.edyn").read_text()


def read_edyn(txt):
    tok = txt.split()
    assert tok[0] == "EDYNMECH" and tok[1] == "1"
    i = 2
    assert tok[i] == "ELEMENTS"
    ne = int(tok[i + 1])
    i += 2
    elems = []
    for _ in range(ne):
        elems.append((tok[i], float(tok[i + 1])))
        i += 2
    assert tok[i] == "SPECIES"
    ns = int(tok[i + 1])
    i += 2
    sp = []
    for _ in range(ns):
        name = tok[i]
        W, tlo, tmid, thi = map(float, tok[i + 1:i + 5])
        a = [float(v) for v in tok[i + 5:i + 19]]
        cnt = [int(v) for v in tok[i + 19:i + 19 + ne]]
        sp.append(dict(name=name, W=W, tlo=tlo, tmid=tmid, thi=thi, low=a[:7], high=a[7:], cnt=cnt))
        i += 19 + ne
    assert tok[i] == "REACTIONS"
    nr = int(tok[i + 1])
    i += 2
    rx = []
    for _ in range(nr):
        eq, rev = tok[i], int(tok[i + 1])
        i += 2
        slots = []
        for _ in range(6):
            slots.append((int(tok[i]), int(tok[i + 1])))
            i += 2
        A, b, E = map(float, tok[i:i + 3])
        tb, kfal, ifop = map(int, tok[i + 3:i + 6])
        low = [float(v) for v in tok[i + 6:i + 9]]
        troe = [float(v) for v in tok[i + 9:i + 13]]
        dup, neff = int(tok[i + 13]), int(tok[i + 14])
        i += 15
        eff = {}
        for _ in range(neff):
            eff[int(tok[i])] = float(tok[i + 1])
            i += 2
        rx.append(dict(eq=eq, rev=rev, slots=slots, A=A, beta=b, E_R=E, tb=tb, kfal=kfal, ifop=ifop, low=low,
                       troe=troe, dup=dup, eff=eff))
    assert tok[i] == "END"
    return elems, sp, rx


ELEMS, SP, RX = read_edyn(MECH_TXT)
NAMES = [s["name"] for s in SP]


def test_counts():
    assert len(SP) == 53 and len(RX) == 325
    assert [s["name"] for s in GOLD["species"]] == NAMES
    assert sum(r["tb"] == 2 for r in RX) == 29
    assert sum(r["ifop"] >= 3 for r in RX) == 26
    assert sum(r["dup"] for r in RX) == sum(r["dup"] for r in GOLD["reactions"])


def test_species_tables_bitwise():
    for s, g in zip(SP, GOLD["species"]):
        assert s["W"] == g["W"], s["name"]
        assert (s["tlo"], s["tmid"], s["thi"]) == (g["tlo"], g["tmid"], g["thi"])
        assert s["low"] == g["low"] and s["high"] == g["high"], s["name"]


def test_molecular_weights_use_single_precision_atomic_weights():
    # CH4 = C + 4 H with the interpreter's float literals, summed in card order
    w = float(np.float32(12.01115)) + float(np.float32(1.00797)) * 4.0
    assert SP[NAMES.index("CH4")]["W"] == w
    assert abs(SP[NAMES.index("CH4")]["W"] - 16.04303) < 1e-4


def test_reactions_match_independent_reader():
    for r, g in zip(RX, GOLD["reactions"]):
        reac, prod = {}, {}
        for q, (k, nu) in enumerate(r["slots"]):
            if k < 0:
                continue
            (reac if q < 3 else prod)[NAMES[k]] = abs(nu)
        assert reac == g["reac"] and prod == g["prod"], g["eq"]
        assert bool(r["rev"]) == g["rev"], g["eq"]
        assert r["A"] == g["A"] and r["beta"] == g["beta"]
        assert r["E_R"] == g["E_R"], g["eq"]
        assert (r["tb"] == 1) == g["tb"], g["eq"]
        assert (r["tb"] == 2) == (g["falloff"] is not None), g["eq"]
        if g["low"]:
            assert r["low"] == g["low"], g["eq"]
        if g["troe"]:
            assert r["troe"][:len(g["troe"])] == g["troe"]
            assert r["ifop"] == (3 if len(g["troe"]) == 3 else 4)
        elif g["falloff"]:
            assert r["ifop"] == 1
        assert {NAMES[k]: v for k, v in r["eff"].items()} == g["eff"], g["eq"]
        assert bool(r["dup"]) == g["dup"]


def test_element_balance():
    for r in RX:
        bal = np.zeros(len(ELEMS))
        for k, nu in r["slots"]:
            if k >= 0:
                bal += nu * np.array(SP[k]["cnt"])
        assert not bal.any(), r["eq"]


def test_library_parser_reproduces_committed_table(tmp_path):
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference checkout not present")
    from fortrancfd_gb300 import mech_compile

    out = tmp_path / "mech.edyn"
    mech_compile(ref / "WORK/Examples/CH4_GRI3.0/SOD/GRI3.0_CH4", out)
    assert out.read_text() == MECH_TXT


def test_library_parser_rejects_missing_dir(tmp_path):
    from fortrancfd_gb300 import EdynError, mech_compile

    with pytest.raises(EdynError):
        mech_compile(tmp_path / "nowhere", tmp_path / "x.edyn")
