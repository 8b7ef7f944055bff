"""The error model of the FP32 pre-check of the inert-cell test.

The pre-check accepts a cell when dt (|f32| + KAPPA g + EPS) passes the
inert test, g being the gross rates. That is sound when every FP32 rate of
progress is within a relative DELTA < KAPPA of its FP64 value. Each such
rate is an exponential of a sum of terms (ln A, beta ln T, E/RT for the
forward constant; the species' S/R - H/RT and the pressure factor for the
equilibrium constant; the low-pressure terms for fall-off), so its relative
FP32 error is bounded by a count of roundings, each at most one FP32 ulp of
the largest value it touches. This test evaluates that worst-case count for
every reaction of GRI-Mech 3.0 from 300 to 3500 K with the oracle's
mechanism data and checks DELTA <= KAPPA / 10.
"""
import ctypes

import numpy as np

KAPPA = 1e-2  # PRE_KAPPA of the library's pre-check
MAXSP, MAXRX = 64, 512


class _Mech(ctypes.Structure):
    _fields_ = [("nelem", ctypes.c_int), ("kk", ctypes.c_int), ("ii", ctypes.c_int),
                ("ename", ctypes.c_char * 4 * 8), ("awt", ctypes.c_double * 8),
                ("kname", ctypes.c_char * 24 * MAXSP), ("wt", ctypes.c_double * MAXSP),
                ("tt", ctypes.c_double * 3 * MAXSP), ("aa", ctypes.c_double * 7 * 2 * MAXSP),
                ("ncf", ctypes.c_int * 8 * MAXSP), ("nspec_sign", ctypes.c_int * MAXRX),
                ("nu", ctypes.c_int * 6 * MAXRX), ("nunk", ctypes.c_int * 6 * MAXRX),
                ("par", ctypes.c_double * 3 * MAXRX), ("tb", ctypes.c_int * MAXRX), ("kfal", ctypes.c_int * MAXRX),
                ("ifop", ctypes.c_int * MAXRX), ("fpar", ctypes.c_double * 7 * MAXRX),
                ("ntbs", ctypes.c_int * MAXRX), ("nktb", ctypes.c_int * 16 * MAXRX),
                ("aik", ctypes.c_double * 16 * MAXRX), ("ru", ctypes.c_double), ("patm", ctypes.c_double),
                ("hf298", ctypes.c_double * MAXSP)]


def _worst_delta(m):
    kk, ii = m.kk, m.ii
    aa = np.array([[list(m.aa[k][r]) for r in range(2)] for k in range(kk)])
    tmid = np.array([m.tt[k][1] for k in range(kk)])
    par = np.array([list(m.par[i]) for i in range(ii)])
    nu = np.array([list(m.nu[i]) for i in range(ii)])
    nunk = np.array([list(m.nunk[i]) for i in range(ii)])
    rev = np.array([m.nspec_sign[i] for i in range(ii)]) > 0
    tb = np.array([m.tb[i] for i in range(ii)])
    fpar = np.array([list(m.fpar[i]) for i in range(ii)])
    u = 2.0 ** -23
    worst = 0.0
    for T in np.geomspace(300.0, 3500.0, 24):
        a = aa[np.arange(kk), (T > tmid).astype(int)]
        lnT = np.log(T)
        terms = np.stack([np.abs(a[:, 0] * (lnT - 1)), np.abs(a[:, 1] / 2 * T), np.abs(a[:, 2] / 6 * T ** 2),
                          np.abs(a[:, 3] / 12 * T ** 3), np.abs(a[:, 4] / 20 * T ** 4), np.abs(a[:, 5] / T),
                          np.abs(a[:, 6])], axis=1)
        smh = (a[:, 0] * (lnT - 1) + a[:, 1] / 2 * T + a[:, 2] / 6 * T ** 2 + a[:, 3] / 12 * T ** 3
               + a[:, 4] / 20 * T ** 4 - a[:, 5] / T + a[:, 6])
        # S/R - H/RT: eight roundings, each at most an ulp of the largest
        # partial value, and the FP32 coefficients (2^-24 each)
        err_smh = u * (8 * np.maximum(terms.max(axis=1), np.abs(smh)) + terms.sum(axis=1))
        fwd = u * 4 * (np.abs(np.log(np.abs(par[:, 0]) + 1e-300)) + np.abs(par[:, 1] * lnT) + np.abs(par[:, 2] / T))
        revp = np.zeros(ii)
        for i in np.nonzero(rev)[0]:
            idx = nunk[i] >= 0
            revp[i] = (np.abs(nu[i][idx]) * err_smh[nunk[i][idx]]).sum()
            revp[i] += u * 4 * abs(nu[i].sum()) * abs(np.log(m.patm / (m.ru * T)))
        low = (np.abs(np.log(np.abs(fpar[:, 0]) + 1e-300) - np.log(np.abs(par[:, 0]) + 1e-300))
               + np.abs((fpar[:, 1] - par[:, 1]) * lnT) + np.abs((fpar[:, 2] - par[:, 2]) / T))
        # fall-off: the reduced pressure's exponent and the Troe blend (a few
        # ulp of quantities of order one)
        fall = np.where(tb == 2, u * 4 * low + 1e-5, 0.0)
        worst = max(worst, float((fwd + revp + fall + 1e-6).max()))
    return worst


def test_fp32_rate_error_bound_is_a_tenth_of_kappa(oracle):
    m = _Mech.from_buffer(oracle.mech)
    assert ctypes.sizeof(_Mech) == oracle.L.or_mech_sizeof()
    assert m.kk == 53 and m.ii == 325
    delta = _worst_delta(m)
    assert 1e-4 < delta <= KAPPA / 10, delta
