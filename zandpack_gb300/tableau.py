"""Runge-Kutta tableaux in the reference's layout (Zandpack/mpi_RK4pars_dev.py).

``A`` are the stage time fractions, ``B`` the Butcher rows with an extra last
column that multiplies the stored y (the array layout ``[k_1, ..., k_RK_N, y0]``),
``CT`` the error weights (b5 - b4), ``CH`` the update weights with the trailing
1 for y0, and ``idxholder[i]`` the columns stage i reads.  The method is chosen
like the reference does: ``k0nfig.RK_Method`` ('DOP54'), overridable by the
environment variable ``RK_method`` (Zandpack/mpi_RK4pars_dev.py:23-36).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np


@dataclasses.dataclass(frozen=True)
class Tableau:
    name: str
    RK_N: int
    A: np.ndarray
    B: np.ndarray
    CT: np.ndarray
    CH: np.ndarray
    idxholder: dict
    clamp: tuple = None  # (min factor, max factor) of the step-size update, RK78 only
    order: float = 0.2

    def hnew(self, h, TE, eps):
        """Step-size update after an attempt (hnew_func): 0.9 h (eps/TE)^order,
        clamped for RK78 (Zandpack/mpi_RK4pars_dev.py:62-64,112-116,148-149)."""
        with np.errstate(divide="ignore"):
            fact = 0.9 * (eps / np.float64(TE)) ** self.order
        if self.clamp is not None:
            fact = min(max(fact, self.clamp[0]), self.clamp[1])
        return float(h * fact)


def _dop54():
    V = np.full((7, 8), np.nan)
    V[0, 0] = 0
    V[1, 0:2] = 1 / 5, 1 / 5
    V[2, 0:3] = 3 / 10, 3 / 40, 9 / 40
    V[3, 0:4] = 4 / 5, 44 / 45, -56 / 15, 32 / 9
    V[4, 0:5] = 8 / 9, 19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729
    V[5, 0:6] = 1, 9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656
    V[6, 0:7] = 1, 35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84
    b5 = np.array([35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84, 0])
    b4 = np.array([5179 / 57600, 0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40])
    B = np.zeros((7, 8))
    B[:, :7] = V[:, 1:]
    B[1:, 7] = 1.0
    idx = {0: None, 1: [0, 7], 2: [0, 1, 7], 3: [0, 1, 2, 7], 4: [0, 1, 2, 3, 7],
           5: [0, 1, 2, 3, 4, 7], 6: [0, 1, 2, 3, 4, 5, 7]}
    return Tableau("DOP54", 7, V[:, 0].copy(), B, b5 - b4, np.hstack((b5, [1.0])), idx)


def _rk45():
    nan = np.nan
    A = np.array([0, 1 / 4, 3 / 8, 12 / 13, 1, 1 / 2])
    B = np.array([[nan, nan, nan, nan, nan, nan, 1],
                  [1 / 4, nan, nan, nan, nan, nan, 1],
                  [3 / 32, 9 / 32, nan, nan, nan, nan, 1],
                  [1932 / 2197, -7200 / 2197, 7296 / 2197, nan, nan, nan, 1],
                  [439 / 216, -8, 3680 / 513, -845 / 4104, nan, nan, 1],
                  [-8 / 27, 2, -3544 / 2565, 1859 / 4104, -11 / 40, nan, 1]])
    CH = np.array([16 / 135, 0, 6656 / 12825, 28561 / 56430, -9 / 50, 2 / 55, 1])
    CT = np.array([1 / 360, 0, -128 / 4275, -2197 / 75240, 1 / 50, 2 / 55])
    idx = {0: None, 1: [0, 6], 2: [0, 1, 6], 3: [0, 1, 2, 6], 4: [0, 1, 2, 3, 6], 5: [0, 1, 2, 3, 4, 6]}
    return Tableau("RK45", 6, A, B, CT, CH, idx)


def _cash_karp():
    nan = np.nan
    A = np.array([.0, 1 / 5, 3 / 10, 3 / 5, 1, 7 / 8])
    B = np.array([[nan, nan, nan, nan, nan, nan, 1],
                  [1 / 5, nan, nan, nan, nan, nan, 1],
                  [3 / 40, 9 / 40, nan, nan, nan, nan, 1],
                  [3 / 10, -9 / 10, 6 / 5, nan, nan, nan, 1],
                  [-11 / 54, 5 / 2, -70 / 27, 35 / 27, nan, nan, 1],
                  [1631 / 55296, 175 / 512, 575 / 13824, 44274 / 110592, 253 / 4096, nan, 1]])
    b5 = np.array([37 / 378, 0, 250 / 621, 125 / 594, 0, 512 / 1771])
    b4 = np.array([2825 / 27648, 0, 18575 / 48384, 13525 / 55296, 277 / 14336, 1 / 4])
    idx = {0: None, 1: [0, 6], 2: [0, 1, 6], 3: [0, 1, 2, 6], 4: [0, 1, 2, 3, 6], 5: [0, 1, 2, 3, 4, 6]}
    return Tableau("cash-karp", 6, A, B, b5 - b4, np.hstack((b5, [1.0])), idx)


def _rk78():
    arr = np.array
    A = arr([0., 2 / 27, 1 / 9, 1 / 6, 5 / 12, 1 / 2, 5 / 6, 1 / 6, 2 / 3, 1 / 3, 1, 0, 1])
    B = np.zeros((13, 14)) * np.nan
    B[1, 0] = 2 / 27
    B[2, 0:2] = 1 / 36, 1 / 12
    B[3, 0:3] = 1 / 24, 0, 1 / 8
    B[4, 0:4] = 5 / 12, 0, -25 / 16, 25 / 16
    B[5, 0:5] = 1 / 20, 0, 0, 1 / 4, 1 / 5
    B[6, 0:6] = -25 / 108, 0, 0, 125 / 108, -65 / 27, 125 / 54
    B[7, 0:7] = 31 / 300, 0, 0, 0, 61 / 225, -2 / 9, 13 / 900
    B[8, 0:8] = 2.0, 0, 0, -53 / 6, 704 / 45, -107 / 9, 67 / 90, 3.0
    B[9, 0:9] = -91 / 108, 0, 0, 23 / 108, -976 / 135, 311 / 54, -19 / 60, 17 / 6, -1 / 12
    B[10, 0:10] = 2383 / 4100, 0, 0, -341 / 164, 4496 / 1025, -301 / 82, 2133 / 4100, 45 / 82, 45 / 164, 18 / 41
    B[11, 0:11] = 3 / 205, 0, 0, 0, 0, -6 / 41, -3 / 205, -3 / 41, 3 / 41, 6 / 41, 0
    B[12, 0:12] = -1777 / 4100, 0, 0, -341 / 164, 4496 / 1025, -289 / 82, 2193 / 4100, 51 / 82, 33 / 164, 12 / 41, 0, 1.0
    B[1:, 13] = 1
    CT = (41 / 840) * arr([1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1])
    CH = arr([0, 0, 0, 0, 0, 34 / 105, 9 / 35, 9 / 35, 9 / 280, 9 / 280, 0, 41 / 840, 41 / 840, 1])
    idx = {0: None, 1: [0, 13], 2: [0, 1, 13], 3: [0, 2, 13], 4: [0, 2, 3, 13], 5: [0, 3, 4, 13],
           6: [0, 3, 4, 5, 13], 7: [0, 4, 5, 6, 13], 8: [0, 3, 4, 5, 6, 7, 13], 9: [0, 3, 4, 5, 6, 7, 8, 13],
           10: [0, 3, 4, 5, 6, 7, 8, 9, 13], 11: [0, 5, 6, 7, 8, 9, 10, 13],
           12: [0, 3, 4, 5, 6, 7, 8, 9, 10, 11, 13]}
    return Tableau("RK78", 13, A, B, CT, CH, idx, clamp=(0.125, 4.0), order=1 / 8)


DOP54 = _dop54()
TABLEAUX = {"DOP54": DOP54, "RK45": _rk45(), "cash-karp": _cash_karp(), "RK78": _rk78()}


def selected(default="DOP54"):
    """The tableau the reference would pick: env ``RK_method`` overrides the default."""
    return TABLEAUX[os.environ.get("RK_method", default)]
