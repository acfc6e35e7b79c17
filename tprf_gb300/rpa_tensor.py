"""Interaction-vertex builders for ``solve_rpa_PH`` (numpy, host side).

Restates the numpy parts of ``python/triqs_tprf/rpa_tensor.py``: the Kanamori
charge / spin tensors (``:87-120``), their spin-resolved combination
(``:175-195``) and ``kanamori_quartic_tensor`` (``:198-233``). Tensors are in
the particle-hole order that ``solve_rpa_PH`` expects.
"""
from __future__ import annotations

import itertools

import numpy as np

__all__ = ["kanamori_charge_and_spin_quartic_interaction_tensors", "quartic_tensor_from_charge_and_spin",
           "kanamori_quartic_tensor"]


def kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp):
    shape = [norb] * 4
    U_c = np.zeros(shape, dtype=complex)
    U_s = np.zeros(shape, dtype=complex)
    for a, abar, b, bbar in itertools.product(range(norb), repeat=4):
        sc = ss = 0.0
        if a == abar == b == bbar:
            sc, ss = U, U
        if a == bbar and a != b and abar == b:
            sc, ss = -Up + 2 * J, Up
        if a == abar and a != b and b == bbar:
            sc, ss = 2 * Up - J, J
        if a == b and a != abar and abar == bbar:
            sc, ss = Jp, Jp
        U_c[a, abar, b, bbar] = sc
        U_s[a, abar, b, bbar] = ss
    return U_c, U_s


def quartic_tensor_from_charge_and_spin(U_c, U_s):
    norb = U_c.shape[0]
    U_8 = np.zeros([2] * 4 + [norb] * 4, dtype=complex)
    U_uu = -0.5 * (U_c - U_s)
    U_ud = 0.5 * (U_c + U_s)
    for s1, s2 in itertools.product(range(2), repeat=2):
        if s1 == s2:
            U_8[s1, s1, s1, s1] = U_uu
        else:
            U_8[s1, s1, s2, s2] = -U_ud
            U_8[s1, s2, s2, s1] = U_s
    U_8 = np.transpose(U_8, (0, 4, 1, 5, 2, 6, 3, 7))
    return U_8.reshape([2 * norb] * 4)


def kanamori_quartic_tensor(norb, U, Up, J, Jp):
    U_c, U_s = kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp)
    return quartic_tensor_from_charge_and_spin(U_c, U_s)
