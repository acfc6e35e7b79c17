"""Interaction-vertex builders for ``solve_rpa_PH`` (numpy, host side).

The Kanamori vertex of ``python/triqs_tprf/rpa_tensor.py`` (charge / spin
tensors ``:87-120``, their spin-resolved combination ``:175-195``,
``kanamori_quartic_tensor`` ``:198-233``), written as sums of Kronecker-delta
tensors. In the particle-hole order [a, abar, b, bbar] that ``solve_rpa_PH``
takes, the Kanamori terms have four index patterns:

* D  = delta(a = abar = b = bbar)              (intra-orbital, U)
* P1 = delta(a = bbar) delta(abar = b) - D     (inter-orbital pair, U')
* P2 = delta(a = abar) delta(b = bbar) - D     (inter-orbital density, J)
* P3 = delta(a = b) delta(abar = bbar) - D     (pair hopping / spin flip, J')

and U_s = U D + U' P1 + J P2 + J' P3, U_c = U D + (2J - U') P1 + (2U' - J) P2
+ J' P3. The spin-resolved tensor (spin the slow index) puts
-(U_c - U_s)/2 on the equal-spin blocks, -(U_c + U_s)/2 on (s, s, s', s') and
U_s on (s, s', s', s) for s != s'.
"""
from __future__ import annotations

import numpy as np

__all__ = ["kanamori_charge_and_spin_quartic_interaction_tensors", "quartic_tensor_from_charge_and_spin",
           "kanamori_quartic_tensor"]


def _delta_patterns(n: int):
    """(D, P1, P2, P3) of the module docstring for n orbitals (or spins)."""
    I = np.eye(n)
    D = np.einsum("ij,jk,kl->ijkl", I, I, I)
    P1 = np.einsum("il,jk->ijkl", I, I) - D
    P2 = np.einsum("ij,kl->ijkl", I, I) - D
    P3 = np.einsum("ik,jl->ijkl", I, I) - D
    return D, P1, P2, P3


def kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp):
    """(U_c, U_s) of the Kanamori interaction in particle-hole order."""
    D, P1, P2, P3 = _delta_patterns(int(norb))
    U_s = U * D + Up * P1 + J * P2 + Jp * P3
    U_c = U * D + (2 * J - Up) * P1 + (2 * Up - J) * P2 + Jp * P3
    return U_c.astype(complex), U_s.astype(complex)


def quartic_tensor_from_charge_and_spin(U_c, U_s):
    """Spin-resolved tensor (spin the slow index of each combined index) from the
    charge and spin channels."""
    U_c, U_s = np.asarray(U_c, dtype=complex), np.asarray(U_s, dtype=complex)
    norb = U_c.shape[0]
    D, _, P2, _ = _delta_patterns(2)
    same = D                                    # (s, s, s, s)
    dens = P2                                   # (s, s, s', s'), s != s'
    flip = np.einsum("il,jk->ijkl", np.eye(2), np.eye(2)) - D  # (s, s', s', s), s != s'
    blocks = (np.einsum("pqrs,abcd->paqbrcsd", same, -0.5 * (U_c - U_s))
              + np.einsum("pqrs,abcd->paqbrcsd", dens, -0.5 * (U_c + U_s))
              + np.einsum("pqrs,abcd->paqbrcsd", flip, U_s))
    return blocks.reshape((2 * norb,) * 4)


def kanamori_quartic_tensor(norb, U, Up, J, Jp):
    """Spin-resolved Kanamori vertex (spin slow) for solve_rpa_PH."""
    return quartic_tensor_from_charge_and_spin(*kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp))
